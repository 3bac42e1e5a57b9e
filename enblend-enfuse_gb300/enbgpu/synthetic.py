"""Seeded synthetic exposure stacks and panorama pairs.

No public image suite exists for this path, so the benchmark and parity
workloads are generated: a log2-radiance field made of Gaussian-filtered
white noise (sigma 32 px) scaled to span a given number of stops, plus 40
axis-aligned rectangles and discs with constant log-radiance offsets
U(-2, 2); a weak per-channel tint field (+-0.25 stop) gives the channels
different values.  An exposure of EV e is clip((radiance * 2^e)^(1/2.2), 0, 1)
quantised to the sample type, optionally with Gaussian sensor noise added
before quantisation.
"""
from __future__ import annotations

import numpy as np
from scipy import ndimage


def _smooth_noise(rng: np.random.Generator, h: int, w: int, sigma: float) -> np.ndarray:
    # Filter at reduced resolution and upsample: the field is band-limited by
    # the sigma-32 filter, so an 8x coarser grid represents it well.
    f = 8
    hs, ws = max(4, -(-h // f) + 2), max(4, -(-w // f) + 2)
    n = rng.standard_normal((hs, ws))
    n = ndimage.gaussian_filter(n, sigma / f, mode="wrap")
    up = ndimage.zoom(n, f, order=1)[:h, :w]
    up -= up.mean()
    s = up.std()
    return up / (s if s > 0 else 1.0)


def log_radiance(h: int, w: int, stops: float, seed: int, shapes: int = 40) -> np.ndarray:
    """(H, W, 3) log2 radiance spanning about `stops` stops."""
    rng = np.random.default_rng(seed)
    base = _smooth_noise(rng, h, w, 32.0)
    lo, hi = np.percentile(base, [0.5, 99.5])
    # centred on 18% grey, which EV 0 maps to mid-grey
    base = (base - lo) / max(hi - lo, 1e-9) * stops - stops / 2.0 + np.log2(0.18)
    yy, xx = np.mgrid[0:h, 0:w]
    for _ in range(shapes):
        off = rng.uniform(-2.0, 2.0)
        cx, cy = rng.uniform(0, w), rng.uniform(0, h)
        r = rng.uniform(0.02, 0.12) * min(h, w)
        if rng.random() < 0.5:
            x0, x1 = int(max(0, cx - r)), int(min(w, cx + r * rng.uniform(0.5, 1.5)))
            y0, y1 = int(max(0, cy - r)), int(min(h, cy + r * rng.uniform(0.5, 1.5)))
            base[y0:y1, x0:x1] += off
        else:
            y0, y1 = int(max(0, cy - r)), int(min(h, cy + r + 1))
            x0, x1 = int(max(0, cx - r)), int(min(w, cx + r + 1))
            sub = (xx[y0:y1, x0:x1] - cx) ** 2 + (yy[y0:y1, x0:x1] - cy) ** 2 <= r * r
            base[y0:y1, x0:x1][sub] += off
    tint = np.stack([_smooth_noise(rng, h, w, 64.0) * 0.25 for _ in range(3)], axis=-1)
    return base[..., None] + tint


def expose(lograd: np.ndarray, ev: float, dtype, noise: float = 0.0, seed: int = 0,
           gain: float = 1.0) -> np.ndarray:
    """clip((2^lograd * gain * 2^ev)^(1/2.2), 0, 1) quantised to dtype."""
    v = np.exp2(lograd + ev) * gain
    v = np.clip(v, 0.0, None) ** (1.0 / 2.2)
    if noise > 0.0:
        v = v + np.random.default_rng(seed).normal(0.0, noise, v.shape)
    v = np.clip(v, 0.0, 1.0)
    if dtype == np.float32:
        return v.astype(np.float32)
    maxv = np.iinfo(dtype).max
    return np.rint(v * maxv).astype(dtype)


def exposure_stack(h: int, w: int, evs, dtype, stops: float, seed: int, noise: float = 0.0):
    """List of exposures of one scene (enfuse input)."""
    lr = log_radiance(h, w, stops, seed)
    return [expose(lr, ev, dtype, noise, seed + 1000 + i) for i, ev in enumerate(evs)]


def panorama_pair(h: int, w: int, offset: int, dtype, seed: int, stops: float = 8.0):
    """Two overlapping RGBA images on their union canvas and a seam mask.

    Image 0 ("black") covers x in [0, w), image 1 ("white") covers
    [offset, offset + w); each has a gain U(0.9, 1.1) and full alpha inside
    its footprint.  The 0/255 white mask follows a vertical random walk
    (one pixel per row) through the overlap.  Returns (white, black, mask)
    as (H, W_union, 4) arrays and an (H, W_union) uint8 mask.
    """
    rng = np.random.default_rng(seed)
    wu = offset + w
    lr = log_radiance(h, wu, stops, seed)
    maxv = 1.0 if np.dtype(dtype) == np.float32 else np.iinfo(dtype).max
    out = []
    for i, x0 in enumerate((0, offset)):
        gain = rng.uniform(0.9, 1.1)
        img = np.zeros((h, wu, 4), dtype)
        img[:, x0:x0 + w, :3] = expose(lr[:, x0:x0 + w], 0.0, dtype, gain=gain)
        img[:, x0:x0 + w, 3] = maxv
        out.append(img)
    black, white = out
    lo, hi = offset, w  # overlap [offset, w)
    steps = rng.integers(-1, 2, size=h)
    seam = np.clip((lo + hi) // 2 + np.cumsum(steps), lo + 1, hi - 1)
    mask = (np.arange(wu)[None, :] >= seam[:, None]).astype(np.uint8) * 255
    return white, black, mask


# Workloads named by what they are (sizes from the benchmark configurations).
def enfuse_3x1024x768_u8(seed: int = 1):
    return exposure_stack(768, 1024, [-2.0, 0.0, 2.0], np.uint8, 8.0, seed)


def enfuse_9x6000x4000_u16(seed: int = 3, h: int = 4000, w: int = 6000):
    return exposure_stack(h, w, [float(e) for e in range(-4, 5)], np.uint16, 12.0, seed, noise=2.0 ** -12)


def enblend_2x4096x3072_u16(seed: int = 2, h: int = 3072, w: int = 4096, offset: int = 2867):
    return panorama_pair(h, w, offset, np.uint16, seed)


# ---- device-side generator (torch) for the large batched workload ----------

def _smooth_noise_torch(gen, h: int, w: int, sigma: float, device):
    import torch
    import torch.nn.functional as F
    f = 8
    hs, ws = max(4, -(-h // f) + 2), max(4, -(-w // f) + 2)
    n = torch.randn((1, 1, hs, ws), generator=gen, device=device)
    s = sigma / f
    r = int(4 * s + 0.5)
    x = torch.arange(-r, r + 1, device=device, dtype=torch.float32)
    k = torch.exp(-0.5 * (x / s) ** 2)
    k = k / k.sum()
    n = F.pad(n, (r, r, 0, 0), mode="circular")
    n = F.conv2d(n, k.view(1, 1, 1, -1))
    n = F.pad(n, (0, 0, r, r), mode="circular")
    n = F.conv2d(n, k.view(1, 1, -1, 1))
    up = F.interpolate(n, scale_factor=f, mode="bilinear", align_corners=False)[0, 0, :h, :w]
    up = up - up.mean()
    sd = up.std()
    return up / torch.clamp(sd, min=1e-12)


def log_radiance_torch(h: int, w: int, stops: float, seed: int, device="cuda", shapes: int = 40):
    """(H, W, 3) log2 radiance on the device, built like log_radiance (smooth
    noise spanning `stops` stops, 40 rectangles and discs with log offsets
    U(-2, 2), a +-0.25 stop tint per channel) from a torch generator."""
    import torch
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    rng = np.random.default_rng(seed)
    base = _smooth_noise_torch(gen, h, w, 32.0, device)
    q = torch.quantile(base[:: max(1, h // 256), :: max(1, w // 256)].flatten(),
                       torch.tensor([0.005, 0.995], device=device))
    lo, hi = float(q[0]), float(q[1])
    base = (base - lo) / max(hi - lo, 1e-9) * stops - stops / 2.0 + float(np.log2(0.18))
    yy = torch.arange(h, device=device, dtype=torch.float32)[:, None]
    xx = torch.arange(w, device=device, dtype=torch.float32)[None, :]
    for _ in range(shapes):
        off = rng.uniform(-2.0, 2.0)
        cx, cy = rng.uniform(0, w), rng.uniform(0, h)
        r = rng.uniform(0.02, 0.12) * min(h, w)
        if rng.random() < 0.5:
            x0, x1 = int(max(0, cx - r)), int(min(w, cx + r * rng.uniform(0.5, 1.5)))
            y0, y1 = int(max(0, cy - r)), int(min(h, cy + r * rng.uniform(0.5, 1.5)))
            base[y0:y1, x0:x1] += off
        else:
            base += off * (((xx - cx) ** 2 + (yy - cy) ** 2) <= r * r).float()
    tint = torch.stack([_smooth_noise_torch(gen, h, w, 64.0, device) * 0.25 for _ in range(3)], dim=-1)
    return base[..., None] + tint


def expose_torch(lograd, ev: float):
    """clip((2^lograd * 2^ev)^(1/2.2), 0, 1) as float32 on the device."""
    import torch
    return torch.clamp(torch.exp2(lograd + ev) ** (1.0 / 2.2), 0.0, 1.0).contiguous()


def exposure_stack_torch(h: int, w: int, evs, dtype, stops: float, seed: int, noise: float = 0.0, device="cuda"):
    """Device-resident exposures of one scene (as exposure_stack, from the
    device generator): clip((radiance * 2^ev)^(1/2.2) + N(0, noise), 0, 1)
    quantised to uint8 / uint16 (torch tensors of shape (H, W, 3))."""
    import torch
    lr = log_radiance_torch(h, w, stops, seed, device)
    gen = torch.Generator(device=device)
    gen.manual_seed(seed + 7919)
    maxv = 255.0 if np.dtype(dtype) == np.uint8 else 65535.0
    out = []
    for ev in evs:
        v = torch.exp2(lr + ev) ** (1.0 / 2.2)
        if noise > 0.0:
            v = v + noise * torch.randn(v.shape, generator=gen, device=device)
        q = torch.round(torch.clamp(v, 0.0, 1.0) * maxv).to(torch.int32)
        if maxv == 255.0:
            out.append(q.to(torch.uint8).contiguous())
        else:
            out.append(q.to(torch.int16).view(torch.uint16).contiguous())
        del v, q
    del lr
    return out


def uneven_stack_specs(n: int = 64, seed: int = 4, lo: int = 512, hi: int = 4096, kmin: int = 3, kmax: int = 7):
    """The batched workload: n stacks with width and height log-uniform in
    [lo, hi] and an exposure count uniform in {kmin..kmax}, EVs evenly spaced
    over +-(count - 1) stops.  Returns [(h, w, evs, seed)]."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n):
        w = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
        h = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
        K = int(rng.integers(kmin, kmax + 1))
        specs.append((h, w, list(np.linspace(-(K - 1), K - 1, K)), seed * 1000 + i))
    return specs


def uneven_stacks_torch(specs, stops: float = 8.0, device="cuda"):
    """Device-resident FP32 RGB exposure stacks of the given specs."""
    out = []
    for (h, w, evs, s) in specs:
        lr = log_radiance_torch(h, w, stops, s, device)
        out.append([expose_torch(lr, ev) for ev in evs])
        del lr
    return out
