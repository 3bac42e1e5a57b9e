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
