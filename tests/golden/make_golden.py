"""Generate tests/golden/reference_pyramid.npz, reference_float.npz,
reference_enfuse.npz and reference_nft.npz from the reference's own code.

Runs the reference-code oracle (oracle/reference_build.py: the reference's
pyramid.h / blend.h / fixmath.h, and enfuse.h's enfuseMask and enfuseMain,
compiled unmodified against the project's shims) on small seeded inputs and
stores inputs and outputs, so that machines without the reference tree can
check the C oracle and the CUDA path against the reference's results.
Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[2]
sys.path[:0] = [str(REPO), str(REPO / "enblend-enfuse_gb300")]

from enbgpu import synthetic  # noqa: E402
from oracle import oracle as orc  # noqa: E402
from oracle import reference_build as ref  # noqa: E402

OUT = Path(__file__).resolve().parent / "reference_pyramid.npz"
OUT_FLOAT = Path(__file__).resolve().parent / "reference_float.npz"
OUT_ENFUSE = Path(__file__).resolve().parent / "reference_enfuse.npz"
OUT_NFT = Path(__file__).resolve().parent / "reference_nft.npz"

# enfuseMask cases: weighting options in the keyword form of
# oracle.reference_build.enfuse_params (cutoffs as (value, is_percentage) pairs)
MASK_CASES = [
    dict(exposure_weight=1.0),
    dict(exposure_weight=1.0, saturation_weight=0.2),
    dict(exposure_weight=1.0, exposure_optimum=0.35, exposure_width=0.35, exposure_weight_function="lorentzian"),
    dict(exposure_weight=0.8, exposure_weight_function="halfsine"),
    dict(exposure_weight=1.0, exposure_weight_function="fullsine", saturation_weight=0.5),
    dict(exposure_weight=1.0, exposure_weight_function="bisquare"),
    dict(exposure_weight=0.0, contrast_weight=0.5, contrast_window_size=3),
    dict(exposure_weight=1.0, contrast_weight=0.5, contrast_window_size=5),
    dict(exposure_weight=0.0, contrast_weight=1.0, contrast_window_size=7),
    dict(exposure_weight=0.0, entropy_weight=0.3, entropy_window_size=3),
    dict(exposure_weight=1.0, entropy_weight=0.3, entropy_window_size=5),
    dict(exposure_weight=0.0, entropy_weight=1.0, entropy_window_size=7),
    dict(exposure_weight=1.0, saturation_weight=0.2, contrast_weight=0.5, entropy_weight=0.3, entropy_window_size=5),
    dict(exposure_weight=1.0, gray_projector="value", contrast_weight=0.3),
    dict(exposure_weight=1.0, gray_projector="anti-value", contrast_weight=0.3),
    dict(exposure_weight=1.0, gray_projector="lightness", contrast_weight=0.3),
    dict(exposure_weight=1.0, gray_projector="luminance", contrast_weight=0.3),
    dict(exposure_weight=1.0, gray_projector="channel-mixer:0.375:0.5:0.125", contrast_weight=0.3),
    dict(exposure_weight=1.0, exposure_cutoff=((10.0, True), (90.0, True))),
    dict(exposure_weight=1.0, exposure_cutoff=((40.0, False), (100.0, True))),
    dict(exposure_weight=1.0, exposure_cutoff=((0.0, True), (95.0, True)),
         exposure_cutoff_projectors=("lightness", "luminance")),
    dict(exposure_weight=1.0, exposure_cutoff=((12.5, True), (87.5, True)),
         exposure_cutoff_projectors=("average", "average"), saturation_weight=0.2),
    dict(exposure_weight=0.0, entropy_weight=0.3, entropy_window_size=5, entropy_cutoff=((10.0, True), (90.0, True))),
    dict(exposure_weight=0.0, entropy_weight=0.3, entropy_window_size=3, entropy_cutoff=((0.0, True), (-10.0, True))),
    dict(exposure_weight=1.0, entropy_weight=0.3, entropy_window_size=5, entropy_cutoff=((30.0, False), (100.0, True))),
]

# float images: absolute cutoffs (a percentage of the float maximum is no
# useful limit for images in [0, 1])
MASK_CASES_F = [c for c in MASK_CASES if "exposure_cutoff" not in c and "entropy_cutoff" not in c] + [
    dict(exposure_weight=1.0, exposure_cutoff=((0.2, False), (0.8, False))),
    dict(exposure_weight=1.0, exposure_cutoff=((0.1, False), (100.0, True)),
         exposure_cutoff_projectors=("lightness", "luminance")),
    dict(exposure_weight=0.0, entropy_weight=0.3, entropy_window_size=5, entropy_cutoff=((0.2, False), (0.8, False))),
]

# enfuseMain cases: (sample type, samples a pixel, K, options, run options)
MAIN_CASES = [
    ("u8", 3, 3, dict(exposure_weight=1.0, saturation_weight=0.2), {}),
    ("u8", 3, 3, dict(exposure_weight=1.0, saturation_weight=0.2, contrast_weight=0.5, entropy_weight=0.3,
                      entropy_window_size=5), {}),
    ("u8", 4, 3, dict(exposure_weight=1.0, saturation_weight=0.2, contrast_weight=0.5), {}),
    ("u8", 1, 3, dict(exposure_weight=1.0, contrast_weight=0.5), {}),
    ("u8", 3, 3, dict(exposure_weight=1.0, saturation_weight=0.2, hard_mask=True), {}),
    ("u8", 3, 3, dict(exposure_weight=1.0, saturation_weight=0.2), dict(wrap=True)),
    ("u8", 3, 4, dict(exposure_weight=0.0, contrast_weight=0.5), {}),
    ("u8", 3, 3, dict(exposure_weight=1.0, exposure_cutoff=((10.0, True), (90.0, True))), {}),
    ("u16", 3, 3, dict(exposure_weight=1.0, saturation_weight=0.2), {}),
    ("u16", 3, 3, dict(exposure_weight=1.0, saturation_weight=0.2, contrast_weight=0.5, entropy_weight=0.3,
                       entropy_window_size=5), {}),
    ("u16", 4, 3, dict(exposure_weight=1.0, saturation_weight=0.2, contrast_weight=0.5), {}),
    ("u16", 1, 3, dict(exposure_weight=1.0, contrast_weight=0.5), {}),
    ("u16", 3, 3, dict(exposure_weight=1.0, saturation_weight=0.2, hard_mask=True), dict(wrap=True)),
    ("u16", 3, 3, dict(exposure_weight=1.0), dict(levels=3)),
    ("u16", 3, 3, dict(exposure_weight=1.0), dict(load=True)),
    ("u16", 3, 9, dict(exposure_weight=1.0, saturation_weight=0.2, contrast_weight=0.5, entropy_weight=0.3,
                       entropy_window_size=5), {}),
    ("f32", 3, 3, dict(exposure_weight=1.0, saturation_weight=0.2), {}),
    ("f32", 4, 3, dict(exposure_weight=1.0, saturation_weight=0.2, contrast_weight=0.5), {}),
    ("f32", 3, 3, dict(exposure_weight=1.0, saturation_weight=0.2, hard_mask=True), dict(wrap=True)),
]

_NP = {"u8": np.uint8, "u16": np.uint16, "f32": np.float32}


def main_inputs(dt, S, K, seed, h=37, w=53):
    """K exposures of the synthetic scene (RGBA: some pixels transparent after
    the import threshold; gray: the green samples)."""
    dtype = _NP[dt]
    imgs = synthetic.exposure_stack(h, w, list(np.linspace(-2.0, 2.0, K)), dtype, 8.0, seed=seed)
    if S == 4:
        rng = np.random.default_rng(seed)
        top = np.iinfo(dtype).max if dtype != np.float32 else 1.0
        low = top // 3 if dtype != np.float32 else 0.2
        imgs = [np.concatenate([x, np.full((h, w, 1), top, dtype)], axis=2) for x in imgs]
        for i, x in enumerate(imgs):
            x[rng.random((h, w)) < 0.1, 3] = low
            x[5 + i:12 + i, 7:20, 3] = 0
    if S == 1:
        imgs = [np.ascontiguousarray(x[..., 1]) for x in imgs]
    return imgs


def enfuse_cases() -> None:
    """enfuse: the reference's enfuseMask weights and enfuseMain results."""
    data = {}
    rng = np.random.default_rng(20261205)
    k = 0
    j = 0
    for dt in ("u8", "u16", "f32"):
        for C in (3, 1):
            img = synthetic.exposure_stack(33, 47, [0.7], _NP[dt], 8.0, seed=11 + j)[0]
            if C == 1:
                img = np.ascontiguousarray(img[..., 1])
            alpha = (rng.random((33, 47)) < 0.85).astype(np.uint8) * 255
            alpha[4:9, 10:18] = 0
            data[f"maskimg{j}_image"] = img
            data[f"maskimg{j}_alpha"] = alpha
            for opts in (MASK_CASES_F if dt == "f32" else MASK_CASES):
                if C == 1 and opts.get("gray_projector", "").startswith("channel"):
                    continue
                data[f"mask{k}_img"] = np.array(j)
                data[f"mask{k}_opts"] = np.array(json.dumps(opts))
                data[f"mask{k}_weight"] = ref.enfuse_mask(img, alpha, ref.enfuse_params(**opts))
                k += 1
            j += 1
    data["mask_count"] = np.array(k)
    k = 0
    for dt, S, K, opts, run in MAIN_CASES:
        imgs = main_inputs(dt, S, K, seed=40 + k)
        masks = None
        if run.get("load"):
            mr = np.random.default_rng(70 + k)
            masks = [(mr.random(imgs[0].shape[:2]) * 3).astype(np.float32) for _ in range(K)]
            for m in masks:
                m[:4, :] = 0.0     # all-zero weights: the integer 255/K fallback
        levels, wrap = run.get("levels", 0), run.get("wrap", False)
        prm = ref.enfuse_params(**opts)
        for i, x in enumerate(imgs):
            data[f"main{k}_image{i}"] = x
        if masks is not None:
            for i, m in enumerate(masks):
                data[f"main{k}_mask{i}"] = m
        data[f"main{k}_meta"] = np.array([K, levels, int(wrap), int(masks is not None)], np.int32)
        data[f"main{k}_opts"] = np.array(json.dumps(opts))
        draws = (0, 0xFFFFFFFF) if dt != "f32" else (-1,)
        for j, d in enumerate(draws):
            r = ref.enfuse_main(imgs, prm, levels=levels, wrap=wrap, masks=masks, dither=d,
                                save_masks=masks is None)
            data[f"main{k}_out{j}"] = r["out"]
            if j == 0:
                data[f"main{k}_alpha"] = r["alpha"]
                if r["masks"] is not None:
                    data[f"main{k}_saved_masks"] = r["masks"]
        k += 1
    data["main_count"] = np.array(k)
    np.savez_compressed(OUT_ENFUSE, **data)
    print(f"wrote {OUT_ENFUSE} ({OUT_ENFUSE.stat().st_size} bytes)")


def float_cases() -> None:
    """Float images: the reference's double pyramids (reduce, expand, enblend)."""
    rng = np.random.default_rng(20261204)
    data = {}
    k = 0
    for (h, w, off) in [(24, 36, 20), (41, 57, 33)]:
        for wrap in (False, True):
            white, black, mask = synthetic.panorama_pair(h, w, off, np.float32, seed=300 + k)
            mask[: h // 3, off + 2: off + 9] = 128
            wa, ba = orc.alpha_of(white).copy(), orc.alpha_of(black)
            wa[3:7, off + 3: off + 11] = 0
            W, B = np.ascontiguousarray(white[..., :3]), np.ascontiguousarray(black[..., :3])
            W[0, 0] = -0.25  # negative samples take the rational branch of the mapping
            levels = orc.num_levels(w, h)
            l0, out = ref.enblend_f(W, wa, B, ba, mask, levels, wrap)
            for name, a in (("white", W), ("white_alpha", wa), ("black", B), ("black_alpha", ba),
                            ("mask", mask), ("level0", l0), ("out", out)):
                data[f"fenblend{k}_{name}"] = a
            data[f"fenblend{k}_meta"] = np.array([levels, int(wrap)], np.int32)
            k += 1
    data["fenblend_count"] = np.array(k)
    k = 0
    for C in (1, 3):
        for wrap in (False, True):
            h, w = int(rng.integers(5, 23)), int(rng.integers(5, 23))
            src = rng.random((h, w, C)) * 2.0 + 0.5
            alpha = np.where(rng.random((h, w)) < 0.8, 255, 0).astype(np.uint8)
            d, da = ref.reduce_f(src, alpha, wrap)
            coarse = rng.random(((h + 1) >> 1, (w + 1) >> 1, C)) - 0.5
            fine = rng.random((h, w, C)) * 2.0
            for name, a in (("src", src), ("alpha", alpha), ("dst", d), ("dst_alpha", da), ("coarse", coarse),
                            ("fine", fine), ("sub", ref.expand_f(coarse, fine, False, wrap)),
                            ("add", ref.expand_f(coarse, fine, True, wrap))):
                data[f"fstep{k}_{name}"] = a
            data[f"fstep{k}_meta"] = np.array([int(wrap)], np.int32)
            k += 1
    data["fstep_count"] = np.array(k)
    np.savez_compressed(OUT_FLOAT, **data)
    print(f"wrote {OUT_FLOAT} ({OUT_FLOAT.stat().st_size} bytes)")


def nft_footprints(h: int, w: int, kind: int, rng) -> tuple:
    """Alpha footprints of an image pair: overlapping strips, discs, noise
    with holes (kind 0, 1, 2)."""
    wa = np.zeros((h, w), np.uint8)
    ba = np.zeros((h, w), np.uint8)
    if kind == 0:
        a = int(rng.integers(w // 3, w - 2))
        b = int(rng.integers(1, a))
        wa[:, :a] = 255
        ba[:, b:] = 255
        wa[int(rng.integers(0, h)), :a // 2] = 0
    elif kind == 1:
        yy, xx = np.mgrid[:h, :w]
        for img in (wa, ba):
            for _ in range(3):
                cy, cx, r = rng.integers(0, h), rng.integers(0, w), rng.integers(4, max(5, min(h, w)))
                img[(yy - cy) ** 2 + (xx - cx) ** 2 < r * r] = 255
    else:
        wa[rng.random((h, w)) < 0.55] = 255
        ba[rng.random((h, w)) < 0.55] = 255
    return wa, ba


def nft_cases() -> None:
    """enblend's nearest-feature seam masks (src/nearest.h) of seeded
    footprints, open and periodic, including pairs the reference rejects."""
    rng = np.random.default_rng(20261204)
    data = {}
    k = 0
    for (h, w) in [(9, 9), (24, 40), (37, 61), (64, 48), (80, 130), (120, 200)]:
        for kind in (0, 1, 2):
            for wrap in (False, True):
                wa, ba = nft_footprints(h, w, kind, rng)
                m = ref.nft_mask(wa, ba, wrap)
                data[f"nft{k}_white"] = wa
                data[f"nft{k}_black"] = ba
                data[f"nft{k}_wrap"] = np.array(int(wrap))
                data[f"nft{k}_mask"] = m if m is not None else np.zeros((0, 0), np.uint8)
                k += 1
    # nearly complete overlap: rejected
    wa = np.full((30, 40), 255, np.uint8)
    ba = wa.copy()
    ba[0, 0] = 0
    data[f"nft{k}_white"], data[f"nft{k}_black"], data[f"nft{k}_wrap"] = wa, ba, np.array(0)
    m = ref.nft_mask(wa, ba, False)
    data[f"nft{k}_mask"] = m if m is not None else np.zeros((0, 0), np.uint8)
    k += 1
    data["nft_count"] = np.array(k)
    np.savez_compressed(OUT_NFT, **data)
    print(f"wrote {OUT_NFT} ({OUT_NFT.stat().st_size} bytes)")


def main() -> None:
    if ref.lib() is None:
        raise SystemExit("the reference tree is not available here")
    rng = np.random.default_rng(20261203)
    data = {}
    # enblend pyramid blend: mask GP, white/black LP with alpha, blend, collapse
    k = 0
    for dt in (np.uint8, np.uint16):
        for (h, w, off) in [(21, 30, 17), (40, 64, 40), (48, 80, 44)]:
            for wrap in (False, True):
                white, black, mask = synthetic.panorama_pair(h, w, off, dt, seed=100 + k)
                mask[: h // 3, off + 2: off + 9] = 128
                wa, ba = orc.alpha_of(white).copy(), orc.alpha_of(black)
                wa[3:7, off + 3: off + 11] = 0
                W, B = np.ascontiguousarray(white[..., :3]), np.ascontiguousarray(black[..., :3])
                levels = orc.num_levels(W.shape[1], W.shape[0])
                l0 = ref.enblend_level0(W, wa, B, ba, mask, levels, wrap)
                for name, a in (("white", W), ("white_alpha", wa), ("black", B), ("black_alpha", ba),
                                ("mask", mask), ("level0", l0)):
                    data[f"enblend{k}_{name}"] = a
                data[f"enblend{k}_meta"] = np.array([levels, int(wrap)], np.int32)
                k += 1
    data["enblend_count"] = np.array(k)
    # single reduce / expand steps on random levels (source width >= 2)
    k = 0
    for bits in (8, 16):
        for C in (1, 3):
            for wrap in (False, True):
                for alpha_on in ((True,) if C == 3 else (False, True)):
                    h, w = int(rng.integers(5, 23)), int(rng.integers(5, 23))
                    maxv = 255 if bits == 8 else 65535
                    src = (rng.integers(0, maxv + 1, size=(h, w, C)) << 7).astype(np.int32)
                    alpha = np.where(rng.random((h, w)) < 0.8, 255, 0).astype(np.uint8) if alpha_on else None
                    r = ref.reduce(src, alpha, bits, wrap)
                    data[f"reduce{k}_src"] = src
                    data[f"reduce{k}_meta"] = np.array([bits, int(wrap), int(alpha_on)], np.int32)
                    if alpha_on:
                        data[f"reduce{k}_alpha"] = alpha
                        data[f"reduce{k}_dst"], data[f"reduce{k}_dst_alpha"] = r
                    else:
                        data[f"reduce{k}_dst"] = r
                    lim = 1 << (14 if bits == 8 else 22)
                    coarse = rng.integers(-lim, lim, size=((h + 1) >> 1, (w + 1) >> 1, C)).astype(np.int32)
                    fine = rng.integers(-lim, lim, size=(h, w, C)).astype(np.int32)
                    data[f"expand{k}_src"] = coarse
                    data[f"expand{k}_dst"] = fine
                    data[f"expand{k}_sub"] = ref.expand(coarse, fine, False, bits, wrap)
                    data[f"expand{k}_add"] = ref.expand(coarse, fine, True, bits, wrap)
                    k += 1
    data["step_count"] = np.array(k)
    # output conversion with the reference's dither draws
    for bits, dt in ((8, np.uint8), (16, np.uint16)):
        maxv = 255 if bits == 8 else 65535
        l0 = rng.integers(-3000, min((maxv + 3) << 7, 32768 if bits == 8 else 1 << 30),
                          size=(24, 32, 3)).astype(np.int32)
        alpha = np.where(rng.random((24, 32)) < 0.9, 255, 0).astype(np.uint8)
        data[f"convert{bits}_level0"] = l0
        data[f"convert{bits}_alpha"] = alpha
        data[f"convert{bits}_out"] = ref.from_pyramid(l0, alpha, dt, fill=7)
    np.savez_compressed(OUT, **data)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes)")
    float_cases()
    enfuse_cases()
    nft_cases()


if __name__ == "__main__":
    if "--nft-only" in sys.argv:
        if ref.lib() is None:
            raise SystemExit("the reference tree is not available here")
        nft_cases()
        raise SystemExit(0)
    if "--enfuse-only" in sys.argv:
        if ref.lib() is None:
            raise SystemExit("the reference tree is not available here")
        enfuse_cases()
    else:
        main()
