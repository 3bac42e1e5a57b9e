"""Generate tests/golden/reference_pyramid.npz and reference_float.npz from the reference's own code.

Runs the reference-code oracle (oracle/reference_build.py: the reference's
pyramid.h / blend.h / fixmath.h compiled unmodified against the project's
shims) on small seeded inputs and stores inputs and outputs, so that machines
without the reference tree can check the C oracle and the CUDA path against
the reference's results.  Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

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


if __name__ == "__main__":
    main()
