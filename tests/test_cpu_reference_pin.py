"""The C oracle against the reference's own code.

tests/golden/reference_pyramid.npz holds outputs of the reference's
pyramid.h / blend.h / fixmath.h (compiled unmodified against the project's
VIGRA/GSL/LCMS2 shims by oracle/reference_build.py; regenerate with
tests/golden/make_golden.py).  The golden tests run everywhere; the live tests
also compare random cases when the reference tree is present.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import reference_build as ref

GOLDEN = np.load(Path(__file__).resolve().parent / "golden" / "reference_pyramid.npz")


def _pbits(bits):
    return 16 if bits == 8 else 32


@pytest.mark.parametrize("k", range(int(GOLDEN["enblend_count"])))
def test_golden_enblend_level0(orc, k):
    """mask GP + white/black LP with alpha holes + blend (incl. mask 128) + collapse."""
    g = {n: GOLDEN[f"enblend{k}_{n}"] for n in ("white", "white_alpha", "black", "black_alpha", "mask", "level0")}
    levels, wrap = (int(v) for v in GOLDEN[f"enblend{k}_meta"])
    res = orc.enblend(g["white"], g["black"], g["mask"], white_alpha=g["white_alpha"],
                      black_alpha=g["black_alpha"], levels=levels, wrap=bool(wrap), want_level0=True)
    assert np.array_equal(res["level0"], g["level0"])


@pytest.mark.parametrize("k", range(int(GOLDEN["step_count"])))
def test_golden_reduce_expand(orc, k):
    bits, wrap, alpha_on = (int(v) for v in GOLDEN[f"reduce{k}_meta"])
    src = GOLDEN[f"reduce{k}_src"]
    if alpha_on:
        dst, da = orc.reduce(src, GOLDEN[f"reduce{k}_alpha"], _pbits(bits), bool(wrap))
        assert np.array_equal(da, GOLDEN[f"reduce{k}_dst_alpha"])
    else:
        dst = orc.reduce(src, None, _pbits(bits), bool(wrap))
    assert np.array_equal(dst, GOLDEN[f"reduce{k}_dst"])
    coarse, fine = GOLDEN[f"expand{k}_src"], GOLDEN[f"expand{k}_dst"]
    assert np.array_equal(orc.expand(coarse, fine, False, _pbits(bits), bool(wrap)), GOLDEN[f"expand{k}_sub"])
    assert np.array_equal(orc.expand(coarse, fine, True, _pbits(bits), bool(wrap)), GOLDEN[f"expand{k}_add"])


@pytest.mark.parametrize("bits", [8, 16])
def test_golden_conversion_rule(orc, bits):
    """copyFromPyramidImageIf: outside the dither band the result is fixed
    (q for f < 1/4, q+1 for f >= 3/4, clamped) and must equal the oracle's;
    inside it the reference's draw picks q or q+1; alpha-0 pixels untouched."""
    l0, alpha, out = (GOLDEN[f"convert{bits}_{n}"] for n in ("level0", "alpha", "out"))
    dt = np.uint8 if bits == 8 else np.uint16
    maxv = 255 if bits == 8 else 65535
    q, f = l0 >> 7, l0 & 127
    band = (f >= 32) & (f < 96)
    lo, hi = np.clip(q, 0, maxv), np.clip(q + 1, 0, maxv)
    on = np.broadcast_to(alpha[..., None] != 0, l0.shape)
    assert np.all(out[~on] == 7)
    ours = orc.from_fixed(l0, alpha, dt, frac=7, dither="hash", seed=11)
    assert np.array_equal(out[on & ~band], ours[on & ~band])
    inb = out[on & band].astype(np.int64)
    assert np.all((inb == lo[on & band]) | (inb == hi[on & band]))
    ours_b = ours[on & band].astype(np.int64)
    assert np.all((ours_b == lo[on & band]) | (ours_b == hi[on & band]))


live = pytest.mark.skipif(not ref.available(), reason="reference tree not present")


@live
@pytest.mark.parametrize("seed", range(6))
def test_live_reduce_expand(orc, seed):
    rng = np.random.default_rng(seed)
    for _ in range(12):
        bits = int(rng.choice([8, 16]))
        C = int(rng.choice([1, 3]))
        wrap = bool(rng.integers(2))
        h, w = int(rng.integers(2, 40)), int(rng.integers(4, 40))
        maxv = 255 if bits == 8 else 65535
        src = (rng.integers(0, maxv + 1, size=(h, w, C)) << 7).astype(np.int32)
        alpha = np.where(rng.random((h, w)) < 0.8, 255, 0).astype(np.uint8) if (C == 3 or rng.random() < 0.5) else None
        r = ref.reduce(src, alpha, bits, wrap)
        o = orc.reduce(src, alpha, _pbits(bits), wrap)
        if alpha is None:
            assert np.array_equal(o, r)
        else:
            assert np.array_equal(o[0], r[0]) and np.array_equal(o[1], r[1])
        # expand from a source at least 2 wide (the reference's expand reads
        # uninitialised state for one-column sources, which roiBounds never
        # lets a pyramid reach)
        lim = 1 << (14 if bits == 8 else 22)
        coarse = rng.integers(-lim, lim, size=((h + 1) >> 1, (w + 1) >> 1, C)).astype(np.int32)
        fine = rng.integers(-lim, lim, size=(h, w, C)).astype(np.int32)
        for add in (False, True):
            assert np.array_equal(orc.expand(coarse, fine, add, _pbits(bits), wrap),
                                  ref.expand(coarse, fine, add, bits, wrap))


@live
@pytest.mark.parametrize("dt", [np.uint8, np.uint16])
@pytest.mark.parametrize("wrap", [False, True])
def test_live_enblend(orc, dt, wrap):
    from enbgpu import synthetic
    for (h, w, off) in [(90, 120, 80), (33, 50, 20)]:
        white, black, mask = synthetic.panorama_pair(h, w, off, dt, seed=7)
        mask[: h // 2, off + 1: off + 6] = 200
        wa, ba = orc.alpha_of(white), orc.alpha_of(black)
        W, B = np.ascontiguousarray(white[..., :3]), np.ascontiguousarray(black[..., :3])
        levels = orc.num_levels(W.shape[1], W.shape[0])
        want = ref.enblend_level0(W, wa, B, ba, mask, levels, wrap)
        got = orc.enblend(W, B, mask, white_alpha=wa, black_alpha=ba, wrap=wrap, want_level0=True)["level0"]
        assert np.array_equal(got, want)


# ---- float images: the reference's double pyramids ------------------------

GOLDEN_F = np.load(Path(__file__).resolve().parent / "golden" / "reference_float.npz")


@pytest.mark.parametrize("k", range(int(GOLDEN_F["fenblend_count"])))
def test_golden_float_enblend(orc, k):
    """Float enblend: double level 0 to 1e-13 relative (summation order), output pixels identical."""
    g = {n: GOLDEN_F[f"fenblend{k}_{n}"]
         for n in ("white", "white_alpha", "black", "black_alpha", "mask", "level0", "out")}
    levels, wrap = (int(v) for v in GOLDEN_F[f"fenblend{k}_meta"])
    res = orc.enblend_f(g["white"], g["black"], g["mask"], white_alpha=g["white_alpha"],
                        black_alpha=g["black_alpha"], levels=levels, wrap=bool(wrap), want_level0=True)
    assert np.allclose(res["level0"], g["level0"], rtol=1e-13, atol=1e-13)
    assert np.array_equal(res["out"], g["out"])


@pytest.mark.parametrize("k", range(int(GOLDEN_F["fstep_count"])))
def test_golden_float_reduce_expand(orc, k):
    (wrap,) = (bool(v) for v in GOLDEN_F[f"fstep{k}_meta"])
    d, da = orc.reduce_d(GOLDEN_F[f"fstep{k}_src"], GOLDEN_F[f"fstep{k}_alpha"], wrap)
    assert np.array_equal(da, GOLDEN_F[f"fstep{k}_dst_alpha"])
    assert np.allclose(d, GOLDEN_F[f"fstep{k}_dst"], rtol=1e-14, atol=1e-14)
    coarse, fine = GOLDEN_F[f"fstep{k}_coarse"], GOLDEN_F[f"fstep{k}_fine"]
    assert np.allclose(orc.expand_d(coarse, fine, False, wrap), GOLDEN_F[f"fstep{k}_sub"], rtol=1e-14, atol=1e-14)
    assert np.allclose(orc.expand_d(coarse, fine, True, wrap), GOLDEN_F[f"fstep{k}_add"], rtol=1e-14, atol=1e-14)


@live
@pytest.mark.parametrize("wrap", [False, True])
def test_live_float_enblend(orc, wrap):
    from enbgpu import synthetic
    for (h, w, off) in [(60, 90, 50), (31, 45, 24)]:
        white, black, mask = synthetic.panorama_pair(h, w, off, np.float32, seed=17)
        mask[: h // 2, off + 1: off + 6] = 200
        wa, ba = orc.alpha_of(white), orc.alpha_of(black)
        W, B = np.ascontiguousarray(white[..., :3]), np.ascontiguousarray(black[..., :3])
        W[1, 1], B[2, 2] = -0.5, 1.75
        levels = orc.num_levels(W.shape[1], W.shape[0])
        l0, out = ref.enblend_f(W, wa, B, ba, mask, levels, wrap)
        got = orc.enblend_f(W, B, mask, white_alpha=wa, black_alpha=ba, wrap=wrap, want_level0=True)
        assert np.allclose(got["level0"], l0, rtol=1e-13, atol=1e-13)
        assert np.array_equal(got["out"], out)


# ---- enfuse: the reference's enfuseMask and enfuseMain --------------------------------

import json  # noqa: E402

EGOLDEN = np.load(Path(__file__).resolve().parent / "golden" / "reference_enfuse.npz")
_DT = {np.dtype(np.uint8): "u8", np.dtype(np.uint16): "u16", np.dtype(np.float32): "f32"}


def _mask_case(k):
    j = int(EGOLDEN[f"mask{k}_img"])
    return (EGOLDEN[f"maskimg{j}_image"], EGOLDEN[f"maskimg{j}_alpha"], json.loads(str(EGOLDEN[f"mask{k}_opts"])),
            EGOLDEN[f"mask{k}_weight"])


@pytest.mark.parametrize("k", range(int(EGOLDEN["mask_count"])))
def test_golden_enfuse_mask(orc, k):
    """enfuseMask (src/enfuse.h:962-1212): exposure functions, gray projectors,
    saturation, contrast and entropy windows, exposure and entropy cutoffs, on
    u8/u16/float RGB and gray images with alpha holes.  Integer images: the
    oracle's weights equal the reference's bit for bit.  Float images: equal
    too when the oracle forms the contrast windows with the reference's float
    running sums (NaN where the reference's float variance goes negative)."""
    img, alpha, opts, want = _mask_case(k)
    if img.dtype == np.float32:
        got = orc.enfuse_mask_f(img, alpha, orc.params_from_options(opts, float_sliding_sums=True))
        assert np.array_equal(got, want, equal_nan=True)
    else:
        got = orc.enfuse_mask(img, alpha, orc.params_from_options(opts))
        assert np.array_equal(got, want)


def _main_case(k):
    K, levels, wrap, load = (int(v) for v in EGOLDEN[f"main{k}_meta"])
    imgs = [EGOLDEN[f"main{k}_image{i}"] for i in range(K)]
    masks = [EGOLDEN[f"main{k}_mask{i}"] for i in range(K)] if load else None
    return imgs, masks, levels, bool(wrap), json.loads(str(EGOLDEN[f"main{k}_opts"]))


@pytest.mark.parametrize("k", range(int(EGOLDEN["main_count"])))
def test_golden_enfuse_main(orc, k):
    """enfuseMain (src/enfuse.h:1217-1617) end to end: import with the alpha
    threshold, weights or --load-masks, normalisation (integer 255/K where all
    weights are 0), hard mask, Laplacian and mask pyramids, merge, collapse and
    the dithered output.  Integer images: the reference ran with every dither
    draw returning 0 and with every draw returning 0xffffffff; the oracle's
    collapsed level 0, converted under the same draws, gives the same pixels
    both times (which fixes whether each fraction reaches 1/4 and 3/4).  Float
    images: the output pixels are equal.  The masks the reference saved
    (--save-masks) equal the oracle's weights (hard mask: the hard masks)."""
    imgs, masks, levels, wrap, opts = _main_case(k)
    hard = bool(opts.get("hard_mask", False))
    if imgs[0].dtype == np.float32:
        res = orc.enfuse_f(imgs, None, orc.params_from_options(opts, float_sliding_sums=True), masks=masks,
                           levels=levels, wrap=wrap, hard_mask=hard, want_masks=True)
        C = 3 if imgs[0].ndim == 3 else 1
        assert np.array_equal(res["out"][..., :C] if imgs[0].ndim == 3 else res["out"], EGOLDEN[f"main{k}_out0"])
    else:
        res = orc.enfuse(imgs, None, orc.params_from_options(opts), masks=masks, levels=levels, wrap=wrap,
                         hard_mask=hard, want_level0=True, want_masks=True)
        l0 = res["level0"] if imgs[0].ndim == 3 else res["level0"][..., 0]
        for j, draw in enumerate((0, 0xFFFFFFFF)):
            assert np.array_equal(orc.convert_with_draw(l0, res["alpha"], imgs[0].dtype, draw),
                                  EGOLDEN[f"main{k}_out{j}"]), draw
    assert np.array_equal((res["alpha"] != 0).astype(np.uint8), EGOLDEN[f"main{k}_alpha"])
    if f"main{k}_saved_masks" in EGOLDEN:
        saved = EGOLDEN[f"main{k}_saved_masks"]
        if hard:
            assert np.array_equal(res["masks"], saved)
        else:
            for i, x in enumerate(imgs):
                a = orc.alpha_of(x)
                if x.dtype == np.float32:
                    w = orc.enfuse_mask_f(x, a, orc.params_from_options(opts, float_sliding_sums=True))
                else:
                    w = orc.enfuse_mask(x, a, orc.params_from_options(opts))
                assert np.array_equal(w, saved[i], equal_nan=True), i


@pytest.mark.skipif(not ref.available(), reason="the reference tree is not present")
@pytest.mark.parametrize("seed", range(4))
def test_live_enfuse_against_reference(orc, seed):
    """Random weighting options and images: oracle == reference (enfuseMask
    and enfuseMain under both constant dither draws)."""
    from enbgpu import synthetic
    rng = np.random.default_rng(1000 + seed)
    dt = [np.uint8, np.uint16][seed % 2]
    h, w, K = int(rng.integers(20, 45)), int(rng.integers(20, 60)), int(rng.integers(2, 6))
    opts = dict(exposure_weight=float(rng.choice([0.0, 1.0])), saturation_weight=float(rng.choice([0.0, 0.2])),
                contrast_weight=float(rng.choice([0.0, 0.5])), entropy_weight=float(rng.choice([0.0, 0.3])),
                contrast_window_size=int(rng.choice([3, 5])), entropy_window_size=int(rng.choice([3, 5])),
                exposure_weight_function=str(rng.choice(["gaussian", "lorentzian", "bisquare"])))
    if sum(opts[k] for k in ("exposure_weight", "saturation_weight", "contrast_weight", "entropy_weight")) == 0:
        opts["exposure_weight"] = 1.0
    imgs = synthetic.exposure_stack(h, w, list(np.linspace(-2, 2, K)), dt, 8.0, seed=seed)
    for x in imgs:
        assert np.array_equal(orc.enfuse_mask(x, None, orc.params_from_options(opts)),
                              ref.enfuse_mask(x, orc.alpha_of(x), ref.enfuse_params(**opts)))
    res = orc.enfuse(imgs, None, orc.params_from_options(opts), want_level0=True)
    for draw in (0, 0xFFFFFFFF):
        r = ref.enfuse_main(imgs, ref.enfuse_params(**opts), dither=draw)
        assert np.array_equal(orc.convert_with_draw(res["level0"], res["alpha"], dt, draw), r["out"])


# ---- enblend: the reference's nearest-feature seam mask ------------------------------

NGOLDEN = np.load(Path(__file__).resolve().parent / "golden" / "reference_nft.npz")


@pytest.mark.parametrize("k", range(int(NGOLDEN["nft_count"])))
def test_golden_nft_mask(orc, k):
    """nearestFeatureTransform (src/nearest.h:427-553) with the
    Felzenszwalb-Huttenlocher transform of the reference's OpenMP build
    (src/openmp_vigra.h:257-433): open and periodic, strips, discs, noisy
    footprints; a pair with too much overlap is rejected as the reference
    rejects it."""
    wa, ba, wrap = NGOLDEN[f"nft{k}_white"], NGOLDEN[f"nft{k}_black"], bool(int(NGOLDEN[f"nft{k}_wrap"]))
    want = NGOLDEN[f"nft{k}_mask"]
    if want.size == 0:
        with pytest.raises(ValueError):
            orc.nft_mask(wa, ba, wrap)
    else:
        assert np.array_equal(orc.nft_mask(wa, ba, wrap), want)


@pytest.mark.skipif(not ref.available(), reason="the reference tree is not present")
@pytest.mark.parametrize("seed", range(6))
def test_live_nft_mask(orc, seed):
    rng = np.random.default_rng(500 + seed)
    for _ in range(20):
        h, w = int(rng.integers(8, 90)), int(rng.integers(8, 140))
        wa = np.where(rng.random((h, w)) < rng.uniform(0.3, 0.9), 255, 0).astype(np.uint8)
        ba = np.where(rng.random((h, w)) < rng.uniform(0.3, 0.9), 255, 0).astype(np.uint8)
        wrap = bool(rng.integers(2))
        want = ref.nft_mask(wa, ba, wrap)
        if want is None:
            with pytest.raises(ValueError):
                orc.nft_mask(wa, ba, wrap)
        else:
            assert np.array_equal(orc.nft_mask(wa, ba, wrap), want)
