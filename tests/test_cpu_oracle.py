"""Known-answer and property checks of the CPU oracle (no GPU)."""
import numpy as np
import pytest


def test_reduce_of_constant_is_constant(orc):
    for (h, w) in [(2, 2), (3, 5), (17, 9), (64, 33)]:
        for wrap in (False, True):
            src = np.full((h, w, 3), 12345, np.int32)
            a = np.full((h, w), 255, np.uint8)
            d, da = orc.reduce(src, a, 32, wrap)
            assert (d == 12345).all() and (da == 255).all()
            assert (orc.reduce(src, None, 32, wrap) == 12345).all()


def test_reduce_alpha_excludes_transparent_taps(orc):
    src = np.zeros((5, 5, 1), np.int32)
    src[..., 0] = np.arange(25).reshape(5, 5) * 100
    a = np.zeros((5, 5), np.uint8)
    a[2, 2] = 255
    d, da = orc.reduce(src, a, 32)
    # only the centre tap is opaque: output (1,1) equals it, others transparent
    assert d[1, 1, 0] == 1200 and da[1, 1] == 255
    assert da[0, 0] == 255 and d[0, 0, 0] == 1200  # centre (2,2) is in the 5x5 window of (0,0)
    a[:] = 0
    d, da = orc.reduce(src, a, 32)
    assert (da == 0).all() and (d == 0).all()


def test_reduce_truncates_toward_zero(orc):
    src = np.full((4, 4, 1), -7, np.int32)
    src[0, 0, 0] = -8
    a = np.full((4, 4), 255, np.uint8)
    d, _ = orc.reduce(src, a, 32)
    # weighted mean slightly below -7 truncates to -7 (C division), never floors to -8
    assert d[0, 0, 0] == -7


def test_expand_of_constant_reconstructs_constant(orc):
    for (h, w) in [(1, 2), (2, 2), (3, 3), (5, 8), (9, 17)]:
        sh, sw = (h + 1) >> 1, (w + 1) >> 1
        src = np.full((sh, sw, 1), 640, np.int32)
        dst = np.zeros((h, w, 1), np.int32)
        assert (orc.expand(src, dst, True, 32, False) == 640).all()
        if sw > 1:
            assert (orc.expand(src, dst, True, 32, True) == 640).all()


def test_expand_single_source_column_wrap_quirk(orc):
    # With wrap-around and a one-column source the reference's SKIPSM keeps
    # the wrapped left state in the numerator over the divisor 6
    # (pyramid.h:1233-1236): even columns come out as 7/6 of the value.
    src = np.full((2, 1, 1), 600, np.int32)
    dst = np.zeros((4, 2, 1), np.int32)
    out = orc.expand(src, dst, True, 32, True)
    assert out[0, 0, 0] == 700 and out[0, 1, 0] == 600


def test_expand_interior_weights(orc):
    # delta at the centre of a 3x3 source -> 5x5 destination
    src = np.zeros((3, 3, 1), np.int32)
    src[1, 1, 0] = 64 * 1000
    dst = np.zeros((5, 5, 1), np.int32)
    out = orc.expand(src, dst, True, 32)[..., 0]
    assert out[2, 2] == 64 * 1000 * 36 // 64           # (6/8)^2
    assert out[2, 3] == 64 * 1000 * 24 // 64           # (6/8)*(4/8)
    assert out[3, 3] == 64 * 1000 * 16 // 64           # (4/8)^2
    assert out[0, 0] == 64 * 1000 * 1 // 49            # corner: (1/7)^2


def test_int16_pyramid_store_semantics(orc):
    src = np.zeros((1, 1, 1), np.int32)
    src[0, 0, 0] = 30000
    dst = np.full((2, 2, 1), 30000, np.int32)
    assert (orc.expand(src, dst, True, 16) == 32767).all()      # fromPromote saturates
    dst = np.full((2, 2, 1), -30000, np.int32)
    assert (orc.expand(src, dst, False, 16) == 5536).all()      # static_cast wraps


def test_mask_multiply_rounding(orc):
    D = 255 << 15
    lp = np.array([[[3], [-3], [5], [-5], [7]]], np.int32)
    m = np.array([[D // 2, D // 2, D, 0, D // 4]], np.int32)
    out = orc.mask_multiply(lp, m, D, 32)[0, :, 0]
    # 1.5 -> 2, -1.5 -> -2 (half away from zero), x1 and x0 exact, 1.75 -> 2
    assert list(out) == [2, -2, 5, 0, 2]


def test_blend_coefficients(orc):
    W = 255 << 15
    white = np.array([[[100], [100], [100], [101]]], np.int32)
    black = np.array([[[0], [0], [0], [0]]], np.int32)
    mask = np.array([[W, 0, W // 2, W // 2]], np.int32)
    out = orc.blend(mask, white, black, W, 32)[0, :, 0]
    assert list(out) == [100, 0, 50, 51]


def test_from_fixed_rule(orc):
    frac = 7
    v = np.array([[[0], [31], [32], [64], [95], [96], [127], [-1], [40000]]], np.int32)
    a = np.full((1, 9), 255, np.uint8)
    near = orc.from_fixed(v, a, np.uint8, frac, "nearest")[0, :, 0]
    assert list(near) == [0, 0, 0, 1, 1, 1, 1, 0, 255]
    for seed in range(20):
        d = orc.from_fixed(v, a, np.uint8, frac, "hash", seed=seed)[0, :, 0]
        assert d[0] == 0 and d[1] == 0 and d[5] == 1 and d[6] == 1   # outside [1/4, 3/4)
        assert d[2] in (0, 1) and d[3] in (0, 1) and d[4] in (0, 1)
        assert d[7] == 0 and d[8] == 255


def test_enfuse_zero_weights_use_integer_fallback(orc):
    img = np.full((20, 24, 3), 128, np.uint8)
    masks = [np.zeros((20, 24), np.float32) for _ in range(9)]
    r = orc.enfuse([img] * 9, masks=masks, want_masks=True, dither="nearest")
    assert (r["masks"] == 28.0).all()          # 255 / 9 in integer arithmetic
    # each exposure contributes 28/255 of the image: the sum is darker than the input
    assert r["out"].max() < 128


def test_enfuse_identical_exposures_reproduce_input(orc):
    rng = np.random.default_rng(1)
    img = rng.integers(0, 256, (33, 41, 3), dtype=np.uint8)
    r = orc.enfuse([img, img], prm=orc.params(saturation_weight=0.2), dither="nearest", want_level0=True)
    assert np.abs(r["out"].astype(int) - img).max() <= 1
