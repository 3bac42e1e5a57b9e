"""The allocation-free Gaussian pyramid entry point (enb_gaussian_pyramid_noalloc).

Some callers cannot allocate device memory while they run: a host
application that reserves its GPU budget up front in its own pool and forbids
driver allocations inside its processing callbacks, or a fixed-budget
embedded pipeline.  For them the library keeps the reduced alpha planes in a
static device array.  These tests call the entry point through the C ABI and
check every level against the allocating enb_gaussian_pyramid and, for the
fixed-point pyramids, against the oracle's Gaussian pyramid, on two calls in a
row with different images (the scratch keeps the previous call's contents,
which must not leak into the next result).  The cases cover both alpha
branches, U8/U16 pixels, an F32 weight plane into an Int32 9.15 pyramid and
F32 images (one and three channels) into FP32 pyramids.  The file is collected
last, so a failure here never hides another test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

# (height, width, wrap) of the two calls in a row
CALLS = [(301, 517, False), (257, 389, True)]


def _img(rng, h, w, dtype):
    maxv = np.iinfo(dtype).max
    return rng.integers(0, maxv + 1, size=(h, w, 3)).astype(dtype)


def _alpha(rng, h, w):
    a = (rng.random((h, w)) < 0.7).astype(np.uint8) * 255
    a[: h // 3, : w // 4] = 0
    return a


def _oracle_pyramid(orc, level0, alpha, levels, bits, wrap):
    """gaussianPyramid (src/pyramid.h:1468-1636) in the oracle: level 0 given,
    levels 1.. by the reduce with (level 1 from the input alpha, then the
    reduced alpha) or without alpha."""
    out = [level0]
    a = alpha
    for _ in range(1, levels):
        if a is None:
            out.append(orc.reduce(out[-1], None, bits, wrap))
        else:
            nxt, a = orc.reduce(out[-1], a, bits, wrap)
            out.append(nxt)
    return out


def _noalloc(ctx, src_desc, alpha, levels, w, h, C, code, wrap, frac):
    import enbgpu
    got = ctx.pyramid(levels, w, h, C, code)
    a = ctypes.byref(enbgpu.plane_image(alpha)) if alpha is not None else None
    ctx._check(ctx.lib.enb_gaussian_pyramid_noalloc(ctx.handle, int(wrap), ctypes.byref(src_desc), a, frac,
                                                    got.handle))
    ctx.synchronize()
    return got


def _context():
    import enbgpu
    from enbgpu import _build
    _build.build()
    return enbgpu.Context(0)


@pytest.mark.parametrize("with_alpha", [True, False])
@pytest.mark.parametrize("dtype,pdt", [(np.uint8, "i16"), (np.uint16, "i32")])
def test_noalloc_pixels_match_allocating_entry_point_and_oracle(orc, dtype, pdt, with_alpha):
    import enbgpu
    ctx = _context()
    code = enbgpu.ENB_I16 if pdt == "i16" else enbgpu.ENB_I32
    bits = 16 if pdt == "i16" else 32
    rng = np.random.default_rng(7)
    try:
        for call, (h, w, wrap) in enumerate(CALLS):
            levels = enbgpu.num_levels(w, h)
            img_np = _img(rng, h, w, dtype)
            alpha_np = _alpha(rng, h, w) if with_alpha else None
            img = torch.from_numpy(img_np).cuda()
            alpha = torch.from_numpy(alpha_np).cuda() if with_alpha else None
            ref = ctx.gaussian_pyramid(img, levels, alpha=alpha, wrap=wrap, dtype=code)
            got = _noalloc(ctx, enbgpu.pixel_image(img), alpha, levels, w, h, 3, code, wrap, 7)
            want = _oracle_pyramid(orc, orc.to_fixed(img_np, 7), alpha_np, levels, bits, wrap)
            for l in range(levels):
                g = got.read(l)
                assert np.array_equal(g, ref.read(l)), (call, l)
                assert np.array_equal(g.astype(np.int32), np.moveaxis(want[l], 2, 0)), (call, l)
            ref.free()
            got.free()
    finally:
        ctx.close()


@pytest.mark.parametrize("with_alpha", [True, False])
def test_noalloc_weight_plane_into_mask_pyramid(orc, with_alpha):
    """An F32 weight plane into an Int32 9.15 mask pyramid (fromRealPromote(v * 2^15) at level 0)."""
    import enbgpu
    ctx = _context()
    rng = np.random.default_rng(11)
    try:
        for call, (h, w, wrap) in enumerate(CALLS):
            levels = enbgpu.num_levels(w, h)
            m_np = (rng.random((h, w)) * 255.0).astype(np.float32)
            alpha_np = _alpha(rng, h, w) if with_alpha else None
            m = torch.from_numpy(m_np).cuda()
            alpha = torch.from_numpy(alpha_np).cuda() if with_alpha else None
            ref = ctx.gaussian_pyramid(m, levels, alpha=alpha, wrap=wrap, frac_bits=15, dtype=enbgpu.ENB_I32)
            got = _noalloc(ctx, enbgpu.plane_image(m), alpha, levels, w, h, 1, enbgpu.ENB_I32, wrap, 15)
            l0 = orc.float_to_fixed(m_np, 15, 32)[:, :, None]
            want = _oracle_pyramid(orc, l0, alpha_np, levels, 32, wrap)
            for l in range(levels):
                g = got.read(l)
                assert np.array_equal(g, ref.read(l)), (call, l)
                assert np.array_equal(g, np.moveaxis(want[l], 2, 0)), (call, l)
            ref.free()
            got.free()
    finally:
        ctx.close()


@pytest.mark.parametrize("with_alpha", [True, False])
@pytest.mark.parametrize("channels", [1, 3])
def test_noalloc_float_image_into_f32_pyramid(channels, with_alpha):
    """F32 images into FP32 pyramids (the logarithmic mapping at level 0), as enb_gaussian_pyramid does."""
    import enbgpu
    ctx = _context()
    rng = np.random.default_rng(13)
    try:
        for call, (h, w, wrap) in enumerate(CALLS):
            levels = enbgpu.num_levels(w, h)
            shape = (h, w, channels) if channels == 3 else (h, w)
            img = torch.from_numpy(rng.random(shape).astype(np.float32)).cuda()
            alpha = torch.from_numpy(_alpha(rng, h, w)).cuda() if with_alpha else None
            desc = enbgpu.pixel_image(img)
            ref = ctx.pyramid(levels, w, h, channels, enbgpu.ENB_F32)
            a = ctypes.byref(enbgpu.plane_image(alpha)) if alpha is not None else None
            ctx._check(ctx.lib.enb_gaussian_pyramid(ctx.handle, int(wrap), ctypes.byref(desc), a, 0, ref.handle))
            got = _noalloc(ctx, desc, alpha, levels, w, h, channels, enbgpu.ENB_F32, wrap, 0)
            for l in range(levels):
                assert np.array_equal(got.read(l), ref.read(l)), (call, l)
            # level 0 is the mapping v >= 0 ? 1 + log1p(v) : 1 / (1 - v), not a fixed-point integer
            l0 = got.read(0)
            src = img.cpu().numpy().reshape(h, w, channels)
            assert np.allclose(np.moveaxis(l0, 0, 2), 1.0 + np.log1p(src), rtol=1e-6, atol=0)
            ref.free()
            got.free()
    finally:
        ctx.close()


def test_noalloc_rejects_mismatched_sources():
    """Sources the allocating entry point rejects are rejected here too, with a message."""
    import enbgpu
    ctx = _context()
    try:
        h, w = 64, 96
        levels = enbgpu.num_levels(w, h)
        pix = torch.zeros((h, w, 3), dtype=torch.uint8, device="cuda")
        pyr = ctx.pyramid(levels, w, h, 3, enbgpu.ENB_F32)   # U8 pixels into an F32 pyramid
        st = ctx.lib.enb_gaussian_pyramid_noalloc(ctx.handle, 0, ctypes.byref(enbgpu.pixel_image(pix)), None, 7,
                                                  pyr.handle)
        assert st == enbgpu.ENB_ERR_INVALID
        assert b"F32 pyramid" in ctx.lib.enb_last_error(ctx.handle)
        pyr.free()
    finally:
        ctx.close()


def test_noalloc_rejects_images_beyond_the_scratch():
    import enbgpu
    ctx = _context()
    try:
        h, w = 6000, 9000   # alpha planes of levels >= 1 need about 18 MB
        levels = enbgpu.num_levels(w, h)
        img = torch.zeros((h, w, 3), dtype=torch.uint8, device="cuda")
        alpha = torch.full((h, w), 255, dtype=torch.uint8, device="cuda")
        pyr = ctx.pyramid(levels, w, h, 3, enbgpu.ENB_I16)
        st = ctx.lib.enb_gaussian_pyramid_noalloc(ctx.handle, 0, ctypes.byref(enbgpu.pixel_image(img)),
                                                  ctypes.byref(enbgpu.plane_image(alpha)), 7, pyr.handle)
        assert st == enbgpu.ENB_ERR_INVALID
        assert b"scratch" in ctx.lib.enb_last_error(ctx.handle)
        pyr.free()
    finally:
        ctx.close()
