"""The allocation-free Gaussian pyramid entry point (enb_gaussian_pyramid_noalloc).

Some callers cannot allocate device memory while they run: a host
application that reserves its GPU budget up front in its own pool and forbids
driver allocations inside its processing callbacks, or a fixed-budget
embedded pipeline.  For them the library keeps the reduced alpha planes in a
static device array.  This test calls the entry point through the C ABI and
checks every level against the allocating enb_gaussian_pyramid, on two calls
in a row with different images (the scratch keeps the previous call's
contents, which must not leak into the next result).  It lives in its own
file, collected last, so a failure here never hides another test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _img(rng, h, w, dtype):
    maxv = np.iinfo(dtype).max
    return rng.integers(0, maxv + 1, size=(h, w, 3)).astype(dtype)


def _alpha(rng, h, w):
    a = (rng.random((h, w)) < 0.7).astype(np.uint8) * 255
    a[: h // 3, : w // 4] = 0
    return a


@pytest.mark.parametrize("dtype,pdt", [(np.uint8, "i16"), (np.uint16, "i32")])
def test_noalloc_gaussian_pyramid_matches_allocating_entry_point(dtype, pdt):
    import enbgpu
    from enbgpu import _build
    _build.build()
    ctx = enbgpu.Context(0)
    lib = ctx.lib
    code = enbgpu.ENB_I16 if pdt == "i16" else enbgpu.ENB_I32
    rng = np.random.default_rng(7)
    try:
        for call, (h, w, wrap) in enumerate([(301, 517, False), (257, 389, True)]):
            levels = enbgpu.num_levels(w, h)
            img = torch.from_numpy(_img(rng, h, w, dtype)).cuda()
            alpha = torch.from_numpy(_alpha(rng, h, w)).cuda()
            ref = ctx.gaussian_pyramid(img, levels, alpha=alpha, wrap=wrap, dtype=code)
            got = ctx.pyramid(levels, w, h, 3, code)
            src = enbgpu.pixel_image(img)
            a = enbgpu.plane_image(alpha)
            ctx._check(lib.enb_gaussian_pyramid_noalloc(ctx.handle, int(wrap), ctypes.byref(src),
                                                        ctypes.byref(a), 7, got.handle))
            ctx.synchronize()
            for l in range(levels):
                assert np.array_equal(got.read(l), ref.read(l)), (call, l)
            ref.free()
            got.free()
    finally:
        ctx.close()


def test_noalloc_rejects_images_beyond_the_scratch():
    import enbgpu
    from enbgpu import _build
    _build.build()
    ctx = enbgpu.Context(0)
    try:
        h, w = 6000, 9000   # alpha planes of levels >= 1 need about 18 MB
        levels = enbgpu.num_levels(w, h)
        img = torch.zeros((h, w, 3), dtype=torch.uint8, device="cuda")
        alpha = torch.full((h, w), 255, dtype=torch.uint8, device="cuda")
        pyr = ctx.pyramid(levels, w, h, 3, enbgpu.ENB_I16)
        st = ctx.lib.enb_gaussian_pyramid_noalloc(ctx.handle, 0, ctypes.byref(enbgpu.pixel_image(img)),
                                                  ctypes.byref(enbgpu.plane_image(alpha)), 7, pyr.handle)
        assert st == 1
        assert b"scratch" in ctx.lib.enb_last_error(ctx.handle)
        pyr.free()
    finally:
        ctx.close()
