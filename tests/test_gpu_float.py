"""Float images: the CUDA path's FP32 pyramids against the oracle's double pyramids.

The reference builds double pyramids for float images (src/numerictraits.h:185);
the CUDA path keeps them in float.  The oracle's double restatement is pinned
to the reference's own code (tests/test_cpu_reference_pin.py), and here the
GPU results are held to float-rounding tolerances written beside each check:
pyramid operators and merged results within a few float ulps of the level
values, weight maps within 1e-5 relative of the double oracle, output pixels
within 1e-5 relative.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SIZES = [(2, 2), (3, 2), (2, 3), (5, 7), (17, 9), (33, 31), (65, 17), (100, 37), (257, 130)]
# one float operation on values of magnitude ~1..3 (the log-mapped range)
LEVEL_RTOL, LEVEL_ATOL = 2e-6, 2e-6
WEIGHT_RTOL = 1e-5


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _hwc(chw):
    return np.transpose(chw, (1, 2, 0)).astype(np.float64)


def _chw(hwc):
    return np.transpose(np.asarray(hwc, np.float32), (2, 0, 1))


def _level(rng, h, w, c, signed=False):
    v = rng.random((h, w, c)) * 2.0 + 0.5
    if signed:
        v = rng.random((h, w, c)) * 0.4 - 0.2
    return v.astype(np.float32).astype(np.float64)


def _alpha(rng, h, w, kind):
    if kind == "opaque":
        return np.full((h, w), 255, np.uint8)
    if kind == "holes":
        return (rng.random((h, w)) < 0.6).astype(np.uint8) * 255
    a = np.full((h, w), 255, np.uint8)
    a[: h // 2, : w // 3] = 0
    return a


def _close(got, ref, rtol, atol, what):
    err = np.abs(got - ref)
    bad = err > atol + rtol * np.abs(ref)
    assert not bad.any(), f"{what}: {bad.sum()} values off, max error {err.max():.3e}"


@pytest.mark.parametrize("wrap", [False, True])
@pytest.mark.parametrize("akind", ["opaque", "holes", "block"])
def test_reduce_f32(ctx, orc, wrap, akind):
    import enbgpu
    rng = np.random.default_rng(41)
    for (w, h) in SIZES:
        for c in (1, 3):
            src = _level(rng, h, w, c)
            a = _alpha(rng, h, w, akind)
            ref, ref_a = orc.reduce_d(src, a, wrap)
            p = ctx.pyramid(2, w, h, c, enbgpu.ENB_F32)
            p.write(0, _chw(src))
            dh, dw = (h + 1) >> 1, (w + 1) >> 1
            da = torch.zeros((dh, dw), dtype=torch.uint8, device="cuda")
            ctx.reduce(p, 0, p, 1, wrap=wrap, src_alpha=_dev(a), dst_alpha=da)
            _close(_hwc(p.read(1)), ref, LEVEL_RTOL, LEVEL_ATOL, f"reduce {w}x{h}x{c}")
            assert np.array_equal(da.cpu().numpy(), ref_a)


@pytest.mark.parametrize("wrap", [False, True])
@pytest.mark.parametrize("add", [False, True])
def test_expand_f32(ctx, orc, wrap, add):
    import enbgpu
    rng = np.random.default_rng(42)
    for (w, h) in SIZES + [(1, 1), (2, 1), (1, 2)]:
        for c in (1, 3):
            if w == 1 and wrap:
                continue  # one-column wrap reads uninitialised state in the reference
            sw, sh = (w + 1) >> 1, (h + 1) >> 1
            src = _level(rng, sh, sw, c, signed=True)
            dst = _level(rng, h, w, c)
            ref = orc.expand_d(src, dst, add, wrap)
            ps = ctx.pyramid(1, sw, sh, c, enbgpu.ENB_F32)
            pd = ctx.pyramid(1, w, h, c, enbgpu.ENB_F32)
            ps.write(0, _chw(src))
            pd.write(0, _chw(dst))
            ctx.expand(ps, 0, pd, 0, add=add, wrap=wrap)
            _close(_hwc(pd.read(0)), ref, LEVEL_RTOL, LEVEL_ATOL, f"expand {w}x{h}x{c}")


def test_blend_and_mask_multiply_f32(ctx, orc):
    import enbgpu
    rng = np.random.default_rng(43)
    wv = 255 << 15
    for (w, h) in SIZES:
        mask = rng.integers(-5, wv + 5, size=(h, w)).astype(np.int32)
        mask[rng.random((h, w)) < 0.2] = 0
        mask[rng.random((h, w)) < 0.2] = wv
        white, black = _level(rng, h, w, 3, signed=True), _level(rng, h, w, 3, signed=True)
        pm = ctx.pyramid(1, w, h, 1, enbgpu.ENB_I32)
        pw = ctx.pyramid(1, w, h, 3, enbgpu.ENB_F32)
        pb = ctx.pyramid(1, w, h, 3, enbgpu.ENB_F32)
        pm.write(0, mask[None])
        pw.write(0, _chw(white))
        pb.write(0, _chw(black))
        ctx.blend_level(pm, pw, pb, 0, wv)
        _close(_hwc(pb.read(0)), orc.blend_d(mask, white, black, wv), 1e-6, 1e-7, f"blend {w}x{h}")

        m2 = np.clip(mask, 0, wv)
        pr = ctx.pyramid(1, w, h, 3, enbgpu.ENB_F32)
        prev = _level(rng, h, w, 3, signed=True)
        pr.write(0, _chw(prev))
        pm.write(0, m2[None])
        ctx.mask_multiply_accumulate(pw, pm, pr, 0, wv, accumulate=True)
        _, ref = orc.mask_multiply_d(white, m2, wv, prev)
        _close(_hwc(pr.read(0)), ref, 1e-6, 1e-7, f"mask multiply {w}x{h}")


def test_conversions_f32(ctx, orc):
    import enbgpu
    rng = np.random.default_rng(44)
    h, w = 37, 53
    img = (rng.random((h, w, 3)) * 1.5 - 0.25).astype(np.float32)
    img[0, :5] = [0.0, 1.0, -0.0]
    p = ctx.pyramid(1, w, h, 3, enbgpu.ENB_F32)
    g = _dev(img)
    ctx.lib.enb_to_pyramid(ctx.handle, __import__("ctypes").byref(enbgpu.pixel_image(g)),
                           __import__("ctypes").byref(p.level_image(0)), 0)
    lvl = _hwc(p.read(0))
    ref = orc.real_to_pyramid(img)
    _close(lvl, ref, 2e-7, 0.0, "to pyramid")
    alpha = _alpha(rng, h, w, "holes")
    out = torch.full((h, w, 3), 7.0, device="cuda")
    ctx.from_pyramid(p, 0, _dev(alpha), out)
    got = out.cpu().numpy().astype(np.float64)
    refo = orc.real_from_pyramid(lvl, alpha, np.full((h, w, 3), 7.0, np.float32)).astype(np.float64)
    _close(got, refo, 2e-6, 1e-7, "from pyramid")
    assert np.array_equal(got[alpha == 0], refo[alpha == 0])


PROJECTORS = ["average", "value", "anti-value", "lightness", "luminance", "channel-mixer"]


@pytest.mark.parametrize("float_range", [0.0, 1.0])
@pytest.mark.parametrize("projector", PROJECTORS)
def test_enfuse_mask_f32(ctx, orc, float_range, projector):
    import enbgpu
    from enbgpu import synthetic
    rng = np.random.default_rng(45)
    h, w = 96, 130
    lr = synthetic.log_radiance(h, w, 8.0, seed=5)
    img = synthetic.expose(lr, -1.0, np.float32)
    img[10:20, 10:40] = 1.0  # clipped: repeated values in the entropy windows
    img[30:36, 50:70] = 0.0  # and the dark clip value, with -0 among them
    img[33, 55:60] = -0.0
    img[40:44, 80:90, 1] = 0.375  # a repeated value that is no clip value
    alpha = _alpha(rng, h, w, "holes")
    fnames = ["gaussian", "lorentzian", "halfsine", "fullsine", "bisquare"]
    for i, fn in enumerate(fnames):
        kw = dict(exposure_weight=1.0, saturation_weight=0.2, contrast_weight=0.5,
                  entropy_weight=0.3 if float_range > 0 else 0.0, exposure_optimum=0.45,
                  exposure_width=0.2, exposure_weight_function=fn, contrast_window_size=5,
                  entropy_window_size=5, gray_projector=projector, mixer=(0.2, 0.5, 0.3))
        prm_o = orc.params(**kw)
        ref = orc.enfuse_mask_f(img, alpha, prm_o, float_range if float_range > 0 else orc.FLT_MAX)
        out = torch.zeros((h, w), dtype=torch.float32, device="cuda")
        ctx.enfuse_mask(_dev(img), _dev(alpha), out, enbgpu.enfuse_params(float_range=float_range, **kw))
        got = out.cpu().numpy().astype(np.float64)
        # 1e-5 relative; values that cancel to ~0 (a weight function's support edge) are held to
        # 1e-7 of the map's largest weight instead
        _close(got, ref.astype(np.float64), WEIGHT_RTOL, 1e-7 * np.abs(ref).max(), f"weights {fn}")
        assert np.all(got[alpha == 0] == 0.0)


@pytest.mark.parametrize("h,w", [(5, 5), (17, 33), (61, 97), (130, 257)])
@pytest.mark.parametrize("windows", [(5, 5), (3, 3), (5, 3), (3, 5), (0, 5), (5, 0), (7, 5)])
@pytest.mark.parametrize("akind", ["opaque", "holes"])
def test_enfuse_mask_f32_windows(ctx, orc, h, w, windows, akind):
    """Contrast windows of 3, 5 and 7 and entropy windows of 3 and 5 (either
    weight off), odd and even widths, images narrower than a tile, alpha
    holes, clipped and repeated samples, both cutoffs on the larger sizes."""
    import enbgpu
    from enbgpu import synthetic
    rng = np.random.default_rng(100 + h + w)
    img = synthetic.expose(synthetic.log_radiance(h, w, 8.0, seed=h), 0.5, np.float32)
    img[h // 4: h // 2, w // 5: w // 2] = 1.0
    img[h // 2: h // 2 + 3, : w // 3, 2] = 0.0
    img[: h // 3, w // 2:, 0] = 0.625
    alpha = _alpha(rng, h, w, akind)
    cw, ew = windows
    if min(h, w) < max(cw, ew):
        pytest.skip("window larger than the image")
    kw = dict(exposure_weight=1.0, saturation_weight=0.2, contrast_weight=0.5 if cw else 0.0,
              entropy_weight=0.3 if ew else 0.0, contrast_window_size=cw or 5, entropy_window_size=ew or 5)
    if h > 20:
        kw.update(exposure_cutoff=((2.0, True), (97.0, True)), entropy_cutoff=((5.0, True), (95.0, True)))
    ref = orc.enfuse_mask_f(img, alpha, orc.params(**kw), 1.0)
    out = torch.zeros((h, w), dtype=torch.float32, device="cuda")
    ctx.enfuse_mask(_dev(img), _dev(alpha), out, enbgpu.enfuse_params(float_range=1.0, **kw))
    got = out.cpu().numpy().astype(np.float64)
    _close(got, ref.astype(np.float64), WEIGHT_RTOL, 1e-7 * np.abs(ref).max(), f"weights {windows}")
    assert np.all(got[alpha == 0] == 0.0)


@pytest.mark.parametrize("levels", [4, 32, 1024])
@pytest.mark.parametrize("ew", [3, 5])
def test_enfuse_mask_f32_repeated_samples(ctx, orc, levels, ew):
    """Float samples quantised to a few levels: nearly every entropy window
    holds repeated samples (bins of several taps besides the clip values),
    in every channel, with alpha holes."""
    import enbgpu
    from enbgpu import synthetic
    rng = np.random.default_rng(levels + ew)
    h, w = 70, 101
    img = synthetic.expose(synthetic.log_radiance(h, w, 8.0, seed=9), 0.5, np.float32)
    img = (np.round(img * levels) / levels).astype(np.float32)
    alpha = _alpha(rng, h, w, "holes")
    kw = dict(exposure_weight=1.0, saturation_weight=0.2, contrast_weight=0.5, entropy_weight=0.3,
              contrast_window_size=5, entropy_window_size=ew)
    ref = orc.enfuse_mask_f(img, alpha, orc.params(**kw), 1.0)
    out = torch.zeros((h, w), dtype=torch.float32, device="cuda")
    ctx.enfuse_mask(_dev(img), _dev(alpha), out, enbgpu.enfuse_params(float_range=1.0, **kw))
    _close(out.cpu().numpy().astype(np.float64), ref.astype(np.float64), WEIGHT_RTOL, 1e-7 * np.abs(ref).max(),
           f"weights, {levels} levels")


@pytest.mark.parametrize("shape", [(61, 97), (40, 33, 2)])
def test_enfuse_mask_f32_gray(ctx, orc, shape):
    """Gray float images (one channel, alone or with an alpha sample): the
    weight kernels' one-channel build (no saturation; contrast and entropy of
    the one channel) against the oracle."""
    import enbgpu
    from enbgpu import synthetic
    h, w = shape[:2]
    g = synthetic.expose(synthetic.log_radiance(h, w, 8.0, seed=12), 0.5, np.float32)[..., 1]
    g[h // 3: h // 2, : w // 2] = 1.0
    g[: h // 4, w // 2:] = np.round(g[: h // 4, w // 2:] * 16) / 16
    img = g if len(shape) == 2 else np.stack([g, np.ones_like(g)], axis=-1)
    kw = dict(exposure_weight=1.0, saturation_weight=0.2, contrast_weight=0.5, entropy_weight=0.3,
              contrast_window_size=5, entropy_window_size=5)
    ref = orc.enfuse_mask_f(img, None, orc.params(**kw), 1.0)
    out = torch.zeros((h, w), dtype=torch.float32, device="cuda")
    ctx.enfuse_mask(_dev(img), None, out, enbgpu.enfuse_params(float_range=1.0, **kw))
    _close(out.cpu().numpy().astype(np.float64), ref.astype(np.float64), WEIGHT_RTOL, 1e-7 * np.abs(ref).max(),
           "gray weights")


def test_enfuse_mask_f32_entropy_compat(ctx, orc):
    """The reference's float entropy weight (H * FLT_MAX) on its own."""
    import enbgpu
    from enbgpu import synthetic
    h, w = 64, 80
    img = synthetic.expose(synthetic.log_radiance(h, w, 8.0, seed=6), 0.0, np.float32)
    img[5:15, 5:25] = 0.25
    alpha = np.full((h, w), 255, np.uint8)
    kw = dict(exposure_weight=0.0, entropy_weight=0.3, entropy_window_size=3)
    ref = orc.enfuse_mask_f(img, alpha, orc.params(**kw), orc.FLT_MAX)
    out = torch.zeros((h, w), dtype=torch.float32, device="cuda")
    ctx.enfuse_mask(_dev(img), _dev(alpha), out, enbgpu.enfuse_params(**kw))
    _close(out.cpu().numpy().astype(np.float64), ref.astype(np.float64), WEIGHT_RTOL, 0.0, "entropy compat")


def _stack(h, w, K, seed):
    from enbgpu import synthetic
    evs = np.linspace(-(K - 1) / 2.0, (K - 1) / 2.0, K)
    return synthetic.exposure_stack(h, w, evs, np.float32, 8.0, seed)


@pytest.mark.parametrize("hard", [False, True])
@pytest.mark.parametrize("wrap", [False, True])
def test_enfuse_f32_injected_masks(ctx, orc, hard, wrap):
    """Same float masks on both sides: the fuse itself (double vs FP32 pyramids)."""
    rng = np.random.default_rng(46)
    h, w, K = 75, 101, 4
    imgs = _stack(h, w, K, 7)
    masks = [rng.random((h, w)).astype(np.float32) for _ in range(K)]
    alphas = [_alpha(rng, h, w, "opaque")] * (K - 1) + [_alpha(rng, h, w, "block")]
    ref = orc.enfuse_f(imgs, alphas, masks=masks, hard_mask=hard, wrap=wrap, want_level0=True)
    l0 = torch.zeros((h, w, 3), dtype=torch.float32, device="cuda")
    out, oa = ctx.enfuse([_dev(x) for x in imgs], alphas=[_dev(a) for a in alphas],
                         masks=[_dev(m) for m in masks], hard_mask=hard, wrap=wrap, level0=l0)
    assert np.array_equal(oa.cpu().numpy(), ref["alpha"])
    _close(l0.cpu().numpy().astype(np.float64), ref["level0"], 1e-5, 1e-6, "level 0")
    _close(out.cpu().numpy().astype(np.float64), ref["out"].astype(np.float64), 1e-5, 1e-6, "pixels")


@pytest.mark.parametrize("K,h,w", [(3, 64, 96), (5, 130, 67)])
def test_enfuse_f32_weights_normalised(ctx, orc, K, h, w):
    """End to end with the weights of the 9-exposure configuration in normalised-float mode."""
    import enbgpu
    imgs = _stack(h, w, K, 8 + K)
    kw = dict(exposure_weight=1.0, saturation_weight=0.2, contrast_weight=0.5, entropy_weight=0.3,
              contrast_window_size=5, entropy_window_size=5)
    ref = orc.enfuse_f(imgs, prm=orc.params(**kw), range_=1.0, want_level0=True, want_masks=True)
    out, _ = ctx.enfuse([_dev(x) for x in imgs], params=enbgpu.enfuse_params(float_range=1.0, **kw))
    _close(out.cpu().numpy().astype(np.float64), ref["out"].astype(np.float64), 1e-4, 1e-5, "pixels")


def test_enfuse_f32_host_buffers(ctx, orc):
    imgs = _stack(40, 52, 3, 21)
    ref = orc.enfuse_f(imgs, prm=orc.params(saturation_weight=0.2), range_=1.0)
    import enbgpu
    out, oa = ctx.enfuse(imgs, params=enbgpu.enfuse_params(saturation_weight=0.2, float_range=1.0))
    assert np.array_equal(oa, ref["alpha"])
    _close(out.astype(np.float64), ref["out"].astype(np.float64), 1e-4, 1e-5, "pixels")


@pytest.mark.parametrize("wrap", [False, True])
@pytest.mark.parametrize("stride", [3, 4])
def test_enblend_f32(ctx, orc, wrap, stride):
    from enbgpu import synthetic
    h, w = 70, 121
    lr = synthetic.log_radiance(h, w, 8.0, seed=9)
    white = synthetic.expose(lr, 0.3, np.float32)
    black = synthetic.expose(lr, -0.2, np.float32)
    wa = np.zeros((h, w), np.uint8)
    wa[:, : 2 * w // 3] = 255
    ba = np.zeros((h, w), np.uint8)
    ba[:, w // 3:] = 255
    mask = np.zeros((h, w), np.uint8)
    mask[:, : w // 2] = 255
    if stride == 4:
        white = np.concatenate([white, (wa[..., None] / 255.0).astype(np.float32)], axis=2)
        black = np.concatenate([black, (ba[..., None] / 255.0).astype(np.float32)], axis=2)
        wa_arg = ba_arg = None
    else:
        wa_arg, ba_arg = wa, ba
    ref = orc.enblend_f(white, black, mask, wa, ba, wrap=wrap, want_level0=True)
    l0 = torch.zeros((h, w, 3), dtype=torch.float32, device="cuda")
    out, oa = ctx.enblend(_dev(white), _dev(black), _dev(mask),
                          white_alpha=_dev(wa_arg) if wa_arg is not None else None,
                          black_alpha=_dev(ba_arg) if ba_arg is not None else None, wrap=wrap, level0=l0)
    assert np.array_equal(oa.cpu().numpy(), ref["alpha"])
    _close(l0.cpu().numpy().astype(np.float64), ref["level0"], 1e-5, 1e-6, "level 0")
    _close(out.cpu().numpy().astype(np.float64), ref["out"].astype(np.float64), 1e-5, 1e-6, "pixels")
