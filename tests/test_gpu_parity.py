"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Integer and fixed-point stages must be bit-exact; enfuse weights are
compared exactly as well (the kernels reproduce the reference's float/double
rounding), and so are the final pixels for the same dither seed.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SIZES = [(2, 2), (3, 2), (2, 3), (3, 3), (4, 5), (5, 7), (8, 8), (17, 9), (33, 31), (64, 16),
         (65, 17), (100, 37), (257, 130)]


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _rand_level(rng, h, w, c, dtype, signed=False):
    if dtype == "i16":
        lo, hi = (-32640, 32640) if signed else (0, 32640)
    else:
        lo, hi = (-(1 << 23), 1 << 23) if signed else (0, 65535 << 7)
    return rng.integers(lo, hi + 1, size=(h, w, c)).astype(np.int32)


def _alpha(rng, h, w, kind):
    if kind == "opaque":
        return np.full((h, w), 255, np.uint8)
    if kind == "holes":
        return (rng.random((h, w)) < 0.6).astype(np.uint8) * 255
    a = np.full((h, w), 255, np.uint8)
    a[: h // 2, : w // 3] = 0
    return a


def _pyr(ctx, enbgpu, w, h, c, dt, levels=2):
    return ctx.pyramid(levels, w, h, c, enbgpu.ENB_I16 if dt == "i16" else enbgpu.ENB_I32)


def _hwc(level_chw):
    return np.transpose(level_chw, (1, 2, 0)).astype(np.int32)


@pytest.mark.parametrize("dt", ["i16", "i32"])
@pytest.mark.parametrize("wrap", [False, True])
@pytest.mark.parametrize("akind", ["opaque", "holes", "block"])
def test_reduce_alpha(ctx, orc, dt, wrap, akind):
    import enbgpu
    rng = np.random.default_rng(11)
    bits = 16 if dt == "i16" else 32
    for (w, h) in SIZES:
        for c in (1, 3):
            src = _rand_level(rng, h, w, c, dt)
            a = _alpha(rng, h, w, akind)
            ref, ref_a = orc.reduce(src, a, bits, wrap)
            p = _pyr(ctx, enbgpu, w, h, c, dt)
            p.write(0, np.transpose(src, (2, 0, 1)))
            dh, dw = (h + 1) >> 1, (w + 1) >> 1
            sa, da = _dev(a), torch.zeros((dh, dw), dtype=torch.uint8, device="cuda")
            ctx.reduce(p, 0, p, 1, wrap=wrap, src_alpha=sa, dst_alpha=da)
            got = _hwc(p.read(1))
            assert np.array_equal(got, ref), (w, h, c)
            assert np.array_equal(da.cpu().numpy(), ref_a), (w, h, c)


@pytest.mark.parametrize("dt", ["i16", "i32"])
@pytest.mark.parametrize("wrap", [False, True])
def test_reduce_noalpha(ctx, orc, dt, wrap):
    import enbgpu
    rng = np.random.default_rng(12)
    bits = 16 if dt == "i16" else 32
    for (w, h) in SIZES:
        for c in (1, 3):
            src = _rand_level(rng, h, w, c, dt)
            ref = orc.reduce(src, None, bits, wrap)
            p = _pyr(ctx, enbgpu, w, h, c, dt)
            p.write(0, np.transpose(src, (2, 0, 1)))
            ctx.reduce(p, 0, p, 1, wrap=wrap)
            assert np.array_equal(_hwc(p.read(1)), ref), (w, h, c)


@pytest.mark.parametrize("dt", ["i16", "i32"])
@pytest.mark.parametrize("wrap", [False, True])
@pytest.mark.parametrize("add", [False, True])
def test_expand(ctx, orc, dt, wrap, add):
    import enbgpu
    rng = np.random.default_rng(13)
    bits = 16 if dt == "i16" else 32
    sizes = SIZES + [(1, 1), (2, 1), (1, 2), (1, 5), (6, 1)]
    for (w, h) in sizes:
        for c in (1, 3):
            dh, dw = h, w
            sh, sw = (h + 1) >> 1, (w + 1) >> 1
            src = _rand_level(rng, sh, sw, c, dt, signed=True)
            dst = _rand_level(rng, dh, dw, c, dt, signed=True)
            if dt == "i16":
                # full int16 range: exercises wrap-around (subtract) and saturation (add)
                dst = rng.integers(-32768, 32768, size=dst.shape).astype(np.int32)
            ref = orc.expand(src, dst, add, bits, wrap)
            p = _pyr(ctx, enbgpu, w, h, c, dt)
            p.write(0, np.transpose(dst, (2, 0, 1)))
            p.write(1, np.transpose(src, (2, 0, 1)))
            ctx.expand(p, 1, p, 0, add=add, wrap=wrap)
            assert np.array_equal(_hwc(p.read(0)), ref), (w, h, c)


@pytest.mark.parametrize("dt", ["i16", "i32"])
def test_blend_level(ctx, orc, dt):
    import enbgpu
    rng = np.random.default_rng(14)
    bits = 16 if dt == "i16" else 32
    mfrac = 7 if dt == "i16" else 15
    white_value = 255 << mfrac
    for (w, h) in [(64, 16), (100, 37), (257, 130)]:
        white = _rand_level(rng, h, w, 3, dt, signed=True)
        black = _rand_level(rng, h, w, 3, dt, signed=True)
        mask = rng.integers(-3, white_value + 3, size=(h, w, 1)).astype(np.int32)
        mask[rng.random((h, w)) < 0.3] = 0
        mask[rng.random((h, w)) < 0.3] = white_value
        ref = orc.blend(mask, white, black, white_value, bits)
        pw, pb, pm = (_pyr(ctx, enbgpu, w, h, 3, dt, 1), _pyr(ctx, enbgpu, w, h, 3, dt, 1),
                      _pyr(ctx, enbgpu, w, h, 1, dt, 1))
        pw.write(0, np.transpose(white, (2, 0, 1)))
        pb.write(0, np.transpose(black, (2, 0, 1)))
        pm.write(0, np.transpose(mask, (2, 0, 1)))
        ctx.blend_level(pm, pw, pb, 0, white_value)
        assert np.array_equal(_hwc(pb.read(0)), ref)


@pytest.mark.parametrize("dt", ["i16", "i32"])
@pytest.mark.parametrize("accumulate", [False, True])
def test_mask_multiply_accumulate(ctx, orc, dt, accumulate):
    import enbgpu
    rng = np.random.default_rng(15)
    bits = 16 if dt == "i16" else 32
    mfrac = 7 if dt == "i16" else 15
    D = 255 << mfrac
    w, h = 257, 130
    lp = _rand_level(rng, h, w, 3, dt, signed=True)
    res = _rand_level(rng, h, w, 3, dt, signed=True)
    mask = rng.integers(0, D + 1, size=(h, w, 1)).astype(np.int32)
    # exact half-integer products: m = D/2 with odd lp, m = D/4 with lp = 2 mod 4
    mask[:10] = D // 2
    mask[10:20] = D // 4
    mask[20:25] = 0
    mask[25:30] = D
    lp[:10] |= 1
    lp[10:20] = (lp[10:20] & ~3) | 2
    prod = orc.mask_multiply(lp, mask, D, bits)
    ref = orc.accumulate(prod, res, bits) if accumulate else prod
    pl, pm, pr = (_pyr(ctx, enbgpu, w, h, 3, dt, 1), _pyr(ctx, enbgpu, w, h, 1, dt, 1),
                  _pyr(ctx, enbgpu, w, h, 3, dt, 1))
    pl.write(0, np.transpose(lp, (2, 0, 1)))
    pm.write(0, np.transpose(mask, (2, 0, 1)))
    pr.write(0, np.transpose(res, (2, 0, 1)))
    ctx.mask_multiply_accumulate(pl, pm, pr, 0, D, accumulate)
    assert np.array_equal(_hwc(pr.read(0)), ref)


@pytest.mark.parametrize("dt,out_dtype", [("i16", np.uint8), ("i32", np.uint16)])
@pytest.mark.parametrize("dither", ["hash", "nearest"])
def test_from_pyramid(ctx, orc, dt, out_dtype, dither):
    import enbgpu
    rng = np.random.default_rng(16)
    w, h = 257, 130
    maxv = np.iinfo(out_dtype).max
    src = rng.integers(-300, (maxv + 2) << 7, size=(h, w, 3)).astype(np.int32)
    if dt == "i16":
        src = np.clip(src, -32768, 32767)
    alpha = _alpha(rng, h, w, "holes")
    ref = orc.from_fixed(src, alpha, out_dtype, 7, dither, seed=1234)
    p = _pyr(ctx, enbgpu, w, h, 3, dt, 1)
    p.write(0, np.transpose(src, (2, 0, 1)))
    dst = torch.zeros((h, w, 3), dtype=torch.uint8 if out_dtype == np.uint8 else torch.uint16, device="cuda")
    ctx.from_pyramid(p, 0, _dev(alpha), dst, 7, dither, seed=1234)
    assert np.array_equal(dst.cpu().numpy(), ref)


@pytest.mark.parametrize("dt", [np.uint8, np.uint16])
@pytest.mark.parametrize("proj", ["average", "value", "anti-value", "lightness", "luminance", "channel-mixer"])
def test_enfuse_mask(ctx, orc, dt, proj):
    import enbgpu
    from enbgpu import synthetic
    rng = np.random.default_rng(17)
    h, w = 61, 83
    lr = synthetic.log_radiance(h, w, 10.0, seed=5)
    for ev in (-2.0, 0.0, 2.5):
        img = synthetic.expose(lr, ev, dt, noise=2.0 ** -10, seed=3)
        alpha = _alpha(rng, h, w, "holes" if ev > 0 else "opaque")
        kw = dict(exposure_weight=1.0, saturation_weight=0.2, contrast_weight=0.5, entropy_weight=0.3,
                  contrast_window_size=5, entropy_window_size=5, gray_projector=proj, mixer=(0.3, 0.59, 0.11))
        ref = orc.enfuse_mask(img, alpha, orc.params(**kw))
        out = torch.zeros((h, w), dtype=torch.float32, device="cuda")
        ctx.enfuse_mask(_dev(img), _dev(alpha), out, enbgpu.enfuse_params(**kw))
        got = out.cpu().numpy()
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), np.abs(got - ref).max()


@pytest.mark.parametrize("fn", ["gaussian", "lorentzian", "halfsine", "fullsine", "bisquare"])
@pytest.mark.parametrize("window", [3, 7])
def test_enfuse_mask_functions(ctx, orc, fn, window):
    import enbgpu
    from enbgpu import synthetic
    h, w = 40, 52
    img = synthetic.exposure_stack(h, w, [0.5], np.uint16, 8.0, seed=9)[0]
    alpha = np.full((h, w), 255, np.uint8)
    kw = dict(exposure_weight=0.7, saturation_weight=0.4, contrast_weight=0.9, entropy_weight=0.6,
              exposure_optimum=0.4, exposure_width=0.25, exposure_weight_function=fn,
              contrast_window_size=window, entropy_window_size=window)
    ref = orc.enfuse_mask(img, alpha, orc.params(**kw))
    out = torch.zeros((h, w), dtype=torch.float32, device="cuda")
    ctx.enfuse_mask(_dev(img), _dev(alpha), out, enbgpu.enfuse_params(**kw))
    assert np.array_equal(out.cpu().numpy().view(np.uint32), ref.view(np.uint32))


def _stack(dt, h, w, n, seed):
    from enbgpu import synthetic
    evs = np.linspace(-2, 2, n)
    return synthetic.exposure_stack(h, w, evs, dt, 8.0, seed, noise=2.0 ** -11)


@pytest.mark.parametrize("dt", [np.uint8, np.uint16])
@pytest.mark.parametrize("hard", [False, True])
@pytest.mark.parametrize("wrap", [False, True])
def test_enfuse_end_to_end(ctx, orc, dt, hard, wrap):
    import enbgpu
    h, w = 75, 97
    imgs = _stack(dt, h, w, 3, seed=21)
    rng = np.random.default_rng(3)
    alphas = [np.full((h, w), 255, np.uint8) for _ in imgs]
    alphas[1][10:30, 5:40] = 0
    kw = dict(exposure_weight=1.0, saturation_weight=0.2, contrast_weight=0.5, entropy_weight=0.3,
              contrast_window_size=5, entropy_window_size=5)
    ref = orc.enfuse(imgs, alphas, orc.params(**kw), hard_mask=hard, wrap=wrap, seed=77, want_level0=True)
    l0 = torch.zeros((h, w, 3), dtype=torch.int32, device="cuda")
    out, oa = ctx.enfuse([_dev(x) for x in imgs], [_dev(a) for a in alphas], enbgpu.enfuse_params(**kw),
                         hard_mask=hard, wrap=wrap, seed=77, level0=l0)
    assert np.array_equal(l0.cpu().numpy(), ref["level0"])
    assert np.array_equal(oa.cpu().numpy(), ref["alpha"])
    assert np.array_equal(out.cpu().numpy(), ref["out"])


@pytest.mark.parametrize("dt", [np.uint8, np.uint16])
def test_enfuse_host_buffers_and_injected_masks(ctx, orc, dt):
    import enbgpu
    h, w = 50, 66
    imgs = _stack(dt, h, w, 4, seed=22)
    rng = np.random.default_rng(4)
    masks = [rng.random((h, w)).astype(np.float32) for _ in imgs]
    masks[0][:5] = 0.0
    for m in masks:
        m[:5, :5] = 0.0  # all-zero weights -> integer 255/K fallback
    ref = orc.enfuse(imgs, None, masks=masks, seed=5, want_level0=True)
    l0 = np.zeros((h, w, 3), np.int32)
    out, oa = ctx.enfuse(imgs, masks=masks, seed=5, level0=l0)
    assert np.array_equal(l0, ref["level0"])
    assert np.array_equal(out, ref["out"])


# pass structures of the enblend driver: fused level passes with every level
# in its own launches (default), fused passes with all levels below level 1 in
# one cluster launch, and one kernel per reference operation
MODES = {"fused": {}, "cluster": {"coarse_pixels": 1 << 30}, "plain": {"plain": True}}


@pytest.mark.parametrize("dt", [np.uint8, np.uint16])
@pytest.mark.parametrize("wrap", [False, True])
@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("geom", [(90, 120, 80), (7, 9, 5), (21, 30, 17), (40, 64, 40)])
def test_enblend_end_to_end(ctx, orc, dt, wrap, mode, geom):
    """Every pass structure against the oracle.

    Geometries give 8, 1, 2 and 4 pyramid levels (union canvases 200x90,
    14x7, 47x21, 104x40)."""
    from enbgpu import synthetic
    h, w, off = geom
    white, black, mask = synthetic.panorama_pair(h, w, off, dt, seed=31)
    if w > 20:
        mask[: h // 3, off + 2: off + 9] = 128   # intermediate seam weights at level 0 too
    ref = orc.enblend(white, black, mask, wrap=wrap, seed=9, want_level0=True)
    l0 = torch.zeros((h, w + off, 3), dtype=torch.int32, device="cuda")
    out, oa = ctx.enblend(_dev(white), _dev(black), _dev(mask), wrap=wrap, seed=9, level0=l0, **MODES[mode])
    assert np.array_equal(l0.cpu().numpy(), ref["level0"])
    assert np.array_equal(oa.cpu().numpy(), ref["alpha"])
    assert np.array_equal(out.cpu().numpy(), ref["out"])
    # host-buffer entry point gives the same image
    out2, _ = ctx.enblend(white, black, mask, wrap=wrap, seed=9, **MODES[mode])
    assert np.array_equal(out2, ref["out"])


@pytest.mark.parametrize("wrap", [False, True])
@pytest.mark.parametrize("coarse", [32768, 4000, 1 << 30])
def test_enblend_coarse_split(ctx, orc, wrap, coarse):
    """Per-level launches above, the cluster launch below, on a 700x300
    canvas: coarse from 175x75 down (32768 pixels), a split further down
    (4000 pixels) and everything but level 1 in the cluster launch."""
    from enbgpu import synthetic
    white, black, mask = synthetic.panorama_pair(300, 400, 300, np.uint16, seed=37)
    mask[40:90, 310:330] = 77
    ref = orc.enblend(white, black, mask, wrap=wrap, seed=4, want_level0=True)
    l0 = torch.zeros((300, 700, 3), dtype=torch.int32, device="cuda")
    out, oa = ctx.enblend(_dev(white), _dev(black), _dev(mask), wrap=wrap, seed=4, level0=l0, coarse_pixels=coarse)
    assert np.array_equal(l0.cpu().numpy(), ref["level0"])
    assert np.array_equal(out.cpu().numpy(), ref["out"])
    assert np.array_equal(oa.cpu().numpy(), ref["alpha"])


@pytest.mark.parametrize("plain", [False, True])
def test_enblend_alpha_sources(ctx, orc, plain):
    """Alpha from planes, from the 4th component, mixed, and RGB images without alpha."""
    from enbgpu import synthetic
    white, black, mask = synthetic.panorama_pair(64, 96, 50, np.uint16, seed=33)
    wa, ba = orc.alpha_of(white), orc.alpha_of(black)
    wa[5:20, 60:80] = 0          # a hole in the white image's alpha plane
    ref = orc.enblend(white, black, mask, white_alpha=wa, black_alpha=ba, seed=1)
    for wa_arg, ba_arg in [(wa, ba), (wa, None)]:
        out, oa = ctx.enblend(_dev(white), _dev(black), _dev(mask),
                              white_alpha=_dev(wa) if wa_arg is not None else None,
                              black_alpha=_dev(ba) if ba_arg is not None else None, seed=1, plain=plain)
        assert np.array_equal(out.cpu().numpy(), ref["out"])
        assert np.array_equal(oa.cpu().numpy(), ref["alpha"])
    rgb_w, rgb_b = np.ascontiguousarray(white[..., :3]), np.ascontiguousarray(black[..., :3])
    ref = orc.enblend(rgb_w, rgb_b, mask, seed=2)
    out, oa = ctx.enblend(_dev(rgb_w), _dev(rgb_b), _dev(mask), seed=2, plain=plain)
    assert np.array_equal(out.cpu().numpy(), ref["out"])


@pytest.mark.parametrize("dt", [np.uint8, np.uint16])
@pytest.mark.parametrize("wrap", [False, True])
@pytest.mark.parametrize("planes", [False, True])
@pytest.mark.parametrize("off", [240, 241])
def test_enblend_level0_tma(ctx, orc, dt, wrap, planes, off):
    """RGBA level 0 through the TMA pipeline (profile name out0_tma), on
    canvases whose rows start on 16-byte boundaries (width 640) and off them
    (641: every row box starts before its first pixel), alpha from the 4th
    component or from planes, against the oracle; the host-buffer entry
    point runs it per output band (1100 rows).  RGB images take the tile
    kernel (out0)."""
    from enbgpu import synthetic
    h = 1100 if planes else 300
    white, black, mask = synthetic.panorama_pair(h, 400, off, dt, seed=43)
    mask[40:200, 250:300] = 111
    kw, dkw = {}, {}
    if planes:
        wa, ba = orc.alpha_of(white).copy(), orc.alpha_of(black)
        wa[300:340, 250:290] = 0
        kw = dict(white_alpha=wa, black_alpha=ba)
        dkw = dict(white_alpha=_dev(wa), black_alpha=_dev(ba))
    ref = orc.enblend(white, black, mask, wrap=wrap, seed=8, want_level0=True, **kw)
    l0 = torch.zeros((h, 400 + off, 3), dtype=torch.int32, device="cuda")
    ctx.profile(True)
    out, oa = ctx.enblend(_dev(white), _dev(black), _dev(mask), wrap=wrap, seed=8, level0=l0, **dkw)
    names = set(ctx.profile_report())
    ctx.profile(False)
    assert "out0_tma" in names and "out0" not in names
    assert np.array_equal(l0.cpu().numpy(), ref["level0"])
    assert np.array_equal(out.cpu().numpy(), ref["out"])
    assert np.array_equal(oa.cpu().numpy(), ref["alpha"])
    out2, oa2 = ctx.enblend(white, black, mask, wrap=wrap, seed=8, **kw)
    assert np.array_equal(out2, ref["out"])
    assert np.array_equal(oa2, ref["alpha"])
    if not planes:
        rgb_w, rgb_b = np.ascontiguousarray(white[..., :3]), np.ascontiguousarray(black[..., :3])
        ref = orc.enblend(rgb_w, rgb_b, mask, wrap=wrap, seed=8)
        ctx.profile(True)
        out, _ = ctx.enblend(_dev(rgb_w), _dev(rgb_b), _dev(mask), wrap=wrap, seed=8)
        names = set(ctx.profile_report())
        ctx.profile(False)
        assert "out0" in names and "out0_tma" not in names
        assert np.array_equal(out.cpu().numpy(), ref["out"])


def test_level0_wait_timeout_is_reported(ctx, orc):
    """The level-0 pipeline's bounded waits: with every stage barrier armed for
    16 bytes more than its copies deliver (enb_debug_overarm_tile_waits), each
    CTA's first wait runs out after about half a second, the kernel records it
    in the context's error word and returns without writing the tiles it was
    waiting for, and enb_synchronize fails with ENB_ERR_CUDA and the message.
    Nothing faults and no wait is unbounded; the same context then blends
    correctly again."""
    import enbgpu
    from enbgpu import synthetic
    white, black, mask = synthetic.panorama_pair(300, 400, 240, np.uint16, seed=43)   # 640 wide: TMA rows
    ref = orc.enblend(white, black, mask, seed=8)
    dw, db, dm = _dev(white), _dev(black), _dev(mask)
    sentinel = 0x1234
    out = torch.full(black.shape, sentinel, dtype=torch.uint16, device="cuda")
    ctx._check(ctx.lib.enb_debug_overarm_tile_waits(ctx.handle, 16))
    try:
        ctx.enblend(dw, db, dm, out=out, seed=8)
        with pytest.raises(enbgpu.EnbError) as err:
            ctx.synchronize()
        assert err.value.status == enbgpu.ENB_ERR_CUDA
        assert "timed out" in str(err.value)
    finally:
        ctx._check(ctx.lib.enb_debug_overarm_tile_waits(ctx.handle, 0))
    got = out.cpu().numpy()
    assert (got[..., :3] == sentinel).any(), "the tiles whose wait ran out must stay unwritten"
    ctx.synchronize()   # the error word was cleared by the failed synchronisation
    ctx.profile(True)
    out2, oa2 = ctx.enblend(dw, db, dm, seed=8)
    names = set(ctx.profile_report())
    ctx.profile(False)
    assert "out0_tma" in names
    assert np.array_equal(out2.cpu().numpy(), ref["out"])
    assert np.array_equal(oa2.cpu().numpy(), ref["alpha"])


def test_enblend_in_place(ctx, orc):
    """out may alias the black image (the reference writes into it)."""
    from enbgpu import synthetic
    white, black, mask = synthetic.panorama_pair(50, 70, 40, np.uint16, seed=35)
    ref = orc.enblend(white, black, mask, seed=3)
    dw, db, dm = _dev(white), _dev(black), _dev(mask)
    out, _ = ctx.enblend(dw, db, dm, out=db, seed=3)
    assert np.array_equal(db.cpu().numpy(), ref["out"])


# ---- against the reference's own code (tests/golden/make_golden.py) ------------

def _golden():
    from pathlib import Path
    return np.load(Path(__file__).resolve().parent / "golden" / "reference_pyramid.npz")


@pytest.mark.parametrize("mode", ["fused", "plain"])
def test_reference_golden_enblend(ctx, mode):
    """The collapsed level 0 of the CUDA blend equals the reference's
    pyramid.h/blend.h result on the stored cases (alpha holes, mask 128, wrap)."""
    g = _golden()
    for k in range(int(g["enblend_count"])):
        levels, wrap = (int(v) for v in g[f"enblend{k}_meta"])
        W, B = g[f"enblend{k}_white"], g[f"enblend{k}_black"]
        h, w, _ = W.shape
        l0 = torch.zeros((h, w, 3), dtype=torch.int32, device="cuda")
        ctx.enblend(_dev(W), _dev(B), _dev(g[f"enblend{k}_mask"]), white_alpha=_dev(g[f"enblend{k}_white_alpha"]),
                    black_alpha=_dev(g[f"enblend{k}_black_alpha"]), levels=levels, wrap=bool(wrap), level0=l0,
                    plain=(mode == "plain"))
        assert np.array_equal(l0.cpu().numpy(), g[f"enblend{k}_level0"]), k


def test_reference_golden_reduce_expand(ctx):
    import enbgpu
    g = _golden()
    for k in range(int(g["step_count"])):
        bits, wrap, alpha_on = (int(v) for v in g[f"reduce{k}_meta"])
        dt = "i16" if bits == 8 else "i32"
        src = g[f"reduce{k}_src"]
        h, w, c = src.shape
        p = _pyr(ctx, enbgpu, w, h, c, dt)
        p.write(0, np.transpose(src, (2, 0, 1)))
        if alpha_on:
            da = torch.zeros(((h + 1) >> 1, (w + 1) >> 1), dtype=torch.uint8, device="cuda")
            ctx.reduce(p, 0, p, 1, wrap=bool(wrap), src_alpha=_dev(g[f"reduce{k}_alpha"]), dst_alpha=da)
            assert np.array_equal(da.cpu().numpy(), g[f"reduce{k}_dst_alpha"]), k
        else:
            ctx.reduce(p, 0, p, 1, wrap=bool(wrap))
        assert np.array_equal(_hwc(p.read(1)), g[f"reduce{k}_dst"]), k
        for add, key in ((False, "sub"), (True, "add")):
            q = _pyr(ctx, enbgpu, w, h, c, dt)
            q.write(0, np.transpose(g[f"expand{k}_dst"], (2, 0, 1)))
            q.write(1, np.transpose(g[f"expand{k}_src"], (2, 0, 1)))
            ctx.expand(q, 1, q, 0, add=add, wrap=bool(wrap))
            assert np.array_equal(_hwc(q.read(0)), g[f"expand{k}_{key}"]), (k, key)


@pytest.mark.parametrize("dt", [np.uint8, np.uint16])
@pytest.mark.parametrize("planes", [False, True])
def test_enblend_host_bands(ctx, orc, dt, planes):
    """Host buffers: inputs copied in 256-row bands while the level-1 reduces
    run, output copied back in 512-row bands (1100 rows: 5 and 3 bands)."""
    from enbgpu import synthetic
    white, black, mask = synthetic.panorama_pair(1100, 300, 200, dt, seed=41)
    mask[100:700, 210:240] = 90
    kw = {}
    if planes:
        wa, ba = orc.alpha_of(white).copy(), orc.alpha_of(black)
        wa[300:340, 220:260] = 0
        white, black = np.ascontiguousarray(white[..., :3]), np.ascontiguousarray(black[..., :3])
        kw = dict(white_alpha=wa, black_alpha=ba)
    ref = orc.enblend(white, black, mask, seed=6, want_level0=True, **kw)
    l0 = np.zeros(black.shape[:2] + (3,), np.int32)
    out, oa = ctx.enblend(white, black, mask, seed=6, level0=l0, **kw)
    assert np.array_equal(l0, ref["level0"])
    assert np.array_equal(out, ref["out"])
    assert np.array_equal(oa, ref["alpha"])
