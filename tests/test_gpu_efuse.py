"""The fused enfuse driver (enb_efuse.cu) against the oracle and against the
per-operation pass structure (enb_fuse_options.plain).

The fused passes must give the same integers as the reference's pass
structure: the collapsed level 0 and the dithered pixels are compared bit for
bit.  Cases cover 8- and 16-bit RGB, RGBA (alpha thresholded from the 4th
component), gray and explicit alpha planes, 1 to 16 exposures, odd and tiny
canvases (2 to 9 pyramid levels), wrap-around, the hard mask, --load-masks and
the exposure and entropy cutoffs; more than 16 exposures take the
per-operation passes.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

W_ALL = dict(exposure_weight=1.0, saturation_weight=0.2, contrast_weight=0.5, entropy_weight=0.3,
             contrast_window_size=5, entropy_window_size=5)


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _stack(dt, h, w, K, seed, S=3):
    from enbgpu import synthetic
    imgs = synthetic.exposure_stack(h, w, list(np.linspace(-3.0, 3.0, K)), dt, 8.0, seed=seed)
    if S == 4:
        rng = np.random.default_rng(seed)
        top = np.iinfo(dt).max
        imgs = [np.concatenate([x, np.full((h, w, 1), top, dt)], axis=2) for x in imgs]
        for i, x in enumerate(imgs):
            x[rng.random((h, w)) < 0.1, 3] = top // 3
            x[2 + i: 9 + i, 3:17, 3] = 0
    if S == 1:
        imgs = [np.ascontiguousarray(x[..., 1]) for x in imgs]
    return imgs


def _run(ctx, imgs, kw, **opt):
    import enbgpu
    h, w = imgs[0].shape[:2]
    C = 3 if imgs[0].ndim == 3 else 1
    l0 = torch.zeros((h, w, C), dtype=torch.int32, device="cuda")
    out, oa = ctx.enfuse([_dev(x) for x in imgs], params=enbgpu.enfuse_params(**kw) if kw is not None else None,
                         level0=l0, **opt)
    return l0.cpu().numpy(), out.cpu().numpy(), oa.cpu().numpy()


@pytest.mark.parametrize("dt", [np.uint8, np.uint16])
@pytest.mark.parametrize("S", [3, 4, 1])
@pytest.mark.parametrize("geom", [(75, 97, 3), (40, 33, 1), (6, 7, 2), (130, 257, 5), (33, 64, 16)])
def test_fused_enfuse_against_oracle(ctx, orc, dt, S, geom):
    h, w, K = geom
    imgs = _stack(dt, h, w, K, seed=h + w + K, S=S)
    kw = W_ALL if min(h, w) >= 5 else dict(exposure_weight=1.0, saturation_weight=0.2)
    ref = orc.enfuse(imgs, None, orc.params(**kw), seed=17, want_level0=True)
    ctx.profile(True)
    l0, out, oa = _run(ctx, imgs, kw, seed=17)
    names = set(ctx.profile_report())
    ctx.profile(False)
    # a canvas whose short side is at most 8 pixels has one pyramid level,
    # which the per-operation passes take
    assert ("ef_out0" in names) == (orc.num_levels(w, h) >= 2), names
    C = 3 if S != 1 else 1
    assert np.array_equal(l0 if C == 3 else l0[..., 0], ref["level0"] if C == 3 else ref["level0"][..., 0])
    assert np.array_equal(oa, ref["alpha"])
    assert np.array_equal(out, ref["out"])


@pytest.mark.parametrize("dt", [np.uint8, np.uint16])
@pytest.mark.parametrize("variant", ["hard", "wrap", "levels3", "alpha_planes", "cutoffs", "nearest"])
def test_fused_enfuse_equals_plain_passes(ctx, dt, variant):
    """The fused passes and one kernel per reference operation give the same bits."""
    h, w, K = 61, 83, 4
    imgs = _stack(dt, h, w, K, seed=5)
    kw, opt = dict(W_ALL), {}
    if variant == "hard":
        opt["hard_mask"] = True
    elif variant == "wrap":
        opt["wrap"] = True
    elif variant == "levels3":
        opt["levels"] = 3
    elif variant == "alpha_planes":
        rng = np.random.default_rng(9)
        opt["alphas"] = [_dev(((rng.random((h, w)) < 0.9) * 255).astype(np.uint8)) for _ in range(K)]
    elif variant == "cutoffs":
        kw.update(exposure_cutoff=((5.0, True), (95.0, True)), entropy_cutoff=((10.0, True), (90.0, True)))
    elif variant == "nearest":
        opt["dither"] = "nearest"
    a = _run(ctx, imgs, kw, seed=3, **opt)
    b = _run(ctx, imgs, kw, seed=3, plain=True, **opt)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("dt", [np.uint8, np.uint16])
@pytest.mark.parametrize("hard", [False, True])
def test_fused_enfuse_loaded_masks(ctx, orc, dt, hard):
    """--load-masks: the weights come from the caller; all-zero weights take
    the integer 255/K fallback (soft) or 255/K (hard)."""
    h, w, K = 50, 66, 3
    imgs = _stack(dt, h, w, K, seed=22)
    rng = np.random.default_rng(4)
    masks = [rng.random((h, w)).astype(np.float32) for _ in imgs]
    for m in masks:
        m[:5, :7] = 0.0
    ref = orc.enfuse(imgs, None, masks=masks, hard_mask=hard, seed=5, want_level0=True)
    l0, out, oa = _run(ctx, imgs, None, masks=[_dev(m) for m in masks], hard_mask=hard, seed=5)
    assert np.array_equal(l0, ref["level0"])
    assert np.array_equal(out, ref["out"])
    assert np.array_equal(oa, ref["alpha"])


def test_more_than_sixteen_exposures_take_the_plain_passes(ctx, orc):
    h, w, K = 24, 31, 17
    imgs = _stack(np.uint8, h, w, K, seed=8)
    kw = dict(exposure_weight=1.0, saturation_weight=0.2)
    ref = orc.enfuse(imgs, None, orc.params(**kw), seed=2, want_level0=True)
    ctx.profile(True)
    l0, out, oa = _run(ctx, imgs, kw, seed=2)
    names = set(ctx.profile_report())
    ctx.profile(False)
    assert "ef_out0" not in names
    assert np.array_equal(l0, ref["level0"])
    assert np.array_equal(out, ref["out"])


@pytest.mark.parametrize("dt", [np.uint8, np.uint16])
def test_fused_enfuse_host_buffers(ctx, orc, dt):
    h, w, K = 45, 70, 3
    imgs = _stack(dt, h, w, K, seed=12, S=4)
    ref = orc.enfuse(imgs, None, orc.params(**W_ALL), seed=6)
    import enbgpu
    out, oa = ctx.enfuse(imgs, params=enbgpu.enfuse_params(**W_ALL), seed=6)
    assert np.array_equal(out, ref["out"])
    assert np.array_equal(oa, ref["alpha"])
