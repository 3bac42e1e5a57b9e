"""The batched fuse of uneven float stacks (enb_fuse_stacks).

Each stack of a batch must come out as enb_enfuse makes it on its own (the
plain per-stack path: the same FP32 arithmetic, up to the order in which the
compiler may fuse multiply-adds, held to 1e-5 relative) and as the double
oracle makes it (1e-4 relative, as in the float-path tests).  The coarse-level
kernel and the graph replay must not change a single bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _close(got, ref, rtol, atol, what):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    err = np.abs(got - ref)
    bad = err > atol + rtol * np.abs(ref)
    assert not bad.any(), f"{what}: {bad.sum()} values off, max error {err.max():.3e}"


SHAPES = [(37, 53, 3), (130, 67, 5), (200, 151, 1), (64, 64, 7), (9, 7, 2), (300, 411, 4), (18, 33, 3)]


def _batch(seed=5, shapes=SHAPES):
    from enbgpu import synthetic
    stacks = []
    for i, (h, w, K) in enumerate(shapes):
        evs = np.linspace(-(K - 1), K - 1, K) if K > 1 else [0.0]
        stacks.append(synthetic.exposure_stack(h, w, evs, np.float32, 8.0, seed + i))
    return stacks


KW = dict(exposure_weight=1.0, saturation_weight=0.2, contrast_weight=0.5, entropy_weight=0.3,
          contrast_window_size=5, entropy_window_size=5)


def _params(**extra):
    import enbgpu
    kw = dict(KW)
    kw.update(extra)
    return enbgpu.enfuse_params(float_range=1.0, **kw)


@pytest.mark.parametrize("hard", [False, True])
@pytest.mark.parametrize("wrap", [False, True])
def test_batch_matches_plain_and_oracle(ctx, orc, hard, wrap):
    stacks = _batch()
    dev = [[_dev(x) for x in st] for st in stacks]
    p = _params()
    outs = ctx.fuse_stacks(dev, params=p, hard_mask=hard, wrap=wrap)
    plain = ctx.fuse_stacks(dev, params=p, hard_mask=hard, wrap=wrap, plain=True)
    for i, st in enumerate(stacks):
        got = outs[i].cpu().numpy()
        _close(got, plain[i].cpu().numpy(), 1e-5, 1e-6, f"stack {i} vs plain")
        ref = orc.enfuse_f(st, prm=orc.params(**KW), range_=1.0, hard_mask=hard, wrap=wrap)
        _close(got, ref["out"], 1e-4, 1e-5, f"stack {i} vs oracle")


@pytest.mark.parametrize("levels", [16, 256])
def test_batch_repeated_samples_bit_identical(ctx, orc, levels):
    """Samples quantised to a few levels, so that most entropy windows of
    every exposure hold repeated samples: the batched fuse equals the
    per-stack path bit for bit (the same weight arithmetic, whichever
    exposure of a tile is weighted), and the double oracle within 1e-4."""
    stacks = [[(np.round(x * levels) / levels).astype(np.float32) for x in st]
              for st in _batch(seed=41, shapes=[(120, 150, 5), (77, 301, 4), (260, 90, 7)])]
    dev = [[_dev(x) for x in st] for st in stacks]
    p = _params()
    outs = ctx.fuse_stacks(dev, params=p)
    plain = ctx.fuse_stacks(dev, params=p, plain=True)
    for i, st in enumerate(stacks):
        got = outs[i].cpu().numpy()
        assert np.array_equal(got, plain[i].cpu().numpy()), i
        ref = orc.enfuse_f(st, prm=orc.params(**KW), range_=1.0)
        _close(got, ref["out"], 1e-4, 1e-5, f"stack {i} vs oracle")


def test_batch_gray_stacks_bit_identical(ctx, orc):
    """One-channel float stacks: the batched fuse equals the per-stack path
    bit for bit, and the double oracle within 1e-4."""
    stacks = [[np.ascontiguousarray(x[..., 1]) for x in st]
              for st in _batch(seed=51, shapes=[(90, 130, 4), (61, 47, 3)])]
    dev = [[_dev(x) for x in st] for st in stacks]
    p = _params()
    outs = ctx.fuse_stacks(dev, params=p)
    plain = ctx.fuse_stacks(dev, params=p, plain=True)
    for i, st in enumerate(stacks):
        got = outs[i].cpu().numpy()
        assert np.array_equal(got, plain[i].cpu().numpy()), i
        ref = orc.enfuse_f(st, prm=orc.params(**KW), range_=1.0)
        _close(got, ref["out"], 1e-4, 1e-5, f"stack {i} vs oracle")


def test_batch_coarse_and_graph_bit_identical(ctx):
    stacks = _batch(seed=11)
    dev = [[_dev(x) for x in st] for st in stacks]
    p = _params()
    base = [o.cpu().numpy() for o in ctx.fuse_stacks(dev, params=p, graph=False, coarse_pixels=-1)]
    for kw in (dict(graph=True), dict(graph=True, coarse_pixels=1 << 30), dict(graph=False, coarse_pixels=256),
               dict(graph=True)):
        outs = ctx.fuse_stacks(dev, params=p, **kw)
        for i in range(len(stacks)):
            assert np.array_equal(outs[i].cpu().numpy(), base[i]), (kw, i)


def test_batch_rgba_alphas_and_host_buffers(ctx, orc):
    rng = np.random.default_rng(3)
    stacks = _batch(seed=21, shapes=[(41, 60, 3), (90, 77, 4)])
    rgba, alphas = [], []
    for st in stacks:
        h, w, _ = st[0].shape
        al = []
        imgs = []
        for k, x in enumerate(st):
            a = np.full((h, w), 255, np.uint8)
            a[rng.integers(0, h // 2):, : rng.integers(1, w // 3)] = 0 if k == 1 else 255
            al.append(a)
            imgs.append(np.concatenate([x, (a[..., None] / 255.0).astype(np.float32)], axis=2))
        rgba.append(imgs)
        alphas.append(al)
    p = _params()
    outs = [np.zeros_like(st[0]) for st in rgba]
    oalphas = [np.zeros(st[0].shape[:2], np.uint8) for st in rgba]
    ctx.fuse_stacks(rgba, params=p, outs=outs, out_alphas=oalphas, alphas=alphas)
    for i, st in enumerate(rgba):
        ref = orc.enfuse_f(st, alphas=alphas[i], prm=orc.params(**KW), range_=1.0)
        assert np.array_equal(oalphas[i], ref["alpha"])
        _close(outs[i], ref["out"], 1e-4, 1e-5, f"rgba stack {i}")
    # the same through device buffers
    dev_out = ctx.fuse_stacks([[_dev(x) for x in st] for st in rgba], params=p,
                              alphas=[[_dev(a) for a in al] for al in alphas])
    for i in range(len(rgba)):
        assert np.array_equal(dev_out[i].cpu().numpy(), outs[i])


def test_batch_reference_mode_weights(ctx, orc):
    """float_range 0: the reference's FLT_MAX scale (exposure weight constant)."""
    import enbgpu
    stacks = _batch(seed=31, shapes=[(50, 70, 3), (33, 45, 2)])
    dev = [[_dev(x) for x in st] for st in stacks]
    kw = dict(exposure_weight=1.0, saturation_weight=0.2, contrast_weight=0.5)
    outs = ctx.fuse_stacks(dev, params=enbgpu.enfuse_params(**kw))
    for i, st in enumerate(stacks):
        ref = orc.enfuse_f(st, prm=orc.params(**kw), range_=orc.FLT_MAX)
        _close(outs[i].cpu().numpy(), ref["out"], 1e-4, 1e-5, f"stack {i}")


def test_level_schedule_autotuner(ctx):
    """enb_fuse_stacks_tune times each candidate coarse threshold, keeps the
    fastest for the batch geometry, and later default calls on a batch of
    that geometry (other buffers) use it; every schedule gives the same bits."""
    stacks = _batch(seed=13)
    dev = [[_dev(x) for x in st] for st in stacks]
    p = _params()
    ref = [o.clone() for o in ctx.fuse_stacks(dev, params=p, coarse_pixels=-1)]
    cands = [-1, 256, 4096]
    r = ctx.tune_stacks(dev, params=p, candidates=cands, reps=1)
    assert r["best"] in cands and set(r["ms"]) == set(cands)
    assert all(t > 0 for t in r["ms"].values())
    assert r["ms"][r["best"]] == min(r["ms"].values())
    # same geometry, new buffers: the tuned schedule, the same result
    dev2 = [[x.clone() for x in st] for st in dev]
    outs = ctx.fuse_stacks(dev2, params=p)
    for a, b in zip(outs, ref):
        assert torch.equal(a, b)
    with pytest.raises(Exception):
        ctx.tune_stacks(dev, params=p, candidates=[0])
