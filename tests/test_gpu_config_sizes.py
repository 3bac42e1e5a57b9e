"""Parity at the full sizes of the benchmark workloads, on the benchmark's own
inputs (the same scene generators and seeds as bench.py):

  enfuse 3 x 1024x768 RGB u8 (exposure 1.0, saturation 0.2): the collapsed
      level 0, the dithered pixels and the output alpha bit-exact against the
      oracle;
  enblend 2 x 4096x3072 RGBA u16 on the 6963x3072 union canvas: level 0,
      pixels and alpha bit-exact against the oracle;
  enfuse 9 x 6000x4000 RGB u16 (exposure 1.0, saturation 0.2, contrast 0.5
      in 5x5, entropy 0.3 in 5x5): level 0, pixels and alpha bit-exact
      against the oracle (about half a minute of the oracle on 16 cores);
  the differentiable fuse, 8 x 2048x2048 FP32 RGB with logit maps at 0: the
      loss, the fused image and every gradient against the FP64 autograd
      model (run by torch in float64 on the GPU as the checker), and the
      gradients against FP64 central differences (step 1e-6) on 32 random
      coordinates, to 1e-4 relative.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

import bench  # noqa: E402  (the workload definitions)


def _enfuse_full(ctx, orc, name):
    import enbgpu
    from enbgpu import synthetic
    sp = bench.ENFUSE_WORKLOADS[name]
    h, w, K = sp["h"], sp["w"], len(sp["evs"])
    imgs = synthetic.exposure_stack_torch(h, w, sp["evs"], sp["dtype"], sp["stops"], sp["seed"], sp["noise"])
    l0 = torch.zeros((h, w, 3), dtype=torch.int32, device="cuda")
    ctx.profile(True)
    out, oa = ctx.enfuse(imgs, params=enbgpu.enfuse_params(**sp["kw"]), level0=l0, seed=17)
    names = set(ctx.profile_report())
    ctx.profile(False)
    assert "ef_out0" in names and "ef_weights" in names, names   # the fused driver ran
    host = [x.cpu().numpy() for x in imgs]
    del imgs
    ref = orc.enfuse(host, None, orc.params(**sp["kw"]), seed=17, want_level0=True)
    assert np.array_equal(l0.cpu().numpy(), ref["level0"])
    assert np.array_equal(oa.cpu().numpy(), ref["alpha"])
    assert np.array_equal(out.cpu().numpy(), ref["out"])


def test_enfuse_3x1024x768_u8_full_size(ctx, orc):
    _enfuse_full(ctx, orc, "enfuse_3x1024x768_u8")


def test_enfuse_9x6000x4000_u16_full_size(ctx, orc):
    _enfuse_full(ctx, orc, "enfuse_9x6000x4000_u16")


def test_enblend_2x4096x3072_u16_full_size(ctx, orc):
    """The headline workload: bench.make_inputs with bench's default seed."""
    white, black, mask = bench.make_inputs(2)
    h, w = mask.shape
    assert (h, w) == (3072, 6963)
    l0 = torch.zeros((h, w, 3), dtype=torch.int32, device="cuda")
    dev = [torch.from_numpy(x).cuda() for x in (white, black, mask)]
    out, oa = ctx.enblend(*dev, seed=9, level0=l0)
    ref = orc.enblend(white, black, mask, seed=9, want_level0=True)
    assert np.array_equal(l0.cpu().numpy(), ref["level0"])
    assert np.array_equal(oa.cpu().numpy(), ref["alpha"])
    assert np.array_equal(out.cpu().numpy(), ref["out"])
    # and through the host-buffer entry point the benchmark's e2e leg times
    out2, oa2 = ctx.enblend(white, black, mask, seed=9)
    assert np.array_equal(np.asarray(out2), ref["out"])
    assert np.array_equal(np.asarray(oa2), ref["alpha"])


def test_adjoint_8x2048x2048_full_size(ctx):
    import enbgpu
    from enbgpu import synthetic
    from oracle import adjoint_ref as ar
    h = w = 2048
    lr = synthetic.log_radiance_torch(h, w, 8.0, seed=5)
    evs = np.arange(-3.5, 3.6, 1.0)
    imgs = [synthetic.expose_torch(lr, ev) for ev in evs]
    rad = torch.exp2(lr)
    target = ((rad / (1.0 + rad)) ** (1.0 / 2.2)).float().contiguous()
    del lr, rad
    K = len(imgs)
    theta = [0.5, 0.2, 1.0, 0.2, 0.5]
    logits = [torch.zeros((h, w), device="cuda") for _ in range(K)]
    grads = [torch.zeros_like(x) for x in logits]
    out = torch.zeros_like(imgs[0])
    prm = enbgpu.enfuse_params(exposure_optimum=theta[0], exposure_width=theta[1], exposure_weight=theta[2],
                               saturation_weight=theta[3], contrast_weight=theta[4], contrast_window_size=5,
                               float_range=1.0)
    r = ctx.fuse_grad(imgs, target, params=prm, logits=logits, grad_logits=grads, out=out)
    gl = torch.stack(grads).double()
    # the FP64 model, on the GPU in float64
    x = torch.stack(imgs).double()
    t = target.double()
    del imgs
    lg = torch.zeros((K, h, w), dtype=torch.float64, device="cuda", requires_grad=True)
    th = torch.tensor(theta, dtype=torch.float64, device="cuda", requires_grad=True)
    ref_out = ar.fuse(x, lg, th)
    loss = ((ref_out - t) ** 2).mean()
    loss.backward()
    assert abs(r["loss"] - loss.item()) <= 1e-5 * loss.item()
    assert torch.allclose(out.double(), ref_out.detach(), rtol=1e-4, atol=1e-5)
    gt = np.array([r["d_exp_optimum"], r["d_exp_width"], r["d_w_exposure"], r["d_w_saturation"], r["d_w_contrast"]])
    at = th.grad.cpu().numpy()
    assert np.all(np.abs(gt - at) <= 1e-4 * np.abs(at) + 1e-6 * np.abs(at).max()), (gt, at)
    al = lg.grad
    scale = al.abs().max().item()
    assert bool(((gl - al).abs() <= 1e-4 * al.abs() + 1e-4 * scale).all())
    del ref_out, loss
    # FP64 central differences (step 1e-6) on 32 coordinates: the 5
    # parameters and 27 logit samples
    rng = np.random.default_rng(23)
    coords = [("theta", i) for i in range(5)] + [("logit", int(rng.integers(K)), int(rng.integers(h)),
                                                 int(rng.integers(w))) for _ in range(27)]
    fd = ar.central_differences(x, lg.detach(), th.detach(), t, coords, step=1e-6)
    glh = gl.cpu().numpy()
    ours = np.array([gt[c[1]] if c[0] == "theta" else glh[c[1], c[2], c[3]] for c in coords])
    tol = np.where([c[0] == "theta" for c in coords], 1e-4 * np.abs(fd) + 1e-6 * np.abs(gt).max(),
                   1e-4 * np.abs(fd) + 1e-4 * scale)
    assert np.all(np.abs(ours - fd) <= tol), (ours, fd)
