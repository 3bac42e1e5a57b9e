"""The CUDA adjoint (enb_fuse_grad) against the FP64 reference model.

oracle/adjoint_ref.py restates the differentiable float enfuse in float64
torch operators (its forward agrees with the C oracle, its autograd with
central differences: tests/test_cpu_adjoint_ref.py).  The CUDA forward runs in
FP32, so the tolerances are: the loss and the fused image to 1e-5 / 1e-4
relative; the gradients to 1e-4 relative, where a per-pixel logit gradient
far below the map's largest is held to 1e-4 of that largest instead.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from oracle import adjoint_ref as ar  # noqa: E402


def _scene(K=4, h=72, w=96, seed=7, stops=8.0):
    from enbgpu import synthetic
    lr = synthetic.log_radiance(h, w, stops, seed=seed)
    evs = np.linspace(-(K - 1) / 2.0, (K - 1) / 2.0, K)
    imgs = np.stack([synthetic.expose(lr, ev, np.float32) for ev in evs])
    rad = np.exp2(lr)
    target = ((rad / (1.0 + rad)) ** (1.0 / 2.2)).astype(np.float32)
    return imgs, target


def _gpu(ctx, imgs, target, logits, theta, fn="gaussian"):
    import enbgpu
    dev = [torch.from_numpy(x).cuda() for x in imgs]
    t = torch.from_numpy(target).cuda()
    lg = [torch.from_numpy(x.astype(np.float32)).cuda() for x in logits]
    gl = [torch.zeros_like(x) for x in lg]
    out = torch.zeros_like(dev[0])
    prm = enbgpu.enfuse_params(exposure_optimum=theta[0], exposure_width=theta[1], exposure_weight=theta[2],
                               saturation_weight=theta[3], contrast_weight=theta[4], exposure_weight_function=fn,
                               float_range=1.0)
    r = ctx.fuse_grad(dev, t, params=prm, logits=lg, grad_logits=gl, out=out)
    return r, np.stack([g.cpu().numpy() for g in gl]), out.cpu().numpy()


@pytest.mark.parametrize("fn", ["gaussian", "lorentzian", "halfsine"])
def test_adjoint_matches_fp64_autograd_and_differences(ctx, fn):
    imgs, target = _scene()
    rng = np.random.default_rng(11)
    logits = rng.normal(0.0, 0.3, imgs.shape[:3])
    theta = [0.5, 0.2, 1.0, 0.2, 0.5]
    r, gl, out = _gpu(ctx, imgs, target, logits, theta, fn)
    x = torch.from_numpy(imgs.astype(np.float64))
    t = torch.from_numpy(target.astype(np.float64))
    lg = torch.from_numpy(logits).requires_grad_(True)
    th = torch.tensor(theta, dtype=torch.float64, requires_grad=True)
    ref_out = ar.fuse(x, lg, th, fn=fn)
    loss = ((ref_out - t) ** 2).mean()
    loss.backward()
    assert abs(r["loss"] - loss.item()) <= 1e-5 * loss.item()
    assert np.allclose(out, ref_out.detach().numpy(), rtol=1e-4, atol=1e-5)
    gt = np.array([r["d_exp_optimum"], r["d_exp_width"], r["d_w_exposure"], r["d_w_saturation"], r["d_w_contrast"]])
    at = th.grad.numpy()
    assert np.all(np.abs(gt - at) <= 1e-4 * np.abs(at) + 1e-6 * np.abs(at).max()), (gt, at)
    al = lg.grad.numpy()
    scale = np.abs(al).max()
    assert np.all(np.abs(gl - al) <= 1e-4 * np.abs(al) + 1e-4 * scale)
    # FP64 central differences (step 1e-6) on 32 coordinates
    K, H, W = imgs.shape[:3]
    coords = [("theta", i) for i in range(5)] + [("logit", int(rng.integers(K)), int(rng.integers(H)),
                                                 int(rng.integers(W))) for _ in range(27)]
    fd = ar.central_differences(x, torch.from_numpy(logits), torch.tensor(theta, dtype=torch.float64), t, coords,
                                step=1e-6, fn=fn)
    ours = np.array([gt[c[1]] if c[0] == "theta" else gl[c[1], c[2], c[3]] for c in coords])
    tol = np.where([c[0] == "theta" for c in coords], 1e-4 * np.abs(fd) + 1e-6 * np.abs(gt).max(),
                   1e-4 * np.abs(fd) + 1e-4 * scale)
    assert np.all(np.abs(ours - fd) <= tol), (ours, fd)


def test_autograd_function_wrapper(ctx):
    """The thin torch.autograd.Function returns enb_fuse_grad's gradients."""
    from enbgpu.autograd import FuseLoss
    imgs, target = _scene(K=3, h=40, w=64, seed=9)
    dev = [torch.from_numpy(x).cuda() for x in imgs]
    t = torch.from_numpy(target).cuda()
    logits = torch.zeros((3, 40, 64), device="cuda", requires_grad=True)
    theta = torch.tensor([0.5, 0.2, 1.0, 0.2, 0.5], dtype=torch.float64, requires_grad=True)
    loss = FuseLoss.apply(logits, theta, ctx, dev, t, {})
    loss.backward()
    r, gl, _ = _gpu(ctx, imgs, target, np.zeros((3, 40, 64)), [0.5, 0.2, 1.0, 0.2, 0.5])
    assert float(loss) == pytest.approx(r["loss"], rel=1e-12)
    assert np.allclose(logits.grad.cpu().numpy(), gl, rtol=0, atol=0)
    assert theta.grad[0].item() == pytest.approx(r["d_exp_optimum"], rel=1e-12)


def test_adjoint_rejects_entropy(ctx):
    import enbgpu
    imgs, target = _scene(K=2, h=24, w=24)
    dev = [torch.from_numpy(x).cuda() for x in imgs]
    with pytest.raises(enbgpu.EnbError):
        ctx.fuse_grad(dev, torch.from_numpy(target).cuda(), params=enbgpu.enfuse_params(entropy_weight=0.3))
