"""The FP64 reference of the differentiable float enfuse (oracle/adjoint_ref.py).

Its forward at zero logits is the float enfuse of the C oracle (which follows
the reference's code) up to the masks' 9.15 quantisation that the
differentiable model drops; its autograd gradients agree with FP64 central
differences.  These two checks make it the checker of the CUDA adjoint.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import adjoint_ref as ar  # noqa: E402


def _scene(K=3, h=40, w=52, seed=3):
    from enbgpu import synthetic
    lr = synthetic.log_radiance(h, w, 8.0, seed=seed)
    evs = np.linspace(-(K - 1), K - 1, K)
    imgs = np.stack([synthetic.expose(lr, ev, np.float32) for ev in evs])
    rad = np.exp2(lr)
    target = (rad / (1.0 + rad)) ** (1.0 / 2.2)
    return imgs, target


def test_forward_matches_oracle_enfuse(orc):
    imgs, _ = _scene()
    kw = dict(exposure_weight=1.0, saturation_weight=0.2, contrast_weight=0.5, contrast_window_size=5)
    ref = orc.enfuse_f(list(imgs), prm=orc.params(**kw), range_=1.0)["out"]
    theta = torch.tensor([0.5, 0.2, 1.0, 0.2, 0.5], dtype=torch.float64)
    out = ar.fuse(torch.from_numpy(imgs.astype(np.float64)), torch.zeros(imgs.shape[:3], dtype=torch.float64), theta)
    # the masks differ by their quantisation to 1/(255 * 2^15): well below 1e-4 of the pixels
    assert np.allclose(out.numpy(), ref, rtol=1e-4, atol=1e-5)


@pytest.mark.parametrize("fn", ["gaussian", "lorentzian", "bisquare"])
def test_autograd_matches_central_differences(fn):
    imgs, target = _scene(K=3, h=24, w=30, seed=5)
    x = torch.from_numpy(imgs.astype(np.float64))
    t = torch.from_numpy(target)
    rng = np.random.default_rng(1)
    logits = torch.from_numpy(rng.normal(0.0, 0.3, imgs.shape[:3]))
    theta = torch.tensor([0.45, 0.25, 1.0, 0.2, 0.5], dtype=torch.float64)
    lg = logits.clone().requires_grad_(True)
    th = theta.clone().requires_grad_(True)
    ar.loss(x, lg, th, t, fn=fn).backward()
    coords = [("theta", i) for i in range(5)] + [("logit", int(rng.integers(3)), int(rng.integers(24)),
                                                 int(rng.integers(30))) for _ in range(6)]
    fd = ar.central_differences(x, logits, theta, t, coords, step=1e-6, fn=fn)
    ad = np.array([float(th.grad[c[1]]) if c[0] == "theta" else float(lg.grad[c[1], c[2], c[3]]) for c in coords])
    scale = np.abs(ad).max()
    assert np.all(np.abs(fd - ad) <= 1e-6 * np.abs(ad) + 1e-7 * scale), (fd, ad)
