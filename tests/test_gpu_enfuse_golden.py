"""The CUDA enfuse weights and driver against the reference's own enfuse.

tests/golden/reference_enfuse.npz holds outputs of the reference's
enfuseMask and enfuseMain (src/enfuse.h compiled unmodified against the
project's shims by oracle/reference_build.py; regenerated with
tests/golden/make_golden.py).  Integer images: the CUDA weights equal the
reference's bit for bit, and the CUDA driver's collapsed level 0, converted
under the two constant dither draws the reference ran with, gives the
reference's output pixels.  Float images: the weights are within the float
tolerance of this suite (1e-5 relative, 1e-7 of the map's largest weight);
the contrast window of float images is checked against the oracle's exact
double window sums, which the reference's float running sums differ from
(see test_cpu_reference_pin.py), and the float driver's output within the
float pyramids' tolerance.
"""
import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

G = np.load(Path(__file__).resolve().parent / "golden" / "reference_enfuse.npz")

W_RTOL, W_ATOL_REL = 1e-5, 1e-7   # float weights (as test_gpu_float.py)
OUT_TOL = 1e-4                     # float driver output pixels (computed weights)


def _gpu_params(opts, **extra):
    """enbgpu.enfuse_params of options in the reference driver's keyword form."""
    import enbgpu
    kw = {k: v for k, v in opts.items() if k != "hard_mask"}
    gp = kw.pop("gray_projector", "") or "average"
    if gp.startswith("channel-mixer"):
        kw["mixer"] = tuple(float(v) for v in gp.split(":")[1:4])
        gp = "channel-mixer"
    kw["gray_projector"] = gp
    for key in ("exposure_cutoff", "entropy_cutoff"):
        if key in kw:
            kw[key] = tuple(tuple(x) for x in kw[key])
    kw.update(extra)
    return enbgpu.enfuse_params(**kw)


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("k", range(int(G["mask_count"])))
def test_gpu_enfuse_mask_against_reference(ctx, orc, k):
    j = int(G[f"mask{k}_img"])
    img, alpha = G[f"maskimg{j}_image"], G[f"maskimg{j}_alpha"]
    opts = json.loads(str(G[f"mask{k}_opts"]))
    want = G[f"mask{k}_weight"]
    out = torch.zeros(img.shape[:2], dtype=torch.float32, device="cuda")
    ctx.enfuse_mask(_dev(img), _dev(alpha), out, params=_gpu_params(opts))
    got = out.cpu().numpy()
    if img.dtype != np.float32:
        assert np.array_equal(got, want)
        return
    if opts.get("contrast_weight", 0.0) > 0.0:
        # the reference's float running sums are not reproduced: exact sums
        want = orc.enfuse_mask_f(img, alpha, orc.params_from_options(opts))
    ref = want.astype(np.float64)
    err = np.abs(got.astype(np.float64) - ref)
    tol = W_RTOL * np.abs(ref) + W_ATOL_REL * np.nanmax(np.abs(ref))
    assert not (err > tol).any(), f"{int((err > tol).sum())} weights off, max error {err.max():.3e}"


@pytest.mark.parametrize("k", range(int(G["main_count"])))
def test_gpu_enfuse_driver_against_reference(ctx, orc, k):
    """The driver end to end (import threshold of RGBA inputs, weights or
    --load-masks, normalisation, hard mask, pyramids, merge, collapse): the
    collapsed level 0 converted under the reference's two constant dither
    draws equals the reference's output pixels; the union alpha is equal."""
    K, levels, wrap, load = (int(v) for v in G[f"main{k}_meta"])
    imgs = [G[f"main{k}_image{i}"] for i in range(K)]
    masks = [_dev(G[f"main{k}_mask{i}"]) for i in range(K)] if load else None
    opts = json.loads(str(G[f"main{k}_opts"]))
    hard = bool(opts.get("hard_mask", False))
    h, w = imgs[0].shape[:2]
    C = 3 if imgs[0].ndim == 3 else 1
    dev = [_dev(x) for x in imgs]
    if imgs[0].dtype == np.float32:
        out, oa = ctx.enfuse(dev, params=_gpu_params(opts), masks=masks, levels=levels, wrap=wrap, hard_mask=hard)
        got = out.cpu().numpy()[..., :C]
        want = G[f"main{k}_out0"]
        host = [np.ascontiguousarray(x) for x in imgs]
        if hard and masks is None:
            # a hard mask of float weights follows the argmax of weights that
            # are only tolerance-equal to the reference's: the merge is
            # checked on the CUDA weights (argmax ties decide alike)
            ws = []
            for d, x in zip(dev, host):
                wk = torch.zeros(x.shape[:2], dtype=torch.float32, device="cuda")
                ctx.enfuse_mask(d, _dev(orc.alpha_of(x)), wk, params=_gpu_params(opts))
                ws.append(wk.cpu().numpy())
            want = orc.enfuse_f(host, None, orc.params_from_options(opts), masks=ws, levels=levels, wrap=wrap,
                                hard_mask=True)["out"][..., :C]
        elif opts.get("contrast_weight", 0.0) > 0.0:
            # the contrast of float images against the oracle's exact window
            # sums (the reference's float running sums are not reproduced)
            want = orc.enfuse_f(host, None, orc.params_from_options(opts), masks=None if masks is None else
                                [m.cpu().numpy() for m in masks], levels=levels, wrap=wrap, hard_mask=hard)["out"]
            want = want[..., :C]
        assert np.array_equal((oa.cpu().numpy() != 0).astype(np.uint8), G[f"main{k}_alpha"])
        on = G[f"main{k}_alpha"] != 0
        err = np.abs(got - want)[on]
        assert err.max() <= OUT_TOL, err.max()
        return
    l0 = torch.zeros((h, w, C), dtype=torch.int32, device="cuda")
    out, oa = ctx.enfuse(dev, params=_gpu_params(opts), masks=masks, levels=levels, wrap=wrap, hard_mask=hard,
                         level0=l0)
    alpha = oa.cpu().numpy()
    assert np.array_equal((alpha != 0).astype(np.uint8), G[f"main{k}_alpha"])
    lv = l0.cpu().numpy() if C == 3 else l0.cpu().numpy()[..., 0]
    for j, draw in enumerate((0, 0xFFFFFFFF)):
        assert np.array_equal(orc.convert_with_draw(lv, alpha, imgs[0].dtype, draw), G[f"main{k}_out{j}"]), draw
