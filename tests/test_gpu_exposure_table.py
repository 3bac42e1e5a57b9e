"""User-defined exposure weight functions on the GPU: the function's values at
the sample values (enb_enfuse_params.exposure_table) replace the built-in
function in the weights of 8- and 16-bit images, bit-exact against the oracle
given the same table (weights, collapsed level 0, dithered pixels), also under
the exposure cutoff; float images and tables of the wrong size are rejected;
and the enfuse front end loads a shared-object weight function, tabulates it
and gives the oracle's output."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _tent(y, opt=0.5, width=0.2):
    """The `tent` object of tests/cpp/exposure_weights.cc in the same double operations."""
    t = 1.0 - abs((y - opt) / width) / 4.0
    return t if t > 0.0 else 0.0


def _stack(dt, h=83, w=117, K=4, seed=3):
    from enbgpu import synthetic
    return synthetic.exposure_stack(h, w, list(np.linspace(-3.0, 3.0, K)), dt, 8.0, seed=seed)


@pytest.mark.parametrize("dt", [np.uint8, np.uint16])
@pytest.mark.parametrize("cutoff", [False, True])
def test_exposure_table_enfuse_against_oracle(ctx, orc, dt, cutoff):
    import enbgpu
    bits = 8 if dt == np.uint8 else 16
    table = enbgpu.exposure_table_of(_tent, bits)
    kw = dict(saturation_weight=0.2, contrast_weight=0.3, entropy_weight=0.1, entropy_window_size=5)
    if cutoff:
        kw["exposure_cutoff"] = ((5.0, True), (90.0, True))
    imgs = _stack(dt)
    h, w = imgs[0].shape[:2]
    dev = [torch.from_numpy(x).cuda() for x in imgs]
    prm = enbgpu.enfuse_params(exposure_table=table, **kw)
    oprm = orc.params(exposure_table=table, **kw)
    # the weights of one image
    wt = torch.zeros((h, w), dtype=torch.float32, device="cuda")
    ctx.enfuse_mask(dev[1], None, wt, params=prm)
    assert np.array_equal(wt.cpu().numpy(), orc.enfuse_mask(imgs[1], None, oprm))
    # the fused driver
    l0 = torch.zeros((h, w, 3), dtype=torch.int32, device="cuda")
    out, oa = ctx.enfuse(dev, params=prm, level0=l0, seed=11)
    ref = orc.enfuse(imgs, None, oprm, seed=11, want_level0=True)
    assert np.array_equal(l0.cpu().numpy(), ref["level0"])
    assert np.array_equal(out.cpu().numpy(), ref["out"])
    assert np.array_equal(oa.cpu().numpy(), ref["alpha"])
    # and the table differs from the built-in Gaussian in the result
    built_in = orc.enfuse(imgs, None, orc.params(**kw), seed=11)
    assert not np.array_equal(built_in["out"], ref["out"])


def test_exposure_table_rejections(ctx):
    import enbgpu
    imgs = _stack(np.uint8, 40, 40, 2)
    dev = [torch.from_numpy(x).cuda() for x in imgs]
    with pytest.raises(enbgpu.EnbError):  # 16-bit table for 8-bit images
        ctx.enfuse(dev, params=enbgpu.enfuse_params(exposure_table=enbgpu.exposure_table_of(_tent, 16)))
    fl = [torch.from_numpy(x.astype(np.float32) / 255.0).cuda() for x in imgs]
    with pytest.raises(enbgpu.EnbError):  # float images have no table
        ctx.enfuse(fl, params=enbgpu.enfuse_params(exposure_table=enbgpu.exposure_table_of(_tent, 8)))
    # without the exposure weight the table is not read (src/enfuse.cc:1913)
    out, _ = ctx.enfuse(dev, params=enbgpu.enfuse_params(exposure_weight=0.0, saturation_weight=1.0,
                                                         exposure_table=np.zeros(3)))
    assert out.shape == dev[0].shape


@pytest.mark.parametrize("dt", [np.uint8, np.uint16])
def test_front_end_shared_object_weight(orc, tmp_path, dt):
    """enbgpu-enfuse --exposure-weight-function=SO:tent on .npy files."""
    import subprocess
    import enbgpu
    from enbgpu import _build
    from test_cpu_frontend import build_weight_plugin
    bins = {p.name: p for p in _build.build_frontends()}
    so = build_weight_plugin(tmp_path)
    imgs = _stack(dt, 70, 96, 3, seed=8)
    files = []
    for i, x in enumerate(imgs):
        files.append(str(tmp_path / f"in{i}.npy"))
        np.save(files[-1], x)
    out = tmp_path / "out.npy"
    r = subprocess.run([str(bins["enbgpu-enfuse"]), "--saturation-weight=0.2", f"--exposure-weight-function={so}:tent",
                        "-o", str(out), *files], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    table = enbgpu.exposure_table_of(_tent, 8 if dt == np.uint8 else 16)
    ref = orc.enfuse(imgs, None, orc.params(saturation_weight=0.2, exposure_table=table), seed=0x5eed)
    got = np.load(out)
    assert np.array_equal(got[..., :3], ref["out"])
