"""The enfuse / enblend front ends on image files, on the GPU: their output
equals the oracle's for the same options (the dithered pixels with the
default seed) and carries the union alpha as its last band; --save-masks
writes the weights, which --load-masks reads back to the same result."""
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bins():
    from enbgpu import _build
    return {p.name: p for p in _build.build_frontends()}


def _run(binary, *args):
    r = subprocess.run([str(binary), *args], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    return r


@pytest.mark.parametrize("dt", [np.uint8, np.uint16])
def test_enfuse_front_end(bins, orc, tmp_path, dt):
    from enbgpu import synthetic
    imgs = synthetic.exposure_stack(90, 130, [-2.0, 0.0, 2.0], dt, 8.0, seed=5)
    files = []
    for i, x in enumerate(imgs):
        files.append(str(tmp_path / f"in{i}.npy"))
        np.save(files[-1], x)
    out = tmp_path / "out.tif"
    _run(bins["enbgpu-enfuse"], "--saturation-weight=0.2", "--contrast-weight=0.5", "--entropy-weight=0.3",
         "--entropy-window-size=5", "--save-masks=" + str(tmp_path / "w-%n.npy"), "-o", str(out), *files)
    ref = orc.enfuse(imgs, None, orc.params(saturation_weight=0.2, contrast_weight=0.5, entropy_weight=0.3,
                                           entropy_window_size=5), seed=0x5eed)
    conv = tmp_path / "out.npy"
    from enbgpu import _build  # noqa: F401
    # read the TIFF back through numpy: baseline little-endian, one strip
    raw = out.read_bytes()
    ifd = int.from_bytes(raw[4:8], "little")
    ent = {int.from_bytes(raw[ifd + 2 + 12 * i: ifd + 4 + 12 * i], "little"): ifd + 2 + 12 * i
           for i in range(int.from_bytes(raw[ifd:ifd + 2], "little"))}
    off = int.from_bytes(raw[ent[273] + 8: ent[273] + 12], "little")
    got = np.frombuffer(raw[off: off + 90 * 130 * 4 * np.dtype(dt).itemsize], dt).reshape(90, 130, 4)
    assert np.array_equal(got[..., :3], ref["out"])
    maxv = np.iinfo(dt).max
    assert np.array_equal(got[..., 3], np.where(ref["alpha"] != 0, maxv, 0).astype(dt))
    for i, x in enumerate(imgs):
        w = np.load(tmp_path / f"w-{i + 1}.npy")
        assert np.array_equal(w, orc.enfuse_mask(x, None, orc.params(saturation_weight=0.2, contrast_weight=0.5,
                                                                    entropy_weight=0.3, entropy_window_size=5)))
    _run(bins["enbgpu-enfuse"], "--load-masks=" + str(tmp_path / "w-%n.npy"), "-o", str(conv), *files)
    again = np.load(conv)
    assert np.array_equal(again[..., :3], ref["out"])


def test_enblend_front_end(bins, orc, tmp_path):
    from enbgpu import synthetic
    white, black, mask = synthetic.panorama_pair(70, 110, 60, np.uint16, seed=11)
    np.save(tmp_path / "black.npy", black)
    np.save(tmp_path / "white.npy", white)
    np.save(tmp_path / "seam-1.npy", mask)
    out = tmp_path / "out.npy"
    _run(bins["enbgpu-enblend"], "--load-masks=" + str(tmp_path / "seam-%n.npy"), "-o", str(out),
         str(tmp_path / "black.npy"), str(tmp_path / "white.npy"))
    ref = orc.enblend(white, black, mask, seed=0x5eed)
    got = np.load(out)
    assert np.array_equal(got[..., :3], ref["out"][..., :3])
    assert np.array_equal(got[..., 3] != 0, ref["alpha"] != 0)
