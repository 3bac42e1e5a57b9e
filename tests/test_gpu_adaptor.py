"""The header-only C++ adaptor on the GPU: the enblend pyramid section
written against it (tests/cpp/adaptor_enblend.cpp) equals the oracle's
enblend, pixel for pixel with the same dither seed."""
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_adaptor_enblend(orc, tmp_path):
    from test_cpu_adaptor import build_adaptor_program
    from enbgpu import synthetic
    exe = build_adaptor_program(tmp_path)
    white, black, mask = synthetic.panorama_pair(60, 90, 50, np.uint16, seed=21)
    W, B = np.ascontiguousarray(white[..., :3]), np.ascontiguousarray(black[..., :3])
    h, w = mask.shape
    wa = (W.sum(axis=2) > 0).astype(np.uint8) * 255
    ba = (B.sum(axis=2) > 0).astype(np.uint8) * 255
    levels = orc.num_levels(w, h)
    for name, a in (("w", W), ("b", B), ("m", mask)):
        np.ascontiguousarray(a).tofile(tmp_path / f"{name}.raw")
    r = subprocess.run([str(exe), str(w), str(h), str(levels)] +
                       [str(tmp_path / f"{n}.raw") for n in ("w", "b", "m", "o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(tmp_path / "o.raw", np.uint16).reshape(h, w, 3)
    ref = orc.enblend(W, B, mask, white_alpha=wa, black_alpha=ba, levels=levels, seed=0x5eed)
    assert np.array_equal(got, ref["out"])
