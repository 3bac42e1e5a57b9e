"""The enfuse / enblend command-line front ends (C++ over the C ABI).

CPU tests: both front ends build, parse the reference's options into the
library's parameters (--dry-run prints them), reject the options this build
does not provide with a message, and the image files they read and write
(uncompressed TIFF, .npy) round-trip.  The GPU test runs them on files."""
import json
import subprocess
from pathlib import Path

import numpy as np
import pytest


@pytest.fixture(scope="module")
def bins():
    import enbgpu  # noqa: F401  (paths)
    from enbgpu import _build
    return {p.name: p for p in _build.build_frontends()}


def _run(binary, *args, check=True):
    r = subprocess.run([str(binary), *args], capture_output=True, text=True, timeout=60)
    if check:
        assert r.returncode == 0, r.stderr
    return r


def test_enfuse_options_parse_like_the_reference(bins):
    """src/enfuse.cc: weights clamped to [0, 1], windows made odd and >= 3,
    cutoffs as values or percentages with the projectors, levels and wrap."""
    r = _run(bins["enbgpu-enfuse"], "--dry-run", "--exposure-weight=0.7", "--saturation-weight=1.5",
             "--contrast-weight=0.5", "--entropy-weight=0.3", "--exposure-optimum=0.4", "--exposure-width=0.25",
             "--exposure-weight-function=bi-square", "--contrast-window-size=6", "--entropy-window-size=2",
             "--exposure-cutoff=5%:250:lightness:value", "--entropy-cutoff=10%:-5%", "--gray-projector=luminance",
             "--hard-mask", "-l", "-2", "--wrap=horizontal", "-o", "out.tif", "a.tif", "b.tif", "c.tif")
    p = json.loads(r.stdout)
    assert p["w_exposure"] == 0.7 and p["w_saturation"] == 1.0 and p["w_contrast"] == 0.5
    assert "greater than 1" in r.stderr
    assert p["exp_optimum"] == 0.4 and p["exp_width"] == 0.25 and p["exp_function"] == 4
    assert p["contrast_window"] == 7 and p["entropy_window"] == 3
    assert p["exp_cutoff"] == [[5.0, True], [250.0, False]] and p["exp_cutoff_projectors"] == [3, 1]
    assert p["ent_cutoff"] == [[10.0, True], [-5.0, True]]
    assert p["gray_projector"] == 4 and p["hard_mask"] == 1 and p["levels"] == -2 and p["wrap"] == 1
    assert p["inputs"] == 3 and p["output"] == "out.tif"


def test_enfuse_mask_templates_and_defaults(bins):
    p = json.loads(_run(bins["enbgpu-enfuse"], "--dry-run", "--save-masks=w-%n.npy:h-%n.npy", "x.npy").stdout)
    assert p["save_masks"] and p["soft_template"] == "w-%n.npy" and p["hard_template"] == "h-%n.npy"
    p = json.loads(_run(bins["enbgpu-enfuse"], "--dry-run", "x.npy").stdout)
    # enfuse.cc:117-160 defaults
    assert (p["w_exposure"], p["w_saturation"], p["w_contrast"], p["w_entropy"]) == (1.0, 0.0, 0.0, 0.0)
    assert (p["contrast_window"], p["entropy_window"], p["levels"], p["wrap"]) == (5, 3, 0, 0)
    assert p["exp_cutoff"] == [[0.0, True], [100.0, True]] and p["exp_cutoff_projectors"] == [2, 1]


@pytest.mark.parametrize("args,msg", [
    (["--gpu"], "not supported"),
    (["--blend-colorspace=cielab"], "ICC"),
    (["--gray-projector=l-star"], "not supported"),
    (["--exposure-weight-function=./plugin.so"], "unknown built-in"),
    (["--contrast-edge-scale=0.3"], "not supported"),
    (["--levels=abc"], "integer"),
    (["--wrap=diagonal"], "wrap-around"),
    (["--no-such-option"], "unknown option"),
])
def test_enfuse_rejects_unsupported_options(bins, args, msg):
    r = _run(bins["enbgpu-enfuse"], "--dry-run", *args, "x.tif", check=False)
    assert r.returncode == 1 and msg in r.stderr


def test_enblend_options(bins):
    p = json.loads(_run(bins["enbgpu-enblend"], "--dry-run", "--load-masks=seam-%n.tif", "-l", "7", "-w",
                        "a.tif", "b.tif").stdout)
    assert p == {"levels": 7, "wrap": 1, "mask_template": "seam-%n.tif", "output": "a.tif", "inputs": 2}
    r = _run(bins["enbgpu-enblend"], "--dry-run", "a.tif", "b.tif", check=False)
    assert r.returncode == 1 and "--load-masks" in r.stderr
    r = _run(bins["enbgpu-enblend"], "--dry-run", "--load-masks", "--fine-mask", "a.tif", "b.tif", check=False)
    assert r.returncode == 1 and "seam" in r.stderr


CONVERT = r"""
#include "image_io.hpp"
int main(int argc, char** argv) { enbfront::write_image(argv[2], enbfront::read_image(argv[1])); return 0; }
"""


@pytest.mark.parametrize("dtype,S", [(np.uint8, 3), (np.uint16, 4), (np.float32, 1), (np.uint16, 2)])
def test_image_files_round_trip(bins, tmp_path, dtype, S):
    """The front ends' reader and writer: .npy -> TIFF -> .npy keeps every
    sample; the TIFF is little-endian baseline (uncompressed, chunky) with the
    extra sample marked as alpha."""
    from enbgpu import _build
    src = tmp_path / "convert.cpp"
    src.write_text(CONVERT)
    exe = tmp_path / "convert"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(_build.ROOT / "frontend"), str(src),
                    str(_build.ROOT / "frontend" / "image_io.cpp"), "-o", str(exe)], check=True)
    rng = np.random.default_rng(3)
    shape = (11, 17, S) if S > 1 else (11, 17)
    img = (rng.random(shape) * (1.0 if dtype == np.float32 else np.iinfo(dtype).max)).astype(dtype)
    np.save(tmp_path / "a.npy", img)
    subprocess.run([str(exe), str(tmp_path / "a.npy"), str(tmp_path / "b.tif")], check=True)
    subprocess.run([str(exe), str(tmp_path / "b.tif"), str(tmp_path / "c.npy")], check=True)
    back = np.load(tmp_path / "c.npy")
    assert back.dtype == img.dtype and np.array_equal(back, img)
    raw = (tmp_path / "b.tif").read_bytes()
    assert raw[:4] == b"II*\x00"
    ifd = int.from_bytes(raw[4:8], "little")
    tags = {int.from_bytes(raw[ifd + 2 + 12 * i: ifd + 4 + 12 * i], "little")
            for i in range(int.from_bytes(raw[ifd:ifd + 2], "little"))}
    assert {256, 257, 258, 259, 262, 273, 277, 278, 279, 284, 339} <= tags
    assert (338 in tags) == (S in (2, 4))
