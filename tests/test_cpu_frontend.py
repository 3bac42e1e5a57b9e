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
    assert p == {"levels": 7, "wrap": 1, "mask_template": "seam-%n.tif", "output": "a.tif", "inputs": 2,
                 "seams": "loaded", "save_masks": False}
    # the reference's default seams (coarse mask, optimised) are not built
    r = _run(bins["enbgpu-enblend"], "--dry-run", "a.tif", "b.tif", check=False)
    assert r.returncode == 1 and "--fine-mask --no-optimize" in r.stderr and "--load-masks" in r.stderr
    r = _run(bins["enbgpu-enblend"], "--dry-run", "--fine-mask", "a.tif", "b.tif", check=False)
    assert r.returncode == 1 and "optimisation" in r.stderr
    p = json.loads(_run(bins["enbgpu-enblend"], "--dry-run", "--fine-mask", "--no-optimize", "--save-masks=s-%n.npy",
                        "a.tif", "b.tif", "c.tif").stdout)
    assert p["seams"] == "nearest-feature" and p["save_masks"] and p["mask_template"] == "s-%n.npy"
    r = _run(bins["enbgpu-enblend"], "--dry-run", "--load-masks", "--save-masks", "a.tif", "b.tif", check=False)
    assert r.returncode == 1 and "exclude" in r.stderr
    r = _run(bins["enbgpu-enblend"], "--dry-run", "--fine-mask", "--no-optimize", "--primary-seam-generator=gc",
             "a.tif", "b.tif", check=False)
    assert r.returncode == 1 and "not supported" in r.stderr


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


# ---- user-defined exposure weight functions (shared objects) ----------------

REPO = Path(__file__).resolve().parents[1]


def build_weight_plugin(tmp: Path) -> Path:
    """tests/cpp/exposure_weights.cc as a shared object (the interface header
    include/enbgpu_exposure_weight.hpp)."""
    so = tmp / "exposure_weights.so"
    subprocess.run(["g++", "-std=c++17", "-O2", "-shared", "-fPIC", "-I", str(REPO / "include"),
                    str(REPO / "tests" / "cpp" / "exposure_weights.cc"), "-o", str(so)], check=True)
    return so


@pytest.fixture(scope="module")
def plugin(tmp_path_factory):
    return build_weight_plugin(tmp_path_factory.mktemp("plugin"))


def test_user_exposure_weight_function_loads(bins, plugin):
    """SHARED-OBJECT:SYMBOL[:ARGUMENT...]: the object is initialised with the
    optimum, the width and the arguments (src/exposure_weight.cc:96-129)."""
    import math
    r = _run(bins["enbgpu-enfuse"], "--dry-run", "--exposure-optimum=0.4", "--exposure-width=0.3",
             f"--exposure-weight-function={plugin}:cosine_power:3", "x.tif")
    u = json.loads(r.stdout)["user_weight"]
    assert u["symbol"] == "cosine_power" and u["arguments"] == ["3"]

    def cosp(y):
        z = abs((y - 0.4) / 0.3)
        return 0.0 if z >= 1.5707963267948966 else math.pow(math.cos(z), 3.0)
    assert u["samples"] == [cosp(i / 4.0) for i in range(5)]
    u = json.loads(_run(bins["enbgpu-enfuse"], "--dry-run", f"--exposure-weight-function={plugin};tent",
                        "x.tif").stdout)["user_weight"]
    assert u["samples"] == [max(1.0 - abs((i / 4.0 - 0.5) / 0.2) / 4.0, 0.0) for i in range(5)]
    # not loaded without the exposure weight (src/enfuse.cc:1913)
    p = json.loads(_run(bins["enbgpu-enfuse"], "--dry-run", "--exposure-weight=0",
                        f"--exposure-weight-function={plugin}:negative", "x.tif").stdout)
    assert "user_weight" not in p


@pytest.mark.parametrize("spec,msg", [
    ("negative", "at least one weight is negative"),
    ("above_one", "at least one weight is larger than one"),
    ("all_zero", "too many zeros"),
    ("old_interface", "matches interface version 1, but enbgpu-enfuse requires version 2"),
    ("cosine_power:abc", "raised exception: exponent is not a number"),
    ("cosine_power:9", "raised exception: exponent outside (0, 8]"),
    ("no_such_symbol", "not found in shared object"),
])
def test_user_exposure_weight_function_rejected(bins, plugin, spec, msg):
    """The reference's checks (src/exposure_weight.cc:54-66, 237-264, src/enfuse.cc:1920-1945)."""
    r = _run(bins["enbgpu-enfuse"], "--dry-run", f"--exposure-weight-function={plugin}:{spec}", "x.tif", check=False)
    assert r.returncode == 1 and msg in r.stderr, r.stderr


def test_user_exposure_weight_missing_library(bins, tmp_path):
    r = _run(bins["enbgpu-enfuse"], "--dry-run", f"--exposure-weight-function={tmp_path}/none.so:f", "x.tif",
             check=False)
    assert r.returncode == 1 and "cannot load" in r.stderr


def test_reference_example_plugin_loads(bins, tmp_path):
    """The reference's own example weight function (doc/examples/enfuse/
    variable_power.cc), compiled against the reference's exposure_weight_base.h,
    loads into this front end: the interface classes agree in layout."""
    from oracle import reference_build as ref
    if not ref.available():
        pytest.skip("reference tree not present")
    import math
    src = ref.REF_SRC.parent / "doc" / "examples" / "enfuse" / "variable_power.cc"
    so = tmp_path / "variable_power.so"
    subprocess.run(["g++", "-std=c++17", "-O2", "-shared", "-fPIC", "-I", str(ref.REF_SRC), str(src), "-o", str(so)],
                   check=True)
    u = json.loads(_run(bins["enbgpu-enfuse"], "--dry-run", f"--exposure-weight-function={so}:vpower:3",
                        "x.tif").stdout)["user_weight"]
    # max(1 - |(y - opt) / w'|^e, 0), w' = width * FWHM_gauss / (2 / exp(ln 2 / e))
    wp = 0.2 * 2.3548200450309493820231386529193992755 / (2.0 / math.exp(math.log(2.0) / 3.0))
    want = [max(1.0 - math.pow(abs((i / 4.0 - 0.5) / wp), 3.0), 0.0) for i in range(5)]
    assert u["samples"] == pytest.approx(want, rel=1e-14, abs=1e-15)
