"""CPU-side checks of the C ABI library: it loads, exports every symbol the
header declares, and its host-only logic matches the oracle (no GPU needed)."""
import ctypes

import numpy as np
import pytest


@pytest.fixture(scope="module")
def lib():
    from enbgpu import _build
    _build.build()
    import enbgpu
    return enbgpu.load_library()


def test_exports_every_header_symbol(lib):
    import enbgpu
    names = enbgpu.header_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version(lib):
    assert lib.enb_abi_version() == 6


def test_num_levels_matches_oracle(lib, orc):
    rng = np.random.default_rng(0)
    sizes = [(1, 1), (8, 8), (9, 9), (16, 17), (768, 1024), (3072, 6963), (4000, 6000), (2048, 2048)]
    sizes += [tuple(rng.integers(1, 20000, 2)) for _ in range(200)]
    for h, w in sizes:
        for exact in (0, 1, 3, 50, -1, -4, -100):
            assert lib.enb_num_levels(int(w), int(h), 1, exact) == orc.num_levels(int(w), int(h), 1, exact)


def test_level_counts_of_the_workloads(lib):
    # roiBounds: 768 -> 8, 3072 -> 10, 4000 -> 10, 2048 -> 9 levels
    assert lib.enb_num_levels(1024, 768, 1, 0) == 8
    assert lib.enb_num_levels(6963, 3072, 1, 0) == 10
    assert lib.enb_num_levels(6000, 4000, 1, 0) == 10
    assert lib.enb_num_levels(2048, 2048, 1, 0) == 9


def test_defaults_match_enfuse_cli(lib):
    import enbgpu
    p = enbgpu.EnbEnfuseParams()
    lib.enb_default_enfuse_params(ctypes.byref(p))
    assert (p.w_exposure, p.w_saturation, p.w_contrast, p.w_entropy) == (1.0, 0.0, 0.0, 0.0)
    assert (p.exp_optimum, p.exp_width) == (0.5, 0.2)
    assert (p.contrast_window, p.entropy_window) == (5, 3)


def test_create_without_device_fails_cleanly(lib):
    """No CUDA device in this container: enb_create reports ENB_ERR_CUDA, never falls back."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    h = ctypes.c_void_p()
    assert lib.enb_create(0, ctypes.byref(h)) == 3
    assert not h.value


def test_null_context_is_rejected(lib):
    assert lib.enb_synchronize(None) == 1
    assert lib.enb_destroy(None) == 1
    # the batched fuse, its autotuner and the adjoint reject a null context before any device work
    assert lib.enb_fuse_stacks(None, None, 0, None, None) == 1
    assert lib.enb_fuse_stacks_tune(None, None, 0, None, None, None, 0, 1, None, None) == 1
    assert lib.enb_fuse_grad(None, None, 0, None, None, None, None, None, None, None) == 1


def test_device_only_wrappers_reject_host_arrays():
    """The autotuner and the adjoint take device tensors only: host arrays are refused before any call."""
    import enbgpu
    c = enbgpu.Context.__new__(enbgpu.Context)   # no device needed for the argument check
    with pytest.raises(TypeError):
        enbgpu.Context.tune_stacks(c, [[np.zeros((8, 8, 3), np.float32)]])
    with pytest.raises(TypeError):
        enbgpu.Context.fuse_grad(c, [np.zeros((8, 8, 3), np.float32)], np.zeros((8, 8, 3), np.float32))


@pytest.mark.parametrize("lang", ["c", "c++"])
def test_header_is_plain_c(lang, tmp_path):
    """include/enbgpu.h compiles as C99 and as C++ on its own (a C ABI: no CUDA
    or C++ types in the signatures)."""
    import shutil
    import subprocess
    from pathlib import Path
    cc = shutil.which("gcc" if lang == "c" else "g++")
    if not cc:
        pytest.skip("no host compiler")
    inc = Path(__file__).resolve().parents[1] / "include"
    src = tmp_path / ("t.c" if lang == "c" else "t.cpp")
    src.write_text('#include "enbgpu.h"\nint main(void) { return enb_abi_version() == ENBGPU_ABI_VERSION ? 0 : 1; }\n')
    std = ["-std=c99"] if lang == "c" else ["-std=c++11"]
    r = subprocess.run([cc, *std, "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I", str(inc), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
