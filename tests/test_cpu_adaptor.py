"""The header-only C++ adaptor (include/enbgpu.hpp): a program written like
the reference's enblendMain pyramid section against it compiles warning-free
and links to libenbgpu.so; without a GPU, Context throws enbgpu::Error with
ENB_ERR_CUDA (the program exits 2).  tests/test_gpu_adaptor.py runs it."""
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent


def build_adaptor_program(out_dir: Path) -> Path:
    from enbgpu import _build
    _build.build()
    cuda = _build._cuda_home()
    exe = out_dir / "adaptor_enblend"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", str(_build.INCLUDE),
                    "-I", str(cuda / "include"), str(HERE / "cpp" / "adaptor_enblend.cpp"), "-o", str(exe),
                    "-L", str(_build.PKG_DIR), "-lenbgpu", "-L", str(cuda / "lib64"), "-lcudart",
                    "-Wl,-rpath," + str(_build.PKG_DIR), "-Wl,-rpath," + str(cuda / "lib64")], check=True)
    return exe


def test_adaptor_compiles_and_reports_missing_gpu(tmp_path):
    torch = pytest.importorskip("torch")
    exe = build_adaptor_program(tmp_path)
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: tests/test_gpu_adaptor.py runs the program")
    r = subprocess.run([str(exe), "4", "4", "1", "w", "b", "m", "o"], capture_output=True, text=True)
    assert r.returncode == 2 and "enb_create" in r.stderr
