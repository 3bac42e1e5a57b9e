"""Build of libenbgpu.so: the sm_103a kernels and the C ABI (include/enbgpu.h).

The library is built in-tree (next to this file) with nvcc for
``-gencode arch=compute_103a,code=sm_103a`` only; each translation unit is
compiled in parallel and then linked against the CUDA runtime.
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
ROOT = PKG_DIR.parent                      # enblend-enfuse_gb300/
REPO = ROOT.parent
CSRC = ROOT / "csrc"
INCLUDE = REPO / "include"
BUILD_DIR = ROOT / "_build"
LIB_PATH = PKG_DIR / "libenbgpu.so"

SOURCES = ["enb_kernels.cu", "enb_fused.cu", "enb_efuse.cu", "enb_nft.cu", "enb_coarse.cu", "enb_float.cu", "enb_batch.cu", "enb_adjoint.cu",
           "enb_api.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libenbgpu.so")
    return cand


def _stale() -> bool:
    if not LIB_PATH.exists():
        return True
    t = LIB_PATH.stat().st_mtime
    deps = [CSRC / s for s in SOURCES] + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [INCLUDE / "enbgpu.h"]
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile libenbgpu.so if it is missing or older than its sources."""
    if not force and not _stale():
        return LIB_PATH
    nvcc = _nvcc()
    BUILD_DIR.mkdir(exist_ok=True)
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-I", str(INCLUDE), "-I", str(CSRC)]
    if verbose:
        common += ["-Xptxas", "-v"]

    def compile_one(src: str) -> Path:
        obj = BUILD_DIR / (Path(src).stem + ".o")
        cmd = [nvcc] + common + ["-c", str(CSRC / src), "-o", str(obj)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{res.stderr}")
        if verbose and res.stderr:
            print(res.stderr)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB_PATH.with_suffix(".so.tmp")
    cmd = [nvcc] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objs] + ["-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


FRONTEND = ROOT / "frontend"
FRONTEND_BINS = {"enbgpu-enfuse": ["enfuse_main.cpp", "image_io.cpp"],
                 "enbgpu-enblend": ["enblend_main.cpp", "image_io.cpp"]}


def _cuda_home() -> Path:
    return Path(_nvcc()).resolve().parent.parent


def build_frontends(force: bool = False) -> list:
    """The enfuse / enblend command-line front ends (C++ host code over the
    C ABI), linked against libenbgpu.so next to them."""
    build(force)
    outs = []
    cuda = _cuda_home()
    for name, srcs in FRONTEND_BINS.items():
        out = PKG_DIR / name
        deps = [FRONTEND / x for x in srcs] + list(FRONTEND.glob("*.hpp")) + list(INCLUDE.glob("enbgpu*")) + [LIB_PATH]
        if force or not out.exists() or any(d.stat().st_mtime > out.stat().st_mtime for d in deps):
            tmp = out.with_name(out.name + ".tmp")
            cmd = ["g++", "-std=c++17", "-O2", "-I", str(INCLUDE), "-I", str(cuda / "include"), "-o", str(tmp)]
            cmd += [str(FRONTEND / x) for x in srcs]
            cmd += ["-L", str(PKG_DIR), "-lenbgpu", "-L", str(cuda / "lib64"), "-lcudart", "-ldl",
                    "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + str(cuda / "lib64")]
            res = subprocess.run(cmd, capture_output=True, text=True)
            if res.returncode != 0:
                raise RuntimeError(f"front end {name} failed to build:\n{res.stderr}")
            os.replace(tmp, out)
        outs.append(out)
    return outs


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
