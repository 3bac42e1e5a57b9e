"""Build and binding of the reference-code oracle.

TEST INFRASTRUCTURE ONLY.  Compiles the reference's own pyramid, blend and
fixed-point code (src/pyramid.h, src/blend.h, src/fixmath.h,
src/numerictraits.h, src/openmp_vigra.h, src/minimizer.cc, src/mersenne.cc),
unmodified and in place in the reference tree, against the project's
VIGRA/GSL/LCMS2 shims (oracle/refshim/) into oracle/_ref/libenb_ref.so, with
ref_driver.cpp as the C entry points.  It pins the C restatement in
enb_oracle.c (and through it the CUDA path) to the reference's code; the
committed fixtures under tests/golden/ carry that pin to machines without the
reference tree.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path
from typing import Optional

import numpy as np

HERE = Path(__file__).resolve().parent
REF_SRC = Path(os.environ.get("ENB_REFERENCE_SRC", "/root/reference/src"))
OUT_DIR = HERE / "_ref"
LIB_PATH = OUT_DIR / "libenb_ref.so"
SHIM = HERE / "refshim"
SOURCES = [HERE / "ref_driver.cpp", SHIM / "gsl_shim.cpp"]
REF_UNITS = ["minimizer.cc", "mersenne.cc"]


def available() -> bool:
    """The reference tree is present (it is not on the GPU machines)."""
    return (REF_SRC / "pyramid.h").exists()


def _deps():
    return SOURCES + sorted(SHIM.rglob("*.h")) + sorted(SHIM.rglob("*.hxx"))


def build_if_available(force: bool = False) -> Optional[Path]:
    """Compile libenb_ref.so when the reference tree is present; None otherwise."""
    if not available():
        return None
    if not force and LIB_PATH.exists() and all(LIB_PATH.stat().st_mtime >= d.stat().st_mtime for d in _deps()):
        return LIB_PATH
    OUT_DIR.mkdir(exist_ok=True)
    tmp = LIB_PATH.with_suffix(".so.tmp")
    cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", "-fPIC", "-shared", "-DHAVE_CONFIG_H",
           "-Wno-deprecated-declarations", "-I", str(SHIM), "-I", str(REF_SRC), "-o", str(tmp)]
    cmd += [str(s) for s in SOURCES] + [str(REF_SRC / u) for u in REF_UNITS]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("reference oracle build failed:\n" + res.stderr[-4000:])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib() -> Optional[ctypes.CDLL]:
    global _lib
    if _lib is None:
        path = build_if_available()
        if path is None:
            return None
        L = ctypes.CDLL(str(path))
        vp, i = ctypes.c_void_p, ctypes.c_int
        L.ref_reduce.argtypes = [i, i, i, i, vp, vp, i, i, vp, vp]
        L.ref_expand.argtypes = [i, i, i, i, vp, i, i, vp, i, i]
        L.ref_enblend.argtypes = [i, i, i, vp, vp, vp, vp, vp, i, i, vp]
        L.ref_from_pyramid.argtypes = [i, vp, vp, i, i, vp]
        L.ref_reduce_f.argtypes = [i, i, i, vp, vp, i, i, vp, vp]
        L.ref_expand_f.argtypes = [i, i, i, vp, i, i, vp, i, i]
        L.ref_enblend_f.argtypes = [i, i, vp, vp, vp, vp, vp, i, i, vp, vp]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _ptype(bits: int):
    return np.int16 if bits == 8 else np.int32


def reduce(src: np.ndarray, alpha: Optional[np.ndarray], bits: int, wrap: bool = False):
    """Reduce of one (H, W, C) level of the bits-bit image pyramid (Int16 9.7 / Int32 17.7).
    Returns (dst, dst_alpha) with alpha, else dst (int32 arrays)."""
    h, w, C = src.shape
    s = np.ascontiguousarray(src.astype(_ptype(bits)))
    dh, dw = (h + 1) >> 1, (w + 1) >> 1
    d = np.zeros((dh, dw, C), _ptype(bits))
    da = np.zeros((dh, dw), np.uint8)
    a = np.ascontiguousarray(alpha, np.uint8) if alpha is not None else None
    if lib().ref_reduce(bits, C, int(alpha is not None), int(wrap), _p(s), _p(a), w, h, _p(d), _p(da)):
        raise ValueError("reference reduce failed")
    return (d.astype(np.int32), da) if alpha is not None else d.astype(np.int32)


def expand(src: np.ndarray, dst: np.ndarray, add: bool, bits: int, wrap: bool = False) -> np.ndarray:
    """Expand src into dst (add: collapse step; else Laplacian step)."""
    s = np.ascontiguousarray(src.astype(_ptype(bits)))
    d = np.ascontiguousarray(dst.astype(_ptype(bits)))
    sh, sw, C = s.shape
    dh, dw, _ = d.shape
    if lib().ref_expand(bits, C, int(add), int(wrap), _p(s), sw, sh, _p(d), dw, dh):
        raise ValueError("reference expand failed")
    return d.astype(np.int32)


def enblend_level0(white: np.ndarray, white_alpha: np.ndarray, black: np.ndarray, black_alpha: np.ndarray,
                   mask: np.ndarray, levels: int, wrap: bool = False) -> np.ndarray:
    """The collapsed level 0 of enblendMain's pyramid blend on (H, W, 3) RGB images."""
    h, w, _ = white.shape
    bits = 8 if white.dtype == np.uint8 else 16
    l0 = np.zeros((h, w, 3), np.int32)
    args = [np.ascontiguousarray(x) for x in (white, white_alpha, black, black_alpha, mask)]
    if lib().ref_enblend(bits, levels, int(wrap), *[_p(a) for a in args], w, h, _p(l0)):
        raise ValueError("reference enblend failed")
    return l0


def from_pyramid(level0: np.ndarray, alpha: np.ndarray, dtype, fill: int = 0) -> np.ndarray:
    """copyFromPyramidImageIf with the reference's dither draws; pixels with
    alpha 0 keep `fill`."""
    h, w, _ = level0.shape
    bits = 8 if np.dtype(dtype) == np.uint8 else 16
    out = np.full((h, w, 3), fill, dtype)
    l0 = np.ascontiguousarray(level0, np.int32)
    if lib().ref_from_pyramid(bits, _p(l0), _p(np.ascontiguousarray(alpha, np.uint8)), w, h, _p(out)):
        raise ValueError("reference conversion failed")
    return out


# ---- float images: double pyramids ------------------------------------------

def reduce_f(src: np.ndarray, alpha: Optional[np.ndarray], wrap: bool = False):
    """Reduce of one (H, W, C) double level of a float image's pyramid.
    Returns (dst, dst_alpha) with alpha, else dst (float64 arrays)."""
    s = np.ascontiguousarray(src, np.float64)
    h, w, C = s.shape
    dh, dw = (h + 1) >> 1, (w + 1) >> 1
    d = np.zeros((dh, dw, C), np.float64)
    da = np.zeros((dh, dw), np.uint8)
    a = np.ascontiguousarray(alpha, np.uint8) if alpha is not None else None
    if lib().ref_reduce_f(C, int(alpha is not None), int(wrap), _p(s), _p(a), w, h, _p(d), _p(da)):
        raise ValueError("reference reduce failed")
    return (d, da) if alpha is not None else d


def expand_f(src: np.ndarray, dst: np.ndarray, add: bool, wrap: bool = False) -> np.ndarray:
    s = np.ascontiguousarray(src, np.float64)
    d = np.array(dst, np.float64, copy=True, order="C")
    sh, sw, C = s.shape
    dh, dw, _ = d.shape
    if lib().ref_expand_f(C, int(add), int(wrap), _p(s), sw, sh, _p(d), dw, dh):
        raise ValueError("reference expand failed")
    return d


def enblend_f(white: np.ndarray, white_alpha: np.ndarray, black: np.ndarray, black_alpha: np.ndarray,
              mask: np.ndarray, levels: int, wrap: bool = False):
    """enblendMain's pyramid blend of (H, W, 3) float32 images.  Returns
    (collapsed double level 0, float output: black where the union alpha is 0)."""
    h, w, _ = white.shape
    l0 = np.zeros((h, w, 3), np.float64)
    out = np.array(black, np.float32, copy=True, order="C")
    args = [np.ascontiguousarray(x) for x in (white.astype(np.float32), white_alpha, black.astype(np.float32),
                                              black_alpha, mask)]
    if lib().ref_enblend_f(levels, int(wrap), *[_p(a) for a in args], w, h, _p(l0), _p(out)):
        raise ValueError("reference enblend failed")
    return l0, out
