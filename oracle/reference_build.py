"""Build and binding of the reference-code oracle.

TEST INFRASTRUCTURE ONLY.  Compiles the reference's own code, unmodified and
in place in the reference tree, against the project's VIGRA/GSL/LCMS2 shims
(oracle/refshim/):
  * oracle/_ref/libenb_ref.so: the pyramid, blend and fixed-point code
    (src/pyramid.h, src/blend.h, src/fixmath.h, src/numerictraits.h,
    src/openmp_vigra.h, src/minimizer.cc, src/mersenne.cc) with
    ref_driver.cpp as the C entry points;
  * oracle/_ref/libenb_ref_enfuse.so: enfuse itself (src/enfuse.h with
    enfuseMask and enfuseMain, src/assemble.h, src/mga.h,
    src/exposure_weight.h, src/alternativepercentage.cc, src/parameter.cc,
    src/error_message.cc) with ref_enfuse.cpp as the C entry points;
  * oracle/_ref/libenb_ref_nft.so: enblend's nearest-feature seam mask
    (src/nearest.h and the distance transform of src/openmp_vigra.h, built
    with OPENMP defined as the reference's OpenMP build is) with ref_nft.cpp
    as the C entry point.
They pin the C restatement in enb_oracle.c (and through it the CUDA path) to
the reference's code; the committed fixtures under tests/golden/ carry that
pin to machines without the reference tree.

The reference tree is found through the ENB_REFERENCE_SRC environment
variable (its src/ directory), else as reference/src beside the directory
that holds this repository.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path
from typing import Optional

import numpy as np

HERE = Path(__file__).resolve().parent
REF_SRC = Path(os.environ.get("ENB_REFERENCE_SRC") or HERE.parents[1] / "reference" / "src")
OUT_DIR = HERE / "_ref"
LIB_PATH = OUT_DIR / "libenb_ref.so"
ENFUSE_LIB_PATH = OUT_DIR / "libenb_ref_enfuse.so"
SHIM = HERE / "refshim"
SOURCES = [HERE / "ref_driver.cpp", SHIM / "gsl_shim.cpp"]
REF_UNITS = ["minimizer.cc", "mersenne.cc"]
ENFUSE_SOURCES = [HERE / "ref_enfuse.cpp", SHIM / "gsl_shim.cpp"]
ENFUSE_REF_UNITS = ["minimizer.cc", "mersenne.cc", "alternativepercentage.cc", "parameter.cc", "error_message.cc"]
NFT_LIB_PATH = OUT_DIR / "libenb_ref_nft.so"
NFT_SOURCES = [HERE / "ref_nft.cpp"]
NFT_REF_UNITS = ["parameter.cc", "error_message.cc", "timer.cc", "filenameparse.cc"]


def available() -> bool:
    """The reference tree is present (it is not on the GPU machines)."""
    return (REF_SRC / "pyramid.h").exists()


def _deps(sources):
    return list(sources) + sorted(SHIM.rglob("*.h")) + sorted(SHIM.rglob("*.hxx"))


def _compile(path: Path, sources, units, force: bool, defines=()) -> Path:
    if not force and path.exists() and all(path.stat().st_mtime >= d.stat().st_mtime for d in _deps(sources)):
        return path
    OUT_DIR.mkdir(exist_ok=True)
    tmp = path.with_suffix(".so.tmp")
    cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", "-fPIC", "-shared", "-DHAVE_CONFIG_H"] + list(defines) + [
           "-Wno-deprecated-declarations", "-I", str(SHIM), "-I", str(REF_SRC),
           "-I", str(REF_SRC / "layer_selection"), "-o", str(tmp)]
    cmd += [str(s) for s in sources] + [str(REF_SRC / u) for u in units]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("reference oracle build failed:\n" + res.stderr[-4000:])
    os.replace(tmp, path)
    return path


def build_if_available(force: bool = False) -> Optional[Path]:
    """Compile libenb_ref.so and libenb_ref_enfuse.so when the reference tree
    is present; None otherwise."""
    if not available():
        return None
    _compile(ENFUSE_LIB_PATH, ENFUSE_SOURCES, ENFUSE_REF_UNITS, force)
    _compile(NFT_LIB_PATH, NFT_SOURCES, NFT_REF_UNITS, force, ("-DOPENMP",))
    return _compile(LIB_PATH, SOURCES, REF_UNITS, force)


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


# ---- enfuse: the reference's enfuseMask and enfuseMain ----------------------

class RefEnfuseParams(ctypes.Structure):
    """ref_enfuse_params of ref_enfuse.cpp: enfuse's weighting options."""
    _fields_ = [("w_exposure", ctypes.c_double), ("w_saturation", ctypes.c_double),
                ("w_contrast", ctypes.c_double), ("w_entropy", ctypes.c_double),
                ("exp_optimum", ctypes.c_double), ("exp_width", ctypes.c_double),
                ("exp_function", ctypes.c_int32), ("contrast_window", ctypes.c_int32),
                ("entropy_window", ctypes.c_int32), ("hard_mask", ctypes.c_int32),
                ("exp_cutoff", ctypes.c_double * 2), ("exp_cutoff_pct", ctypes.c_int32 * 2),
                ("ent_cutoff", ctypes.c_double * 2), ("ent_cutoff_pct", ctypes.c_int32 * 2),
                ("gray_projector", ctypes.c_char * 96), ("exp_cutoff_projector", (ctypes.c_char * 32) * 2)]


EXPOSURE_FUNCTIONS = {"gaussian": 0, "lorentzian": 1, "halfsine": 2, "fullsine": 3, "bisquare": 4}

_elib = None


def enfuse_lib() -> Optional[ctypes.CDLL]:
    global _elib
    if _elib is None:
        if build_if_available() is None:
            return None
        L = ctypes.CDLL(str(ENFUSE_LIB_PATH))
        vp, i = ctypes.c_void_p, ctypes.c_int
        L.ref_enfuse_mask.argtypes = [ctypes.POINTER(RefEnfuseParams), i, i, vp, vp, i, i, vp]
        L.ref_enfuse_main.argtypes = [ctypes.POINTER(RefEnfuseParams), i, i, i, ctypes.POINTER(vp), i, i, i, i,
                                      ctypes.POINTER(vp), ctypes.c_longlong, vp, vp]
        _elib = L
    return _elib


def enfuse_params(exposure_weight=1.0, saturation_weight=0.0, contrast_weight=0.0, entropy_weight=0.0,
                  exposure_optimum=0.5, exposure_width=0.2, exposure_weight_function="gaussian",
                  contrast_window_size=5, entropy_window_size=3, gray_projector="", hard_mask=False,
                  exposure_cutoff=((0.0, True), (100.0, True)), exposure_cutoff_projectors=("anti-value", "value"),
                  entropy_cutoff=((0.0, True), (100.0, True))) -> RefEnfuseParams:
    """enfuse's options as the reference reads them (src/enfuse.cc:117-160): cutoffs are (value,
    is_percentage) pairs, lower then upper, as --exposure-cutoff / --entropy-cutoff set them."""
    p = RefEnfuseParams()
    p.w_exposure, p.w_saturation, p.w_contrast, p.w_entropy = (exposure_weight, saturation_weight,
                                                                contrast_weight, entropy_weight)
    p.exp_optimum, p.exp_width = exposure_optimum, exposure_width
    p.exp_function = EXPOSURE_FUNCTIONS[exposure_weight_function]
    p.contrast_window, p.entropy_window = contrast_window_size, entropy_window_size
    p.hard_mask = int(hard_mask)
    for j in range(2):
        p.exp_cutoff[j], p.exp_cutoff_pct[j] = exposure_cutoff[j][0], int(exposure_cutoff[j][1])
        p.ent_cutoff[j], p.ent_cutoff_pct[j] = entropy_cutoff[j][0], int(entropy_cutoff[j][1])
        p.exp_cutoff_projector[j].value = exposure_cutoff_projectors[j].encode()
    p.gray_projector = gray_projector.encode()
    return p


def _depth(a: np.ndarray) -> int:
    return {np.dtype(np.uint8): 8, np.dtype(np.uint16): 16, np.dtype(np.float32): 32}[a.dtype]


def enfuse_mask(img: np.ndarray, alpha: Optional[np.ndarray], prm: RefEnfuseParams) -> np.ndarray:
    """The reference's enfuseMask (src/enfuse.h:962-1212) of an (H, W, 3) or (H, W) image."""
    img = np.ascontiguousarray(img)
    h, w = img.shape[:2]
    C = img.shape[2] if img.ndim == 3 else 1
    out = np.zeros((h, w), np.float32)
    a = np.ascontiguousarray(alpha, np.uint8) if alpha is not None else None
    if enfuse_lib().ref_enfuse_mask(ctypes.byref(prm), _depth(img), C, _p(img), _p(a), w, h, _p(out)):
        raise ValueError("reference enfuseMask failed")
    return out


def enfuse_main(images, prm: RefEnfuseParams, levels: int = 0, wrap: bool = False, masks=None,
                dither: int = -1, save_masks: bool = False):
    """The reference's enfuseMain (src/enfuse.h:1217-1617) on K union-sized images of one type:
    (H, W, 3) RGB, (H, W, 4) RGBA (alpha thresholded on import), (H, W) gray.  masks: K (H, W) float32
    weight planes for --load-masks.  dither: -1 the Mersenne-Twister draws, else every draw returns it.
    Returns {"out": image (C colour samples), "alpha": 0/1 union alpha, "masks": (K, H, W) saved soft
    (or hard) masks or None}."""
    imgs = [np.ascontiguousarray(x) for x in images]
    K = len(imgs)
    h, w = imgs[0].shape[:2]
    S = imgs[0].shape[2] if imgs[0].ndim == 3 else 1
    C = 3 if S >= 3 else 1
    out = np.zeros((h, w, C + 1), imgs[0].dtype)
    ptrs = (ctypes.c_void_p * K)(*[x.ctypes.data for x in imgs])
    mks = None
    if masks is not None:
        ms = [np.ascontiguousarray(m, np.float32) for m in masks]
        mks = (ctypes.c_void_p * K)(*[m.ctypes.data for m in ms])
    saved = np.zeros((K, h, w), np.float32) if save_masks else None
    rc = enfuse_lib().ref_enfuse_main(ctypes.byref(prm), _depth(imgs[0]), S, K, ptrs, w, h, levels, int(wrap),
                                      mks, dither, _p(out), _p(saved))
    if rc:
        raise ValueError(f"reference enfuseMain failed ({rc})")
    img = out[..., :C] if C == 3 else out[..., 0]
    return {"out": np.ascontiguousarray(img), "alpha": (out[..., C] != 0).astype(np.uint8), "masks": saved}


_nlib = None


def nft_mask(white_alpha: np.ndarray, black_alpha: np.ndarray, wrap: bool = False) -> Optional[np.ndarray]:
    """The reference's nearest-feature seam mask of two alpha planes (255
    where the white image wins); None where the reference exits for
    excessive overlap."""
    global _nlib
    if _nlib is None:
        if build_if_available() is None:
            raise RuntimeError("the reference tree is not present")
        L = ctypes.CDLL(str(NFT_LIB_PATH))
        vp, i = ctypes.c_void_p, ctypes.c_int
        L.ref_nft_mask.argtypes = [vp, vp, i, i, i, vp]
        _nlib = L
    wa = np.ascontiguousarray(white_alpha, np.uint8)
    ba = np.ascontiguousarray(black_alpha, np.uint8)
    h, w = wa.shape
    m = np.zeros((h, w), np.uint8)
    rc = _nlib.ref_nft_mask(_p(wa), _p(ba), w, h, int(wrap), _p(m))
    if rc == 2:
        return None
    if rc:
        raise ValueError(f"ref_nft_mask failed ({rc})")
    return m
