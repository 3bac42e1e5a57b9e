"""ctypes binding of the CPU oracle (enb_oracle.c).

TEST INFRASTRUCTURE ONLY: the parity checker of the CUDA path and the timed
CPU baseline ("port") of bench.py.  Only tests/, __graft_entry__.smoke() and
bench.py's cpu_baseline leg may import this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD_DIR = HERE / "_build"
LIB_PATH = BUILD_DIR / "libenb_oracle.so"
SOURCES = [HERE / "enb_oracle.c"]

ORC_U8, ORC_U16, ORC_F32 = 0, 1, 2
DITHER = {"hash": 0, "nearest": 1}
EXPOSURE_FUNCTIONS = {"gaussian": 0, "lorentzian": 1, "halfsine": 2, "fullsine": 3, "bisquare": 4}
GRAY_PROJECTORS = {"average": 0, "value": 1, "anti-value": 2, "lightness": 3, "luminance": 4,
                   "channel-mixer": 5}


class OrcParams(ctypes.Structure):
    _fields_ = [("w_exposure", ctypes.c_double), ("w_saturation", ctypes.c_double),
                ("w_contrast", ctypes.c_double), ("w_entropy", ctypes.c_double),
                ("exp_optimum", ctypes.c_double), ("exp_width", ctypes.c_double),
                ("exp_function", ctypes.c_int), ("contrast_window", ctypes.c_int),
                ("entropy_window", ctypes.c_int), ("gray_projector", ctypes.c_int),
                ("mixer", ctypes.c_double * 3),
                ("exp_cutoff", ctypes.c_double * 2), ("exp_cutoff_pct", ctypes.c_int * 2),
                ("exp_cutoff_proj", ctypes.c_int * 2),
                ("ent_cutoff", ctypes.c_double * 2), ("ent_cutoff_pct", ctypes.c_int * 2),
                ("float_sliding_sums", ctypes.c_int), ("exposure_table", ctypes.c_void_p)]


def build(force: bool = False) -> Path:
    """Compile the oracle with gcc: -O3 with OpenMP, no FP contraction and no
    fast-math (IEEE results as the reference's), and portable flags only
    (the same build runs on x86-64 and on Arm hosts)."""
    BUILD_DIR.mkdir(exist_ok=True)
    if not force and LIB_PATH.exists() and all(LIB_PATH.stat().st_mtime >= s.stat().st_mtime
                                               for s in SOURCES + [HERE / "enb_oracle.h"]):
        return LIB_PATH
    tmp = LIB_PATH.with_suffix(".so.tmp")
    cmd = ["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", "-o", str(tmp)] + [str(s) for s in SOURCES] + ["-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + res.stderr)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        L = ctypes.CDLL(str(build()))
        vp, i, i64, u64, dbl = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_uint64, ctypes.c_double
        L.orc_num_levels.argtypes = [i, i, i, i]
        L.orc_fixed_from_int.argtypes = [vp, i, i64, i, i, vp, i]
        L.orc_fixed_from_float.argtypes = [vp, i64, vp, i, i]
        L.orc_reduce_alpha.argtypes = [i, vp, vp, i, i, i, vp, vp, i]
        L.orc_reduce.argtypes = [i, vp, i, i, i, vp, i]
        L.orc_expand.argtypes = [i, i, vp, i, i, vp, i, i, i, i]
        L.orc_blend.argtypes = [vp, vp, vp, i64, i, ctypes.c_int32, i]
        L.orc_mask_multiply.argtypes = [vp, vp, i64, i, ctypes.c_int32, i]
        L.orc_accumulate.argtypes = [vp, vp, i64, i]
        L.orc_from_fixed.argtypes = [vp, vp, i64, i, vp, i, i, i, i, u64]
        L.orc_dither_bits.argtypes = [u64, u64, i, i, i]
        L.orc_dither_bits.restype = ctypes.c_uint32
        L.orc_enfuse_mask.argtypes = [vp, i, i, i, i, i, vp, ctypes.POINTER(OrcParams), vp]
        L.orc_local_stddev.argtypes = [vp, vp, i, i, i, vp]
        L.orc_local_entropy.argtypes = [vp, i, i, i, i, i, vp, i, vp]
        L.orc_enfuse.argtypes = [i, vp, vp, i, i, i, i, i, ctypes.POINTER(OrcParams), i, i, i, vp, vp, vp, i, u64,
                                 vp, vp]
        L.orc_enblend.argtypes = [vp, vp, vp, vp, vp, i, i, i, i, i, i, i, vp, vp, i, u64, vp]
        L.orc_real_to_pyramid.argtypes = [vp, i64, i, i, vp]
        L.orc_real_from_pyramid.argtypes = [vp, vp, i64, i, vp, i]
        L.orc_reduce_alpha_d.argtypes = [i, vp, vp, i, i, i, vp, vp]
        L.orc_expand_d.argtypes = [i, i, vp, i, i, vp, i, i, i]
        L.orc_blend_d.argtypes = [vp, vp, vp, i64, i, ctypes.c_int32]
        L.orc_mask_multiply_d.argtypes = [vp, vp, i64, i, ctypes.c_int32, vp]
        L.orc_enfuse_mask_f.argtypes = [vp, i, i, i, i, vp, ctypes.POINTER(OrcParams), dbl, vp]
        L.orc_enfuse_f.argtypes = [i, vp, vp, i, i, i, i, ctypes.POINTER(OrcParams), dbl, i, i, i, vp, vp, vp,
                                   vp, vp]
        L.orc_enblend_f.argtypes = [vp, vp, vp, vp, vp, i, i, i, i, i, i, vp, vp, vp]
        _lib = L
    return _lib


def _p(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


def _dtype(a: np.ndarray) -> int:
    return {np.dtype(np.uint8): ORC_U8, np.dtype(np.uint16): ORC_U16, np.dtype(np.float32): ORC_F32}[a.dtype]


def _geom(img: np.ndarray):
    img = np.ascontiguousarray(img)
    if img.ndim == 2:
        h, w = img.shape
        return img, w, h, 1, 1
    h, w, s = img.shape
    return img, w, h, (3 if s >= 3 else 1), s


def params(exposure_weight=1.0, saturation_weight=0.0, contrast_weight=0.0, entropy_weight=0.0,
           exposure_optimum=0.5, exposure_width=0.2, exposure_weight_function="gaussian",
           contrast_window_size=5, entropy_window_size=3, gray_projector="average",
           mixer=(0.0, 0.0, 0.0), exposure_cutoff=((0.0, True), (100.0, True)),
           exposure_cutoff_projectors=("anti-value", "value"), entropy_cutoff=((0.0, True), (100.0, True)),
           float_sliding_sums=False, exposure_table=None) -> OrcParams:
    """enfuse's weighting options.  Cutoffs are (value, is_percentage) pairs, lower then upper, as
    --exposure-cutoff and --entropy-cutoff give them; float_sliding_sums reproduces the reference's float
    rounding of the contrast windows of float images; exposure_table holds a user-defined exposure weight
    function's values at y = g / max (integer images)."""
    p = OrcParams()
    p.w_exposure, p.w_saturation, p.w_contrast, p.w_entropy = (exposure_weight, saturation_weight,
                                                               contrast_weight, entropy_weight)
    p.exp_optimum, p.exp_width = exposure_optimum, exposure_width
    p.exp_function = EXPOSURE_FUNCTIONS[exposure_weight_function]
    p.contrast_window, p.entropy_window = contrast_window_size, entropy_window_size
    p.gray_projector = GRAY_PROJECTORS[gray_projector]
    p.mixer[:] = list(mixer)
    for j in range(2):
        p.exp_cutoff[j], p.exp_cutoff_pct[j] = exposure_cutoff[j][0], int(exposure_cutoff[j][1])
        p.exp_cutoff_proj[j] = GRAY_PROJECTORS[exposure_cutoff_projectors[j]]
        p.ent_cutoff[j], p.ent_cutoff_pct[j] = entropy_cutoff[j][0], int(entropy_cutoff[j][1])
    p.float_sliding_sums = int(float_sliding_sums)
    if exposure_table is not None:
        t = np.ascontiguousarray(exposure_table, dtype=np.float64)
        p._exposure_table = t
        p.exposure_table = t.ctypes.data
    return p


def num_levels(w, h, min_levels=1, exact_levels=0) -> int:
    return lib().orc_num_levels(w, h, min_levels, exact_levels)


def alpha_of(img: np.ndarray) -> np.ndarray:
    """Alpha plane of an image: thresholded 4th component (src/assemble.h:240-253) or opaque."""
    if img.ndim == 3 and img.shape[2] == 4 and img.dtype == np.float32:
        a = img[..., 3]
        return np.where((a >= np.float32(0.5)) & (a <= np.float32(1.0)), 255, 0).astype(np.uint8)
    if img.ndim == 3 and img.shape[2] == 4:
        maxv = 255 if img.dtype == np.uint8 else 65535
        lo = int(maxv / 2.0)
        a = img[..., 3]
        return np.where((a >= lo) & (a <= maxv), 255, 0).astype(np.uint8)
    return np.full(img.shape[:2], 255, np.uint8)


def to_fixed(img: np.ndarray, frac: int = 7) -> np.ndarray:
    img, w, h, C, s = _geom(img)
    out = np.empty((h, w, C), np.int32)
    lib().orc_fixed_from_int(_p(img), _dtype(img), w * h, C, s, _p(out), frac)
    return out


def float_to_fixed(m: np.ndarray, frac: int, bits: int) -> np.ndarray:
    m = np.ascontiguousarray(m, np.float32)
    out = np.empty(m.shape, np.int32)
    lib().orc_fixed_from_float(_p(m), m.size, _p(out), frac, bits)
    return out


def reduce(src: np.ndarray, alpha: Optional[np.ndarray], bits: int, wrap: bool = False):
    """src: (H, W, C) int32. Returns dst (and dst alpha when alpha is given)."""
    src = np.ascontiguousarray(src, np.int32)
    h, w, C = src.shape
    dh, dw = (h + 1) >> 1, (w + 1) >> 1
    dst = np.empty((dh, dw, C), np.int32)
    if alpha is None:
        rc = lib().orc_reduce(int(wrap), _p(src), w, h, C, _p(dst), bits)
        if rc:
            raise ValueError("reduce precondition failed")
        return dst
    alpha = np.ascontiguousarray(alpha, np.uint8)
    da = np.empty((dh, dw), np.uint8)
    rc = lib().orc_reduce_alpha(int(wrap), _p(src), _p(alpha), w, h, C, _p(dst), _p(da), bits)
    if rc:
        raise ValueError("reduce precondition failed")
    return dst, da


def expand(src: np.ndarray, dst: np.ndarray, add: bool, bits: int, wrap: bool = False) -> np.ndarray:
    src = np.ascontiguousarray(src, np.int32)
    out = np.array(dst, np.int32, copy=True, order="C")
    sh, sw, C = src.shape
    dh, dw, _ = out.shape
    rc = lib().orc_expand(int(add), int(wrap), _p(src), sw, sh, _p(out), dw, dh, C, bits)
    if rc:
        raise ValueError("expand precondition failed")
    return out


def blend(mask: np.ndarray, white: np.ndarray, black: np.ndarray, white_value: int, bits: int) -> np.ndarray:
    mask = np.ascontiguousarray(mask, np.int32)
    white = np.ascontiguousarray(white, np.int32)
    out = np.array(black, np.int32, copy=True, order="C")
    C = out.shape[2]
    lib().orc_blend(_p(mask), _p(white), _p(out), mask.size, C, white_value, bits)
    return out


def mask_multiply(lp: np.ndarray, mask: np.ndarray, divisor: int, bits: int) -> np.ndarray:
    out = np.array(lp, np.int32, copy=True, order="C")
    mask = np.ascontiguousarray(mask, np.int32)
    lib().orc_mask_multiply(_p(out), _p(mask), mask.size, out.shape[2], divisor, bits)
    return out


def accumulate(lp: np.ndarray, res: np.ndarray, bits: int) -> np.ndarray:
    out = np.array(res, np.int32, copy=True, order="C")
    lp = np.ascontiguousarray(lp, np.int32)
    lib().orc_accumulate(_p(lp), _p(out), out.size, bits)
    return out


def from_fixed(src: np.ndarray, alpha: np.ndarray, dtype, frac: int = 7, dither: str = "hash",
               seed: int = 0x5eed, out: Optional[np.ndarray] = None) -> np.ndarray:
    src = np.ascontiguousarray(src, np.int32)
    h, w, C = src.shape
    if out is None:
        out = np.zeros((h, w, C), dtype)
    out = np.ascontiguousarray(out)
    lib().orc_from_fixed(_p(src), _p(np.ascontiguousarray(alpha, np.uint8)), w * h, C, _p(out), _dtype(out),
                         out.shape[2] if out.ndim == 3 else 1, frac, DITHER[dither], seed)
    return out


def dither_bits(seed: int, pixel: int, C: int = 3, c: int = 0, frac: int = 7) -> int:
    return int(lib().orc_dither_bits(seed, pixel, C, c, frac))


def enfuse_mask(img: np.ndarray, alpha: Optional[np.ndarray], prm: OrcParams) -> np.ndarray:
    img, w, h, C, s = _geom(img)
    if alpha is None:
        alpha = alpha_of(img)
    alpha = np.ascontiguousarray(alpha, np.uint8)
    out = np.zeros((h, w), np.float32)
    rc = lib().orc_enfuse_mask(_p(img), _dtype(img), w, h, C, s, _p(alpha), ctypes.byref(prm), _p(out))
    if rc:
        raise ValueError(f"orc_enfuse_mask failed ({rc})")
    return out


def local_stddev(gray: np.ndarray, alpha: np.ndarray, window: int) -> np.ndarray:
    gray = np.ascontiguousarray(gray, np.int32)
    h, w = gray.shape
    out = np.zeros((h, w), np.int32)
    rc = lib().orc_local_stddev(_p(gray), _p(np.ascontiguousarray(alpha, np.uint8)), w, h, window, _p(out))
    if rc:
        raise ValueError("local_stddev failed")
    return out


def enfuse(images: Sequence[np.ndarray], alphas: Optional[Sequence[np.ndarray]] = None,
           prm: Optional[OrcParams] = None, masks: Optional[Sequence[np.ndarray]] = None, levels: int = 0,
           wrap: bool = False, hard_mask: bool = False, dither: str = "hash", seed: int = 0x5eed,
           want_level0: bool = False, want_masks: bool = False):
    """enfuseMain restated.  Returns dict(out, alpha[, level0][, masks])."""
    imgs = [_geom(x)[0] for x in images]
    _, w, h, C, s = _geom(imgs[0])
    K = len(imgs)
    if alphas is None:
        alphas = [alpha_of(x) for x in imgs]
    alphas = [np.ascontiguousarray(a, np.uint8) for a in alphas]
    prm = prm if prm is not None else params()
    ip = (ctypes.c_void_p * K)(*[x.ctypes.data for x in imgs])
    ap = (ctypes.c_void_p * K)(*[a.ctypes.data for a in alphas])
    mp = None
    if masks is not None:
        masks = [np.ascontiguousarray(m, np.float32) for m in masks]
        mp = (ctypes.c_void_p * K)(*[m.ctypes.data for m in masks])
    out = np.zeros_like(imgs[0])
    oa = np.zeros((h, w), np.uint8)
    l0 = np.zeros((h, w, C), np.int32) if want_level0 else None
    mo = np.zeros((K, h, w), np.float32) if want_masks else None
    rc = lib().orc_enfuse(K, ip, ap, _dtype(imgs[0]), w, h, C, s, ctypes.byref(prm), levels, int(wrap),
                          int(hard_mask), mp, _p(out), _p(oa), DITHER[dither], seed, _p(l0), _p(mo))
    if rc:
        raise ValueError(f"orc_enfuse failed ({rc})")
    res = {"out": out, "alpha": oa}
    if want_level0:
        res["level0"] = l0
    if want_masks:
        res["masks"] = mo
    return res


def enblend(white: np.ndarray, black: np.ndarray, mask: np.ndarray, white_alpha=None, black_alpha=None,
            levels: int = 0, wrap: bool = False, dither: str = "hash", seed: int = 0x5eed,
            want_level0: bool = False):
    white, w, h, C, s = _geom(white)
    black = _geom(black)[0]
    wa = np.ascontiguousarray(white_alpha if white_alpha is not None else alpha_of(white), np.uint8)
    ba = np.ascontiguousarray(black_alpha if black_alpha is not None else alpha_of(black), np.uint8)
    mask = np.ascontiguousarray(mask, np.uint8)
    out = np.zeros_like(black)
    oa = np.zeros((h, w), np.uint8)
    l0 = np.zeros((h, w, C), np.int32) if want_level0 else None
    rc = lib().orc_enblend(_p(white), _p(wa), _p(black), _p(ba), _p(mask), _dtype(white), w, h, C, s, levels,
                           int(wrap), _p(out), _p(oa), DITHER[dither], seed, _p(l0))
    if rc:
        raise ValueError(f"orc_enblend failed ({rc})")
    res = {"out": out, "alpha": oa}
    if want_level0:
        res["level0"] = l0
    return res


# ---- float images: double pyramids ------------------------------------------

FLT_MAX = float(np.finfo(np.float32).max)


def real_to_pyramid(img: np.ndarray) -> np.ndarray:
    """(H, W, S) float32 image -> (H, W, C) double level 0 (log mapping)."""
    img, w, h, C, s = _geom(np.asarray(img, np.float32))
    out = np.empty((h, w, C), np.float64)
    lib().orc_real_to_pyramid(_p(img), w * h, C, s, _p(out))
    return out


def real_from_pyramid(src: np.ndarray, alpha: np.ndarray, out: Optional[np.ndarray] = None) -> np.ndarray:
    src = np.ascontiguousarray(src, np.float64)
    h, w, C = src.shape
    if out is None:
        out = np.zeros((h, w, C), np.float32)
    out = np.ascontiguousarray(out, np.float32)
    lib().orc_real_from_pyramid(_p(src), _p(np.ascontiguousarray(alpha, np.uint8)), w * h, C, _p(out),
                                out.shape[2] if out.ndim == 3 else 1)
    return out


def reduce_d(src: np.ndarray, alpha: np.ndarray, wrap: bool = False):
    src = np.ascontiguousarray(src, np.float64)
    h, w, C = src.shape
    dh, dw = (h + 1) >> 1, (w + 1) >> 1
    dst = np.empty((dh, dw, C), np.float64)
    da = np.empty((dh, dw), np.uint8)
    if lib().orc_reduce_alpha_d(int(wrap), _p(src), _p(np.ascontiguousarray(alpha, np.uint8)), w, h, C, _p(dst),
                                _p(da)):
        raise ValueError("reduce precondition failed")
    return dst, da


def expand_d(src: np.ndarray, dst: np.ndarray, add: bool, wrap: bool = False) -> np.ndarray:
    src = np.ascontiguousarray(src, np.float64)
    out = np.array(dst, np.float64, copy=True, order="C")
    sh, sw, C = src.shape
    dh, dw, _ = out.shape
    if lib().orc_expand_d(int(add), int(wrap), _p(src), sw, sh, _p(out), dw, dh, C):
        raise ValueError("expand precondition failed")
    return out


def blend_d(mask: np.ndarray, white: np.ndarray, black: np.ndarray, white_value: int) -> np.ndarray:
    mask = np.ascontiguousarray(mask, np.int32)
    white = np.ascontiguousarray(white, np.float64)
    out = np.array(black, np.float64, copy=True, order="C")
    lib().orc_blend_d(_p(mask), _p(white), _p(out), mask.size, out.shape[2], white_value)
    return out


def mask_multiply_d(lp: np.ndarray, mask: np.ndarray, divisor: int, res: Optional[np.ndarray] = None):
    """Returns (lp * mask / divisor, res + that) (res None: only the product)."""
    out = np.array(lp, np.float64, copy=True, order="C")
    r = None if res is None else np.array(res, np.float64, copy=True, order="C")
    mask = np.ascontiguousarray(mask, np.int32)
    lib().orc_mask_multiply_d(_p(out), _p(mask), mask.size, out.shape[2], divisor, _p(r))
    return out, r


def enfuse_mask_f(img: np.ndarray, alpha: Optional[np.ndarray], prm: OrcParams, range_: float = FLT_MAX):
    img, w, h, C, s = _geom(np.asarray(img, np.float32))
    if alpha is None:
        alpha = alpha_of(img)
    alpha = np.ascontiguousarray(alpha, np.uint8)
    out = np.zeros((h, w), np.float32)
    rc = lib().orc_enfuse_mask_f(_p(img), w, h, C, s, _p(alpha), ctypes.byref(prm), range_, _p(out))
    if rc:
        raise ValueError(f"orc_enfuse_mask_f failed ({rc})")
    return out


def enfuse_f(images: Sequence[np.ndarray], alphas: Optional[Sequence[np.ndarray]] = None,
             prm: Optional[OrcParams] = None, range_: float = FLT_MAX, masks=None, levels: int = 0,
             wrap: bool = False, hard_mask: bool = False, want_level0: bool = False, want_masks: bool = False):
    """enfuseMain for float32 images (double pyramids).  Returns dict(out, alpha[, level0][, masks])."""
    imgs = [_geom(np.asarray(x, np.float32))[0] for x in images]
    _, w, h, C, s = _geom(imgs[0])
    K = len(imgs)
    if alphas is None:
        alphas = [alpha_of(x) for x in imgs]
    alphas = [np.ascontiguousarray(a, np.uint8) for a in alphas]
    prm = prm if prm is not None else params()
    ip = (ctypes.c_void_p * K)(*[x.ctypes.data for x in imgs])
    ap = (ctypes.c_void_p * K)(*[a.ctypes.data for a in alphas])
    mp = None
    if masks is not None:
        masks = [np.ascontiguousarray(m, np.float32) for m in masks]
        mp = (ctypes.c_void_p * K)(*[m.ctypes.data for m in masks])
    out = np.zeros_like(imgs[0])
    oa = np.zeros((h, w), np.uint8)
    l0 = np.zeros((h, w, C), np.float64) if want_level0 else None
    mo = np.zeros((K, h, w), np.float32) if want_masks else None
    rc = lib().orc_enfuse_f(K, ip, ap, w, h, C, s, ctypes.byref(prm), range_, levels, int(wrap), int(hard_mask), mp,
                            _p(out), _p(oa), _p(l0), _p(mo))
    if rc:
        raise ValueError(f"orc_enfuse_f failed ({rc})")
    res = {"out": out, "alpha": oa}
    if want_level0:
        res["level0"] = l0
    if want_masks:
        res["masks"] = mo
    return res


def enblend_f(white: np.ndarray, black: np.ndarray, mask: np.ndarray, white_alpha=None, black_alpha=None,
              levels: int = 0, wrap: bool = False, want_level0: bool = False):
    white, w, h, C, s = _geom(np.asarray(white, np.float32))
    black = _geom(np.asarray(black, np.float32))[0]
    wa = np.ascontiguousarray(white_alpha if white_alpha is not None else alpha_of(white), np.uint8)
    ba = np.ascontiguousarray(black_alpha if black_alpha is not None else alpha_of(black), np.uint8)
    mask = np.ascontiguousarray(mask, np.uint8)
    out = np.zeros_like(black)
    oa = np.zeros((h, w), np.uint8)
    l0 = np.zeros((h, w, C), np.float64) if want_level0 else None
    rc = lib().orc_enblend_f(_p(white), _p(wa), _p(black), _p(ba), _p(mask), w, h, C, s, levels, int(wrap), _p(out),
                             _p(oa), _p(l0))
    if rc:
        raise ValueError(f"orc_enblend_f failed ({rc})")
    res = {"out": out, "alpha": oa}
    if want_level0:
        res["level0"] = l0
    return res


# ---- the reference's option form (oracle.reference_build.enfuse_params keywords) ----------

def params_from_options(opts: dict, **extra) -> OrcParams:
    """OrcParams of enfuse options given in the keyword form of
    oracle.reference_build.enfuse_params: gray_projector "" is the default
    ("average"), "channel-mixer:R:G:B" the mixer with those weights; hard_mask is
    not a weighting option and is ignored here."""
    kw = {k: v for k, v in opts.items() if k != "hard_mask"}
    gp = kw.pop("gray_projector", "") or "average"
    if gp.startswith("channel-mixer"):
        kw["mixer"] = tuple(float(v) for v in gp.split(":")[1:4])
        gp = "channel-mixer"
    kw["gray_projector"] = gp
    kw.update(extra)
    return params(**kw)


def convert_with_draw(level0: np.ndarray, alpha: np.ndarray, dtype, draw: int, frac: int = 7) -> np.ndarray:
    """copyFromPyramidImageIf's dither rule (src/fixmath.h:251-277) when every
    random draw returns `draw`: q + 1 iff the fraction f >= 3/4, or f lies in
    [1/4, 3/4) and (draw & (2^(frac-1) - 1)) + 2^(frac-2) <= f; clamped to the
    type; 0 where alpha is 0."""
    l0 = np.asarray(level0, np.int64)
    Q = 1 << (frac - 2)
    q, f = l0 >> frac, l0 & ((1 << frac) - 1)
    t = (draw & (2 * Q - 1)) + Q
    v = np.where(f < Q, q, np.where(f >= 3 * Q, q + 1, np.where(t <= f, q + 1, q)))
    v = np.clip(v, 0, np.iinfo(dtype).max).astype(dtype)
    on = np.asarray(alpha) != 0
    return np.where(on[..., None] if v.ndim == 3 else on, v, np.zeros_like(v))


def nft_mask(white_alpha: np.ndarray, black_alpha: np.ndarray, wrap: bool = False) -> np.ndarray:
    """enblend's nearest-feature seam mask (fine, not optimised) of two alpha
    planes: 255 where the white image wins.  Raises ValueError on the
    reference's "excessive image overlap"."""
    wa = np.ascontiguousarray(white_alpha, np.uint8)
    ba = np.ascontiguousarray(black_alpha, np.uint8)
    h, w = wa.shape
    m = np.zeros((h, w), np.uint8)
    L = lib()
    L.orc_nft_mask.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                               ctypes.c_void_p]
    rc = L.orc_nft_mask(_p(wa), _p(ba), w, h, int(wrap), _p(m))
    if rc == 2:
        raise ValueError("excessive image overlap")
    if rc:
        raise ValueError(f"orc_nft_mask failed ({rc})")
    return m
