"""enbgpu -- Python binding of the GB300 enblend/enfuse multiresolution path.

A thin ctypes layer over the C ABI of ``libenbgpu.so`` (``include/enbgpu.h``).
The names mirror the reference's internal API (``gaussianPyramid``,
``laplacianPyramid``, ``collapsePyramid``, ``blend``, ``enfuseMask``,
``enfuseMain``/``enblendMain``) and its command-line weighting options.  Every
computation runs in the CUDA library; there is no CPU fallback, and importing
this package fails if the library has not been built.

Arrays: numpy arrays are host buffers (the library copies them on its
stream); ``torch`` CUDA tensors are used in place.  Pixel images are
``(H, W, S)`` arrays of uint8/uint16 with S = 3 (RGB) or 4 (RGBA, alpha in
the 4th component), or ``(H, W)`` for gray; alpha and seam masks are
``(H, W)`` uint8; weight masks ``(H, W)`` float32.
"""
from __future__ import annotations

import ctypes
import os
import re
from dataclasses import dataclass, field
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

from . import _build

LIB_PATH = _build.LIB_PATH
HEADER = _build.INCLUDE / "enbgpu.h"

ENB_OK, ENB_ERR_INVALID, ENB_ERR_UNSUPPORTED, ENB_ERR_CUDA, ENB_ERR_NOMEM = range(5)
ENB_U8, ENB_U16, ENB_F32, ENB_I16, ENB_I32 = range(5)
DITHER = {"hash": 0, "nearest": 1}
EXPOSURE_FUNCTIONS = {"gaussian": 0, "lorentzian": 1, "halfsine": 2, "fullsine": 3, "bisquare": 4}
GRAY_PROJECTORS = {"average": 0, "value": 1, "anti-value": 2, "lightness": 3, "luminance": 4,
                   "channel-mixer": 5}


class EnbError(RuntimeError):
    """A failed C-ABI call; ``status`` is the enb_status code."""

    def __init__(self, status: int, message: str):
        super().__init__(f"enbgpu status {status}: {message}")
        self.status = status


class EnbImage(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("pitch", ctypes.c_int64), ("plane_pitch", ctypes.c_int64),
                ("width", ctypes.c_int32), ("height", ctypes.c_int32), ("channels", ctypes.c_int32),
                ("pix_stride", ctypes.c_int32), ("dtype", ctypes.c_int32), ("planar", ctypes.c_int32)]


class EnbEnfuseParams(ctypes.Structure):
    _fields_ = [("w_exposure", ctypes.c_double), ("w_saturation", ctypes.c_double),
                ("w_contrast", ctypes.c_double), ("w_entropy", ctypes.c_double),
                ("exp_optimum", ctypes.c_double), ("exp_width", ctypes.c_double),
                ("exp_function", ctypes.c_int32), ("contrast_window", ctypes.c_int32),
                ("entropy_window", ctypes.c_int32), ("gray_projector", ctypes.c_int32),
                ("mixer", ctypes.c_double * 3), ("float_range", ctypes.c_double),
                ("exp_cutoff_lower", ctypes.c_double), ("exp_cutoff_upper", ctypes.c_double),
                ("exp_cutoff_lower_pct", ctypes.c_int32), ("exp_cutoff_upper_pct", ctypes.c_int32),
                ("exp_cutoff_lower_projector", ctypes.c_int32), ("exp_cutoff_upper_projector", ctypes.c_int32),
                ("ent_cutoff_lower", ctypes.c_double), ("ent_cutoff_upper", ctypes.c_double),
                ("ent_cutoff_lower_pct", ctypes.c_int32), ("ent_cutoff_upper_pct", ctypes.c_int32),
                ("exposure_table", ctypes.c_void_p), ("exposure_table_size", ctypes.c_int32)]


class EnbFuseOptions(ctypes.Structure):
    _fields_ = [("levels", ctypes.c_int32), ("wrap", ctypes.c_int32), ("hard_mask", ctypes.c_int32),
                ("dither", ctypes.c_int32), ("seed", ctypes.c_uint64), ("host_buffers", ctypes.c_int32),
                ("plain", ctypes.c_int32), ("level0_out", ctypes.c_void_p), ("coarse_pixels", ctypes.c_int32),
                ("graph", ctypes.c_int32)]


class EnbFuseGradResult(ctypes.Structure):
    _fields_ = [("loss", ctypes.c_double), ("d_exp_optimum", ctypes.c_double), ("d_exp_width", ctypes.c_double),
                ("d_w_exposure", ctypes.c_double), ("d_w_saturation", ctypes.c_double),
                ("d_w_contrast", ctypes.c_double)]


class EnbStack(ctypes.Structure):
    _fields_ = [("K", ctypes.c_int32), ("images", ctypes.POINTER(EnbImage)), ("alphas", ctypes.POINTER(EnbImage)),
                ("out", ctypes.POINTER(EnbImage)), ("out_alpha", ctypes.POINTER(EnbImage))]


_P = ctypes.POINTER
_IMG = _P(EnbImage)
_SIGNATURES = {
    "enb_abi_version": (ctypes.c_int, []),
    "enb_create": (ctypes.c_int, [ctypes.c_int, _P(ctypes.c_void_p)]),
    "enb_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "enb_set_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "enb_synchronize": (ctypes.c_int, [ctypes.c_void_p]),
    "enb_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "enb_debug_overarm_tile_waits": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32]),
    "enb_launch_count": (ctypes.c_uint64, [ctypes.c_void_p]),
    "enb_profile_enable": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "enb_profile_count": (ctypes.c_int, [ctypes.c_void_p]),
    "enb_profile_entry": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _P(ctypes.c_char_p), _P(ctypes.c_uint64),
                                         _P(ctypes.c_double), _P(ctypes.c_double)]),
    "enb_default_enfuse_params": (None, [_P(EnbEnfuseParams)]),
    "enb_default_fuse_options": (None, [_P(EnbFuseOptions)]),
    "enb_num_levels": (ctypes.c_int, [ctypes.c_int] * 4),
    "enb_pyramid_create": (ctypes.c_int, [ctypes.c_void_p] + [ctypes.c_int] * 5 + [_P(ctypes.c_void_p)]),
    "enb_pyramid_free": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "enb_pyramid_levels": (ctypes.c_int, [ctypes.c_void_p]),
    "enb_pyramid_level": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _IMG]),
    "enb_pyramid_read_level": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "enb_pyramid_write_level": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "enb_to_pyramid": (ctypes.c_int, [ctypes.c_void_p, _IMG, _IMG, ctypes.c_int]),
    "enb_reduce": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _IMG, _IMG, _IMG, _IMG]),
    "enb_expand": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _IMG, _IMG]),
    "enb_blend": (ctypes.c_int, [ctypes.c_void_p, _IMG, _IMG, _IMG, ctypes.c_int32]),
    "enb_mask_multiply_accumulate": (ctypes.c_int, [ctypes.c_void_p, _IMG, _IMG, ctypes.c_int32, _IMG, ctypes.c_int]),
    "enb_from_pyramid": (ctypes.c_int, [ctypes.c_void_p, _IMG, _IMG, _IMG, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_uint64]),
    "enb_gaussian_pyramid": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _IMG, _IMG, ctypes.c_int,
                                            ctypes.c_void_p]),
    "enb_gaussian_pyramid_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _IMG, _IMG, ctypes.c_int,
                                                    ctypes.c_void_p]),
    "enb_laplacian_pyramid": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _IMG, _IMG, ctypes.c_int,
                                             ctypes.c_void_p]),
    "enb_collapse_pyramid": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "enb_blend_pyramids": (ctypes.c_int, [ctypes.c_void_p] * 4 + [ctypes.c_int32]),
    "enb_enfuse_mask": (ctypes.c_int, [ctypes.c_void_p, _P(EnbEnfuseParams), _IMG, _IMG, _IMG]),
    "enb_enfuse": (ctypes.c_int, [ctypes.c_void_p, _P(EnbEnfuseParams), ctypes.c_int, _IMG, _IMG, _IMG, _IMG,
                                  _IMG, _P(EnbFuseOptions)]),
    "enb_fuse_grad": (ctypes.c_int, [ctypes.c_void_p, _P(EnbEnfuseParams), ctypes.c_int, _IMG, _IMG, _IMG, _IMG,
                                      _IMG, _P(EnbFuseGradResult), _P(EnbFuseOptions)]),
    "enb_fuse_stacks": (ctypes.c_int, [ctypes.c_void_p, _P(EnbEnfuseParams), ctypes.c_int, _P(EnbStack),
                                        _P(EnbFuseOptions)]),
    "enb_fuse_stacks_tune": (ctypes.c_int, [ctypes.c_void_p, _P(EnbEnfuseParams), ctypes.c_int, _P(EnbStack),
                                            _P(EnbFuseOptions), _P(ctypes.c_int32), ctypes.c_int, ctypes.c_int,
                                            _P(ctypes.c_float), _P(ctypes.c_int32)]),
    "enb_enblend": (ctypes.c_int, [ctypes.c_void_p, _IMG, _IMG, _IMG, _IMG, _IMG, _IMG, _IMG,
                                   _P(EnbFuseOptions)]),
    "enb_nft_mask": (ctypes.c_int, [ctypes.c_void_p, _IMG, _IMG, _IMG, _P(EnbFuseOptions)]),
}


def header_functions() -> list[str]:
    """Names of the functions declared in include/enbgpu.h."""
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(enb_[a-z0-9_]+)\s*\(", text)))


_lib: Optional[ctypes.CDLL] = None


def load_library() -> ctypes.CDLL:
    """Load libenbgpu.so (built by ``_build.build()``); raise if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: build the CUDA library first (enbgpu._build.build())")
    lib = ctypes.CDLL(str(LIB_PATH))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


# --------------------------------------------------------------------------
# descriptors
# --------------------------------------------------------------------------

_NP_DTYPE = {np.dtype(np.uint8): ENB_U8, np.dtype(np.uint16): ENB_U16, np.dtype(np.float32): ENB_F32,
             np.dtype(np.int16): ENB_I16, np.dtype(np.int32): ENB_I32}


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def _dtype_code(x) -> int:
    if _is_torch(x):
        import torch
        m = {torch.uint8: ENB_U8, torch.uint16: ENB_U16, torch.float32: ENB_F32, torch.int16: ENB_I16,
             torch.int32: ENB_I32}
        return m[x.dtype]
    return _NP_DTYPE[np.dtype(x.dtype)]


def _ptr_and_strides(x):
    if _is_torch(x):
        return x.data_ptr(), [s * x.element_size() for s in x.stride()], x.is_cuda
    return x.ctypes.data, list(x.strides), False


def pixel_image(x, channels: Optional[int] = None) -> EnbImage:
    """Descriptor of an interleaved (H, W, S) or (H, W) pixel array."""
    ptr, strides, _ = _ptr_and_strides(x)
    if x.ndim == 2:
        h, w = x.shape
        s = 1
    else:
        h, w, s = x.shape
    es = x.element_size() if _is_torch(x) else x.itemsize
    if strides[-1] != es or (x.ndim == 3 and strides[1] != s * es):
        raise ValueError("pixel arrays must be contiguous within a row")
    c = channels if channels is not None else (3 if s >= 3 else 1)
    return EnbImage(ptr, strides[0], 0, w, h, c, s, _dtype_code(x), 0)


def plane_image(x) -> EnbImage:
    """Descriptor of an (H, W) plane (alpha, seam mask or weight mask)."""
    ptr, strides, _ = _ptr_and_strides(x)
    h, w = x.shape
    es = x.element_size() if _is_torch(x) else x.itemsize
    if strides[1] != es:
        raise ValueError("planes must be contiguous within a row")
    return EnbImage(ptr, strides[0], 0, w, h, 1, 1, _dtype_code(x), 0)


def _pyramid_dtype(img: EnbImage, weight_plane: bool = False) -> int:
    """EnblendNumericTraits' image pyramid type (src/numerictraits.h:168-185): Int16 for 8-bit samples, Int32
    for 16-bit samples and float weight planes, FP32 (the reference's double) for float images."""
    if img.dtype == ENB_U8:
        return ENB_I16
    if img.dtype == ENB_F32 and not weight_plane:
        return ENB_F32
    return ENB_I32


def enfuse_params(exposure_weight: float = 1.0, saturation_weight: float = 0.0, contrast_weight: float = 0.0,
                  entropy_weight: float = 0.0, exposure_optimum: float = 0.5, exposure_width: float = 0.2,
                  exposure_weight_function: str = "gaussian", contrast_window_size: int = 5,
                  entropy_window_size: int = 3, gray_projector: str = "average",
                  mixer: Sequence[float] = (0.0, 0.0, 0.0), float_range: float = 0.0,
                  exposure_cutoff=((0.0, True), (100.0, True)), exposure_cutoff_projectors=("anti-value", "value"),
                  entropy_cutoff=((0.0, True), (100.0, True)), exposure_table=None) -> EnbEnfuseParams:
    """enfuse's weighting options (src/enfuse.cc:117-160, same defaults).

    float_range: float images only; 0 takes the reference's NumericTraits<float>::max() as the sample scale of
    the exposure and entropy weights, 1.0 is the normalised-float mode for images in [0, 1].
    exposure_cutoff / entropy_cutoff: (lower, upper) limits, each (value, is_percentage), as
    --exposure-cutoff and --entropy-cutoff give them; exposure_cutoff_projectors judge the two limits.
    exposure_table: a user-defined exposure weight function tabulated at y = g / max for every sample value g
    (256 entries for 8-bit, 65536 for 16-bit images; see exposure_table_of); the parameters keep it alive."""
    p = EnbEnfuseParams()
    p.w_exposure, p.w_saturation = exposure_weight, saturation_weight
    p.w_contrast, p.w_entropy = contrast_weight, entropy_weight
    p.exp_optimum, p.exp_width = exposure_optimum, exposure_width
    p.exp_function = EXPOSURE_FUNCTIONS[exposure_weight_function]
    p.contrast_window, p.entropy_window = contrast_window_size, entropy_window_size
    p.gray_projector = GRAY_PROJECTORS[gray_projector]
    p.mixer[:] = list(mixer)
    p.float_range = float_range
    (p.exp_cutoff_lower, p.exp_cutoff_lower_pct), (p.exp_cutoff_upper, p.exp_cutoff_upper_pct) = \
        [(float(v), int(bool(pct))) for v, pct in exposure_cutoff]
    p.exp_cutoff_lower_projector = GRAY_PROJECTORS[exposure_cutoff_projectors[0]]
    p.exp_cutoff_upper_projector = GRAY_PROJECTORS[exposure_cutoff_projectors[1]]
    (p.ent_cutoff_lower, p.ent_cutoff_lower_pct), (p.ent_cutoff_upper, p.ent_cutoff_upper_pct) = \
        [(float(v), int(bool(pct))) for v, pct in entropy_cutoff]
    if exposure_table is not None:
        t = np.ascontiguousarray(exposure_table, dtype=np.float64)
        p._exposure_table = t  # kept alive with the parameters
        p.exposure_table, p.exposure_table_size = t.ctypes.data, t.size
    return p


def exposure_table_of(weight, bits: int) -> np.ndarray:
    """weight(y) of a Python callable at y = g / max for g = 0..max (max = 2^bits - 1): the table a
    user-defined exposure weight function becomes (the same y the reference's ExposureFunctor forms,
    src/enfuse.h:638)."""
    maxv = (1 << bits) - 1
    return np.array([weight(g / maxv) for g in range(maxv + 1)], dtype=np.float64)


# --------------------------------------------------------------------------
# context
# --------------------------------------------------------------------------

class Pyramid:
    """A device-resident pyramid (std::vector<PyramidImageType*> of the reference)."""

    def __init__(self, ctx: "Context", handle: ctypes.c_void_p, dtype: int, channels: int):
        self.ctx, self.handle, self.dtype, self.channels = ctx, handle, dtype, channels

    @property
    def levels(self) -> int:
        return self.ctx.lib.enb_pyramid_levels(self.handle)

    def level_image(self, l: int) -> EnbImage:
        img = EnbImage()
        self.ctx._check(self.ctx.lib.enb_pyramid_level(self.handle, l, ctypes.byref(img)))
        return img

    def _np_type(self):
        return {ENB_I16: np.int16, ENB_I32: np.int32, ENB_F32: np.float32}[self.dtype]

    def read(self, l: int) -> np.ndarray:
        """Level l as a (C, H, W) int16/int32/float32 array."""
        img = self.level_image(l)
        a = np.empty((img.channels, img.height, img.width), self._np_type())
        self.ctx._check(self.ctx.lib.enb_pyramid_read_level(self.ctx.handle, self.handle, l, a.ctypes.data))
        return a

    def write(self, l: int, a: np.ndarray) -> None:
        img = self.level_image(l)
        a = np.ascontiguousarray(a, dtype=self._np_type()).reshape(img.channels, img.height, img.width)
        self.ctx._check(self.ctx.lib.enb_pyramid_write_level(self.ctx.handle, self.handle, l, a.ctypes.data))

    def free(self) -> None:
        if self.handle:
            self.ctx.lib.enb_pyramid_free(self.ctx.handle, self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Context:
    """One CUDA device and stream (enb_ctx)."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = ctypes.c_void_p()
        st = self.lib.enb_create(device, ctypes.byref(h))
        if st != ENB_OK:
            raise EnbError(st, "enb_create failed (no usable CUDA device)")
        self.handle = h

    def close(self) -> None:
        if self.handle:
            self.lib.enb_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int) -> None:
        if st != ENB_OK:
            raise EnbError(st, self.lib.enb_last_error(self.handle).decode())

    def set_stream(self, stream_ptr: int) -> None:
        self._check(self.lib.enb_set_stream(self.handle, ctypes.c_void_p(stream_ptr)))

    def synchronize(self) -> None:
        self._check(self.lib.enb_synchronize(self.handle))

    @property
    def launches(self) -> int:
        return int(self.lib.enb_launch_count(self.handle))

    def profile(self, enable: bool) -> None:
        """Start (or stop) per-kernel CUDA-event timing; clears earlier records."""
        self._check(self.lib.enb_profile_enable(self.handle, int(enable)))

    def profile_report(self) -> dict:
        """{kernel: {"launches", "ms", "bytes"}} of the launches since profiling started."""
        out = {}
        for i in range(self.lib.enb_profile_count(self.handle)):
            name, n, ms, b = ctypes.c_char_p(), ctypes.c_uint64(), ctypes.c_double(), ctypes.c_double()
            self._check(self.lib.enb_profile_entry(self.handle, i, ctypes.byref(name), ctypes.byref(n),
                                                   ctypes.byref(ms), ctypes.byref(b)))
            out[name.value.decode()] = {"launches": int(n.value), "ms": ms.value, "bytes": b.value}
        return out

    # ---- pyramids ---------------------------------------------------------
    def pyramid(self, levels: int, width: int, height: int, channels: int, dtype: int) -> Pyramid:
        h = ctypes.c_void_p()
        self._check(self.lib.enb_pyramid_create(self.handle, levels, width, height, channels, dtype, ctypes.byref(h)))
        return Pyramid(self, h, dtype, channels)

    def reduce(self, src: Pyramid, l: int, dst: Pyramid, dl: int, wrap: bool = False,
               src_alpha=None, dst_alpha=None) -> None:
        """reduce (src/pyramid.h:166-848) from level l of src into level dl of dst."""
        si, di = src.level_image(l), dst.level_image(dl)
        sa = ctypes.byref(plane_image(src_alpha)) if src_alpha is not None else None
        da = ctypes.byref(plane_image(dst_alpha)) if dst_alpha is not None else None
        self._check(self.lib.enb_reduce(self.handle, int(wrap), ctypes.byref(si), sa, ctypes.byref(di), da))

    def expand(self, src: Pyramid, l: int, dst: Pyramid, dl: int, add: bool, wrap: bool = False) -> None:
        """expand (src/pyramid.h:1102-1457) of level l of src into level dl of dst."""
        si, di = src.level_image(l), dst.level_image(dl)
        self._check(self.lib.enb_expand(self.handle, int(add), int(wrap), ctypes.byref(si), ctypes.byref(di)))

    def gaussian_pyramid(self, image, levels: int, alpha=None, wrap: bool = False, frac_bits: int = 7,
                         dtype: Optional[int] = None) -> Pyramid:
        """gaussianPyramid (src/pyramid.h:1468-1636) of a device image."""
        weight_plane = image.ndim == 2 and _dtype_code(image) == ENB_F32
        img = plane_image(image) if weight_plane else pixel_image(image)
        if dtype is None:
            dtype = _pyramid_dtype(img, weight_plane)
        pyr = self.pyramid(levels, img.width, img.height, img.channels, dtype)
        a = ctypes.byref(plane_image(alpha)) if alpha is not None else None
        self._check(self.lib.enb_gaussian_pyramid(self.handle, int(wrap), ctypes.byref(img), a, frac_bits,
                                                  pyr.handle))
        return pyr

    def laplacian_pyramid(self, image, levels: int, alpha=None, wrap: bool = False, frac_bits: int = 7,
                          dtype: Optional[int] = None) -> Pyramid:
        """laplacianPyramid (src/pyramid.h:1647-1747) of a device image."""
        img = pixel_image(image)
        if dtype is None:
            dtype = _pyramid_dtype(img)
        pyr = self.pyramid(levels, img.width, img.height, img.channels, dtype)
        a = ctypes.byref(plane_image(alpha)) if alpha is not None else None
        self._check(self.lib.enb_laplacian_pyramid(self.handle, int(wrap), ctypes.byref(img), a, frac_bits,
                                                   pyr.handle))
        return pyr

    def collapse_pyramid(self, pyr: Pyramid, wrap: bool = False) -> None:
        self._check(self.lib.enb_collapse_pyramid(self.handle, int(wrap), pyr.handle))

    def blend_pyramids(self, mask_gp: Pyramid, white_lp: Pyramid, black_lp: Pyramid, white_value: int) -> None:
        self._check(self.lib.enb_blend_pyramids(self.handle, mask_gp.handle, white_lp.handle, black_lp.handle,
                                                white_value))

    def blend_level(self, mask: Pyramid, white: Pyramid, black: Pyramid, l: int, white_value: int) -> None:
        m, w, b = mask.level_image(l), white.level_image(l), black.level_image(l)
        self._check(self.lib.enb_blend(self.handle, ctypes.byref(m), ctypes.byref(w), ctypes.byref(b), white_value))

    def mask_multiply_accumulate(self, lp: Pyramid, mask: Pyramid, result: Pyramid, l: int, divisor: int,
                                 accumulate: bool) -> None:
        a, m, r = lp.level_image(l), mask.level_image(l), result.level_image(l)
        self._check(self.lib.enb_mask_multiply_accumulate(self.handle, ctypes.byref(a), ctypes.byref(m), divisor,
                                                          ctypes.byref(r), int(accumulate)))

    def from_pyramid(self, pyr: Pyramid, l: int, alpha, dst, frac_bits: int = 7, dither: str = "hash",
                     seed: int = 0x5eed) -> None:
        s = pyr.level_image(l)
        self._check(self.lib.enb_from_pyramid(self.handle, ctypes.byref(s), ctypes.byref(plane_image(alpha)),
                                              ctypes.byref(pixel_image(dst, channels=s.channels)), frac_bits,
                                              DITHER[dither], seed))

    # ---- weights and drivers ---------------------------------------------
    def enfuse_mask(self, image, alpha, out, params: Optional[EnbEnfuseParams] = None) -> None:
        """enfuseMask (src/enfuse.h:962-1212) into a device float plane."""
        p = params if params is not None else enfuse_params()
        a = ctypes.byref(plane_image(alpha)) if alpha is not None else None
        self._check(self.lib.enb_enfuse_mask(self.handle, ctypes.byref(p), ctypes.byref(pixel_image(image)), a,
                                             ctypes.byref(plane_image(out))))

    def _options(self, levels, wrap, hard_mask, dither, seed, host, level0, plain=False,
                 coarse_pixels: int = 0) -> EnbFuseOptions:
        o = EnbFuseOptions()
        self.lib.enb_default_fuse_options(ctypes.byref(o))
        o.levels, o.wrap, o.hard_mask = levels, int(wrap), int(hard_mask)
        o.dither, o.seed, o.host_buffers = DITHER[dither], seed, int(host)
        o.plain = int(plain)
        o.level0_out = level0
        o.coarse_pixels = coarse_pixels
        return o

    def enfuse(self, images, alphas=None, params: Optional[EnbEnfuseParams] = None, masks=None, out=None,
               out_alpha=None, levels: int = 0, wrap: bool = False, hard_mask: bool = False,
               dither: str = "hash", seed: int = 0x5eed, level0=None, plain: bool = False):
        """enfuseMain (src/enfuse.h:1217-1617).  Host (numpy) or device (torch) arrays.

        Returns (out, out_alpha)."""
        K = len(images)
        host = not _is_torch(images[0])
        if out is None:
            out = np.zeros_like(images[0]) if host else images[0].new_zeros(images[0].shape)
        if out_alpha is None:
            shp = images[0].shape[:2]
            out_alpha = np.zeros(shp, np.uint8) if host else images[0].new_zeros(shp, dtype=__import__("torch").uint8)
        imgs = (EnbImage * K)(*[pixel_image(x) for x in images])
        al = (EnbImage * K)(*[plane_image(a) for a in alphas]) if alphas is not None else None
        ms = (EnbImage * K)(*[plane_image(m) for m in masks]) if masks is not None else None
        p = params if params is not None else enfuse_params()
        l0 = None
        if level0 is not None:
            l0 = _ptr_and_strides(level0)[0]
        o = self._options(levels, wrap, hard_mask, dither, seed, host, l0, plain)
        self._check(self.lib.enb_enfuse(self.handle, ctypes.byref(p), K, imgs, al, ms,
                                        ctypes.byref(pixel_image(out)), ctypes.byref(plane_image(out_alpha)),
                                        ctypes.byref(o)))
        return out, out_alpha

    def _stack_descs(self, stacks, outs, out_alphas, alphas, keep):
        descs = (EnbStack * len(stacks))()
        for i, st in enumerate(stacks):
            imgs = (EnbImage * len(st))(*[pixel_image(x) for x in st])
            al = (EnbImage * len(st))(*[plane_image(a) for a in alphas[i]]) if alphas is not None else None
            out = pixel_image(outs[i])
            oa = plane_image(out_alphas[i]) if out_alphas is not None else None
            keep += [imgs, al, out, oa]
            descs[i].K = len(st)
            descs[i].images = ctypes.cast(imgs, ctypes.POINTER(EnbImage))
            descs[i].alphas = ctypes.cast(al, ctypes.POINTER(EnbImage)) if al is not None else None
            descs[i].out = ctypes.pointer(out)
            descs[i].out_alpha = ctypes.pointer(oa) if oa is not None else None
        return descs

    def tune_stacks(self, stacks, params: Optional[EnbEnfuseParams] = None, outs=None, alphas=None,
                    candidates=None, reps: int = 2, levels: int = 0, wrap: bool = False,
                    hard_mask: bool = False) -> dict:
        """Autotune the level schedule of the batched fuse on these device stacks (enb_fuse_stacks_tune):
        {"best": threshold, "ms": {threshold: ms per call}}.  Later fuse_stacks calls on batches of this
        geometry with coarse_pixels=0 use the chosen threshold."""
        if not all(_is_torch(x) for st in stacks for x in st):
            raise TypeError("tune_stacks: the stacks must be device tensors (the batched device path is tuned)")
        if outs is None:
            outs = [st[0].new_zeros(st[0].shape) for st in stacks]
        keep = []
        descs = self._stack_descs(stacks, outs, None, alphas, keep)
        p = params if params is not None else enfuse_params()
        o = self._options(levels, wrap, hard_mask, "hash", 0, False, None)
        cands = list(candidates) if candidates is not None else [-1, 1024, 4096, 16384, 65536]
        carr = (ctypes.c_int32 * len(cands))(*cands)
        times = (ctypes.c_float * len(cands))()
        best = ctypes.c_int32()
        self._check(self.lib.enb_fuse_stacks_tune(self.handle, ctypes.byref(p), len(stacks), descs, ctypes.byref(o),
                                                  carr, len(cands), reps, times, ctypes.byref(best)))
        del keep
        return {"best": int(best.value), "ms": {c: float(t) for c, t in zip(cands, times)}}

    def fuse_stacks(self, stacks, params: Optional[EnbEnfuseParams] = None, outs=None, out_alphas=None,
                    alphas=None, levels: int = 0, wrap: bool = False, hard_mask: bool = False, plain: bool = False,
                    graph: bool = True, coarse_pixels: int = 0):
        """Batched enfuse of independent float stacks (enb_fuse_stacks).  stacks: list of lists of (H, W, S)
        float32 arrays (numpy: host buffers; torch: device).  Returns the list of outputs (and fills out_alphas
        when given).  coarse_pixels=0: the threshold tune_stacks chose for this batch geometry, else 64x64."""
        host = not _is_torch(stacks[0][0])
        if outs is None:
            outs = [np.zeros_like(st[0]) if host else st[0].new_zeros(st[0].shape) for st in stacks]
        keep = []
        descs = self._stack_descs(stacks, outs, out_alphas, alphas, keep)
        p = params if params is not None else enfuse_params()
        o = self._options(levels, wrap, hard_mask, "hash", 0, host, None, plain, coarse_pixels)
        o.graph = int(graph)
        self._check(self.lib.enb_fuse_stacks(self.handle, ctypes.byref(p), len(stacks), descs, ctypes.byref(o)))
        del keep
        return outs

    def fuse_grad(self, images, target, params: Optional[EnbEnfuseParams] = None, logits=None, out=None,
                  grad_logits=None, levels: int = 0) -> dict:
        """Loss of the float enfuse against `target` and its gradients (enb_fuse_grad).  images: K (H, W, 3)
        float32 device tensors; logits / grad_logits: K (H, W) float32 device tensors or None."""
        arrays = list(images) + [target] + [x for x in (out,) if x is not None] + list(logits or []) + list(grad_logits or [])
        if not all(_is_torch(x) for x in arrays):
            raise TypeError("fuse_grad: images, target, out, logits and grad_logits must be device tensors")
        K = len(images)
        imgs = (EnbImage * K)(*[pixel_image(x) for x in images])
        lg = (EnbImage * K)(*[plane_image(a) for a in logits]) if logits is not None else None
        gl = (EnbImage * K)(*[plane_image(a) for a in grad_logits]) if grad_logits is not None else None
        p = params if params is not None else enfuse_params(float_range=1.0)
        o = self._options(levels, False, False, "hash", 0, False, None)
        r = EnbFuseGradResult()
        self._check(self.lib.enb_fuse_grad(self.handle, ctypes.byref(p), K, imgs, lg, ctypes.byref(pixel_image(target)),
                                           ctypes.byref(pixel_image(out)) if out is not None else None, gl,
                                           ctypes.byref(r), ctypes.byref(o)))
        return {f: getattr(r, f) for f, _ in EnbFuseGradResult._fields_}

    def enblend(self, white, black, mask, white_alpha=None, black_alpha=None, out=None, out_alpha=None,
                levels: int = 0, wrap: bool = False, dither: str = "hash", seed: int = 0x5eed, level0=None,
                plain: bool = False, coarse_pixels: int = 0):
        """enblendMain's pyramid blend (src/enblend.h:330-510).  Returns (out, out_alpha).

        plain=True runs the reference's pass structure (one kernel per reference operation) instead of the
        fused level passes; coarse_pixels sets which levels run in the single coarse launch (0 default,
        negative never).  The result is the same either way."""
        host = not _is_torch(black)
        if out is None:
            out = np.zeros_like(black) if host else black.new_zeros(black.shape)
        if out_alpha is None:
            shp = black.shape[:2]
            out_alpha = np.zeros(shp, np.uint8) if host else black.new_zeros(shp, dtype=__import__("torch").uint8)
        wa = ctypes.byref(plane_image(white_alpha)) if white_alpha is not None else None
        ba = ctypes.byref(plane_image(black_alpha)) if black_alpha is not None else None
        l0 = _ptr_and_strides(level0)[0] if level0 is not None else None
        o = self._options(levels, wrap, False, dither, seed, host, l0, plain, coarse_pixels)
        self._check(self.lib.enb_enblend(self.handle, ctypes.byref(pixel_image(white)), wa,
                                         ctypes.byref(pixel_image(black)), ba, ctypes.byref(plane_image(mask)),
                                         ctypes.byref(pixel_image(out)), ctypes.byref(plane_image(out_alpha)),
                                         ctypes.byref(o)))
        return out, out_alpha

    def nft_mask(self, white_alpha, black_alpha, mask=None, wrap: bool = False):
        """enblend's seam mask from the nearest-feature transform (enb_nft_mask): 255 where the white image
        wins.  Alpha planes (H, W) uint8, numpy (host buffers) or torch (device); returns the mask."""
        host = not _is_torch(white_alpha)
        if mask is None:
            shp = white_alpha.shape
            mask = np.zeros(shp, np.uint8) if host else white_alpha.new_zeros(shp)
        o = self._options(0, wrap, False, "hash", 0, host, None)
        self._check(self.lib.enb_nft_mask(self.handle, ctypes.byref(plane_image(white_alpha)),
                                          ctypes.byref(plane_image(black_alpha)), ctypes.byref(plane_image(mask)),
                                          ctypes.byref(o)))
        return mask


def pitched(x, align: int = 128):
    """A CUDA copy of the image x ((H, W) or (H, W, S), numpy or torch) whose
    rows start on `align`-byte boundaries, the layout the host-buffer entry
    points stage into (as cudaMallocPitch would give): the level-0 passes then
    move whole tiles with 2-D TMA boxes whatever the image width."""
    import torch
    t = x if _is_torch(x) else torch.from_numpy(np.ascontiguousarray(x))
    es = t.element_size()
    row = t.shape[1] * (t.shape[2] if t.ndim == 3 else 1) * es
    pitch = (row + align - 1) // align * align
    buf = torch.empty(t.shape[0] * pitch // es, dtype=t.dtype, device="cuda")
    strides = (pitch // es,) + tuple(t.stride()[1:])
    out = buf.as_strided(tuple(t.shape), strides)
    out.copy_(t)
    return out


def num_levels(width: int, height: int, min_levels: int = 1, exact_levels: int = 0) -> int:
    """roiBounds level count (src/bounds.h:97-177)."""
    return load_library().enb_num_levels(width, height, min_levels, exact_levels)


__all__ = ["Context", "Pyramid", "EnbError", "EnbImage", "EnbEnfuseParams", "EnbFuseOptions", "enfuse_params",
           "num_levels", "pitched", "exposure_table_of", "load_library", "header_functions", "pixel_image", "plane_image",
           "ENB_U8", "ENB_U16", "ENB_F32", "ENB_I16", "ENB_I32"]
