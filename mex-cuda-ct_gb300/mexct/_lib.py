"""ctypes binding of libmexct.so (the C ABI of include/mexct.h).

The library is built in-tree by ``mex-cuda-ct_gb300/build.py`` into
``mex-cuda-ct_gb300/_build/libmexct.so``.  Loading fails loudly when it is missing:
there is no CPU fallback behind this module.
"""
from __future__ import annotations

import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(_HERE)
LIB_PATH = os.path.join(PKG, "_build", "libmexct.so")

OK, ERR_ARG, ERR_CUDA, ERR_OOM, ERR_UNSUPPORTED, ERR_TIMEOUT, ERR_BUDGET, ERR_IO = range(8)
F32, F16, BF16 = 0, 1, 2
FP_EXPLICIT, FP_TEXTURE, FP_RAY, FP_AUTO = 0, 1, 2, 3
OP_FP, OP_BP = 0, 1
TUNE_FIXED, TUNE_HEURISTIC, TUNE_AUTO = 0, 1, 2

_lock = threading.Lock()
_lib = None


class Detector(ctypes.Structure):
    """struct mexct_detector: det_w x det_h pixels of pitch du x dv, ss x ss FP rays per pixel."""

    _fields_ = [("det_w", ctypes.c_int), ("det_h", ctypes.c_int), ("du", ctypes.c_float),
                ("dv", ctypes.c_float), ("ss", ctypes.c_int)]


class MexctError(RuntimeError):
    """A libmexct call returned a non-zero status."""

    def __init__(self, status: int, msg: str):
        super().__init__("mexct status %d: %s" % (status, msg))
        self.status = status


_c = ctypes
_P = _c.c_void_p
_F = _c.POINTER(_c.c_float)
_I32 = _c.POINTER(_c.c_int32)
_i, _f = _c.c_int, _c.c_float

# name -> argtypes (restype is int status unless listed in _RESTYPES)
SIGNATURES = {
    "mexct_last_error": [],
    "mexct_version": [],
    "mexct_ctx_create": [_i, _c.POINTER(_P)],
    "mexct_ctx_destroy": [_P],
    "mexct_ctx_trim": [_P],
    "mexct_fp": [_P, _P, _i, _i, _f, _P, _i, _i, _P],
    "mexct_bp": [_P, _P, _i, _i, _i, _f, _P, _i, _P],
    "mexct_g3d_fp": [_P, _P, _i, _i, _P, _P, _i, _i, _i, _i, _P],
    "mexct_g3d_bp": [_P, _P, _i, _i, _i, _P, _P, _i, _i, _i, _P],
    "mexct_osc_iter": [_P, _P, _P, _P, _i, _i, _i, _i, _P, _P, _f, _i],
    "mexct_tvmin3d": [_P, _P, _i, _i, _i, _f, _i, _P],
    "mexct_prefilter": [_P, _P, _P, _i, _i, _i, _P, _i, _f, _i, _f, _f, _P],
    "mexct_fbp": [_P, _P, _P, _i, _i, _i, _P, _i, _f, _i, _f, _f, _P],
    "mexct_parker_weight": [_P, _i, _i, _i, _P, _i, _c.c_double, _c.c_double, _P],
    "mexct_fp_dev": [_P, _P, _i, _i, _f, _P, _i, _i, _P, _P],
    "mexct_bp_dev": [_P, _P, _i, _i, _i, _f, _P, _i, _P, _P],
    "mexct_g3d_fp_dev": [_P, _P, _i, _i, _P, _P, _i, _i, _i, _i, _P, _P],
    "mexct_g3d_bp_dev": [_P, _P, _i, _i, _i, _P, _P, _i, _i, _i, _P, _P],
    "mexct_g3d_bp_matched": [_P, _P, _i, _i, _i, _P, _P, _i, _i, _i, _P],
    "mexct_osc_iter_det_dev": [_P, _P, _P, _P, _P, _i, _i, _i, _i, _P, _P, _f, _i, _P],
    "mexct_g3d_bp_matched_dev": [_P, _P, _i, _i, _i, _P, _P, _i, _i, _i, _P, _P],
    "mexct_osc_iter_dev": [_P, _P, _P, _P, _i, _i, _i, _i, _P, _P, _f, _i, _P],
    "mexct_tvmin3d_dev": [_P, _P, _i, _i, _i, _f, _i, _P, _P],
    "mexct_prefilter_dev": [_P, _P, _P, _i, _i, _i, _P, _i, _f, _i, _f, _f, _P, _P],
    "mexct_fp_dev_ex": [_P, _P, _i, _i, _i, _f, _P, _i, _i, _P, _i, _i, _P],
    "mexct_bp_dev_ex": [_P, _P, _i, _i, _i, _i, _f, _P, _i, _P, _i, _P],
    "mexct_fp_det_dev": [_P, _P, _i, _i, _f, _P, _i, _i, _P, _P, _P],
    "mexct_bp_det_dev": [_P, _P, _P, _i, _f, _P, _i, _i, _i, _P, _P],
    "mexct_fp_det": [_P, _P, _i, _i, _f, _P, _i, _i, _P, _P],
    "mexct_bp_det": [_P, _P, _P, _i, _f, _P, _i, _i, _i, _P],
    "mexct_sub_rows": [_i, _i, _f, _i, _i, _i, _c.POINTER(_i), _c.POINTER(_i)],
    "mexct_fp_sub_dev": [_P, _P, _i, _i, _i, _i, _f, _P, _i, _i, _P, _i, _P],
    "mexct_bp_sub_dev": [_P, _P, _i, _i, _i, _i, _i, _f, _P, _i, _i, _i, _P, _i, _P],
    "mexct_fp_ooc": [_P, _P, _i, _i, _f, _P, _i, _i, _c.c_size_t, _P],
    "mexct_bp_ooc": [_P, _P, _i, _i, _i, _f, _P, _i, _c.c_size_t, _P],
    "mexct_mat_list": [_c.c_char_p, _c.c_char_p, _c.c_size_t],
    "mexct_mat_info": [_c.c_char_p, _c.c_char_p, _c.POINTER(_i), _c.POINTER(_c.c_longlong)],
    "mexct_mat_read": [_c.c_char_p, _c.c_char_p, _P, _c.c_longlong],
    "mexct_mat_write": [_c.c_char_p, _c.c_char_p, _P, _i, _c.POINTER(_c.c_longlong), _i],
    "mexct_mat_write_ex": [_c.c_char_p, _c.c_char_p, _P, _i, _c.POINTER(_c.c_longlong), _i, _i],
    "mexct_vff_info": [_c.c_char_p, _c.POINTER(_i), _F, _c.POINTER(_i)],
    "mexct_vff_read": [_c.c_char_p, _P, _c.c_longlong],
    "mexct_vff_write": [_c.c_char_p, _P, _c.POINTER(_i), _F, _i],
    "mexct_fp_slab_occupancy": [_c.POINTER(_i)],
    "mexct_ctx_set_wait_limit": [_P, _i],
    "mexct_ctx_device_errors": [_P, _c.POINTER(_c.c_uint), _i],
}
_RESTYPES = {"mexct_last_error": _c.c_char_p, "mexct_version": _c.c_char_p}
OPTIONAL = {}  # symbols declared later in the header are added by their modules


def lib_path() -> str:
    return LIB_PATH


def load(path: str | None = None):
    """Load libmexct.so once; raise if it was not built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise RuntimeError("libmexct.so not built (%s): run __graft_entry__.build() "
                               "or python mex-cuda-ct_gb300/build.py" % p)
        lib = _c.CDLL(p)
        for name, args in {**SIGNATURES, **OPTIONAL}.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = _RESTYPES.get(name, _c.c_int)
        _lib = lib
        return lib


def register(name: str, argtypes, restype=_c.c_int):
    """Declare an additional symbol (used by modules that wrap newer entry points)."""
    OPTIONAL[name] = argtypes
    if restype is not _c.c_int:
        _RESTYPES[name] = restype
    if _lib is not None:
        fn = getattr(_lib, name)
        fn.argtypes = argtypes
        fn.restype = restype


def last_error() -> str:
    return load().mexct_last_error().decode(errors="replace")


def check(status: int) -> None:
    if status != OK:
        raise MexctError(status, last_error())


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args))
