"""Launch shapes and autotuning of FP / BP (include/mexct.h, "launch shapes and
autotuning").  No counterpart in the reference, whose kernels have one launch shape.

Every FP / BP call belongs to a shape class (operator, geometry, W, H, view count
rounded up to a power of two, storage types); a context keeps one shape per class.
``set_mode(TUNE_AUTO)`` makes the first call of each class time every candidate on
its own buffers; ``shape_set`` pins a shape; ``autotune_fp`` / ``autotune_bp`` tune a
class now.  All functions act on the default context of the current device.
"""
from __future__ import annotations

import ctypes

from . import _lib
from .ops import _angles, _dptr, _dtype_code, _geom_flag, _ptr, _stream

_P, _i, _f, _d = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_double
FIXED, HEURISTIC, AUTO = _lib.TUNE_FIXED, _lib.TUNE_HEURISTIC, _lib.TUNE_AUTO
FP, BP = _lib.OP_FP, _lib.OP_BP


class Shape(ctypes.Structure):
    _fields_ = [("variant", _i), ("zc", _i), ("rows", _i), ("vblocks", _i)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_SP = ctypes.POINTER(Shape)
_DP = ctypes.POINTER(_d)
_lib.register("mexct_ctx_set_tune_mode", [_P, _i])
_lib.register("mexct_shape_set", [_P, _i, _i, _i, _i, _i, _i, _i, _SP])
_lib.register("mexct_shape_get", [_P, _i, _i, _i, _i, _i, _i, _i, _SP, _DP, ctypes.POINTER(_i)])
_lib.register("mexct_shape_clear", [_P])
_lib.register("mexct_autotune_fp", [_P, _P, _i, _i, _i, _f, _P, _i, _i, _P, _i, _P, _SP, _DP])
_lib.register("mexct_autotune_bp", [_P, _P, _i, _i, _i, _i, _f, _P, _i, _P, _i, _P, _SP, _DP])

_CODES = {"float32": _lib.F32, "float16": _lib.F16, "bfloat16": _lib.BF16}


def _code(t):
    if isinstance(t, int):
        return t
    return _CODES[str(t).replace("torch.", "")]


def set_mode(mode: int) -> None:
    _lib.call("mexct_ctx_set_tune_mode", None, int(mode))


def shape_set(op, geom, W, H, nP, in_dtype="float32", out_dtype="float32", variant=0, zc=16,
              rows=8, vblocks=1) -> None:
    s = Shape(int(variant), int(zc), int(rows), int(vblocks))
    _lib.call("mexct_shape_set", None, int(op), _geom_flag(geom), int(W), int(H), int(nP),
              _code(in_dtype), _code(out_dtype), ctypes.byref(s))


def shape_get(op, geom, W, H, nP, in_dtype="float32", out_dtype="float32") -> dict:
    s, ms, tuned = Shape(), _d(), _i()
    _lib.call("mexct_shape_get", None, int(op), _geom_flag(geom), int(W), int(H), int(nP),
              _code(in_dtype), _code(out_dtype), ctypes.byref(s), ctypes.byref(ms),
              ctypes.byref(tuned))
    out = s.as_dict()
    out.update(ms=ms.value, tuned=tuned.value)
    return out


def clear() -> None:
    _lib.call("mexct_shape_clear", None)


def autotune_bp(sino, sad, angles, geom, out=None, out_dtype=None, stream=None):
    """Tune the BP class of this call and return (volume, shape dict, best ms)."""
    import torch
    nP, H, W = sino.shape
    ang = _angles(angles, nP)
    if out is None:
        out = torch.empty((H, W, W), dtype=out_dtype or torch.float32, device=sino.device)
    s, ms = Shape(), _d()
    _lib.call("mexct_autotune_bp", None, _dptr(sino), _dtype_code(sino), W, H, nP, float(sad),
              _ptr(ang), _geom_flag(geom), _dptr(out), _dtype_code(out), _stream(stream),
              ctypes.byref(s), ctypes.byref(ms))
    return out, s.as_dict(), ms.value


def autotune_fp(vol, sad, angles, geom, out=None, out_dtype=None, stream=None):
    """Tune the FP class of this call and return (sinogram, shape dict, best ms)."""
    import torch
    H, W, _ = vol.shape
    ang = _angles(angles, 0)
    nP = ang.size
    if out is None:
        out = torch.empty((nP, H, W), dtype=out_dtype or vol.dtype, device=vol.device)
    s, ms = Shape(), _d()
    _lib.call("mexct_autotune_fp", None, _dptr(vol), _dtype_code(vol), W, H, float(sad), _ptr(ang),
              nP, _geom_flag(geom), _dptr(out), _dtype_code(out), _stream(stream),
              ctypes.byref(s), ctypes.byref(ms))
    return out, s.as_dict(), ms.value
