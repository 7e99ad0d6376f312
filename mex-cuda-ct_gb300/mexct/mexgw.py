"""Call the MEX gateways (mex-cuda-ct_gb300/mex/*.cpp) through the stub MEX runtime.

The gateways are compiled against the stub ``mex.h`` into ``_build/libmexct_mex.so``;
``call("CUDAmex_FP", vol, SAD, angles, nProj, geomFlag)`` builds mxArrays from numpy
values (float32 -> single, float64 -> double, int32 -> int32, Python scalars -> 1x1
double), invokes the gateway exactly as MATLAB would, and returns plhs as numpy
arrays.  Arguments that a gateway updates in place (CUDAmex_oscIter's mu) are
copied back into the caller's array, as MATLAB's shared data would show them.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _lib

_CLS = {np.dtype(np.float64): 6, np.dtype(np.float32): 7, np.dtype(np.int32): 12}
_DT = {6: np.float64, 7: np.float32, 12: np.int32}
_mex = None


class MexError(RuntimeError):
    def __init__(self, ident: str, msg: str):
        super().__init__("%s: %s" % (ident, msg))
        self.identifier = ident


def load():
    global _mex
    if _mex is not None:
        return _mex
    _lib.load()  # libmexct first (the stub links against it)
    path = os.path.join(_lib.PKG, "_build", "libmexct_mex.so")
    if not os.path.exists(path):
        raise RuntimeError("MEX stub harness not built: %s" % path)
    m = ctypes.CDLL(path)
    P = ctypes.c_void_p
    m.mxs_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_size_t), P]
    m.mxs_create.restype = P
    m.mxs_destroy.argtypes = [P]
    m.mxs_data.argtypes = [P]
    m.mxs_data.restype = P
    m.mxs_class.argtypes = [P]
    m.mxs_ndim.argtypes = [P]
    m.mxs_dim.argtypes = [P, ctypes.c_int]
    m.mxs_dim.restype = ctypes.c_size_t
    m.mxs_error.restype = ctypes.c_char_p
    m.mxs_error_id.restype = ctypes.c_char_p
    m.mxs_call.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(P), ctypes.c_int,
                           ctypes.POINTER(P)]
    _mex = m
    return m


def _to_mx(m, v):
    a = np.asarray(v)
    if a.dtype not in _CLS:
        if np.issubdtype(a.dtype, np.number) or a.dtype == bool:
            a = a.astype(np.float64)
        else:
            raise TypeError("unsupported MATLAB value %r" % (v,))
    a = np.asfortranarray(a)
    dims = list(a.shape) or [1, 1]
    if len(dims) == 1:
        dims = [dims[0], 1]
    cd = (ctypes.c_size_t * len(dims))(*dims)
    h = m.mxs_create(_CLS[a.dtype], len(dims), cd, ctypes.c_void_p(a.ctypes.data) if a.size else None)
    return h


def _from_mx(m, h):
    cls = m.mxs_class(h)
    nd = m.mxs_ndim(h)
    shape = tuple(int(m.mxs_dim(h, i)) for i in range(nd))
    n = int(np.prod(shape))
    dt = np.dtype(_DT[cls])
    buf = (ctypes.c_char * (n * dt.itemsize)).from_address(m.mxs_data(h)) if n else b""
    return np.frombuffer(bytes(buf), dtype=dt).reshape(shape, order="F").copy(order="F")


def call(name: str, *args, nlhs: int = 1, inplace: tuple = ()):
    """Invoke a gateway; returns a tuple of nlhs outputs (or a single array)."""
    m = load()
    hs = [_to_mx(m, a) for a in args]
    prhs = (ctypes.c_void_p * max(1, len(hs)))(*hs)
    plhs = (ctypes.c_void_p * max(1, nlhs))()
    try:
        rc = m.mxs_call(name.encode(), nlhs, plhs, len(hs), prhs)
        if rc == 2:
            raise ValueError("unknown gateway %s" % name)
        if rc == 1:
            raise MexError(m.mxs_error_id().decode(), m.mxs_error().decode())
        for i in inplace:
            out = _from_mx(m, hs[i])
            np.copyto(args[i], out.reshape(np.shape(args[i]), order="F"))
        outs = [_from_mx(m, plhs[i]) for i in range(nlhs) if plhs[i]]
    finally:
        for h in hs:
            m.mxs_destroy(h)
        for i in range(nlhs):
            if plhs[i]:
                m.mxs_destroy(plhs[i])
    if nlhs <= 1:
        return outs[0] if outs else None
    return tuple(outs)
