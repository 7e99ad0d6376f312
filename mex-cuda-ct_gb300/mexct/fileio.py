"""Scanner data files: MATLAB MAT-files (Level 5 read and written, -v7.3 / HDF5 read)
and VFF volumes (include/mexct.h,
"scanner data files").  Arrays come back as float32, column-major (Fortran order),
the layout the MEX-style entry points take."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


def _b(s):
    return None if s is None else str(s).encode()


def mat_list(path) -> list[str]:
    """Names of the variables in a MAT-file: in file order (Level 5), in name order
    (-v7.3)."""
    buf = ctypes.create_string_buffer(1 << 16)
    _lib.call("mexct_mat_list", _b(path), buf, len(buf))
    txt = buf.value.decode()
    return txt.split("\n") if txt else []


def read_mat(path, name=None) -> np.ndarray:
    """Real part of a numeric variable (the first numeric one if name is None) as float32."""
    nd = ctypes.c_int()
    dims = (ctypes.c_longlong * 8)()
    _lib.call("mexct_mat_info", _b(path), _b(name), ctypes.byref(nd), dims)
    shape = tuple(int(dims[i]) for i in range(nd.value))
    out = np.empty(shape, dtype=np.float32, order="F")
    _lib.call("mexct_mat_read", _b(path), _b(name), ctypes.c_void_p(out.ctypes.data),
              int(out.size))
    return out


FORMATS = {None: 0, "auto": 0, "v5": 5, "v7.3": 73}


def write_mat(path, name, arr, append=False, format=None) -> None:
    """Write arr as a single-precision variable (at least 2 dimensions, as MATLAB has).
    format: "v5" (Level 5), "v7.3" (HDF5) or None (the appended file's format, else
    -v7.3 for 2 GB or more)."""
    a = np.asfortranarray(np.asarray(arr, dtype=np.float32))
    if a.ndim < 2:
        a = a.reshape((1, -1) if a.ndim == 1 else (1, 1), order="F")
    dims = (ctypes.c_longlong * a.ndim)(*a.shape)
    _lib.call("mexct_mat_write_ex", _b(path), _b(name), ctypes.c_void_p(a.ctypes.data), a.ndim,
              dims, 1 if append else 0, FORMATS[format])


def read_vff(path):
    """(volume [X, Y, Z] float32 Fortran order, spacing (3,), bits)."""
    dims = (ctypes.c_int * 3)()
    sp = (ctypes.c_float * 3)()
    bits = ctypes.c_int()
    _lib.call("mexct_vff_info", _b(path), dims, sp, ctypes.byref(bits))
    out = np.empty(tuple(dims), dtype=np.float32, order="F")
    _lib.call("mexct_vff_read", _b(path), ctypes.c_void_p(out.ctypes.data), int(out.size))
    return out, np.array(list(sp), dtype=np.float32), bits.value


def write_vff(path, vol, spacing=(1.0, 1.0, 1.0), bits=32) -> None:
    """Write a volume [X, Y, Z] (bits 16: rounded, saturated to int16; 32: float)."""
    a = np.asfortranarray(np.asarray(vol, dtype=np.float32))
    if a.ndim == 2:
        a = a[:, :, None]
    dims = (ctypes.c_int * 3)(*a.shape)
    sp = (ctypes.c_float * 3)(*[float(x) for x in spacing])
    _lib.call("mexct_vff_write", _b(path), ctypes.c_void_p(a.ctypes.data), dims, sp, int(bits))
