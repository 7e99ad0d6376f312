"""Batched FP/BP over many independent problems (include/mexct_batch.h).

``Batch([...])`` plans one persistent FP launch and per-problem BP launches (fanned
out over 8 streams) over problems of different sizes, geometries and view counts;
``fp()`` / ``bp()`` are stream-ordered and can be captured in a CUDA graph.  Each problem is a dict with
``vol`` (H, W, W) float32 CUDA tensor, ``sino`` (nP, H, W), ``rec`` (H, W, W),
``angles`` (float32 numpy), ``sad`` and ``geom``.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

_P, _i, _f = ctypes.c_void_p, ctypes.c_int, ctypes.c_float


class Problem(ctypes.Structure):
    _fields_ = [("W", _i), ("H", _i), ("nP", _i), ("geom", _i), ("sad", _f), ("angles", _P),
                ("d_vol", _P), ("d_sino", _P), ("d_rec", _P)]


_lib.register("mexct_batch_create", [_P, ctypes.POINTER(Problem), _i, ctypes.POINTER(_P)])
_lib.register("mexct_batch_fp", [_P, _P])
_lib.register("mexct_batch_bp", [_P, _P])
_lib.register("mexct_batch_destroy", [_P])


class Batch:
    def __init__(self, problems):
        self._keep = []
        arr = (Problem * len(problems))()
        for i, p in enumerate(problems):
            H, W, _ = p["vol"].shape
            ang = np.ascontiguousarray(np.asarray(p["angles"], dtype=np.float32).ravel())
            self._keep.append(ang)
            arr[i] = Problem(W, H, ang.size, int(p["geom"]), float(p["sad"]), ang.ctypes.data,
                             p["vol"].data_ptr(), p["sino"].data_ptr(), p["rec"].data_ptr())
        h = _P()
        _lib.call("mexct_batch_create", None, arr, len(problems), ctypes.byref(h))
        self.h = h
        self.problems = problems

    def fp(self, stream=None):
        import torch

        s = stream if stream is not None else torch.cuda.current_stream()
        _lib.call("mexct_batch_fp", self.h, _P(s.cuda_stream))

    def bp(self, stream=None):
        import torch

        s = stream if stream is not None else torch.cuda.current_stream()
        _lib.call("mexct_batch_bp", self.h, _P(s.cuda_stream))

    def close(self):
        if getattr(self, "h", None):
            _lib.load().mexct_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
