"""Request server (include/mexct_serve.h): continuous batching of FDK / OSC-TV requests.

``Server(slots, budget_bytes)`` admits queued requests to free slots while their HBM
footprint fits the budget; each slot runs on its own stream so requests overlap on
the device.  ``submit_fdk`` / ``submit_osctv`` take MATLAB-layout numpy arrays (pre,
post [W, H, nP] float32) and return a ticket; ``wait(ticket)`` returns the
reconstruction [W, W, H] and the queue / run / total seconds.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .ops import FILTERS, _angles, _f32F

_P, _i, _f, _d = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_double
FDK, OSCTV = 0, 1


class Request(ctypes.Structure):
    _fields_ = [("kind", _i), ("W", _i), ("H", _i), ("nP", _i), ("geom", _i), ("sad", _f),
                ("mu_type", _i), ("angles", _P), ("pre", _P), ("post", _P), ("recon", _P),
                ("filter", _i), ("cutoff", _f), ("q", _f), ("n_iter", _i), ("tv_const", _f),
                ("n_sub_init", _i), ("n_sub_final", _i), ("p_val", _f), ("first_picks", _P),
                ("simulate_s", _d), ("data_type", _i)]


class Stats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_longlong), ("completed", ctypes.c_longlong),
                ("failed", ctypes.c_longlong), ("rejected", ctypes.c_longlong),
                ("bytes_in_use", ctypes.c_size_t), ("peak_bytes", ctypes.c_size_t),
                ("budget", ctypes.c_size_t), ("max_concurrent", _i)]


_U64 = ctypes.c_ulonglong
_lib.register("mexct_request_bytes", [ctypes.POINTER(Request)], ctypes.c_size_t)
_lib.register("mexct_server_create", [_i, _i, ctypes.c_size_t, ctypes.POINTER(_P)])
_lib.register("mexct_server_submit", [_P, ctypes.POINTER(Request), ctypes.POINTER(_U64)])
_lib.register("mexct_server_wait", [_P, _U64, _d, ctypes.POINTER(_i), ctypes.POINTER(_d),
                                    ctypes.POINTER(_d), ctypes.POINTER(_d)])
_lib.register("mexct_server_stats_get", [_P, ctypes.POINTER(Stats)])
_lib.register("mexct_server_destroy", [_P])


class Server:
    def __init__(self, slots=4, budget_bytes=64 << 30, device=0):
        h = _P()
        _lib.call("mexct_server_create", int(device), int(slots), int(budget_bytes), ctypes.byref(h))
        self.h = h
        self._keep = {}

    def _submit(self, req, keep):
        t = _U64()
        _lib.call("mexct_server_submit", self.h, ctypes.byref(req), ctypes.byref(t))
        self._keep[t.value] = keep
        return t.value

    def _arrays(self, pre, post, angles):
        pre = _f32F(pre, "pre")
        post = _f32F(post, "post")
        W, H, nP = post.shape
        ang = _angles(angles, nP)
        rec = np.zeros((W, W, H), dtype=np.float32, order="F")
        return pre, post, ang, rec, W, H, nP

    def submit_fdk(self, pre, post, angles, geom, sad=1000.0, filt="hamming", cutoff=1.0, q=1.0):
        pre, post, ang, rec, W, H, nP = self._arrays(pre, post, angles)
        r = Request(FDK, W, H, nP, int(geom), float(sad), 0, ang.ctypes.data, pre.ctypes.data,
                    post.ctypes.data, rec.ctypes.data, FILTERS[filt], float(cutoff), float(q),
                    0, 0.0, 0, 0, 0.0, None, 0.0)
        return self._submit(r, (pre, post, ang, rec))

    def submit_osctv(self, pre, post, angles, geom, first_picks, n_iter=10, tv_const=0.2,
                     n_sub=10, sad=1000.0, mu_type=_lib.F32, n_sub_final=None, p_val=1.0,
                     data_type=_lib.F32):
        """data_type: storage of the residual views (F32, or F16 with FP32 mu)."""
        pre, post, ang, rec, W, H, nP = self._arrays(pre, post, angles)
        fp = np.ascontiguousarray(np.asarray(first_picks, dtype=np.int32).ravel())
        r = Request(OSCTV, W, H, nP, int(geom), float(sad), int(mu_type), ang.ctypes.data,
                    pre.ctypes.data, post.ctypes.data, rec.ctypes.data, 0, 0.0, 0.0, int(n_iter),
                    float(tv_const), int(n_sub), int(n_sub if n_sub_final is None else n_sub_final),
                    float(p_val), fp.ctypes.data, 0.0, int(data_type))
        return self._submit(r, (pre, post, ang, rec, fp))

    def submit_simulated(self, seconds, W=64, H=64, nP=60, kind=FDK):
        r = Request(kind, W, H, nP, 0, 1000.0, 0, None, None, None, None, 4, 1.0, 1.0, 1, 0.0,
                    1, 1, 1.0, None, float(seconds))
        return self._submit(r, None)

    @staticmethod
    def request_bytes(kind, W, H, nP, mu_type=_lib.F32, n_sub=1, data_type=_lib.F32):
        r = Request(kind, W, H, nP, 0, 1000.0, int(mu_type), None, None, None, None, 0, 0.0, 0.0,
                    1, 0.0, int(n_sub), int(n_sub), 1.0, None, 0.0, int(data_type))
        return int(_lib.load().mexct_request_bytes(ctypes.byref(r)))

    def wait(self, ticket, timeout=-1.0):
        st, q, r, t = _i(), _d(), _d(), _d()
        _lib.call("mexct_server_wait", self.h, _U64(ticket), float(timeout), ctypes.byref(st),
                  ctypes.byref(q), ctypes.byref(r), ctypes.byref(t))
        keep = self._keep.pop(ticket)
        if st.value != 0:
            raise _lib.MexctError(st.value, _lib.last_error())
        rec = keep[3] if keep is not None else None
        return rec, {"queue_s": q.value, "run_s": r.value, "total_s": t.value}

    def stats(self):
        s = Stats()
        _lib.call("mexct_server_stats_get", self.h, ctypes.byref(s))
        return {k: getattr(s, k) for k, _ in Stats._fields_}

    def close(self):
        if getattr(self, "h", None):
            _lib.load().mexct_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
