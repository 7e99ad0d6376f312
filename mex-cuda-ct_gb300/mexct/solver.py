"""Device-resident OSC-TV (include/mexct_solver.h) and the OSC_TV_recon mirror.

``OSC_TV_recon(pre, post, angles, geom, numIter, TV_constant, numSubsInit,
numSubsFinal, pVal, first_picks)`` keeps the MATLAB driver's argument list
(iterative_reconstruction/OSC_TV_recon.m:1); the randperm draw of each iteration's
first subset is passed explicitly (``first_picks``, 0-based) so results are
reproducible.  ``OscTvSolver`` keeps mu, pre and post on the device across calls,
can capture iterations as CUDA graphs, and snapshots / restores its state.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .ops import _angles, _f32F, _geom_struct, _ptr

_P, _i, _f, _d = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_double


class Params(ctypes.Structure):
    _fields_ = [("n_iter", _i), ("tv_const", _f), ("n_sub_init", _i), ("n_sub_final", _i),
                ("p_val", _f), ("use_graph", _i), ("objective", _i)]


_lib.register("mexct_osctv_create", [_P, _P, _P, _i, _i, _i, _P, _f, _i, _i, _P, ctypes.POINTER(_P)])
_lib.register("mexct_osctv_create_ex", [_P, _P, _P, _i, _i, _i, _P, _f, _i, _i, _i, _P,
                                        ctypes.POINTER(_P)])
_lib.register("mexct_osctv_run", [_P, ctypes.POINTER(Params), _P, _i, _P])
_lib.register("mexct_osctv_mu", [_P, _P, _P])
_lib.register("mexct_osctv_stats", [_P, ctypes.POINTER(_i), ctypes.POINTER(_d), ctypes.POINTER(_d)])
_lib.register("mexct_osctv_state_bytes", [_P], ctypes.c_size_t)
_lib.register("mexct_osctv_snapshot", [_P, _P, _P])
_lib.register("mexct_osctv_restore", [_P, _P, _P])
_lib.register("mexct_osctv_destroy", [_P])
_lib.register("mexct_osc_tv_recon", [_P, _P, _P, _i, _i, _i, _P, _f, _i, _i, _f, _i, _i, _f, _P, _P])
_lib.register("mexct_osc_tv_recon_ooc", [_P, _P, _P, _i, _i, _i, _P, _f, _i, _i, _f, _i, _i, _f, _P,
                                         ctypes.c_size_t, _P, ctypes.POINTER(_i)])
_lib.register("mexct_osc_tv_ooc_plan", [_i, _i, _i, _i, _i, _i, _i, _f, ctypes.c_size_t,
                                        ctypes.POINTER(_i), ctypes.POINTER(ctypes.c_size_t)])
_lib.register("mexct_num_subsets", [_i, _i, _f, _i, _i])
_lib.register("mexct_subset_order", [_i, _i, _P])


def num_subsets(s_init, s_final, p_val, max_iters, k):
    return int(_lib.load().mexct_num_subsets(int(s_init), int(s_final), float(p_val),
                                             int(max_iters), int(k)))


def subset_order(n, first):
    out = np.zeros(int(n), dtype=np.int32)
    _lib.call("mexct_subset_order", int(n), int(first), _ptr(out))
    return out


def random_first_picks(numIter, numSubsInit, numSubsFinal, pVal, seed=None):
    """One random first subset per iteration, 0-based, as OSC_TV_recon.m draws it
    (randperm(numSubsets, 1), :82) for that iteration's subset count (:76-78)."""
    rng = np.random.default_rng(seed)
    return np.array([rng.integers(0, max(1, num_subsets(numSubsInit, numSubsFinal, pVal,
                                                          numIter, k)))
                     for k in range(1, int(numIter) + 1)], dtype=np.int32)


def _picks(first_picks, numIter, numSubsInit, numSubsFinal, pVal):
    if first_picks is None:
        return random_first_picks(numIter, numSubsInit, numSubsFinal, pVal)
    fp = np.ascontiguousarray(np.asarray(first_picks, dtype=np.int32).ravel())
    if fp.size < int(numIter):
        raise ValueError("first_picks needs one entry per iteration")
    return fp


def OSC_TV_recon(pre, post, scanAngles, geom, numIter, TV_constant, numSubsInit, numSubsFinal,
                 pVal, first_picks=None):
    """recon = OSC_TV_recon(...) on the GPU (host arrays in, float32 [W, W, H] out).
    first_picks: each iteration's first subset (0-based); None draws them at random
    as the reference does."""
    pre = _f32F(pre, "pre")
    post = _f32F(post, "post")
    W, H, nP = post.shape
    g, sad = _geom_struct(geom)
    ang = _angles(scanAngles, nP)
    fp = _picks(first_picks, numIter, numSubsInit, numSubsFinal, pVal)
    out = np.empty((W, W, H), dtype=np.float32, order="F")
    _lib.call("mexct_osc_tv_recon", None, _ptr(pre), _ptr(post), W, H, nP, _ptr(ang), float(sad),
              g, int(numIter), float(TV_constant), int(numSubsInit), int(numSubsFinal),
              float(pVal), _ptr(fp), _ptr(out))
    return out


def ooc_plan(W, H, nP, geom, numIter, numSubsInit, numSubsFinal, pVal, budget_bytes):
    """(slab thickness in slices, device bytes) of OSC_TV_recon_ooc within budget_bytes."""
    g = int(geom) if isinstance(geom, (int, np.integer)) else _geom_struct(geom)[0]
    planes, nbytes = _i(0), ctypes.c_size_t(0)
    _lib.call("mexct_osc_tv_ooc_plan", int(W), int(H), int(nP), g, int(numIter), int(numSubsInit),
              int(numSubsFinal), float(pVal), int(budget_bytes), ctypes.byref(planes),
              ctypes.byref(nbytes))
    return planes.value, nbytes.value


def OSC_TV_recon_ooc(pre, post, scanAngles, geom, numIter, TV_constant, numSubsInit,
                     numSubsFinal, pVal, first_picks, budget_bytes):
    """OSC_TV_recon with mu in host memory, streamed through the device in
    z-slabs within budget_bytes of device memory.  Returns (recon, slab
    thickness in slices); first_picks None draws them as the reference does."""
    pre = _f32F(pre, "pre")
    post = _f32F(post, "post")
    W, H, nP = post.shape
    g, sad = _geom_struct(geom)
    ang = _angles(scanAngles, nP)
    fp = _picks(first_picks, numIter, numSubsInit, numSubsFinal, pVal)
    out = np.empty((W, W, H), dtype=np.float32, order="F")
    planes = _i(0)
    _lib.call("mexct_osc_tv_recon_ooc", None, _ptr(pre), _ptr(post), W, H, nP, _ptr(ang),
              float(sad), g, int(numIter), float(TV_constant), int(numSubsInit),
              int(numSubsFinal), float(pVal), _ptr(fp), int(budget_bytes), _ptr(out),
              ctypes.byref(planes))
    return out, planes.value


class OscTvSolver:
    """Resident OSC-TV state for device tensors pre/post (nP, H, W) float32.

    mu_dtype: storage of mu (float32, bfloat16; float16 underflows the initial
    mu).  data_dtype: storage of the residual views between the forward pass and
    the dual BP (float32, or float16 with one power-of-two scale; FP32 mu only)."""

    def __init__(self, pre, post, angles, sad, geom, mu_dtype=None, stream=None,
                 data_dtype=None):
        import torch

        self._torch = torch
        nP, H, W = pre.shape
        self.W, self.H, self.nP = W, H, nP
        self.angles = _angles(angles, nP)
        codes = {None: _lib.F32, torch.float32: _lib.F32, torch.float16: _lib.F16,
                 torch.bfloat16: _lib.BF16}
        code, dcode = codes[mu_dtype], codes[data_dtype]
        self.stream = stream if stream is not None else torch.cuda.current_stream()
        h = _P()
        _lib.call("mexct_osctv_create_ex", None, _P(pre.data_ptr()), _P(post.data_ptr()), W, H,
                  nP, _ptr(self.angles), float(sad), int(geom), code, dcode,
                  _P(self.stream.cuda_stream), ctypes.byref(h))
        self.h = h

    def run(self, first_picks, n_iter, tv_const, n_sub_init, n_sub_final, p_val, use_graph=True,
            count=None, objective=False):
        """Run iterations; first_picks holds one first subset per iteration of this
        call.  objective: also compute the FP64 data-fidelity objective
        sum(pre e^-l + post l) of mu after each iteration (see stats())."""
        fp = np.ascontiguousarray(np.asarray(first_picks, dtype=np.int32).ravel())
        count = fp.size if count is None else int(count)
        p = Params(int(n_iter), float(tv_const), int(n_sub_init), int(n_sub_final), float(p_val),
                   1 if use_graph else 0, 1 if objective else 0)
        _lib.call("mexct_osctv_run", self.h, ctypes.byref(p), _ptr(fp), count,
                  _P(self.stream.cuda_stream))

    def mu(self):
        out = self._torch.empty((self.H, self.W, self.W), dtype=self._torch.float32, device="cuda")
        _lib.call("mexct_osctv_mu", self.h, _P(out.data_ptr()), _P(self.stream.cuda_stream))
        return out

    def stats(self):
        """(iterations run, last d_a, last objective or NaN when the last
        iteration did not compute it)."""
        it, da, ob = _i(), _d(), _d()
        _lib.call("mexct_osctv_stats", self.h, ctypes.byref(it), ctypes.byref(da), ctypes.byref(ob))
        return it.value, da.value, ob.value

    def snapshot(self):
        n = _lib.load().mexct_osctv_state_bytes(self.h)
        buf = np.zeros(n, dtype=np.uint8)
        _lib.call("mexct_osctv_snapshot", self.h, _ptr(buf), _P(self.stream.cuda_stream))
        return buf

    def restore(self, buf):
        buf = np.ascontiguousarray(buf, dtype=np.uint8)
        _lib.call("mexct_osctv_restore", self.h, _ptr(buf), _P(self.stream.cuda_stream))

    def close(self):
        if getattr(self, "h", None):
            _lib.load().mexct_osctv_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
