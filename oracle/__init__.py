"""FP64 CPU oracle for the mex-cuda-CT projection-operator path.

TEST INFRASTRUCTURE ONLY.  This package is the correctness checker and the
timed CPU baseline: it may be imported by ``tests/``, by
``__graft_entry__.smoke()`` and by the CPU-baseline / reference arm of
``bench.py``, and by nothing else.  The CUDA library under
``mex-cuda-ct_gb300/`` never imports, links or calls it.

The C++ restatement lives in ``oracle.cpp`` (every function cites the
reference file:line it follows); this module builds it with g++/OpenMP into
``oracle/_build/liboracle.so`` and wraps it with ctypes.  Arrays are numpy,
MATLAB column-major (``order='F'``) with the shapes of the MEX interface.

Parity pinning: the reference ships no tests, golden vectors or fixtures, and
its texture-reference CUDA kernels do not compile under CUDA 13, so the oracle
is pinned by the reference source and by the known-answer tests in
``tests/test_oracle_kat.py``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "liboracle.so")
_lock = threading.Lock()
_lib = None

FILTERS = {"none": 0, "ramp": 1, "shepp-logan": 2, "cosine": 3, "hamming": 4, "hann": 5}


def build(force: bool = False) -> str:
    """Compile oracle.cpp into oracle/_build/liboracle.so (g++, OpenMP)."""
    src = os.path.join(_HERE, "oracle.cpp")
    hdr = os.path.join(_HERE, "oracle.h")
    os.makedirs(_BUILD, exist_ok=True)
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return _LIB_PATH
    tmp = _LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", tmp, src]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def _load():
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        build()
        lib = ctypes.CDLL(_LIB_PATH)
        F = ctypes.POINTER(ctypes.c_float)
        D = ctypes.POINTER(ctypes.c_double)
        I32 = ctypes.POINTER(ctypes.c_int32)
        i, f, d = ctypes.c_int, ctypes.c_float, ctypes.c_double
        sig = {
            "orc_fp": [F, i, i, f, F, i, i, D],
            "orc_bp": [F, i, i, i, f, F, i, D],
            "orc_fp_det": [F, i, i, f, F, i, i, i, i, f, f, i, D],
            "orc_bp_det": [F, i, i, i, f, F, i, i, i, f, f, D],
            "orc_g3d_fp": [F, i, i, F, F, i, i, i, i, D],
            "orc_g3d_bp": [F, i, i, i, F, F, i, i, i, D],
            "orc_g3d_bp_matched": [F, i, i, i, F, F, i, i, i, D],
            "orc_osc_iter": [D, F, F, i, i, i, i, I32, F, f, i],
            "orc_osc_iter_det": [D, F, F, i, i, i, i, I32, F, f, i, i, i, f, f],
            "orc_tvmin3d": [D, i, i, i, d, i],
            "orc_osc_fp": [D, i, i, f, F, i, i, D],
            "orc_tv_gradient": [D, i, i, i, D],
            "orc_num_subsets": [i, i, d, i, i],
            "orc_subset_order": [i, i, I32],
            "orc_prefilter": [F, i, i, i, F, i, d, i, d, d, D],
            "orc_parker_window": [i, i, F, i, d, d, D],
            "orc_filter_response": [i, i, d, D, i],
            "orc_set_threads": [i],
            "orc_get_threads": [],
            "orc_set_tex_weights": [i],
            "orc_get_tex_weights": [],
            "orc_set_ref_steps": [i],
            "orc_get_ref_steps": [],
        }
        for name, args in sig.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = None if name in ("orc_set_threads", "orc_set_tex_weights",
                                          "orc_set_ref_steps") else ctypes.c_int
        cb = ctypes.CFUNCTYPE(None, ctypes.c_int, D, ctypes.c_void_p)
        lib.orc_osc_tv.argtypes = [F, F, i, i, i, F, f, i, i, d, i, i, d, I32, D, cb, ctypes.c_void_p]
        lib.orc_osc_tv.restype = ctypes.c_int
        lib._cbtype = cb
        _lib = lib
        return lib


def _f32(a, shape=None):
    a = np.asarray(a, dtype=np.float32)
    a = np.asfortranarray(a)
    if shape is not None and a.shape != tuple(shape):
        raise ValueError("expected shape %s, got %s" % (shape, a.shape))
    return a


def _p(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def _check(rc, what):
    if rc != 0:
        raise RuntimeError("oracle %s failed (rc=%d)" % (what, rc))


def set_threads(n: int) -> None:
    _load().orc_set_threads(int(n))


def get_threads() -> int:
    return int(_load().orc_get_threads())


TEX_EXACT, TEX8_NEAREST, TEX8_TRUNC, TEX_HW = 0, 1, 2, 3


def set_tex_weights(mode: int) -> None:
    """Texture-fetch weights of every oracle operator: TEX_EXACT (default),
    TEX8_NEAREST or TEX8_TRUNC (each weight in 1/256 fixed point), or TEX_HW
    (the GPU texture unit's own weight rule, measured on a GB300)."""
    _load().orc_set_tex_weights(int(mode))


def get_tex_weights() -> int:
    return int(_load().orc_get_tex_weights())


class tex_weights:
    """Context manager: run oracle calls with the given texture-weight mode."""

    def __init__(self, mode: int):
        self.mode = mode

    def __enter__(self):
        self.prev = get_tex_weights()
        set_tex_weights(self.mode)
        return self

    def __exit__(self, *exc):
        set_tex_weights(self.prev)
        return False


def set_ref_steps(mode: int) -> None:
    """Sample positions of every FP / BP / OSC operator: 0 = FP64 p0 + k*d
    (default), 1 = the reference's binary32 incremental stepping
    (``currentpoint += stepsize``, ``proj_z += U``).  Sums stay FP64."""
    _load().orc_set_ref_steps(int(mode))


def get_ref_steps() -> int:
    return int(_load().orc_get_ref_steps())


class ref_steps:
    """Context manager: run oracle calls with the given stepping mode."""

    def __init__(self, mode: int = 1):
        self.mode = mode

    def __enter__(self):
        self.prev = get_ref_steps()
        set_ref_steps(self.mode)
        return self

    def __exit__(self, *exc):
        set_ref_steps(self.prev)
        return False


def fp(vol, sad, angles, n_proj, geom):
    """Forward projection, CUDAmex_FP semantics: vol [W,W,H] -> [W,H,nP] (float64)."""
    lib = _load()
    vol = _f32(vol)
    W, _, H = vol.shape
    ang = np.ascontiguousarray(np.asarray(angles, dtype=np.float32).ravel())
    out = np.zeros((W, H, int(n_proj)), dtype=np.float64, order="F")
    _check(lib.orc_fp(_p(vol, ctypes.c_float), W, H, float(sad), _p(ang, ctypes.c_float),
                      int(n_proj), int(geom), _p(out, ctypes.c_double)), "fp")
    return out


def bp(sino, sad, angles, geom):
    """Backprojection, CUDAmex_BP semantics: sino [W,H,nP] -> vol [W,W,H] (float64)."""
    lib = _load()
    sino = _f32(sino)
    if sino.ndim == 2:
        sino = sino[:, :, None]
    W, H, nP = sino.shape
    ang = np.ascontiguousarray(np.asarray(angles, dtype=np.float32).ravel())
    out = np.zeros((W, W, H), dtype=np.float64, order="F")
    _check(lib.orc_bp(_p(sino, ctypes.c_float), W, H, nP, float(sad), _p(ang, ctypes.c_float),
                      int(geom), _p(out, ctypes.c_double)), "bp")
    return out


def fp_det(vol, sad, angles, geom, det_w, det_h, du=1.0, dv=1.0, ss=1):
    """FP onto a Wd x Hd detector of pitch du, dv with ss x ss rays per pixel:
    vol [W,W,H] -> [Wd,Hd,nP] (float64)."""
    lib = _load()
    vol = _f32(vol)
    W, _, H = vol.shape
    ang = np.ascontiguousarray(np.asarray(angles, dtype=np.float32).ravel())
    out = np.zeros((int(det_w), int(det_h), ang.size), dtype=np.float64, order="F")
    _check(lib.orc_fp_det(_p(vol, ctypes.c_float), W, H, float(sad), _p(ang, ctypes.c_float),
                          ang.size, int(geom), int(det_w), int(det_h), float(du), float(dv),
                          int(ss), _p(out, ctypes.c_double)), "fp_det")
    return out


def bp_det(sino, sad, angles, geom, W, H, du=1.0, dv=1.0):
    """BP of a Wd x Hd x nP sinogram of pitch du, dv into a W x W x H volume."""
    lib = _load()
    sino = _f32(sino)
    Wd, Hd, nP = sino.shape
    ang = np.ascontiguousarray(np.asarray(angles, dtype=np.float32).ravel())
    out = np.zeros((int(W), int(W), int(H)), dtype=np.float64, order="F")
    _check(lib.orc_bp_det(_p(sino, ctypes.c_float), Wd, Hd, nP, float(sad),
                          _p(ang, ctypes.c_float), int(geom), int(W), int(H), float(du),
                          float(dv), _p(out, ctypes.c_double)), "bp_det")
    return out


def g3d_fp(vol, angles, pts, n_proj):
    """general3D FP: vol [S,S,Z], pts [W,H,6] or [W,H,6,nP] -> [W,H,nP] (float64)."""
    lib = _load()
    vol = _f32(vol)
    S, _, Z = vol.shape
    pts = _f32(pts)
    W, H = pts.shape[0], pts.shape[1]
    per_view = 1 if pts.ndim == 4 else 0
    ang = np.ascontiguousarray(np.asarray(angles, dtype=np.float32).ravel())
    out = np.zeros((W, H, int(n_proj)), dtype=np.float64, order="F")
    _check(lib.orc_g3d_fp(_p(vol, ctypes.c_float), S, Z, _p(ang, ctypes.c_float),
                          _p(pts, ctypes.c_float), W, H, int(n_proj), per_view,
                          _p(out, ctypes.c_double)), "g3d_fp")
    return out


def g3d_bp(sino, angles, pts, S, Z):
    """general3D BP: sino [W,H,nP], pts [W,H,6] or [W,H,6,nP] -> vol [S,S,Z] (float64)."""
    lib = _load()
    sino = _f32(sino)
    if sino.ndim == 2:
        sino = sino[:, :, None]
    W, H, nP = sino.shape
    pts = _f32(pts)
    per_view = 1 if pts.ndim == 4 else 0
    ang = np.ascontiguousarray(np.asarray(angles, dtype=np.float32).ravel())
    out = np.zeros((int(S), int(S), int(Z)), dtype=np.float64, order="F")
    _check(lib.orc_g3d_bp(_p(sino, ctypes.c_float), W, H, nP, _p(ang, ctypes.c_float),
                          _p(pts, ctypes.c_float), per_view, int(S), int(Z),
                          _p(out, ctypes.c_double)), "g3d_bp")
    return out


def g3d_bp_matched(sino, angles, pts, S, Z):
    """The exact transpose of g3d_fp (eight-corner trilinear scatter at the FP's
    sample positions): sino [W,H,nP] -> vol [S,S,Z] (float64)."""
    lib = _load()
    sino = _f32(sino)
    if sino.ndim == 2:
        sino = sino[:, :, None]
    W, H, nP = sino.shape
    pts = _f32(pts)
    per_view = 1 if pts.ndim == 4 else 0
    ang = np.ascontiguousarray(np.asarray(angles, dtype=np.float32).ravel())
    out = np.zeros((int(S), int(S), int(Z)), dtype=np.float64, order="F")
    _check(lib.orc_g3d_bp_matched(_p(sino, ctypes.c_float), W, H, nP, _p(ang, ctypes.c_float),
                                  _p(pts, ctypes.c_float), per_view, int(S), int(Z),
                                  _p(out, ctypes.c_double)), "g3d_bp_matched")
    return out


def osc_iter(mu, pre, post, n_sub, picks, angles, sad, geom):
    """One OSC iteration; returns the updated mu (float64).  Inputs are not modified."""
    lib = _load()
    mu = np.array(mu, dtype=np.float64, order="F", copy=True)
    pre = _f32(pre)
    post = _f32(post)
    W, _, H = mu.shape
    nP = pre.shape[2] if pre.ndim == 3 else 1
    picks = np.ascontiguousarray(np.asarray(picks, dtype=np.int32).ravel())
    ang = np.ascontiguousarray(np.asarray(angles, dtype=np.float32).ravel())
    _check(lib.orc_osc_iter(_p(mu, ctypes.c_double), _p(pre, ctypes.c_float),
                            _p(post, ctypes.c_float), W, H, nP, int(n_sub),
                            _p(picks, ctypes.c_int32), _p(ang, ctypes.c_float), float(sad),
                            int(geom)), "osc_iter")
    return mu


def osc_iter_det(mu, pre, post, n_sub, picks, angles, sad, geom, du, dv):
    """One OSC iteration onto a decoupled detector: pre/post [Wd,Hd,nP] counts of
    pitch du x dv; returns the updated mu [W,W,H] (float64)."""
    lib = _load()
    mu = np.array(mu, dtype=np.float64, order="F", copy=True)
    pre = _f32(pre)
    post = _f32(post)
    W, _, H = mu.shape
    Wd, Hd, nP = pre.shape
    picks = np.ascontiguousarray(np.asarray(picks, dtype=np.int32).ravel())
    ang = np.ascontiguousarray(np.asarray(angles, dtype=np.float32).ravel())
    _check(lib.orc_osc_iter_det(_p(mu, ctypes.c_double), _p(pre, ctypes.c_float),
                                _p(post, ctypes.c_float), W, H, nP, int(n_sub),
                                _p(picks, ctypes.c_int32), _p(ang, ctypes.c_float), float(sad),
                                int(geom), Wd, Hd, float(du), float(dv)), "osc_iter_det")
    return mu


def tv_gradient(vol):
    lib = _load()
    v = np.array(vol, dtype=np.float64, order="F", copy=True)
    g = np.zeros_like(v, order="F")
    Nx, Ny, Nz = v.shape
    _check(lib.orc_tv_gradient(_p(v, ctypes.c_double), Nx, Ny, Nz, _p(g, ctypes.c_double)),
           "tv_gradient")
    return g


def tvmin3d(vol, c, n_steps=20):
    """CUDAmex_TVmin_3D semantics in FP64: returns the descended volume."""
    lib = _load()
    v = np.array(vol, dtype=np.float64, order="F", copy=True)
    Nx, Ny, Nz = v.shape
    _check(lib.orc_tvmin3d(_p(v, ctypes.c_double), Nx, Ny, Nz, float(c), int(n_steps)),
           "tvmin3d")
    return v


def num_subsets(s_init, s_final, p_val, max_iters, k):
    return int(_load().orc_num_subsets(int(s_init), int(s_final), float(p_val), int(max_iters),
                                       int(k)))


def subset_order(n, first):
    out = np.zeros(int(n), dtype=np.int32)
    _check(_load().orc_subset_order(int(n), int(first), _p(out, ctypes.c_int32)), "subset_order")
    return out


def osc_tv(pre, post, angles, sad, geom, n_iter, tv_const, n_sub_init, n_sub_final, p_val,
           first_picks, callback=None):
    """OSC_TV_recon.m in FP64.  callback(k, mu_copy) after every iteration."""
    lib = _load()
    pre = _f32(pre)
    post = _f32(post)
    W, H, nP = pre.shape
    ang = np.ascontiguousarray(np.asarray(angles, dtype=np.float32).ravel())
    fp_ = np.ascontiguousarray(np.asarray(first_picks, dtype=np.int32).ravel())
    if fp_.size < n_iter:
        raise ValueError("first_picks needs one entry per iteration")
    mu = np.zeros((W, W, H), dtype=np.float64, order="F")

    def _cb(k, ptr, _user):
        if callback is not None:
            arr = np.ctypeslib.as_array(ptr, shape=(W * W * H,)).copy()
            callback(int(k), arr.reshape((W, W, H), order="F"))

    cb = lib._cbtype(_cb)
    _check(lib.orc_osc_tv(_p(pre, ctypes.c_float), _p(post, ctypes.c_float), W, H, nP,
                          _p(ang, ctypes.c_float), float(sad), int(geom), int(n_iter),
                          float(tv_const), int(n_sub_init), int(n_sub_final), float(p_val),
                          _p(fp_, ctypes.c_int32), _p(mu, ctypes.c_double), cb, None), "osc_tv")
    return mu


def osc_fp(mu, sad, angles, geom):
    """The OSC forward pass (step 0.5, border addressing, CUDAmex_oscIter.cu:
    140-259) of mu [W,W,H] -> [W,H,nP] (float64)."""
    mu = np.asfortranarray(np.asarray(mu, dtype=np.float64))
    W, H = mu.shape[0], mu.shape[2]
    ang = np.ascontiguousarray(np.asarray(angles, dtype=np.float32).ravel())
    out = np.zeros((W, H, ang.size), dtype=np.float64, order="F")
    _check(_load().orc_osc_fp(_p(mu, ctypes.c_double), W, H, float(sad), _p(ang, ctypes.c_float),
                              ang.size, int(geom), _p(out, ctypes.c_double)), "osc_fp")
    return out


def filter_response(W, filt="ramp", cutoff=1.0):
    lib = _load()
    buf = np.zeros(1 << 16, dtype=np.float64)
    order = lib.orc_filter_response(int(W), FILTERS[filt.lower()], float(cutoff),
                                    _p(buf, ctypes.c_double), buf.size)
    if order <= 0:
        raise RuntimeError("filter_response failed")
    return buf[:order].copy()


def parker_window(W, angles, geom, q, sad=1000.0):
    """parker_weight.m's window per view and row element in FP64 -> [nP, W] float64."""
    lib = _load()
    ang = np.ascontiguousarray(np.asarray(angles, dtype=np.float32).ravel())
    out = np.zeros((ang.size, W), dtype=np.float64)
    rc = lib.orc_parker_window(int(W), ang.size, _p(ang, ctypes.c_float), int(geom), float(sad),
                               float(q), _p(out, ctypes.c_double))
    _check(rc, "parker_window")
    return out


def prefilter(sino, geom, angles, filt, cutoff, q, sad=1000.0):
    """preFilterSinogram.m (+ parker_weight.m) in FP64 -> [W,H,nP] float64."""
    lib = _load()
    sino = _f32(sino)
    W, H, nP = sino.shape
    ang = np.ascontiguousarray(np.asarray(angles, dtype=np.float32).ravel())
    out = np.zeros((W, H, nP), dtype=np.float64, order="F")
    rc = lib.orc_prefilter(_p(sino, ctypes.c_float), W, H, nP, _p(ang, ctypes.c_float),
                           int(geom), float(sad), FILTERS[filt.lower()], float(cutoff), float(q),
                           _p(out, ctypes.c_double))
    _check(rc, "prefilter")
    return out
