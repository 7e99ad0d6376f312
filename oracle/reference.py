"""The reference's own CUDA kernels, run on the GPU (oracle/ref_launch.cu).

TEST INFRASTRUCTURE ONLY.  This module may be used by ``tests/golden/make_ref_golden.py``
(which writes the reference-output fixtures), by ``tests/`` and by ``bench.py``'s
reference timing, and by nothing in the product.

The kernels come from ``oracle/_ref/*.cubin``, compiled unmodified from the
reference's .cu files by ``oracle/ref_build.py`` (device code, so the same cubins
load on any host).  The host-side steps of each MEX gateway are restated in
``ref_launch.cu``, which this module compiles into ``oracle/_ref/libreflaunch.so``
with nvcc on the machine that runs it.  Arrays follow the MEX interface: numpy,
MATLAB column-major (``order='F'``), float32.
"""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(_HERE, "_ref")
_SRC = os.path.join(_HERE, "ref_launch.cu")
_LIB = os.path.join(REF_DIR, "libreflaunch.so")
CUBINS = ["ref_fp.cubin", "ref_bp.cubin", "ref_g3d_fp.cubin", "ref_g3d_bp.cubin", "ref_osc.cubin",
          "ref_tv.cubin"]
_lock = threading.Lock()
_lib = None


def cubins_present() -> bool:
    return all(os.path.exists(os.path.join(REF_DIR, c)) for c in CUBINS)


def available() -> bool:
    """Whether the reference's kernels can run here: cubins built, launcher built,
    a CUDA driver and device present."""
    if not cubins_present():
        return False
    try:
        _load()
        return True
    except (OSError, RuntimeError):
        return False


def build_launcher(force: bool = False) -> str:
    """Compile ref_launch.cu into oracle/_ref/libreflaunch.so (nvcc, this host)."""
    os.makedirs(REF_DIR, exist_ok=True)
    if not force and os.path.exists(_LIB) and os.path.getmtime(_LIB) >= os.path.getmtime(_SRC):
        return _LIB
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    tmp = _LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc, "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC",
           "-gencode", "arch=compute_103a,code=sm_103a", "-o", tmp, _SRC, "-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference launcher build failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, _LIB)
    return _LIB


def _load():
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not cubins_present():
            raise RuntimeError("reference cubins missing from %s (built by oracle/ref_build.py "
                               "where the reference sources are present)" % REF_DIR)
        lib = ctypes.CDLL(build_launcher())
        F = ctypes.POINTER(ctypes.c_float)
        I32 = ctypes.POINTER(ctypes.c_int32)
        i, f = ctypes.c_int, ctypes.c_float
        sig = {
            "ref_init": [ctypes.c_char_p],
            "ref_fp": [F, i, i, f, F, i, i, F],
            "ref_bp": [F, i, i, i, f, F, i, F],
            "ref_g3d_fp": [F, i, i, F, F, i, i, i, F],
            "ref_g3d_bp": [F, i, i, i, F, F, i, i, F],
            "ref_osc_iter": [F, F, F, i, i, i, i, I32, F, f, i],
            "ref_tvmin3d": [F, i, i, i, f, F],
        }
        for name, args in sig.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        lib.ref_last_error.restype = ctypes.c_char_p
        lib.ref_last_ms.restype = ctypes.c_double
        if lib.ref_init(REF_DIR.encode()) != 0:
            raise RuntimeError("reference launcher: %s" % lib.ref_last_error().decode())
        _lib = lib
        return lib


def _check(rc, what):
    if rc != 0:
        raise RuntimeError("reference %s failed: %s" % (what, _load().ref_last_error().decode()))


def _f32(a):
    return np.asfortranarray(np.asarray(a, dtype=np.float32))


def _need(cond, what):
    if not cond:
        raise ValueError(what)


def _p(a, ct=ctypes.c_float):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def last_ms() -> float:
    """Host wall time of the last call (allocation, copies and kernels, as the
    gateway spends it)."""
    return float(_load().ref_last_ms())


def fp(vol, sad, angles, n_proj, geom):
    """CUDAmex_FP(vol, SAD, angles, nProj, geomFlag): [W,W,H] -> [W,H,nP] float32."""
    vol, ang = _f32(vol), _f32(angles).ravel()
    _need(vol.ndim == 3 and vol.shape[0] == vol.shape[1], "vol must be [W,W,H]")
    _need(len(ang) >= int(n_proj), "fewer angles than views")
    W, H = vol.shape[0], vol.shape[2]
    out = np.zeros((W, H, int(n_proj)), dtype=np.float32, order="F")
    _check(_load().ref_fp(_p(vol), W, H, float(sad), _p(ang), int(n_proj), int(geom), _p(out)), "fp")
    return out


def bp(sino, sad, angles, geom):
    """CUDAmex_BP(sino, SAD, angles, geomFlag): [W,H,nP] -> [W,W,H] float32."""
    sino, ang = _f32(sino), _f32(angles).ravel()
    _need(sino.ndim == 3, "sino must be [W,H,nP]")
    W, H, nP = sino.shape
    _need(len(ang) >= nP, "fewer angles than views")
    out = np.zeros((W, W, H), dtype=np.float32, order="F")
    _check(_load().ref_bp(_p(sino), W, H, nP, float(sad), _p(ang), int(geom), _p(out)), "bp")
    return out


def g3d_fp(vol, angles, pts, n_proj):
    """CUDAmex_general3D_FP(vol, angles, pts, nProj): pts [W,H,6] -> [W,H,nP]."""
    vol, ang, pts = _f32(vol), _f32(angles).ravel(), _f32(pts)
    _need(vol.ndim == 3 and vol.shape[0] == vol.shape[1], "vol must be [S,S,Z]")
    _need(pts.ndim == 3 and pts.shape[2] == 6, "pts must be [W,H,6]")
    _need(len(ang) >= int(n_proj), "fewer angles than views")
    S, Z = vol.shape[0], vol.shape[2]
    W, H = pts.shape[0], pts.shape[1]
    out = np.zeros((W, H, int(n_proj)), dtype=np.float32, order="F")
    _check(_load().ref_g3d_fp(_p(vol), S, Z, _p(ang), _p(pts), W, H, int(n_proj), _p(out)), "g3d_fp")
    return out


def g3d_bp(sino, angles, pts, S, Z):
    """CUDAmex_general3D_BP(sino, angles, pts, S, Z): [W,H,nP] -> [S,S,Z]."""
    sino, ang, pts = _f32(sino), _f32(angles).ravel(), _f32(pts)
    _need(sino.ndim == 3 and pts.ndim == 3 and pts.shape[2] == 6, "sino [W,H,nP], pts [W,H,6]")
    _need(pts.shape[:2] == sino.shape[:2], "pts and sino detector sizes differ")
    W, H, nP = sino.shape
    _need(len(ang) >= nP, "fewer angles than views")
    out = np.zeros((int(S), int(S), int(Z)), dtype=np.float32, order="F")
    _check(_load().ref_g3d_bp(_p(sino), W, H, nP, _p(ang), _p(pts), int(S), int(Z), _p(out)), "g3d_bp")
    return out


def osc_iter(mu, pre, post, n_sub, picks, angles, sad, geom):
    """CUDAmex_oscIter(mu, pre, post, nSub, subsetPicks, angles, SAD, geomFlag).

    Returns (mu, pre, post) after the call: new arrays, the inputs untouched (the
    gateway itself updates mu in place and overwrites pre/post with residuals)."""
    mu = np.array(mu, dtype=np.float32, order="F", copy=True)
    pre = np.array(pre, dtype=np.float32, order="F", copy=True)
    post = np.array(post, dtype=np.float32, order="F", copy=True)
    picks = np.ascontiguousarray(np.asarray(picks, dtype=np.int32).ravel())
    ang = _f32(angles).ravel()
    _need(mu.ndim == 3 and mu.shape[0] == mu.shape[1], "mu must be [W,W,H]")
    W, H = mu.shape[0], mu.shape[2]
    _need(pre.shape == post.shape and pre.ndim == 3 and pre.shape[:2] == (W, H), "pre/post must be [W,H,nP]")
    nP = pre.shape[2]
    _need(len(ang) >= nP and len(picks) >= int(n_sub), "angles / picks too short")
    _need(bool(np.all((picks >= 0) & (picks < max(int(n_sub), 1)))), "picks out of range")
    _check(_load().ref_osc_iter(_p(mu), _p(pre), _p(post), W, H, nP, int(n_sub), _p(picks, ctypes.c_int32),
                                _p(ang), float(sad), int(geom)), "osc_iter")
    return mu, pre, post


def tvmin3d(vol, c):
    """CUDAmex_TVmin_3D(vol, c): 20 TV descent steps, [Nx,Ny,Nz] float32."""
    vol = _f32(vol)
    _need(vol.ndim == 3, "vol must be 3-D")
    out = np.zeros(vol.shape, dtype=np.float32, order="F")
    nx, ny, nz = vol.shape
    _check(_load().ref_tvmin3d(_p(vol), nx, ny, nz, float(c), _p(out)), "tvmin3d")
    return out
