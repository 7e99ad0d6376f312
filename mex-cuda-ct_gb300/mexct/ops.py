"""MATLAB-interface mirror of the mex-cuda-CT operators over libmexct's C ABI.

Host functions keep the reference's names, argument order and array layouts:
numpy arrays in MATLAB shape and column-major order (``order='F'``), float32
("single") data, float32 angles.  Each call goes through the host entry point of
the C ABI (copy in, GPU compute, copy out), exactly like the MEX gateways
(parker_weight computes on the host):

=========================  ==============================================  =====================
function                    reference                                       C ABI
=========================  ==============================================  =====================
CUDAmex_FP                  projection_kernels/CUDAmex_FP.cu:350            mexct_fp
CUDAmex_BP                  projection_kernels/CUDAmex_BP.cu:223            mexct_bp
CUDAmex_general3D_FP        projection_kernels/CUDAmex_general3D_FP.cu:154  mexct_g3d_fp
CUDAmex_general3D_BP        projection_kernels/CUDAmex_general3D_BP.cu:194  mexct_g3d_bp
CUDAmex_oscIter             iterative_reconstruction/CUDAmex_oscIter.cu:362 mexct_osc_iter
CUDAmex_TVmin_3D            iterative_reconstruction/CUDAmex_TVmin_3D.cu:162 mexct_tvmin3d
preFilterSinogram           fbp_reconstruction/preFilterSinogram.m:1        mexct_prefilter
parker_weight               fbp_reconstruction/parker_weight.m:1            mexct_parker_weight
FBP_recon                   fbp_reconstruction/FBP_recon.m:1                mexct_fbp
=========================  ==============================================  =====================

Device functions (``*_dev``) take torch CUDA tensors: a volume is a C-contiguous
tensor of shape (H, W, W) = (z, y, x) and a sinogram (nP, H, W) = (view, v, u), which
is the same memory as the MATLAB arrays above.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

GEOM_NAMES = {"par3d": 0, "fan3d": 1, "cone3d": 2, "cone": 2}
FILTERS = {"none": 0, "ramp": 1, "shepp-logan": 2, "cosine": 3, "hamming": 4, "hann": 5}


def _f32F(a, name):
    a = np.asarray(a)
    if a.dtype != np.float32:
        raise TypeError("%s must be single (float32), got %s" % (name, a.dtype))
    return np.asfortranarray(a)


def _angles(angles, n_needed, name="angles"):
    a = np.asarray(angles)
    if a.dtype != np.float32:
        # The reference reads angles through a float* (CUDAmex_FP.cu:359): a
        # non-single array is misread there; here it is rejected.
        raise TypeError("%s must be single (float32), got %s" % (name, a.dtype))
    a = np.ascontiguousarray(a.ravel())
    if a.size < n_needed:
        raise ValueError("%s has %d entries, %d views requested" % (name, a.size, n_needed))
    return a


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def _scalar(x, name):
    v = np.asarray(x).ravel()
    if v.size != 1:
        raise ValueError("%s must be a scalar" % name)
    return float(v[0])


def _geom_flag(g):
    g = int(g)
    if g not in (0, 1, 2):
        raise ValueError("invalid geometry %r (0 = parallel, 1 = fan, 2 = cone)" % g)
    return g


def CUDAmex_FP(vol, SAD, angles, nProj, geomFlag=0):
    """fp = CUDAmex_FP(vol, SAD, angles, nProj, geomFlag) -> float32 [W, H, nProj].

    geomFlag defaults to 0 when omitted (the reference reads an undefined prhs[4]
    for a 4-argument call, as examples/general3D_projection_test.m:36 makes)."""
    vol = _f32F(vol, "vol")
    if vol.ndim == 2:
        vol = vol[:, :, None]
    if vol.ndim != 3 or vol.shape[0] != vol.shape[1]:
        raise ValueError("vol must be [W, W, H], got %s" % (vol.shape,))
    W, _, H = vol.shape
    nP = int(_scalar(nProj, "nProj"))
    if nP < 0:
        raise ValueError("nProj must be >= 0")
    ang = _angles(angles, nP)
    out = np.empty((W, H, nP), dtype=np.float32, order="F")
    _lib.call("mexct_fp", None, _ptr(vol), W, H, _scalar(SAD, "SAD"), _ptr(ang), nP,
              _geom_flag(geomFlag), _ptr(out))
    return out


def CUDAmex_BP(sino, SAD, angles, geomFlag):
    """bp = CUDAmex_BP(sino, SAD, angles, geomFlag) -> float32 [W, W, H]."""
    sino = _f32F(sino, "projections")
    if sino.ndim == 2:
        sino = sino[:, :, None]
    W, H, nP = sino.shape
    ang = _angles(angles, nP)
    out = np.empty((W, W, H), dtype=np.float32, order="F")
    _lib.call("mexct_bp", None, _ptr(sino), W, H, nP, _scalar(SAD, "SAD"), _ptr(ang),
              _geom_flag(geomFlag), _ptr(out))
    return out


def _pts(pts):
    pts = _f32F(pts, "pts")
    if pts.ndim == 3 and pts.shape[2] == 6:
        return pts, 0
    if pts.ndim == 4 and pts.shape[2] == 6:
        return pts, 1
    raise ValueError("pts must be [W, H, 6] (or [W, H, 6, nProj]), got %s" % (pts.shape,))


def CUDAmex_general3D_FP(vol, angles, pts, nProj):
    """fp = CUDAmex_general3D_FP(vol, angles, pts, nProj) -> float32 [W, H, nProj]."""
    vol = _f32F(vol, "vol")
    if vol.ndim == 2:
        vol = vol[:, :, None]
    S, _, Z = vol.shape
    pts, per_view = _pts(pts)
    W, H = pts.shape[0], pts.shape[1]
    nP = int(_scalar(nProj, "nProj"))
    if per_view and pts.shape[3] < nP:
        raise ValueError("per-view pts has %d views, %d requested" % (pts.shape[3], nP))
    ang = _angles(angles, nP)
    out = np.empty((W, H, nP), dtype=np.float32, order="F")
    _lib.call("mexct_g3d_fp", None, _ptr(vol), S, Z, _ptr(ang), _ptr(pts), W, H, nP, per_view,
              _ptr(out))
    return out


def CUDAmex_general3D_BP(sino, angles, pts, M, N):
    """bp = CUDAmex_general3D_BP(sino, angles, pts, M, N) -> float32 [M, M, N]."""
    sino = _f32F(sino, "projections")
    if sino.ndim == 2:
        sino = sino[:, :, None]
    W, H, nP = sino.shape
    pts, per_view = _pts(pts)
    if pts.shape[:2] != (W, H):
        raise ValueError("pts is %s, projections are %s" % (pts.shape[:2], (W, H)))
    ang = _angles(angles, nP)
    S, Z = int(_scalar(M, "M")), int(_scalar(N, "N"))
    out = np.empty((S, S, Z), dtype=np.float32, order="F")
    _lib.call("mexct_g3d_bp", None, _ptr(sino), W, H, nP, _ptr(ang), _ptr(pts), per_view, S, Z,
              _ptr(out))
    return out


def general3D_BP_matched(sino, angles, pts, M, N):
    """The transpose of CUDAmex_general3D_FP (no counterpart in the reference):
    eight-corner trilinear scatter at the FP's own sample positions, so that
    <FP(x), y> = <x, BP(y)> up to FP32 rounding.  Same arguments as
    CUDAmex_general3D_BP -> float32 [M, M, N]."""
    sino = _f32F(sino, "projections")
    if sino.ndim == 2:
        sino = sino[:, :, None]
    W, H, nP = sino.shape
    pts, per_view = _pts(pts)
    if pts.shape[:2] != (W, H):
        raise ValueError("pts is %s, projections are %s" % (pts.shape[:2], (W, H)))
    ang = _angles(angles, nP)
    S, Z = int(_scalar(M, "M")), int(_scalar(N, "N"))
    out = np.empty((S, S, Z), dtype=np.float32, order="F")
    _lib.call("mexct_g3d_bp_matched", None, _ptr(sino), W, H, nP, _ptr(ang), _ptr(pts), per_view,
              S, Z, _ptr(out))
    return out


def CUDAmex_oscIter(mu, pre, post, numSubsets, subsetPicks, angles, SAD, geomFlag):
    """CUDAmex_oscIter(mu, pre, post, nSub, subsetPicks, angles, SAD, geomFlag).

    Updates ``mu`` (float32, Fortran-ordered, writable) in place like the MEX does.
    pre/post are left unchanged (the reference overwrites them)."""
    if not (isinstance(mu, np.ndarray) and mu.dtype == np.float32 and mu.flags.f_contiguous
            and mu.flags.writeable):
        raise TypeError("mu must be a writable Fortran-ordered float32 array (updated in place)")
    pre = _f32F(pre, "pre")
    post = _f32F(post, "post")
    if pre.ndim == 2:
        pre, post = pre[:, :, None], post[:, :, None]
    W, _, H = mu.shape
    if pre.shape != post.shape or pre.shape[:2] != (W, H):
        raise ValueError("pre/post must be [W, H, nP] matching mu [W, W, H]")
    nP = pre.shape[2]
    nSub = int(_scalar(numSubsets, "numSubsets"))
    picks = np.asarray(subsetPicks)
    if picks.dtype != np.int32:
        raise TypeError("subsetPicks must be int32 (OSC_TV_recon.m:102)")
    picks = np.ascontiguousarray(picks.ravel())
    if picks.size < nSub:
        raise ValueError("subsetPicks has %d entries, numSubsets is %d" % (picks.size, nSub))
    ang = _angles(angles, nP)
    _lib.call("mexct_osc_iter", None, _ptr(mu), _ptr(pre), _ptr(post), W, H, nP, nSub,
              _ptr(picks), _ptr(ang), _scalar(SAD, "SAD"), _geom_flag(geomFlag))


def CUDAmex_TVmin_3D(vol, c, n_steps=20):
    """out = CUDAmex_TVmin_3D(vol, c): 20 TV-descent steps (hard-coded in the reference)."""
    vol = _f32F(vol, "image_in")
    if vol.ndim == 2:
        vol = vol[:, :, None]
    Nx, Ny, Nz = vol.shape
    out = np.empty_like(vol, order="F")
    _lib.call("mexct_tvmin3d", None, _ptr(vol), Nx, Ny, Nz, _scalar(c, "tvConst"), int(n_steps),
              _ptr(out))
    return out


def _geom_struct(geom):
    if isinstance(geom, dict):
        t = str(geom.get("type", "")).lower()
        sad = float(geom.get("SAD", 1000.0))
    else:
        t, sad = str(getattr(geom, "type")).lower(), float(getattr(geom, "SAD", 1000.0))
    if t not in GEOM_NAMES:
        raise ValueError("Invalid Geometry Selection: %r" % t)
    return GEOM_NAMES[t], sad


def preFilterSinogram(sino, geom, angles, filter="ramp", frequencyCutoff=1.0, parker_q=1.0):
    """filteredSinogram = preFilterSinogram(sino, geom, angles, filter, cutoff, q)."""
    sino = _f32F(sino, "sino")
    W, H, nP = sino.shape
    g, sad = _geom_struct(geom)
    ang = _angles(angles, nP)
    out = np.empty((W, H, nP), dtype=np.float32, order="F")
    _lib.call("mexct_prefilter", None, _ptr(sino), None, W, H, nP, _ptr(ang), g, sad,
              FILTERS[str(filter).lower()], float(frequencyCutoff), float(parker_q), _ptr(out))
    return out


def parker_weight(sino, angles, geom, q_value=1.0):
    """weightedSino = parker_weight(sino, angles, geom, q_value) on the host (float32)."""
    sino = _f32F(sino, "sino")
    if sino.ndim == 2:
        sino = sino[:, :, None]
    W, H, nP = sino.shape
    g, sad = _geom_struct(geom)
    ang = _angles(angles, nP)
    out = np.empty((W, H, nP), dtype=np.float32, order="F")
    _lib.call("mexct_parker_weight", _ptr(sino), W, H, nP, _ptr(ang), g, float(sad),
              float(q_value), _ptr(out))
    return out


def FBP_recon(pre, post, scanAngles, geom, filter="ramp", filterCutoff=1.0, parker_q=1.0):
    """recon = FBP_recon(pre, post, angles, geom, filter, cutoff, q) on the device."""
    pre = _f32F(pre, "pre")
    post = _f32F(post, "post")
    W, H, nP = post.shape
    g, sad = _geom_struct(geom)
    ang = _angles(scanAngles, nP)
    out = np.empty((W, W, H), dtype=np.float32, order="F")
    _lib.call("mexct_fbp", None, _ptr(pre), _ptr(post), W, H, nP, _ptr(ang), g, sad,
              FILTERS[str(filter).lower()], float(filterCutoff), float(parker_q), _ptr(out))
    return out


# ---------------------------------------------------------------------------
# Device (torch) twins.
# ---------------------------------------------------------------------------
_TYPES = {}


def _dtype_code(t):
    import torch
    if not _TYPES:
        _TYPES.update({torch.float32: _lib.F32, torch.float16: _lib.F16, torch.bfloat16: _lib.BF16})
    return _TYPES[t.dtype]


def _stream(stream):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _dptr(t):
    if not t.is_cuda or not t.is_contiguous():
        raise ValueError("expected a contiguous CUDA tensor")
    return ctypes.c_void_p(t.data_ptr())


def fp_dev(vol, sad, angles, geom, out=None, out_dtype=None, variant=_lib.FP_AUTO, stream=None):
    """FP of a device volume (H, W, W) -> sinogram (nP, H, W), stream-ordered.  variant:
    FP_AUTO (the context's shape table, see mexct.tune), FP_EXPLICIT, FP_RAY or FP_TEXTURE."""
    import torch
    H, W, W2 = vol.shape
    assert W == W2, "volume must be (H, W, W)"
    ang = _angles(angles, 0)
    nP = ang.size
    if out is None:
        out = torch.empty((nP, H, W), dtype=out_dtype or vol.dtype, device=vol.device)
    _lib.call("mexct_fp_dev_ex", None, _dptr(vol), _dtype_code(vol), W, H, float(sad), _ptr(ang),
              nP, _geom_flag(geom), _dptr(out), _dtype_code(out), int(variant), _stream(stream))
    return out


def bp_dev(sino, sad, angles, geom, out=None, out_dtype=None, stream=None):
    """BP of a device sinogram (nP, H, W) -> volume (H, W, W), stream-ordered."""
    import torch
    nP, H, W = sino.shape
    ang = _angles(angles, nP)
    if out is None:
        out = torch.empty((H, W, W), dtype=out_dtype or torch.float32, device=sino.device)
    _lib.call("mexct_bp_dev_ex", None, _dptr(sino), _dtype_code(sino), W, H, nP, float(sad),
              _ptr(ang), _geom_flag(geom), _dptr(out), _dtype_code(out), _stream(stream))
    return out


def fp_det_dev(vol, sad, angles, geom, det_w, det_h, du=1.0, dv=1.0, ss=1, out=None,
               stream=None):
    """FP of an FP32 device volume (H, W, W) onto a det_w x det_h detector of pitch du x dv
    with ss x ss rays per pixel -> sinogram (nP, det_h, det_w), stream-ordered."""
    import torch
    H, W, W2 = vol.shape
    assert W == W2, "volume must be (H, W, W)"
    ang = _angles(angles, 0)
    nP = ang.size
    det = _lib.Detector(int(det_w), int(det_h), float(du), float(dv), int(ss))
    if out is None:
        out = torch.empty((nP, int(det_h), int(det_w)), dtype=torch.float32, device=vol.device)
    _lib.call("mexct_fp_det_dev", None, _dptr(vol), W, H, float(sad), _ptr(ang), nP,
              _geom_flag(geom), ctypes.addressof(det), _dptr(out), _stream(stream))
    return out


def bp_det_dev(sino, sad, angles, geom, W, H, du=1.0, dv=1.0, out=None, stream=None):
    """BP of an FP32 device sinogram (nP, det_h, det_w) of pitch du x dv -> volume (H, W, W)."""
    import torch
    nP, det_h, det_w = sino.shape
    ang = _angles(angles, nP)
    det = _lib.Detector(int(det_w), int(det_h), float(du), float(dv), 1)
    if out is None:
        out = torch.empty((int(H), int(W), int(W)), dtype=torch.float32, device=sino.device)
    _lib.call("mexct_bp_det_dev", None, _dptr(sino), ctypes.addressof(det), nP, float(sad),
              _ptr(ang), _geom_flag(geom), int(W), int(H), _dptr(out), _stream(stream))
    return out


def fp_det(vol, sad, angles, geom, det_w, det_h, du=1.0, dv=1.0, ss=1):
    """FP of a host volume [W, W, H] onto a det_w x det_h detector of pitch du x dv
    with ss x ss rays per pixel -> float32 sinogram [det_w, det_h, nP] (MATLAB layout)."""
    vol = _f32F(vol, "vol")
    if vol.ndim == 2:
        vol = vol[:, :, None]
    if vol.ndim != 3 or vol.shape[0] != vol.shape[1]:
        raise ValueError("vol must be [W, W, H], got %s" % (vol.shape,))
    W, _, H = vol.shape
    ang = _angles(angles, 0)
    nP = ang.size
    det = _lib.Detector(int(det_w), int(det_h), float(du), float(dv), int(ss))
    out = np.empty((int(det_w), int(det_h), nP), dtype=np.float32, order="F")
    _lib.call("mexct_fp_det", None, _ptr(vol), W, H, float(sad), _ptr(ang), nP, _geom_flag(geom),
              ctypes.addressof(det), _ptr(out))
    return out


def bp_det(sino, sad, angles, geom, W, H, du=1.0, dv=1.0):
    """BP of a host sinogram [det_w, det_h, nP] of pitch du x dv -> float32 volume
    [W, W, H] (MATLAB layout)."""
    sino = _f32F(sino, "projections")
    if sino.ndim == 2:
        sino = sino[:, :, None]
    if sino.ndim != 3:
        raise ValueError("projections must be [det_w, det_h, nP], got %s" % (sino.shape,))
    det_w, det_h, nP = sino.shape
    ang = _angles(angles, nP)
    det = _lib.Detector(int(det_w), int(det_h), float(du), float(dv), 1)
    out = np.empty((int(W), int(W), int(H)), dtype=np.float32, order="F")
    _lib.call("mexct_bp_det", None, _ptr(sino), ctypes.addressof(det), nP, float(sad), _ptr(ang),
              _geom_flag(geom), int(W), int(H), _ptr(out))
    return out


def sub_rows(W, H, sad, geom, z0, nz):
    """Detector rows (row0, nrows) that the BP of slab z0 .. z0 + nz - 1 reads."""
    r0, nr = ctypes.c_int(), ctypes.c_int()
    _lib.call("mexct_sub_rows", int(W), int(H), float(sad), _geom_flag(geom), int(z0), int(nz),
              ctypes.byref(r0), ctypes.byref(nr))
    return r0.value, nr.value


def fp_sub_dev(slab, H, z0, sad, angles, geom, out=None, accumulate=False, stream=None):
    """FP of a device slab (nz, W, W) = slices z0 .. z0 + nz - 1 of an H-slice volume into a
    sinogram (nP, H, W): stores, or adds to `out` with accumulate."""
    import torch
    nz, W, W2 = slab.shape
    assert W == W2, "slab must be (nz, W, W)"
    ang = _angles(angles, 0)
    nP = ang.size
    if out is None:
        out = torch.zeros((nP, int(H), W), dtype=torch.float32, device=slab.device)
    _lib.call("mexct_fp_sub_dev", None, _dptr(slab), W, int(H), int(z0), nz, float(sad), _ptr(ang),
              nP, _geom_flag(geom), _dptr(out), 1 if accumulate else 0, _stream(stream))
    return out


def bp_sub_dev(rows, row0, H, sad, angles, geom, z0, nz, out=None, accumulate=False,
               stream=None):
    """BP into slab z0 .. z0 + nz - 1 (nz, W, W) from detector rows row0 .. of every view
    (device array (nP, nrows, W))."""
    import torch
    nP, nrows, W = rows.shape
    ang = _angles(angles, nP)
    if out is None:
        out = torch.empty((int(nz), W, W), dtype=torch.float32, device=rows.device)
    _lib.call("mexct_bp_sub_dev", None, _dptr(rows), int(row0), nrows, W, int(H), nP, float(sad),
              _ptr(ang), _geom_flag(geom), int(z0), int(nz), _dptr(out),
              1 if accumulate else 0, _stream(stream))
    return out


def fp_ooc(vol, sad, angles, geom, budget_bytes):
    """CUDAmex_FP of a host volume [W, W, H] with at most budget_bytes of device memory."""
    vol = _f32F(vol, "vol")
    W, _, H = vol.shape
    ang = _angles(angles, 0)
    out = np.empty((W, H, ang.size), dtype=np.float32, order="F")
    _lib.call("mexct_fp_ooc", None, _ptr(vol), W, H, float(sad), _ptr(ang), ang.size,
              _geom_flag(geom), int(budget_bytes), _ptr(out))
    return out


def bp_ooc(sino, sad, angles, geom, budget_bytes):
    """CUDAmex_BP of a host sinogram [W, H, nP] with at most budget_bytes of device memory."""
    sino = _f32F(sino, "projections")
    W, H, nP = sino.shape
    ang = _angles(angles, nP)
    out = np.empty((W, W, H), dtype=np.float32, order="F")
    _lib.call("mexct_bp_ooc", None, _ptr(sino), W, H, nP, float(sad), _ptr(ang),
              _geom_flag(geom), int(budget_bytes), _ptr(out))
    return out


def g3d_fp_dev(vol, angles, pts, out=None, stream=None):
    """general3D FP: vol (Z, S, S); pts (6, H, W) or (nP, 6, H, W) -> (nP, H, W)."""
    import torch
    Z, S, _ = vol.shape
    ang = _angles(angles, 0)
    nP = ang.size
    per_view = 1 if pts.dim() == 4 else 0
    H, W = pts.shape[-2], pts.shape[-1]
    if out is None:
        out = torch.empty((nP, H, W), dtype=torch.float32, device=vol.device)
    _lib.call("mexct_g3d_fp_dev", None, _dptr(vol), S, Z, _ptr(ang), _dptr(pts), W, H, nP,
              per_view, _dptr(out), _stream(stream))
    return out


def g3d_bp_dev(sino, angles, pts, S, Z, out=None, stream=None):
    import torch
    nP, H, W = sino.shape
    ang = _angles(angles, nP)
    per_view = 1 if pts.dim() == 4 else 0
    if out is None:
        out = torch.empty((Z, S, S), dtype=torch.float32, device=sino.device)
    _lib.call("mexct_g3d_bp_dev", None, _dptr(sino), W, H, nP, _ptr(ang), _dptr(pts), per_view,
              int(S), int(Z), _dptr(out), _stream(stream))
    return out


def g3d_bp_matched_dev(sino, angles, pts, S, Z, out=None, stream=None):
    """Device form of general3D_BP_matched: sino (nP, H, W) -> (Z, S, S)."""
    import torch
    nP, H, W = sino.shape
    ang = _angles(angles, nP)
    per_view = 1 if pts.dim() == 4 else 0
    if out is None:
        out = torch.empty((Z, S, S), dtype=torch.float32, device=sino.device)
    _lib.call("mexct_g3d_bp_matched_dev", None, _dptr(sino), W, H, nP, _ptr(ang), _dptr(pts),
              per_view, int(S), int(Z), _dptr(out), _stream(stream))
    return out


def osc_iter_dev(mu, pre, post, n_sub, picks, angles, sad, geom, stream=None):
    """One OSC iteration on device tensors; mu (H, W, W) float32 is updated in place."""
    H, W, _ = mu.shape
    nP = pre.shape[0]
    picks = np.ascontiguousarray(np.asarray(picks, dtype=np.int32).ravel())
    ang = _angles(angles, nP)
    _lib.call("mexct_osc_iter_dev", None, _dptr(mu), _dptr(pre), _dptr(post), W, H, nP,
              int(n_sub), _ptr(picks), _ptr(ang), float(sad), _geom_flag(geom), _stream(stream))
    return mu


def osc_iter_det_dev(mu, pre, post, n_sub, picks, angles, sad, geom, du=1.0, dv=1.0, stream=None):
    """One OSC iteration onto a decoupled detector: mu (H, W, W) float32 updated in
    place; pre/post (nP, det_h, det_w) float32 counts of pitch du x dv."""
    H, W, _ = mu.shape
    nP, det_h, det_w = pre.shape
    picks = np.ascontiguousarray(np.asarray(picks, dtype=np.int32).ravel())
    ang = _angles(angles, nP)
    det = _lib.Detector(int(det_w), int(det_h), float(du), float(dv), 1)
    _lib.call("mexct_osc_iter_det_dev", None, _dptr(mu), _dptr(pre), _dptr(post),
              ctypes.addressof(det), W, H, nP, int(n_sub), _ptr(picks), _ptr(ang), float(sad),
              _geom_flag(geom), _stream(stream))
    return mu


def tvmin3d_dev(vol, c, n_steps=20, out=None, stream=None):
    import torch
    Nz, Ny, Nx = vol.shape
    if out is None:
        out = torch.empty_like(vol)
    _lib.call("mexct_tvmin3d_dev", None, _dptr(vol), Nx, Ny, Nz, float(c), int(n_steps),
              _dptr(out), _stream(stream))
    return out


def prefilter_dev(sino, angles, geom, sad, filt="ramp", cutoff=1.0, q=1.0, pre=None, out=None,
                  stream=None):
    import torch
    nP, H, W = sino.shape
    ang = _angles(angles, nP)
    if out is None:
        out = torch.empty_like(sino)
    _lib.call("mexct_prefilter_dev", None, _dptr(sino), None if pre is None else _dptr(pre), W, H,
              nP, _ptr(ang), _geom_flag(geom), float(sad), FILTERS[filt.lower()], float(cutoff),
              float(q), _dptr(out), _stream(stream))
    return out


# ---------------------------------------------------------------------------
# Bounded waits of the default context (include/mexct.h).
# ---------------------------------------------------------------------------
def fp_slab_occupancy() -> int:
    """Resident CTAs per SM of the cone FP32 slab kernel (occupancy calculator)."""
    n = ctypes.c_int()
    _lib.call("mexct_fp_slab_occupancy", ctypes.byref(n))
    return n.value


def set_wait_limit(us: int) -> None:
    """Limit of one bounded wait of the slab FP in microseconds (0: give up at once,
    < 0: the 2 s default)."""
    _lib.call("mexct_ctx_set_wait_limit", None, int(us))


def device_errors(clear: bool = False) -> int:
    """Flags of the default context's device error word (bit 0: a bounded wait gave up);
    call after the covered work has finished."""
    f = ctypes.c_uint(0)
    _lib.call("mexct_ctx_device_errors", None, ctypes.byref(f), 1 if clear else 0)
    return int(f.value)
