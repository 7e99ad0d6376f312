"""C ABI of libmexct (CPU only): the library loads, exports every symbol that
include/mexct.h declares, and validates arguments before touching a device."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))
           if f.endswith(".h")]


def declared_symbols():
    names = set()
    for h in HEADERS:
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names.update(re.findall(r"\b(mexct_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_header_declares_the_mex_operators():
    names = declared_symbols()
    for n in ("mexct_fp", "mexct_bp", "mexct_g3d_fp", "mexct_g3d_bp", "mexct_osc_iter",
              "mexct_tvmin3d", "mexct_prefilter", "mexct_fbp"):
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, "not exported: %s" % missing


def test_version_and_last_error(lib):
    from mexct import _lib

    assert b"sm_103a" in lib.mexct_version()
    assert isinstance(_lib.last_error(), str)


F = np.float32


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def test_fp_rejects_bad_geometry_before_any_device_work(lib):
    from mexct import _lib

    vol = np.zeros((8, 8, 4), F)
    out = np.zeros((8, 4, 2), F)
    ang = np.zeros(2, F)
    rc = lib.mexct_fp(None, _p(vol), 8, 4, 1000.0, _p(ang), 2, 7, _p(out))
    assert rc == _lib.ERR_ARG
    assert "invalid geometry 7" in _lib.last_error()


@pytest.mark.parametrize("W,H,nP", [(0, 4, 1), (8, -1, 1), (8, 4, -3)])
def test_fp_rejects_bad_dims(lib, W, H, nP):
    from mexct import _lib

    buf = np.zeros(64, F)
    rc = lib.mexct_fp(None, _p(buf), W, H, 1000.0, _p(buf), nP, 0, _p(buf))
    assert rc == _lib.ERR_ARG


def test_null_pointers_are_rejected(lib):
    from mexct import _lib

    buf = np.zeros(64, F)
    assert lib.mexct_bp(None, None, 4, 4, 1, 1000.0, _p(buf), 0, _p(buf)) == _lib.ERR_ARG
    assert lib.mexct_tvmin3d(None, _p(buf), 4, 4, 4, 0.1, 20, None) == _lib.ERR_ARG
    assert lib.mexct_g3d_fp(None, _p(buf), 4, 4, _p(buf), None, 2, 2, 1, 0, _p(buf)) == _lib.ERR_ARG


def test_osc_requires_positive_subsets(lib):
    from mexct import _lib

    buf = np.zeros(4096, F)
    picks = np.zeros(1, np.int32)
    rc = lib.mexct_osc_iter(None, _p(buf), _p(buf), _p(buf), 8, 4, 2, 0, _p(picks), _p(buf),
                            1000.0, 2)
    assert rc == _lib.ERR_ARG and "nSub" in _lib.last_error()


def test_prefilter_requires_square_detector(lib):
    """parker_weight.m:225 multiplies a W x H projection by an H x H window: the
    reference errors for W != H; the library reports MEXCT_ERR_UNSUPPORTED."""
    from mexct import _lib

    buf = np.zeros(4096, F)
    ang = np.linspace(0, 1, 4).astype(F)
    rc = lib.mexct_prefilter(None, _p(buf), None, 8, 6, 4, _p(ang), 2, 1000.0, 4, 1.0, 1.0, _p(buf))
    assert rc == _lib.ERR_UNSUPPORTED and "square" in _lib.last_error()
    rc = lib.mexct_prefilter(None, _p(buf), None, 8, 8, 1, _p(ang), 2, 1000.0, 4, 1.0, 1.0, _p(buf))
    assert rc == _lib.ERR_ARG


def test_valid_call_without_gpu_reports_cuda_error(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from mexct import _lib

    vol = np.zeros((8, 8, 4), F)
    out = np.zeros((8, 4, 2), F)
    ang = np.zeros(2, F)
    rc = lib.mexct_fp(None, _p(vol), 8, 4, 1000.0, _p(ang), 2, 0, _p(out))
    assert rc == _lib.ERR_CUDA
    assert "CUDA" in _lib.last_error()


def test_python_mirror_validates_types(lib):
    import mexct

    with pytest.raises(TypeError):
        mexct.CUDAmex_FP(np.zeros((4, 4, 4)), 1000, np.zeros(1, F), 1, 0)  # double volume
    with pytest.raises(TypeError):
        mexct.CUDAmex_FP(np.zeros((4, 4, 4), F), 1000, np.zeros(1), 1, 0)  # double angles
    with pytest.raises(ValueError):
        mexct.CUDAmex_FP(np.zeros((4, 4, 4), F), 1000, np.zeros(1, F), 3, 0)  # too few angles
    with pytest.raises(ValueError):
        mexct.CUDAmex_FP(np.zeros((4, 4, 4), F), 1000, np.zeros(1, F), 1, 5)  # bad geom
    mu = np.zeros((4, 4, 4), F)  # C-ordered: cannot be updated in place as MATLAB data
    with pytest.raises(TypeError):
        mexct.CUDAmex_oscIter(mu, np.zeros((4, 4, 2), F), np.zeros((4, 4, 2), F), 1,
                              np.zeros(1, np.int32), np.zeros(2, F), 1000, 0)


def test_detector_entry_points_validate_the_detector(lib):
    """mexct_fp_det_dev / mexct_bp_det_dev reject a NULL or malformed detector
    before any device work."""
    from mexct import _lib

    buf = np.zeros(64, F)
    ang = np.zeros(2, F)
    for det in [(0, 4, 1.0, 1.0, 1), (8, 4, 0.0, 1.0, 1), (8, 4, 1.0, float("nan"), 1),
                (8, 4, 1.0, 1.0, 0), (8, 4, 1.0, 1.0, 9)]:
        d = _lib.Detector(*det)
        rc = lib.mexct_fp_det_dev(None, _p(buf), 8, 4, 1000.0, _p(ang), 2, 0,
                                  ctypes.addressof(d), _p(buf), None)
        assert rc == _lib.ERR_ARG, det
    assert lib.mexct_fp_det_dev(None, _p(buf), 8, 4, 1000.0, _p(ang), 2, 0, None, _p(buf),
                                None) == _lib.ERR_ARG
    assert "NULL detector" in _lib.last_error()
    d = _lib.Detector(8, 4, 1.0, 1.0, 1)
    assert lib.mexct_bp_det_dev(None, _p(buf), ctypes.addressof(d), 2, 1000.0, _p(ang), 5, 8, 4,
                                _p(buf), None) == _lib.ERR_ARG
    assert "invalid geometry 5" in _lib.last_error()


def test_host_detector_entry_points_validate_before_device_work(lib):
    """The host-array forms mexct_fp_det / mexct_bp_det check the detector, the
    geometry and their pointers before any upload; with valid arguments and no
    GPU they stop at the missing device."""
    import torch
    from mexct import _lib

    buf = np.zeros(64, F)
    ang = np.zeros(2, F)
    for det in [(0, 4, 1.0, 1.0, 1), (8, 4, -1.0, 1.0, 1), (8, 4, 1.0, 1.0, 9)]:
        d = _lib.Detector(*det)
        assert lib.mexct_fp_det(None, _p(buf), 8, 4, 1000.0, _p(ang), 2, 0, ctypes.addressof(d),
                                _p(buf)) == _lib.ERR_ARG, det
    assert lib.mexct_fp_det(None, _p(buf), 8, 4, 1000.0, _p(ang), 2, 0, None,
                            _p(buf)) == _lib.ERR_ARG
    d = _lib.Detector(8, 4, 1.0, 1.0, 1)
    assert lib.mexct_fp_det(None, None, 8, 4, 1000.0, _p(ang), 2, 0, ctypes.addressof(d),
                            _p(buf)) == _lib.ERR_ARG
    assert lib.mexct_bp_det(None, _p(buf), ctypes.addressof(d), 2, 1000.0, _p(ang), 5, 8, 4,
                            _p(buf)) == _lib.ERR_ARG
    assert "invalid geometry 5" in _lib.last_error()
    assert lib.mexct_bp_det(None, _p(buf), ctypes.addressof(d), 2, 1000.0, _p(ang), 0, 8, 4,
                            None) == _lib.ERR_ARG
    if not torch.cuda.is_available():
        assert lib.mexct_fp_det(None, _p(buf), 8, 4, 1000.0, _p(ang), 2, 0, ctypes.addressof(d),
                                _p(buf)) == _lib.ERR_CUDA
        assert lib.mexct_bp_det(None, _p(buf), ctypes.addressof(d), 2, 1000.0, _p(ang), 0, 8, 4,
                                _p(buf)) == _lib.ERR_CUDA
