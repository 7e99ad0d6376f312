"""Decoupled detector (mexct_fp_det_dev / mexct_bp_det_dev and their host-array
forms mexct_fp_det / mexct_bp_det) against the oracle.

The reference's detector is the volume's face: W x H pixels of unit pitch and
one ray per pixel centre.  These entry points take any det_w x det_h detector
of pitch du x dv and (FP) ss x ss rays per pixel; the oracle's orc_fp_det /
orc_bp_det restate the same formulas in FP64 and reduce to orc_fp / orc_bp
at the defaults.  Bound: rel-L2 1e-5 as for the reference's own operators.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5
W, H, NP = 24, 16, 9

# (det_w, det_h, du, dv, ss): larger and smaller detectors, odd sizes,
# coarser and finer pitch, super-sampling
DETECTORS = [
    (48, 40, 1.0, 1.0, 1),
    (20, 12, 1.5, 1.25, 1),
    (33, 17, 0.75, 0.8, 1),
    (31, 21, 1.1, 0.9, 2),
    (24, 16, 1.0, 1.0, 3),
]


@pytest.fixture(scope="module")
def case(cuda):
    import torch
    from mexct import phantoms

    vol = phantoms.ellipsoids(W, count=4, seed=11, nz=H)
    vol[:, :, 0] += 0.5  # non-zero edge slices: rays beyond them must see nothing
    vol[:, :, -1] += 0.5
    ang = np.linspace(0, 2 * np.pi, NP, endpoint=False).astype(np.float32) + np.float32(0.1)
    d = torch.from_numpy(np.ascontiguousarray(vol.transpose(2, 1, 0))).cuda()
    return vol, ang, d


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, np.float32).transpose(2, 1, 0))).cuda()


def _host(t):
    import torch

    torch.cuda.synchronize()
    return t.cpu().numpy().transpose(2, 1, 0)


@pytest.mark.parametrize("geom", [0, 1, 2])
@pytest.mark.parametrize("det", DETECTORS, ids=lambda d: "%dx%d_%.2gx%.2g_ss%d" % d)
def test_fp_det_matches_oracle(case, orc, geom, det):
    from mexct import ops

    vol, ang, d = case
    Wd, Hd, du, dv, ss = det
    got = _host(ops.fp_det_dev(d, 1000.0, ang, geom, Wd, Hd, du, dv, ss))
    assert got.shape == (Wd, Hd, NP)
    ref = orc.fp_det(vol, 1000.0, ang, geom, Wd, Hd, du, dv, ss)
    e = rel_l2(got, ref)
    print("FP geom %d det %s: rel-L2 %.3g" % (geom, det, e))
    assert e <= TOL


@pytest.mark.parametrize("geom", [0, 1, 2])
@pytest.mark.parametrize("det", DETECTORS[:4], ids=lambda d: "%dx%d_%.2gx%.2g" % d[:4])
def test_bp_det_matches_oracle(case, orc, geom, det):
    from mexct import ops

    Wd, Hd, du, dv, _ = det
    rng = np.random.default_rng(Wd * 100 + Hd)
    sino = np.asfortranarray(rng.uniform(0, 1, (Wd, Hd, NP)).astype(np.float32))
    _, ang, _ = case
    got = _host(ops.bp_det_dev(_dev(sino), 1000.0, ang, geom, W, H, du, dv))
    ref = orc.bp_det(sino, 1000.0, ang, geom, W, H, du, dv)
    e = rel_l2(got, ref)
    print("BP geom %d det %s: rel-L2 %.3g" % (geom, det, e))
    assert e <= TOL


@pytest.mark.parametrize("geom", [0, 1, 2])
def test_default_detector_is_the_standard_operator(case, geom):
    """det_w = W, det_h = H, unit pitch, one ray: FP bit-identical to the slab
    FP of mexct_fp_dev_ex; BP within FP32 rounding of mexct_bp_dev (its par /
    fan columns read texel rows instead of interpolating with weight 0)."""
    import torch
    from mexct import _lib, ops

    _, ang, d = case
    fp = ops.fp_det_dev(d, 1000.0, ang, geom, W, H)
    fp_std = ops.fp_dev(d, 1000.0, ang, geom, variant=_lib.FP_EXPLICIT)
    torch.cuda.synchronize()
    assert torch.equal(fp, fp_std)
    bp = ops.bp_det_dev(fp, 1000.0, ang, geom, W, H)
    bp_std = ops.bp_dev(fp, 1000.0, ang, geom)
    torch.cuda.synchronize()
    e = (torch.linalg.vector_norm((bp - bp_std).double()) /
         torch.linalg.vector_norm(bp_std.double())).item()
    assert e <= 1e-6


@pytest.mark.parametrize("geom", [0, 2])
def test_host_array_forms_equal_the_device_forms(case, geom):
    """mexct_fp_det / mexct_bp_det take host arrays in the MATLAB layouts and
    return what the device entry points return, bit for bit (super-sampled FP
    onto a 31 x 21 detector of pitch 1.1 x 0.9, then its BP)."""
    from mexct import ops

    vol, ang, d = case
    Wd, Hd, du, dv, ss = DETECTORS[3]
    fh = ops.fp_det(vol, 1000.0, ang, geom, Wd, Hd, du, dv, ss)
    fd = _host(ops.fp_det_dev(d, 1000.0, ang, geom, Wd, Hd, du, dv, ss))
    assert fh.shape == (Wd, Hd, NP) and np.array_equal(fh, fd)
    bh = ops.bp_det(fh, 1000.0, ang, geom, W, H, du, dv)
    bd = _host(ops.bp_det_dev(_dev(fh), 1000.0, ang, geom, W, H, du, dv))
    assert bh.shape == (W, W, H) and np.array_equal(bh, bd)


def test_supersampled_fp_is_the_mean_of_shifted_detectors(case):
    """ss = 2 on a W x H detector of pitch 1 traces the rays of a 2W x 2H
    detector of pitch 1/2 (sub-ray offsets -1/4 and +1/4 pixel) and returns the
    mean of each 2 x 2 group of them."""
    import torch
    from mexct import ops

    vol, ang, d = case
    sub = _host(ops.fp_det_dev(d, 1000.0, ang, 0, 2 * W, 2 * H, 0.5, 0.5, 1))
    mean = 0.25 * (sub[0::2, 0::2] + sub[1::2, 0::2] + sub[0::2, 1::2] + sub[1::2, 1::2])
    ss2 = _host(ops.fp_det_dev(d, 1000.0, ang, 0, W, H, 1.0, 1.0, 2))
    assert rel_l2(ss2, mean) <= TOL
    assert np.all(np.isfinite(ss2))
    torch.cuda.synchronize()


def test_detector_missing_the_volume_projects_zero(case):
    """A detector far wider than the volume: the outer columns see no voxel."""
    from mexct import ops

    _, ang, d = case
    got = _host(ops.fp_det_dev(d, 1000.0, ang, 0, 256, H, 1.0, 1.0, 1))
    assert np.all(np.isfinite(got))
    assert np.count_nonzero(got[:64]) == 0 and np.count_nonzero(got[-64:]) == 0
    assert np.count_nonzero(got[112:144]) > 0


def test_no_views_and_bad_detectors(case):
    import torch
    from mexct import _lib, ops

    _, _, d = case
    out = ops.fp_det_dev(d, 1000.0, np.zeros(0, np.float32), 2, 40, 30)
    assert out.shape == (0, 30, 40)
    vol = torch.full((H, W, W), 3.0, device="cuda")
    ops.bp_det_dev(torch.zeros((0, 30, 40), device="cuda"), 1000.0, np.zeros(0, np.float32), 2,
                   W, H, out=vol)
    torch.cuda.synchronize()
    assert torch.count_nonzero(vol).item() == 0
    for bad in [dict(du=0.0), dict(dv=-1.0), dict(ss=0), dict(ss=9)]:
        with pytest.raises(_lib.MexctError):
            kw = dict(du=1.0, dv=1.0, ss=1)
            kw.update(bad)
            ops.fp_det_dev(d, 1000.0, np.zeros(3, np.float32), 0, 8, 8, **kw)


@pytest.mark.gpu
@pytest.mark.parametrize("geom", [0, 1, 2])
@pytest.mark.parametrize("det", [(48, 30, 0.75, 0.8), (30, 22, 1.25, 1.5), (40, 28, 1.0, 1.0)])
def test_osc_iteration_on_a_decoupled_detector_matches_oracle(cuda, orc, geom, det):
    """One OSC iteration with the detector decoupled from the volume (finer,
    coarser, and the volume's own detector) against the FP64 oracle: forward
    rays through the pixel centres, residuals sampled bilinearly in u and v by
    the dual BP.  The volume's own detector gives the standard OSC iteration."""
    import torch
    from mexct import ops, phantoms

    W, H, nP, nsub = 40, 28, 12, 3
    Wd, Hd, du, dv = det
    vol = phantoms.ellipsoids(W, count=4, seed=9, nz=H)
    ang = phantoms.angles_full(nP)
    fp = orc.fp_det(vol, 1000.0, ang, geom, Wd, Hd, du, dv, 1).astype(np.float32)
    pre, post = phantoms.poisson_counts(fp * 0.5, 1e5, seed=3)
    mu0 = np.full((W, W, H), 1e-3, dtype=np.float32, order="F")
    picks = [2, 0, 1]
    ref = orc.osc_iter_det(mu0, pre, post, nsub, picks, ang, 1000.0, geom, du, dv)
    dmu = torch.from_numpy(np.ascontiguousarray(mu0.transpose(2, 1, 0))).cuda()
    dpre = torch.from_numpy(np.ascontiguousarray(pre.transpose(2, 1, 0))).cuda()
    dpost = torch.from_numpy(np.ascontiguousarray(post.transpose(2, 1, 0))).cuda()
    ops.osc_iter_det_dev(dmu, dpre, dpost, nsub, picks, ang, 1000.0, geom, du, dv)
    got = dmu.cpu().numpy().transpose(2, 1, 0)
    assert rel_l2(got, ref) <= 2e-5
    if (Wd, Hd, du, dv) == (W, H, 1.0, 1.0):
        std = orc.osc_iter(mu0, pre, post, nsub, picks, ang, 1000.0, geom)
        assert rel_l2(ref, std) <= 1e-12
