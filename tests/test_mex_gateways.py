"""The MEX gateways (the reference's six plus CUDAmex_OSC_TV_recon, the OSC_TV_recon.m
driver in one call), compiled against the stub mex.h, called as MATLAB would.

CPU tests cover argument checking (count, class, shape) -- the reference checks
only nrhs < 2.  GPU tests check that each gateway returns exactly what the C ABI
host entry point returns and keeps the reference's in-place semantics.
"""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def gw(lib):
    import __graft_entry__ as ge

    ge._builder().build_mex_stub()
    from mexct import mexgw

    mexgw.load()
    return mexgw


F = np.float32


def test_unknown_gateway(gw):
    with pytest.raises(ValueError):
        gw.call("CUDAmex_nope", 1.0)


@pytest.mark.parametrize("name,args,ident", [
    ("CUDAmex_TVmin_3D", (np.zeros((4, 4, 4), F),), "mexct:nrhs"),
    ("CUDAmex_TVmin_3D", (np.zeros((4, 4, 4), F), 0.1, 3), "mexct:nrhs"),
    ("CUDAmex_TVmin_3D", (np.zeros((4, 4, 4)), 0.1), "mexct:class"),
    ("CUDAmex_FP", (np.zeros((4, 4, 4)), 1000.0, np.zeros(2, F), 2, 0), "mexct:class"),
    ("CUDAmex_FP", (np.zeros((4, 4, 4), F), 1000.0, np.zeros(2), 2, 0), "mexct:class"),
    ("CUDAmex_FP", (np.zeros((4, 5, 4), F), 1000.0, np.zeros(2, F), 2, 0), "mexct:dims"),
    ("CUDAmex_FP", (np.zeros((4, 4, 4), F), 1000.0, np.zeros(1, F), 2, 0), "mexct:invalidInput"),
    ("CUDAmex_FP", (np.zeros((4, 4, 4), F), 1000.0, np.zeros(2, F), 2, 9), "mexct:invalidInput"),
    ("CUDAmex_BP", (np.zeros((4, 4, 3), F), 1000.0, np.zeros(3, F)), "mexct:nrhs"),
    ("CUDAmex_general3D_FP", (np.zeros((4, 4, 4), F), np.zeros(2, F), np.zeros((2, 2, 5), F), 2),
     "mexct:dims"),
    ("CUDAmex_oscIter", (np.zeros((4, 4, 2), F), np.zeros((4, 2, 3), F), np.zeros((4, 2, 3), F), 1,
                         np.zeros(1), np.zeros(3, F), 1000.0, 0), "mexct:class"),
    ("CUDAmex_oscIter", (np.zeros((4, 4, 2), F), np.zeros((4, 2, 3), F), np.zeros((4, 2, 3), F), 0,
                         np.zeros(1, np.int32), np.zeros(3, F), 1000.0, 0), "mexct:invalidInput"),
])
def test_gateway_argument_checks(gw, name, args, ident):
    with pytest.raises(gw.MexError) as ei:
        gw.call(name, *args)
    assert ei.value.identifier == ident


def _osctv_args(W=8, H=4, nP=6, n_iter=2, picks=None, pre=None):
    cnt = np.full((W, H, nP), 1e4, F, order="F")
    ang = np.linspace(0, 2 * np.pi, nP, endpoint=False).astype(F)
    picks = np.zeros(n_iter, np.int32) if picks is None else picks
    return [cnt if pre is None else pre, cnt.copy(order="F"), ang, 1000.0, 2, n_iter, 0.2, 3, 2,
            1.0, picks]


@pytest.mark.parametrize("change,ident", [
    (lambda a: a[:10], "mexct:nrhs"),
    (lambda a: a + [1e9, 5], "mexct:nrhs"),
    (lambda a: [a[0].astype(np.float64)] + a[1:], "mexct:class"),
    (lambda a: a[:2] + [a[2].astype(np.float64)] + a[3:], "mexct:class"),
    (lambda a: a[:10] + [np.zeros(2)], "mexct:class"),
    (lambda a: [np.zeros((8, 5, 6), F)] + a[1:], "mexct:dims"),
    (lambda a: a[:2] + [a[2][:4]] + a[3:], "mexct:invalidInput"),
    (lambda a: a[:5] + [0] + a[6:], "mexct:invalidInput"),
    (lambda a: a[:10] + [np.zeros(1, np.int32)], "mexct:invalidInput"),
    (lambda a: a + [0.0], "mexct:invalidInput"),
    (lambda a: a[:4] + [7] + a[5:], "mexct:invalidInput"),
])
def test_osc_tv_recon_gateway_argument_checks(gw, change, ident):
    """CUDAmex_OSC_TV_recon: count, class and shape checks in the gateway; the
    geometry flag is checked by the library before any device work."""
    with pytest.raises(gw.MexError) as ei:
        gw.call("CUDAmex_OSC_TV_recon", *change(_osctv_args()))
    assert ei.value.identifier == ident


def test_osc_tv_recon_gateway_reaches_the_library_without_gpu(gw):
    """Valid arguments pass the gateway's and the library's checks and stop at
    the missing device (both forms)."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    for extra in ([], [float(1 << 30)]):
        with pytest.raises(gw.MexError) as ei:
            gw.call("CUDAmex_OSC_TV_recon", *(_osctv_args() + extra))
        assert ei.value.identifier == "mexct:cuda"


@pytest.mark.gpu
def test_gateways_match_c_abi(cuda, gw):
    import mexct
    from mexct import phantoms

    W, H, nP = 32, 24, 12
    vol = phantoms.ellipsoids(W, count=4, seed=3, nz=H)
    ang = phantoms.angles_full(nP)
    for geom in (0, 1, 2):
        a = gw.call("CUDAmex_FP", vol, 1000.0, ang, nP, geom)
        b = mexct.CUDAmex_FP(vol, 1000.0, ang, nP, geom)
        assert a.dtype == np.float32 and a.shape == (W, H, nP) and np.array_equal(a, b)
        c = gw.call("CUDAmex_BP", a, 1000.0, ang, geom)
        assert c.shape == (W, W, H) and np.array_equal(c, mexct.CUDAmex_BP(a, 1000.0, ang, geom))
    # 4-argument call defaults geomFlag to 0 (examples/general3D_projection_test.m:36).
    assert np.array_equal(gw.call("CUDAmex_FP", vol, 1000.0, ang, nP),
                          mexct.CUDAmex_FP(vol, 1000.0, ang, nP, 0))
    pts = phantoms.parallel_pts(W, H)
    g = gw.call("CUDAmex_general3D_FP", vol, ang, pts, nP)
    assert np.array_equal(g, mexct.CUDAmex_general3D_FP(vol, ang, pts, nP))
    gb = gw.call("CUDAmex_general3D_BP", g, ang, pts, W, H)
    assert gb.shape == (W, W, H)
    tv = gw.call("CUDAmex_TVmin_3D", vol, 0.01)
    assert np.array_equal(tv, mexct.CUDAmex_TVmin_3D(vol, 0.01))


@pytest.mark.gpu
def test_osc_gateway_updates_mu_in_place(cuda, gw):
    import mexct
    from mexct import phantoms

    W, H, nP = 24, 16, 12
    ang = phantoms.angles_full(nP)
    vol = phantoms.ellipsoids(W, count=3, seed=5, nz=H)
    fp = mexct.CUDAmex_FP(vol, 1000.0, ang, nP, 2)
    pre, post = phantoms.poisson_counts(fp, 1e5, seed=2)
    mu_a = np.full((W, W, H), 1e-10, F, order="F")
    mu_b = mu_a.copy(order="F")
    picks = np.array([2, 0, 1], np.int32)
    out = gw.call("CUDAmex_oscIter", mu_a, pre, post, 3, picks, ang, 1000.0, 2, nlhs=0,
                  inplace=(0,))
    assert out is None
    mexct.CUDAmex_oscIter(mu_b, pre, post, 3, picks, ang, 1000.0, 2)
    assert np.array_equal(mu_a, mu_b) and not np.all(mu_a == np.float32(1e-10))


@pytest.mark.gpu
def test_osc_tv_recon_gateway_matches_c_abi(cuda, gw):
    """The one-call OSC-TV gateway returns what the C ABI returns, in core and
    out of core (with the slab thickness as a second output); pre / post are
    left as given."""
    from mexct import phantoms, solver

    W, H, nP = 32, 16, 12
    ang = phantoms.angles_full(nP)
    vol = phantoms.ellipsoids(W, count=3, seed=8, nz=H)
    import oracle

    fp = oracle.fp(vol, 1000.0, ang, nP, 1).astype(np.float32)
    pre, post = phantoms.poisson_counts(fp, 1e5, seed=4)
    pre0, post0 = pre.copy(), post.copy()
    picks = np.array([1, 0, 2], np.int32)
    a = gw.call("CUDAmex_OSC_TV_recon", pre, post, ang, 1000.0, 1, 3, 0.2, 4, 2, 1.0, picks)
    b = solver.OSC_TV_recon(pre, post, ang, {"type": "fan3d", "SAD": 1000.0}, 3, 0.2, 4, 2, 1.0,
                            picks)
    assert a.dtype == np.float32 and a.shape == (W, W, H) and np.array_equal(a, b)
    assert np.array_equal(pre, pre0) and np.array_equal(post, post0)
    budget = float(1 << 34)
    c, planes = gw.call("CUDAmex_OSC_TV_recon", pre, post, ang, 1000.0, 1, 3, 0.2, 4, 2, 1.0,
                        picks, budget, nlhs=2)
    d, nz = solver.OSC_TV_recon_ooc(pre, post, ang, {"type": "fan3d", "SAD": 1000.0}, 3, 0.2, 4,
                                    2, 1.0, picks, int(budget))
    assert np.shape(planes) == (1, 1) and planes.item() == nz == H and np.array_equal(c, d)
