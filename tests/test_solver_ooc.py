"""OSC-TV out of core: mu in host memory, streamed through the device in z-slabs
(mexct_osc_tv_recon_ooc; the sub-volume reconstruction the reference lists as a
TODO at iterative_reconstruction/CUDAmex_oscIter.cu:28-29).

CPU: the slab planner (whole volume when it fits, else the thickest multiple of 4
slices within the budget; MEXCT_ERR_BUDGET below the smallest slab).
GPU: several slabs (and a ragged last slab) against the in-core solver and the
FP64 oracle driver; one slab against the in-core solver.  Per voxel the slab
sweeps run the in-core kernels' operations; the line integrals of a subset are
FP32 sums of the slabs' parts, so the iterates differ from the in-core ones by
rounding, which the TV step amplifies from iteration 2 on (as for the in-core
solver against the FP64 oracle).
"""
import numpy as np
import pytest

from conftest import rel_l2

SAD = 1000.0
GEOMS = ["par3d", "fan3d", "cone3d"]


def _budget_for(W, H, nP, geom, n_iter, s0, s1, p, planes):
    """Smallest budget whose slab is `planes` slices thick (bisection on the planner)."""
    from mexct import solver

    lo, hi = 1, 1 << 40
    while hi - lo > 1:
        mid = (lo + hi) // 2
        try:
            nz, _ = solver.ooc_plan(W, H, nP, geom, n_iter, s0, s1, p, mid)
        except RuntimeError:
            nz = 0
        if nz >= planes:
            hi = mid
        else:
            lo = mid
    nz, _ = solver.ooc_plan(W, H, nP, geom, n_iter, s0, s1, p, hi)
    assert nz == planes, (nz, planes)
    return hi


def test_planner(lib):
    from mexct import solver

    full, full_bytes = solver.ooc_plan(48, 40, 24, 2, 3, 6, 3, 1.0, 1 << 40)
    assert full == 40
    prev = 40
    for frac in (0.9, 0.8, 0.7, 0.64):
        nz, nbytes = solver.ooc_plan(48, 40, 24, 2, 3, 6, 3, 1.0, int(full_bytes * frac))
        assert nz % 4 == 0 and 4 <= nz <= prev and nbytes <= full_bytes * frac
        prev = nz
    with pytest.raises(RuntimeError, match="status 6"):
        solver.ooc_plan(48, 40, 24, 2, 3, 6, 3, 1.0, 100_000)
    with pytest.raises(RuntimeError, match="status 1"):
        solver.ooc_plan(48, 40, 24, 5, 3, 6, 3, 1.0, 1 << 30)


def _problem(W, H, nP, geom, seed=0):
    from mexct import phantoms

    import oracle

    vol = phantoms.ellipsoids(W, count=4, seed=seed, nz=H)
    ang = phantoms.angles_full(nP)
    fp = oracle.fp(vol, SAD, ang, nP, geom).astype(np.float32)
    pre, post = phantoms.poisson_counts(fp, 1e5, seed=seed + 1)
    return ang, pre, post


@pytest.mark.gpu
@pytest.mark.parametrize("geom,H", [(0, 40), (2, 42)])
def test_ooc_slabs_vs_in_core_and_fp64_oracle(cuda, orc, geom, H):
    """48 x 48 x H, 24 views, 8-slice slabs (H = 42: a ragged last slab of 2
    slices), 3 iterations of 6 -> 3 subsets with TV from iteration 2."""
    from mexct import solver

    W, nP, n_iter = 48, 24, 3
    kw = dict(n_iter=n_iter, s0=6, s1=3, p=1.0)
    ang, pre, post = _problem(W, H, nP, geom, seed=geom)
    picks = [1, 4, 0]
    g = {"type": GEOMS[geom], "SAD": SAD}
    budget = _budget_for(W, H, nP, geom, planes=8, **kw)
    # iteration 1 alone (OSC only; a one-iteration schedule has s1 subsets)
    one, nz = solver.OSC_TV_recon_ooc(pre, post, ang, g, 1, 0.2, 6, 3, 1.0, picks[:1], budget)
    assert nz == 8
    one_in = solver.OSC_TV_recon(pre, post, ang, g, 1, 0.2, 6, 3, 1.0, picks[:1])
    e1 = rel_l2(one, one_in)
    # three iterations
    got, nz = solver.OSC_TV_recon_ooc(pre, post, ang, g, n_iter, 0.2, 6, 3, 1.0, picks, budget)
    assert nz == 8
    incore = solver.OSC_TV_recon(pre, post, ang, g, n_iter, 0.2, 6, 3, 1.0, picks)
    ref = {}
    orc.osc_tv(pre, post, ang, SAD, geom, n_iter, 0.2, 6, 3, 1.0, picks,
               callback=lambda k, m: ref.__setitem__(k, m))
    e_in, e_orc = rel_l2(got, incore), rel_l2(got, ref[n_iter])
    print("out of core: iteration 1 vs in-core %.3g; iteration %d vs in-core %.3g, vs FP64 "
          "oracle %.3g (in-core vs oracle %.3g)" % (e1, n_iter, e_in, e_orc,
                                                     rel_l2(incore, ref[n_iter])))
    assert np.isfinite(got).all()
    # parallel rays keep their z, so each ray's samples lie in one slab: the
    # slab parts are the in-core sums (measured: equal after iteration 1, 5e-7
    # after 3); cone rays cross slabs (FP32 sums of parts: 6.5e-8, then 8e-5)
    assert e1 <= (1e-7 if geom == 0 else 2e-6)
    assert e_in <= (2e-5 if geom == 0 else 1e-3)
    assert e_orc <= 5e-3


@pytest.mark.gpu
def test_ooc_one_slab_equals_in_core(cuda):
    """With the whole volume in one slab the sweeps differ from the in-core solver
    only in how the FP64 norms are combined."""
    from mexct import solver

    W, H, nP = 32, 24, 24
    ang, pre, post = _problem(W, H, nP, 1, seed=5)
    g = {"type": "fan3d", "SAD": SAD}
    got, nz = solver.OSC_TV_recon_ooc(pre, post, ang, g, 3, 0.2, 6, 3, 1.0, [2, 0, 1], 1 << 34)
    assert nz == H
    incore = solver.OSC_TV_recon(pre, post, ang, g, 3, 0.2, 6, 3, 1.0, [2, 0, 1])
    assert rel_l2(got, incore) <= 1e-6


@pytest.mark.gpu
def test_ooc_empty_subsets_match_in_core(cuda):
    """More subsets than views: the empty subsets' update (num = den = 0) zeroes
    mu, as in the in-core solver."""
    from mexct import solver

    W, H, nP = 32, 16, 5
    ang, pre, post = _problem(W, H, nP, 2, seed=7)
    g = {"type": "cone3d", "SAD": SAD}
    budget = _budget_for(W, H, nP, 2, 2, 7, 7, 1.0, 4)
    got, nz = solver.OSC_TV_recon_ooc(pre, post, ang, g, 2, 0.2, 7, 7, 1.0, [3, 6], budget)
    assert nz == 4
    incore = solver.OSC_TV_recon(pre, post, ang, g, 2, 0.2, 7, 7, 1.0, [3, 6])
    assert np.isfinite(got).all() and np.isfinite(incore).all()
    assert np.array_equal(got == 0, incore == 0)
    assert np.allclose(got, incore, rtol=2e-3, atol=1e-12)


def test_ooc_argument_errors(lib):
    """Arguments are checked before any device work (no GPU needed)."""
    from mexct import _lib, solver

    pre = np.ones((16, 8, 6), dtype=np.float32, order="F")
    ang = np.linspace(0, np.pi, 6).astype(np.float32)
    g = {"type": "cone3d", "SAD": SAD}
    with pytest.raises(_lib.MexctError, match="status 1"):
        solver.OSC_TV_recon_ooc(pre, pre, ang, g, 0, 0.2, 3, 3, 1.0, [0], 1 << 30)
    with pytest.raises(ValueError):
        solver.OSC_TV_recon_ooc(pre, pre, ang, g, 2, 0.2, 3, 3, 1.0, [0], 1 << 30)
    with pytest.raises(_lib.MexctError, match="status 1"):
        _lib.call("mexct_osc_tv_recon_ooc", None, None, None, 16, 8, 6, None, 1000.0, 2, 1, 0.2,
                  3, 3, 1.0, None, 1 << 30, None, None)
