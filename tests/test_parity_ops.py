"""GPU parity of every operator against the FP64 oracle, through the C ABI.

FP32 results must be within 1e-5 relative L2 of the oracle (the required tolerance);
the per-operator tolerance is written next to each assertion.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5  # FP32 vs FP64 oracle, relative L2


def _phantom(W, H, seed=3, count=6):
    from mexct import phantoms

    return phantoms.ellipsoids(W, count=count, seed=seed, nz=H)


@pytest.mark.parametrize("geom", [0, 1, 2])
@pytest.mark.parametrize("W,H,nP", [(48, 40, 24), (37, 29, 13), (64, 64, 32)])
def test_fp_matches_oracle(cuda, orc, geom, W, H, nP):
    import mexct
    from mexct import phantoms

    vol = _phantom(W, H)
    ang = phantoms.angles_full(nP)
    got = mexct.CUDAmex_FP(vol, 1000.0, ang, nP, geom)
    ref = orc.fp(vol, 1000.0, ang, nP, geom)
    assert got.shape == (W, H, nP)
    assert rel_l2(got, ref) <= TOL


@pytest.mark.parametrize("geom", [0, 1, 2])
def test_fp_short_sad_and_odd_angles(cuda, orc, geom):
    """Strong magnification (SAD = 60 voxels) and irregular angles exercise the clip."""
    import mexct

    W, H, nP = 40, 36, 11
    vol = _phantom(W, H, seed=9)
    ang = np.random.default_rng(1).uniform(-7, 7, nP).astype(np.float32)
    got = mexct.CUDAmex_FP(vol, 60.0, ang, nP, geom)
    ref = orc.fp(vol, 60.0, ang, nP, geom)
    assert rel_l2(got, ref) <= TOL


@pytest.mark.parametrize("geom", [0, 1, 2])
@pytest.mark.parametrize("W,H,nP", [(48, 40, 24), (37, 29, 13), (64, 64, 32)])
def test_bp_matches_oracle(cuda, orc, geom, W, H, nP):
    import mexct
    from mexct import phantoms

    rng = np.random.default_rng(W + H + geom)
    sino = np.asfortranarray(rng.uniform(-1, 2, (W, H, nP)).astype(np.float32))
    ang = phantoms.angles_full(nP)
    got = mexct.CUDAmex_BP(sino, 1000.0, ang, geom)
    ref = orc.bp(sino, 1000.0, ang, geom)
    assert got.shape == (W, W, H)
    assert rel_l2(got, ref) <= TOL


def test_config1_cylinder_cone_fp_then_bp(cuda, orc):
    """Cone FP then BP of the 128^3 uniform cylinder (0.02 inside x^2+y^2 <= 47^2),
    256 float32 angles linspace(0, 2*pi), SAD 1000, against the FP64 oracle."""
    import mexct
    from mexct import phantoms

    vol = phantoms.cylinder(128, 128, radius=47.0, value=0.02)
    ang = phantoms.angles_full(256)
    fp = mexct.CUDAmex_FP(vol, 1000.0, ang, 256, 2)
    ref_fp = orc.fp(vol, 1000.0, ang, 256, 2)
    assert rel_l2(fp, ref_fp) <= TOL
    bp = mexct.CUDAmex_BP(fp, 1000.0, ang, 2)
    ref_bp = orc.bp(fp, 1000.0, ang, 2)
    assert rel_l2(bp, ref_bp) <= TOL


@pytest.mark.parametrize("geom", [0, 2])
def test_fp_texture_variant_difference(cuda, orc, geom):
    """The hardware-texture FP follows the reference's arithmetic (the texture
    unit's 8-bit filter weights, binary32 stepping), so it sits ~1e-4 from the
    exact-weight oracle and lands on the oracle run with the texture unit's weight
    rule and the reference's stepping (FP32 summation is the only difference)."""
    import oracle
    import torch
    from mexct import ops, phantoms

    W, H, nP = 64, 64, 32
    vol = _phantom(W, H)
    ang = phantoms.angles_full(nP)
    dvol = torch.from_numpy(np.ascontiguousarray(vol.transpose(2, 1, 0))).cuda()
    out = ops.fp_dev(dvol, 1000.0, ang, geom, variant=1)
    got = out.cpu().numpy().transpose(2, 1, 0)
    errs = {}
    for name, mode in [("exact", oracle.TEX_EXACT), ("tex8_nearest", oracle.TEX8_NEAREST),
                       ("hw", oracle.TEX_HW)]:
        with oracle.tex_weights(mode):
            errs[name] = rel_l2(got, orc.fp(vol, 1000.0, ang, nP, geom))
    with oracle.tex_weights(oracle.TEX_HW), oracle.ref_steps(1):
        errs["hw_steps"] = rel_l2(got, orc.fp(vol, 1000.0, ang, nP, geom))
    print("texture FP rel-L2 vs oracle (geom %d):" % geom,
          {k: "%.3g" % v for k, v in errs.items()})
    assert errs["exact"] <= 5e-4
    assert errs["hw_steps"] <= 5e-6
    assert errs["hw_steps"] < errs["tex8_nearest"] < errs["exact"]


def test_general3d_fp_parallel_pts_matches_oracle(cuda, orc):
    import mexct
    from mexct import phantoms

    S, Z = 40, 32
    vol = _phantom(S, Z, seed=5)
    pts = phantoms.parallel_pts(S, Z, L=1000.0)
    ang = phantoms.angles_full(9)
    got = mexct.CUDAmex_general3D_FP(vol, ang, pts, 9)
    ref = orc.g3d_fp(vol, ang, pts, 9)
    assert rel_l2(got, ref) <= TOL


def test_general3d_fp_helix_per_view(cuda, orc):
    import mexct
    from mexct import phantoms

    S, Z = 40, 36
    vol = _phantom(S, Z, seed=6)
    pts, ang = phantoms.helix_pts(24, 20, 10, Z, sad=300.0, seed=2)
    got = mexct.CUDAmex_general3D_FP(vol, ang, pts, 10)
    ref = orc.g3d_fp(vol, ang, pts, 10)
    assert rel_l2(got, ref) <= TOL


@pytest.mark.parametrize("kind", ["parallel", "helix"])
def test_general3d_bp_matches_oracle(cuda, orc, kind):
    """Two-corner scatter: voxel indices/weights are binary32-exact, only the
    accumulation order (atomics vs FP64 sum) differs."""
    import mexct
    from mexct import phantoms

    S, Z = 36, 28
    if kind == "parallel":
        pts = phantoms.parallel_pts(S, Z, L=1000.0)
        ang = phantoms.angles_full(8)
        W, H = S, Z
    else:
        W, H = 20, 16
        pts, ang = phantoms.helix_pts(W, H, 8, Z, sad=300.0, seed=4)
    rng = np.random.default_rng(7)
    sino = np.asfortranarray(rng.uniform(0, 1, (W, H, 8)).astype(np.float32))
    got = mexct.CUDAmex_general3D_BP(sino, ang, pts, S, Z)
    ref = orc.g3d_bp(sino, ang, pts, S, Z)
    assert rel_l2(got, ref) <= TOL


@pytest.mark.parametrize("geom", [0, 1, 2])
def test_osc_iteration_matches_oracle(cuda, orc, geom):
    """One full OSC iteration (all subsets, in the given order) from the driver's
    initial state mu = 1e-10; FP32 GPU vs FP64 oracle."""
    import mexct
    from mexct import phantoms

    W, H, nP, nsub = 40, 32, 24, 6
    vol = _phantom(W, H, seed=11)
    ang = phantoms.angles_full(nP)
    fp = orc.fp(vol, 1000.0, ang, nP, geom).astype(np.float32)
    pre, post = phantoms.poisson_counts(fp, 1e5, seed=1)
    mu = np.full((W, W, H), np.float32(1e-10), dtype=np.float32, order="F")
    picks = orc.subset_order(nsub, 2)
    ref = orc.osc_iter(mu, pre, post, nsub, picks, ang, 1000.0, geom)
    pre0, post0 = pre.copy(), post.copy()
    mexct.CUDAmex_oscIter(mu, pre, post, nsub, picks, ang, 1000.0, geom)
    assert np.array_equal(pre, pre0) and np.array_equal(post, post0)
    assert rel_l2(mu, ref) <= TOL


def test_osc_empty_subset_zeroes_circle(cuda, orc):
    """A subset with no views divides 0 by 0 in the update: the reference's fmaxf
    turns the NaN into 0 inside the circle; outside it mu is untouched."""
    import mexct
    from mexct import phantoms

    W, H, nP = 24, 16, 6
    ang = phantoms.angles_full(nP)
    pre = np.full((W, H, nP), 1e5, dtype=np.float32, order="F")
    post = np.full((W, H, nP), 9e4, dtype=np.float32, order="F")
    mu = np.full((W, W, H), np.float32(0.01), dtype=np.float32, order="F")
    picks = np.array([7], dtype=np.int32)  # subset 7 of 1: no view
    ref = orc.osc_iter(mu, pre, post, 1, picks, ang, 1000.0, 2)
    mexct.CUDAmex_oscIter(mu, pre, post, 1, picks, ang, 1000.0, 2)
    assert np.array_equal(mu, ref.astype(np.float32))
    assert mu[W // 2, W // 2, 0] == 0.0 and mu[0, 0, 0] == np.float32(0.01)


@pytest.mark.parametrize("shape", [(32, 32, 32), (33, 27, 19), (64, 48, 40)])
def test_tvmin3d_matches_oracle(cuda, orc, shape):
    import mexct
    from mexct import phantoms

    vol = phantoms.ellipsoids(shape[0], count=5, seed=2, nz=shape[2])[:, : shape[1], :]
    vol = np.asfortranarray(vol + np.random.default_rng(0).normal(0, 1e-3, vol.shape).astype(np.float32))
    got = mexct.CUDAmex_TVmin_3D(vol, 0.05)
    ref = orc.tvmin3d(vol, 0.05, 20)
    assert rel_l2(got, ref) <= TOL


@pytest.mark.parametrize("shape", [(124, 15, 33), (248, 31, 65), (128, 16, 32), (36, 20, 17),
                                   (123, 15, 33)])
def test_tv_steps_match_oracle_at_tile_edges(cuda, orc, shape):
    """One and two TV steps on shapes at the tiles' edges: the four-voxel kernel
    (x extent a multiple of 4: tiles of 124 x 15 outputs, the last lane and row
    only supplying neighbour terms) and the scalar one (odd x extent) against the
    FP64 oracle.  Over 20 steps the descent's normalised step amplifies rounding
    (2e-6 .. 3e-5 on these thin shapes), so the steps are checked one by one."""
    import torch
    from mexct import ops, phantoms

    nx, ny, nz = shape
    v = phantoms.ellipsoids(max(nx, ny), count=5, seed=3, nz=nz)[:nx, :ny, :]
    v = np.asfortranarray(v + np.random.default_rng(2).normal(0, 2e-3, v.shape).astype(np.float32))
    d = torch.from_numpy(np.ascontiguousarray(v.transpose(2, 1, 0))).cuda()
    for steps in (1, 2):
        got = ops.tvmin3d_dev(d, 0.03, steps).cpu().numpy().transpose(2, 1, 0)
        assert rel_l2(got, orc.tvmin3d(v, 0.03, steps)) <= 2e-7, steps


@pytest.mark.parametrize("geom", [0, 1, 2])
@pytest.mark.parametrize("filt", ["ramp", "hamming", "shepp-logan"])
def test_prefilter_matches_oracle(cuda, orc, geom, filt):
    import mexct
    from mexct import phantoms

    W, nP = 48, 40
    rng = np.random.default_rng(geom)
    sino = np.asfortranarray(rng.uniform(0, 3, (W, W, nP)).astype(np.float32))
    ang = phantoms.angles_full(nP)
    gs = {"type": ["par3d", "fan3d", "cone3d"][geom], "SAD": 1000.0}
    got = mexct.preFilterSinogram(sino, gs, ang, filt, 0.9, 1.0)
    ref = orc.prefilter(sino, geom, ang, filt, 0.9, 1.0, sad=1000.0)
    assert rel_l2(got, ref) <= TOL


def test_fbp_recon_matches_oracle_chain(cuda, orc):
    import mexct
    from mexct import phantoms

    W, nP = 48, 64
    vol = _phantom(W, W, seed=4)
    ang = phantoms.angles_full(nP)
    fp = orc.fp(vol, 1000.0, ang, nP, 2).astype(np.float32)
    pre, post = phantoms.poisson_counts(fp, 1e5, seed=3)
    got = mexct.FBP_recon(pre, post, ang, {"type": "cone3d", "SAD": 1000.0}, "hamming", 1.0, 1.0)
    sino = -np.log(post.astype(np.float32) / pre.astype(np.float32))
    sino[~np.isfinite(sino)] = 0
    filt = orc.prefilter(np.asfortranarray(sino.astype(np.float32)), 2, ang, "hamming", 1.0, 1.0)
    ref = orc.bp(filt.astype(np.float32), 1000.0, ang, 2)
    assert rel_l2(got, ref) <= 2 * TOL


@pytest.mark.parametrize("geom", [0, 1, 2])
def test_fp_slab_large_detector_multiple_tiles(cuda, orc, geom):
    """Several detector tiles and slabs per ray (160^2 x 96, 7 views): the
    TMA slab path, its bounding boxes and the slab hand-over are exercised."""
    import mexct
    from mexct import phantoms

    W, H, nP = 160, 96, 7
    vol = _phantom(W, H, seed=21, count=8)
    ang = np.array([0.0, 0.3, 0.7854, 1.2, 2.0, 3.9, 5.5], np.float32)
    got = mexct.CUDAmex_FP(vol, 1000.0, ang, nP, geom)
    ref = orc.fp(vol, 1000.0, ang, nP, geom)
    assert rel_l2(got, ref) <= TOL


@pytest.mark.parametrize("geom", [0, 1, 2])
def test_tall_volume_every_detector_row(cuda, orc, geom):
    """H = 40 > 32 ceil(W / 32) = 32: the reference's FP grid is sized by W
    (CUDAmex_FP.cu:432-440), so its rows 32..39 are never written and stay 0.
    Every row is computed here (a stated deviation), FP and its texture variant
    alike, within the FP32 bar of the oracle; BP covers every slice."""
    import oracle
    import torch
    import mexct
    from mexct import _lib, ops

    W, H, nP = 24, 40, 6
    rng = np.random.default_rng(40 + geom)
    vol = np.asfortranarray(rng.uniform(0.5, 1.5, (W, W, H)).astype(np.float32))
    ang = np.linspace(0.1, 2 * np.pi, nP, endpoint=False).astype(np.float32)
    got = mexct.CUDAmex_FP(vol, 1000.0, ang, nP, geom)
    ref = orc.fp(vol, 1000.0, ang, nP, geom)
    assert np.count_nonzero(got[:, 32:, :]) > 0.9 * got[:, 32:, :].size
    assert rel_l2(got, ref) <= TOL
    dvol = torch.from_numpy(np.ascontiguousarray(vol.transpose(2, 1, 0))).cuda()
    tex = ops.fp_dev(dvol, 1000.0, ang, geom, variant=_lib.FP_TEXTURE)
    tex = tex.cpu().numpy().transpose(2, 1, 0)
    assert np.count_nonzero(tex[:, 32:, :]) > 0.9 * tex[:, 32:, :].size
    with oracle.tex_weights(oracle.TEX_HW), oracle.ref_steps(1):
        ref_hw = orc.fp(vol, 1000.0, ang, nP, geom)  # 8-bit weights, binary32 steps
    assert rel_l2(tex, ref_hw) <= 5e-6
    bp = mexct.CUDAmex_BP(got, 1000.0, ang, geom)
    assert rel_l2(bp, orc.bp(got, 1000.0, ang, geom)) <= TOL


@pytest.mark.parametrize("variant", [0, 2])
def test_fp_variants_agree(cuda, orc, variant):
    """Slab-staged (0) and one-ray-per-thread (2) explicit FP32 paths both meet
    the 1e-5 bar."""
    import torch
    from mexct import ops, phantoms

    W, H, nP = 96, 64, 16
    vol = _phantom(W, H, seed=13)
    ang = phantoms.angles_full(nP)
    dvol = torch.from_numpy(np.ascontiguousarray(vol.transpose(2, 1, 0))).cuda()
    for geom in (0, 1, 2):
        out = ops.fp_dev(dvol, 1000.0, ang, geom, variant=variant)
        got = out.cpu().numpy().transpose(2, 1, 0)
        assert rel_l2(got, orc.fp(vol, 1000.0, ang, nP, geom)) <= TOL


@pytest.mark.parametrize("dt,tol", [("float16", 1e-3), ("bfloat16", 1e-2)])
def test_fp_bp_low_precision_storage(cuda, orc, dt, tol):
    """FP16/BF16 storage of volume and sinogram, FP32 accumulation: relative L2 to
    the FP64 oracle within 1e-3 (FP16; BF16 has an 8-bit mantissa: 1e-2)."""
    import torch
    from mexct import ops, phantoms

    W, H, nP = 64, 48, 24
    vol = _phantom(W, H, seed=17)
    ang = phantoms.angles_full(nP)
    t = getattr(torch, dt)
    dvol = torch.from_numpy(np.ascontiguousarray(vol.transpose(2, 1, 0))).cuda().to(t)
    for geom in (0, 2):
        fp = ops.fp_dev(dvol, 1000.0, ang, geom, out_dtype=torch.float32)
        ref = orc.fp(dvol.float().cpu().numpy().transpose(2, 1, 0).copy(order="F"), 1000.0, ang,
                     nP, geom)
        assert rel_l2(fp.cpu().numpy().transpose(2, 1, 0), ref) <= tol
        sino = fp.to(t)
        bp = ops.bp_dev(sino, 1000.0, ang, geom, out_dtype=torch.float32)
        refb = orc.bp(sino.float().cpu().numpy().transpose(2, 1, 0).copy(order="F"), 1000.0, ang,
                      geom)
        assert rel_l2(bp.cpu().numpy().transpose(2, 1, 0), refb) <= tol


@pytest.mark.gpu
def test_fp_slab_kernel_keeps_four_ctas_per_sm(cuda):
    """The slab FP's shared memory (two 27 KB buffers per CTA) and the largest
    carveout leave room for the 4 resident CTAs its launch bounds assume."""
    from mexct import ops

    assert ops.fp_slab_occupancy() == 4


@pytest.mark.gpu
def test_prefilter_tables_follow_the_scan_geometry(cuda, orc):
    """The context keeps the pre-filter tables of the last scan geometry: a repeat
    call reuses them (identical output), and changed angles, Parker q or SAD
    rebuild them (each result matches the oracle)."""
    import mexct

    rng = np.random.default_rng(9)
    W, nP = 32, 24
    sino = np.asfortranarray(rng.uniform(0, 1, (W, W, nP)).astype(np.float32))
    ang = np.linspace(0, 1.3 * np.pi, nP).astype(np.float32)
    a = mexct.preFilterSinogram(sino, {"type": "cone3d", "SAD": 1000.0}, ang, "ramp", 1.0, 1.0)
    b = mexct.preFilterSinogram(sino, {"type": "cone3d", "SAD": 1000.0}, ang, "ramp", 1.0, 1.0)
    assert np.array_equal(a, b)
    for ang2, q, sad in ((ang * np.float32(0.9), 1.0, 1000.0), (ang, 0.5, 1000.0),
                         (ang, 1.0, 400.0)):
        got = mexct.preFilterSinogram(sino, {"type": "cone3d", "SAD": sad}, ang2, "ramp", 1.0, q)
        ref = orc.prefilter(sino, 2, ang2, "ramp", 1.0, q, sad=sad)
        assert rel_l2(got, ref) <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["random", "wide_helix"])
def test_general3d_fp_hard_rays_match_oracle(cuda, orc, kind):
    """general3D rays the slab kernel cannot box: random end points (mixed
    directions in a tile, rays parallel to a face, rays missing the volume and
    marched between two outside points as the reference does), and a helix whose
    detector is much wider and taller than the volume's shadow.  The volume's
    faces are non-zero, so the border (zero) frame around them matters."""
    import mexct
    from mexct import phantoms

    S, Z = 24, 20
    vol = _phantom(S, Z, seed=8)
    vol[0, :, :] += 0.5
    vol[:, -1, :] += 0.25
    vol[:, :, 0] += 0.75
    if kind == "random":
        rng = np.random.default_rng(12)
        W, H, nP = 40, 16, 5
        pts = rng.uniform(-30, 30, (W, H, 6, nP)).astype(np.float32)
        pts[:4, :, 2, :] = pts[:4, :, 5, :]  # some rays parallel to the z planes
        pts[4:8, :, 0, :] = pts[4:8, :, 3, :]  # some parallel to the x planes
        pts = np.asfortranarray(pts)
        ang = np.linspace(0, 2 * np.pi, nP, endpoint=False).astype(np.float32)
    else:
        W, H, nP = 64, 48, 6
        pts, ang = phantoms.helix_pts(W, H, nP, Z, sad=300.0, seed=3)
    got = mexct.CUDAmex_general3D_FP(vol, ang, pts, nP)
    ref = orc.g3d_fp(vol, ang, pts, nP)
    assert rel_l2(got, ref) <= TOL


def test_general3d_matched_bp_matches_oracle_and_is_the_adjoint(cuda, orc):
    """The matched-adjoint general3D BP against the FP64 oracle's transpose of
    its general3D FP (1e-5), and the GPU pair (slab FP, matched BP) passes the
    dot-product test <FP x, y> = <x, BP y> to FP32 rounding, shared and per-view
    points, rays crossing, grazing and missing the volume."""
    import mexct
    from mexct import phantoms

    S, Z = 48, 36
    rng = np.random.default_rng(7)
    pts, ang = phantoms.helix_pts(40, 30, 12, Z, sad=90.0, seed=5)
    x = np.asfortranarray(rng.uniform(0, 1, (S, S, Z)).astype(np.float32))
    y = np.asfortranarray(rng.uniform(-1, 1, (40, 30, 12)).astype(np.float32))
    for p in (pts, np.asfortranarray(pts[..., 0])):
        bt = mexct.general3D_BP_matched(y, ang, p, S, Z)
        ref = orc.g3d_bp_matched(y, ang, p, S, Z)
        assert rel_l2(bt, ref) <= TOL
        fx = mexct.CUDAmex_general3D_FP(x, ang, p, 12)
        lhs = float(np.sum(fx.astype(np.float64) * y))
        rhs = float(np.sum(x.astype(np.float64) * bt))
        assert abs(lhs - rhs) <= 1e-5 * abs(lhs)
