"""Known-answer tests that pin the FP64 oracle (CPU only).

The reference ships no tests, golden vectors or fixtures, so the oracle is pinned by
its source (every oracle function cites the file:line it restates) and by these
closed-form answers, plus the committed golden fixtures in tests/golden/.
"""
import numpy as np
import pytest

from conftest import rel_l2


def _cyl(W, H, r, val=1.0):
    from mexct import phantoms

    return phantoms.cylinder(W, H, radius=r, value=val)


def _row_counts(W, r):
    c = np.arange(W) - (W - 1) / 2.0
    x, y = np.meshgrid(c, c, indexing="ij")
    return ((x * x + y * y) <= r * r).sum(axis=0)  # count along x for each y


@pytest.mark.parametrize("beta", [0.0, np.pi / 2])
def test_parallel_fp_of_cylinder_is_voxel_count(orc, beta):
    """A parallel ray along a grid axis with step 0.5 and linear interpolation sums
    the voxel values of its row exactly (edge voxels are 0)."""
    W, H, r = 40, 6, 15.0
    vol = _cyl(W, H, r, 1.0)
    fp = orc.fp(vol, 1000.0, np.array([beta], np.float32), 1, 0)
    counts = _row_counts(W, r)
    if beta != 0.0:
        counts = counts[::-1]
    for iy in range(H):
        np.testing.assert_allclose(fp[:, iy, 0], counts, atol=1e-6)


def test_empty_volume_projects_to_zero(orc):
    vol = np.zeros((16, 16, 8), np.float32, order="F")
    for g in (0, 1, 2):
        assert np.all(orc.fp(vol, 1000.0, np.array([0.3], np.float32), 1, g) == 0)


def test_single_voxel_trilinear_hat(orc):
    """A parallel ray through a one-voxel volume samples the clamp-extended trilinear
    hat: the clamp makes every in-box sample equal to the voxel value."""
    vol = np.full((1, 1, 1), 2.0, np.float32, order="F")
    fp = orc.fp(vol, 1000.0, np.array([0.0], np.float32), 1, 0)
    # One ray (u0 = v0 = 0) crosses the unit box in x: 2 samples of 0.5.
    assert fp.shape == (1, 1, 1)
    np.testing.assert_allclose(fp[0, 0, 0], 2.0, atol=1e-12)


@pytest.mark.parametrize("geom", [0, 1, 2])
def test_bp_of_constant_sinogram(orc, geom):
    """BP of a constant c: par gives nP*c inside the circle; fan/cone give
    c * sum(U^2); zero outside the circle h = W/2 - 1 (CUDAmex_BP.cu:73-77)."""
    W, H, nP, c, sad = 20, 6, 7, 0.5, 1000.0
    ang = np.linspace(0, 2 * np.pi, nP).astype(np.float32)
    sino = np.full((W, H, nP), c, np.float32, order="F")
    vol = orc.bp(sino, sad, ang, geom)
    h = W // 2 - 1
    for ix in range(W):
        for iy in range(W):
            inside = (ix - h) ** 2 + (iy - h) ** 2 < h * h
            if not inside:
                assert np.all(vol[ix, iy, :] == 0)
                continue
            if geom == 0:
                exp = nP * c
            else:
                x, y = ix - (h + 0.5), iy - (h + 0.5)
                sb = np.sin(ang.astype(np.float64)).astype(np.float32).astype(np.float64)
                cb = np.cos(ang.astype(np.float64)).astype(np.float32).astype(np.float64)
                s = x * cb + y * sb
                exp = c * np.sum((sad / (sad - s)) ** 2)
            np.testing.assert_allclose(vol[ix, iy, :], exp, rtol=1e-12)


def test_tv_gradient_of_constant_is_zero(orc):
    v = np.full((6, 7, 5), 0.3, np.float64, order="F")
    assert np.all(orc.tv_gradient(v) == 0)


def test_tv_gradient_of_linear_ramp(orc):
    """x = a*i: interior term (3x - xm - ym - zm)/(eps + |.|) minus the forward
    terms; for a ramp along x only: a/(eps+a) - a/(eps+a) = 0."""
    i = np.arange(8, dtype=np.float64)
    v = np.asfortranarray(np.broadcast_to(0.1 * i[:, None, None], (8, 5, 5)).copy())
    g = orc.tv_gradient(v)
    np.testing.assert_allclose(g, 0, atol=1e-12)


def test_tv_step_on_constant_volume_is_nan(orc):
    """||g|| = 0 makes the reference's step -c/0: IEEE arithmetic gives NaN
    everywhere, which OSC_TV_recon.m:69-70 then maps to 0."""
    v = np.full((5, 5, 5), 0.2, np.float64, order="F")
    out = orc.tvmin3d(v, 0.1, 1)
    assert np.all(np.isnan(out))


def test_osc_fixed_point(orc):
    """post = pre*exp(-FP(mu)) makes num = BP(yhat - y) vanish: mu is a fixed point
    of the OSC update (parallel geometry, mu zero near the border so that the
    clamp FP equals the OSC border FP)."""
    from mexct import phantoms

    W, H, nP = 24, 12, 12
    mu = np.zeros((W, W, H), np.float64, order="F")
    mu[6:18, 6:18, 2:10] = 0.01
    ang = phantoms.angles_full(nP)
    l = orc.fp(mu.astype(np.float32), 1000.0, ang, nP, 0)
    pre = np.full((W, H, nP), 1e5, np.float32, order="F")
    post = np.asfortranarray((1e5 * np.exp(-l)).astype(np.float32))
    out = orc.osc_iter(mu, pre, post, 3, np.array([1, 0, 2], np.int32), ang, 1000.0, 0)
    inside = mu > 0
    np.testing.assert_allclose(out[inside], mu[inside], rtol=1e-5)
    assert np.all(out[~inside] == 0)


def test_subset_order_matches_hand_trace(orc):
    """calcSubsetOrder (OSC_TV_recon.m:80-102) traced by hand for 10 subsets with
    randperm's first pick 4 (1-based)."""
    assert orc.subset_order(10, 3).tolist() == [3, 6, 2, 7, 1, 5, 8, 0, 4, 9]
    for n in (1, 2, 5, 16, 64):
        for first in range(n):
            p = orc.subset_order(n, first)
            assert sorted(p.tolist()) == list(range(n)) and p[0] == first


def test_num_subsets_schedule(orc):
    """calcNumSubsets (OSC_TV_recon.m:76-78) with MATLAB round-half-away."""
    assert orc.num_subsets(64, 2, 0.2, 10, 1) == 64
    assert orc.num_subsets(64, 2, 0.2, 10, 10) == 2
    assert orc.num_subsets(10, 10, 0.2, 20, 7) == 10
    v = (64 - 2) / 9 ** 0.2 * (10 - 5) ** 0.2 + 2
    assert orc.num_subsets(64, 2, 0.2, 10, 5) == int(np.floor(v + 0.5))


@pytest.mark.parametrize("filt", ["ramp", "hamming", "shepp-logan", "cosine", "hann"])
def test_filter_response_matches_numpy_fft(orc, filt):
    """designFilter (preFilterSinogram.m:95-152) restated with numpy's FFT."""
    W, d = 50, 0.8
    order = max(64, 1 << int(np.ceil(np.log2(2 * W))))
    n = np.arange(order // 2 + 1)
    h = np.zeros(order // 2 + 1)
    h[0] = 0.25
    h[1::2] = -1.0 / (np.pi * n[1::2]) ** 2
    h = np.concatenate([h, h[-2:0:-1]])
    f = 2 * np.real(np.fft.fft(h))[: order // 2 + 1]
    w = 2 * np.pi * np.arange(f.size) / order
    with np.errstate(divide="ignore", invalid="ignore"):
        win = {"ramp": np.ones_like(w), "hamming": 0.54 + 0.46 * np.cos(w / d),
               "shepp-logan": np.sin(w / (2 * d)) / (w / (2 * d)), "cosine": np.cos(w / (2 * d)),
               "hann": (1 + np.cos(w / d)) / 2}[filt]
    f[1:] *= win[1:]
    f[w > np.pi * d] = 0
    H = np.concatenate([f, f[-2:0:-1]])
    np.testing.assert_allclose(orc.filter_response(W, filt, d), H, atol=1e-12)


def test_prefilter_matches_numpy_fft_chain(orc):
    """preFilterSinogram for cone3d: cosine weight, Parker window, zero-padded FFT
    filter ('symmetric' ifft), dbeta/2 -- restated with numpy for a square detector."""
    W, nP, sad, q = 16, 9, 200.0, 1.0
    rng = np.random.default_rng(0)
    sino = np.asfortranarray(rng.uniform(0, 1, (W, W, nP)).astype(np.float32))
    ang = np.linspace(0, 2 * np.pi, nP).astype(np.float32)
    got = orc.prefilter(sino, 2, ang, "hamming", 1.0, q, sad=sad)
    U = np.arange(1, W + 1)[:, None] - (W - 1) / 2.0
    V = np.arange(1, W + 1)[None, :] - (W - 1) / 2.0
    s = sino.astype(np.float64) * (sad / np.sqrt(sad ** 2 + U ** 2 + V ** 2))[:, :, None]
    alpha = -np.arctan((-W / 2 + 0.5 + np.arange(W)) / sad)  # increasing angles: flipped
    delta = abs(alpha[-1] - alpha[0]) / 2
    ext = abs(float(ang[-1]) - float(ang[0]))
    eps = max(ext - (np.pi + 2 * delta), 0)

    def S(b):
        out = np.zeros_like(b)
        m = np.abs(b) < 0.5
        out[m] = 0.5 * (1 + np.sin(np.pi * b[m]))
        out[b >= 0.5] = 1
        return out

    def b2(a):
        return q * (2 * delta - 2 * a + eps)

    for i in range(nP):
        beta = abs(float(ang[i]) - float(ang[0]))
        wdw = 0.5 * (S(beta / b2(alpha) - 0.5) + S((beta - 2 * delta + 2 * alpha - eps) / b2(alpha) + 0.5)
                     - S((beta - np.pi + 2 * alpha) / b2(-alpha) - 0.5)
                     - S((beta - np.pi - 2 * delta - eps) / b2(-alpha) + 0.5))
        s[:, :, i] *= wdw[:, None]
    H = orc.filter_response(W, "hamming", 1.0)
    order = H.size
    pad = np.zeros((order, W, nP))
    pad[:W] = s
    flt = np.real(np.fft.ifft(np.fft.fft(pad, axis=0) * H[:, None, None], axis=0))[:W]
    db = np.diff(ang.astype(np.float32)).astype(np.float64) / 2
    db = np.concatenate([[db[0]], db])
    exp = flt * db[None, None, :]
    np.testing.assert_allclose(got, exp, atol=1e-10 * np.abs(exp).max())


def test_g3d_fp_parallel_pts_equals_standard_parallel_fp(orc):
    """general3D_projection_test.m:13-38: parallel rays given as pts match
    CUDAmex_FP geom 0.  At beta = 0 and pi/2 both sum whole voxel rows."""
    from mexct import phantoms

    W, H, r = 32, 8, 12.0
    vol = _cyl(W, H, r, 0.5)
    pts = phantoms.parallel_pts(W, H, L=1000.0)
    ang = np.array([0.0, np.pi / 2], np.float32)
    a = orc.g3d_fp(vol, ang, pts, 2)
    b = orc.fp(vol, 1000.0, ang, 2, 0)
    np.testing.assert_allclose(a, b, atol=1e-9)


def test_g3d_bp_two_corner_weights(orc):
    """One ray along x through a 4x4x4 grid at y = z = 0.25 off-centre: each 0.5
    step deposits p*0.5*wxx*wyy*(1-wz) at kL and p*0.5*wxx*wyy*wz at kU with the
    reference's [0.5, 1.5) weights (CUDAmex_general3D_BP.cu:161-170)."""
    S = Z = 4
    pts = np.zeros((1, 1, 6), np.float32, order="F")
    pts[0, 0, :] = [-2, 0.3, 0.3, 2, 0.3, 0.3]  # end points on the box faces: exact clip
    sino = np.ones((1, 1, 1), np.float32, order="F")
    vol = orc.g3d_bp(sino, np.array([0.0], np.float32), pts, S, Z)
    # Samples at x = -2 + 0.5k, k = 0..7 (distance 4, step 0.5).
    exp = np.zeros((S, S, Z))
    fy, fz = np.float32(0.3) + 2, np.float32(0.3) + 2
    jL, kL = int(np.floor(fy)), int(np.floor(fz))
    for k in range(8):
        fx = np.float32(-2.0 + 0.5 * k) + np.float32(2.0)
        iL, iU = int(np.floor(fx)), int(np.ceil(fx))
        if iL < 0 or iU >= S or int(np.ceil(fy)) >= S or int(np.ceil(fz)) >= Z:
            continue
        wxx = np.float32(fx - iL + np.float32(0.5))
        wyy = np.float32(fy - jL + np.float32(0.5))
        wz = np.float32(fz - kL + np.float32(0.5))
        exp[iL, jL, kL] += 0.5 * wxx * wyy * (1 - wz)
        exp[iL, jL, int(np.ceil(fz))] += 0.5 * wxx * wyy * wz
    np.testing.assert_allclose(vol, exp, rtol=1e-6)


def test_osc_tv_driver_runs_and_stays_finite(orc):
    """OSC_TV_recon.m driver: tiny problem, finite non-negative iterates."""
    from mexct import phantoms

    W, H, nP = 16, 8, 12
    vol = phantoms.ellipsoids(W, count=3, seed=1, nz=H)
    ang = phantoms.angles_full(nP)
    fp = orc.fp(vol, 1000.0, ang, nP, 2).astype(np.float32)
    pre, post = phantoms.poisson_counts(fp, 1e5, seed=0)
    seen = []
    mu = orc.osc_tv(pre, post, ang, 1000.0, 2, 3, 0.2, 4, 2, 1.0, [0, 1, 0],
                    callback=lambda k, m: seen.append(k))
    assert seen == [1, 2, 3]
    assert np.all(np.isfinite(mu))


def test_osc_tv_trajectory_is_rounding_sensitive(orc):
    """Conditioning of OSC_TV_recon.m: rounding only the FP64 state mu to binary32
    after each OSC and TV step (all arithmetic FP64) moves the trajectory by orders
    of magnitude more than one rounding, growing about tenfold per iteration.  No
    FP32 implementation can hold the later iterates to 1e-5 of the FP64 oracle;
    per-iterate errors are reported instead."""
    from mexct import phantoms

    W, H, nP, geom = 32, 24, 24, 0
    vol = phantoms.ellipsoids(W, count=4, seed=0, nz=H)
    ang = phantoms.angles_full(nP)
    fp = orc.fp(vol, 1000.0, ang, nP, geom).astype(np.float32)
    pre, post = phantoms.poisson_counts(fp, 1e5, seed=1)

    def run(round32):
        pc, qc = np.maximum(pre, 1e-6), np.maximum(post, 1e-6)
        p2, q2 = pc.copy(order="F"), qc.copy(order="F")
        p2.flat[0] = 0
        q2.flat[0] = 0
        mu = np.full((W, W, H), float(np.float32(1e-10)), order="F")
        out = []
        for k, first in enumerate([1, 4, 0, 2], start=1):
            old = mu.copy()
            old.flat[0] = 0
            ns = orc.num_subsets(6, 3, 1.0, 4, k)
            a, b = (pc, qc) if k == 1 else (p2, q2)
            mu = orc.osc_iter(mu, a, b, ns, orc.subset_order(ns, first % ns), ang, 1000.0, geom)
            if round32:
                mu = mu.astype(np.float32).astype(np.float64)
            if k > 1:
                d = old - mu
                d[np.isnan(d)] = 0
                mu = orc.tvmin3d(mu, 0.2 * np.sqrt((d * d).sum()), 20)
                mu[~np.isfinite(mu)] = 0
                if round32:
                    mu = mu.astype(np.float32).astype(np.float64)
            out.append(mu)
        return out

    a, b = run(False), run(True)
    e = [np.linalg.norm(x - y) / np.linalg.norm(x) for x, y in zip(a, b)]
    assert e[0] < 1e-7 and e[3] > 1e-4 and e[3] > 100 * e[1]


@pytest.mark.parametrize("geom", [0, 2])
def test_texture_weight_difference_is_stated(orc, geom):
    """The reference samples through CUDA's linear texture filter, whose weights
    are 1/256 fixed point.  The oracle's emulation of that states how far the
    reference's texture-filtered FP and BP sit from exact trilinear/bilinear
    output (the form every FP32 kernel here is checked against at 1e-5)."""
    import oracle
    from mexct import phantoms

    W, H, nP = 48, 40, 16
    vol = phantoms.ellipsoids(W, count=6, seed=3, nz=H)
    ang = phantoms.angles_full(nP)
    fp = orc.fp(vol, 1000.0, ang, nP, geom)
    bp = orc.bp(fp.astype(np.float32), 1000.0, ang, geom)
    out = {}
    for name, mode in [("nearest", oracle.TEX8_NEAREST), ("trunc", oracle.TEX8_TRUNC)]:
        with oracle.tex_weights(mode):
            fq = orc.fp(vol, 1000.0, ang, nP, geom)
            bq = orc.bp(fp.astype(np.float32), 1000.0, ang, geom)
        out[name] = (rel_l2(fq, fp), rel_l2(bq, bp))
    assert oracle.get_tex_weights() == oracle.TEX_EXACT
    print("8-bit texture weights vs exact, geom %d (FP, BP):" % geom,
          {k: ("%.3g" % a, "%.3g" % b) for k, (a, b) in out.items()})
    for a, b in out.values():
        # a weight error below 1/256 of a neighbour difference: well above FP32
        # rounding, well below 1e-3
        assert 1e-6 < a < 1e-3
        assert 1e-7 < b < 1e-3


@pytest.mark.parametrize("geom", [0, 1, 2])
def test_detector_generalisation_defaults_are_the_reference_form(orc, geom):
    """fp_det / bp_det with the volume's detector (pitch 1, one ray per pixel) are
    fp / bp bit for bit."""
    from mexct import phantoms

    W, H, nP = 24, 16, 6
    vol = phantoms.ellipsoids(W, count=3, seed=1, nz=H)
    ang = phantoms.angles_full(nP)
    fp = orc.fp(vol, 1000.0, ang, nP, geom)
    assert np.array_equal(orc.fp_det(vol, 1000.0, ang, geom, W, H), fp)
    sino = fp.astype(np.float32)
    assert np.array_equal(orc.bp_det(sino, 1000.0, ang, geom, W, H), orc.bp(sino, 1000.0, ang, geom))


def test_detector_half_pitch_samples_the_cylinder_chord(orc):
    """A parallel detector with twice the pixels at half the pitch, along a grid
    axis: each ray sums its interpolated row, so a row of the detector integrates
    (times the pitch) to the slice's mass exactly, and the flat middle of the
    profile is the cylinder's longest chord, as with the full-pitch detector."""
    W, H, r = 40, 4, 15.0
    vol = _cyl(W, H, r, 1.0)
    ang = np.array([0.0], np.float32)
    full = orc.fp(vol, 1000.0, ang, 1, 0)
    half = orc.fp_det(vol, 1000.0, ang, 0, 2 * W, H, du=0.5)
    for iy in range(H):
        np.testing.assert_allclose(0.5 * half[:, iy, 0].sum(), full[:, iy, 0].sum(), rtol=1e-12)
        assert half[:, iy, 0].max() == full[:, iy, 0].max() == _row_counts(W, r).max()


def test_supersampling_averages_sub_rays(orc):
    """ss = 2: each pixel is the mean of four rays at (+-1/4, +-1/4) pixel, i.e. the
    mean of a 2 x 2 finer detector's pixels."""
    from mexct import phantoms

    W, H = 20, 12
    vol = phantoms.ellipsoids(W, count=3, seed=4, nz=H)
    ang = np.array([0.4, 1.9], np.float32)
    for geom in (0, 2):
        ss = orc.fp_det(vol, 1000.0, ang, geom, W, H, ss=2)
        fine = orc.fp_det(vol, 1000.0, ang, geom, 2 * W, 2 * H, du=0.5, dv=0.5)
        coarse = 0.25 * (fine[0::2, 0::2] + fine[1::2, 0::2] + fine[0::2, 1::2] + fine[1::2, 1::2])
        np.testing.assert_allclose(ss, coarse, rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("geom", [0, 1])
def test_taller_detector_rows_outside_the_volume_are_zero(orc, geom):
    """Par / fan rays are parallel to the z planes.  On a detector 4 rows taller
    than the volume (pitch 1) rows 2..H+1 are the volume's own rows, bit for bit,
    and the two rows beyond each end miss the volume and are exactly zero."""
    from mexct import phantoms

    W, H = 20, 12
    vol = phantoms.ellipsoids(W, count=3, seed=6, nz=H)
    vol[:, :, 0] += 1.0  # non-zero edge slices: a clamped sample would show
    vol[:, :, -1] += 1.0
    ang = np.array([0.3, 2.2], np.float32)
    tall = orc.fp_det(vol, 1000.0, ang, geom, W, H + 4)
    assert np.array_equal(tall[:, 2:H + 2], orc.fp(vol, 1000.0, ang, 2, geom))
    assert np.count_nonzero(tall[:, :2]) == 0 and np.count_nonzero(tall[:, H + 2:]) == 0


def test_matched_general3d_bp_is_the_transpose_of_the_fp(orc):
    """The oracle's matched-adjoint general3D BP is the exact transpose of its
    general3D FP: <FP x, y> = <x, BP y> to FP64 rounding, for helix rays that
    cross, graze and miss the volume."""
    from mexct import phantoms

    S, Z = 24, 18
    pts, ang = phantoms.helix_pts(20, 14, 5, Z, sad=60.0, seed=4)
    rng = np.random.default_rng(3)
    x = np.asfortranarray(rng.uniform(0, 1, (S, S, Z)).astype(np.float32))
    y = np.asfortranarray(rng.uniform(-1, 1, (20, 14, 5)).astype(np.float32))
    fx = orc.g3d_fp(x, ang, pts, 5)
    bty = orc.g3d_bp_matched(y, ang, pts, S, Z)
    lhs = float(np.sum(fx * y.astype(np.float64)))
    rhs = float(np.sum(x.astype(np.float64) * bty))
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0)
