"""Sub-volume (z-slab) FP / BP and the out-of-core drivers.

FP of a slab = FP of the volume with every other slice zero (clamp frame kept at
the volume's own faces), checked against the oracle on that masked volume; the
slabs' FPs add up to the whole FP.  BP of a slab from the detector rows
mexct_sub_rows names is the whole BP's slab bit for bit (fixed launch shape: one
view block).  The out-of-core drivers with budgets that force several slabs and
view chunks match the oracle at the 1e-5 bound, and the BP driver, whose view
chunks continue the stored sums, matches the one-launch BP bit for bit.  mexct_sub_rows is checked on
the CPU against every voxel column's taps.
"""
import ctypes

import numpy as np
import pytest

from conftest import rel_l2

TOL = 1e-5
W, H, NP = 24, 20, 11
SLABS = [(0, 7), (7, 6), (13, 7)]


def _ang(n=NP):
    return (np.linspace(0, 2 * np.pi, n, endpoint=False) + 0.2).astype(np.float32)


@pytest.mark.parametrize("geom,sad", [(0, 1000.0), (1, 60.0), (2, 60.0), (2, 1000.0)])
def test_sub_rows_cover_every_tap(lib, geom, sad):
    """Every voxel column of the slab, at every angle, taps rows inside the band."""
    from mexct import ops

    Wl, Hl = 32, 24
    h = Wl // 2 - 1
    ix, iy = np.meshgrid(np.arange(Wl), np.arange(Wl), indexing="ij")
    inside = (ix - h) ** 2 + (iy - h) ** 2 < h * h
    x = (ix - (h + 0.5))[inside].ravel()
    y = (iy - (h + 0.5))[inside].ravel()
    v0 = (Hl - 1) / 2.0
    for z0, nz in [(0, 5), (5, 9), (14, 10), (0, Hl)]:
        r0, nr = ops.sub_rows(Wl, Hl, sad, geom, z0, nz)
        assert 0 <= r0 and r0 + nr <= Hl
        for beta in np.linspace(0, 2 * np.pi, 64, endpoint=False):
            s = x * np.cos(beta) + y * np.sin(beta)
            U = sad / (sad - s) if geom == 2 else np.ones_like(s)
            for z in range(z0, z0 + nz):
                if geom < 2:
                    lo = hi = z
                else:
                    pz = (z - v0) * U + v0 + 0.5
                    taps = np.floor(pz - 0.5)
                    lo = int(np.clip(taps.min(), 0, Hl - 1))
                    hi = int(np.clip(taps.max() + 1, 0, Hl - 1))
                assert r0 <= lo and hi <= r0 + nr - 1, (z0, nz, z, lo, hi, r0, nr)


@pytest.mark.parametrize("W,H,sad", [(200, 160, 300.0), (257, 96, 1000.0)])
def test_sub_rows_cover_every_tap_wide(lib, W, H, sad):
    """The band bound (the reconstruction circle's radius) at larger, odd and
    strongly magnified sizes: every in-circle column's taps, at angles that put
    the circle's edge nearest to and farthest from the source, stay inside."""
    from mexct import ops

    h = W // 2 - 1
    ix, iy = np.meshgrid(np.arange(W), np.arange(W), indexing="ij")
    inside = (ix - h) ** 2 + (iy - h) ** 2 < h * h
    x = (ix - (h + 0.5))[inside].ravel().astype(np.float64)
    y = (iy - (h + 0.5))[inside].ravel().astype(np.float64)
    v0 = (H - 1) / 2.0
    for z0, nz in [(0, 7), (H // 3, 11), (H - 9, 9), (0, H)]:
        r0, nr = ops.sub_rows(W, H, sad, 2, z0, nz)
        assert 0 <= r0 and r0 + nr <= H
        for beta in np.linspace(0, 2 * np.pi, 16, endpoint=False):
            s = x * np.cos(beta) + y * np.sin(beta)
            U = sad / (sad - s)
            for z in (z0, z0 + nz - 1):  # pz is monotonic in z for each column
                taps = np.floor((z - v0) * U + v0)
                lo = int(np.clip(taps.min(), 0, H - 1))
                hi = int(np.clip(taps.max() + 1, 0, H - 1))
                assert r0 <= lo and hi <= r0 + nr - 1, (W, z0, nz, z, lo, hi, r0, nr)


def test_sub_entry_points_validate(lib):
    from mexct import _lib

    r0, nr = ctypes.c_int(), ctypes.c_int()
    assert lib.mexct_sub_rows(8, 8, 1000.0, 2, 6, 3, ctypes.byref(r0),
                              ctypes.byref(nr)) == _lib.ERR_ARG
    buf = np.zeros(64, np.float32)
    p = ctypes.c_void_p(buf.ctypes.data)
    # rows 2..3 do not hold the rows slab 4..5 reads (par: rows 4..5)
    assert lib.mexct_bp_sub_dev(None, p, 2, 2, 8, 8, 1, 1000.0, p, 0, 4, 2, p, 0,
                                None) == _lib.ERR_ARG
    assert "do not hold" in _lib.last_error()
    assert lib.mexct_fp_sub_dev(None, p, 8, 8, 0, 9, 1000.0, p, 1, 0, p, 0, None) == _lib.ERR_ARG


@pytest.fixture(scope="module")
def case(cuda):
    import torch
    from mexct import phantoms

    vol = phantoms.ellipsoids(W, count=4, seed=21, nz=H)
    vol[:, :, 0] += 0.5  # non-zero faces: the clamp frame matters
    vol[:, :, -1] += 0.25
    d = torch.from_numpy(np.ascontiguousarray(vol.transpose(2, 1, 0))).cuda()
    return vol, d


@pytest.mark.gpu
@pytest.mark.parametrize("geom,sad", [(0, 1000.0), (1, 60.0), (2, 60.0), (2, 1000.0)])
def test_fp_slabs_match_oracle_and_add_up(case, orc, geom, sad):
    import torch
    from mexct import _lib, ops

    vol, d = case
    ang = _ang()
    total = None
    for z0, nz in SLABS:
        part = ops.fp_sub_dev(d[z0:z0 + nz].contiguous(), H, z0, sad, ang, geom)
        masked = np.zeros_like(vol)
        masked[:, :, z0:z0 + nz] = vol[:, :, z0:z0 + nz]
        ref = orc.fp(masked, sad, ang, NP, geom)
        torch.cuda.synchronize()
        e = rel_l2(part.cpu().numpy().transpose(2, 1, 0), ref)
        assert e <= TOL, (z0, nz, e)
        total = part if total is None else total + part
    acc = torch.zeros_like(total)
    for z0, nz in SLABS:  # accumulate mode: the same sum in one buffer
        ops.fp_sub_dev(d[z0:z0 + nz].contiguous(), H, z0, sad, ang, geom, out=acc, accumulate=True)
    full = ops.fp_dev(d, sad, ang, geom, variant=_lib.FP_EXPLICIT)
    torch.cuda.synchronize()
    e = (torch.linalg.vector_norm((total - full).double()) /
         torch.linalg.vector_norm(full.double())).item()
    assert e <= 1e-6
    assert torch.equal(acc, total)


@pytest.mark.gpu
@pytest.mark.parametrize("geom,sad", [(0, 1000.0), (1, 60.0), (2, 60.0), (2, 1000.0)])
def test_bp_slabs_are_the_whole_bp(case, orc, geom, sad):
    import torch
    from mexct import ops, tune

    rng = np.random.default_rng(geom)
    sino = np.asfortranarray(rng.uniform(0, 1, (W, H, NP)).astype(np.float32))
    ds = torch.from_numpy(np.ascontiguousarray(sino.transpose(2, 1, 0))).cuda()
    ang = _ang()
    tune.clear()
    tune.set_mode(tune.FIXED)
    try:
        full = ops.bp_dev(ds, sad, ang, geom)
    finally:
        tune.set_mode(tune.HEURISTIC)
    for z0, nz in SLABS:
        r0, nr = ops.sub_rows(W, H, sad, geom, z0, nz)
        slab = ops.bp_sub_dev(ds[:, r0:r0 + nr].contiguous(), r0, H, sad, ang, geom, z0, nz)
        torch.cuda.synchronize()
        assert torch.equal(slab, full[z0:z0 + nz]), (geom, z0, nz)
    ref = orc.bp(sino, sad, ang, geom)
    assert rel_l2(full.cpu().numpy().transpose(2, 1, 0), ref) <= TOL


@pytest.mark.gpu
@pytest.mark.parametrize("geom,sad", [(0, 1000.0), (2, 60.0)])
def test_out_of_core_drivers_match_oracle(cuda, orc, geom, sad):
    from mexct import phantoms
    from mexct import ops

    Wl, Hl, nP = 32, 28, 40
    vol = phantoms.ellipsoids(Wl, count=5, seed=3, nz=Hl)
    ang = _ang(nP)
    # FP: 18 views and 2 slices per pass; BP: 20 views, a few slices
    budget = 8 * Wl * Hl * 4 * 2 + 5 * (Wl * Wl * 4 + 2 * 40 * 34 * 4)
    fp = ops.fp_ooc(vol, sad, ang, geom, budget)
    ref = orc.fp(vol, sad, ang, nP, geom)
    assert rel_l2(fp, ref) <= TOL
    bp = ops.bp_ooc(ref.astype(np.float32), sad, ang, geom, 64 * 1024)
    assert rel_l2(bp, orc.bp(ref.astype(np.float32), sad, ang, geom)) <= TOL
    # view chunks continue the stored sums: bit for bit the one-launch BP
    import torch
    from mexct import tune
    ds = torch.from_numpy(np.ascontiguousarray(ref.astype(np.float32).transpose(2, 1, 0))).cuda()
    tune.clear()
    tune.set_mode(tune.FIXED)
    try:
        full = ops.bp_dev(ds, sad, ang, geom).cpu().numpy().transpose(2, 1, 0)
    finally:
        tune.set_mode(tune.HEURISTIC)
    assert np.array_equal(bp, full)
    # a budget without room for one slice and one view
    from mexct import _lib
    with pytest.raises(_lib.MexctError) as ei:
        ops.fp_ooc(vol, sad, ang, geom, 1024)
    assert ei.value.status == _lib.ERR_BUDGET
