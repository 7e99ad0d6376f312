"""Launch shapes and autotuning (mexct.tune): every BP launch shape and both exact FP
variants meet the 1e-5 parity bound against the FP64 oracle; shapes without view
blocks are bit-identical to each other; the autotuner records a timed choice that
later calls of the class use."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _sino(W, H, nP, seed):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.uniform(-1, 2, (W, H, nP)).astype(np.float32))


@pytest.fixture
def fresh_table(cuda):
    from mexct import tune

    tune.clear()
    tune.set_mode(tune.HEURISTIC)
    yield tune
    tune.clear()
    tune.set_mode(tune.HEURISTIC)


@pytest.mark.parametrize("geom", [0, 2])
def test_every_bp_shape_matches_oracle(fresh_table, orc, geom):
    import torch
    from mexct import ops, phantoms

    tune = fresh_table
    W, H, nP = 40, 36, 24
    sino = _sino(W, H, nP, geom)
    ang = phantoms.angles_full(nP)
    ref = orc.bp(sino, 1000.0, ang, geom)
    d = torch.from_numpy(np.ascontiguousarray(sino.transpose(2, 1, 0))).cuda()
    base = None
    for zc in (8, 16):
        for rows in (4, 8):
            for vb in (1, 2, 3, 8):
                tune.shape_set(tune.BP, geom, W, H, nP, zc=zc, rows=rows, vblocks=vb)
                got = ops.bp_dev(d, 1000.0, ang, geom)
                torch.cuda.synchronize()
                assert rel_l2(got.cpu().numpy().transpose(2, 1, 0), ref) <= TOL, (zc, rows, vb)
                if vb == 1:
                    # one view block: the same operations in the same order per voxel
                    if base is None:
                        base = got.clone()
                    assert torch.equal(got, base), (zc, rows)


def test_fp_auto_uses_the_pinned_variant(fresh_table, orc):
    import torch
    from mexct import _lib, ops, phantoms

    tune = fresh_table
    W, H, nP = 48, 40, 16
    vol = phantoms.ellipsoids(W, count=5, seed=4, nz=H)
    ang = phantoms.angles_full(nP)
    d = torch.from_numpy(np.ascontiguousarray(vol.transpose(2, 1, 0))).cuda()
    ray = ops.fp_dev(d, 1000.0, ang, 2, variant=_lib.FP_RAY)
    tune.shape_set(tune.FP, 2, W, H, nP, variant=_lib.FP_RAY)
    auto = ops.fp_dev(d, 1000.0, ang, 2)
    torch.cuda.synchronize()
    assert torch.equal(auto, ray)
    assert tune.shape_get(tune.FP, 2, W, H, nP)["tuned"] == 0
    ref = orc.fp(vol, 1000.0, ang, nP, 2)
    assert rel_l2(auto.cpu().numpy().transpose(2, 1, 0), ref) <= TOL


def test_autotune_records_a_timed_shape(fresh_table, orc):
    import torch
    from mexct import ops, phantoms

    tune = fresh_table
    W, H, nP = 64, 48, 40
    sino = _sino(W, H, nP, 7)
    ang = phantoms.angles_full(nP)
    d = torch.from_numpy(np.ascontiguousarray(sino.transpose(2, 1, 0))).cuda()
    assert tune.shape_get(tune.BP, 2, W, H, nP)["tuned"] == -1
    tune.set_mode(tune.AUTO)
    got = ops.bp_dev(d, 1000.0, ang, 2)
    torch.cuda.synchronize()
    entry = tune.shape_get(tune.BP, 2, W, H, nP)
    print("tuned BP shape for 64x64x48, 40 views:", entry)
    assert entry["tuned"] == 1 and np.isfinite(entry["ms"]) and entry["ms"] > 0
    assert rel_l2(got.cpu().numpy().transpose(2, 1, 0), orc.bp(sino, 1000.0, ang, 2)) <= TOL
    # the explicit tuner returns the result of its best shape
    out, shape, ms = tune.autotune_bp(d, 1000.0, ang, 2)
    torch.cuda.synchronize()
    assert shape["vblocks"] >= 1 and ms > 0
    assert rel_l2(out.cpu().numpy().transpose(2, 1, 0), orc.bp(sino, 1000.0, ang, 2)) <= TOL
    vol = torch.rand((H, W, W), device="cuda")
    s2, fshape, fms = tune.autotune_fp(vol, 1000.0, ang, 0)
    torch.cuda.synchronize()
    assert fshape["variant"] in (0, 2) and fms > 0
    assert tune.shape_get(tune.FP, 0, W, H, nP)["tuned"] == 1


def test_shape_set_rejects_bad_shapes(fresh_table):
    from mexct import _lib

    tune = fresh_table
    for kw in (dict(zc=4), dict(rows=16), dict(vblocks=0), dict(vblocks=65)):
        with pytest.raises(_lib.MexctError):
            tune.shape_set(tune.BP, 0, 32, 32, 10, **kw)
    with pytest.raises(_lib.MexctError):
        tune.shape_set(tune.FP, 0, 32, 32, 10, variant=_lib.FP_TEXTURE)
