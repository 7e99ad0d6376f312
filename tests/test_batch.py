"""Batched persistent FP/BP over uneven problems: each problem's result is
bit-identical to the single-problem entry points (same tile / brick code), and
the batch replays correctly from a captured CUDA graph."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problems(seed=0, count=6):
    import torch
    from mexct import phantoms

    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        W = int(rng.choice([24, 40, 64, 96]))
        H = int(rng.choice([16, 32, 48]))
        nP = int(rng.integers(5, 40))
        geom = int(rng.integers(0, 3))
        vol = phantoms.ellipsoids(W, count=3, seed=seed * 100 + i, nz=H)
        ang = np.sort(rng.uniform(0, 2 * np.pi, nP)).astype(np.float32)
        d = torch.from_numpy(np.ascontiguousarray(vol.transpose(2, 1, 0))).cuda()
        out.append({"vol": d, "sino": torch.zeros((nP, H, W), device="cuda"),
                    "rec": torch.zeros((H, W, W), device="cuda"), "angles": ang,
                    "sad": 1000.0, "geom": geom})
    return out


def test_batch_equals_single_problem_calls(cuda):
    import torch
    from mexct import batch, ops

    from mexct import tune

    probs = _problems(1)
    b = batch.Batch(probs)
    b.fp()
    b.bp()
    torch.cuda.synchronize()
    # the batch runs the fixed shapes (slab FP, BP without view blocks)
    tune.clear()
    tune.set_mode(tune.FIXED)
    try:
        for p in probs:
            s = ops.fp_dev(p["vol"], p["sad"], p["angles"], p["geom"])
            r = ops.bp_dev(s, p["sad"], p["angles"], p["geom"])
            torch.cuda.synchronize()
            assert torch.equal(s, p["sino"])
            assert torch.equal(r, p["rec"])
    finally:
        tune.set_mode(tune.HEURISTIC)
    b.close()


def test_batch_graph_replay(cuda):
    import torch
    from mexct import batch

    probs = _problems(2, count=4)
    b = batch.Batch(probs)
    st = torch.cuda.Stream()
    b.fp(st)
    b.bp(st)
    st.synchronize()
    ref = [(p["sino"].clone(), p["rec"].clone()) for p in probs]
    for p in probs:
        p["sino"].zero_()
        p["rec"].zero_()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=st):
        b.fp(st)
        b.bp(st)
    g.replay()
    torch.cuda.synchronize()
    for p, (s, r) in zip(probs, ref):
        assert torch.equal(p["sino"], s) and torch.equal(p["rec"], r)
    b.close()


@pytest.mark.parametrize("geom", [0, 1, 2])
def test_paired_views_equal_single_view_tiles(cuda, geom):
    """Views 1 degree apart at W = 64 are close enough for the slab FP to take two
    per CTA (one box serves both bundles); per ray the arithmetic is that of one
    view, so the result equals the batched kernel's (one view per CTA) bit for
    bit -- with an odd view count (the last CTA has one view) and pairs on both
    sides of 45 and 135 degrees (views that sweep different axes run one at a
    time in their CTA)."""
    import torch
    from mexct import batch, ops, phantoms, tune

    W, H = 64, 40
    ang = np.deg2rad(40.0 + np.arange(101, dtype=np.float64)).astype(np.float32)
    vol = phantoms.ellipsoids(W, count=4, seed=31 + geom, nz=H)
    d = torch.from_numpy(np.ascontiguousarray(vol.transpose(2, 1, 0))).cuda()
    p = {"vol": d, "sino": torch.zeros((len(ang), H, W), device="cuda"),
         "rec": torch.zeros((H, W, W), device="cuda"), "angles": ang, "sad": 1000.0,
         "geom": geom}
    b = batch.Batch([p])
    b.fp()
    torch.cuda.synchronize()
    tune.clear()
    tune.set_mode(tune.FIXED)
    try:
        s = ops.fp_dev(d, 1000.0, ang, geom)
        torch.cuda.synchronize()
        assert torch.equal(s, p["sino"])
    finally:
        tune.set_mode(tune.HEURISTIC)
    b.close()
