"""Request server: admission by HBM footprint and continuous batching.

CPU (host-only server, simulated requests): requests over the budget are
rejected, admission never exceeds the budget, small requests backfill past a
large one that does not fit yet, and independent requests overlap up to the
slot count.  GPU: every served result equals the same request run alone through
the one-request entry points, bit for bit, while other requests run beside it.
"""
import time

import numpy as np
import pytest


def test_request_rejected_over_budget(lib):
    from mexct import _lib, serve

    s = serve.Server(slots=2, budget_bytes=1000, device=-1)
    with pytest.raises(_lib.MexctError) as ei:
        s.submit_simulated(0.01)  # footprint ~1 MiB > 1000 B
    assert ei.value.status == _lib.ERR_BUDGET
    assert s.stats()["rejected"] == 1
    s.close()


def test_budget_caps_concurrency_and_small_requests_backfill(lib):
    from mexct import serve

    one = serve.Server.request_bytes(0, 64, 64, 60)
    s = serve.Server(slots=4, budget_bytes=2 * one + one // 2, device=-1)
    t0 = time.perf_counter()
    tickets = [s.submit_simulated(0.2) for _ in range(4)]
    res = [s.wait(t)[1] for t in tickets]
    el = time.perf_counter() - t0
    st = s.stats()
    assert st["completed"] == 4 and st["max_concurrent"] == 2
    assert st["peak_bytes"] <= st["budget"]
    assert 0.35 < el < 1.5  # two waves of two
    assert min(r["queue_s"] for r in res) < 0.05 and max(r["queue_s"] for r in res) > 0.15
    s.close()


def test_osctv_footprint_counts_the_largest_subset(lib):
    """An OSC-TV request is charged its residual views for the largest subset
    only (two padded quad-layout views per subset view), in FP32 or FP16, next to
    its volumes and counts."""
    from mexct import _lib, serve

    W, H, nP = 512, 512, 720
    b1 = serve.Server.request_bytes(1, W, H, nP, n_sub=1)
    b10 = serve.Server.request_bytes(1, W, H, nP, n_sub=10)
    b10h = serve.Server.request_bytes(1, W, H, nP, n_sub=10, data_type=_lib.F16)
    quad = 4 * (W + 4) * (H + 4)  # values per padded view
    assert b1 - b10 == 2 * quad * 4 * (720 - 72)
    assert b10 - b10h == 2 * quad * 2 * 72
    vol, counts = 4 * W * W * H, 4 * W * H * nP
    assert b10h > 4 * counts + vol  # staging and solver copies of pre / post, and mu


def test_slots_overlap_independent_requests(lib):
    from mexct import serve

    s = serve.Server(slots=4, budget_bytes=1 << 40, device=-1)
    t0 = time.perf_counter()
    ts = [s.submit_simulated(0.3) for _ in range(4)]
    for t in ts:
        s.wait(t)
    assert time.perf_counter() - t0 < 0.9  # the four ran together
    assert s.stats()["max_concurrent"] == 4
    s.close()


def test_small_request_backfills_past_large(lib):
    from mexct import serve

    big = serve.Server.request_bytes(0, 512, 512, 720)
    small = serve.Server.request_bytes(0, 64, 64, 60)
    s = serve.Server(slots=2, budget_bytes=big + small, device=-1)
    a = s.submit_simulated(0.3, W=512, H=512, nP=720)
    b = s.submit_simulated(0.3, W=512, H=512, nP=720)  # does not fit next to a
    c = s.submit_simulated(0.05)                      # fits next to a: runs before b
    rc = s.wait(c)[1]
    rb = s.wait(b)[1]
    s.wait(a)
    assert rc["total_s"] < rb["queue_s"]
    s.close()


@pytest.mark.gpu
def test_served_results_equal_alone(cuda):
    import mexct
    from mexct import phantoms, serve, solver

    import oracle

    rng = np.random.default_rng(0)
    reqs = []
    for i in range(6):
        W = int(rng.choice([32, 48]))
        nP = int(rng.integers(12, 30))
        geom = int(rng.integers(0, 3))
        vol = phantoms.ellipsoids(W, count=3, seed=i, nz=W)
        ang = phantoms.angles_full(nP)
        fp = oracle.fp(vol, 1000.0, ang, nP, geom).astype(np.float32)
        pre, post = phantoms.poisson_counts(fp, 1e5, seed=i)
        kind = i % 2
        reqs.append((kind, pre, post, ang, geom, rng.integers(0, 4, 3)))
    s = serve.Server(slots=3, budget_bytes=8 << 30)
    # a 0.5 s host-side request holds one slot, so real requests overlap it
    hold = s.submit_simulated(0.5)
    tickets = []
    for kind, pre, post, ang, geom, picks in reqs:
        if kind == 0:
            tickets.append(s.submit_fdk(pre, post, ang, geom))
        else:
            tickets.append(s.submit_osctv(pre, post, ang, geom, picks, n_iter=3, n_sub=4))
    served = [s.wait(t)[0] for t in tickets]
    s.wait(hold)
    assert s.stats()["max_concurrent"] >= 2
    s.close()
    gs = {0: "par3d", 1: "fan3d", 2: "cone3d"}
    for (kind, pre, post, ang, geom, picks), got in zip(reqs, served):
        if kind == 0:
            alone = mexct.FBP_recon(pre, post, ang, {"type": gs[geom], "SAD": 1000.0}, "hamming", 1.0, 1.0)
        else:
            alone = solver.OSC_TV_recon(pre, post, ang, {"type": gs[geom], "SAD": 1000.0}, 3, 0.2,
                                        4, 4, 1.0, picks)
        assert np.array_equal(got, alone)
