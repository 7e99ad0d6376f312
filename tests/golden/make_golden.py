"""Generate the golden vectors in tests/golden/golden.npz from the FP64 oracle.

The reference ships no golden vectors (it has no tests); these fixtures are made by
this project's oracle on small seeded inputs and committed, so that (a) any change to
the oracle shows up as a CPU test failure and (b) the GPU tests can check the CUDA
path against fixed numbers that do not depend on the oracle build.

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "mex-cuda-ct_gb300")]

import oracle  # noqa: E402
from mexct import phantoms  # noqa: E402


def inputs():
    """Seeded inputs shared by the generator and the tests."""
    W, H, nP = 20, 14, 10
    vol = phantoms.ellipsoids(W, count=4, seed=11, nz=H)
    ang = phantoms.angles_full(nP)
    rng = np.random.default_rng(5)
    sino = np.asfortranarray(rng.uniform(-0.5, 2.0, (W, H, nP)).astype(np.float32))
    pts, hang = phantoms.helix_pts(12, 10, 6, H, sad=120.0, seed=3)
    hsino = np.asfortranarray(rng.uniform(0.0, 1.0, (12, 10, 6)).astype(np.float32))
    fp2 = oracle.fp(vol, 1000.0, ang, nP, 2).astype(np.float32)
    pre, post = phantoms.poisson_counts(fp2, 1e5, seed=9)
    mu0 = np.full((W, W, H), np.float32(1e-10), dtype=np.float32, order="F")
    tvin = np.asfortranarray(vol + rng.normal(0, 2e-3, vol.shape).astype(np.float32))
    sq = np.asfortranarray(rng.uniform(0, 1, (16, 16, 8)).astype(np.float32))
    sqa = phantoms.angles_full(8)
    return dict(W=W, H=H, nP=nP, vol=vol, ang=ang, sino=sino, pts=pts, hang=hang, hsino=hsino,
                pre=pre, post=post, mu0=mu0, tvin=tvin, sq=sq, sqa=sqa)


def outputs(x):
    out = {}
    for g in (0, 1, 2):
        out["fp%d" % g] = oracle.fp(x["vol"], 1000.0, x["ang"], x["nP"], g)
        out["bp%d" % g] = oracle.bp(x["sino"], 1000.0, x["ang"], g)
        out["osc%d" % g] = oracle.osc_iter(x["mu0"], x["pre"], x["post"], 5,
                                           oracle.subset_order(5, 1), x["ang"], 1000.0, g)
        out["pf%d" % g] = oracle.prefilter(x["sq"], g, x["sqa"], "hamming", 1.0, 1.0, sad=1000.0)
    out["g3dfp"] = oracle.g3d_fp(x["vol"], x["hang"], x["pts"], 6)
    out["g3dbp"] = oracle.g3d_bp(x["hsino"], x["hang"], x["pts"], x["W"], x["H"])
    out["tv"] = oracle.tvmin3d(x["tvin"], 0.02, 20)
    out["order10_3"] = oracle.subset_order(10, 3).astype(np.int64)
    out["order5_1"] = oracle.subset_order(5, 1).astype(np.int64)
    return out


def load():
    """(inputs, outputs) from the committed fixture; inputs are stored too, so no
    platform regenerates them (phantom rasterisation is float arithmetic)."""
    z = np.load(os.path.join(HERE, "golden.npz"))
    x = {k[3:]: z[k] for k in z.files if k.startswith("in_")}
    for k in ("W", "H", "nP"):
        x[k] = int(x[k])
    for k, v in list(x.items()):
        if isinstance(v, np.ndarray) and v.ndim >= 2:
            x[k] = np.asfortranarray(v)
    y = {k[4:]: z[k] for k in z.files if k.startswith("out_")}
    return x, y


if __name__ == "__main__":
    oracle.build()
    x = inputs()
    res = outputs(x)
    blob = {"in_" + k: np.asarray(v) for k, v in x.items()}
    blob.update({"out_" + k: v for k, v in res.items()})
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **blob)
    print("wrote", os.path.join(HERE, "golden.npz"), sorted(blob))
