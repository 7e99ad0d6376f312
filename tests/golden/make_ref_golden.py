"""Generate tests/golden/ref_golden.npz: outputs of the reference's OWN CUDA kernels.

The reference ships no tests or golden vectors.  This script runs its kernels,
compiled unmodified from its .cu files into sm_103a cubins (oracle/ref_build.py,
where the reference sources are present) and launched by the restated gateway
host code of oracle/ref_launch.cu, on a GPU.  The fixture it writes pins the FP64
oracle and the CUDA library to real reference outputs
(tests/test_ref_pin.py).

Cases (inputs are stored beside the outputs; every input is seeded):
  * the inputs of tests/golden/golden.npz: FP and BP for geomFlag 0/1/2, one OSC
    iteration per geometry, general3D FP/BP on helix rays, 20 TV steps;
  * a 40 x 40 x 32 ellipsoid volume with 20 views: FP and BP per geometry;
  * a 48 x 48 x 36 volume with 64 x 40 helix rays over 12 views: general3D FP/BP,
    and 20 TV steps on a noisy 48 x 48 x 36 volume.

Run on a machine with a GPU, from the repository root:
    python tests/golden/make_ref_golden.py [output.npz]
(default output: tests/golden/ref_golden.npz).
"""
import os
import platform
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "mex-cuda-ct_gb300"), os.path.dirname(HERE)]

from golden import make_golden  # noqa: E402
from mexct import phantoms  # noqa: E402
from oracle import reference as ref  # noqa: E402

SAD = 1000.0


def inputs():
    x, y = make_golden.load()
    small = {k: x[k] for k in ("vol", "ang", "sino", "pts", "hang", "hsino", "pre", "post", "mu0", "tvin")}
    small["order5_1"] = y["order5_1"].astype(np.int32)  # the subset order of the golden OSC cases
    rng = np.random.default_rng(2024)
    W, H, nP = 40, 32, 20
    med = {
        "vol": phantoms.ellipsoids(W, count=8, seed=21, nz=H),
        "ang": phantoms.angles_full(nP),
        "sino": np.asfortranarray(rng.uniform(0.0, 3.0, (W, H, nP)).astype(np.float32)),
    }
    S, Z = 48, 36
    pts, hang = phantoms.helix_pts(64, 40, 12, Z, sad=200.0, seed=8)
    tv = phantoms.ellipsoids(S, count=6, seed=5, nz=Z)
    gen = {
        "vol": phantoms.ellipsoids(S, count=6, seed=6, nz=Z),
        "pts": pts, "hang": hang,
        "hsino": np.asfortranarray(rng.uniform(0.0, 1.0, (64, 40, 12)).astype(np.float32)),
        "tvin": np.asfortranarray(tv + rng.normal(0, 3e-3, tv.shape).astype(np.float32)),
    }
    return {"s": small, "m": med, "g": gen}


def g3d_fp_views(vol, hang, pts):
    """general3D FP with one point set per view ([W,H,6,nP]): one nP = 1 call
    per view through the reference's shared-points interface."""
    return np.concatenate([ref.g3d_fp(vol, hang[j:j + 1], pts[..., j], 1) for j in range(len(hang))], axis=2)


def g3d_bp_views(sino, hang, pts, S, Z):
    """general3D BP with one point set per view: per-view calls, summed."""
    acc = np.zeros((S, S, Z), dtype=np.float64, order="F")
    for j in range(len(hang)):
        acc += ref.g3d_bp(sino[..., j:j + 1], hang[j:j + 1], pts[..., j], S, Z)
    return acc


def outputs(x):
    s, m, g = x["s"], x["m"], x["g"]
    out = {}
    for geom in (0, 1, 2):
        out["s_fp%d" % geom] = ref.fp(s["vol"], SAD, s["ang"], len(s["ang"]), geom)
        out["s_bp%d" % geom] = ref.bp(s["sino"], SAD, s["ang"], geom)
        mu, pre, post = ref.osc_iter(s["mu0"], s["pre"], s["post"], 5, s["order5_1"], s["ang"], SAD, geom)
        out["s_osc%d" % geom] = mu
        out["s_oscpre%d" % geom] = pre
        out["s_oscpost%d" % geom] = post
        out["m_fp%d" % geom] = ref.fp(m["vol"], SAD, m["ang"], len(m["ang"]), geom)
        out["m_bp%d" % geom] = ref.bp(m["sino"], SAD, m["ang"], geom)
    W, H = s["vol"].shape[0], s["vol"].shape[2]
    out["s_g3dfp"] = g3d_fp_views(s["vol"], s["hang"], s["pts"])
    out["s_g3dbp"] = g3d_bp_views(s["hsino"], s["hang"], s["pts"], W, H)
    out["s_tv"] = ref.tvmin3d(s["tvin"], 0.02)
    S, Z = g["vol"].shape[0], g["vol"].shape[2]
    out["g_g3dfp"] = g3d_fp_views(g["vol"], g["hang"], g["pts"])
    out["g_g3dbp"] = g3d_bp_views(g["hsino"], g["hang"], g["pts"], S, Z)
    out["g_tv"] = ref.tvmin3d(g["tvin"], 0.05)
    return out


def _gpu_name():
    try:
        return subprocess.run(["nvidia-smi", "--query-gpu=name", "--format=csv,noheader"],
                              capture_output=True, text=True).stdout.strip().splitlines()[0]
    except Exception:  # noqa: BLE001
        return "unknown"


def load(path=None):
    """(inputs, outputs, meta) from the committed fixture."""
    z = np.load(path or os.path.join(HERE, "ref_golden.npz"))
    x = {"s": {}, "m": {}, "g": {}}
    y, meta = {}, {}
    for k in z.files:
        if k.startswith("in_"):
            grp, name = k[3:].split("_", 1)
            v = z[k]
            x[grp][name] = np.asfortranarray(v) if v.ndim >= 2 else v
        elif k.startswith("out_"):
            y[k[4:]] = np.asfortranarray(z[k]) if z[k].ndim >= 2 else z[k]
        elif k.startswith("meta_"):
            meta[k[5:]] = str(z[k])
    return x, y, meta


if __name__ == "__main__":
    dst = sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "ref_golden.npz")
    x = inputs()
    y = outputs(x)
    blob = {}
    for grp, d in x.items():
        for k, v in d.items():
            blob["in_%s_%s" % (grp, k)] = np.asarray(v)
    blob.update({"out_" + k: np.asarray(v, dtype=np.float32) for k, v in y.items()})
    blob["meta_gpu"] = np.array(_gpu_name())
    blob["meta_host"] = np.array(platform.machine())
    blob["meta_kernels"] = np.array("reference .cu files compiled unmodified (nvcc -cubin -O3, sm_103a) "
                                    "with oracle/ref_compat.h; host steps restated in oracle/ref_launch.cu")
    np.savez_compressed(dst, **blob)
    print("wrote", dst, "%.1f KB" % (os.path.getsize(dst) / 1024))
