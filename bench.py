"""Benchmark of the mex-cuda-CT projection-operator path on one GB300.

Headline step: one cone-beam (geomFlag 2) forward projection of a 512^3 float32
random-ellipsoid phantom over 720 views (SAD 1000) plus one backprojection of
that sinogram, through the C ABI of libmexct, plain FP32 form (explicit FP32
trilinear, the 1e-5 parity path).

  value   whole-job GUPS = 2 * 512^3 * 720 * steps * ranks / max-rank time,
          device-resident inputs, CUDA events on the launching stream
  e2e     the same metric through the host entry points mexct_fp / mexct_bp with
          pinned host buffers (H2D and D2H inside the timed region)
  extra   FP/BP GUPS for geomFlag 0 and 1; the chosen forms (hardware-texture FP,
          FP16 storage) with their relative L2 to the plain FP32 result; OSC-TV
          p50/p99 seconds per reconstruction (256^3, 60 views, 20 iterations x 10
          subsets) plain (FP32, eager launches) vs chosen (CUDA graphs); the
          reference's own kernels on the same GPU; the FP64 C++/OpenMP CPU
          implementation on a bounded sample (cpu_baseline).

--impl reference times the reference's own implementation of the step: its CUDA
kernels, compiled unmodified from its .cu files into oracle/_ref (the reference has
no CPU path), launched per view by the host steps of its MEX gateways restated in
oracle/ref_launch.cu, with host arrays in and out as the gateways take them.  Where
those cubins are absent it falls back to the FP64 CPU restatement (the oracle).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Multi-GPU: one process per GPU (torchrun); every rank runs its own full problem
(replicas: the path is independent per problem); value aggregates all ranks.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "mex-cuda-ct_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
# DRAM bytes (read + write) per view of the slab FP kernel, cone 512^3 x 720 views:
# one single-pass ncu capture of the whole 720-view launch (dram__bytes_read.sum +
# dram__bytes_write.sum = 14.92 GB + 0.761 GB), per view.  Fewer views per launch
# reuse less of each tile's bundle from L2 (64 views: 185 MB per view).
FP_SLAB_DRAM_BYTES_PER_VIEW = (14.92e9 + 0.76112e9) / 720


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=512)
    ap.add_argument("--views", type=int, default=720)
    ap.add_argument("--geom", type=int, default=2)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true")
    ap.add_argument("--osc-reps", type=int, default=5)
    ap.add_argument("--batch-problems", type=int, default=48)
    ap.add_argument("--serve-requests", type=int, default=60)
    ap.add_argument("--cpu-configs", action="store_true",
                    help="time the FP64 oracle at the cylinder / ellipsoid / OSC-TV workloads "
                         "(minutes of host time) beside the library's host entry points")
    ap.add_argument("--config5", action="store_true",
                    help="run only the serving workload at its stated mix (minutes of GPU time)")
    ap.add_argument("--ops-once", action="store_true",
                    help="run one call of each secondary operator on 256^3 and exit "
                         "(the workload of the secondary-kernel profiles)")
    return ap.parse_args()


def hbm_peak():
    try:
        with open(PEAKS) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


_phantom_cache = {}


def cpu_sample(size, views, geom, seconds_target=15.0):
    """Time the FP64 oracle (FP + BP) on a bounded view sample; returns GUPS."""
    import oracle
    from mexct import phantoms

    oracle.build()
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    n = size
    vol = _phantom_cache.get(n)
    if vol is None:
        vol = _phantom_cache[n] = phantoms.ellipsoids(n, count=12, seed=2024, nz=n)
    ang_all = phantoms.angles_full(views)
    k, used = 1, 0.0
    while True:
        ang = ang_all[::max(1, views // k)][:k]
        t0 = time.perf_counter()
        sino = oracle.fp(vol, 1000.0, ang, k, geom).astype(np.float32)
        oracle.bp(sino, 1000.0, ang, geom)
        dt = time.perf_counter() - t0
        used += dt
        gups = 2.0 * n ** 3 * k / dt / 1e9
        if used + 2.2 * dt > seconds_target or k >= views:
            break
        k = min(views, k * 2)
    return {"value": round(gups, 4), "unit": "GUPS", "cores": threads, "kind": "port",
            "sample": "%d^3 volume, FP+BP over %d of %d views, geomFlag %d (FP64 C++/OpenMP "
                      "restatement of the reference, %d threads)" % (n, k, views, geom, threads)}


def cpu_configs():
    """The FP64 oracle (the CPU baseline) at the cylinder, ellipsoid and few-view
    OSC-TV workloads at full size on all host cores, beside the library's host entry
    points on the same inputs (host arrays in and out).  Opt-in: bench.py
    --cpu-configs (minutes of host time)."""
    import mexct
    import oracle
    from mexct import phantoms, solver

    oracle.build()
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    out = {"cores": threads}

    def timed(fn):
        t = time.perf_counter()
        r = fn()
        return r, time.perf_counter() - t

    # cylinder 128^3, 256 cone views: FP, then BP of that FP
    vol = phantoms.cylinder(128)
    ang = np.linspace(0, 2 * np.pi, 256).astype(np.float32)
    sino, t_cf = timed(lambda: oracle.fp(vol, 1000.0, ang, 256, 2).astype(np.float32))
    _, t_cb = timed(lambda: oracle.bp(sino, 1000.0, ang, 2))
    mexct.CUDAmex_FP(vol, 1000.0, ang, 256, 2)  # warm-up
    gs, t_gf = timed(lambda: mexct.CUDAmex_FP(vol, 1000.0, ang, 256, 2))
    _, t_gb = timed(lambda: mexct.CUDAmex_BP(gs, 1000.0, ang, 2))
    out["cylinder_128_cone_256views"] = {"cpu_s": round(t_cf + t_cb, 3),
                                         "gpu_host_calls_s": round(t_gf + t_gb, 4)}
    # ellipsoids 384^3, 512 views: FP, Hamming FDK (pre-filter + BP) per geometry
    vol = phantoms.ellipsoids(384, count=12, seed=2)
    ang = phantoms.angles_full(512)
    for geom in (0, 1, 2):
        g = {"type": ["par3d", "fan3d", "cone3d"][geom], "SAD": 1000.0}
        sino, t_cf = timed(lambda: oracle.fp(vol, 1000.0, ang, 512, geom).astype(np.float32))
        filt, t_cp = timed(lambda: oracle.prefilter(sino, geom, ang, "hamming", 1.0, 1.0).astype(np.float32))
        _, t_cb = timed(lambda: oracle.bp(filt, 1000.0, ang, geom))
        gs, t_gf = timed(lambda: mexct.CUDAmex_FP(vol, 1000.0, ang, 512, geom))
        gfl, t_gp = timed(lambda: mexct.preFilterSinogram(gs, g, ang, "hamming", 1.0, 1.0))
        _, t_gb = timed(lambda: mexct.CUDAmex_BP(gfl, 1000.0, ang, geom))
        out["ellipsoid_384_512views_geom%d" % geom] = {
            "cpu_fp_s": round(t_cf, 2), "cpu_fdk_s": round(t_cp + t_cb, 2),
            "gpu_host_calls_fp_s": round(t_gf, 4), "gpu_host_calls_fdk_s": round(t_gp + t_gb, 4)}
    # few-view OSC-TV: 256^3, 60 cone views, 20 iterations x 10 subsets
    vol = phantoms.ellipsoids(256, count=10, seed=7)
    ang = phantoms.angles_full(60)
    fp = mexct.CUDAmex_FP(vol, 1000.0, ang, 60, 2).astype(np.float64)
    rng = np.random.default_rng(11)
    post = np.asfortranarray(rng.poisson(1e5 * np.exp(-fp)).astype(np.float32))
    pre = np.full(post.shape, 1e5, dtype=np.float32, order="F")
    picks = rng.integers(0, 10, 20).astype(np.int32)
    _, t_c = timed(lambda: oracle.osc_tv(pre, post, ang, 1000.0, 2, 20, 0.2, 10, 10, 1.0, picks))
    g = {"type": "cone3d", "SAD": 1000.0}
    solver.OSC_TV_recon(pre, post, ang, g, 1, 0.2, 10, 10, 1.0, picks[:1])  # warm-up
    _, t_g = timed(lambda: solver.OSC_TV_recon(pre, post, ang, g, 20, 0.2, 10, 10, 1.0, picks))
    out["osc_tv_256_60views_20x10"] = {"cpu_s": round(t_c, 2), "gpu_host_call_s": round(t_g, 4)}
    return out


def metric_name(args):
    return "FP+BP GUPS at %d^3 x %d views (cone geomFlag %d), plain FP32" % (
        args.size, args.views, args.geom)


def workload_config(args, world=1):
    return {"workload": "cone FP+BP %d^3 x %d views, SAD 1000, float32" % (args.size, args.views),
            "l2": "inputs larger than L2 (volume %d MiB, sinogram %d MiB)"
                  % (4 * args.size ** 3 >> 20, 4 * args.size ** 2 * args.views >> 20),
            "parallelism": "replicas" if world > 1 else "single"}


def reference_step_times(vol, ang, geom, reps):
    """Host wall time of the reference's own FP then BP (its kernels from oracle/_ref,
    per view, with its gateways' copies and synchronisations), per call."""
    from oracle import reference

    fps, bps = [], []
    sino = None
    for _ in range(reps):
        t = time.perf_counter()
        sino = reference.fp(vol, 1000.0, ang, len(ang), geom)
        fps.append(time.perf_counter() - t)
        t = time.perf_counter()
        reference.bp(sino, 1000.0, ang, geom)
        bps.append(time.perf_counter() - t)
    return fps, bps


def run_reference(args, rank):
    """The reference's own implementation of the step on the same GPU: rank 0 only
    (the other ranks exit without work).  Falls back to the FP64 CPU restatement
    when the reference's cubins are absent."""
    if rank != 0:
        return
    from mexct import phantoms
    from oracle import reference

    n, views, geom = args.size, args.views, args.geom
    if not reference.available():
        return run_reference_cpu(args)
    vol = phantoms.ellipsoids(n, count=12, seed=2024, nz=n)
    ang = phantoms.angles_full(views)
    reference_step_times(vol, ang, geom, max(args.warmup, 1))
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    t = time.perf_counter()
    fps, bps = reference_step_times(vol, ang, geom, max(args.steps, 1))
    el = time.perf_counter() - t
    clk = clocks.stop()
    k = max(args.steps, 1)
    gups = 2.0 * n ** 3 * views * k / el / 1e9
    N, P = n ** 3, n * n
    line = {"metric": metric_name(args), "value": round(gups, 3), "unit": "GUPS",
            "n_gpus": args.gpus, "steps": k, "warmup": args.warmup,
            "ms_per_step": round(el / k * 1e3, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded 12-ellipsoid phantom)", "impl": "reference",
            "config": workload_config(args),
            "fp_ms": round(float(np.median(fps)) * 1e3, 1),
            "bp_ms": round(float(np.median(bps)) * 1e3, 1),
            "clocks": clk,
            "cpu_baseline": {"value": round(gups, 3), "unit": "GUPS", "cores": 1, "kind": "reference",
                             "sample": "the full step (FP then BP of all %d views at %d^3): the "
                                       "reference's CUDA kernels compiled unmodified for sm_103a, "
                                       "one launch + synchronisation + host copy per view as its "
                                       "gateways do, driven by one host thread (the reference "
                                       "has no CPU path)" % (views, n)},
            "e2e": {"value": round(gups, 3), "unit": "GUPS",
                    "h2d_bytes_per_step": 4 * (N + P * views), "d2h_bytes_per_step": 4 * (P * views + N),
                    "path": "host arrays in and out, as the MEX gateways take them"}}
    print(json.dumps(line), flush=True)


def run_reference_cpu(args):
    """The FP64 C++/OpenMP restatement on the host cores, each step a bounded sample
    (FP+BP over a few of the views), when the reference's kernels are not built."""
    cpu_sample(min(args.size, 64), 4, args.geom, seconds_target=0.5)  # warm-up (threads, pages)
    per_step = max(5.0, 60.0 / max(args.steps, 1))
    t = time.perf_counter()
    samples = [cpu_sample(args.size, args.views, args.geom, seconds_target=per_step)
               for _ in range(max(args.steps, 1))]
    el = time.perf_counter() - t
    value = float(np.mean([x["value"] for x in samples]))
    s = dict(samples[-1])
    s["value"] = round(value, 4)
    line = {"metric": metric_name(args), "value": s["value"], "unit": "GUPS",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(el / max(args.steps, 1) * 1e3, 1),
            "ms_per_step_note": "time of each step's bounded sample, not of a full step",
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded 12-ellipsoid phantom)", "impl": "reference",
            "config": workload_config(args), "cpu_baseline": s,
            "e2e": {"value": s["value"], "unit": "GUPS", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def max_over_ranks(x, dist, device):
    """The largest of every rank's x (x itself with one rank): replicas are timed
    by the slowest one."""
    if dist is None:
        return x
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rel(a, b):
    import torch

    a = a.double()
    b = b.double()
    return float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return

    import torch

    import __graft_entry__ as ge

    ge._builder().build()
    from mexct import _lib, ops, phantoms

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    lib = _lib.load()
    V = ctypes.c_void_p
    if args.ops_once:
        ops_once()
        return
    if args.config5:
        if rank == 0:
            config5(args)
        return
    if args.cpu_configs:
        if rank == 0:
            print(json.dumps({"cpu_configs": cpu_configs()}), flush=True)
        return

    n, views, geom = args.size, args.views, args.geom
    N = n * n * n
    P = n * n
    vol_h = phantoms.ellipsoids(n, count=12, seed=2024 + rank, nz=n)
    ang = phantoms.angles_full(views)
    dev = torch.device("cuda", local)
    vol = torch.from_numpy(np.ascontiguousarray(vol_h.transpose(2, 1, 0))).to(dev)
    sino = torch.empty((views, n, n), dtype=torch.float32, device=dev)
    rec = torch.empty((n, n, n), dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sptr = V(stream.cuda_stream)
    angp = V(ang.ctypes.data)

    def fp(g=geom, out=sino):
        _lib.check(lib.mexct_fp_dev(None, V(vol.data_ptr()), n, n, 1000.0, angp, views, g,
                                    V(out.data_ptr()), sptr))

    def bp(g=geom, src=sino):
        _lib.check(lib.mexct_bp_dev(None, V(src.data_ptr()), n, n, views, 1000.0, angp, g,
                                    V(rec.data_ptr()), sptr))

    def step():
        fp()
        bp()

    def timed(fn, reps=1):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(reps):
                fn()
            e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps / 1e3

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # Per-operator times (events on the launching stream) for the roofline.
    fp_t = float(np.median([timed(fp) for _ in range(2)]))
    bp_t = float(np.median([timed(bp) for _ in range(2)]))

    clocks = ClockSampler(local)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(args.steps):
        step()
    t1.record(stream)
    t1.synchronize()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = max_over_ranks(t0.elapsed_time(t1), dist, dev)
    ms_step = ms / args.steps
    gups = 2.0 * N * views * args.steps * world / (ms / 1e3) / 1e9

    # e2e through the host entry points (pinned host buffers).
    e2e = None
    if not args.no_e2e:
        vol_pin = torch.from_numpy(np.ascontiguousarray(vol_h.transpose(2, 1, 0))).pin_memory()
        sino_pin = torch.empty((views, n, n), dtype=torch.float32).pin_memory()
        rec_pin = torch.empty((n, n, n), dtype=torch.float32).pin_memory()

        def e2e_step():
            _lib.check(lib.mexct_fp(None, V(vol_pin.data_ptr()), n, n, 1000.0, angp, views, geom,
                                    V(sino_pin.data_ptr())))
            _lib.check(lib.mexct_bp(None, V(sino_pin.data_ptr()), n, n, views, 1000.0, angp, geom,
                                    V(rec_pin.data_ptr())))

        for _ in range(max(2, min(args.warmup, 3))):  # first calls grow the context's buffers
            e2e_step()
        if dist is not None:
            dist.barrier()
        k = max(1, args.steps)
        t = time.perf_counter()
        for _ in range(k):
            e2e_step()
        el = max_over_ranks(time.perf_counter() - t, dist, dev)
        e2e = {"value": round(2.0 * N * views * k * world / el / 1e9, 3), "unit": "GUPS",
               "h2d_bytes_per_step": 4 * (N + P * views), "d2h_bytes_per_step": 4 * (P * views + N),
               "path": "mexct_fp + mexct_bp host entry points, pinned buffers"}

    peak, peak_kind = hbm_peak()
    fp_bytes = 4.0 * (N + P * views)
    bp_bytes = 4.0 * (P * views + N)
    dom = ("fp_slab_kernel (cone FP)", fp_t, fp_bytes, FP_SLAB_DRAM_BYTES_PER_VIEW * views) \
        if fp_t >= bp_t else ("bp_kernel (cone BP)", bp_t, bp_bytes, None)
    achieved = dom[2] / dom[1] / 1e9
    line = {
        "metric": metric_name(args),
        "value": round(gups, 3), "unit": "GUPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_step, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded 12-ellipsoid phantom)",
        "config": workload_config(args, world),
        "fp_slab_ctas_per_sm": ops.fp_slab_occupancy(),
        "fp_gups": round(N * views / fp_t / 1e9, 3), "bp_gups": round(N * views / bp_t / 1e9, 3),
        "fp_ms": round(fp_t * 1e3, 3), "bp_ms": round(bp_t * 1e3, 3),
        "roofline": {"bound": "hbm", "kernel": dom[0], "achieved": round(achieved, 2),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 5),
                     "peak_source": "%s (MEASURED_PEAKS.json hbm_gbs)" % peak_kind
                     if peak_kind == "measured" else "fallback 6.8 TB/s",
                     "traffic": dom[3],
                     "note": "gather-bound projector: compulsory bytes 4(N+P*nP) over the "
                             "launch; its bound is on chip (ncu: the L1/shared-memory data "
                             "pipe at ~80 % of its wavefront peak, 67-71 % of issue slots)"},
        "clocks": clk,
        # per step: pad_x, pad_transpose, fp_slab, pad_sino_quad, bp_pad
        "gpu_launches": 5 * args.steps,
        "e2e": e2e,
    }

    if not args.no_extra and rank == 0:
        extra = {}
        # geomFlag 0 and 1 at the same size.
        for g in (0, 1):
            if g == geom:
                continue
            fp(g)
            tf = timed(lambda: fp(g))
            tb = timed(lambda: bp(g))
            extra["geom%d" % g] = {"fp_gups": round(N * views / tf / 1e9, 3),
                                   "bp_gups": round(N * views / tb / 1e9, 3)}
        # Chosen forms of FP: hardware texture (8-bit filter weights) and FP16 storage.
        # (Every launch goes to `stream`; it is synchronised before torch reads.)
        fp()
        stream.synchronize()
        ref_sino = sino.clone()
        tex = torch.empty_like(sino)
        _lib.check(lib.mexct_fp_dev_ex(None, V(vol.data_ptr()), 0, n, n, 1000.0, angp, views, geom,
                                       V(tex.data_ptr()), 0, 1, sptr))
        tt = timed(lambda: lib.mexct_fp_dev_ex(None, V(vol.data_ptr()), 0, n, n, 1000.0, angp,
                                               views, geom, V(tex.data_ptr()), 0, 1, sptr))
        stream.synchronize()
        extra["fp_texture"] = {"fp_gups": round(N * views / tt / 1e9, 3),
                               "rel_l2_vs_fp32": rel(tex, ref_sino)}
        del tex
        vol16 = vol.half()
        s16 = torch.empty((views, n, n), dtype=torch.float16, device=dev)
        r16 = torch.empty((n, n, n), dtype=torch.float16, device=dev)

        def fp16():
            _lib.check(lib.mexct_fp_dev_ex(None, V(vol16.data_ptr()), 1, n, n, 1000.0, angp, views,
                                           geom, V(s16.data_ptr()), 1, 0, sptr))

        def bp16():
            _lib.check(lib.mexct_bp_dev_ex(None, V(s16.data_ptr()), 1, n, n, views, 1000.0, angp,
                                           geom, V(r16.data_ptr()), 1, sptr))

        fp16()
        bp16()
        t16f, t16b = timed(fp16), timed(bp16)
        bp()
        stream.synchronize()
        extra["fp16_storage"] = {"fp_gups": round(N * views / t16f / 1e9, 3),
                                 "bp_gups": round(N * views / t16b / 1e9, 3),
                                 "fp_rel_l2_vs_fp32": rel(s16.float(), ref_sino),
                                 "bp_rel_l2_vs_fp32": rel(r16.float(), rec)}
        del vol16, s16, r16
        # The reference's own kernels on this GPU at the same workload (host arrays
        # in and out, as its gateways take them), beside ours.
        try:
            extra["reference_kernels"] = reference_section(vol_h, ang, geom, n, views, fp_t, bp_t,
                                                           ref_sino)
        except Exception as ex:  # reported, never fatal
            extra["reference_kernels"] = {"error": "%s: %s" % (type(ex).__name__, ex)}
        # The same step from the standalone C++ benchmark (C ABI, cudaMalloc buffers).
        try:
            extra["cpp_bench"] = cpp_bench(n, views, geom)
        except Exception as ex:  # reported, never fatal
            extra["cpp_bench"] = {"error": "%s: %s" % (type(ex).__name__, ex)}
        # OSC-TV reconstruction latency (config: 256^3, 60 views, 20 it x 10 subsets).
        del ref_sino
        for name, fn in (("autotune", autotune_section),
                         ("osc_tv", lambda: osc_tv_latency(args.osc_reps)),
                         ("batched", lambda: batched_uneven(args.batch_problems)),
                         ("serving", lambda: serving(args.serve_requests)),
                         ("config2", config2),
                         ("detector", detector_section),
                         ("other_operators", other_operators),
                         ("out_of_core", out_of_core)):
            try:
                extra[name] = fn()
            except Exception as ex:  # reported, never fatal
                extra[name] = {"error": "%s: %s" % (type(ex).__name__, ex)}
            torch.cuda.empty_cache()
        line["extra"] = extra
    if rank == 0 and not args.no_cpu:
        try:
            line["cpu_baseline"] = cpu_sample(n, views, geom, seconds_target=12.0)
        except Exception as ex:  # reported, never fatal
            line["cpu_baseline"] = {"error": str(ex)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def cpp_bench(n, views, geom):
    """The headline step from mex-cuda-ct_gb300/bench/mexct_bench.cpp: the same C ABI
    driven from C++ with cudaMalloc buffers and CUDA events (no Python in the loop)."""
    import __graft_entry__ as ge

    exe = ge._builder().build_bench()
    r = subprocess.run([exe, "--size", str(n), "--views", str(views), "--geom", str(geom),
                        "--steps", "5", "--warmup", "2"], capture_output=True, text=True, timeout=600)
    if r.returncode != 0:
        return {"error": r.stderr.strip()[-600:]}
    d = json.loads(r.stdout.strip().splitlines()[-1])
    return {k: d[k] for k in ("value", "ms_per_step", "fp_ms", "bp_ms", "e2e", "impl")}


def reference_section(vol_h, ang, geom, n, views, fp_t, bp_t, our_sino):
    """Reference FP and BP (its own kernels, per view, host arrays) at the headline
    workload; its FP against our texture variant (bit for bit) and our exact path."""
    import torch
    from mexct import _lib, ops
    from oracle import reference

    if not reference.available():
        return {"unavailable": "reference cubins not built or no CUDA device"}
    fps, bps = reference_step_times(vol_h, ang, geom, 1)
    rf = reference.fp(vol_h, 1000.0, ang, views, geom)
    dvol = torch.from_numpy(np.ascontiguousarray(vol_h.transpose(2, 1, 0))).cuda()
    tex = ops.fp_dev(dvol, 1000.0, ang, geom, variant=_lib.FP_TEXTURE).cpu().numpy().transpose(2, 1, 0)
    ours = our_sino.cpu().numpy().transpose(2, 1, 0)
    N = n ** 3
    return {"fp_ms": round(fps[0] * 1e3, 1), "bp_ms": round(bps[0] * 1e3, 1),
            "fp_gups": round(N * views / fps[0] / 1e9, 2), "bp_gups": round(N * views / bps[0] / 1e9, 2),
            "ours_fp_ms": round(fp_t * 1e3, 2), "ours_bp_ms": round(bp_t * 1e3, 2),
            "texture_variant_equals_reference": bool(np.array_equal(tex, rf)),
            "rel_l2_exact_path_vs_reference": rel_np(ours, rf),
            "note": "reference: its CUDA kernels compiled unmodified for sm_103a, one launch, "
                    "synchronisation and host copy per view, as its gateways run them"}


def osc_tv_latency(reps, forms=("plain_fp32", "chosen_graph_fp32", "chosen_graph_fp16_data",
                               "chosen_graph_bf16")):
    """p50/p99 seconds per OSC-TV reconstruction, plain (eager, FP32) vs chosen (graphs):
    FP32 throughout; FP32 mu with FP16 counts and residual views (the form within a
    1e-3 accuracy bound); BF16 mu (outside it: an 8-bit mantissa)."""
    import torch

    from mexct import ops, phantoms, solver

    n, nv = 256, 60
    vol = phantoms.ellipsoids(n, count=10, seed=7, nz=n)
    ang = phantoms.angles_full(nv)
    dvol = torch.from_numpy(np.ascontiguousarray(vol.transpose(2, 1, 0))).cuda()
    fp = ops.fp_dev(dvol, 1000.0, ang, 2)
    torch.cuda.synchronize()
    rng = np.random.default_rng(11)
    pre = torch.full_like(fp, 1e5)
    post = torch.from_numpy(rng.poisson(1e5 * np.exp(-fp.double().cpu().numpy())).astype(np.float32)).cuda()
    picks = rng.integers(0, 10, 20)
    out = {}
    for name, graph, dt, ddt in (("plain_fp32", False, None, None),
                                 ("chosen_graph_fp32", True, None, None),
                                 ("chosen_graph_fp16_data", True, None, torch.float16),
                                 ("chosen_graph_bf16", True, torch.bfloat16, None)):
        if name not in forms:
            continue
        times = []
        mu_last = None
        for r in range(reps + 1):
            torch.cuda.synchronize()
            t = time.perf_counter()
            s = solver.OscTvSolver(pre, post, ang, 1000.0, 2, mu_dtype=dt, data_dtype=ddt)
            s.run(picks, n_iter=20, tv_const=0.2, n_sub_init=10, n_sub_final=10, p_val=1.0,
                  use_graph=graph)
            mu_last = s.mu()
            torch.cuda.synchronize()
            el = time.perf_counter() - t
            s.close()
            if r > 0:  # first run warms up (graph capture, lazy module load)
                times.append(el)
        out[name] = {"p50_s": round(float(np.percentile(times, 50)), 4),
                     "p99_s": round(float(np.percentile(times, 99)), 4),
                     "volumes_per_s": round(1.0 / float(np.mean(times)), 3), "reps": reps}
        out[name]["_mu"] = mu_last
    ref = out["plain_fp32"].pop("_mu") if "plain_fp32" in out else None
    for k in ("chosen_graph_fp32", "chosen_graph_fp16_data", "chosen_graph_bf16"):
        if k in out:
            mu = out[k].pop("_mu")
            if ref is not None:
                out[k]["rel_l2_vs_plain"] = rel(mu, ref)
    if "chosen_graph_bf16" in out:
        out["chosen_graph_bf16"]["note"] = "BF16 mu: outside a 1e-3 accuracy bound"
    out["workload"] = "256^3, 60 cone views, 20 iterations x 10 subsets, TV 20 steps at 0.2*d_a"
    return out


def batched_uneven(count, seed=2026):
    """48 uneven problems (geom 0/1/2, 64^3..256^3, 90..720 views): FP + BP + 5 OSC-TV
    iterations (8 subsets) each.  plain: one problem at a time, one launch per
    operator call, eager OSC-TV.  chosen: all FPs in one persistent launch and all
    BPs as concurrent per-problem launches on 8 streams, each captured in a CUDA graph;
    OSC-TV solvers replay per-iteration graphs on 8 concurrent streams."""
    import torch

    from mexct import batch, ops, phantoms, solver

    rng = np.random.default_rng(seed)
    probs = []
    for i in range(count):
        n = int(rng.choice([64, 96, 128, 192, 256]))
        nv = int(rng.integers(90, 721))
        g = int(rng.integers(0, 3))
        vol = phantoms.ellipsoids(n, count=6, seed=seed + i, nz=n)
        ang = phantoms.angles_full(nv)
        d = torch.from_numpy(np.ascontiguousarray(vol.transpose(2, 1, 0))).cuda()
        probs.append({"vol": d, "sino": torch.empty((nv, n, n), device="cuda"),
                      "rec": torch.empty((n, n, n), device="cuda"), "angles": ang, "sad": 1000.0,
                      "geom": g, "picks": rng.integers(0, 8, 5)})
    vu = sum(p["vol"].numel() * p["angles"].size for p in probs)  # voxel-view updates per op
    # Counts for OSC-TV: pre = 1e5, post = noiseless 1e5*exp(-FP) (the FP is computed once).
    for p in probs:
        ops.fp_dev(p["vol"], p["sad"], p["angles"], p["geom"], out=p["sino"])
    torch.cuda.synchronize()
    pre = [torch.full_like(p["sino"], 1e5) for p in probs]
    post = [1e5 * torch.exp(-p["sino"]) for p in probs]
    kw = dict(n_iter=5, tv_const=0.2, n_sub_init=8, n_sub_final=8, p_val=1.0)

    def plain():
        for p in probs:
            ops.fp_dev(p["vol"], p["sad"], p["angles"], p["geom"], out=p["sino"])
        torch.cuda.synchronize()
        t_f = time.perf_counter()
        for p in probs:
            ops.bp_dev(p["sino"], p["sad"], p["angles"], p["geom"], out=p["rec"])
        torch.cuda.synchronize()
        t_fb = time.perf_counter()
        for k, p in enumerate(probs):
            sv = solver.OscTvSolver(pre[k], post[k], p["angles"], p["sad"], p["geom"])
            sv.run(p["picks"], use_graph=False, **kw)
            torch.cuda.synchronize()
            sv.close()
        return t_f, t_fb

    b = batch.Batch(probs)
    st = torch.cuda.Stream()
    b.fp(st)
    b.bp(st)
    st.synchronize()
    g_fp, g_bp = torch.cuda.CUDAGraph(), torch.cuda.CUDAGraph()
    with torch.cuda.graph(g_fp, stream=st):
        b.fp(st)
    with torch.cuda.graph(g_bp, stream=st):
        b.bp(st)
    streams = [torch.cuda.Stream() for _ in range(8)]

    def chosen():
        g_fp.replay()
        torch.cuda.synchronize()
        t_f = time.perf_counter()
        g_bp.replay()
        torch.cuda.synchronize()
        t_fb = time.perf_counter()
        solvers = []
        for k, p in enumerate(probs):
            s_ = streams[k % len(streams)]
            sv = solver.OscTvSolver(pre[k], post[k], p["angles"], p["sad"], p["geom"], stream=s_)
            sv.run(p["picks"], use_graph=True, **kw)
            solvers.append(sv)
        torch.cuda.synchronize()
        for sv in solvers:
            sv.close()
        return t_f, t_fb

    out = {"problems": count, "voxel_view_updates_per_op": vu}
    for name, fn in (("plain", plain), ("chosen", chosen)):
        fn()  # warm-up (graph capture, lazy loading)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        t_f, t_fb = fn()
        t1 = time.perf_counter()
        out[name] = {"total_s": round(t1 - t0, 4), "fp_s": round(t_f - t0, 4),
                     "bp_s": round(t_fb - t_f, 4), "osc_tv_s": round(t1 - t_fb, 4),
                     "fp_gups": round(vu / (t_f - t0) / 1e9, 3),
                     "bp_gups": round(vu / (t_fb - t_f) / 1e9, 3)}
    out["speedup_total"] = round(out["plain"]["total_s"] / out["chosen"]["total_s"], 3)
    out["workload"] = ("%d problems: geom 0/1/2, 64^3..256^3, 90..720 views, SAD 1000; FP, BP, "
                       "5 OSC-TV iterations x 8 subsets each" % count)
    b.close()
    return out


def ops_once(n=256, nv=90):
    """One call of each secondary operator on a small case: general3D FP and BP (helix,
    per-view points), one TV step, one OSC iteration (60 cone views, 10 subsets), the
    FDK pre-filter of those views."""
    import torch

    from mexct import ops, phantoms

    vol = phantoms.ellipsoids(n, count=10, seed=5, nz=n)
    d = torch.from_numpy(np.ascontiguousarray(vol.transpose(2, 1, 0))).cuda()
    pts, ang = phantoms.helix_pts(n, n, nv, n, sad=1000.0, turns=1.0, pitch=0.5)
    dp = torch.from_numpy(np.ascontiguousarray(pts.transpose(3, 2, 1, 0))).cuda()
    sino = ops.g3d_fp_dev(d, ang, dp)
    rec = ops.g3d_bp_dev(sino, ang, dp, n, n)
    tv = ops.tvmin3d_dev(d, 0.2, 1)
    ang6 = phantoms.angles_full(60)
    s6 = ops.fp_dev(d, 1000.0, ang6, 2)
    pre = torch.full_like(s6, 1e5)
    post = 1e5 * torch.exp(-s6)
    mu = torch.full_like(d, 1e-3)
    ops.osc_iter_dev(mu, pre, post, 10, np.arange(10, dtype=np.int32), ang6, 1000.0, 2)
    f = ops.prefilter_dev(s6, ang6, 2, 1000.0, "ramp")
    torch.cuda.synchronize()
    print(json.dumps({"ops_once": "ok", "checksums": [float(t.double().sum()) for t in
                                                      (sino, rec, tv, mu, f)]}))


def other_operators():
    """The remaining operators at representative sizes, device-resident inputs, CUDA-synchronised
    wall time (3 runs after a warm-up): general3D FP / BP on a cone helix (256^3, 256 x 256
    detector, 360 views, per-view points), TV descent (512^3, 20 steps), FDK pre-filter
    (512 x 512 x 720 cone views, ramp), OSC iteration (256^3, 60 cone views, 10 subsets)."""
    import torch

    from mexct import ops, phantoms

    def timed(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / reps

    out = {}
    n, nv = 256, 360
    vol = phantoms.ellipsoids(n, count=10, seed=5, nz=n)
    d = torch.from_numpy(np.ascontiguousarray(vol.transpose(2, 1, 0))).cuda()
    pts, ang = phantoms.helix_pts(n, n, nv, n, sad=1000.0, turns=1.0, pitch=0.5)
    dp = torch.from_numpy(np.ascontiguousarray(pts.transpose(3, 2, 1, 0))).cuda()
    sino = ops.g3d_fp_dev(d, ang, dp)
    tf = timed(lambda: ops.g3d_fp_dev(d, ang, dp, out=sino))
    rec = torch.empty_like(d)
    tb = timed(lambda: ops.g3d_bp_dev(sino, ang, dp, n, n, out=rec))
    vu = float(n) ** 3 * nv
    out["general3d_helix_256cube_360views"] = {"fp_s": round(tf, 4), "bp_s": round(tb, 4),
                                               "fp_gups": round(vu / tf / 1e9, 3),
                                               "bp_gups": round(vu / tb / 1e9, 3)}
    del sino, rec, dp
    m = 512
    v5 = torch.from_numpy(np.ascontiguousarray(
        phantoms.ellipsoids(m, count=12, seed=2024, nz=m).transpose(2, 1, 0))).cuda()
    tv_out = torch.empty_like(v5)
    t = timed(lambda: ops.tvmin3d_dev(v5, 0.2, 20, out=tv_out))
    N = float(m) ** 3
    out["tv_512cube_20steps"] = {"s": round(t, 4), "ms_per_step": round(t / 20 * 1e3, 3),
                                 "gbs_per_step": round(4 * 3 * N / (t / 20) / 1e9, 1)}
    ang7 = phantoms.angles_full(720)
    s7 = ops.fp_dev(v5, 1000.0, ang7, 2)
    f7 = torch.empty_like(s7)
    t = timed(lambda: ops.prefilter_dev(s7, ang7, 2, 1000.0, "ramp", out=f7))
    out["prefilter_cone_512x512x720_ramp"] = {"s": round(t, 4),
                                              "gbs": round(2 * 4 * s7.numel() / t / 1e9, 1)}
    del s7, f7, v5, tv_out
    ang6 = phantoms.angles_full(60)
    s6 = ops.fp_dev(d, 1000.0, ang6, 2)
    pre = torch.full_like(s6, 1e5)
    post = 1e5 * torch.exp(-s6)
    mu = torch.zeros_like(d)
    picks = np.arange(10, dtype=np.int32)
    t = timed(lambda: ops.osc_iter_dev(mu, pre, post, 10, picks, ang6, 1000.0, 2))
    out["osc_iteration_256cube_60views_10subsets"] = {"s": round(t, 4)}
    return out


def config2(n=384, views=512):
    """The ellipsoid workload: 384^3 (12 ellipsoids), 512 views over 2 pi, SAD 1000: FP for
    geomFlag 0/1/2, the Hamming FDK chain (pre-filter then BP), and general3D FP / BP on
    384 x 512 rays per view over a 2-turn helix (pitch 1, per-view points), all
    device-resident; CUDA events over 3 runs after a warm-up."""
    import torch

    from mexct import ops, phantoms

    def timed(fn, reps=3):
        fn()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record()
        for _ in range(reps):
            fn()
        b.record()
        b.synchronize()
        return a.elapsed_time(b) / reps / 1e3

    vol = phantoms.ellipsoids(n, count=12, seed=2)
    d = torch.from_numpy(np.ascontiguousarray(vol.transpose(2, 1, 0))).cuda()
    ang = phantoms.angles_full(views)
    vu = float(n) ** 3 * views
    out = {"workload": "%d^3 ellipsoids x %d views over 2 pi, SAD 1000, device-resident" % (n, views)}
    for geom in (0, 1, 2):
        s = ops.fp_dev(d, 1000.0, ang, geom)
        tf = timed(lambda: ops.fp_dev(d, 1000.0, ang, geom, out=s))
        f = torch.empty_like(s)
        tp = timed(lambda: ops.prefilter_dev(s, ang, geom, 1000.0, "hamming", out=f))
        r = torch.empty_like(d)
        tb = timed(lambda: ops.bp_dev(f, 1000.0, ang, geom, out=r))
        out["geom%d" % geom] = {"fp_ms": round(tf * 1e3, 2), "fp_gups": round(vu / tf / 1e9, 1),
                                "hamming_prefilter_ms": round(tp * 1e3, 2),
                                "fdk_bp_ms": round(tb * 1e3, 2), "bp_gups": round(vu / tb / 1e9, 1),
                                "fdk_chain_ms": round((tp + tb) * 1e3, 2)}
        del s, f, r
    pts, hang = phantoms.helix_pts(n, 512, views, n, sad=1000.0, seed=4)
    dp = torch.from_numpy(np.ascontiguousarray(pts.transpose(3, 2, 1, 0))).cuda()
    del pts
    s = ops.g3d_fp_dev(d, hang, dp)
    tf = timed(lambda: ops.g3d_fp_dev(d, hang, dp, out=s))
    rec = torch.empty_like(d)
    tb = timed(lambda: ops.g3d_bp_dev(s, hang, dp, n, n, out=rec))
    rays = float(n) * 512 * views
    out["general3d_helix_384x512_rays_x%d" % views] = {
        "fp_ms": round(tf * 1e3, 2), "bp_ms": round(tb * 1e3, 2),
        "fp_grays_per_s": round(rays / tf / 1e9, 3), "bp_grays_per_s": round(rays / tb / 1e9, 3)}
    return out


def detector_section(n=512, views=180, geom=2):
    """Decoupled detector at 512^3 cone, 180 views: FP onto a 1.5x finer detector
    (768 x 768, pitch 2/3) with one and with 2 x 2 rays per pixel, BP from it,
    against the volume's own detector (512 x 512, pitch 1)."""
    import torch

    from mexct import _lib, ops, phantoms

    vol = phantoms.ellipsoids(n, count=12, seed=2024, nz=n)
    d = torch.from_numpy(np.ascontiguousarray(vol.transpose(2, 1, 0))).cuda()
    ang = phantoms.angles_full(views)
    N = float(n) ** 3

    def timed(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / reps

    out = {"workload": "cone %d^3, %d views, SAD 1000; GUPS = voxels x views / s" % (n, views)}
    sino = ops.fp_dev(d, 1000.0, ang, geom, variant=_lib.FP_EXPLICIT)
    t = timed(lambda: ops.fp_dev(d, 1000.0, ang, geom, out=sino, variant=_lib.FP_EXPLICIT))
    out["fp_own_detector_512"] = {"s": round(t, 4), "gups": round(N * views / t / 1e9, 3)}
    m = n * 3 // 2
    fine = torch.empty((views, m, m), device="cuda")
    for ss in (1, 2):
        t = timed(lambda: ops.fp_det_dev(d, 1000.0, ang, geom, m, m, 2 / 3, 2 / 3, ss, out=fine))
        out["fp_det_%d_ss%d" % (m, ss)] = {"s": round(t, 4), "gups": round(N * views / t / 1e9, 3)}
    rec = torch.empty_like(d)
    t = timed(lambda: ops.bp_dev(sino, 1000.0, ang, geom, out=rec))
    out["bp_own_detector_512"] = {"s": round(t, 4), "gups": round(N * views / t / 1e9, 3)}
    t = timed(lambda: ops.bp_det_dev(fine, 1000.0, ang, geom, n, n, 2 / 3, 2 / 3, out=rec))
    out["bp_det_%d" % m] = {"s": round(t, 4), "gups": round(N * views / t / 1e9, 3)}
    return out


def out_of_core(n=768, views=360, geom=2, budget=1 << 30):
    """Host volume 768^3 (1.7 GiB) and sinogram (0.8 GiB), cone, 360 views: FP and BP
    through the host entry points with the whole problem on the device, against the
    out-of-core drivers held to a 1 GiB device working set (slabs / view chunks /
    row bands streamed from host memory)."""
    import mexct
    from mexct import ops, phantoms

    vol = phantoms.ellipsoids(n, count=12, seed=77, nz=n)
    ang = phantoms.angles_full(views)
    N = float(n) ** 3
    out = {"workload": "cone %d^3 x %d views, SAD 1000, host arrays; budget %d MiB"
                       % (n, views, budget >> 20)}
    mexct.CUDAmex_FP(vol[:, :, :8].copy(order="F"), 1000.0, ang, 4, geom)  # warm-up
    t0 = time.perf_counter()
    fp_in = mexct.CUDAmex_FP(vol, 1000.0, ang, views, geom)
    t1 = time.perf_counter()
    fp_oc = ops.fp_ooc(vol, 1000.0, ang, geom, budget)
    t2 = time.perf_counter()
    bp_in = mexct.CUDAmex_BP(fp_in, 1000.0, ang, geom)
    t3 = time.perf_counter()
    bp_oc = ops.bp_ooc(fp_in, 1000.0, ang, geom, budget)
    t4 = time.perf_counter()
    out["fp_in_core"] = {"s": round(t1 - t0, 3), "gups": round(N * views / (t1 - t0) / 1e9, 3)}
    out["fp_out_of_core"] = {"s": round(t2 - t1, 3), "gups": round(N * views / (t2 - t1) / 1e9, 3),
                             "rel_l2_vs_in_core": rel_np(fp_oc, fp_in)}
    out["bp_in_core"] = {"s": round(t3 - t2, 3), "gups": round(N * views / (t3 - t2) / 1e9, 3)}
    out["bp_out_of_core"] = {"s": round(t4 - t3, 3), "gups": round(N * views / (t4 - t3) / 1e9, 3),
                             "rel_l2_vs_in_core": rel_np(bp_oc, bp_in)}
    del vol, fp_in, fp_oc, bp_in, bp_oc
    out["osc_tv"] = osc_tv_out_of_core()
    return out


def osc_tv_out_of_core(n=256, views=60, n_iter=20, nsub=10, slabs=4):
    """OSC-TV at the few-view workload (256^3 ellipsoids, 60 cone views, 20
    iterations x 10 subsets, TV 0.2), host arrays in and out: the in-core one-shot
    entry point against the out-of-core solver (mu in host memory, z-slabs) held to
    the budget of `slabs` slabs."""
    from mexct import phantoms, solver

    vol = phantoms.ellipsoids(n, count=10, seed=3, nz=n)
    ang = phantoms.angles_full(views)
    fp = line_integrals(vol, ang)
    pre, post = phantoms.poisson_counts(fp, 1e5, seed=4)
    picks = [int(v) for v in np.random.default_rng(5).integers(0, nsub, n_iter)]
    g = {"type": "cone3d", "SAD": 1000.0}
    _, full = solver.ooc_plan(n, n, views, 2, n_iter, nsub, nsub, 1.0, 1 << 40)
    budget = full // slabs * 2  # two slab buffer sets of ~1/slabs of the volume each
    nz, nbytes = solver.ooc_plan(n, n, views, 2, n_iter, nsub, nsub, 1.0, budget)
    solver.OSC_TV_recon(pre, post, ang, g, 1, 0.2, nsub, nsub, 1.0, picks[:1])  # warm-up
    t0 = time.perf_counter()
    ref = solver.OSC_TV_recon(pre, post, ang, g, n_iter, 0.2, nsub, nsub, 1.0, picks)
    t1 = time.perf_counter()
    got, _ = solver.OSC_TV_recon_ooc(pre, post, ang, g, n_iter, 0.2, nsub, nsub, 1.0, picks, budget)
    t2 = time.perf_counter()
    return {"workload": "cone %d^3 x %d views, %d iterations x %d subsets, TV 0.2, host arrays"
                        % (n, views, n_iter, nsub),
            "in_core_s": round(t1 - t0, 3), "out_of_core_s": round(t2 - t1, 3),
            "slab_slices": nz, "device_bytes": int(nbytes),
            "one_slab_device_bytes": int(full),
            "rel_l2_vs_in_core": rel_np(got, ref)}


def line_integrals(vol, ang):
    """Noise-free line integrals for the count model (the library's own FP)."""
    import mexct

    return mexct.CUDAmex_FP(vol, 1000.0, ang, len(ang), 2)


def rel_np(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def autotune_section(classes=((64, 90, 2), (96, 180, 0), (128, 360, 2), (256, 720, 2))):
    """FP and BP of small and mid-size classes under the three shape modes: fixed
    (slab FP, BP without view blocks), heuristic (the default) and autotuned (every
    candidate timed on the first call).  GUPS from CUDA events over >= 3 runs and
    >= ~20 ms of work after warm-up."""
    import torch

    from mexct import ops, phantoms, tune

    out = {}
    for n, nv, g in classes:
        vol = phantoms.ellipsoids(n, count=6, seed=n + nv, nz=n)
        ang = phantoms.angles_full(nv)
        d = torch.from_numpy(np.ascontiguousarray(vol.transpose(2, 1, 0))).cuda()
        sino = ops.fp_dev(d, 1000.0, ang, g)
        rec = torch.empty_like(d)
        res = {}
        for mode, name in ((tune.FIXED, "fixed"), (tune.HEURISTIC, "heuristic"),
                           (tune.AUTO, "autotuned")):
            tune.clear()
            tune.set_mode(mode)
            row = {}
            for op, fn in (("fp", lambda: ops.fp_dev(d, 1000.0, ang, g, out=sino)),
                           ("bp", lambda: ops.bp_dev(sino, 1000.0, ang, g, out=rec))):
                fn()  # tunes in auto mode
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                fn()
                e1.record()
                torch.cuda.synchronize()
                reps = int(min(200, max(3, np.ceil(20.0 / max(e0.elapsed_time(e1), 1e-3)))))
                e0.record()
                for _ in range(reps):  # >= ~20 ms of work per measurement
                    fn()
                e1.record()
                torch.cuda.synchronize()
                t = e0.elapsed_time(e1) / reps / 1e3
                row[op + "_gups"] = round(n ** 3 * nv / t / 1e9, 2)
            row["bp_shape"] = tune.shape_get(tune.BP, g, n, n, nv)
            row["fp_variant"] = tune.shape_get(tune.FP, g, n, n, nv)["variant"]
            for k in ("ms",):
                row["bp_shape"].pop(k, None)
            res[name] = row
        out["%d^3x%d_geom%d" % (n, nv, g)] = res
    tune.clear()
    tune.set_mode(tune.HEURISTIC)
    return out


def serving(count, seed=7, sizes=(128, 256), size_p=(0.7, 0.3), views=(60, 180, 360),
            serial_sample=None, saturated=True, budget_gb=48):
    """Open-loop Poisson arrivals of FDK / OSC-TV (10 iterations x 10 subsets)
    requests on seeded ellipsoid volumes of the given sizes and view counts, random
    geometry, FP32 or FP16 storage (OSC-TV: FP16 residual views with FP32 mu);
    lambda set for ~80% of the one-at-a-time service rate.  The same request stream
    runs through a one-slot server (plain: FIFO, one request on the device at a time)
    and a four-slot server (chosen: admission by HBM footprint, requests overlap on
    their own streams).  Reports p50/p99 latency (submission to completion) and
    volumes/s, and checks results against the one-request entry points: every
    request (serial_sample None), or a seeded sample of serial_sample requests, whose
    mean service time then sets lambda."""
    import torch

    import mexct
    from mexct import _lib, ops, phantoms, serve, solver

    rng = np.random.default_rng(seed)
    datasets = {}
    for n in sizes:
        vol = phantoms.ellipsoids(n, count=8, seed=n, nz=n)
        d = torch.from_numpy(np.ascontiguousarray(vol.transpose(2, 1, 0))).cuda()
        for nv in views:
            ang = phantoms.angles_full(nv)
            fpd = ops.fp_dev(d, 1000.0, ang, 2)
            torch.cuda.synchronize()
            fp = fpd.cpu().numpy().transpose(2, 1, 0)
            del fpd
            pre = np.full(fp.shape, 1e5, dtype=np.float32, order="F")
            post = np.asfortranarray(rng.poisson(1e5 * np.exp(-fp.astype(np.float64)))
                                     .astype(np.float32))
            datasets[(n, nv)] = (pre, post, ang)
        del d
        torch.cuda.empty_cache()
    reqs = []
    for i in range(count):
        n = int(rng.choice(list(sizes), p=list(size_p)))
        nv = int(rng.choice(list(views)))
        reqs.append({"kind": int(rng.integers(0, 2)), "key": (n, nv), "geom": int(rng.integers(0, 3)),
                     "f16": bool(rng.integers(0, 2)), "picks": rng.integers(0, 10, 10)})
    gs = {0: "par3d", 1: "fan3d", 2: "cone3d"}

    def alone(r):
        pre, post, ang = datasets[r["key"]]
        if r["kind"] == 0:
            return mexct.FBP_recon(pre, post, ang, {"type": gs[r["geom"]], "SAD": 1000.0},
                                   "hamming", 1.0, 1.0)
        if not r["f16"]:
            return solver.OSC_TV_recon(pre, post, ang, {"type": gs[r["geom"]], "SAD": 1000.0}, 10,
                                       0.2, 10, 10, 1.0, r["picks"])
        srv = serve.Server(slots=1, budget_bytes=64 << 30)
        t = srv.submit_osctv(pre, post, ang, r["geom"], r["picks"], n_iter=10, n_sub=10,
                             data_type=_lib.F16)
        out = srv.wait(t)[0]
        srv.close()
        return out

    import hashlib

    def digest(a):  # results are compared by digest: the full arrays need not stay in memory
        return hashlib.sha256(np.ascontiguousarray(a).view(np.uint8)).hexdigest()

    alone(reqs[0])  # warm-up
    check = list(range(count)) if serial_sample is None else sorted(
        rng.choice(count, min(serial_sample, count), replace=False).tolist())
    serial = {}
    t0 = time.perf_counter()
    for i in check:
        serial[i] = digest(alone(reqs[i]))
    mean_s = (time.perf_counter() - t0) / len(check)
    lam = 0.8 / mean_s
    gaps = rng.exponential(1.0 / lam, count)

    def submit(srv, r):
        pre, post, ang = datasets[r["key"]]
        if r["kind"] == 0:
            return srv.submit_fdk(pre, post, ang, r["geom"])
        return srv.submit_osctv(pre, post, ang, r["geom"], r["picks"], n_iter=10, n_sub=10,
                                data_type=_lib.F16 if r["f16"] else _lib.F32)

    def run(slots, open_loop):
        """The request stream through a server with `slots` slots: open loop (the
        Poisson arrival times) or closed (everything queued at once, for peak
        volumes/s).  Latency = completion - submission."""
        srv = serve.Server(slots=slots, budget_bytes=int(budget_gb) << 30)
        tickets = []
        lat, same = [], [0]
        # A collector thread waits for the tickets in submission order while
        # requests are still arriving, so finished reconstructions are released.
        cv = threading.Condition()

        def collect():
            for i in range(count):
                with cv:
                    while len(tickets) <= i:
                        cv.wait()
                    t = tickets[i]
                rec, tm = srv.wait(t)
                lat.append(tm["total_s"])
                if i in serial:
                    same[0] += int(digest(rec) == serial[i])
                del rec

        th = threading.Thread(target=collect)
        th.start()
        t0 = time.perf_counter()
        due = t0
        for r, gap in zip(reqs, gaps):
            if open_loop:
                due += gap
                now = time.perf_counter()
                if due > now:
                    time.sleep(due - now)
            t = submit(srv, r)
            with cv:
                tickets.append(t)
                cv.notify()
        th.join()
        makespan = time.perf_counter() - t0
        st = srv.stats()
        srv.close()
        return {"p50_s": round(float(np.percentile(lat, 50)), 4),
                "p99_s": round(float(np.percentile(lat, 99)), 4),
                "volumes_per_s": round(count / makespan, 3),
                "identical_to_alone": "%d/%d" % (same[0], len(serial)),
                "max_concurrent": st["max_concurrent"],
                "peak_hbm_gb": round(st["peak_bytes"] / 2**30, 2)}

    out = {"requests": count, "lambda_per_s": round(lam, 3),
           "mean_service_s": round(mean_s, 4), "serial_checked": len(check)}
    print(json.dumps({"serving_progress": dict(out)}), file=sys.stderr, flush=True)
    out["plain"] = {"slots": 1, "poisson": run(1, True)}
    print(json.dumps({"serving_progress": out["plain"]}), file=sys.stderr, flush=True)
    out["chosen"] = {"slots": 4, "poisson": run(4, True)}
    print(json.dumps({"serving_progress": out["chosen"]}), file=sys.stderr, flush=True)
    if saturated:
        out["plain"]["saturated"] = run(1, False)
        out["chosen"]["saturated"] = run(4, False)
    out["workload"] = ("FDK or OSC-TV (10 it x 10 subsets) on %s^3 volumes, %s views, geom 0/1/2, "
                       "FP32 or FP16 storage (OSC-TV FP16 residual views); Poisson arrivals at 80%% "
                       "of the one-at-a-time service rate (%.3f /s)%s"
                       % ("/".join(map(str, sizes)), "/".join(map(str, views)), lam,
                          ", and all requests queued at once (saturated)" if saturated else ""))
    return out


def config5(args):
    """The serving workload at its stated mix: Poisson arrivals at ~80% load of FDK or
    OSC-TV (10 x 10) requests on 128^3..512^3 volumes with 60..720 views, random
    geometry, FP32 or FP16 storage; p50/p99 and volumes/s of a one-slot and a four-slot
    server, results checked against one-request calls on a seeded sample.  Opt-in
    (bench.py --config5 [--serve-requests N]): at ~0.3-0.5 s of GPU work per request
    and two servers it runs for ~1 minute per 100 requests (the stated 2,000
    requests take over 40 minutes of one GPU)."""
    line = {"config5": serving(args.serve_requests, seed=11, sizes=(128, 256, 384, 512),
                               size_p=(0.25, 0.25, 0.25, 0.25), views=(60, 240, 480, 720),
                               serial_sample=min(60, args.serve_requests), saturated=False,
                               budget_gb=96)}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
