"""Benchmark: cone-beam FP + BP GUPS at 512^3 x 720 views on one GB300.

A step is one forward projection (volume -> 720-view sinogram) plus one
backprojection (sinogram -> volume) of a 512^3 float32 random-ellipsoid phantom,
geomFlag 2 (cone), SAD 1000, through the C ABI of libmexct.

  value  = whole-job GUPS = 2 * 512^3 * 720 * steps * n_ranks / max-rank time
           (device-resident inputs, CUDA events on the launching stream)
  e2e    = the same metric through the host entry points mexct_fp / mexct_bp
           with pinned host buffers: H2D and D2H copies inside the timed region
  --impl reference times the FP64 C++/OpenMP CPU implementation on a bounded
  sample of the same workload (the reference has no CPU path of its own; the
  oracle restates its algorithm).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Multi-GPU: one process per GPU (torchrun); every rank runs the full problem
(replicas: the path is independent per problem), value aggregates all ranks.
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


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=512)
    ap.add_argument("--views", type=int, default=720)
    ap.add_argument("--geom", type=int, default=2)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
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


def cpu_sample(size, views, geom, seconds_target=15.0):
    """Time the FP64 oracle (FP + BP) on a bounded view sample; returns GUPS."""
    import oracle
    from mexct import phantoms

    oracle.build()
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    n = size
    vol = phantoms.ellipsoids(n, count=12, seed=2024, nz=n)
    ang_all = phantoms.angles_full(views)
    k = 1
    gups = []
    t_used = 0.0
    while True:
        ang = ang_all[: k]
        t0 = time.perf_counter()
        sino = oracle.fp(vol, 1000.0, ang, k, geom).astype(np.float32)
        oracle.bp(sino, 1000.0, ang, geom)
        dt = time.perf_counter() - t0
        t_used += dt
        gups.append(2.0 * n ** 3 * k / dt / 1e9)
        if t_used > seconds_target or k >= views:
            break
        k = min(views, k * 2)
    return {"value": round(gups[-1], 4), "unit": "GUPS", "cores": threads, "kind": "port",
            "sample": "%d^3 volume, FP+BP over %d of %d cone views (FP64 C++/OpenMP oracle, "
                      "%d threads)" % (n, k, views, threads)}


def run_reference(args, rank):
    if rank != 0:
        return
    s = cpu_sample(args.size, args.views, args.geom)
    steps, warm = args.steps, args.warmup
    line = {"metric": "FP+BP GUPS, cone geomFlag 2, %d^3 x %d views" % (args.size, args.views),
            "value": s["value"], "unit": "GUPS", "n_gpus": args.gpus, "steps": steps,
            "warmup": warm, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded ellipsoid phantom)",
            "impl": "reference",
            "config": {"workload": "cone FP+BP %d^3 x %d views, SAD 1000" % (args.size, args.views)},
            "cpu_baseline": s,
            "e2e": {"value": s["value"], "unit": "GUPS", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


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
    from mexct import _lib, phantoms
    from mexct import ops

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    lib = _lib.load()

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
    sptr = ctypes.c_void_p(stream.cuda_stream)
    angp = ctypes.c_void_p(ang.ctypes.data)

    def step():
        _lib.check(lib.mexct_fp_dev(None, ctypes.c_void_p(vol.data_ptr()), n, n, 1000.0, angp,
                                    views, geom, ctypes.c_void_p(sino.data_ptr()), sptr))
        _lib.check(lib.mexct_bp_dev(None, ctypes.c_void_p(sino.data_ptr()), n, n, views, 1000.0,
                                    angp, geom, ctypes.c_void_p(rec.data_ptr()), sptr))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    # Per-operator timing (events on the launching stream) for the roofline.
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    fp_ms, bp_ms = [], []
    for _ in range(max(1, min(2, args.steps))):
        with torch.cuda.stream(stream):
            ev[0].record(stream)
            _lib.check(lib.mexct_fp_dev(None, ctypes.c_void_p(vol.data_ptr()), n, n, 1000.0, angp,
                                        views, geom, ctypes.c_void_p(sino.data_ptr()), sptr))
            ev[1].record(stream)
            _lib.check(lib.mexct_bp_dev(None, ctypes.c_void_p(sino.data_ptr()), n, n, views,
                                        1000.0, angp, geom, ctypes.c_void_p(rec.data_ptr()), sptr))
            ev[2].record(stream)
        stream.synchronize()
        fp_ms.append(ev[0].elapsed_time(ev[1]))
        bp_ms.append(ev[1].elapsed_time(ev[2]))

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
    ms = t0.elapsed_time(t1)
    if dist is not None:
        tt = torch.tensor([ms], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms = float(tt.item())
    ms_step = ms / args.steps
    gups = 2.0 * N * views * args.steps * world / (ms / 1e3) / 1e9

    # e2e through the host entry points (pinned host buffers).
    e2e = None
    if not args.no_e2e:
        vol_pin = torch.from_numpy(np.ascontiguousarray(vol_h.transpose(2, 1, 0))).pin_memory()
        sino_pin = torch.empty((views, n, n), dtype=torch.float32).pin_memory()
        rec_pin = torch.empty((n, n, n), dtype=torch.float32).pin_memory()

        def e2e_step():
            _lib.check(lib.mexct_fp(None, ctypes.c_void_p(vol_pin.data_ptr()), n, n, 1000.0, angp,
                                    views, geom, ctypes.c_void_p(sino_pin.data_ptr())))
            _lib.check(lib.mexct_bp(None, ctypes.c_void_p(sino_pin.data_ptr()), n, n, views,
                                    1000.0, angp, geom, ctypes.c_void_p(rec_pin.data_ptr())))

        e2e_step()
        if dist is not None:
            dist.barrier()
        k = max(1, min(args.steps, 3))
        t = time.perf_counter()
        for _ in range(k):
            e2e_step()
        el = time.perf_counter() - t
        if dist is not None:
            tt = torch.tensor([el], device=dev)
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            el = float(tt.item())
        e2e = {"value": round(2.0 * N * views * k * world / el / 1e9, 3), "unit": "GUPS",
               "h2d_bytes_per_step": 4 * (N + P * views), "d2h_bytes_per_step": 4 * (P * views + N)}

    peak, peak_kind = hbm_peak()
    fp_t = float(np.median(fp_ms)) / 1e3
    bp_t = float(np.median(bp_ms)) / 1e3
    fp_bytes = 4.0 * (N + P * views)
    bp_bytes = 4.0 * (P * views + N)
    dom = ("fp", fp_t, fp_bytes) if fp_t >= bp_t else ("bp", bp_t, bp_bytes)
    achieved = dom[2] / dom[1] / 1e9
    line = {
        "metric": "FP+BP GUPS, cone geomFlag 2, %d^3 x %d views" % (n, views),
        "value": round(gups, 3), "unit": "GUPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_step, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded 12-ellipsoid phantom)",
        "config": {"workload": "cone FP+BP %d^3 x %d views, SAD 1000, float32" % (n, views),
                   "l2": "inputs larger than L2 (volume 512 MiB, sinogram 720 MiB)",
                   "parallelism": "replicas" if world > 1 else "single"},
        "fp_gups": round(N * views / fp_t / 1e9, 3), "bp_gups": round(N * views / bp_t / 1e9, 3),
        "fp_ms": round(fp_t * 1e3, 3), "bp_ms": round(bp_t * 1e3, 3),
        "roofline": {"bound": "hbm", "kernel": dom[0], "achieved": round(achieved, 2),
                     "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": round(achieved / peak, 5), "traffic": None},
        "clocks": clk,
        "gpu_launches": 3 * args.steps,
        "e2e": e2e,
    }
    if rank == 0 and not args.no_cpu:
        try:
            line["cpu_baseline"] = cpu_sample(min(n, 256), views, geom, seconds_target=10.0)
        except Exception as ex:  # reported, never fatal
            line["cpu_baseline"] = {"error": str(ex)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
