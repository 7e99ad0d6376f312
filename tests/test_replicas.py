"""The multi-GPU path of bench.py is replicas only: each rank runs its own step and the
job is timed by the slowest rank; the reference arm runs on rank 0 alone.  These host
parts are checked here with two gloo ranks on the CPU (no GPU)."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_RANK_SCRIPT = r"""
import os, sys
sys.path.insert(0, sys.argv[1])
import torch.distributed as dist
import bench
rank = int(os.environ["RANK"])
dist.init_process_group("gloo", init_method="env://")
got = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")
print("RESULT", rank, got, flush=True)
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_max_over_ranks_two_gloo_ranks():
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", _RANK_SCRIPT, ROOT], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                                      text=True))
    outs = [p.communicate(timeout=120)[0] for p in procs]
    for p, out in zip(procs, outs):
        assert p.returncode == 0, out
    vals = sorted(line.split()[1:] for out in outs for line in out.splitlines()
                  if line.startswith("RESULT"))
    assert vals == [["0", "15.0"], ["1", "15.0"]]


def test_max_over_ranks_single_process_is_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5


def test_reference_arm_runs_on_rank_zero_only():
    """A non-zero rank of the reference arm exits 0 without work or output; rank 0
    prints one JSON line on the same metric and config as the library's arm."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--size", "16",
                        "--views", "8", "--steps", "1", "--warmup", "1"], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == ""
    env = dict(os.environ, RANK="0", WORLD_SIZE="1")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--size", "16",
                        "--views", "8", "--steps", "1", "--warmup", "1"], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    sys.path.insert(0, ROOT)
    import bench

    class A:
        size, views, geom = 16, 8, 2

    assert line["impl"] == "reference" and line["metric"] == bench.metric_name(A)
    assert line["config"]["workload"] == bench.workload_config(A)["workload"]
    assert line["value"] > 0 and line["e2e"]["value"] == line["value"]
