"""The standalone C++ benchmark (mex-cuda-ct_gb300/bench/mexct_bench.cpp): the C ABI
with cudaMalloc buffers and CUDA events, no Python or torch in the process."""
import json
import os
import subprocess

import pytest


def _binary():
    import __graft_entry__ as ge

    return ge._builder().build_bench()


def test_cpp_bench_builds(lib):
    assert os.access(_binary(), os.X_OK)


@pytest.mark.gpu
def test_cpp_bench_prints_one_json_line(cuda):
    r = subprocess.run([_binary(), "--size", "128", "--views", "90", "--steps", "2", "--warmup", "1"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["unit"] == "GUPS" and d["value"] > 0 and d["e2e"]["value"] > 0
    assert d["fp_ms"] > 0 and d["bp_ms"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 4 * (128 ** 3 + 128 * 128 * 90)
