"""Build libmexct.so (CUDA, sm_103a) in-tree: mex-cuda-ct_gb300/_build/libmexct.so.

Each translation unit is compiled by nvcc in parallel, then linked into one shared
library with the C ABI of include/mexct.h.  No torch, cmake or Python extension
machinery is involved: the library is plain CUDA C++ that MEX gateways, a C++ bench
or ctypes can load.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libmexct.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["k_proj.cu", "k_slab.cu", "k_iter.cu", "batch.cu", "api.cu", "ops.cu", "solver.cu",
           "serve.cu", "noalloc.cu", "tune.cu", "subvol.cu", "solver_ooc.cu", "fileio.cpp",
           "mat73.cpp"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmexct")
    return path


def _deps(src: str) -> list[str]:
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    incs = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    return [src] + hdrs + incs


def _compile(src: str, verbose: bool) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in _deps(path)):
        return obj
    cmd = [nvcc(), "-c", path, "-o", obj + ".tmp", *ARCH, "-O3", "-lineinfo", "-std=c++17",
           "-Xcompiler", "-fPIC", "-Xcompiler", "-O2", "--expt-relaxed-constexpr",
           "-I", os.path.join(ROOT, "include")]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    if verbose:
        sys.stderr.write(r.stderr)
    os.replace(obj + ".tmp", obj)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    if force:
        for s in srcs:
            o = os.path.join(BUILD, s.replace(".cu", ".o"))
            if os.path.exists(o):
                os.remove(o)
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs):
        return LIB
    cmd = [nvcc(), "-shared", "-o", LIB + ".tmp", *objs, *ARCH, "-cudart", "shared",
           "-Xlinker", "-rpath,/usr/local/cuda/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(LIB + ".tmp", LIB)
    return LIB


MEX_DIR = os.path.join(HERE, "mex")
MEX_LIB = os.path.join(BUILD, "libmexct_mex.so")


def build_mex_stub(force: bool = False) -> str:
    """The MEX gateways against the stub mex.h, linked into one shared
    library with a by-name call interface (mxs_call), for testing without MATLAB."""
    lib = build(force=force)
    srcs = sorted(os.path.join(MEX_DIR, f) for f in os.listdir(MEX_DIR) if f.endswith(".cpp"))
    srcs.append(os.path.join(MEX_DIR, "mexstub", "mexstub.cpp"))
    deps = srcs + [os.path.join(MEX_DIR, "gateway.h"), os.path.join(MEX_DIR, "mexstub", "mex.h"),
                   os.path.join(ROOT, "include", "mexct.h"),
                   os.path.join(ROOT, "include", "mexct_solver.h"), lib]
    if (not force and os.path.exists(MEX_LIB)
            and os.path.getmtime(MEX_LIB) >= max(os.path.getmtime(d) for d in deps)):
        return MEX_LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-DMEXCT_STUB",
           "-I", os.path.join(MEX_DIR, "mexstub"), "-I", os.path.join(ROOT, "include"),
           "-o", MEX_LIB + ".tmp", *srcs, "-L", BUILD, "-lmexct", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("MEX stub build failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(MEX_LIB + ".tmp", MEX_LIB)
    return MEX_LIB


BENCH_SRC = os.path.join(HERE, "bench", "mexct_bench.cpp")
BENCH_BIN = os.path.join(BUILD, "mexct_bench")


def build_bench(force: bool = False) -> str:
    """The standalone C++ benchmark (bench/mexct_bench.cpp) against libmexct:
    the C ABI and the CUDA runtime only (shared, as libmexct uses it)."""
    lib = build(force=force)
    deps = [BENCH_SRC, os.path.join(ROOT, "include", "mexct.h"), lib]
    if (not force and os.path.exists(BENCH_BIN)
            and os.path.getmtime(BENCH_BIN) >= max(os.path.getmtime(d) for d in deps)):
        return BENCH_BIN
    cmd = [nvcc(), "-O2", "-std=c++17", "-x", "c++", BENCH_SRC, "-o", BENCH_BIN + ".tmp",
           "-I", os.path.join(ROOT, "include"), "-L", BUILD, "-lmexct", "-cudart", "shared",
           "-Xlinker", "-rpath,$ORIGIN", "-Xlinker", "-rpath,/usr/local/cuda/lib64",
           "-Xlinker", "-export-dynamic"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("C++ bench build failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(BENCH_BIN + ".tmp", BENCH_BIN)
    return BENCH_BIN


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
    print(build_mex_stub())
    print(build_bench())
