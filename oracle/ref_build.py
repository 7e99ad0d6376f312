"""Recipe: compile the reference's own CUDA sources, unmodified, into sm_103a cubins.

TEST INFRASTRUCTURE ONLY (the oracle's reference runs; see oracle/reference.py).

Each of the six reference files is compiled where it lies under /root/reference
with ``nvcc -cubin`` (device code only, so the x86 host code of the MEX gateways
is parsed but not built).  Flags follow the reference's own build line
(compile.m:25-68: ``nvcc -c <file>.cu -O3 -gencode ...``), with the architecture
set to sm_103a.  Two include-time aids make CUDA 13 accept the sources without
editing them:
  * the MEX stub header of this repository (mex-cuda-ct_gb300/mex/mexstub/mex.h)
    stands in for MATLAB's mex.h, which only the host code uses;
  * oracle/ref_compat.h, force-included, restates the texture and surface
    references that CUDA 12 removed (four of the six files use them) as
    __device__ handles to texture / surface objects.
Outputs go to oracle/_ref/ only.  The cubins hold device code, so the same files
load on any host architecture; the launcher that loads them (ref_launch.cu) is
compiled on the machine that runs it.

Run from the repository root:  python oracle/ref_build.py
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REF = "/root/reference"
OUT = os.path.join(HERE, "_ref")
MEXSTUB = os.path.join(ROOT, "mex-cuda-ct_gb300", "mex", "mexstub")
COMPAT = os.path.join(HERE, "ref_compat.h")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (reference source, cubin name, needs the texture/surface compatibility header)
SOURCES = [
    ("projection_kernels/CUDAmex_FP.cu", "ref_fp.cubin", True),
    ("projection_kernels/CUDAmex_BP.cu", "ref_bp.cubin", True),
    ("projection_kernels/CUDAmex_general3D_FP.cu", "ref_g3d_fp.cubin", True),
    ("projection_kernels/CUDAmex_general3D_BP.cu", "ref_g3d_bp.cubin", True),
    ("iterative_reconstruction/CUDAmex_oscIter.cu", "ref_osc.cubin", True),
    ("iterative_reconstruction/CUDAmex_TVmin_3D.cu", "ref_tv.cubin", False),
]


def available() -> bool:
    return os.path.isdir(REF)


def _nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def _one(src: str, name: str, compat: bool, force: bool) -> str:
    path = os.path.join(REF, src)
    out = os.path.join(OUT, name)
    deps = [path, COMPAT, os.path.join(MEXSTUB, "mex.h"), __file__]
    if not force and os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(d) for d in deps):
        return out
    cmd = [_nvcc(), "-cubin", *ARCH, "-O3", "-I", MEXSTUB, "-w", "-o", out + ".tmp", path]
    if compat:
        cmd[1:1] = ["-include", COMPAT]
    else:
        cmd[1:1] = ["-DcudaThreadSynchronize=cudaDeviceSynchronize"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    os.replace(out + ".tmp", out)
    return out


def build(force: bool = False) -> list[str]:
    """Build every cubin into oracle/_ref/ (no-op when the reference is absent)."""
    if not available():
        return []
    os.makedirs(OUT, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        return list(ex.map(lambda s: _one(*s, force), SOURCES))


if __name__ == "__main__":
    for p in build(force="--force" in sys.argv):
        print(p)
