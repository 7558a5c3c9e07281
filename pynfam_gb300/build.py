"""In-tree build of the CUDA library ``libpnfam_gb300.so`` (sm_103a only).

``python -m pynfam_gb300.build`` compiles ``csrc/pnfam_gpu.cu`` with nvcc into
the package directory.  No torch, no cmake: one translation unit, one
``-gencode``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libpnfam_gb300.so")
SOURCES = ["pnfam_gpu.cu"]
DEPS = SOURCES + ["pnfam_kernels.cuh", "tc.cuh", "pair_gemm.cuh", "tbc.cuh", "hfb.cuh"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc_path() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the pnFAM CUDA library cannot be built")


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    inc = os.path.join(os.path.dirname(HERE), "include", "pnfam_gpu.h")
    files = [os.path.join(CSRC, f) for f in DEPS] + [inc]
    return any(os.path.getmtime(f) > t for f in files if os.path.exists(f))


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    cmd = [nvcc_path(), ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-pthread", "-shared",
           "-o", LIB + ".tmp"] + [os.path.join(CSRC, s) for s in SOURCES]
    if verbose:
        print(" ".join(cmd))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed:\n" + r.stdout + r.stderr)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
