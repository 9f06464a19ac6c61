"""Builds the engine's shared library, cyrsoxs_gb300/_build/libcyrsoxs_gb300.so,
for sm_103a with nvcc (one translation unit; no torch or cmake involved).

    python -m cyrsoxs_gb300.build          # build (no-op when up to date)
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libcyrsoxs_gb300.so")
SOURCES = ["engine.cu"]
DEPS = SOURCES + ["kernels.cuh", "fields.cuh", "fp64.cuh", "geometry.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, d) for d in DEPS] + [os.path.join(REPO, "include", "cyrsoxs.h"), __file__]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp"
    # host float geometry (k frames, rotations, warp coefficients) without fused multiply-adds, so that it
    # rounds as the reference's x86 build and the oracle do on every host architecture
    cmd = [nvcc(), "-std=c++17", "-O3", "-lineinfo", *ARCH, "-shared", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off",
           "-Xcompiler", "-fvisibility=hidden", "-DCYR_BUILDING_LIBRARY", "-I", os.path.join(REPO, "include"),
           *[os.path.join(CSRC, s) for s in SOURCES], "-o", tmp, "-lcudart"]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
