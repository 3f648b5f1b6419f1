"""Build libcanvas_ity_gb300.so in-tree (nvcc for sm_103a, g++ for host code).

The CUDA sources are compiled with --fmad=false so every float operation
rounds like the reference's x86-64 SSE code; host sources with
-ffp-contract=off for the same reason (the Arm host would otherwise fuse).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIB_DIR, "libcanvas_ity_gb300.so")

CUDA_SOURCES = ["engine.cu"]
HOST_SOURCES = ["canvas.cpp", "capi.cpp", "server.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-v"]
HOST_FLAGS = ["-O3", "-std=c++17", "-ffp-contract=off", "-fPIC", "-Wall", "-Wno-unused-function"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps() -> list:
    out = []
    for d in (CSRC, os.path.join(HERE, "..", "include")):
        for f in os.listdir(d):
            out.append(os.path.join(d, f))
    return out


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile the CUDA engine and host library; returns the .so path."""
    if not force and os.path.exists(LIB):
        newest = max(os.path.getmtime(p) for p in _deps())
        if os.path.getmtime(LIB) >= newest:
            return LIB
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    nvcc = _nvcc()
    jobs, objs = [], []
    for src in CUDA_SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
        jobs.append((cmd, src))
        objs.append(obj)
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    for src in HOST_SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        cmd = ["g++", *HOST_FLAGS, "-I", cuda_inc, "-c", os.path.join(CSRC, src), "-o", obj]
        jobs.append((cmd, src))
        objs.append(obj)
    procs = [(subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True), s)
             for c, s in jobs]
    failed = []
    for p, s in procs:
        out, _ = p.communicate()
        if verbose or p.returncode:
            sys.stderr.write(f"--- {s}\n{out}")
        if p.returncode:
            failed.append(s)
    if failed:
        raise RuntimeError(f"compilation failed: {failed}")
    tmp = LIB + ".tmp"
    subprocess.check_call([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lstdc++"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
