"""Build recipe of libsmartcore_gb300.so (sm_103a only, in-tree).

    python -m smartcore_gb300.build        # or __graft_entry__.build()

Each source is compiled in parallel with nvcc (one -gencode: compute_103a /
sm_103a), then linked into smartcore_gb300/_build/libsmartcore_gb300.so.
exact.cu and batch.cu are compiled with -fmad=false: their FP64 kernels
reproduce the reference's unfused operation order bit for bit.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libsmartcore_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
               "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"] + ARCH

SOURCES = {
    "capi.cu": [],
    "exact.cu": ["-fmad=false"],
    "update.cu": [],
    "split.cu": [],
    "knn_split.cu": [],
    "noalloc.cu": [],
    "batch.cu": ["-fmad=false"],
    "host_rng.cpp": None,  # host compiler
}


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build smartcore_gb300")
    return p


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(os.path.dirname(HERE), "include", "smartcore_gb300.h")]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    jobs = []
    objs = []
    for src, extra in SOURCES.items():
        obj = os.path.join(BUILD, src + ".o")
        path = os.path.join(CSRC, src)
        if extra is None:
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-c", path, "-o", obj]
        else:
            cmd = [nvcc()] + NVCC_COMMON + extra + ["-c", path, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        jobs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
        objs.append(obj)
    failed = []
    for src, p in jobs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((src, out))
        elif verbose and out.strip():
            print(out)
    if failed:
        raise RuntimeError("build failed:\n" + "\n".join(f"--- {s}\n{o}" for s, o in failed))
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcuda"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
