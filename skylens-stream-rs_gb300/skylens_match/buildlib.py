"""Build recipe for libslm.so: nvcc for sm_103a, parallel translation units.

Produces ``skylens-stream-rs_gb300/build/libslm.so`` (git-ignored). Runs the
same way on x86_64 and aarch64 hosts; no host-architecture flags are used.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)                      # skylens-stream-rs_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(REPO, "include")
OUT = os.path.join(ROOT, "build")
LIB = os.path.join(OUT, "libslm.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["k_exact.cu", "k_compact.cu", "k_shortlist.cu", "k_noalloc.cu"]
CPP_SOURCES = ["slm.cpp"]
HEADERS = ["pack.cuh", "ptx.cuh", "slm_internal.h", "slm_shortlist.h"]


def _nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return p


def _sources():
    return [s for s in CU_SOURCES + CPP_SOURCES if os.path.exists(os.path.join(CSRC, s))]


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src, os.path.join(INCLUDE, "slm.h")] + [os.path.join(CSRC, h) for h in HEADERS]
    return any(os.path.exists(d) and os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every CUDA/C++ source of libslm for sm_103a and link libslm.so."""
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    common = ["-std=c++17", "-O3", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-I", INCLUDE, "-I", CSRC]
    jobs = []
    objs = []
    for src in _sources():
        path = os.path.join(CSRC, src)
        obj = os.path.join(OUT, src + ".o")
        objs.append(obj)
        if not force and not _stale(obj, path):
            continue
        if src.endswith(".cu"):
            cmd = [nvcc, *ARCH, "-lineinfo", "--fmad=false", *common, "-c", path, "-o", obj]
        else:
            cmd = [nvcc, *common, "-x", "c++", "-c", path, "-o", obj]
        jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode:
            raise RuntimeError(f"libslm build failed: {' '.join(cmd)}\n{r.stderr}")
        return r

    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            list(ex.map(run, jobs))
    if force or jobs or not os.path.exists(LIB):
        tmp = LIB + f".tmp{os.getpid()}"
        run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-cudart=static"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
