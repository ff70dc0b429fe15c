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
CU_SOURCES = ["k_exact.cu", "k_compact.cu", "k_shortlist.cu", "k_noalloc.cu", "k_sampson.cu", "k_features.cu", "k_tracks.cu"]
CPP_SOURCES = ["slm.cpp"]
HEADERS = ["pack.cuh", "ptx.cuh", "slm_internal.h", "slm_shortlist.h", "fmath_cr.h", "fmath_tables.h"]


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


SAN_LIB = os.path.join(OUT, "asan", "libslm.so")


def build_sanitized(verbose: bool = False) -> str:
    """libslm with its host C++ (the context, stores, plans, autotuner, serving
    and coalescing threads) under AddressSanitizer and UBSan, the CUDA
    translation units as in build(). Load it through SLM_LIB_PATH with the
    sanitizer runtimes preloaded, e.g.

        LD_PRELOAD=$(gcc -print-file-name=libasan.so):$(gcc -print-file-name=libubsan.so) \\
        ASAN_OPTIONS=detect_leaks=0:protect_shadow_gap=0 SLM_LIB_PATH=<this path> \\
        python -m pytest tests -m gpu

    (leak detection off: the Python interpreter itself is not instrumented;
    protect_shadow_gap=0: the CUDA driver maps memory where ASan would
    otherwise reserve its shadow gap)."""
    build(verbose=verbose)  # the CUDA objects
    d = os.path.dirname(SAN_LIB)
    os.makedirs(d, exist_ok=True)
    cuda = os.path.dirname(os.path.dirname(_nvcc()))
    obj = os.path.join(d, "slm.cpp.o")
    cmds = [["g++", "-std=c++17", "-O1", "-g", "-fPIC", "-fno-omit-frame-pointer", "-fsanitize=address,undefined",
             "-ffp-contract=off", "-I", INCLUDE, "-I", CSRC, "-I", os.path.join(cuda, "include"), "-c",
             os.path.join(CSRC, "slm.cpp"), "-o", obj],
            ["g++", "-shared", "-fsanitize=address,undefined", "-o", SAN_LIB, obj,
             *[os.path.join(OUT, s + ".o") for s in CU_SOURCES],
             "-L", os.path.join(cuda, "lib64"), "-lcudart_static", "-ldl", "-lpthread", "-lrt"]]
    for cmd in cmds:
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode:
            raise RuntimeError(f"sanitized libslm build failed: {' '.join(cmd)}\n{r.stderr}")
    return SAN_LIB


if __name__ == "__main__":
    if "--sanitize" in sys.argv:
        print(build_sanitized(verbose="-v" in sys.argv))
    else:
        print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
