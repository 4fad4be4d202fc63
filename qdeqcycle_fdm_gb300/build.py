"""Build the sm_103a shared library ``_build/libqdeq_gb300.so`` with nvcc.

Each CUDA translation unit compiles in parallel for exactly one target,
``-gencode arch=compute_103a,code=sm_103a``; the library links only cudart.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libqdeq_gb300.so")
SOURCES = ["capi.cu", "mg.cu", "mg_fused.cu", "fault.cu", "medium.cu", "dropin.cpp", "noalloc.cu", "mg_graph.cu", "unet.cu", "io.cu", "history.cu", "autotune.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build qdeq_gb300")
    return p


def _stale(src_paths, target) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(p) > t for p in src_paths)


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    for h in ("qdeq.h", "qdeq_unet.h"):
        headers.append(os.path.join(os.path.dirname(HERE), "include", h))
    objs = []
    jobs = []
    for src in SOURCES:
        sp = os.path.join(CSRC, src)
        obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        objs.append(obj)
        if force or _stale([sp] + headers, obj):
            cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra_flags, "-c", sp, "-o", obj]
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        futs = [ex.submit(subprocess.run, c, capture_output=True, text=True) for c in jobs]
        for c, f in zip(jobs, futs):
            r = f.result()
            if verbose or r.returncode != 0:
                print(" ".join(c))
                print(r.stdout, r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {c[-3]}")
    if force or jobs or _stale(objs, LIB):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            print(r.stdout, r.stderr)
            raise RuntimeError("link of libqdeq_gb300.so failed")
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
