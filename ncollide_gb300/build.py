"""Builds libncg.so (the CUDA kernels + C ABI) in-tree with nvcc for sm_103a.

The library is compiled with -fmad=false: no multiply-add contraction, IEEE
division and square root, so each pair's result is a deterministic function
of its inputs in the reference's evaluation order.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "_lib")
# NCG_LIB selects another build of the library (launch-tuning variants built
# with NCG_DEFINES, e.g. "-DNCG_EPA_THREAD_VC=64"); the default is the in-tree build.
LIB_PATH = os.environ.get("NCG_LIB") or os.path.join(LIB_DIR, "libncg.so")
SOURCES = ["ncg_kernels.cu", "ncg_gjk.cu", "ncg_epa_stages.cu", "ncg_gjk_f32.cu", "ncg_epa_stages_f32.cu",
           "ncg_mlp.cu", "ncg_toi.cu", "ncg_bp.cu", "ncg_manifold.cu", "ncg_hull.cpp"]
HEADERS = ["ncg_core.cuh", "ncg_epa.cuh", "ncg_dw.cuh", "ncg_query.cuh", "ncg_tc.cuh", "ncg_mlp.h", "ncg_toi.cuh", "ncg_toi.h", "ncg_sort.cuh", "ncg_pipeline.cuh", "ncg_bp.h", "ncg_manifold.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-O2", "-Xcompiler", "-ffp-contract=off", "-shared"]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stale():
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    deps.append(os.path.join(HERE, "..", "include", "ncg.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False, extra=()):
    """Compiles each translation unit in parallel, then links libncg.so."""
    if not force and not _stale():
        return LIB_PATH
    os.makedirs(LIB_DIR, exist_ok=True)
    tag = os.path.splitext(os.path.basename(LIB_PATH))[0]
    objs = [os.path.join(LIB_DIR, f"{tag}_{os.path.splitext(s)[0]}.o") for s in SOURCES]
    flags = [f for f in NVCC_FLAGS if f != "-shared"] + os.environ.get("NCG_DEFINES", "").split()
    cmds = [[nvcc(), *ARCH, *flags, *extra, "-c", "-o", o, os.path.join(CSRC, s)] for s, o in zip(SOURCES, objs)]
    if verbose:
        for c in cmds:
            print(" ".join(c), file=sys.stderr)
    procs = [subprocess.Popen(c) for c in cmds]
    rcs = [p.wait() for p in procs]
    if any(rcs):
        raise RuntimeError(f"nvcc failed: {rcs}")
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    tmp = LIB_PATH + ".tmp"
    link = [nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", tmp, *objs]
    subprocess.run(link, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, extra=["-Xptxas", "-v"] if "-v" in sys.argv else [])
