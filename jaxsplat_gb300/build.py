"""Build libsplat.so (the CUDA kernels + C ABI) in-tree for sm_103a.

    python -m jaxsplat_gb300.build [--verbose-ptxas]

Each translation unit is compiled in parallel with nvcc, then linked into
jaxsplat_gb300/_lib/libsplat.so.  nvcc's default floating-point contraction
(-fmad=true) is kept on purpose: the reference is compiled with it, and the
integer outputs (tile counts, keys, final_idx) depend on the rounding of the
float expressions that feed them.
"""

from __future__ import annotations

import argparse
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libsplat.so")
SOURCES = ["api.cu", "project.cu", "sort.cu", "raster.cu", "fit.cu", "noalloc.cu", "batch.cu", "gemm_tc.cu", "nn.cu"]
HEADERS = ["splat_internal.cuh", "splat_math.cuh", "project_math.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr", "-Xcompiler", "-fvisibility=hidden"]


def _deps():
    inc = os.path.join(os.path.dirname(HERE), "include", "splat.h")
    return [os.path.join(CSRC, h) for h in HEADERS] + [inc, os.path.abspath(__file__)]


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    deps = _deps()
    objs, procs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ_DIR, src.replace(".cu", ".o"))
        objs.append(o)
        if force or verbose_ptxas or _stale(o, [s, *deps]):
            cmd = [NVCC, "-c", *ARCH, *FLAGS, "-o", o, s]
            if verbose_ptxas:
                cmd.insert(1, "-Xptxas=-v")
            procs.append((cmd, subprocess.Popen(cmd)))
    for cmd, p in procs:
        if p.wait() != 0:
            raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if force or procs or _stale(LIB, objs):
        cmd = [NVCC, "-shared", *ARCH, "-o", LIB, *objs, "-lcudart"]
        subprocess.check_call(cmd)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose-ptxas", action="store_true")
    a = ap.parse_args()
    print(build(a.force, a.verbose_ptxas), file=sys.stderr)
