"""Build recipe for the checker (TEST INFRASTRUCTURE ONLY).

* ``build_oracle()``  -- gcc builds oracle/_build/liboracle{32,64}.so from
  splat_oracle.c (the CPU restatement).
* ``build_ref_cubins(ref_dir)`` -- nvcc compiles the reference's own kernel
  sources lib/kernels/{forward,backward,other}.cu, unmodified and where they
  lie under ``ref_dir``, into device-only cubins in oracle/_ref/.  The
  reference's CMake build compiles them with ``-std=c++17`` for the native
  architecture (CMakeLists.txt:3-7); on a GB300 that is sm_103, which is what
  is used here.  Only run where the reference sources exist; the cubins then
  travel with the working tree (they are not host binaries).
* ``build_harness()`` -- nvcc builds oracle/_build/libref_harness.so from
  ref_harness.cu (host code of this repository that loads those cubins and
  repeats lib/ops.cu's orchestration with CUB from the CUDA toolkit).

Usage: ``python oracle/build.py [--ref /path/to/reference]``.  The
reference sources are looked up in ``--ref``, else in the environment
variable SPLAT_REFERENCE_DIR, else in REFERENCE_DIR_DEFAULT below (where this
recipe's build machine keeps the read-only reference checkout).  Machines
without the sources (the GPU machine) skip the cubin build and use the cubins
that travelled with the working tree.
"""

from __future__ import annotations

import argparse
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
REF_ARCH = ["-gencode", "arch=compute_103,code=sm_103"]
NVCC = os.environ.get("NVCC", "nvcc")
REFERENCE_DIR_DEFAULT = "/root/reference"


def reference_dir() -> str:
    """Where the reference sources are read from (SPLAT_REFERENCE_DIR
    overrides the recipe's default)."""
    return os.environ.get("SPLAT_REFERENCE_DIR", REFERENCE_DIR_DEFAULT)


def _stale(out: str, *srcs: str) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_oracle(force: bool = False) -> None:
    """gcc: fp32 and fp64 builds of splat_oracle.c into oracle/_build/."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "splat_oracle.c")
    for prec, extra in (("32", []), ("64", ["-DORACLE_F64"])):
        out = os.path.join(BUILD, f"liboracle{prec}.so")
        if not force and not _stale(out, src):
            continue
        cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
               "-fno-fast-math", *extra, "-o", out, src, "-lm"]
        subprocess.check_call(cmd)


def ref_cubins_present() -> bool:
    return all(os.path.exists(os.path.join(REF_OUT, f"{n}.cubin"))
               for n in ("forward", "backward", "other"))


def build_ref_cubins(ref_dir: str, force: bool = False) -> bool:
    lib = os.path.join(ref_dir, "lib")
    if not os.path.isdir(lib):
        return False
    os.makedirs(REF_OUT, exist_ok=True)
    procs = []
    for name in ("forward", "backward", "other"):
        src = os.path.join(lib, "kernels", f"{name}.cu")
        out = os.path.join(REF_OUT, f"{name}.cubin")
        if not force and not _stale(out, src):
            continue
        cmd = [NVCC, "-cubin", "-std=c++17", *REF_ARCH, "-I", lib, "-I",
               os.path.join(lib, "kernels"), "-o", out, src]
        procs.append((cmd, subprocess.Popen(cmd)))
    for cmd, p in procs:
        if p.wait() != 0:
            raise RuntimeError("reference cubin build failed: " + " ".join(cmd))
    return True


def build_harness(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "ref_harness.cu")
    out = os.path.join(BUILD, "libref_harness.so")
    if force or _stale(out, src):
        cmd = [NVCC, "-shared", "-Xcompiler", "-fPIC", "-std=c++17", "-O2", *REF_ARCH, "-o",
               out, src, "-lcuda"]
        subprocess.check_call(cmd)
    return out


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--no-harness", action="store_true")
    a = ap.parse_args()
    build_oracle(a.force)
    built = build_ref_cubins(a.ref or reference_dir(), a.force)
    print("reference cubins:", "built" if built else "skipped (no sources)",
          "present" if ref_cubins_present() else "absent")
    if not a.no_harness and ref_cubins_present():
        print("harness:", build_harness(a.force))


if __name__ == "__main__":
    main()
