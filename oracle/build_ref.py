#!/usr/bin/env python3
"""Build the reference Cas-OFFinder 3.0.0 from its own sources, for the oracle.

TEST INFRASTRUCTURE.  Compiles the reference's unmodified host sources
(main.cpp, cas-offinder.cpp, read_fasta.cpp, read_twobit.cpp, oclfunctions.cpp)
and its kernels (cas-offinder.cl, compiled as C++) against the host OpenCL
emulator in ref_shim/.  Outputs (git-ignored, never committed):
  oracle/_ref/cas-offinder-ref   the reference program; device C runs its
                                 finder_cpu/comparer_cpu kernels on all host
                                 cores (OpenMP over the NDRange)
  oracle/_ref/ref-predicate      dumps the reference kernel's mismatch
                                 predicate as a 256x256 table

Where the sources come from: the reference checkout named by --ref or by the
COF_REFERENCE_DIR environment variable.  Its sources (the files above and the
headers they include) are first staged unmodified into oracle/_ref/src/,
which is git-ignored like the rest of oracle/_ref/ and travels with the
working tree to machines without the checkout; with neither --ref nor the
variable set, the staged copy is built.  Nothing of the reference is ever
committed.

The reference as shipped cannot be built here: its CMake step generates
config.h and oclkernels.h, and it links a vendor OpenCL runtime that this image
does not have.  ref_shim/ replaces exactly those three things.  It is compiled
with -fsigned-char, the char type of the x86 builds it was written for.

Usage: python oracle/build_ref.py [--ref DIR]
Does nothing (exit 0, message) when neither a checkout nor a staged copy exists.
"""
import argparse
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
STAGE = os.path.join(OUT_DIR, "src")
OUT = os.path.join(OUT_DIR, "cas-offinder-ref")
PRED = os.path.join(OUT_DIR, "ref-predicate")
SOURCES = ["main.cpp", "cas-offinder.cpp", "read_fasta.cpp", "read_twobit.cpp", "oclfunctions.cpp"]
HEADERS = ["cas-offinder.h", "oclfunctions.h", "read_fasta.h", "read_twobit.h"]
KERNELS = "cas-offinder.cl"


def stage(ref):
    """Copies the reference's sources unmodified into oracle/_ref/src/ (only
    files that changed, so the staged timestamps stay put)."""
    os.makedirs(STAGE, exist_ok=True)
    for name in SOURCES + HEADERS + [KERNELS]:
        src, dst = os.path.join(ref, name), os.path.join(STAGE, name)
        if not os.path.exists(dst) or open(src, "rb").read() != open(dst, "rb").read():
            shutil.copyfile(src, dst)


def build(ref=None, quiet=False):
    ref = ref or os.environ.get("COF_REFERENCE_DIR")
    if ref and os.path.isfile(os.path.join(ref, KERNELS)):
        stage(ref)
    if not all(os.path.isfile(os.path.join(STAGE, n)) for n in SOURCES + HEADERS + [KERNELS]):
        if not quiet:
            print("build_ref: no reference checkout (--ref / COF_REFERENCE_DIR) and no staged copy; skipped")
        return None
    shim = os.path.join(HERE, "ref_shim")
    srcs = [os.path.join(STAGE, s) for s in SOURCES] + [os.path.join(shim, "cl_host_emulator.cpp")]
    deps = srcs + [os.path.join(STAGE, h) for h in HEADERS + [KERNELS]] + \
        [os.path.join(shim, f) for f in ("CL/cl.h", "config.h", "oclkernels.h", "ref_predicate.cpp")] + [__file__]
    newest_src = max(os.path.getmtime(s) for s in deps)
    if all(os.path.exists(o) and os.path.getmtime(o) >= newest_src for o in (OUT, PRED)):
        return OUT
    kernels = f'-DCOF_REFERENCE_KERNELS="{os.path.join(STAGE, KERNELS)}"'
    subprocess.run(["g++", "-O2", "-fopenmp", "-fsigned-char", "-w", "-std=c++11", "-I", shim, "-I", STAGE,
                    kernels, *srcs, "-o", OUT], check=True)
    subprocess.run(["g++", "-O1", "-fsigned-char", "-w", "-std=c++11", kernels,
                    os.path.join(shim, "ref_predicate.cpp"), "-o", PRED], check=True)
    return OUT


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None, help="reference checkout (default: $COF_REFERENCE_DIR, else the staged copy)")
    a = ap.parse_args()
    out = build(a.ref)
    print(out or "skipped")
    sys.exit(0)
