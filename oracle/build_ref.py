#!/usr/bin/env python3
"""Build the reference Cas-OFFinder 3.0.0 from its own sources, for the oracle.

TEST INFRASTRUCTURE.  Compiles the reference's unmodified host sources
(main.cpp, cas-offinder.cpp, read_fasta.cpp, read_twobit.cpp, oclfunctions.cpp)
and its kernels (cas-offinder.cl, compiled as C++) where they lie under the
reference checkout, against the host OpenCL emulator in ref_shim/.  Outputs
(git-ignored): oracle/_ref/cas-offinder-ref, and oracle/_ref/ref-predicate,
which dumps the reference kernel's mismatch predicate as a 256x256 table.

The reference as shipped cannot be built here: its CMake step generates
config.h and oclkernels.h, and it links a vendor OpenCL runtime that this image
does not have.  ref_shim/ replaces exactly those three things.

Usage: python oracle/build_ref.py [--ref /path/to/reference]
Does nothing (exit 0, message) when the reference checkout is absent.
"""
import argparse
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
OUT = os.path.join(OUT_DIR, "cas-offinder-ref")
SOURCES = ["main.cpp", "cas-offinder.cpp", "read_fasta.cpp", "read_twobit.cpp", "oclfunctions.cpp"]


def build(ref="/root/reference", quiet=False):
    if not os.path.isfile(os.path.join(ref, "cas-offinder.cl")):
        if not quiet:
            print(f"build_ref: reference checkout not found at {ref}; skipped")
        return None
    os.makedirs(OUT_DIR, exist_ok=True)
    shim = os.path.join(HERE, "ref_shim")
    srcs = [os.path.join(ref, s) for s in SOURCES] + [os.path.join(shim, "cl_host_emulator.cpp")]
    pred = os.path.join(OUT_DIR, "ref-predicate")
    newest_src = max(os.path.getmtime(s) for s in srcs + [os.path.join(shim, "CL", "cl.h"),
                                                            os.path.join(shim, "ref_predicate.cpp")])
    if all(os.path.exists(o) and os.path.getmtime(o) >= newest_src for o in (OUT, pred)):
        return OUT
    cmd = ["g++", "-O2", "-fopenmp", "-w", "-std=c++11",
           "-I", shim,
           f'-DCOF_REFERENCE_KERNELS="{os.path.join(ref, "cas-offinder.cl")}"',
           *srcs, "-o", OUT]
    subprocess.run(cmd, check=True)
    subprocess.run(["g++", "-O1", "-w", "-std=c++11",
                    f'-DCOF_REFERENCE_KERNELS="{os.path.join(ref, "cas-offinder.cl")}"',
                    os.path.join(shim, "ref_predicate.cpp"), "-o", pred], check=True)
    return OUT


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    a = ap.parse_args()
    out = build(a.ref)
    print(out or "skipped")
    sys.exit(0)
