#!/usr/bin/env python3
"""Build the oracle: the CPU restatement cof_oracle.cpp -> oracle/_build/cof-oracle.

TEST INFRASTRUCTURE: the oracle is the checker for the parity tests and the
timed CPU baseline of bench.py; the product never runs it.  It also builds the
reference itself (oracle/_ref/cas-offinder-ref, see build_ref.py) when the
reference checkout is present.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build", "cof-oracle")
SRC = os.path.join(HERE, "cof_oracle.cpp")


def build(with_reference=True):
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    if not os.path.exists(OUT) or os.path.getmtime(OUT) < os.path.getmtime(SRC):
        subprocess.run(["g++", "-O3", "-std=c++17", "-fopenmp", "-Wall", SRC, "-o", OUT], check=True)
    ref = None
    if with_reference:
        sys.path.insert(0, HERE)
        try:
            import build_ref
            ref = build_ref.build(quiet=True)
        finally:
            sys.path.pop(0)
    return OUT, ref


if __name__ == "__main__":
    print(build())
