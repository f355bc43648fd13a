#!/usr/bin/env python3
"""Builds libcasoff.so (CUDA kernels + C ABI) and the cas-offinder CLI in-tree.

Outputs (git-ignored):
  cas-offinder_gb300/lib/libcasoff.so    the engine (CUDA kernels + C ABI)
  cas-offinder_gb300/bin/cas-offinder    the drop-in CLI
  cas-offinder_gb300/bin/cof-synth       synthetic genome writer (host only;
                                         used by bench.py's CPU arms, which
                                         load no library of this package)
  cas-offinder_gb300/lib/libcofrates.so  integer-pipe probe that bench.py
                                         uses for the comparer's roofline
                                         denominator (measurement only, not
                                         part of the engine)
Objects go to cas-offinder_gb300/_build/.  Translation units compile in
parallel; a unit is rebuilt when its source or any header is newer than its
object.  CUDA code is compiled for sm_103a only.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "lib", "libcasoff.so")
CLI = os.path.join(PKG, "bin", "cas-offinder")
SYNTH = os.path.join(PKG, "bin", "cof-synth")
RATES_LIB = os.path.join(PKG, "lib", "libcofrates.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
              "--expt-relaxed-constexpr", *ARCH]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function"]

CU_SOURCES = ["kernels.cu", "comparer_bs.cu", "engine.cu", "server.cu", "noalloc.cu"]
CPP_SOURCES = ["input.cpp", "genome_io.cpp", "synth.cpp", "router.cpp", "gzip_out.cpp"]
# comparer_bs_inst.cu is compiled once per (table row words, window words,
# concrete-only) instance set of the bit-sliced comparer.
BS_INSTANCES = [(row, nk, conc) for row, nk in ((36, 1), (36, 2), (68, 2)) for conc in (1, 0)]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(ROOT, "include", "cof.h"))
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stderr


def build_synth():
    """Only the synthetic genome writer (no CUDA, no engine)."""
    os.makedirs(os.path.dirname(SYNTH), exist_ok=True)
    srcs = [os.path.join(CSRC, "synth.cpp"), os.path.join(CSRC, "synth_main.cpp")]
    if _stale(SYNTH, srcs + [os.path.join(ROOT, "include", "cof_tools.h")]):
        _run(["g++", *CXX_FLAGS, *srcs, "-o", SYNTH, "-pthread"])
    return SYNTH


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    os.makedirs(os.path.dirname(CLI), exist_ok=True)
    hdrs = _headers()
    jobs = []
    objs = []
    units = [(src, src + ".o", []) for src in CU_SOURCES + CPP_SOURCES]
    units += [("comparer_bs_inst.cu", f"comparer_bs_{row}_{nk}_{conc}.o",
               [f"-DCOF_BS_ROW={row}", f"-DCOF_BS_NK={nk}", f"-DCOF_BS_CONC={conc}"])
              for row, nk, conc in BS_INSTANCES]
    for src, oname, defs in units:
        path = os.path.join(CSRC, src)
        if not os.path.exists(path):
            continue
        obj = os.path.join(BUILD, oname)
        objs.append(obj)
        if not _stale(obj, [path] + hdrs):
            continue
        if src.endswith(".cu"):
            cmd = [nvcc(), *NVCC_FLAGS, *defs, "-c", path, "-o", obj]
        else:
            cmd = ["g++", *CXX_FLAGS, "-c", path, "-o", obj]
        jobs.append(cmd)
    rates_src = os.path.join(CSRC, "pipe_rates.cu")
    rates_obj = os.path.join(BUILD, "pipe_rates.cu.o")
    if _stale(rates_obj, [rates_src]):
        jobs.append([nvcc(), *NVCC_FLAGS, "-c", rates_src, "-o", rates_obj])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out:
                print(out, file=sys.stderr)
    if _stale(LIB, objs):
        _run([nvcc(), "-shared", *ARCH, "-o", LIB, *objs, "-cudart", "static", "-lpthread", "-ldl"])
    if _stale(RATES_LIB, [rates_obj]):
        _run([nvcc(), "-shared", *ARCH, "-o", RATES_LIB, rates_obj, "-cudart", "static"])
    build_synth()
    cli_src = os.path.join(CSRC, "cli.cpp")
    if _stale(CLI, [cli_src, LIB] + hdrs):
        _run(["g++", *CXX_FLAGS, cli_src, "-o", CLI, "-L" + os.path.dirname(LIB), "-lcasoff",
              "-Wl,-rpath,$ORIGIN/../lib"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
