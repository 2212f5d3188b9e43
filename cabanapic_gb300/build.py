"""Builds libcpic.so (the CUDA kernels + C ABI) for sm_103a, in-tree.

Each translation unit under csrc/ is compiled by nvcc in parallel, then
linked into cabanapic_gb300/_build/libcpic.so.  Every unit but push_fast.cu
is built with --fmad=false: the exact push and the field stencils then round
every multiply and add separately, which makes particle states and field
values bit-identical to a CPU build of the reference compiled without FMA
contraction.  IEEE division and square root are nvcc's defaults (no
--use_fast_math).  push_fast.cu, the production push, is built with fused
multiply-adds.

The C++ example driver (csrc/minipic.cpp: the reference's time loop written
against the C++ push() interface in include/cpic/cabana.hpp) is linked into
cabanapic_gb300/_build/minipic (real_t = float), minipic_f64 (real_t = double) and
minipic_f64_left (real_t = double, the accumulator in Kokkos' LayoutLeft as in a
Kokkos-Cuda build).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libcpic.so")
MINIPIC = os.path.join(OUT, "minipic")
MINIPIC_F64 = os.path.join(OUT, "minipic_f64")
MINIPIC_F64_LEFT = os.path.join(OUT, "minipic_f64_left")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-O2", "-I", INCLUDE, "-I", CSRC]
CU_UNITS = ["push.cu", "push_fast.cu", "fields.cu", "sort.cu", "diagnostics.cu", "adjoint_fields.cu",
            "adjoint_push.cu", "uncenter.cu", "dumps.cu", "init.cu"]
# units built with fused multiply-adds (the production push variant)
FMA_UNITS = {"push_fast.cu", "adjoint_push.cu"}
# units whose FP32 division and square root may be the fast approximations
# (the adjoint push: its results are checked against finite differences to a
# tolerance, not bit for bit)
FAST_DIV_UNITS = {"adjoint_push.cu"}


def _nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return path


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _sources():
    return [os.path.join(CSRC, u) for u in CU_UNITS]


def _newest_input() -> float:
    files = _sources() + [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(INCLUDE, "cpic", f) for f in os.listdir(os.path.join(INCLUDE, "cpic"))]
    return max(os.path.getmtime(f) for f in files)


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compiles libcpic.so (and the minipic driver); returns the library path."""
    os.makedirs(OUT, exist_ok=True)
    # tuning macros of the push kernels (tile shapes), e.g.
    # CPIC_NVCC_FLAGS="-DCPIC_TILE_CHUNKS=5 -DCPIC_TILE_WXMAX=44"; a change of
    # flags rebuilds
    stamp = os.path.join(OUT, "nvcc_flags.txt")
    flags_now = os.environ.get("CPIC_NVCC_FLAGS", "")
    flags_then = open(stamp).read() if os.path.exists(stamp) else ""
    if (not force and flags_now == flags_then and os.path.exists(LIB) and os.path.exists(MINIPIC)
            and os.path.exists(MINIPIC_F64) and os.path.exists(MINIPIC_F64_LEFT)
            and os.path.getmtime(LIB) >= _newest_input()):
        return LIB
    nvcc = _nvcc()
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    extra += flags_now.split()

    def compile_one(src):
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        flags = list(NVCC_FLAGS)
        if os.path.basename(src) in FMA_UNITS:
            flags[flags.index("--fmad=false")] = "--fmad=true"
        if os.path.basename(src) in FAST_DIV_UNITS:
            flags += ["--prec-div=false", "--prec-sqrt=false"]
        log = _run([nvcc, *ARCH, *flags, *extra, "-c", src, "-o", obj])
        return obj, log

    with ThreadPoolExecutor(max_workers=len(CU_UNITS)) as ex:
        results = list(ex.map(compile_one, _sources()))
    if verbose or ptxas_info:
        for _, log in results:
            if log.strip():
                print(log)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-o", tmp, *objs])
    os.replace(tmp, LIB)
    minipic_src = os.path.join(CSRC, "minipic.cpp")
    def link_driver(args):
        exe, defs = args
        _run([nvcc, *ARCH, "-O2", "-std=c++17", "-Xcompiler", "-ffp-contract=off", *defs,
              "-I", INCLUDE, "-o", exe + ".tmp", minipic_src, "-L", OUT, "-lcpic",
              "-Xlinker", "-rpath=$ORIGIN"])
        os.replace(exe + ".tmp", exe)

    with ThreadPoolExecutor(max_workers=3) as ex:
        list(ex.map(link_driver, [(MINIPIC, []), (MINIPIC_F64, ["-DREAL_TYPE=double"]),
                                  (MINIPIC_F64_LEFT, ["-DREAL_TYPE=double", "-DCPIC_ACCUMULATOR_LAYOUT_LEFT"])]))
    with open(stamp, "w") as fh:
        fh.write(flags_now)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                ptxas_info="--ptxas" in sys.argv))
