"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/cpic_oracle.cpp into oracle/_build/libcpic_oracle.so with g++.
-ffp-contract=off keeps every multiply and add separately rounded, so the
oracle gives the same bits on x86-64 and on aarch64 (where GCC would otherwise
fuse multiply-adds).  No -march=native: the library must run on both hosts.

The reference itself cannot be compiled here (it needs Kokkos and Cabana,
which are not vendored), so there is no oracle/_ref build.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cpic_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libcpic_oracle.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared",
           "-ffp-contract=off", "-fno-fast-math", "-Wall", "-o", LIB + ".tmp", SRC]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
