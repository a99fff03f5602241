"""Build recipe for the CPU oracle (test infrastructure).

    python oracle/build_oracle.py      -> oracle/_build/liboracle.so

Compiled with -O2 -ffp-contract=off and without fast-math so that every
Fortran expression of the reference keeps its evaluation order and rounding
(gcc contracts a*b+c into an FMA by default on aarch64; that is switched
off).  OpenMP parallelises the independent particle classes for the
all-cores CPU baseline; results do not depend on the thread count.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SRC = os.path.join(HERE, "f3d_oracle.cpp")
FLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
         "-std=c++17", "-Wall"]


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    hdr = os.path.join(HERE, "..", "include", "fall3d_gpu.h")
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if t >= os.path.getmtime(SRC) and t >= os.path.getmtime(hdr):
            return LIB
    tmp = LIB + f".{os.getpid()}.tmp"
    cmd = ["g++", *FLAGS, "-o", tmp, SRC]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
