"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/nraps_oracle.cpp into oracle/_build/liboracle.so with g++.
-ffp-contract=off is required: the restatement must round every expression
exactly as written, on x86_64 and on aarch64 (where GCC would otherwise fuse
multiply-adds).  The reference itself is Rust and is not built here.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SRC = os.path.join(HERE, "nraps_oracle.cpp")
DEPS = [SRC, os.path.join(HERE, "..", "include", "nraps_gpu.h"),
        os.path.join(HERE, "..", "nraps_gb300", "csrc", "nr_math.h")]


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB):
        lib_t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= lib_t for d in DEPS):
            return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread",
           "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unused-function",
           SRC, "-o", LIB + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
