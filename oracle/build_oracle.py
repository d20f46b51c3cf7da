"""Build recipe for the C oracle (test infrastructure): oracle/oakref.c -> oracle/liboakref.so.

The reference itself (Fortran 90 + LAPACK) cannot be compiled on these machines: there is no
Fortran compiler, so there is no oracle/_ref build; the oracle is the C/NumPy restatement.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "oakref.c")
LIB = os.path.join(HERE, "liboakref.so")


def build(force: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-shared", "-fPIC",
           "-Wall", "-o", tmp, SRC, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
