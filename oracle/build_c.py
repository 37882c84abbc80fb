"""Compile the C oracle (oracle/fe_oracle_c.c) into oracle/_build/libfeoracle.so.

Test infrastructure: the library is the second oracle and the timed CPU
baseline; nothing in the product package loads it.  gcc with OpenMP when the
compiler supports it, else a single-threaded build.  Portable flags only (the
same recipe runs on x86_64 and aarch64).
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "fe_oracle_c.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libfeoracle.so")


def build(force: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + f".tmp{os.getpid()}"
    base = ["gcc", "-O3", "-std=gnu11", "-shared", "-fPIC", "-fno-fast-math", SRC, "-o", tmp, "-lm"]
    err = None
    for extra in (["-fopenmp"], []):
        r = subprocess.run(base[:1] + extra + base[1:], capture_output=True, text=True)
        if r.returncode == 0:
            os.replace(tmp, LIB)
            return LIB
        err = r.stderr
    raise RuntimeError(f"C oracle build failed:\n{err}")


if __name__ == "__main__":
    print(build(force=True))
