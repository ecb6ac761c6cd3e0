"""Build the oracle shared library (test infrastructure only).

Compiles oracle/ddla_oracle.c with gcc into oracle/_build/libddla_oracle.so.
Uses OpenMP when the compiler supports it (the threaded CPU baseline), else a
serial build.  No reference sources are compiled: DDLA is C#/.NET and cannot be
built here.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libddla_oracle.so")
SRC = os.path.join(HERE, "ddla_oracle.c")


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    base = ["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", SRC, "-o", LIB, "-lm"]
    try:
        subprocess.run(base[:1] + ["-fopenmp"] + base[1:], check=True, capture_output=True)
    except subprocess.CalledProcessError:
        subprocess.run(base, check=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
