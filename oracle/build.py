"""Builds the CPU oracle (test infrastructure) into oracle/_build/.

    python oracle/build.py

The restatement is compiled with -ffp-contract=off so that, like Rust, no
multiply-add is contracted into an FMA, and without -ffast-math so that
division, sqrt and NaN handling stay IEEE.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libeuc_oracle.so")
SRC = os.path.join(HERE, "euc_oracle.cpp")
FLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread"]


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = [SRC, os.path.join(HERE, "..", "include", "euc_gb300.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    cmd = ["g++"] + FLAGS + [SRC, "-o", LIB + ".tmp"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
