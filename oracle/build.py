"""Builds the CPU oracle (test infrastructure) into oracle/_build/.

    python oracle/build.py

The restatement is compiled with -ffp-contract=off and without fast-math so
that every FP32 operation is one IEEE-754 operation in source order on both
x86-64 and aarch64 (gcc contracts a*b+c into FMA by default on aarch64).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SOURCES = [os.path.join(HERE, "sr_oracle.cpp")]
HEADERS = [os.path.join(HERE, "sr_oracle.h"),
           os.path.join(HERE, "..", "include", "sr_shaders.h")]

FLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-pthread",
         "-ffp-contract=off", "-fno-fast-math", "-fno-finite-math-only",
         "-Wall", "-Wno-unused-function"]


def stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in SOURCES + HEADERS + [__file__])


def build(force=False):
    if not force and not stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++"] + FLAGS + SOURCES + ["-o", tmp]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
