"""Build recipe for the oracle's C++ restatement (test infrastructure only).

Compiles oracle/fgoracle.cpp and oracle/fmm_cpu.cpp into oracle/_build/libfgoracle.so with g++ and OpenMP.
Plain -O2 without fast-math, so the FP64 arithmetic follows IEEE order of operations.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libfgoracle.so")


SOURCES = ["fgoracle.cpp", "fmm_cpu.cpp"]


def build(force=False, quiet=True):
    srcs = [os.path.join(HERE, f) for f in SOURCES]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(f) for f in srcs):
        return LIB
    os.makedirs(OUT, exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-o", LIB + ".tmp"] + srcs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("oracle build failed")
    os.replace(LIB + ".tmp", LIB)
    if not quiet:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force=True, quiet=False)
