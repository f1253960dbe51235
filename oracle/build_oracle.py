"""Build recipe for the CPU oracle (test infrastructure).

Compiles oracle/oracle_capi.cpp into oracle/_build/liboracle.so with g++.
-ffp-contract=off keeps every float32 multiply and add separately rounded, as
the reference's float32 arithmetic is written (the gait timer must be
bit-exact).  No -march flags: the same recipe builds on x86_64 and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SOURCES = ["oracle_capi.cpp"]
HEADERS = ["oracle.hpp", "refgen.hpp", "flops.hpp"]


def needs_build():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(os.path.join(HERE, f)) > t for f in SOURCES + HEADERS)


def build(force=False, verbose=False):
    """Compile the oracle shared library; returns its path."""
    if not force and not needs_build():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-o", tmp] + [os.path.join(HERE, s) for s in SOURCES]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
