"""Build recipe for the oracle (test infrastructure only).

Compiles oracle/tina_oracle.cpp -- the CPU restatement of Tina's raster + shade
path -- into oracle/_build/libtina_oracle.so with the flags that keep its FP32
arithmetic in the reference's operation order: -O2 -ffp-contract=off (no fused
multiply-add on any line), no -ffast-math, OpenMP for the parallel (timed
baseline) mode.  No -march flags: the same source builds on x86-64 and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libtina_oracle.so")
SOURCES = [os.path.join(HERE, "tina_oracle.cpp")]
HEADERS = [os.path.join(HERE, "..", "include", "tina3.h")]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in SOURCES + HEADERS + [__file__])


def build(force=False, verbose=False):
    """Compile the oracle library if it is missing or older than its sources."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
           "-fPIC", "-shared", "-Wall", "-Wno-unused-function", *SOURCES, "-o", LIB + ".tmp"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
