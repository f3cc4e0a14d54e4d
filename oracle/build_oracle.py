"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``opx_oracle.c`` into ``oracle/libopx_oracle.so`` with gcc.  The flags
keep Java's floating-point semantics: no fused multiply-add contraction and no
fast-math, so that the oracle evaluates every expression as the reference does.
OpenMP is used only by ``orc_update_grid_omp`` (the timed CPU baseline).
``-O3`` without ``-march=native``: the same flags build on the x86 and the Arm
hosts and give the same results on both.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "opx_oracle.c")
LIB = os.path.join(HERE, "libopx_oracle.so")


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "opx_oracle.h"))):
        return LIB
    cmd = ["gcc", "-O3", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", "-Wall", "-o", LIB + ".tmp", SRC, "-lm"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
