"""Build recipe for the oracle (test infrastructure, not the product).

Compiles oracle/oracle.cpp into oracle/liboracle.so with g++ and OpenMP.
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and
reference arms load the result.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SRC = [os.path.join(HERE, "oracle.cpp"), os.path.join(HERE, "gen_grid_rmat.cpp")]


def build(force: bool = False, verbose: bool = False) -> str:
    deps = SRC + [os.path.join(HERE, "oracle.h"), os.path.join(HERE, "gen_common.h"),
                  os.path.join(HERE, "..", "include", "kamsta_gpu.h")]
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in deps):
            return LIB
    # -ffp-contract=off: the generators' floating-point definitions are
    # evaluated without fused multiply-add, exactly like the device code
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
           "-Wall", "-Wno-unused-function", "-o", LIB + ".tmp"] + SRC
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
