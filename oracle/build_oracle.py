"""Build recipe for the oracle (test infrastructure only).

Compiles oracle/oracle.cpp -- the CPU restatement of RAJA's seq/omp
semantics -- into oracle/liboracle.so with g++ and OpenMP.  The output is
git-ignored and rebuilt on each machine (x86 here, aarch64 on the GPU host).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "oracle.cpp")
OUT = os.path.join(HERE, "liboracle.so")


def build(force: bool = False) -> str:
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= os.path.getmtime(SRC):
        return OUT
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", OUT + ".tmp", SRC]
    subprocess.run(cmd, check=True)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
