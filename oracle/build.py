"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``fdga_oracle.cpp`` into ``oracle/_build/libfdga_oracle.so`` with g++ and OpenMP.
The reference (fdDGAsolver.jl) is pure Julia, so there is no reference source that compiles
here and no ``oracle/_ref`` build; the C++ restatement is the oracle.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "fdga_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
OUT = os.path.join(OUT_DIR, "libfdga_oracle.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= os.path.getmtime(SRC):
        return OUT
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", SRC, "-o", OUT + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
