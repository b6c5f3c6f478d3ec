"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``oracle/fd2d_oracle.cpp`` into ``oracle/libfd2d_oracle.so`` with
``-ffp-contract=off`` so that no fused multiply-add changes the reference's
evaluation order (gfortran on x86-64 without ``-march`` forms none either).

The reference solver itself (``fd2dmpi/*.f90``) needs gfortran and an MPI
Fortran compiler; neither exists in this image, so there is no ``oracle/_ref``
build and this C++ restatement is the oracle.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "fd2d_oracle.cpp")
LIB = os.path.join(HERE, "libfd2d_oracle.so")


def build(force: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["g++", "-O3", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-pthread", "-o", LIB + ".tmp", SRC]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
