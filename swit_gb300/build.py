"""Builds the engine library ``swit_gb300/libswit_gb300.so`` for sm_103a.

Two translation units (csrc/engine.cu, csrc/noalloc.cu), one ``-gencode``; static cudart so the
library needs nothing but the driver at run time.  ``--fmad=false`` and the host
``-ffp-contract=off`` keep the reference's floating-point evaluation order
(no fused multiply-add is formed on either side), which makes FP32 results
bit-identical to a non-FMA CPU evaluation.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libswit_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-shared", "-cudart", "static"]


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith((".cu", ".cuh", ".h"))] + [
        os.path.join(INCLUDE, "swit_gb300.h")]


def build(force: bool = False, verbose: bool = False, extra=()) -> str:
    newest = max(os.path.getmtime(s) for s in sources())
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest and not extra:
        return LIB
    units = [os.path.join(CSRC, f) for f in ("engine.cu", "noalloc.cu")]
    cmd = [_nvcc()] + NVCC_FLAGS + list(extra) + ["-o", LIB + ".tmp"] + units
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    extra = [a for a in sys.argv[1:] if a.startswith(("-X", "-D"))]
    print(build(force=True, verbose=True, extra=extra))
