"""Builds the in-tree CUDA library ``libeqfluid.so`` for sm_103a with nvcc.

The library is the product: every kernel of the frame step and the C ABI of
``include/eqfluid.h``. It is built in place (next to this file) so that the
test and bench processes load it from the source tree.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libeqfluid.so")
SOURCES = ["eqfluid.cu"]
HEADERS = ["common.cuh", "kernels.cuh", "linsolve.cuh", "noalloc.cu", "wave.cuh", "batch.cuh",
           "batch.cu", "half.cuh", "mg.cuh", "half.cu", "store.cuh",
           "frame.cuh", "frame.cu", "adjoint.cuh", "adjoint.cu", "lscl.cuh"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: device FP stays un-contracted even outside the explicitly
# rounded intrinsics; -ffp-contract=off does the same for host-side scalars
# (diffusion coefficients, 1/c), which gcc on aarch64 would otherwise fuse.
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fno-fast-math",
              "-shared", "-cudart", "shared"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _inputs():
    files = [os.path.join(CSRC, s) for s in SOURCES + HEADERS]
    files.append(os.path.join(ROOT, "include", "eqfluid.h"))
    files.append(os.path.abspath(__file__))
    return files


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _inputs())


def build(force: bool = False, verbose: bool = False, extra=()) -> str:
    if not force and up_to_date():
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-o", tmp,
           *[os.path.join(CSRC, s) for s in SOURCES]]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True,
          extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else ())
