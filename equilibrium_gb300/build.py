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
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libeqfluid.so")
# The same library built with FMA contraction: the plain form's a*b+c fused
# (the reference's f32 results within 1e-6 relative instead of bit for bit).
LIB_FMA = os.path.join(HERE, "libeqfluid_fma.so")
# Translation units, compiled in parallel and linked into one library: the
# main one (the C ABI, every kernel of the plain, precision, frame and
# differentiation forms) and the batched frame kernel's instances, one unit
# per storage format.
UNITS = [("eqfluid.cu", ())] + [("batch_kernels.cu", (f"-DEQ_BATCH_STORE={st}",))
                                for st in range(4)]
SOURCES = sorted({u for u, _ in UNITS})
HEADERS = ["common.cuh", "kernels.cuh", "linsolve.cuh", "noalloc.cu", "wave.cuh", "batch.cuh",
           "batch.cu", "half.cuh", "mg.cuh", "half.cu", "store.cuh",
           "frame.cuh", "frame.cu", "adjoint.cuh", "adjoint.cu", "lscl.cuh", "lscs.cuh", "lssw.cuh"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: device FP stays un-contracted even outside the explicitly
# rounded intrinsics; -ffp-contract=off does the same for host-side scalars
# (diffusion coefficients, 1/c), which gcc on aarch64 would otherwise fuse.
# -static-global-template-stub=false: the batched frame kernel's instances
# are defined in batch_kernels.cu and launched from eqfluid.cu, so their host
# stubs need external linkage (each instance exists in exactly one unit).
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fno-fast-math",
              "-static-global-template-stub=false"]
LINK_FLAGS = ["-shared", "-cudart", "shared"]


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
    if not (os.path.exists(LIB) and os.path.exists(LIB_FMA)):
        return False
    t = min(os.path.getmtime(LIB), os.path.getmtime(LIB_FMA))
    return all(os.path.getmtime(f) <= t for f in _inputs())


def build(force: bool = False, verbose: bool = False, extra=()) -> str:
    if not force and up_to_date():
        return LIB
    tmpdir = tempfile.mkdtemp(prefix="eqfluid_build_")
    try:
        procs = []
        objs = []
        for q, (unit, defs) in enumerate(UNITS):
            obj = os.path.join(tmpdir, f"u{q}.o")
            cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *defs, *extra, "-c", "-o", obj,
                   os.path.join(CSRC, unit)]
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            procs.append((cmd, subprocess.Popen(cmd)))
            objs.append(obj)
        # the FMA build of the main unit (the batched frame kernels are shared)
        fma_obj = os.path.join(tmpdir, "fma.o")
        flags = [f for f in NVCC_FLAGS if f != "--fmad=false"] + ["--fmad=true", "-DEQ_FMA=1"]
        cmd = [nvcc(), *ARCH, *flags, *extra, "-c", "-o", fma_obj,
               os.path.join(CSRC, UNITS[0][0])]
        procs.append((cmd, subprocess.Popen(cmd)))
        failed = [cmd for cmd, p in procs if p.wait() != 0]
        if failed:
            raise subprocess.CalledProcessError(1, failed[0])
        for lib, main in ((LIB, objs[0]), (LIB_FMA, fma_obj)):
            tmp = lib + f".tmp{os.getpid()}"
            cmd = [nvcc(), *ARCH, *LINK_FLAGS, "-o", tmp, main, *objs[1:]]
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            subprocess.check_call(cmd)
            os.replace(tmp, lib)
    finally:
        shutil.rmtree(tmpdir, ignore_errors=True)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True,
          extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else ())
