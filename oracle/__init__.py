"""ORACLE -- test infrastructure only, never the product path.

A ctypes front end to ``fluid_oracle.cpp``: a C++ restatement of the
reference's ``src/simulation/fluid.rs`` (vkabadzhova/equilibrium), used by
``tests/`` as the parity checker, by ``__graft_entry__.smoke()`` as the checker
and by ``bench.py``'s CPU-baseline leg as the timed reference port.

Parity status: numeric parity of this restatement is UNPINNED by the reference
itself (the reference ships no numeric golden vectors and its Rust crate cannot
be built here). It is pinned against the reference's own non-numeric fixtures
(wall-mask count, Rectangle validation, index layout) and cross-checked
against an independent pure-Python restatement (``tests/golden/pyref.py``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libeqoracle.so")
SOURCES = [os.path.join(HERE, "fluid_oracle.cpp"), os.path.join(HERE, "fluid_oracle.hpp")]

# Modes (fluid.rs:21-29) and field order (fluid.rs:59-77).
ADJUST_ROW, ADJUST_COLUMN, PASSIVE = 0, 1, 2
FIELDS = ("scratch", "density", "vx", "vy", "vx0", "vy0")

# -ffp-contract=off: Rust never fuses a*b+c; gcc on aarch64 would by default.
CXXFLAGS = ["-O3", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared"]


def build(force: bool = False) -> str:
    """Compile the oracle library in place (g++, a few seconds)."""
    newest = max(os.path.getmtime(s) for s in SOURCES)
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest:
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["g++", *CXXFLAGS, "-o", tmp, SOURCES[0]])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        u32, i64, f32, f64, ci = (ctypes.c_uint32, ctypes.c_int64, ctypes.c_float,
                                  ctypes.c_double, ctypes.c_int)
        sig = {
            "eqo_set_boundaries_f32": (None, [ci, P, u32, P]),
            "eqo_lin_solve_f32": (None, [ci, P, P, f32, f32, u32, i64, P]),
            "eqo_diffuse_f32": (None, [ci, P, P, f32, u32, f32, i64, P]),
            "eqo_project_f32": (None, [P, P, P, P, u32, i64, P]),
            "eqo_advect_f32": (None, [ci, P, P, P, P, u32, f32, P]),
            "eqo_step_f32": (None, [P, P, u32, f32, i64, f32, f32]),
            "eqo_run_f32": (None, [P, P, u32, f32, i64, f32, f32, i64, i64, P, P, P, P, P]),
            "eqo_time_run_f32": (f64, [P, P, u32, f32, i64, f32, f32, i64, i64, P, P, P, P, P]),
            "eqo_new_f32": (None, [u32, P, P]),
            "eqo_reinit_f32": (None, [u32, P, P]),
            "eqo_lin_solve_f64": (None, [ci, P, P, f64, f64, u32, i64, P]),
            "eqo_step_f64": (None, [P, P, u32, f64, i64, f64, f64]),
            "eqo_run_f64": (None, [P, P, u32, f64, i64, f64, f64, i64, i64, P, P, P, P, P]),
            "eqo_new_f64": (None, [u32, P, P]),
            "eqo_fill_obstacle": (None, [P, u32, i64, i64, i64, i64]),
            "eqo_rectangle_valid": (ci, [i64, i64, i64, i64, i64]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


def _ptr6(fields):
    arr = (ctypes.c_void_p * 6)(*[_ptr(f) for f in fields])
    return arr


class OracleFluid:
    """Host-side state of one scene, laid out exactly like the reference's
    ``Fluid`` (six ``size*size`` arrays incl. the ghost frame + a wall mask)."""

    def __init__(self, size: int, delta_t: float, frames: int, diffusion: float,
                 viscousity: float, dtype=np.float32):
        self.size, self.delta_t, self.frames = int(size), delta_t, int(frames)
        self.diffusion, self.viscousity, self.dtype = diffusion, viscousity, np.dtype(dtype)
        n = self.size * self.size
        self.fields = [np.zeros(n, dtype=self.dtype) for _ in range(6)]
        self.cells = np.zeros(n, dtype=np.uint8)
        fn = lib().eqo_new_f32 if self.dtype == np.float32 else lib().eqo_new_f64
        fn(self.size, _ptr6(self.fields), _ptr(self.cells))

    def field(self, name: str) -> np.ndarray:
        return self.fields[FIELDS.index(name)]

    def reinit(self):
        assert self.dtype == np.float32
        lib().eqo_reinit_f32(self.size, _ptr6(self.fields), _ptr(self.cells))

    def fill_obstacle(self, x0: int, y0: int, x1: int, y1: int):
        lib().eqo_fill_obstacle(_ptr(self.cells), self.size, x0, y0, x1, y1)

    def step(self):
        if self.dtype == np.float32:
            lib().eqo_step_f32(_ptr6(self.fields), _ptr(self.cells), self.size,
                               self.delta_t, self.frames, self.diffusion, self.viscousity)
        else:
            lib().eqo_step_f64(_ptr6(self.fields), _ptr(self.cells), self.size,
                               self.delta_t, self.frames, self.diffusion, self.viscousity)

    def run(self, nframes: int, sx, sy, sd, su, sv, timed: bool = False):
        """``nframes`` frames, each = that frame's sources then step().
        Source arrays have shape (nframes, nsrc)."""
        sx = np.ascontiguousarray(sx, dtype=np.uint32)
        sy = np.ascontiguousarray(sy, dtype=np.uint32)
        sd = np.ascontiguousarray(sd, dtype=np.float32)
        su = np.ascontiguousarray(su, dtype=np.float32)
        sv = np.ascontiguousarray(sv, dtype=np.float32)
        nsrc = sx.shape[1] if sx.ndim == 2 else 0
        args = [_ptr6(self.fields), _ptr(self.cells), self.size, self.delta_t, self.frames,
                self.diffusion, self.viscousity, nframes, nsrc, _ptr(sx), _ptr(sy), _ptr(sd),
                _ptr(su), _ptr(sv)]
        if self.dtype == np.float32:
            if timed:
                return lib().eqo_time_run_f32(*args)
            lib().eqo_run_f32(*args)
        else:
            lib().eqo_run_f64(*args)
        return None


def set_boundaries(mode: int, x: np.ndarray, size: int, cells: np.ndarray):
    lib().eqo_set_boundaries_f32(mode, _ptr(x), size, _ptr(cells))


def lin_solve(mode, x, x0, a, c, size, iters, cells):
    if x.dtype == np.float64:
        lib().eqo_lin_solve_f64(mode, _ptr(x), _ptr(x0), a, c, size, iters, _ptr(cells))
    else:
        lib().eqo_lin_solve_f32(mode, _ptr(x), _ptr(x0), a, c, size, iters, _ptr(cells))


def diffuse(mode, x, x0, diff, size, dt, iters, cells):
    lib().eqo_diffuse_f32(mode, _ptr(x), _ptr(x0), diff, size, dt, iters, _ptr(cells))


def project(vx, vy, p, div, size, iters, cells):
    lib().eqo_project_f32(_ptr(vx), _ptr(vy), _ptr(p), _ptr(div), size, iters, _ptr(cells))


def advect(mode, d, d0, u, v, size, dt, cells):
    lib().eqo_advect_f32(mode, _ptr(d), _ptr(d0), _ptr(u), _ptr(v), size, dt, _ptr(cells))


def fill_obstacle(cells, size, x0, y0, x1, y1):
    lib().eqo_fill_obstacle(_ptr(cells), size, x0, y0, x1, y1)


def rectangle_valid(dl, ur, size) -> bool:
    return bool(lib().eqo_rectangle_valid(dl[0], dl[1], ur[0], ur[1], size))
