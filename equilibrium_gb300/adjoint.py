"""The differentiation form: a recorded forward run of a ``Fluid`` and its
reverse-mode derivative (``backward()``), over ``eq_grad_*`` in the C ABI.

The reference's step (fluid.rs:437-524) has no derivative; this adds one for
the loop "each frame, add a density-source field to density and scratch at
every cell, then step()". The forward is the handle's bit-exact f32 step; the
state at every ``checkpoint_every``-th frame stays on the GPU, and
``backward()`` recomputes each segment from its checkpoint, then undoes it
frame by frame with hand-written adjoint kernels (FP32).
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np

from . import _lib
from ._lib import check
from .simulation import Fluid


def _f32(a, n: int, what: str) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32).reshape(-1)
    if a.size != n:
        raise ValueError(f"{what}: expected {n} elements, got {a.size}")
    return a


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class Recorder:
    """``Recorder(fluid, max_frames, checkpoint_every=8)``; ``forward(src)``
    runs len(src) frames from the fluid's current state; ``l2_loss(target)``
    and ``backward()`` give the loss and the gradients."""

    def __init__(self, fluid: Fluid, max_frames: int, checkpoint_every: int = 8):
        self._L = _lib.load()
        self.fluid = fluid
        self.S = int(fluid.simulation_configs.size)
        h = ctypes.c_void_p()
        check(self._L.eq_grad_new(fluid.handle, int(max_frames), int(checkpoint_every),
                                  ctypes.byref(h)))
        self.handle = h
        self.nframes = 0

    def close(self):
        if getattr(self, "handle", None):
            self._L.eq_grad_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self, src=None, nframes: Optional[int] = None):
        """src: (nframes, size, size) density sources (or None with nframes)."""
        n = self.S * self.S
        self.fluid._push_configs()
        if src is None:
            if nframes is None:
                raise ValueError("give src or nframes")
            check(self._L.eq_grad_forward(self.handle, int(nframes), None, 0))
            self.nframes = int(nframes)
            return
        src = np.ascontiguousarray(src, dtype=np.float32)
        nf = src.size // n
        check(self._L.eq_grad_forward(self.handle, nf, _p(_f32(src, nf * n, "src")), nf * n))
        self.nframes = nf

    def l2_loss(self, target, return_adjoint: bool = False):
        n = self.S * self.S
        t = _f32(target, n, "target")
        loss = ctypes.c_double()
        adj = np.zeros(n, np.float32) if return_adjoint else None
        check(self._L.eq_grad_l2_loss(self.handle, _p(t), n, ctypes.byref(loss),
                                      _p(adj) if adj is not None else None))
        return (loss.value, adj) if return_adjoint else loss.value

    def backward(self, adj_final=None, want_init: bool = True, want_src: bool = True):
        """Returns (grad_init (6, n), grad_src (nframes, n)) for the six arrays
        before the run and every frame's source field; adj_final (6, n) is the
        adjoint of the final state (default: the l2_loss seed)."""
        n = self.S * self.S
        a = _f32(adj_final, 6 * n, "adj_final") if adj_final is not None else None
        gi = np.zeros((6, n), np.float32) if want_init else None
        gs = np.zeros((self.nframes, n), np.float32) if want_src else None
        check(self._L.eq_grad_backward(self.handle, _p(a) if a is not None else None,
                                       6 * n if a is not None else 0,
                                       _p(gi) if gi is not None else None, 6 * n if want_init else 0,
                                       _p(gs) if gs is not None else None,
                                       self.nframes * n if want_src else 0))
        return gi, gs

    def set_wavefront_storage(self, max_store: int):
        check(self._L.eq_grad_set_wavefront_storage(self.handle, int(max_store)))

    def wavefront_storage(self):
        """(store, blocks) of the last transposed solve (see the C header)."""
        st, cl = ctypes.c_int(), ctypes.c_int()
        check(self._L.eq_grad_get_wavefront_storage(self.handle, ctypes.byref(st),
                                                    ctypes.byref(cl)))
        return st.value, cl.value

    def launch_count(self) -> int:
        c = ctypes.c_uint64()
        check(self._L.eq_grad_launch_count(self.handle, ctypes.byref(c)))
        return c.value

    # ---- single phases (host arrays in / out) -------------------------------
    def set_boundaries_adj(self, mode: int, xb):
        n = self.S * self.S
        x = _f32(xb, n, "xb").copy()
        check(self._L.eq_grad_set_boundaries_adj(self.handle, mode, _p(x), n))
        return x

    def lin_solve_adj(self, mode: int, xb, x0b, a: float, c: float):
        n = self.S * self.S
        x, x0 = _f32(xb, n, "xb").copy(), _f32(x0b, n, "x0b").copy()
        check(self._L.eq_grad_lin_solve_adj(self.handle, mode, _p(x), _p(x0), a, c, n))
        return x, x0

    def advect_adj(self, mode: int, db, d0b, ub, vb, d0, u, v):
        n = self.S * self.S
        io = [_f32(a, n, "adjoint").copy() for a in (db, d0b, ub, vb)]
        ins = [_f32(a, n, "field") for a in (d0, u, v)]
        check(self._L.eq_grad_advect_adj(self.handle, mode, *[_p(a) for a in io],
                                         *[_p(a) for a in ins], n))
        return io

    def project_adj(self, vxb, vyb, pb, divb):
        n = self.S * self.S
        io = [_f32(a, n, "adjoint").copy() for a in (vxb, vyb, pb, divb)]
        check(self._L.eq_grad_project_adj(self.handle, *[_p(a) for a in io], n))
        return io
