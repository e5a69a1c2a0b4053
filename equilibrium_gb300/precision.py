"""The precision form over the C ABI (``eq_hfluid_*``): one scene whose six
fields are stored in FP16 or BF16 while every operation computes in FP32, with
project's pressure (fluid.rs:353-362) solved by mixed-precision iterative
refinement to a relative residual."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import check


class HalfFluid:
    def __init__(self, size: int, delta_t: float, frames: int, diffusion: float,
                 viscousity: float, storage: str = "f16", pressure_rtol: float = 1e-5,
                 max_refinements: int = 30, device: int = 0):
        L = _lib.load()
        st = {"f16": _lib.STORE_F16, "bf16": _lib.STORE_BF16,
              "f16_scalars": _lib.STORE_F16_SCALARS}[storage]
        fc = _lib.FluidConfigsC(diffusion, viscousity, 0)
        sc = _lib.SimulationConfigsC(delta_t, frames, size)
        h = ctypes.c_void_p()
        check(L.eq_hfluid_new(ctypes.byref(fc), ctypes.byref(sc), st, pressure_rtol,
                              max_refinements, device, ctypes.byref(h)))
        self.handle, self.size, self.storage = h, size, storage

    def close(self):
        if self.handle:
            _lib.load().eq_hfluid_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def fill_obstacle(self, x0, y0, x1, y1):
        check(_lib.load().eq_hfluid_fill_obstacle(self.handle, x0, y0, x1, y1))

    def add_sources(self, xs, ys, d=None, u=None, v=None):
        xs = np.ascontiguousarray(xs, dtype=np.uint32)
        ys = np.ascontiguousarray(ys, dtype=np.uint32)
        conv = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float32)
        d, u, v = conv(d), conv(u), conv(v)
        ptr = lambda a: None if a is None else a.ctypes.data
        check(_lib.load().eq_hfluid_add_sources(self.handle, xs.size, xs.ctypes.data,
                                                ys.ctypes.data, ptr(d), ptr(u), ptr(v)))

    def step(self):
        check(_lib.load().eq_hfluid_step(self.handle))

    def read_field(self, field: int) -> np.ndarray:
        out = np.empty(self.size * self.size, dtype=np.float32)
        check(_lib.load().eq_hfluid_read_field(self.handle, field, out.ctypes.data, out.size))
        return out

    def write_field(self, field: int, values):
        v = np.ascontiguousarray(values, dtype=np.float32).reshape(-1)
        check(_lib.load().eq_hfluid_write_field(self.handle, field, v.ctypes.data, v.size))

    def stats(self) -> dict:
        s = _lib.HStatsC()
        check(_lib.load().eq_hfluid_stats(self.handle, ctypes.byref(s)))
        return {"ir_iterations": list(s.ir_iterations), "rel_residual": list(s.rel_residual),
                "div_norm_before": list(s.div_norm_before), "div_norm": list(s.div_norm)}

    def launch_count(self) -> int:
        c = ctypes.c_uint64()
        check(_lib.load().eq_hfluid_launch_count(self.handle, ctypes.byref(c)))
        return c.value

    def set_concurrency(self, mask: int):
        """Which diffusions run on side streams (bit 1: vy, bit 2: density)."""
        check(_lib.load().eq_hfluid_set_concurrency(self.handle, mask))

    def set_solver(self, solver: int):
        """The kernel of the diffusion solves (as Fluid's eq_fluid_set_solver)."""
        check(_lib.load().eq_hfluid_set_solver(self.handle, solver))


def rel_l2(a: np.ndarray, ref: np.ndarray) -> float:
    """||a - ref||_2 / ||ref||_2 over the interior cells."""
    n = int(round(np.sqrt(ref.size)))
    a = np.asarray(a, dtype=np.float64).reshape(n, n)[1:-1, 1:-1]
    r = np.asarray(ref, dtype=np.float64).reshape(n, n)[1:-1, 1:-1]
    den = np.linalg.norm(r)
    return float(np.linalg.norm(a - r) / den) if den > 0 else float(np.linalg.norm(a - r))


def max_abs(a: np.ndarray, ref: np.ndarray) -> float:
    n = int(round(np.sqrt(ref.size)))
    a = np.asarray(a, dtype=np.float64).reshape(n, n)[1:-1, 1:-1]
    r = np.asarray(ref, dtype=np.float64).reshape(n, n)[1:-1, 1:-1]
    return float(np.abs(a - r).max())
