"""Batches of independent scenes over the C ABI (``eq_batch_*``).

The reference advances one ``Fluid`` per simulation thread
(``renderer.rs:125-128``); a ``Batch`` advances thousands of them together,
each with its own ``SimulationConfigs``/``FluidConfigs`` numbers, one
persistent kernel launch per frame (graph-captured across frames). Each
scene's arrays stay bit-identical to stepping that scene alone.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Iterable, List, Optional, Sequence

import numpy as np

from . import _lib
from ._lib import check


@dataclass
class SceneConfig:
    size: int
    delta_t: float = 0.1
    frames: int = 20
    diffusion: float = 1e-4
    viscousity: float = 1e-4


class Batch:
    def __init__(self, scenes: Sequence[SceneConfig], device: int = 0, storage: str = "f32"):
        L = _lib.load()
        n = len(scenes)
        arr = (_lib.SceneDescC * n)()
        for q, sc in enumerate(scenes):
            arr[q].size = int(sc.size)
            arr[q].delta_t = float(sc.delta_t)
            arr[q].frames = int(sc.frames)
            arr[q].diffusion = float(sc.diffusion)
            arr[q].viscousity = float(sc.viscousity)
        h = ctypes.c_void_p()
        st = {"f32": 0, "f16": _lib.STORE_F16, "bf16": _lib.STORE_BF16,
              "f16_scalars": _lib.STORE_F16_SCALARS}[storage]
        check(L.eq_batch_new_storage(n, arr, st, device, ctypes.byref(h)))
        self.storage = storage
        self.handle = h
        self.scenes = list(scenes)

    def __len__(self):
        return len(self.scenes)

    def _size(self, scene: int) -> int:
        if not 0 <= scene < len(self.scenes):
            raise _lib.EqError(_lib.EQ_ERR_ARG, "scene index out of range")
        return int(self.scenes[scene].size)

    def close(self):
        if self.handle:
            _lib.load().eq_batch_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- set-up
    def fill_obstacle(self, scene: int, x0: int, y0: int, x1: int, y1: int):
        check(_lib.load().eq_batch_fill_obstacle(self.handle, scene, x0, y0, x1, y1))

    def set_sources(self, scene: int, xs, ys, density=None, vx=None, vy=None):
        xs = np.ascontiguousarray(xs, dtype=np.uint32)
        ys = np.ascontiguousarray(ys, dtype=np.uint32)
        conv = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float32)
        d, u, v = conv(density), conv(vx), conv(vy)
        ptr = lambda a: None if a is None else a.ctypes.data
        check(_lib.load().eq_batch_set_sources(self.handle, scene, xs.size, xs.ctypes.data,
                                               ys.ctypes.data, ptr(d), ptr(u), ptr(v)))

    def cells(self, scene: int) -> np.ndarray:
        S = self._size(scene)
        out = np.empty(S * S, dtype=np.uint8)
        check(_lib.load().eq_batch_read_cells(self.handle, scene, out.ctypes.data, out.size))
        return out

    # ---- fields
    def read_field(self, scene: int, field: int) -> np.ndarray:
        S = self._size(scene)
        out = np.empty(S * S, dtype=np.float32)
        check(_lib.load().eq_batch_read_field(self.handle, scene, field, out.ctypes.data,
                                              out.size))
        return out

    def read_fields(self, field: int, out: Optional[np.ndarray] = None) -> np.ndarray:
        """One field of every scene: their dense size*size arrays concatenated in
        scene order (`out` may be a preallocated float32 array, e.g. pinned)."""
        n = sum(self._size(s) ** 2 for s in range(len(self)))
        if out is None:
            out = np.empty(n, dtype=np.float32)
        if out.dtype != np.float32 or out.size != n or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous float32 array of the total cell count")
        check(_lib.load().eq_batch_read_fields(self.handle, field, out.ctypes.data, out.size))
        return out

    def write_field(self, scene: int, field: int, values: np.ndarray):
        v = np.ascontiguousarray(values, dtype=np.float32).reshape(-1)
        check(_lib.load().eq_batch_write_field(self.handle, scene, field, v.ctypes.data,
                                               v.size))

    # ---- stepping
    def step(self, nframes: int = 1, graph: bool = True):
        L = _lib.load()
        fn = L.eq_batch_step if graph else L.eq_batch_step_eager
        check(fn(self.handle, nframes))

    def lin_solve(self, mode: int, x_field: int, x0_field: int, a: float, c: float):
        check(_lib.load().eq_batch_lin_solve(self.handle, mode, x_field, x0_field,
                                             np.float32(a), np.float32(c)))

    def diffuse(self, mode: int, x_field: int, x0_field: int, diffusion: float):
        check(_lib.load().eq_batch_diffuse(self.handle, mode, x_field, x0_field,
                                           np.float32(diffusion)))

    def project(self, vx: int, vy: int, p: int, div: int):
        check(_lib.load().eq_batch_project(self.handle, vx, vy, p, div))

    def advect(self, mode: int, d: int, d0: int, u: int, v: int):
        check(_lib.load().eq_batch_advect(self.handle, mode, d, d0, u, v))

    def set_boundaries(self, mode: int, field: int):
        check(_lib.load().eq_batch_set_boundaries(self.handle, mode, field))

    def synchronize(self):
        check(_lib.load().eq_batch_synchronize(self.handle))

    # ---- tuning
    def set_tuning(self, sweeps_per_pass: int, blocks_per_sm: int = 1):
        check(_lib.load().eq_batch_set_tuning(self.handle, sweeps_per_pass, blocks_per_sm))

    def tuning(self):
        a, b = ctypes.c_int(), ctypes.c_int()
        check(_lib.load().eq_batch_get_tuning(self.handle, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def autotune(self, trial_frames: int = 2) -> List[float]:
        ms = (ctypes.c_double * 64)()
        n = ctypes.c_int()
        check(_lib.load().eq_batch_autotune(self.handle, trial_frames, ms, 64, ctypes.byref(n)))
        return [ms[q] for q in range(min(n.value, 64))]

    def cell_count(self) -> int:
        c = ctypes.c_uint64()
        check(_lib.load().eq_batch_cell_count(self.handle, ctypes.byref(c)))
        return c.value

    def launch_count(self) -> int:
        c = ctypes.c_uint64()
        check(_lib.load().eq_batch_launch_count(self.handle, ctypes.byref(c)))
        return c.value


def partition_scenes(scenes: Sequence, world: int):
    """Splits a batch's scenes over `world` ranks (one GPU each) with no data
    shared between ranks: greedy largest-first bin packing by each scene's
    work, size^2 x sweeps (every scene is an independent Fluid, as each
    simulation thread of the reference owns its own, renderer.rs:126-128).
    Scenes are SceneConfig or (size, dt, sweeps, ...) tuples. Returns the
    scene indices of each rank (ascending) and each rank's total work; the
    same inputs give the same split on every rank."""
    if world < 1:
        raise ValueError("world must be >= 1")

    def work(sc):
        size, sweeps = (sc.size, sc.frames) if isinstance(sc, SceneConfig) else (sc[0], sc[2])
        return int(size) ** 2 * max(int(sweeps), 1)

    cost = [work(sc) for sc in scenes]
    order = sorted(range(len(cost)), key=lambda q: (-cost[q], q))
    loads = [0] * world
    parts: List[List[int]] = [[] for _ in range(world)]
    for q in order:
        r = min(range(world), key=lambda k: (loads[k], k))
        parts[r].append(q)
        loads[r] += cost[q]
    return [sorted(p) for p in parts], loads
