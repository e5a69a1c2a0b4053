"""Shared helpers: seeded scenes mirrored between the GPU library and the oracle."""
from __future__ import annotations

import numpy as np

import oracle
from equilibrium_gb300 import _lib
from equilibrium_gb300.simulation import Fluid, FluidConfigs, SimulationConfigs


def bits(a: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def assert_bitexact(gpu: np.ndarray, ref: np.ndarray, what: str, size: int):
    g, r = bits(gpu), bits(ref)
    if np.array_equal(g, r):
        return
    bad = np.nonzero(g != r)[0]
    q = bad[0]
    raise AssertionError(
        f"{what}: {bad.size} cells differ; first at (i={q % size}, j={q // size}): "
        f"gpu={gpu.reshape(-1)[q]!r} ref={ref.reshape(-1)[q]!r}")


def random_rects(rng: np.random.Generator, size: int, n: int, min_side=1, max_side=None):
    """Rectangles as fill_obstacle gets them (half-open), some touching the frame."""
    max_side = max_side or max(2, size // 3)
    out = []
    for _ in range(n):
        w = int(rng.integers(min_side, max_side + 1))
        h = int(rng.integers(min_side, max_side + 1))
        x0 = int(rng.integers(0, size - 1))
        y0 = int(rng.integers(0, size - 1))
        out.append((x0, y0, min(x0 + w, size - 1), min(y0 + h, size - 1)))
    return out


class Pair:
    """The same scene in the GPU library and in the oracle."""

    def __init__(self, size, frames, dt=0.1, diff=1e-4, visc=1e-4, rects=(), seed=0,
                 randomize=True, vel_scale=1.0):
        self.size, self.frames = size, frames
        self.gpu = Fluid(FluidConfigs(diffusion=diff, viscousity=visc, has_perlin_noise=False),
                         SimulationConfigs(delta_t=dt, frames=frames, size=size))
        self.ref = oracle.OracleFluid(size, dt, frames, diff, visc)
        for r in rects:
            self.ref.fill_obstacle(*r)
            check = _lib.load().eq_fluid_fill_obstacle(self.gpu.handle, *r)
            assert check == 0
        if randomize:
            rng = np.random.default_rng(seed)
            n = size * size
            for f in range(6):
                if f in (_lib.FIELD_VX, _lib.FIELD_VY, _lib.FIELD_VX0, _lib.FIELD_VY0):
                    vals = rng.uniform(-vel_scale, vel_scale, n)
                else:
                    vals = rng.uniform(0.0, 2.0, n)
                self.ref.fields[f][:] = vals.astype(np.float32)
        self.push()

    def push(self):
        for f in range(6):
            self.gpu.write_field(f, self.ref.fields[f])
        assert np.array_equal(self.gpu.cells_type, self.ref.cells)

    def compare(self, what="", fields=range(6)):
        for f in fields:
            assert_bitexact(self.gpu.read_field(f), self.ref.fields[f],
                            f"{what} field {oracle.FIELDS[f]}", self.size)

    def close(self):
        self.gpu.close()
