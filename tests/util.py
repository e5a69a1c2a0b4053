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


def small_workload(nframes: int):
    """The N = 64 workload: size 66, dt 0.1, diffusion = viscosity = 1e-4, 20
    sweeps; one seeded rectangle of ~10 % of the interior (kept off the centre)
    and sources on the 5x5 centre patch every frame (density U[0, 100],
    velocity U[-5, 5]). Returns (size, iters, dt, diff, rect, sx, sy, sd, su, sv)."""
    size, iters, dt, dv = 66, 20, 0.1, 1e-4
    rng = np.random.default_rng(1)
    w = h = 20  # 400 cells of 4096 interior cells ~ 10%
    x0 = int(rng.integers(1, size - 1 - w))
    y0 = int(rng.integers(1, size - 1 - h))
    while abs(x0 + w / 2 - size / 2) < 14 and abs(y0 + h / 2 - size / 2) < 14:
        x0 = int(rng.integers(1, size - 1 - w))
        y0 = int(rng.integers(1, size - 1 - h))
    c = size // 2
    xs, ys = np.meshgrid(np.arange(c - 2, c + 3), np.arange(c - 2, c + 3))
    xs = np.broadcast_to(xs.reshape(-1), (nframes, 25)).astype(np.uint32).copy()
    ys = np.broadcast_to(ys.reshape(-1), (nframes, 25)).astype(np.uint32).copy()
    d = rng.uniform(0, 100, (nframes, 25)).astype(np.float32)
    u = rng.uniform(-5, 5, (nframes, 25)).astype(np.float32)
    v = rng.uniform(-5, 5, (nframes, 25)).astype(np.float32)
    return size, iters, dt, dv, (x0, y0, x0 + w, y0 + h), xs, ys, d, u, v


def state_hashes(fields) -> list:
    """sha256 of each of the six fields' float32 bytes (field order of the
    reference's struct: scratch, density, vx, vy, vx0, vy0)."""
    import hashlib
    return [hashlib.sha256(np.ascontiguousarray(f, dtype=np.float32).tobytes()).hexdigest()
            for f in fields]
