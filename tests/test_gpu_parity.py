"""Bit-exact parity of the sm_103a kernels with the oracle, phase by phase and
for whole frames, through the C ABI (fluid.rs:133-524).

Every array is compared bit for bit (f32 bit patterns), ghost cells included,
because all six arrays are state that later phases and frames read.
"""
import numpy as np
import pytest

import oracle
from equilibrium_gb300 import _lib
from tests.util import Pair, assert_bitexact, random_rects

pytestmark = pytest.mark.gpu

ROW, COL, PAS = _lib.MODE_ADJUST_ROW, _lib.MODE_ADJUST_COLUMN, _lib.MODE_PASSIVE
SC, DE, VX, VY, VX0, VY0 = range(6)


def L():
    return _lib.load()


LAYOUTS = {
    "open": lambda rng, s: [],
    "one_block": lambda rng, s: [(s // 3, s // 4, s // 3 + s // 5, s // 4 + s // 6)],
    "random4": lambda rng, s: random_rects(rng, s, 4),
    "random12_small": lambda rng, s: random_rects(rng, s, 12, 1, 3),
    "touching_frame": lambda rng, s: [(0, 5, 4, 9), (s - 4, 2, s, 6), (6, 0, 9, 3),
                                      (3, s - 3, 8, s)],
    "blocked_row_and_col": lambda rng, s: [(0, s // 2, s, s // 2 + 1),
                                           (s // 3, 0, s // 3 + 2, s)],
    "checker": lambda rng, s: [(x, y, x + 1, y + 1) for x in range(2, s - 2, 3)
                               for y in range(2, s - 2, 3)],
}


@pytest.mark.parametrize("mode", [ROW, COL, PAS])
@pytest.mark.parametrize("layout", list(LAYOUTS))
def test_set_boundaries(eqlib, mode, layout):
    rng = np.random.default_rng(hash((mode, layout)) % 2**32)
    size = 37
    p = Pair(size, 3, rects=LAYOUTS[layout](rng, size), seed=7)
    L().eq_fluid_set_boundaries(p.gpu.handle, mode, DE)
    oracle.set_boundaries(mode, p.ref.fields[DE], size, p.ref.cells)
    p.compare(f"set_boundaries mode={mode} {layout}", [DE])
    p.close()


@pytest.mark.parametrize("mode", [ROW, COL, PAS])
@pytest.mark.parametrize("layout", list(LAYOUTS))
@pytest.mark.parametrize("size,iters", [(20, 1), (23, 3), (40, 20), (66, 7), (97, 33),
                                         (130, 20)])
def test_lin_solve(eqlib, mode, layout, size, iters):
    rng = np.random.default_rng(size * 1000 + iters)
    p = Pair(size, iters, rects=LAYOUTS[layout](rng, size), seed=size + iters)
    a, c = np.float32(0.37), np.float32(1.0) + np.float32(4.0) * np.float32(0.37)
    assert L().eq_fluid_lin_solve(p.gpu.handle, mode, VX0, VX, a, c) == 0
    oracle.lin_solve(mode, p.ref.fields[VX0], p.ref.fields[VX], a, c, size, iters,
                     p.ref.cells)
    p.compare(f"lin_solve mode={mode} {layout} size={size} iters={iters}", [VX0, VX])
    p.close()


def test_lin_solve_many_sweeps_chunked(eqlib):
    """More sweeps than one launch pipelines (64): the solve is split."""
    size, iters = 45, 150
    rng = np.random.default_rng(5)
    p = Pair(size, iters, rects=random_rects(rng, size, 3), seed=9)
    assert L().eq_fluid_lin_solve(p.gpu.handle, PAS, SC, DE, 1.0, 4.0) == 0
    oracle.lin_solve(PAS, p.ref.fields[SC], p.ref.fields[DE], 1.0, 4.0, size, iters,
                     p.ref.cells)
    p.compare("lin_solve chunked", [SC])
    p.close()


@pytest.mark.parametrize("mode", [ROW, COL, PAS])
@pytest.mark.parametrize("vel_scale", [0.05, 1.0, 30.0])
@pytest.mark.parametrize("size", [20, 50, 129])
def test_advect(eqlib, mode, vel_scale, size):
    """Large velocities push backtraces onto the clamps and force row breaks."""
    rng = np.random.default_rng(size + int(vel_scale * 10))
    p = Pair(size, 2, dt=0.1, rects=random_rects(rng, size, 3), seed=size, vel_scale=vel_scale)
    assert L().eq_fluid_advect(p.gpu.handle, mode, DE, SC, VX, VY) == 0
    oracle.advect(mode, p.ref.fields[DE], p.ref.fields[SC], p.ref.fields[VX], p.ref.fields[VY],
                  size, np.float32(0.1), p.ref.cells)
    p.compare(f"advect mode={mode} scale={vel_scale} size={size}", [DE])
    p.close()


def test_advect_forced_row_break(eqlib):
    """Rows whose backtrace hits size-1 at a chosen column: the break copies the
    left neighbour and leaves the rest of the row stale (fluid.rs:420-423)."""
    size = 40
    p = Pair(size, 1, dt=0.1, seed=3, vel_scale=0.2)
    dt0 = np.float32(0.1) * np.float32(size - 2)
    u = p.ref.fields[VX].reshape(size, size)
    for j, i in [(3, 1), (7, 10), (11, size - 2), (20, 2)]:
        # x = i - dt0*u = size-1 exactly when u = (i - (size-1)) / dt0 (clamped anyway)
        u[j, i] = np.float32(-50.0)  # far to the right: clamps to size-1
    p.push()
    assert L().eq_fluid_advect(p.gpu.handle, PAS, DE, SC, VX, VY) == 0
    oracle.advect(PAS, p.ref.fields[DE], p.ref.fields[SC], p.ref.fields[VX], p.ref.fields[VY],
                  size, np.float32(0.1), p.ref.cells)
    p.compare("advect forced break", [DE])
    p.close()


@pytest.mark.parametrize("layout", ["open", "random4", "touching_frame", "checker"])
@pytest.mark.parametrize("size,iters", [(20, 1), (48, 20), (101, 9)])
def test_project(eqlib, layout, size, iters):
    rng = np.random.default_rng(size * 7 + iters)
    p = Pair(size, iters, rects=LAYOUTS[layout](rng, size), seed=size)
    assert L().eq_fluid_project(p.gpu.handle, VX0, VY0, VX, VY) == 0
    oracle.project(p.ref.fields[VX0], p.ref.fields[VY0], p.ref.fields[VX], p.ref.fields[VY],
                   size, iters, p.ref.cells)
    p.compare(f"project {layout} size={size}", [VX0, VY0, VX, VY])
    p.close()


@pytest.mark.parametrize("layout", list(LAYOUTS))
@pytest.mark.parametrize("size,iters,frames", [(20, 1, 3), (34, 4, 5), (66, 20, 3),
                                                (131, 20, 2)])
def test_full_step_random_state(eqlib, layout, size, iters, frames):
    rng = np.random.default_rng(size + 31 * iters)
    p = Pair(size, iters, dt=0.1, diff=1e-3, visc=2e-3, rects=LAYOUTS[layout](rng, size),
             seed=size * 3, vel_scale=2.0)
    for fr in range(frames):
        p.gpu.step()
        p.ref.step()
        p.compare(f"step {fr} {layout} size={size} iters={iters}")
    p.close()


@pytest.mark.parametrize("mask", [0, 1, 2, 3])
@pytest.mark.parametrize("solver", [0, 1, 4])
@pytest.mark.parametrize("size", [66, 258])
def test_full_step_concurrency_masks(eqlib, mask, solver, size):
    """step() with the vy and / or the density diffusion on side streams
    (EQ_CONC_* bits) under both lin_solve kernels: the reference's frames."""
    rng = np.random.default_rng(size + mask)
    p = Pair(size, 20, dt=0.1, diff=1e-3, visc=2e-3, rects=LAYOUTS["random4"](rng, size),
             seed=size + 7 * mask, vel_scale=2.0)
    assert L().eq_fluid_set_concurrency(p.gpu.handle, mask) == 0
    assert L().eq_fluid_set_solver(p.gpu.handle, solver) == 0
    for fr in range(3):
        p.gpu.step()
        p.ref.step()
        p.compare(f"step {fr} mask={mask} solver={solver} size={size}")
    assert L().eq_fluid_set_concurrency(p.gpu.handle, 4) != 0
    p.close()


def test_frames_zero_is_identity(eqlib):
    """frames = 0: lin_solve runs no sweep and no set_boundaries."""
    p = Pair(30, 0, seed=1)
    p.gpu.step()
    p.ref.step()
    p.compare("frames=0 step")
    p.close()


def test_default_fluid_and_obstacle_walls(eqlib):
    """renderer_helpers.rs:222-252: default scene has 1408 DefaultWall cells."""
    from equilibrium_gb300.simulation import CurrentSimulation
    cs = CurrentSimulation.default()
    cs.mark_fluid_obstacles()
    walls = int((cs.fluid.cells_type == 1).sum())
    size = cs.fluid.simulation_configs.size
    assert walls == 2 * (size + size - 2) + 30 * 30 == 1408
    # Default runs init() twice (fluid.rs:83-89)
    vx = cs.fluid.velocities_x
    assert np.all(vx == np.float32(2.0))
    cs.fluid.close()
