"""lin_solve by the strip wavefront (csrc/lssw.cuh, solver 3) against the
oracle, bit for bit: every mode, obstacle layouts that touch the frame and
put walls next to strip edges, sweep counts from 1 to past one launch (20),
sizes from the smallest grid to N = 2048; repeated launches on the same
buffers (the export tags come from a device epoch); full frames under every
concurrency mask; a captured frame loop."""
import numpy as np
import pytest

import oracle
from equilibrium_gb300 import _lib
from equilibrium_gb300.simulation import Fluid, FluidConfigs, SimulationConfigs
from tests.util import assert_bitexact, random_rects

pytestmark = pytest.mark.gpu

ROW, COL, PAS = _lib.MODE_ADJUST_ROW, _lib.MODE_ADJUST_COLUMN, _lib.MODE_PASSIVE


def rects_for(size, rng):
    """Walls on the frame, single cells, thin walls, walls two cells apart, and
    walls along the rows where strips meet (32 b - 2 k)."""
    out = [(0, 5, 4, 9), (size - 4, 2, size, 6), (6, 0, 9, 3), (10, size - 3, 14, size),
           (size // 2, size // 3, size // 2 + 1, size // 3 + 7), (12, 12, 13, 13),
           (14, 12, 15, 13), (size // 3, size // 2, size // 3 + 9, size // 2 + 1)]
    for y in (30, 31, 32, 33, 62, 64):
        if y + 2 < size - 1:
            x0 = int(rng.integers(1, max(2, size - 12)))
            out.append((x0, y, min(size - 1, x0 + 7), y + 1))
    out += random_rects(rng, size, 4)
    return out


def scene(size, K, seed):
    L = _lib.load()
    f = Fluid(FluidConfigs(1e-4, 1e-4, False), SimulationConfigs(0.1, K, size))
    r = oracle.OracleFluid(size, 0.1, K, 1e-4, 1e-4)
    rng = np.random.default_rng(seed)
    for rc in rects_for(size, rng):
        _lib.check(L.eq_fluid_fill_obstacle(f.handle, *rc))
        r.fill_obstacle(*rc)
    _lib.check(L.eq_fluid_set_solver(f.handle, 3))
    return f, r, rng


@pytest.mark.parametrize("size,K", [(20, 1), (20, 20), (34, 3), (66, 20), (97, 7), (130, 21),
                                    (258, 20), (514, 20), (1026, 20), (1026, 45), (2050, 20)])
@pytest.mark.parametrize("mode", [ROW, COL, PAS])
def test_strip_lin_solve_bitexact(eqlib, size, K, mode):
    L = _lib.load()
    f, r, rng = scene(size, K, size * 7 + K + mode)
    n = size * size
    x = rng.normal(size=n).astype(np.float32)
    x0 = rng.normal(size=n).astype(np.float32)
    a = np.float32(0.37) if mode != PAS else np.float32(1.0)
    c = np.float32(1.0) + np.float32(4.0) * a if mode != PAS else np.float32(4.0)
    ref = x.copy()
    oracle.lin_solve(mode, ref, x0, a, c, size, K, r.cells)
    f.write_field(2, x)
    f.write_field(4, x0)
    _lib.check(L.eq_fluid_lin_solve(f.handle, mode, 2, 4, a, c))
    f.synchronize()
    assert_bitexact(f.read_field(2), ref, f"strip lin_solve size {size} mode {mode} K {K}", size)
    f.close()


@pytest.mark.parametrize("size,K,groups", [(66, 20, 1), (66, 20, 3), (97, 13, 2), (258, 20, 5),
                                           (514, 20, 2), (1026, 20, 1), (1026, 20, 4),
                                           (1026, 7, 5)])
@pytest.mark.parametrize("mode", [ROW, COL, PAS])
def test_strip_lin_solve_groups_bitexact(eqlib, size, K, groups, mode):
    """Every split of a strip's sweeps over blocks gives the same bits."""
    L = _lib.load()
    f, r, rng = scene(size, K, size * 11 + K + mode + groups)
    _lib.check(L.eq_fluid_set_strip_groups(f.handle, groups))
    n = size * size
    x = rng.normal(size=n).astype(np.float32)
    x0 = rng.normal(size=n).astype(np.float32)
    a = np.float32(0.61)
    c = np.float32(1.0) + np.float32(4.0) * a
    ref = x.copy()
    oracle.lin_solve(mode, ref, x0, a, c, size, K, r.cells)
    f.write_field(2, x)
    f.write_field(4, x0)
    _lib.check(L.eq_fluid_lin_solve(f.handle, mode, 2, 4, a, c))
    f.synchronize()
    assert_bitexact(f.read_field(2), ref, f"strip groups {groups} size {size} mode {mode}", size)
    f.close()


def test_strip_lin_solve_repeated_launches(eqlib):
    """Thirty solves on the same buffers, each from fresh inputs: every launch
    must ignore the previous launch's exports (the epoch tag)."""
    size, K = 514, 20
    L = _lib.load()
    f, r, rng = scene(size, K, 5)
    n = size * size
    for q in range(30):
        mode = (ROW, COL, PAS)[q % 3]
        x = rng.normal(size=n).astype(np.float32)
        x0 = rng.normal(size=n).astype(np.float32)
        a = np.float32(rng.uniform(0.01, 3.0))
        c = np.float32(1.0) + np.float32(4.0) * a
        f.write_field(2, x)
        f.write_field(4, x0)
        _lib.check(L.eq_fluid_lin_solve(f.handle, mode, 2, 4, a, c))
        f.synchronize()
        if q % 5 == 0 or q == 29:
            ref = x.copy()
            oracle.lin_solve(mode, ref, x0, a, c, size, K, r.cells)
            assert_bitexact(f.read_field(2), ref, f"repeat {q} mode {mode}", size)
    f.close()


@pytest.mark.parametrize("mask", [0, 1, 2, 3])
@pytest.mark.parametrize("size", [130, 1026])
def test_strip_full_steps(eqlib, mask, size):
    """Frames with sources, the strip wavefront in every solve, under every
    concurrency mask (up to three strip solves side by side)."""
    K = 20
    L = _lib.load()
    f = Fluid(FluidConfigs(1e-5, 1e-5, False), SimulationConfigs(0.05, K, size))
    r = oracle.OracleFluid(size, 0.05, K, 1e-5, 1e-5)
    rng = np.random.default_rng(size + mask)
    for rc in random_rects(rng, size, 6):
        _lib.check(L.eq_fluid_fill_obstacle(f.handle, *rc))
        r.fill_obstacle(*rc)
    _lib.check(L.eq_fluid_set_solver(f.handle, 3))
    _lib.check(L.eq_fluid_set_concurrency(f.handle, mask))
    xs = np.array([size // 3, size // 3 + 1, size // 2], dtype=np.uint32)
    ys = np.array([size // 2, size // 2, size // 5], dtype=np.uint32)
    d = np.array([40.0, 10.0, 25.0], dtype=np.float32)
    u = np.array([3.0, -2.0, 0.5], dtype=np.float32)
    v = np.array([-1.0, 4.0, 2.5], dtype=np.float32)
    nfr = 3
    for _ in range(nfr):
        f.add_sources(xs, ys, d, u, v)
        f.step()
    r.run(nfr, np.tile(xs, (nfr, 1)), np.tile(ys, (nfr, 1)), np.tile(d, (nfr, 1)),
          np.tile(u, (nfr, 1)), np.tile(v, (nfr, 1)))
    f.synchronize()
    for k in range(6):
        assert_bitexact(f.read_field(k), r.fields[k], f"mask {mask} field {oracle.FIELDS[k]}",
                        size)
    f.close()


def test_strip_captured_frame_loop(eqlib):
    """The graph-captured frame loop replays strip solves with the device
    epoch: two replays of a 2-frame graph equal four eager frames."""
    size, K = 258, 20
    L = _lib.load()
    f = Fluid(FluidConfigs(1e-4, 1e-4, False), SimulationConfigs(0.1, K, size))
    r = oracle.OracleFluid(size, 0.1, K, 1e-4, 1e-4)
    rng = np.random.default_rng(3)
    for rc in random_rects(rng, size, 5):
        _lib.check(L.eq_fluid_fill_obstacle(f.handle, *rc))
        r.fill_obstacle(*rc)
    _lib.check(L.eq_fluid_set_solver(f.handle, 3))
    for _ in range(2):
        _lib.check(L.eq_fluid_step_graph(f.handle, 2, 0, 0))
    r.run(4, np.zeros((4, 0), np.uint32), np.zeros((4, 0), np.uint32),
          np.zeros((4, 0), np.float32), np.zeros((4, 0), np.float32),
          np.zeros((4, 0), np.float32))
    f.synchronize()
    for k in range(6):
        assert_bitexact(f.read_field(k), r.fields[k], f"graph field {oracle.FIELDS[k]}", size)
    f.close()
