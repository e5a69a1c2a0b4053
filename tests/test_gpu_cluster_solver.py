"""lin_solve by the thread-block-cluster wavefronts (csrc/lscl.cuh: strips
staged whole; csrc/lscs.cuh: strips streamed) against the oracle and against
the multi-block wavefront, bit for bit.

The plain handle picks the cluster form by default where it applies, so every
other plain-handle test at those sizes runs it too; these tests also pin that
it is the form in use and cover the sweep counts and obstacle layouts that
stress its boundary gathers (walls on the frame, single-cell walls, thin
walls, walls two cells apart)."""
import ctypes

import numpy as np
import pytest

import oracle
from equilibrium_gb300 import _lib
from equilibrium_gb300.simulation import Fluid, FluidConfigs, SimulationConfigs
from tests.util import assert_bitexact

pytestmark = pytest.mark.gpu

ROW, COL, PAS = _lib.MODE_ADJUST_ROW, _lib.MODE_ADJUST_COLUMN, _lib.MODE_PASSIVE


def rects_for(size):
    return [(0, 5, 4, 9), (size - 4, 2, size, 6), (6, 0, 9, 3), (10, size - 3, 14, size),
            (size // 2, size // 3, size // 2 + 1, size // 3 + 7), (12, 12, 13, 13),
            (14, 12, 15, 13), (size // 3, size // 2, size // 3 + 9, size // 2 + 1)]


def blocks(f):
    c = ctypes.c_int()
    _lib.check(_lib.load().eq_fluid_get_solver(f.handle, ctypes.byref(c)))
    return c.value


@pytest.mark.parametrize("size,K", [(66, 1), (66, 20), (97, 3), (130, 20), (258, 20),
                                    (258, 32), (290, 7)])
@pytest.mark.parametrize("mode", [ROW, COL, PAS])
def test_cluster_lin_solve_bitexact(eqlib, size, K, mode):
    L = _lib.load()
    f = Fluid(FluidConfigs(1e-4, 1e-4, False), SimulationConfigs(0.1, K, size))
    r = oracle.OracleFluid(size, 0.1, K, 1e-4, 1e-4)
    for rc in rects_for(size):
        _lib.check(L.eq_fluid_fill_obstacle(f.handle, *rc))
        r.fill_obstacle(*rc)
    assert blocks(f) >= 2, "the cluster form should apply at this size"
    _lib.check(L.eq_fluid_set_solver(f.handle, 2))  # the cluster form (0 = the strip wavefront)
    rng = np.random.default_rng(size * 3 + K + mode)
    n = size * size
    x = rng.normal(size=n).astype(np.float32)
    x0 = rng.normal(size=n).astype(np.float32)
    f.write_field(2, x)
    f.write_field(4, x0)
    a = np.float32(0.37)
    c = np.float32(1.0) + np.float32(4.0) * a
    _lib.check(L.eq_fluid_lin_solve(f.handle, mode, 2, 4, a, c))
    f.synchronize()
    ref = x.copy()
    oracle.lin_solve(mode, ref, x0, a, c, size, K, r.cells)
    assert_bitexact(f.read_field(2), ref, f"cluster lin_solve mode {mode} K {K}", size)
    # every barrier interval (1, 2, 3, 4 steps) gives the same bits
    for max_m in (0, 2, 3):
        _lib.check(L.eq_fluid_set_cluster_interval(f.handle, max_m))
        f.write_field(2, x)
        _lib.check(L.eq_fluid_lin_solve(f.handle, mode, 2, 4, a, c))
        f.synchronize()
        assert_bitexact(f.read_field(2), ref, f"cluster interval {max_m + 1} mode {mode}", size)
    _lib.check(L.eq_fluid_set_cluster_interval(f.handle, 1))
    # and the multi-block wavefront gives the same bits
    _lib.check(L.eq_fluid_set_solver(f.handle, 1))
    assert blocks(f) == 0
    f.write_field(2, x)
    _lib.check(L.eq_fluid_lin_solve(f.handle, mode, 2, 4, a, c))
    f.synchronize()
    assert_bitexact(f.read_field(2), ref, f"multi-block lin_solve mode {mode} K {K}", size)
    f.close()


def form(f):
    c = ctypes.c_int()
    _lib.check(_lib.load().eq_fluid_get_cluster_form(f.handle, ctypes.byref(c)))
    return c.value


@pytest.mark.parametrize("size,K,nblocks", [(514, 20, 16), (514, 1, 16), (400, 31, 13),
                                            (700, 13, 16), (1026, 20, 16), (1026, 2, 16)])
@pytest.mark.parametrize("mode", [ROW, COL, PAS])
def test_streamed_cluster_lin_solve_bitexact(eqlib, size, K, nblocks, mode):
    """The streamed form: one position per lane (N = 398, 512), two (N = 698
    with a shorter last strip, N = 1024), 31 sweeps (a full 1024-thread
    block with the loader warp), every barrier interval."""
    L = _lib.load()
    f = Fluid(FluidConfigs(1e-4, 1e-4, False), SimulationConfigs(0.1, K, size))
    r = oracle.OracleFluid(size, 0.1, K, 1e-4, 1e-4)
    for rc in rects_for(size):
        _lib.check(L.eq_fluid_fill_obstacle(f.handle, *rc))
        r.fill_obstacle(*rc)
    assert blocks(f) == nblocks and form(f) == 2, "the streamed cluster form should apply"
    _lib.check(L.eq_fluid_set_solver(f.handle, 2))  # the cluster form for this solve too
    rng = np.random.default_rng(size * 5 + K + mode)
    n = size * size
    x = rng.normal(size=n).astype(np.float32)
    x0 = rng.normal(size=n).astype(np.float32)
    a = np.float32(0.37)
    c = np.float32(1.0) + np.float32(4.0) * a
    ref = x.copy()
    oracle.lin_solve(mode, ref, x0, a, c, size, K, r.cells)
    f.write_field(4, x0)
    for max_m in (1, 0, 2, 3):
        _lib.check(L.eq_fluid_set_cluster_interval(f.handle, max_m))
        f.write_field(2, x)
        _lib.check(L.eq_fluid_lin_solve(f.handle, mode, 2, 4, a, c))
        f.synchronize()
        assert_bitexact(f.read_field(2), ref,
                        f"streamed lin_solve mode {mode} K {K} interval {max_m + 1}", size)
    f.close()


def test_streamed_cluster_frames_match_oracle(eqlib):
    """Three frames with sources at N = 1024: the streamed form in every solve
    (three of them side by side in each step), then three more with the
    split of solver 4 (multi-block on the critical path, streamed on the side
    streams)."""
    size, K = 1026, 20
    L = _lib.load()
    f = Fluid(FluidConfigs(1e-5, 1e-5, False), SimulationConfigs(0.05, K, size))
    r = oracle.OracleFluid(size, 0.05, K, 1e-5, 1e-5)
    for rc in rects_for(size):
        _lib.check(L.eq_fluid_fill_obstacle(f.handle, *rc))
        r.fill_obstacle(*rc)
    assert form(f) == 2
    xs = np.array([300, 301, 700], dtype=np.uint32)
    ys = np.array([420, 420, 160], dtype=np.uint32)
    d = np.array([40.0, 10.0, 25.0], dtype=np.float32)
    u = np.array([3.0, -2.0, 0.5], dtype=np.float32)
    v = np.array([-1.0, 4.0, 2.5], dtype=np.float32)
    for solver in (2, 4):
        _lib.check(L.eq_fluid_set_solver(f.handle, solver))
        for _ in range(3):
            f.add_sources(xs, ys, d, u, v)
            f.step()
        r.run(3, np.tile(xs, (3, 1)), np.tile(ys, (3, 1)), np.tile(d, (3, 1)),
              np.tile(u, (3, 1)), np.tile(v, (3, 1)))
        f.synchronize()
        for k in range(6):
            assert_bitexact(f.read_field(k), r.fields[k],
                            f"solver {solver} field {oracle.FIELDS[k]}", size)
    f.close()


def test_cluster_frames_match_oracle(eqlib):
    """Five frames with sources at N = 256 (the cluster form in every solve)."""
    size, K = 258, 20
    L = _lib.load()
    f = Fluid(FluidConfigs(1e-4, 1e-4, False), SimulationConfigs(0.1, K, size))
    r = oracle.OracleFluid(size, 0.1, K, 1e-4, 1e-4)
    for rc in rects_for(size):
        _lib.check(L.eq_fluid_fill_obstacle(f.handle, *rc))
        r.fill_obstacle(*rc)
    assert blocks(f) == 8
    xs = np.array([100, 101, 180], dtype=np.uint32)
    ys = np.array([120, 120, 60], dtype=np.uint32)
    d = np.array([40.0, 10.0, 25.0], dtype=np.float32)
    u = np.array([3.0, -2.0, 0.5], dtype=np.float32)
    v = np.array([-1.0, 4.0, 2.5], dtype=np.float32)
    for _ in range(5):
        f.add_sources(xs, ys, d, u, v)
        f.step()
    r.run(5, np.tile(xs, (5, 1)), np.tile(ys, (5, 1)), np.tile(d, (5, 1)), np.tile(u, (5, 1)),
          np.tile(v, (5, 1)))
    f.synchronize()
    for k in range(6):
        assert_bitexact(f.read_field(k), r.fields[k], f"field {oracle.FIELDS[k]}", size)
    f.close()
