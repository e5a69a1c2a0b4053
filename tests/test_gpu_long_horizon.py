"""Long-horizon parity: the GPU state of the two plain workloads at frames 1,
10, 100 (N = 64) and 1, 10, 100, 1000 (N = 1024) hashes to the oracle's
state (tests/golden/long_horizon_hashes.json, made by make_long_hashes.py),
all six fields with ghost cells, bit for bit, under several lin_solve
kernels and concurrency masks. A race that shows up once in thousands of
wavefront hand-offs would break the chain of 1000 frames."""
import json
import os

import numpy as np
import pytest

import oracle
from equilibrium_gb300 import _lib
from equilibrium_gb300.simulation import Fluid, FluidConfigs, SimulationConfigs
from tests.util import small_workload, state_hashes

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
HASHES = os.path.join(HERE, "golden", "long_horizon_hashes.json")


def _check(f, want, frame, label):
    got = state_hashes([f.read_field(k) for k in range(6)])
    bad = [oracle.FIELDS[k] for k in range(6) if got[k] != want[k]]
    assert not bad, f"{label}: frame {frame} differs from the oracle in {bad}"


def _run(case, sources, solver, conc, label):
    L = _lib.load()
    c = json.load(open(HASHES))[case]
    f = Fluid(FluidConfigs(c["diffusion"], c["viscosity"], False),
              SimulationConfigs(c["delta_t"], c["iters"], c["size"]), device=0)
    for r in c["rects"]:
        _lib.check(L.eq_fluid_fill_obstacle(f.handle, *r))
    _lib.check(L.eq_fluid_set_solver(f.handle, solver))
    _lib.check(L.eq_fluid_set_concurrency(f.handle, conc))
    sx, sy, sd, su, sv = sources
    done = 0
    for frame in sorted(int(k) for k in c["checkpoints"]):
        for fr in range(done, frame):
            f.add_sources(sx[fr], sy[fr], sd[fr], su[fr], sv[fr])
            f.step()
        done = frame
        f.synchronize()
        _check(f, c["checkpoints"][str(frame)], frame, label)
    f.close()


# solver 0: the strip wavefront; 4: the cluster / multi-block split; 1: the
# multi-block wavefront
@pytest.mark.parametrize("solver,conc", [(0, 3), (1, 0), (4, 3)])
def test_n64_workload_100_frames(eqlib, solver, conc):
    size, iters, dt, dv, rect, xs, ys, d, u, v = small_workload(100)
    _run("n64", (xs, ys, d, u, v), solver, conc, f"N=64 solver {solver} conc {conc}")


@pytest.mark.parametrize("solver,conc", [(0, 3), (0, 0), (4, 3)])
def test_n1024_workload_1000_frames(eqlib, solver, conc):
    import bench
    c = json.load(open(HASHES))["n1024"]
    rects, sx, sy, sd, su, sv = bench.scene(bench.SEED, c["frames"])
    assert [list(r) for r in rects] == c["rects"]
    _run("n1024", (sx, sy, sd, su, sv), solver, conc, f"N=1024 solver {solver} conc {conc}")
