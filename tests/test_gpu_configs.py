"""GPU parity on the golden fixtures and on the workloads themselves, plus the
bounded-wait failure path, all through the C ABI."""
import ctypes
import glob
import os

import numpy as np
import pytest

import oracle
from equilibrium_gb300 import _lib
from equilibrium_gb300.simulation import Fluid, FluidConfigs, SimulationConfigs
from tests.util import small_workload

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def gpu_fluid(size, iters, dt, diff, visc):
    return Fluid(FluidConfigs(float(diff), float(visc), False),
                 SimulationConfigs(float(dt), int(iters), int(size)), device=0)


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
def test_golden_fixture(eqlib, path):
    z = np.load(path)
    s = int(z["size"])
    g = gpu_fluid(s, int(z["iters"]), z["dt"], z["diff"], z["visc"])
    g.cells_type = z["cells"]
    for k in range(6):
        g.write_field(k, z["fields_in"][k])
    for fr in range(z["sx"].shape[0]):
        if z["sx"].shape[1]:
            g.add_sources(z["sx"][fr], z["sy"][fr], z["sd"][fr], z["su"][fr], z["sv"][fr])
        g.step()
    for k in range(6):
        assert np.array_equal(bits(g.read_field(k)), bits(z["fields_out"][k])), oracle.FIELDS[k]
    g.close()


def test_small_workload_100_frames_bitexact(eqlib):
    """N=64 interior, dt=0.1, diff=visc=1e-4, 20 sweeps, 100 frames, sources on
    the 5x5 centre patch every frame, one seeded rectangle of ~10% area."""
    size, iters, dt, dv, rect, xs, ys, d, u, v = small_workload(100)
    x0, y0, x1, y1 = rect
    w, h = x1 - x0, y1 - y0
    g = gpu_fluid(size, iters, dt, dv, dv)
    assert eqlib.eq_fluid_fill_obstacle(g.handle, x0, y0, x0 + w, y0 + h) == 0
    r = oracle.OracleFluid(size, dt, iters, dv, dv)
    r.fill_obstacle(x0, y0, x0 + w, y0 + h)
    done = 0
    for upto in (1, 10, 100):
        for fr in range(done, upto):
            g.add_sources(xs[fr], ys[fr], d[fr], u[fr], v[fr])
            g.step()
        r.run(upto - done, xs[done:upto], ys[done:upto], d[done:upto], u[done:upto],
              v[done:upto])
        done = upto
        for k in range(6):
            assert np.array_equal(bits(g.read_field(k)), bits(r.fields[k])), (upto, k)
    g.close()


def test_large_workload_two_frames_bitexact(eqlib):
    """The benchmark scene itself (N=1024) for two frames against the oracle."""
    import bench
    rects, sx, sy, sd, su, sv = bench.scene(bench.SEED, 2)
    g = gpu_fluid(bench.SIZE, bench.ITERS, bench.DT, bench.DIFF, bench.VISC)
    r = oracle.OracleFluid(bench.SIZE, bench.DT, bench.ITERS, bench.DIFF, bench.VISC)
    for rc in rects:
        assert eqlib.eq_fluid_fill_obstacle(g.handle, *rc) == 0
        r.fill_obstacle(*rc)
    for fr in range(2):
        g.add_sources(sx[fr], sy[fr], sd[fr], su[fr], sv[fr])
        g.step()
    r.run(2, sx, sy, sd, su, sv)
    for k in range(6):
        assert np.array_equal(bits(g.read_field(k)), bits(r.fields[k])), oracle.FIELDS[k]
    g.close()


def test_bounded_wait_reports_timeout_and_recovers(eqlib):
    """A spin budget of one poll makes the multi-block wavefront's waits run
    out: the kernel records EQ_ERR_TIMEOUT in its error word and every block
    returns; the handle stays usable. No fault, trap or hang is involved. (The
    cluster wavefront, the default at this size, has no inter-block waits:
    it synchronises with cluster barriers, so the multi-block form is
    selected here.)"""
    g = gpu_fluid(300, 20, 0.1, 1e-4, 1e-4)
    assert eqlib.eq_fluid_set_solver(g.handle, 1) == 0
    assert eqlib.eq_fluid_set_spin_limit(g.handle, 1) == 0
    g.step()
    rc = eqlib.eq_fluid_synchronize(g.handle)
    assert rc == _lib.EQ_ERR_TIMEOUT, rc
    assert b"bounded" in eqlib.eq_last_error()
    # back to the default budget: a fresh scene steps bit-exactly again
    assert eqlib.eq_fluid_set_spin_limit(g.handle, 1 << 22) == 0
    r = oracle.OracleFluid(300, 0.1, 20, 1e-4, 1e-4)
    for k in range(6):
        g.write_field(k, r.fields[k])
    g.step()
    r.step()
    assert eqlib.eq_fluid_synchronize(g.handle) == 0
    for k in range(6):
        assert np.array_equal(bits(g.read_field(k)), bits(r.fields[k]))
    g.close()


def test_clone_is_a_deep_copy(eqlib):
    g = gpu_fluid(40, 5, 0.1, 1e-3, 1e-3)
    g.step()
    c = g.clone()
    before = c.density.copy()
    g.step()
    assert np.array_equal(bits(c.density), bits(before))
    c.step()
    assert np.array_equal(bits(c.density), bits(g.density))
    g.close()
    c.close()


def test_current_simulation_frame_loop(eqlib):
    """renderer_helpers.rs:52-72 with noise off: obstacles, then step + clone per frame."""
    from equilibrium_gb300.simulation import CurrentSimulation, Rectangle
    fl = gpu_fluid(64, 4, 0.1, 1e-3, 1e-3)
    fl.simulation_configs.frames = 3
    cs = CurrentSimulation(fl, [Rectangle((10, 10), (20, 30), 64)])
    got = []
    cs.simulate(lambda st: got.append((st.frame_number, st.fluid.density)))
    r = oracle.OracleFluid(64, 0.1, 3, 1e-3, 1e-3)
    r.fill_obstacle(10, 10, 20, 30)
    for fr in range(3):
        r.step()
        assert got[fr][0] == fr
        assert np.array_equal(bits(got[fr][1]), bits(r.field("density")))
    fl.close()


def test_cpp_host_mirror_runs_reference_unit_tests(eqlib, tmp_path):
    """Compiles tests/mirror_check.cpp (the reference's unit tests restated on
    the C++ mirror) against libeqfluid.so and runs it."""
    import subprocess
    root = os.path.dirname(HERE)
    libdir = os.path.join(root, "equilibrium_gb300")
    exe = str(tmp_path / "mirror_check")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", root, "-I",
                           os.path.join(libdir, "host"), "-o", exe,
                           os.path.join(HERE, "mirror_check.cpp"), "-L", libdir,
                           "-leqfluid", f"-Wl,-rpath,{libdir}",
                           "-Wl,-rpath,/usr/local/cuda/lib64"])
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "mirror_check: ok" in out.stdout
