"""CPU tests: the oracle against the golden fixtures and the reference's own
fixtures, hand-derived known answers, the order-independence of
set_boundaries that the kernels rely on, and the host-side API checks.
"""
import glob
import os

import numpy as np
import pytest

import oracle
from tests.golden import pyref

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
def test_oracle_matches_golden(path):
    z = np.load(path)
    s = int(z["size"])
    o = oracle.OracleFluid(s, float(z["dt"]), int(z["iters"]), float(z["diff"]), float(z["visc"]))
    for k in range(6):
        o.fields[k][:] = z["fields_in"][k]
    o.cells[:] = z["cells"]
    o.run(z["sx"].shape[0], z["sx"], z["sy"], z["sd"], z["su"], z["sv"])
    for k in range(6):
        assert np.array_equal(bits(o.fields[k]), bits(z["fields_out"][k])), oracle.FIELDS[k]


def test_golden_fixtures_exist():
    assert len(FIXTURES) >= 4


def test_lin_solve_known_answer():
    """One Passive sweep on a 5x5 interior, x = 0, x0 = unit impulse at (3,3),
    a = 1, c = 4, derived by hand from fluid.rs:313-323 and 179-187, 265-271."""
    s = 7
    x = np.zeros(s * s, np.float32)
    x0 = np.zeros(s * s, np.float32)
    x0[3 + 3 * s] = 1.0
    cells = np.zeros(s * s, np.uint8)
    for k in range(s):
        for q in (k, k + (s - 1) * s, k * s, k * s + s - 1):
            cells[q] = 1
    oracle.lin_solve(oracle.PASSIVE, x, x0, 1.0, 4.0, s, 1, cells)
    X = x.reshape(s, s)  # X[j, i]
    want = {(3, 3): 0.25, (4, 3): 0.0625, (5, 3): 0.015625, (3, 4): 0.0625,
            (4, 4): 0.03125, (5, 4): 0.01171875, (3, 5): 0.015625, (4, 5): 0.01171875,
            (5, 5): 0.005859375,
            # ghost copies of the last interior row/column and the corner mean
            (6, 3): 0.015625, (3, 6): 0.015625, (6, 4): 0.01171875, (4, 6): 0.01171875,
            (6, 5): 0.005859375, (5, 6): 0.005859375, (6, 6): 0.005859375}
    for (i, j), v in want.items():
        assert X[j, i] == np.float32(v), (i, j, X[j, i], v)
    nz = {(i, j) for j in range(s) for i in range(s) if X[j, i] != 0}
    assert nz == set(want)


def test_zero_diffusion_leaves_x0():
    """diffusion = 0 gives a = 0, c = 1: every sweep writes x = x0 exactly."""
    s = 24
    rng = np.random.default_rng(0)
    x = rng.uniform(-1, 1, s * s).astype(np.float32)
    x0 = rng.uniform(-1, 1, s * s).astype(np.float32)
    cells = np.zeros(s * s, np.uint8)
    cells.reshape(s, s)[[0, -1], :] = 1
    cells.reshape(s, s)[:, [0, -1]] = 1
    oracle.diffuse(oracle.PASSIVE, x, x0, 0.0, s, 0.1, 3, cells)
    X, X0 = x.reshape(s, s), x0.reshape(s, s)
    assert np.array_equal(bits(X[1:-1, 1:-1]), bits(X0[1:-1, 1:-1]))


@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("seed", range(6))
def test_set_boundaries_is_order_independent(mode, seed):
    """The reference's sequential cell loop equals a per-cell map over
    pre-pass values (writes hit fluid or frame cells only, reads walls or
    the first/last interior rows) -- the property the kernels are built on."""
    rng = np.random.default_rng(seed)
    s = 22
    _, wall = pyref.new_state(s)
    for _ in range(int(rng.integers(0, 8))):
        x0, y0 = rng.integers(0, s - 1, 2)
        w, h = rng.integers(1, 7, 2)
        pyref.fill_obstacle(wall, s, int(x0), int(y0), int(x0 + w), int(y0 + h))
    if seed == 5:  # a fully blocked row and column
        pyref.fill_obstacle(wall, s, 0, 9, s, 10)
        pyref.fill_obstacle(wall, s, 6, 0, 7, s)
    x = rng.uniform(-3, 3, s * s).astype(np.float32)
    a, b = x.copy(), x.copy()
    pyref.set_boundaries(mode, a, s, wall)
    pyref.set_boundaries_parallel(mode, b, s, wall)
    assert np.array_equal(bits(a), bits(b))
    c = x.copy()
    oracle.set_boundaries(mode, c, s, wall)
    assert np.array_equal(bits(a), bits(c))


def test_default_scene_wall_count():
    """renderer_helpers.rs:222-252: the default scene (size 128, rectangle
    (80,80)-(110,110)) has 2*(128+126) + 30*30 = 1408 DefaultWall cells."""
    f = oracle.OracleFluid(128, 0.02, 16, 0.0, 0.001)
    f.fill_obstacle(80, 80, 110, 110)
    assert int(f.cells.sum()) == 1408


def test_rectangle_validation():
    """obstacle.rs:97-115 (both must panic) and the default rectangle."""
    assert not oracle.rectangle_valid((50, 120), (127, 110), 128)
    assert not oracle.rectangle_valid((12, 12), (10, 10), 128)
    assert oracle.rectangle_valid((80, 80), (110, 110), 128)
    assert not oracle.rectangle_valid((0, 0), (0, 5), 128)
    assert not oracle.rectangle_valid((0, 0), (5, 128), 128)
    assert oracle.rectangle_valid((0, 0), (127, 127), 128)


def test_index_layout():
    """fluid.rs:622-636: idx = x + y*size, x fastest."""
    s = 10
    cells = np.zeros(s * s, np.uint8)
    oracle.fill_obstacle(cells, s, 3, 4, 4, 5)
    assert np.nonzero(cells)[0].tolist() == [3 + 4 * s]


def test_fluid_default_runs_init_twice():
    """fluid.rs:83-89: Default calls new() (which inits) and init() again."""
    f = oracle.OracleFluid(128, 0.02, 16, 0.0, 0.001)
    f.reinit()
    assert np.all(f.field("vx") == np.float32(2.0))
    c = 64
    assert f.field("density")[c + c * 128] == np.float32(0.9) + np.float32(0.9)


def test_f64_oracle_tracks_f32():
    """The f64 instantiation stays close to the f32 one over a few frames."""
    a = oracle.OracleFluid(34, 0.1, 20, 1e-4, 1e-4)
    b = oracle.OracleFluid(34, 0.1, 20, 1e-4, 1e-4, dtype=np.float64)
    for f in (a, b):
        f.fill_obstacle(5, 5, 9, 12)
        f.step()
        f.step()
    d32, d64 = a.field("density").astype(np.float64), b.field("density")
    assert np.linalg.norm(d32 - d64) / np.linalg.norm(d64) < 1e-5


def test_render_rule_restatement():
    """render_image's rule on a 3x3 grid: wall, zero density, saturating casts."""
    d = np.array([0.0, 1.5, 300.0, -2.0, np.nan, 0.5, 2.0, 0.0, 1.0], dtype=np.float32)
    cells = np.array([1, 0, 0, 0, 0, 0, 0, 0, 1], dtype=np.uint8)
    img = oracle.render_rgba(d, cells, 3)
    assert tuple(img[0, 0]) == (255, 0, 0, 255) and tuple(img[2, 2]) == (255, 0, 0, 255)
    assert tuple(img[0, 1]) == (255, 88, 1, 1)            # 1.5 * 208 saturates
    assert tuple(img[1, 2]) == (104, 88, 0, 1)            # 0.5 * 208 truncates
    assert tuple(img[0, 2]) == (255, 88, 255, 1)
    assert tuple(img[1, 0]) == (0, 88, 0, 1)          # negative saturates to 0
    assert tuple(img[1, 1]) == (0, 88, 0, 1)          # NaN != 0, casts to 0
    assert tuple(img[2, 1]) == (94, 146, 162, 128)    # zero density: world colour


def test_noise_angle_is_deterministic_and_bounded():
    from equilibrium_gb300 import _lib
    L = _lib.load()
    a = [L.eq_noise_angle(np.float32(dt)) for dt in (0.02, 0.05, 0.1, 0.02)]
    assert a[0] == a[3]
    assert all(abs(x) <= 6.28 * 2 * 1.5 for x in a)


def test_long_horizon_hashes_reproduce_on_this_host():
    """The committed long-horizon fixture's N = 64 checkpoints are the oracle's
    state on this host too (the 1000-frame N = 1024 run is regenerated by
    tests/golden/make_long_hashes.py, tens of minutes)."""
    import json
    from tests.util import small_workload, state_hashes
    c = json.load(open(os.path.join(HERE, "golden", "long_horizon_hashes.json")))["n64"]
    size, iters, dt, dv, rect, xs, ys, d, u, v = small_workload(100)
    assert c["rects"] == [list(rect)] and c["size"] == size
    f = oracle.OracleFluid(size, dt, iters, dv, dv)
    f.fill_obstacle(*rect)
    done = 0
    for fr in (1, 10, 100):
        f.run(fr - done, xs[done:fr], ys[done:fr], d[done:fr], u[done:fr], v[done:fr])
        done = fr
        assert state_hashes(f.fields) == c["checkpoints"][str(fr)], fr
