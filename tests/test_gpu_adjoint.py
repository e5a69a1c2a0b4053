"""The differentiation form (eq_grad_*) against the oracle's tape adjoint.

Single phases are checked against the oracle's f64 (linear phases) or f32
(advect, whose discrete choices follow the f32 forward) adjoints; the whole
backward() against the f32 tape adjoint (same forward, same discrete path:
only the adjoint's FP32 rounding order differs) and the f64 tape adjoint;
directional derivatives against central finite differences of the f64
forward. Tolerances are relative L2 norms, stated per check.
"""
import numpy as np
import pytest

import oracle
from equilibrium_gb300 import _lib
from equilibrium_gb300.adjoint import Recorder
from equilibrium_gb300.simulation import Fluid, FluidConfigs, SimulationConfigs

pytestmark = pytest.mark.gpu

ROW, COL, PAS = _lib.MODE_ADJUST_ROW, _lib.MODE_ADJUST_COLUMN, _lib.MODE_PASSIVE

SCENES = {
    "open": [],
    "box": [(8, 11, 14, 16)],
    # obstacles touching the frame, a thin wall, single-cell walls
    "edges": [(0, 5, 4, 9), (-1, 20, 3, 22), (15, 0, 18, 3), (30, 25, 40, 27), (12, 30, 13, 31),
              (22, 12, 23, 13)],
}


def make(size, K=20, dt=0.1, diff=1e-4, visc=1e-4, rects=()):
    f = Fluid(FluidConfigs(diff, visc, False), SimulationConfigs(dt, K, size))
    for r in rects:
        assert _lib.load().eq_fluid_fill_obstacle(f.handle, *r) == 0
    of = oracle.OracleFluid(size, dt, K, diff, visc)
    for r in rects:
        of.fill_obstacle(*r)
    assert np.array_equal(f.cells_type.reshape(-1), of.cells.reshape(-1))
    return f, of


def rel(a, b):
    """Relative L2 distance (absolute when the reference is exactly zero)."""
    den = float(np.linalg.norm(np.asarray(b, np.float64)))
    num = float(np.linalg.norm(np.asarray(a, np.float64) - np.asarray(b, np.float64)))
    return num / den if den > 0.0 else num


@pytest.mark.parametrize("scene", list(SCENES))
@pytest.mark.parametrize("mode", [ROW, COL, PAS])
def test_set_boundaries_adj(eqlib, scene, mode):
    size = 41
    f, of = make(size, rects=SCENES[scene])
    g = Recorder(f, 1)
    rng = np.random.default_rng(mode)
    xb = rng.normal(size=size * size).astype(np.float32)
    got = g.set_boundaries_adj(mode, xb)
    ref = oracle.set_boundaries_adj_f64(mode, xb.astype(np.float64), size, of.cells)
    assert rel(got, ref) < 1e-6, rel(got, ref)
    g.close()
    f.close()


@pytest.mark.parametrize("store", [3, 2, 1, 0])
@pytest.mark.parametrize("size,K", [(20, 1), (20, 2), (41, 3), (41, 20), (66, 20), (130, 7),
                                    (258, 20), (514, 20), (300, 33)])
@pytest.mark.parametrize("mode", [ROW, COL, PAS])
def test_lin_solve_adj(eqlib, size, K, mode, store):
    """store: where the wavefront keeps its band (3 = a cluster of 8 blocks
    where the size allows it, 2 = one block, shared memory for y and its sum,
    1 = y only, 0 = global memory)."""
    rects = SCENES["edges"] if size >= 41 else [(3, 4, 7, 9)]
    f, of = make(size, K=K, rects=rects)
    g = Recorder(f, 1)
    g.set_wavefront_storage(store)
    rng = np.random.default_rng(size * 7 + K + mode)
    xb = rng.normal(size=size * size).astype(np.float32)
    x0b = rng.normal(size=size * size).astype(np.float32)
    a = np.float32(0.37)
    c = np.float32(1.0) + np.float32(4.0) * a
    gx, gx0 = g.lin_solve_adj(mode, xb, x0b, a, c)
    rx, rx0 = oracle.lin_solve_adj_f64(mode, xb.astype(np.float64), x0b.astype(np.float64),
                                       float(a), float(c), size, K, of.cells)
    assert rel(gx, rx) < 1e-5, ("xb", rel(gx, rx))
    assert rel(gx0, rx0) < 1e-5, ("x0b", rel(gx0, rx0))
    if store == 3:  # the cluster form with a barrier every 1 and every 4 steps
        for max_m in (0, 3):
            _lib.check(_lib.load().eq_grad_set_cluster_interval(g.handle, max_m))
            hx, hx0 = g.lin_solve_adj(mode, xb, x0b, a, c)
            assert rel(hx, rx) < 1e-5 and rel(hx0, rx0) < 1e-5, (max_m, rel(hx, rx))
    g.close()
    f.close()


@pytest.mark.parametrize("scale", [0.5, 30.0])
@pytest.mark.parametrize("mode", [ROW, COL, PAS])
def test_advect_adj(eqlib, mode, scale):
    """scale 30: many backtraces clamp and most rows break early."""
    size = 66
    f, of = make(size, dt=0.1, rects=SCENES["edges"])
    g = Recorder(f, 1)
    rng = np.random.default_rng(int(scale) + mode)
    n = size * size
    d0, u, v = (rng.uniform(-1, 1, n).astype(np.float32),
                rng.normal(0, scale, n).astype(np.float32), rng.normal(0, scale, n).astype(np.float32))
    db, d0b, ub, vb = (rng.normal(size=n).astype(np.float32) for _ in range(4))
    got = g.advect_adj(mode, db, d0b, ub, vb, d0, u, v)
    ref = oracle.advect_adj_f32(mode, db, d0b, ub, vb, d0, u, v, size, np.float32(0.1), of.cells)
    for name, a, b in zip(("db", "d0b", "ub", "vb"), got, ref):
        assert rel(a, b.astype(np.float64)) < 1e-5, (name, rel(a, b))
    g.close()
    f.close()


@pytest.mark.parametrize("scene", ["open", "edges"])
def test_project_adj(eqlib, scene):
    size = 41
    f, of = make(size, K=20, rects=SCENES[scene])
    g = Recorder(f, 1)
    rng = np.random.default_rng(5)
    io = [rng.normal(size=size * size).astype(np.float32) for _ in range(4)]
    got = g.project_adj(*io)
    ref = oracle.project_adj_f64(*[a.astype(np.float64) for a in io], size, 20, of.cells)
    for name, a, b in zip(("vxb", "vyb", "pb", "divb"), got, ref):
        assert rel(a, b) < 1e-5, (name, rel(a, b))
    g.close()
    f.close()


def problem(size, frames, rects, seed=0, vel=0.3, src_amp=0.5):
    rng = np.random.default_rng(seed)
    f, of = make(size, K=20, dt=0.1, diff=1e-4, visc=1e-4, rects=rects)
    n = size * size
    init = [fl.copy() for fl in of.fields]
    init[2] = (init[2] + rng.normal(0, vel, n)).astype(np.float32)
    init[3] = (init[3] + rng.normal(0, vel, n)).astype(np.float32)
    for k in range(6):
        f.write_field(k, init[k])
    src = rng.uniform(0, src_amp, (frames, n)).astype(np.float32)
    target = oracle.gaussian_target(size, 6, (2.0, 5.0), seed=seed + 1).astype(np.float32)
    return f, of, init, src, target


@pytest.mark.parametrize("size,frames,every", [(34, 1, 8), (34, 6, 4), (41, 5, 2), (66, 9, 8)])
def test_backward_vs_tape(eqlib, size, frames, every):
    rects = [(size // 4, size // 3, size // 4 + 5, size // 3 + 4), (size // 2, 2, size // 2 + 3, 9)]
    f, of, init, src, target = problem(size, frames, rects)
    g = Recorder(f, frames, every)
    g.forward(src)
    loss = g.l2_loss(target)
    gi, gs = g.backward()
    # f32 tape: the same forward and discrete path as the recording
    l32, s32, vx32, vy32, src32 = oracle.adjoint_problem_f32(
        of.cells, size, 0.1, 20, 1e-4, 1e-4, init, src, target)
    assert abs(loss - l32) <= 1e-5 * abs(l32), (loss, l32)
    assert rel(gi[2], vx32) < 1e-4, ("vx vs f32 tape", rel(gi[2], vx32))
    assert rel(gi[3], vy32) < 1e-4, ("vy vs f32 tape", rel(gi[3], vy32))
    assert rel(gs, src32) < 1e-4, ("src vs f32 tape", rel(gs, src32))
    # f64 tape
    l64, s64, vx64, vy64, src64 = oracle.adjoint_problem_f64(
        of.cells, size, 0.1, 20, 1e-4, 1e-4, [a.astype(np.float64) for a in init],
        src.astype(np.float64), target.astype(np.float64))
    assert s64 == s32  # the f64 run takes the same discrete path here
    # Against f64 the GPU is as close as the reference's own f32 arithmetic
    # allows: the f32 tape's distance to the f64 tape (1e-6 .. 1.5e-3 here,
    # growing with frames) bounds the GPU's, up to the adjoint's rounding.
    for got, t32, t64 in ((gi[2], vx32, vx64), (gi[3], vy32, vy64), (gs, src32, src64)):
        assert rel(got, t64) <= 1.05 * rel(t32, t64) + 2e-5, (rel(got, t64), rel(t32, t64))
    # backward leaves the handle at the run's final state
    fin = oracle.OracleFluid(size, 0.1, 20, 1e-4, 1e-4)
    for r in rects:
        fin.fill_obstacle(*r)
    for k in range(6):
        fin.fields[k][:] = init[k]
    for fr in range(frames):
        fin.fields[0][:] += src[fr]
        fin.fields[1][:] += src[fr]
        fin.step()
    for k in range(6):
        assert np.array_equal(f.read_field(k), fin.fields[k]), k
    g.close()
    f.close()


@pytest.mark.parametrize("size,K,frames,every,vel,store", [
    (37, 1, 3, 1, 0.3, -1),    # one sweep per solve, a checkpoint every frame, odd size
    (40, 0, 2, 1, 0.3, -1),    # no sweeps: lin_solve is the identity, its adjoint too
    (50, 20, 4, 3, 3.0, -1),   # fast flow: many clamped backtraces and early row breaks
    (66, 20, 3, 2, 0.3, 2),    # the single-block transposed solver
    (66, 20, 3, 2, 0.3, 0),    # the global-memory transposed solver
])
def test_backward_more_cases(eqlib, size, K, frames, every, vel, store):
    """backward() against the f32 tape adjoint (the same forward and discrete
    path) across sweep counts, checkpoint spacings and flow speeds."""
    rects = [(size // 4, size // 3, size // 4 + 5, size // 3 + 4), (size - 9, 0, size - 5, 7)]
    rng = np.random.default_rng(size + K)
    f, of = make(size, K=K, dt=0.1, diff=1e-4, visc=1e-4, rects=rects)
    n = size * size
    init = [fl.copy() for fl in of.fields]
    init[2] = (init[2] * 0.0 + rng.normal(0, vel, n)).astype(np.float32)
    init[3] = (init[3] * 0.0 + rng.normal(0, vel, n)).astype(np.float32)
    for k in range(6):
        f.write_field(k, init[k])
    src = rng.uniform(0, 0.5, (frames, n)).astype(np.float32)
    target = oracle.gaussian_target(size, 6, (2.0, 5.0), seed=3).astype(np.float32)
    g = Recorder(f, frames, every)
    if store >= 0:
        g.set_wavefront_storage(store)
    g.forward(src)
    loss = g.l2_loss(target)
    gi, gs = g.backward()
    l32, _, vx32, vy32, src32 = oracle.adjoint_problem_f32(of.cells, size, 0.1, K, 1e-4, 1e-4,
                                                           init, src, target)
    assert abs(loss - l32) <= 1e-5 * abs(l32), (loss, l32)
    for name, got, ref in (("vx", gi[2], vx32), ("vy", gi[3], vy32), ("src", gs, src32)):
        assert rel(got, ref) < 1e-4, (name, rel(got, ref))
    g.close()
    f.close()


def test_backward_concurrency_matches_one_stream(eqlib):
    """The backward's side-stream solves (the handle's concurrency on, the
    default) give the one-stream backward's gradients, up to the summation
    order of advect^T's float atomics; the forward runs are bit-identical
    (the final states), the losses equal up to their FP64 atomic sum."""
    size, frames = 66, 6
    rects = [(size // 4, size // 3, size // 4 + 5, size // 3 + 4), (size // 2, 2, size // 2 + 3, 9)]
    out = []
    for mask in (0, 3):
        f, of, init, src, target = problem(size, frames, rects, seed=3)
        assert _lib.load().eq_fluid_set_concurrency(f.handle, mask) == 0
        g = Recorder(f, frames, 2)
        g.forward(src)
        loss = g.l2_loss(target)
        gi, gs = g.backward()
        out.append((loss, gi, gs, [f.read_field(k) for k in range(6)]))
        g.close()
        f.close()
    (l0, gi0, gs0, fin0), (l1, gi1, gs1, fin1) = out
    assert abs(l1 - l0) <= 1e-12 * abs(l0)  # an FP64 atomic sum: its order varies
    for k in range(6):
        assert np.array_equal(fin0[k], fin1[k]), k
    assert rel(gi1[2], gi0[2]) < 1e-5 and rel(gi1[3], gi0[3]) < 1e-5
    assert rel(gs1, gs0) < 1e-5


def test_backward_explicit_adjoint_and_linearity(eqlib):
    """backward(adj_final) with the l2 seed given explicitly equals the seeded
    call; scaling the seed scales every gradient."""
    size, frames = 34, 3
    f, of, init, src, target = problem(size, frames, [(9, 9, 14, 13)])
    g = Recorder(f, frames, 2)
    g.forward(src)
    loss, adj = g.l2_loss(target, return_adjoint=True)
    gi1, gs1 = g.backward()
    seed = np.zeros((6, size * size), np.float32)
    seed[_lib.FIELD_DENSITY] = adj
    gi2, gs2 = g.backward(2.0 * seed)
    assert rel(gi2, 2.0 * gi1.astype(np.float64)) < 1e-6
    assert rel(gs2, 2.0 * gs1.astype(np.float64)) < 1e-6
    g.close()
    f.close()


def test_backward_fd_random_directions(eqlib):
    """The GPU gradient's directional derivatives against central differences
    of the f64 forward on seeded random unit directions (h = 1e-4; larger h
    moves backtraces across bilinear cell boundaries)."""
    size, frames = 34, 4
    f, of, init, src, target = problem(size, frames, [(9, 9, 14, 13)])
    g = Recorder(f, frames, 2)
    g.forward(src)
    g.l2_loss(target)
    gi, gs = g.backward()
    n = size * size
    init64 = [a.astype(np.float64) for a in init]
    src64 = src.astype(np.float64)
    tgt64 = target.astype(np.float64)
    args = (of.cells, size, 0.1, 20, 1e-4, 1e-4)
    _, sig = oracle.adjoint_problem_f64(*args, init64, src64, tgt64, grads=False)[:2]
    rng = np.random.default_rng(77)
    h, errs = 1e-4, []
    for _ in range(8):
        d = rng.standard_normal(2 * n + src.size)
        d /= np.linalg.norm(d)
        dvx, dvy, dsrc = d[:n], d[n:2 * n], d[2 * n:].reshape(src.shape)
        pred = gi[2].astype(np.float64) @ dvx + gi[3].astype(np.float64) @ dvy + (
            gs.astype(np.float64) * dsrc).sum()

        def loss_at(sgn):
            ini = [a.copy() for a in init64]
            ini[2] = ini[2] + sgn * h * dvx
            ini[3] = ini[3] + sgn * h * dvy
            return oracle.adjoint_problem_f64(*args, ini, src64 + sgn * h * dsrc, tgt64,
                                              grads=False)[:2]
        (lp, sp), (lm, sm) = loss_at(1), loss_at(-1)
        if sp != sig or sm != sig:
            continue
        fd = (lp - lm) / (2 * h)
        errs.append(abs(fd - pred) / max(abs(fd), 1e-12))
    assert len(errs) >= 4 and np.median(errs) < 1e-3, errs


def test_backward_frozen_path_fd(eqlib):
    """The GPU gradient against central differences (h = 1e-3, f64) whose
    perturbed runs replay the unperturbed run's advect choices: the
    derivative of the smooth piece the recording is on. Errors are scaled by
    the gradient's RMS directional derivative |g| / sqrt(dim)."""
    size, frames = 41, 5
    f, of, init, src, target = problem(size, frames, [(9, 9, 14, 13), (25, 2, 29, 12)], seed=4)
    g = Recorder(f, frames, 2)
    g.forward(src)
    g.l2_loss(target)
    gi, gs = g.backward()
    gv = np.concatenate([gi[2], gi[3], gs.reshape(-1)]).astype(np.float64)
    rms = np.linalg.norm(gv) / np.sqrt(gv.size)
    rng = np.random.default_rng(21)
    for _ in range(6):
        d = rng.standard_normal(gv.size)
        d /= np.linalg.norm(d)
        (lp, lm), = oracle.fd_direction_f64(of.cells, size, 0.1, 20, 1e-4, 1e-4, init, src,
                                            target, d, [1e-3], frozen=True)
        err = abs((lp - lm) / 2e-3 - gv @ d) / rms
        assert err < 1e-3, err
    g.close()
    f.close()


def test_grad_rejects_bad_use(eqlib):
    f, of = make(30, rects=[(5, 5, 9, 9)])
    with pytest.raises(_lib.EqError):
        Recorder(f, 0)
    g = Recorder(f, 2, 1)
    with pytest.raises(_lib.EqError):
        g.backward()  # nothing recorded
    with pytest.raises(_lib.EqError):
        g.forward(nframes=3)  # more than max_frames
    g.forward(nframes=2)
    with pytest.raises(_lib.EqError):
        g.backward()  # no seed
    g.l2_loss(np.zeros(30 * 30, np.float32))
    assert _lib.load().eq_fluid_fill_obstacle(f.handle, 20, 20, 24, 24) == 0
    with pytest.raises(_lib.EqError):
        g.backward()  # the mask changed since the forward
    g.close()
    f.close()
