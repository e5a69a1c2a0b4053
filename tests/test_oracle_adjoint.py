"""The f64 tape adjoint of the oracle (the checker of the GPU adjoint) against
central finite differences of the f64 forward.

Two kinds of check: single components (one initial velocity cell or one
source cell perturbed, h = 1e-5) and seeded random unit directions over all
parameters (h = 1e-4). The forward is piecewise smooth: a backtrace crossing
a bilinear cell boundary is a kink of the interpolant. With h = 1e-3 a random
direction moves thousands of backtraces and some cross one, which puts the
central difference a few percent off (measured: median 2.7e-2); at h = 1e-4
the agreement is 1e-8. Directions whose +h and -h runs take different
discrete paths (an advect row break or a clamp changes) are skipped."""
import numpy as np
import pytest

import oracle

ARGS = dict(dt=0.1, iters=20, diff=1e-4, visc=1e-4)


def problem(size=34, frames=6, seed=0):
    rng = np.random.default_rng(seed)
    of = oracle.OracleFluid(size, 0.1, 20, 1e-4, 1e-4, dtype=np.float64)
    of.fill_obstacle(size // 4, size // 3, size // 4 + 5, size // 3 + 4)
    init = [f.copy() for f in of.fields]
    n = size * size
    init[2] = init[2] + rng.normal(0, 0.3, n)
    init[3] = init[3] + rng.normal(0, 0.3, n)
    src = rng.uniform(0, 0.5, (frames, n))
    target = oracle.gaussian_target(size, 6, (2.0, 5.0), seed=seed + 1)
    return of.cells, size, init, src, target


def run(cells, size, init, src, target, grads=False):
    return oracle.adjoint_problem_f64(cells, size, ARGS["dt"], ARGS["iters"], ARGS["diff"],
                                      ARGS["visc"], init, src, target, grads=grads)


@pytest.mark.parametrize("frames", [1, 3])
def test_tape_adjoint_single_components(frames):
    cells, size, init, src, target = problem(frames=frames)
    loss, sig, gvx, gvy, gsrc = run(cells, size, init, src, target, grads=True)
    rng = np.random.default_rng(frames)
    h, checked = 1e-5, 0
    for which in ("src", "vx", "vy"):
        for k in rng.integers(size + 1, size * size - size - 1, 6):
            f = int(rng.integers(0, frames))

            def loss_at(sgn):
                ini = [a.copy() for a in init]
                s = src.copy()
                if which == "src":
                    s[f, k] += sgn * h
                else:
                    ini[2 if which == "vx" else 3][k] += sgn * h
                return run(cells, size, ini, s, target)[:2]
            (lp, sp), (lm, sm) = loss_at(+1), loss_at(-1)
            if sp != sig or sm != sig:
                continue
            g = {"src": gsrc[f, k], "vx": gvx[k], "vy": gvy[k]}[which]
            fd = (lp - lm) / (2 * h)
            assert abs(fd - g) <= 1e-6 + 1e-5 * abs(g), (which, k, f, fd, g)
            checked += 1
    assert checked >= 12


def test_tape_adjoint_random_directions():
    cells, size, init, src, target = problem(frames=6)
    loss, sig, gvx, gvy, gsrc = run(cells, size, init, src, target, grads=True)
    rng = np.random.default_rng(100)
    n = size * size
    h, errs = 1e-4, []
    for _ in range(12):
        d = rng.standard_normal(2 * n + src.size)
        d /= np.linalg.norm(d)
        dvx, dvy, dsrc = d[:n], d[n:2 * n], d[2 * n:].reshape(src.shape)
        pred = gvx @ dvx + gvy @ dvy + (gsrc * dsrc).sum()

        def loss_at(sgn):
            ini = [a.copy() for a in init]
            ini[2] = ini[2] + sgn * h * dvx
            ini[3] = ini[3] + sgn * h * dvy
            return run(cells, size, ini, src + sgn * h * dsrc, target)[:2]
        (lp, sp), (lm, sm) = loss_at(+1), loss_at(-1)
        if sp != sig or sm != sig:
            continue
        fd = (lp - lm) / (2 * h)
        errs.append(abs(fd - pred) / max(abs(pred), 1e-12))
    assert len(errs) >= 6
    assert np.median(errs) < 1e-6 and max(errs) < 1e-5, errs


def test_tape_adjoint_frozen_path_fd():
    """Central differences whose perturbed runs replay the unperturbed run's
    advect choices (cells, clamps, row breaks) converge to the tape adjoint's
    directional derivative at second order, at any step size."""
    cells, size, init, src, target = problem(frames=5, seed=3)
    loss, sig, gvx, gvy, gsrc = run(cells, size, init, src, target, grads=True)
    g = np.concatenate([gvx, gvy, gsrc.reshape(-1)])
    rms = np.linalg.norm(g) / np.sqrt(g.size)
    rng = np.random.default_rng(9)
    hs = [1e-2, 1e-3]
    for _ in range(4):
        d = rng.standard_normal(g.size)
        d /= np.linalg.norm(d)
        lo = oracle.fd_direction_f64(cells, size, ARGS["dt"], ARGS["iters"], ARGS["diff"],
                                     ARGS["visc"], init, src, target, d, hs, frozen=True)
        err = [abs((p - m) / (2 * h) - g @ d) / rms for (p, m), h in zip(lo, hs)]
        assert err[1] < 1e-4, err
        assert err[1] < err[0] / 20 or err[1] < 1e-9, err  # O(h^2): ~100x per decade
