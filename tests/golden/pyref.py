"""Second, independent restatement of the reference step in pure Python with
numpy float32 scalars (test infrastructure, tiny grids only).

Written separately from oracle/fluid_oracle.hpp so that the two restatements
check each other. It follows src/simulation/fluid.rs (vkabadzhova/equilibrium):
set_boundaries 133-272, diffuse 276-298, lin_solve 301-325, project 330-375,
advect 378-432, step 437-524, init 527-570/602-606, fill_obstacle 610-619.

It also carries the order-independent formulation of set_boundaries that the
GPU kernels use (`set_boundaries_parallel`), so the tests can show that the
reference's sequential cell loop and the per-cell map agree.
"""
from __future__ import annotations

import math

import numpy as np

F = np.float32
ROW, COL, PAS = 0, 1, 2


def _ix(x, y, s):
    x = min(max(x, 0), s - 1)
    y = min(max(y, 0), s - 1)
    return x + y * s


def set_boundaries(mode, x, s, wall):
    """Sequential, literally as fluid.rs:252-272 (j outer, i inner)."""
    for j in range(s):
        for i in range(s):
            if wall[_ix(i, j, s)]:
                continue
            up, down = (i, min(max(j - 1, 0), s - 1)), (i, min(max(j + 1, 0), s - 1))
            left, right = (min(max(i - 1, 0), s - 1), j), (min(max(i + 1, 0), s - 1), j)
            if mode == ROW:
                if wall[_ix(*left, s)]:
                    x[_ix(i, j, s)] = -x[_ix(*left, s)]
                if wall[_ix(*right, s)]:
                    x[_ix(i, j, s)] = -x[_ix(*right, s)]
            elif mode == COL:
                if wall[_ix(*down, s)]:
                    x[_ix(i, j, s)] = -x[_ix(*down, s)]
                if wall[_ix(*up, s)]:
                    x[_ix(i, j, s)] = -x[_ix(*up, s)]
            else:
                x[_ix(i, 0, s)] = x[_ix(i, 1, s)]
                x[_ix(i, s - 1, s)] = x[_ix(i, s - 2, s)]
                x[_ix(0, j, s)] = x[_ix(1, j, s)]
                x[_ix(s - 1, j, s)] = x[_ix(s - 2, j, s)]
    h = F(0.5)
    x[_ix(0, 0, s)] = h * (x[_ix(1, 0, s)] + x[_ix(0, 1, s)])
    x[_ix(0, s - 1, s)] = h * (x[_ix(1, s - 1, s)] + x[_ix(0, s - 2, s)])
    x[_ix(s - 1, 0, s)] = h * (x[_ix(s - 2, 0, s)] + x[_ix(s - 1, 1, s)])
    x[_ix(s - 1, s - 1, s)] = h * (x[_ix(s - 2, s - 1, s)] + x[_ix(s - 1, s - 2, s)])


def set_boundaries_parallel(mode, x, s, wall):
    """Per-cell map (what the kernels compute): every output from pre-pass values."""
    old = x.copy()
    w = np.asarray(wall).reshape(s, s).astype(bool)
    fluid = ~w
    inner = np.zeros((s, s), bool)
    inner[1:-1, 1:-1] = True
    fl = fluid & inner
    rowfl = fl.any(axis=1)  # row j has a fluid cell
    colfl = fl.any(axis=0)  # column i has a fluid cell
    X = x.reshape(s, s)
    O = old.reshape(s, s)
    if mode == ROW:
        for j in range(1, s - 1):
            for i in range(1, s - 1):
                if not fl[j, i]:
                    continue
                if w[j, i + 1]:
                    X[j, i] = -O[j, i + 1]
                elif w[j, i - 1]:
                    X[j, i] = -O[j, i - 1]
    elif mode == COL:
        for j in range(1, s - 1):
            for i in range(1, s - 1):
                if not fl[j, i]:
                    continue
                if w[j - 1, i]:
                    X[j, i] = -O[j - 1, i]
                elif w[j + 1, i]:
                    X[j, i] = -O[j + 1, i]
    else:
        for i in range(1, s - 1):
            if colfl[i]:
                X[0, i] = O[1, i]
                X[s - 1, i] = O[s - 2, i]
        for j in range(1, s - 1):
            if rowfl[j]:
                X[j, 0] = O[j, 1]
                X[j, s - 1] = O[j, s - 2]
    h = F(0.5)
    X[0, 0] = h * (X[0, 1] + X[1, 0])
    X[s - 1, 0] = h * (X[s - 1, 1] + X[s - 2, 0])
    X[0, s - 1] = h * (X[0, s - 2] + X[1, s - 1])
    X[s - 1, s - 1] = h * (X[s - 1, s - 2] + X[s - 2, s - 1])


def lin_solve(mode, x, x0, a, c, s, iters, wall):
    a, c = F(a), F(c)
    cr = F(1.0) / c
    for _ in range(iters):
        for j in range(1, s - 1):
            for i in range(1, s - 1):
                q = i + j * s
                t = ((x[q + 1] + x[q - 1]) + x[q + s]) + x[q - s]
                x[q] = (x0[q] + a * t) * cr
        set_boundaries(mode, x, s, wall)


def diffuse(mode, x, x0, diff, s, dt, iters, wall):
    sf = F(s - 2)
    a = ((F(dt) * F(diff)) * sf) * sf
    lin_solve(mode, x, x0, a, F(1.0) + F(4.0) * a, s, iters, wall)


def project(vx, vy, p, div, s, iters, wall):
    sf = F(s)
    for j in range(1, s - 1):
        for i in range(1, s - 1):
            q = i + j * s
            div[q] = (F(-0.5) * (((vx[q + 1] - vx[q - 1]) + vy[q + s]) - vy[q - s])) / sf
            p[q] = F(0.0)
    set_boundaries(PAS, div, s, wall)
    set_boundaries(PAS, p, s, wall)
    lin_solve(PAS, p, div, 1.0, 4.0, s, iters, wall)
    for j in range(1, s - 1):
        for i in range(1, s - 1):
            q = i + j * s
            vx[q] = vx[q] - (F(0.5) * (p[q + 1] - p[q - 1])) * sf
            vy[q] = vy[q] - (F(0.5) * (p[q + s] - p[q - s])) * sf
    set_boundaries(ROW, vx, s, wall)
    set_boundaries(COL, vy, s, wall)


def _u32(v):
    v = float(v)
    if math.isnan(v) or v <= 0:
        return 0
    return int(v) if v < 4294967295.0 else 4294967295


def advect(mode, d, d0, u, v, s, dt, wall):
    dt0 = F(dt) * F(s - 2)
    sf = F(s)
    hi = sf - F(1.0)
    for j in range(1, s - 1):
        for i in range(1, s - 1):
            q = i + j * s
            x = F(i) - dt0 * u[q]
            y = F(j) - dt0 * v[q]
            if x < F(0.5):
                x = F(0.5)
            if x > hi:
                x = hi
            if y < F(0.5):
                y = F(0.5)
            if y > hi:
                y = hi
            i0 = F(np.floor(x))
            i1 = i0 + F(1.0)
            j0 = F(np.floor(y))
            j1 = j0 + F(1.0)
            s1 = x - i0
            s0 = F(1.0) - s1
            t1 = y - j0
            t0 = F(1.0) - t1
            a0, a1, b0, b1 = _u32(i0), _u32(i1), _u32(j0), _u32(j1)
            if i1 >= sf or j1 >= sf:
                d[q] = d[_ix(i - 1, j, s)]
                break
            d[q] = s0 * (t0 * d0[_ix(a0, b0, s)] + t1 * d0[_ix(a0, b1, s)]) + \
                s1 * (t0 * d0[_ix(a1, b0, s)] + t1 * d0[_ix(a1, b1, s)])
    set_boundaries(mode, d, s, wall)


def step(f, wall, s, dt, iters, diff, visc):
    """f = [scratch, density, vx, vy, vx0, vy0] float32 arrays, updated in place."""
    sc, de, vx, vy, vx0, vy0 = f
    diffuse(ROW, vx0, vx, visc, s, dt, iters, wall)
    diffuse(COL, vy0, vy, visc, s, dt, iters, wall)
    project(vx0, vy0, vx, vy, s, iters, wall)
    advect(ROW, vx, vx0, vx0, vy0, s, dt, wall)
    advect(COL, vy, vy0, vx0, vy0, s, dt, wall)
    project(vx, vy, vx0, vy0, s, iters, wall)
    diffuse(PAS, sc, de, diff, s, dt, iters, wall)
    advect(PAS, de, sc, vx, vy, s, dt, wall)
    sc[:] = de


def new_state(s):
    f = [np.zeros(s * s, F) for _ in range(6)]
    wall = np.zeros(s * s, np.uint8)
    for j in range(s):
        for i in range(s):
            f[2][_ix(i, j, s)] += F(1.0)
            f[3][_ix(i, j, s)] += F(1.0)
    for j in range(s // 2 - 10, s // 2 + 11):
        for i in range(s // 2 - 10, s // 2 + 11):
            f[1][_ix(i, j, s)] += F(0.9)
            f[0][_ix(i, j, s)] += F(0.9)
    for k in range(s):
        for q in (_ix(k, 0, s), _ix(k, s - 1, s), _ix(0, k, s), _ix(s - 1, k, s)):
            wall[q] = 1
    return f, wall


def fill_obstacle(wall, s, x0, y0, x1, y1):
    for x in range(x0, x1):
        for y in range(y0, y1):
            wall[_ix(x, y, s)] = 1
