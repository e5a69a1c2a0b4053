"""Generates the golden frame-step fixtures in this folder from pyref.py.

    python tests/golden/make_golden.py

Each fixture holds the six input arrays, the wall mask, the scene parameters,
the per-frame sources and the six arrays after the frames, all computed by the
pure-Python restatement (independent of oracle/). The C++ oracle and the GPU
library are both checked against these bit for bit.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import pyref  # noqa: E402

F = np.float32

SCENES = {
    # name: size, iters, dt, diff, visc, rects, randomize, vel_scale, frames, sources
    "s20_k2_default_init": dict(size=20, iters=2, dt=0.1, diff=1e-3, visc=2e-3,
                                rects=[(4, 4, 7, 9)], rand=False, vel=0.0, frames=2, nsrc=3),
    "s22_k3_random_state": dict(size=22, iters=3, dt=0.1, diff=1e-3, visc=1e-3,
                                rects=[(0, 5, 4, 9), (15, 2, 22, 6), (8, 12, 11, 20)],
                                rand=True, vel=2.0, frames=1, nsrc=0),
    "s24_k1_row_breaks": dict(size=24, iters=1, dt=0.2, diff=0.0, visc=1e-3,
                              rects=[(10, 0, 12, 24)], rand=True, vel=30.0, frames=1, nsrc=2),
    "s21_k4_blocked_row": dict(size=21, iters=4, dt=0.05, diff=5e-3, visc=5e-3,
                               rects=[(0, 10, 21, 11), (3, 3, 5, 5)], rand=True, vel=1.0,
                               frames=2, nsrc=1),
}


def make(name, p, seed):
    s = p["size"]
    f, wall = pyref.new_state(s)
    for r in p["rects"]:
        pyref.fill_obstacle(wall, s, *r)
    rng = np.random.default_rng(seed)
    if p["rand"]:
        for k in range(6):
            if k >= 2:
                f[k][:] = rng.uniform(-p["vel"], p["vel"], s * s).astype(F)
            else:
                f[k][:] = rng.uniform(0, 2, s * s).astype(F)
    nf, ns = p["frames"], p["nsrc"]
    sx = rng.integers(1, s - 1, (nf, ns)).astype(np.uint32)
    sy = rng.integers(1, s - 1, (nf, ns)).astype(np.uint32)
    sd = rng.uniform(0, 100, (nf, ns)).astype(F)
    su = rng.uniform(-5, 5, (nf, ns)).astype(F)
    sv = rng.uniform(-5, 5, (nf, ns)).astype(F)
    inp = [a.copy() for a in f]
    for fr in range(nf):
        for k in range(ns):
            q = pyref._ix(int(sx[fr, k]), int(sy[fr, k]), s)
            f[1][q] += sd[fr, k]
            f[0][q] += sd[fr, k]
            f[2][q] += su[fr, k]
            f[3][q] += sv[fr, k]
        pyref.step(f, wall, s, p["dt"], p["iters"], p["diff"], p["visc"])
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"), size=s, iters=p["iters"], dt=F(p["dt"]),
        diff=F(p["diff"]), visc=F(p["visc"]), cells=wall, fields_in=np.stack(inp),
        fields_out=np.stack(f), sx=sx, sy=sy, sd=sd, su=su, sv=sv)


if __name__ == "__main__":
    for n, (name, p) in enumerate(SCENES.items()):
        make(name, p, 100 + n)
        print("wrote", name)
