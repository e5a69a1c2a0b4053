"""ORACLE -- test infrastructure only, never the product path.

A ctypes front end to ``fluid_oracle.cpp``: a C++ restatement of the
reference's ``src/simulation/fluid.rs`` (vkabadzhova/equilibrium), used by
``tests/`` as the parity checker, by ``__graft_entry__.smoke()`` as the checker
and by ``bench.py``'s CPU-baseline leg as the timed reference port.

Parity status: numeric parity of this restatement is UNPINNED by the reference
itself (the reference ships no numeric golden vectors and its Rust crate cannot
be built here). It is pinned against the reference's own non-numeric fixtures
(wall-mask count, Rectangle validation, index layout) and cross-checked
against an independent pure-Python restatement (``tests/golden/pyref.py``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libeqoracle.so")
SOURCES = [os.path.join(HERE, "fluid_oracle.cpp"), os.path.join(HERE, "fluid_oracle.hpp"),
           os.path.join(HERE, "adjoint.hpp")]

# Modes (fluid.rs:21-29) and field order (fluid.rs:59-77).
ADJUST_ROW, ADJUST_COLUMN, PASSIVE = 0, 1, 2
FIELDS = ("scratch", "density", "vx", "vy", "vx0", "vy0")

# -ffp-contract=off: Rust never fuses a*b+c; gcc on aarch64 would by default.
CXXFLAGS = ["-O3", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared"]


def build(force: bool = False) -> str:
    """Compile the oracle library in place (g++, a few seconds)."""
    newest = max(os.path.getmtime(s) for s in SOURCES)
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest:
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["g++", *CXXFLAGS, "-o", tmp, SOURCES[0]])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        u32, i64, f32, f64, ci = (ctypes.c_uint32, ctypes.c_int64, ctypes.c_float,
                                  ctypes.c_double, ctypes.c_int)
        sig = {
            "eqo_set_boundaries_f32": (None, [ci, P, u32, P]),
            "eqo_lin_solve_f32": (None, [ci, P, P, f32, f32, u32, i64, P]),
            "eqo_diffuse_f32": (None, [ci, P, P, f32, u32, f32, i64, P]),
            "eqo_project_f32": (None, [P, P, P, P, u32, i64, P]),
            "eqo_advect_f32": (None, [ci, P, P, P, P, u32, f32, P]),
            "eqo_step_f32": (None, [P, P, u32, f32, i64, f32, f32]),
            "eqo_run_f32": (None, [P, P, u32, f32, i64, f32, f32, i64, i64, P, P, P, P, P]),
            "eqo_time_run_f32": (f64, [P, P, u32, f32, i64, f32, f32, i64, i64, P, P, P, P, P]),
            "eqo_new_f32": (None, [u32, P, P]),
            "eqo_reinit_f32": (None, [u32, P, P]),
            "eqo_lin_solve_f64": (None, [ci, P, P, f64, f64, u32, i64, P]),
            "eqo_step_f64": (None, [P, P, u32, f64, i64, f64, f64]),
            "eqo_run_f64": (None, [P, P, u32, f64, i64, f64, f64, i64, i64, P, P, P, P, P]),
            "eqo_new_f64": (None, [u32, P, P]),
            "eqo_set_boundaries_f64": (None, [ci, P, u32, P]),
            "eqo_diffuse_f64": (None, [ci, P, P, f64, u32, f64, i64, P]),
            "eqo_advect_f64": (None, [ci, P, P, P, P, u32, f64, P]),
            "eqo_project_div_f64": (None, [P, P, P, P, u32, P]),
            "eqo_project_grad_f64": (None, [P, P, P, u32, P]),
            "eqo_adjoint_problem_f64": (f64, [P, u32, f64, i64, f64, f64, i64, P, P, P, P, P,
                                              P, P]),
            "eqo_lin_solve_adj_f64": (None, [ci, P, P, f64, f64, u32, i64, P]),
            "eqo_set_boundaries_adj_f64": (None, [ci, P, u32, P]),
            "eqo_advect_adj_f32": (None, [ci, P, P, P, P, P, P, P, u32, f32, P]),
            "eqo_project_adj_f64": (None, [P, P, P, P, u32, i64, P]),
            "eqo_adjoint_problem_f32": (f32, [P, u32, f32, i64, f32, f32, i64, P, P, P, P, P,
                                              P, P]),
            "eqo_fd_direction_f64": (f64, [P, u32, f64, i64, f64, f64, i64, P, P, P, P, P, i64,
                                           ci, P]),
            "eqo_fill_obstacle": (None, [P, u32, i64, i64, i64, i64]),
            "eqo_rectangle_valid": (ci, [i64, i64, i64, i64, i64]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


def _ptr6(fields):
    arr = (ctypes.c_void_p * 6)(*[_ptr(f) for f in fields])
    return arr


class OracleFluid:
    """Host-side state of one scene, laid out exactly like the reference's
    ``Fluid`` (six ``size*size`` arrays incl. the ghost frame + a wall mask)."""

    def __init__(self, size: int, delta_t: float, frames: int, diffusion: float,
                 viscousity: float, dtype=np.float32):
        self.size, self.delta_t, self.frames = int(size), delta_t, int(frames)
        self.diffusion, self.viscousity, self.dtype = diffusion, viscousity, np.dtype(dtype)
        n = self.size * self.size
        self.fields = [np.zeros(n, dtype=self.dtype) for _ in range(6)]
        self.cells = np.zeros(n, dtype=np.uint8)
        fn = lib().eqo_new_f32 if self.dtype == np.float32 else lib().eqo_new_f64
        fn(self.size, _ptr6(self.fields), _ptr(self.cells))

    def field(self, name: str) -> np.ndarray:
        return self.fields[FIELDS.index(name)]

    def reinit(self):
        assert self.dtype == np.float32
        lib().eqo_reinit_f32(self.size, _ptr6(self.fields), _ptr(self.cells))

    def fill_obstacle(self, x0: int, y0: int, x1: int, y1: int):
        lib().eqo_fill_obstacle(_ptr(self.cells), self.size, x0, y0, x1, y1)

    def step(self):
        if self.dtype == np.float32:
            lib().eqo_step_f32(_ptr6(self.fields), _ptr(self.cells), self.size,
                               self.delta_t, self.frames, self.diffusion, self.viscousity)
        else:
            lib().eqo_step_f64(_ptr6(self.fields), _ptr(self.cells), self.size,
                               self.delta_t, self.frames, self.diffusion, self.viscousity)

    def run(self, nframes: int, sx, sy, sd, su, sv, timed: bool = False):
        """``nframes`` frames, each = that frame's sources then step().
        Source arrays have shape (nframes, nsrc)."""
        sx = np.ascontiguousarray(sx, dtype=np.uint32)
        sy = np.ascontiguousarray(sy, dtype=np.uint32)
        sd = np.ascontiguousarray(sd, dtype=np.float32)
        su = np.ascontiguousarray(su, dtype=np.float32)
        sv = np.ascontiguousarray(sv, dtype=np.float32)
        nsrc = sx.shape[1] if sx.ndim == 2 else 0
        args = [_ptr6(self.fields), _ptr(self.cells), self.size, self.delta_t, self.frames,
                self.diffusion, self.viscousity, nframes, nsrc, _ptr(sx), _ptr(sy), _ptr(sd),
                _ptr(su), _ptr(sv)]
        if self.dtype == np.float32:
            if timed:
                return lib().eqo_time_run_f32(*args)
            lib().eqo_run_f32(*args)
        else:
            lib().eqo_run_f64(*args)
        return None


def set_boundaries(mode: int, x: np.ndarray, size: int, cells: np.ndarray):
    lib().eqo_set_boundaries_f32(mode, _ptr(x), size, _ptr(cells))


def lin_solve(mode, x, x0, a, c, size, iters, cells):
    if x.dtype == np.float64:
        lib().eqo_lin_solve_f64(mode, _ptr(x), _ptr(x0), a, c, size, iters, _ptr(cells))
    else:
        lib().eqo_lin_solve_f32(mode, _ptr(x), _ptr(x0), a, c, size, iters, _ptr(cells))


def diffuse(mode, x, x0, diff, size, dt, iters, cells):
    lib().eqo_diffuse_f32(mode, _ptr(x), _ptr(x0), diff, size, dt, iters, _ptr(cells))


def project(vx, vy, p, div, size, iters, cells):
    lib().eqo_project_f32(_ptr(vx), _ptr(vy), _ptr(p), _ptr(div), size, iters, _ptr(cells))


def advect(mode, d, d0, u, v, size, dt, cells):
    lib().eqo_advect_f32(mode, _ptr(d), _ptr(d0), _ptr(u), _ptr(v), size, dt, _ptr(cells))


def fill_obstacle(cells, size, x0, y0, x1, y1):
    lib().eqo_fill_obstacle(_ptr(cells), size, x0, y0, x1, y1)


def rectangle_valid(dl, ur, size) -> bool:
    return bool(lib().eqo_rectangle_valid(dl[0], dl[1], ur[0], ur[1], size))


# ---- f64 reference step with a converged pressure solve --------------------
# Used to measure the precision form (which solves project's pressure equation
# to a relative residual instead of a fixed sweep count) against a reference
# whose only difference is that solve. The pressure equation
#   4 p - (sum of the 4 neighbours) = div,  frame neighbour = adjacent cell
# (set_boundaries(Passive) where every interior row and column holds a fluid
# cell) is the pure-Neumann 5-point Laplacian, which the orthonormal DCT-II
# diagonalises exactly: eigenvalues 4 - 2 cos(pi k / N) - 2 cos(pi l / N). The
# constant mode (zero eigenvalue) is set to zero: zero-mean pressure.


def neumann_pressure_f64(div_interior: np.ndarray) -> np.ndarray:
    from scipy.fft import dctn, idctn
    n = div_interior.shape[0]
    k = np.arange(n)
    lam1 = 2.0 - 2.0 * np.cos(np.pi * k / n)
    lam = lam1[:, None] + lam1[None, :]
    bh = dctn(div_interior, type=2, norm="ortho")
    lam[0, 0] = 1.0
    ph = bh / lam
    ph[0, 0] = 0.0
    return idctn(ph, type=2, norm="ortho")


def _all_rows_cols_fluid(cells: np.ndarray, size: int) -> bool:
    m = cells.reshape(size, size)[1:-1, 1:-1] == 0
    return bool(m.any(axis=1).all() and m.any(axis=0).all())


def converged_step_f64(of: "OracleFluid"):
    """One f64 frame of the reference (fluid.rs:437-524, same aliasing) with both
    pressure solves replaced by the exact pure-Neumann solve."""
    assert of.dtype == np.float64
    S = of.size
    if not _all_rows_cols_fluid(of.cells, S):
        raise ValueError("a fully walled interior row or column makes the frame Dirichlet")
    L = lib()
    sc, de, vx, vy, vx0, vy0 = of.fields
    c = _ptr(of.cells)

    def project(u, v, p, div):
        L.eqo_project_div_f64(_ptr(u), _ptr(v), _ptr(p), _ptr(div), S, c)
        pin = neumann_pressure_f64(div.reshape(S, S)[1:-1, 1:-1].T.copy()).T
        p.reshape(S, S)[1:-1, 1:-1] = pin
        L.eqo_set_boundaries_f64(PASSIVE, _ptr(p), S, c)
        L.eqo_project_grad_f64(_ptr(u), _ptr(v), _ptr(p), S, c)

    dt, K = float(of.delta_t), int(of.frames)
    L.eqo_diffuse_f64(ADJUST_ROW, _ptr(vx0), _ptr(vx), float(of.viscousity), S, dt, K, c)
    L.eqo_diffuse_f64(ADJUST_COLUMN, _ptr(vy0), _ptr(vy), float(of.viscousity), S, dt, K, c)
    project(vx0, vy0, vx, vy)
    L.eqo_advect_f64(ADJUST_ROW, _ptr(vx), _ptr(vx0), _ptr(vx0), _ptr(vy0), S, dt, c)
    L.eqo_advect_f64(ADJUST_COLUMN, _ptr(vy), _ptr(vy0), _ptr(vx0), _ptr(vy0), S, dt, c)
    project(vx, vy, vx0, vy0)
    L.eqo_diffuse_f64(PASSIVE, _ptr(sc), _ptr(de), float(of.diffusion), S, dt, K, c)
    L.eqo_advect_f64(PASSIVE, _ptr(de), _ptr(sc), _ptr(vx), _ptr(vy), S, dt, c)
    sc[:] = de


def add_sources(of: "OracleFluid", xs, ys, d, u, v):
    """add_density / add_velocity (fluid.rs:120-131) in array order, idx!-clamped."""
    S = of.size
    for x, y, dd, uu, vv in zip(xs, ys, d, u, v):
        q = min(int(x), S - 1) + min(int(y), S - 1) * S
        for f, a in ((1, dd), (0, dd), (2, uu), (3, vv)):
            of.fields[f][q] = of.fields[f][q] + of.dtype.type(np.float32(a))


def render_rgba(density: np.ndarray, cells: np.ndarray, size: int,
                fluid=(208, 88, 157, 220), world=(94, 146, 162, 128),
                obstacles=(255, 0, 0, 255)) -> np.ndarray:
    """render_image's per-pixel rule (renderer_helpers.rs:147-164) in numpy:
    wall -> obstacles colour; density != 0 on a fluid cell ->
    ((density * fluid.r) as u8, fluid.g, density as u8, 1) with Rust's
    saturating float-to-u8 casts; otherwise the world colour."""
    def as_u8(v):
        v = np.where(np.isnan(v), 0.0, v)
        return np.clip(np.trunc(v), 0, 255).astype(np.uint8)
    d = np.asarray(density, dtype=np.float32).reshape(size, size)
    w = np.asarray(cells).reshape(size, size) != 0
    out = np.empty((size, size, 4), dtype=np.uint8)
    out[:] = np.array(world, dtype=np.uint8)
    fl = (~w) & (d != 0.0)
    out[fl, 0] = as_u8(d[fl] * np.float32(fluid[0]))
    out[fl, 1] = fluid[1]
    out[fl, 2] = as_u8(d[fl])
    out[fl, 3] = 1
    out[w] = np.array(obstacles, dtype=np.uint8)
    return out


# ---- the differentiable problem (f64 tape adjoint) ---------------------------


def adjoint_problem_f64(cells, size, dt, iters, diff, visc, init, src, target, grads=True):
    """Loss 0.5*sum_interior(density - target)^2 after len(src) frames of
    (density/scratch += src[f]; step) from `init` (six arrays); returns
    (loss, signature, g_vx, g_vy, g_src) with the adjoints of the initial vx,
    vy and of every source field (None when grads=False)."""
    n = size * size
    init = [np.ascontiguousarray(a, dtype=np.float64).reshape(-1) for a in init]
    src = np.ascontiguousarray(src, dtype=np.float64).reshape(-1, n)
    target = np.ascontiguousarray(target, dtype=np.float64).reshape(-1)
    ptrs = (ctypes.c_void_p * 6)(*[_ptr(a) for a in init])
    sig = ctypes.c_uint64()
    if grads:
        gvx, gvy = np.zeros(n), np.zeros(n)
        gsrc = np.zeros_like(src)
        loss = lib().eqo_adjoint_problem_f64(_ptr(cells), size, dt, iters, diff, visc,
                                             src.shape[0], ptrs, _ptr(src), _ptr(target),
                                             _ptr(gvx), _ptr(gvy), _ptr(gsrc), ctypes.byref(sig))
        return loss, sig.value, gvx, gvy, gsrc
    loss = lib().eqo_adjoint_problem_f64(_ptr(cells), size, dt, iters, diff, visc,
                                         src.shape[0], ptrs, _ptr(src), _ptr(target), None, None,
                                         None, ctypes.byref(sig))
    return loss, sig.value, None, None, None


def adjoint_problem_f32(cells, size, dt, iters, diff, visc, init, src, target):
    """adjoint_problem_f64 with the f32 forward and f32 adjoint arithmetic:
    (loss, signature, g_vx, g_vy, g_src)."""
    n = size * size
    init = [np.ascontiguousarray(a, dtype=np.float32).reshape(-1) for a in init]
    src = np.ascontiguousarray(src, dtype=np.float32).reshape(-1, n)
    target = np.ascontiguousarray(target, dtype=np.float32).reshape(-1)
    ptrs = (ctypes.c_void_p * 6)(*[_ptr(a) for a in init])
    sig = ctypes.c_uint64()
    gvx, gvy = np.zeros(n, np.float32), np.zeros(n, np.float32)
    gsrc = np.zeros_like(src)
    loss = lib().eqo_adjoint_problem_f32(_ptr(cells), size, dt, iters, diff, visc, src.shape[0],
                                         ptrs, _ptr(src), _ptr(target), _ptr(gvx), _ptr(gvy),
                                         _ptr(gsrc), ctypes.byref(sig))
    return loss, sig.value, gvx, gvy, gsrc


def fd_direction_f64(cells, size, dt, iters, diff, visc, init, src, target, direction, hs,
                     frozen=False):
    """Losses of the f64 forward at +h and -h along `direction` for each h in
    hs: array (len(hs), 2). frozen: the perturbed runs replay the unperturbed
    run's advect choices (cells, clamps, row breaks), so the central
    difference is the derivative of the piece the adjoint differentiates."""
    n = size * size
    init = [np.ascontiguousarray(a, dtype=np.float64).reshape(-1) for a in init]
    src = np.ascontiguousarray(src, dtype=np.float64).reshape(-1)
    target = np.ascontiguousarray(target, dtype=np.float64).reshape(-1)
    direction = np.ascontiguousarray(direction, dtype=np.float64).reshape(-1)
    assert direction.size == 2 * n + src.size
    hs = np.ascontiguousarray(hs, dtype=np.float64)
    out = np.zeros(2 * hs.size)
    ptrs = (ctypes.c_void_p * 6)(*[_ptr(a) for a in init])
    lib().eqo_fd_direction_f64(_ptr(cells), size, dt, iters, diff, visc, src.size // n, ptrs,
                               _ptr(src), _ptr(target), _ptr(direction), _ptr(hs), hs.size,
                               int(bool(frozen)), _ptr(out))
    return out.reshape(-1, 2)


def set_boundaries_adj_f64(mode, xb, size, cells):
    x = np.ascontiguousarray(xb, dtype=np.float64).copy()
    lib().eqo_set_boundaries_adj_f64(mode, _ptr(x), size, _ptr(cells))
    return x


def lin_solve_adj_f64(mode, xb, x0b, a, c, size, iters, cells):
    x = np.ascontiguousarray(xb, dtype=np.float64).copy()
    x0 = np.ascontiguousarray(x0b, dtype=np.float64).copy()
    lib().eqo_lin_solve_adj_f64(mode, _ptr(x), _ptr(x0), a, c, size, iters, _ptr(cells))
    return x, x0


def advect_adj_f32(mode, db, d0b, ub, vb, d0, u, v, size, dt, cells):
    io = [np.ascontiguousarray(a, dtype=np.float32).copy() for a in (db, d0b, ub, vb)]
    ins = [np.ascontiguousarray(a, dtype=np.float32) for a in (d0, u, v)]
    lib().eqo_advect_adj_f32(mode, *[_ptr(a) for a in io], *[_ptr(a) for a in ins], size, dt,
                             _ptr(cells))
    return io


def project_adj_f64(vxb, vyb, pb, divb, size, iters, cells):
    io = [np.ascontiguousarray(a, dtype=np.float64).copy() for a in (vxb, vyb, pb, divb)]
    lib().eqo_project_adj_f64(*[_ptr(a) for a in io], size, iters, _ptr(cells))
    return io


def gaussian_target(size, nblobs=6, sigma=(8.0, 24.0), seed=0, amplitude=1.0):
    """A seeded target density: the sum of `nblobs` Gaussians with sigma
    uniform in `sigma` (cells), centres uniform over the interior."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:size, 0:size].astype(np.float64)
    t = np.zeros((size, size))
    for _ in range(nblobs):
        cx, cy = rng.uniform(1, size - 1, 2)
        sg = rng.uniform(*sigma)
        t += amplitude * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * sg * sg))
    return t.reshape(-1)
