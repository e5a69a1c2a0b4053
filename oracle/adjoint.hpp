// ORACLE -- test infrastructure only, never the product path.
//
// The adjoint (reverse-mode derivative) of the reference's frame step
// (src/simulation/fluid.rs:437-524), restated sequentially and templated on
// the float type (the f64 instantiation is the "f64 CPU tape adjoint" the GPU
// adjoint kernels are checked against; finite differences check this one).
//
// Every phase of step() is linear in the fields except advect's dependence on
// the velocity it backtraces with; the adjoint of a phase list is the list of
// transposed phases in reverse order, each at the forward state it was applied
// to (the "tape": the fields each advect read, recomputed from a checkpoint).
//   set_boundaries^T : a written cell's adjoint moves to the cell it copied
//                      (negated in the velocity modes), corners first;
//   Gauss-Seidel^T   : the sweep's cells in reverse lexicographic order, each
//                      handing cr * adj to x0 and a * cr * adj to its four
//                      neighbours, then zeroing its own;
//   advect^T         : the transposed bilinear scatter into d0 and the
//                      derivative of the interpolant w.r.t. the backtrace (zero
//                      where it was clamped) into u and v; the row break's copy
//                      and the untouched cells after it pass their adjoints on.
#pragma once
#include <cmath>
#include <cstring>
#include <vector>

#include "fluid_oracle.hpp"

namespace eqo {

template <class T>
inline void set_boundaries_adj(Mode m, T* xb, uint32_t usize, const uint8_t* cells) {
  const int64_t S = usize;
  auto wall = [&](int64_t i, int64_t j) { return cells[idx(i, j, S)] != 0; };
  // corners (computed last in the forward pass from the post-pass frame)
  {
    const T h = (T)0.5;
    struct C { int64_t ci, cj, ai, aj, bi, bj; };
    const C cs[4] = {{0, 0, 1, 0, 0, 1}, {0, S - 1, 1, S - 1, 0, S - 2},
                     {S - 1, 0, S - 2, 0, S - 1, 1}, {S - 1, S - 1, S - 2, S - 1, S - 1, S - 2}};
    for (int k = 3; k >= 0; --k) {
      const T g = xb[idx(cs[k].ci, cs[k].cj, S)];
      xb[idx(cs[k].ci, cs[k].cj, S)] = (T)0;
      xb[idx(cs[k].ai, cs[k].aj, S)] += h * g;
      xb[idx(cs[k].bi, cs[k].bj, S)] += h * g;
    }
  }
  // the per-cell pass is order-independent: reverse it cell by cell
  std::vector<uint8_t> rowfl(S, 0), colfl(S, 0);
  for (int64_t j = 1; j < S - 1; ++j)
    for (int64_t i = 1; i < S - 1; ++i)
      if (!wall(i, j)) rowfl[j] = colfl[i] = 1;
  if (m == Passive) {
    for (int64_t k = 1; k < S - 1; ++k) {
      if (colfl[k]) {
        xb[idx(k, 1, S)] += xb[idx(k, 0, S)];
        xb[idx(k, 0, S)] = (T)0;
        xb[idx(k, S - 2, S)] += xb[idx(k, S - 1, S)];
        xb[idx(k, S - 1, S)] = (T)0;
      }
      if (rowfl[k]) {
        xb[idx(1, k, S)] += xb[idx(0, k, S)];
        xb[idx(0, k, S)] = (T)0;
        xb[idx(S - 2, k, S)] += xb[idx(S - 1, k, S)];
        xb[idx(S - 1, k, S)] = (T)0;
      }
    }
    return;
  }
  for (int64_t j = 1; j < S - 1; ++j)
    for (int64_t i = 1; i < S - 1; ++i) {
      if (wall(i, j)) continue;
      int64_t si = -1, sj = -1;
      if (m == AdjustRow) {
        if (wall(i + 1, j)) { si = i + 1; sj = j; }
        else if (wall(i - 1, j)) { si = i - 1; sj = j; }
      } else {
        if (wall(i, j - 1)) { si = i; sj = j - 1; }
        else if (wall(i, j + 1)) { si = i; sj = j + 1; }
      }
      if (si < 0) continue;
      xb[idx(si, sj, S)] -= xb[idx(i, j, S)];
      xb[idx(i, j, S)] = (T)0;
    }
}

// lin_solve^T: xb (adjoint of x after the solve) -> adjoint of x before it;
// x0b accumulates.
template <class T>
inline void lin_solve_adj(Mode m, T* xb, T* x0b, T a, T c, uint32_t usize, int64_t frames,
                          const uint8_t* cells) {
  const int64_t S = usize;
  const T cr = (T)1.0 / c;
  for (int64_t k = 0; k < frames; ++k) {
    set_boundaries_adj<T>(m, xb, usize, cells);
    for (int64_t j = S - 2; j >= 1; --j)
      for (int64_t i = S - 2; i >= 1; --i) {
        const size_t q = idx(i, j, S);
        const T g = xb[q];
        xb[q] = (T)0;
        x0b[q] += cr * g;
        const T t = a * cr * g;
        xb[idx(i + 1, j, S)] += t;
        xb[idx(i - 1, j, S)] += t;
        xb[idx(i, j + 1, S)] += t;
        xb[idx(i, j - 1, S)] += t;
      }
  }
}

// advect^T at the forward state (d0, u, v as the forward read them).
template <class T>
inline void advect_adj(Mode m, T* db, T* d0b, T* ub, T* vb, const T* d0, const T* u,
                       const T* v, uint32_t size, T delta_t, const uint8_t* cells) {
  const int64_t S = size;
  set_boundaries_adj<T>(m, db, size, cells);
  const T dt0 = delta_t * (T)(S - 2);
  const T hi = (T)S - (T)1.0;
  for (int64_t j = 1; j < S - 1; ++j) {
    // replay the forward row to find its break and each cell's backtrace
    int64_t brk = S - 1;  // no break: every interior cell written
    for (int64_t i = 1; i < S - 1; ++i) {
      T x = (T)i - dt0 * u[idx(i, j, S)];
      T y = (T)j - dt0 * v[idx(i, j, S)];
      x = rust_clamp<T>(x, (T)0.5, hi);
      y = rust_clamp<T>(y, (T)0.5, hi);
      const T fi1 = std::floor(x) + (T)1.0, fj1 = std::floor(y) + (T)1.0;
      if (fi1 >= (T)S || fj1 >= (T)S) {  // the forward's test (fluid.rs:420)
        brk = i;
        break;
      }
    }
    if (brk < S - 1) {  // the break cell copied its left neighbour's new value
      const T g = db[idx(brk, j, S)];
      db[idx(brk, j, S)] = (T)0;
      db[idx(brk - 1, j, S)] += g;  // brk == 1: the old ghost d[0, j]
    }
    for (int64_t i = std::min<int64_t>(brk - 1, S - 2); i >= 1; --i) {
      const size_t q = idx(i, j, S);
      const T g = db[q];
      db[q] = (T)0;
      const T xr = (T)i - dt0 * u[q], yr = (T)j - dt0 * v[q];
      const T x = rust_clamp<T>(xr, (T)0.5, hi), y = rust_clamp<T>(yr, (T)0.5, hi);
      const T fi0 = std::floor(x), fj0 = std::floor(y);
      const uint32_t i0 = rust_as_u32<T>(fi0), i1 = rust_as_u32<T>(fi0 + (T)1.0);
      const uint32_t j0 = rust_as_u32<T>(fj0), j1 = rust_as_u32<T>(fj0 + (T)1.0);
      const T s1 = x - fi0, s0 = (T)1.0 - s1, t1 = y - fj0, t0 = (T)1.0 - t1;
      const T A = d0[idx(i0, j0, S)], B = d0[idx(i0, j1, S)];
      const T C = d0[idx(i1, j0, S)], D = d0[idx(i1, j1, S)];
      d0b[idx(i0, j0, S)] += s0 * t0 * g;
      d0b[idx(i0, j1, S)] += s0 * t1 * g;
      d0b[idx(i1, j0, S)] += s1 * t0 * g;
      d0b[idx(i1, j1, S)] += s1 * t1 * g;
      const bool cx = (xr < (T)0.5) || (xr > hi), cy = (yr < (T)0.5) || (yr > hi);
      if (!cx) ub[q] += -dt0 * g * ((t0 * C + t1 * D) - (t0 * A + t1 * B));
      if (!cy) vb[q] += -dt0 * g * (s0 * (B - A) + s1 * (D - C));
    }
  }
}

// project^T (fluid.rs:330-375) with p and div the aliased arrays.
template <class T>
inline void project_adj(T* vxb, T* vyb, T* pb, T* divb, uint32_t size, int64_t frames,
                        const uint8_t* cells) {
  const int64_t S = size;
  const T sf = (T)size;
  set_boundaries_adj<T>(AdjustColumn, vyb, size, cells);
  set_boundaries_adj<T>(AdjustRow, vxb, size, cells);
  for (int64_t j = S - 2; j >= 1; --j)
    for (int64_t i = S - 2; i >= 1; --i) {
      const T gx = vxb[idx(i, j, S)], gy = vyb[idx(i, j, S)];
      pb[idx(i + 1, j, S)] -= (T)0.5 * sf * gx;
      pb[idx(i - 1, j, S)] += (T)0.5 * sf * gx;
      pb[idx(i, j + 1, S)] -= (T)0.5 * sf * gy;
      pb[idx(i, j - 1, S)] += (T)0.5 * sf * gy;
    }
  lin_solve_adj<T>(Passive, pb, divb, (T)1.0, (T)4.0, size, frames, cells);
  set_boundaries_adj<T>(Passive, pb, size, cells);
  set_boundaries_adj<T>(Passive, divb, size, cells);
  for (int64_t j = S - 2; j >= 1; --j)
    for (int64_t i = S - 2; i >= 1; --i) {
      pb[idx(i, j, S)] = (T)0;  // p = 0 overwrote the interior
      const T g = divb[idx(i, j, S)];
      divb[idx(i, j, S)] = (T)0;
      const T w = (T)-0.5 * g / sf;
      vxb[idx(i + 1, j, S)] += w;
      vxb[idx(i - 1, j, S)] -= w;
      vyb[idx(i, j + 1, S)] += w;
      vyb[idx(i, j - 1, S)] -= w;
    }
}

// One frame's forward, keeping what its adjoint reads: the fields each advect
// read (d0, u, v) at that point of the frame.
template <class T>
struct FrameTape {
  std::vector<T> vx0, vy0, vx, vy, sc;  // after project #1 (vx0, vy0); after project #2 (vx, vy); sc after diffuse
};

template <class T>
inline void step_taped(T* sc, T* de, T* vx, T* vy, T* vx0, T* vy0, const uint8_t* cells,
                       uint32_t size, T dt, int64_t frames, T diff, T visc, FrameTape<T>& tp) {
  const size_t n = (size_t)size * size;
  diffuse<T>(AdjustRow, vx0, vx, visc, size, dt, frames, cells);
  diffuse<T>(AdjustColumn, vy0, vy, visc, size, dt, frames, cells);
  project<T>(vx0, vy0, vx, vy, size, frames, cells);
  tp.vx0.assign(vx0, vx0 + n);
  tp.vy0.assign(vy0, vy0 + n);
  advect<T>(AdjustRow, vx, vx0, vx0, vy0, size, dt, cells);
  advect<T>(AdjustColumn, vy, vy0, vx0, vy0, size, dt, cells);
  project<T>(vx, vy, vx0, vy0, size, frames, cells);
  tp.vx.assign(vx, vx + n);
  tp.vy.assign(vy, vy + n);
  diffuse<T>(Passive, sc, de, diff, size, dt, frames, cells);
  tp.sc.assign(sc, sc + n);
  advect<T>(Passive, de, sc, vx, vy, size, dt, cells);
  std::memcpy(sc, de, sizeof(T) * n);
}

// step^T: the adjoints of the six arrays after the step -> before it.
template <class T>
inline void step_adj(T* scb, T* deb, T* vxb, T* vyb, T* vx0b, T* vy0b, const uint8_t* cells,
                     uint32_t size, T dt, int64_t frames, T diff, T visc,
                     const FrameTape<T>& tp) {
  const int64_t S = size;
  const size_t n = (size_t)S * S;
  // scratch = density.clone()
  for (size_t q = 0; q < n; ++q) {
    deb[q] += scb[q];
    scb[q] = (T)0;
  }
  advect_adj<T>(Passive, deb, scb, vxb, vyb, tp.sc.data(), tp.vx.data(), tp.vy.data(), size, dt,
                cells);
  {  // diffuse(Passive, sc, de, diff)
    const T sf = (T)(S - 2);
    const T a = ((dt * diff) * sf) * sf;
    lin_solve_adj<T>(Passive, scb, deb, a, (T)1.0 + (T)4.0 * a, size, frames, cells);
  }
  project_adj<T>(vxb, vyb, vx0b, vy0b, size, frames, cells);
  advect_adj<T>(AdjustColumn, vyb, vy0b, vx0b, vy0b, tp.vy0.data(), tp.vx0.data(),
                tp.vy0.data(), size, dt, cells);
  advect_adj<T>(AdjustRow, vxb, vx0b, vx0b, vy0b, tp.vx0.data(), tp.vx0.data(), tp.vy0.data(),
                size, dt, cells);
  project_adj<T>(vx0b, vy0b, vxb, vyb, size, frames, cells);
  {
    const T sf = (T)(S - 2);
    const T a = ((dt * visc) * sf) * sf;
    lin_solve_adj<T>(AdjustColumn, vy0b, vyb, a, (T)1.0 + (T)4.0 * a, size, frames, cells);
    lin_solve_adj<T>(AdjustRow, vx0b, vxb, a, (T)1.0 + (T)4.0 * a, size, frames, cells);
  }
}

}  // namespace eqo

namespace eqo {

// The differentiable problem: from `init` (six arrays), each frame adds the
// frame's density-source field src[f] to density and scratch (add_density at
// every cell, fluid.rs:120-124) and steps; loss = 0.5 * sum over the interior
// of (density - target)^2. Returns the loss; with `grads` the adjoints of the
// initial vx, vy and of every source field; `sig` receives a hash of the
// forward's discrete choices (each advect's row breaks and clamped cells), for
// finite-difference checks that must not cross them.
template <class T>
inline T adjoint_problem(const uint8_t* cells, uint32_t size, T dt, int64_t K, T diff, T visc,
                         int64_t nframes, const T* const init[6], const T* src, const T* target,
                         T* g_vx, T* g_vy, T* g_src, uint64_t* sig) {
  const int64_t S = size;
  const size_t n = (size_t)S * S;
  std::vector<T> f[6];
  for (int q = 0; q < 6; ++q) f[q].assign(init[q], init[q] + n);
  std::vector<FrameTape<T>> tapes((size_t)nframes);
  for (int64_t fr = 0; fr < nframes; ++fr) {
    const T* s = src + (size_t)fr * n;
    for (size_t q = 0; q < n; ++q) {
      f[Density][q] += s[q];
      f[Scratch][q] += s[q];
    }
    step_taped<T>(f[Scratch].data(), f[Density].data(), f[VelX].data(), f[VelY].data(),
                  f[VelX0].data(), f[VelY0].data(), cells, size, dt, K, diff, visc, tapes[fr]);
  }
  T loss = 0;
  for (int64_t j = 1; j < S - 1; ++j)
    for (int64_t i = 1; i < S - 1; ++i) {
      const T e = f[Density][idx(i, j, S)] - target[idx(i, j, S)];
      loss += (T)0.5 * e * e;
    }
  if (sig) {
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](uint64_t v) { h = (h ^ v) * 1099511628211ull; };
    const T dt0 = dt * (T)(S - 2), hi = (T)S - (T)1.0;
    for (int64_t fr = 0; fr < nframes; ++fr) {
      const FrameTape<T>& tp = tapes[fr];
      const T* uv[2][2] = {{tp.vx0.data(), tp.vy0.data()}, {tp.vx.data(), tp.vy.data()}};
      for (int a = 0; a < 2; ++a)
        for (int64_t j = 1; j < S - 1; ++j) {
          int64_t brk = S - 1;
          for (int64_t i = 1; i < S - 1; ++i) {
            const T xr = (T)i - dt0 * uv[a][0][idx(i, j, S)], yr = (T)j - dt0 * uv[a][1][idx(i, j, S)];
            mix((uint64_t)((xr < (T)0.5) | ((xr > hi) << 1) | ((yr < (T)0.5) << 2) | ((yr > hi) << 3)));
            const T x = rust_clamp<T>(xr, (T)0.5, hi), y = rust_clamp<T>(yr, (T)0.5, hi);
            if (std::floor(x) + (T)1.0 >= (T)S || std::floor(y) + (T)1.0 >= (T)S) {
              brk = i;
              break;
            }
          }
          mix((uint64_t)brk);
        }
    }
    *sig = h;
  }
  if (!g_vx) return loss;
  std::vector<T> b[6];
  for (int q = 0; q < 6; ++q) b[q].assign(n, (T)0);
  for (int64_t j = 1; j < S - 1; ++j)
    for (int64_t i = 1; i < S - 1; ++i)
      b[Density][idx(i, j, S)] = f[Density][idx(i, j, S)] - target[idx(i, j, S)];
  for (int64_t fr = nframes - 1; fr >= 0; --fr) {
    step_adj<T>(b[Scratch].data(), b[Density].data(), b[VelX].data(), b[VelY].data(),
                b[VelX0].data(), b[VelY0].data(), cells, size, dt, K, diff, visc, tapes[fr]);
    T* gs = g_src + (size_t)fr * n;
    for (size_t q = 0; q < n; ++q) gs[q] = b[Density][q] + b[Scratch][q];
  }
  std::memcpy(g_vx, b[VelX].data(), n * sizeof(T));
  std::memcpy(g_vy, b[VelY].data(), n * sizeof(T));
  return loss;
}

}  // namespace eqo

namespace eqo {

// ---- frozen-path forward: finite differences on the adjoint's smooth piece --
// The forward is piecewise smooth: each advect's cell choice floor(x),
// its clamps and its row break are discrete. The adjoint differentiates the
// piece the recorded run is on; a central difference matches it only if the
// +h and -h runs stay on that piece. A frozen-path run replays the recorded
// choices (cell, clamp side, break column) with the perturbed values, which
// is that piece's polynomial extension: its central difference is what the
// adjoint must equal, to O(h^2), whatever h.
template <class T>
struct AdvectPath {
  std::vector<int64_t> brk;    // per row j: the break column (S - 1: none)
  std::vector<T> fi0, fj0;     // per cell: floor of the clamped backtrace
  std::vector<uint8_t> clamp;  // per cell: 1 x < 0.5, 2 x > S-1, 4 y < 0.5, 8 y > S-1
};

template <class T>
inline void advect_path(Mode m, T* d, const T* d0, const T* u, const T* v, uint32_t size,
                        T delta_t, const uint8_t* cells, AdvectPath<T>& P, bool record) {
  const int64_t S = size;
  const T dt0 = delta_t * (T)(size - 2);
  const T sf = (T)size, hi = sf - (T)1.0;
  if (record) {
    P.brk.assign(S, S - 1);
    P.fi0.assign((size_t)S * S, (T)0);
    P.fj0.assign((size_t)S * S, (T)0);
    P.clamp.assign((size_t)S * S, 0);
  }
  for (int64_t j = 1; j < S - 1; ++j) {
    for (int64_t i = 1; i < S - 1; ++i) {
      const size_t q = idx(i, j, S);
      const T xr = (T)i - dt0 * u[q], yr = (T)j - dt0 * v[q];
      T x, y, fi0, fj0;
      if (record) {
        P.clamp[q] = (uint8_t)((xr < (T)0.5) | ((xr > hi) << 1) | ((yr < (T)0.5) << 2) |
                               ((yr > hi) << 3));
        x = rust_clamp<T>(xr, (T)0.5, hi);
        y = rust_clamp<T>(yr, (T)0.5, hi);
        fi0 = std::floor(x);
        fj0 = std::floor(y);
        P.fi0[q] = fi0;
        P.fj0[q] = fj0;
        if (fi0 + (T)1.0 >= sf || fj0 + (T)1.0 >= sf) {
          P.brk[j] = i;
          d[q] = d[idx(i - 1, j, S)];
          break;
        }
      } else {
        if (i == P.brk[j]) {
          d[q] = d[idx(i - 1, j, S)];
          break;
        }
        const uint8_t c = P.clamp[q];
        x = (c & 1) ? (T)0.5 : (c & 2) ? hi : xr;
        y = (c & 4) ? (T)0.5 : (c & 8) ? hi : yr;
        fi0 = P.fi0[q];
        fj0 = P.fj0[q];
      }
      const T s1 = x - fi0, s0 = (T)1.0 - s1, t1 = y - fj0, t0 = (T)1.0 - t1;
      const int64_t i0 = rust_as_u32<T>(fi0), i1 = rust_as_u32<T>(fi0 + (T)1.0);
      const int64_t j0 = rust_as_u32<T>(fj0), j1 = rust_as_u32<T>(fj0 + (T)1.0);
      d[q] = s0 * (t0 * d0[idx(i0, j0, S)] + t1 * d0[idx(i0, j1, S)]) +
             s1 * (t0 * d0[idx(i1, j0, S)] + t1 * d0[idx(i1, j1, S)]);
    }
  }
  set_boundaries<T>(m, d, size, cells);
}

// adjoint_problem's forward with every advect recording (record = true) or
// replaying its discrete choices; returns the loss.
template <class T>
inline T forward_path(const uint8_t* cells, uint32_t size, T dt, int64_t K, T diff, T visc,
                      int64_t nframes, const T* const init[6], const T* src, const T* target,
                      std::vector<AdvectPath<T>>& paths, bool record) {
  const int64_t S = size;
  const size_t n = (size_t)S * S;
  std::vector<T> f[6];
  for (int q = 0; q < 6; ++q) f[q].assign(init[q], init[q] + n);
  if (record) paths.assign((size_t)nframes * 3, AdvectPath<T>());
  T* sc = f[Scratch].data();
  T* de = f[Density].data();
  T* vx = f[VelX].data();
  T* vy = f[VelY].data();
  T* vx0 = f[VelX0].data();
  T* vy0 = f[VelY0].data();
  for (int64_t fr = 0; fr < nframes; ++fr) {
    const T* s = src + (size_t)fr * n;
    for (size_t q = 0; q < n; ++q) {
      de[q] += s[q];
      sc[q] += s[q];
    }
    AdvectPath<T>* P = &paths[(size_t)fr * 3];
    diffuse<T>(AdjustRow, vx0, vx, visc, size, dt, K, cells);
    diffuse<T>(AdjustColumn, vy0, vy, visc, size, dt, K, cells);
    project<T>(vx0, vy0, vx, vy, size, K, cells);
    advect_path<T>(AdjustRow, vx, vx0, vx0, vy0, size, dt, cells, P[0], record);
    advect_path<T>(AdjustColumn, vy, vy0, vx0, vy0, size, dt, cells, P[1], record);
    project<T>(vx, vy, vx0, vy0, size, K, cells);
    diffuse<T>(Passive, sc, de, diff, size, dt, K, cells);
    advect_path<T>(Passive, de, sc, vx, vy, size, dt, cells, P[2], record);
    std::memcpy(sc, de, sizeof(T) * n);
  }
  T loss = 0;
  for (int64_t j = 1; j < S - 1; ++j)
    for (int64_t i = 1; i < S - 1; ++i) {
      const T e = de[idx(i, j, S)] - target[idx(i, j, S)];
      loss += (T)0.5 * e * e;
    }
  return loss;
}

}  // namespace eqo
