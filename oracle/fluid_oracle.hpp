// ORACLE -- test infrastructure only. Not part of the product path.
//
// A CPU restatement of Equilibrium's stable-fluids frame step, written from
// the reference's src/simulation/fluid.rs (vkabadzhova/equilibrium), templated
// on the arithmetic type T (float reproduces the reference's f32 step; double
// is "the reference step built with f64").
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
// load this code, and only as the checker / the timed CPU baseline.
//
// Parity status: the reference ships no numeric golden vectors for step()
// (its tests pin only the index layout, Rectangle validation and the wall-mask
// count), and the Rust reference cannot be built in this environment, so the
// NUMERIC parity of this restatement is UNPINNED by the reference itself. It is
// cross-checked against a second, independent pure-Python restatement
// (tests/golden/pyref.py) and against hand-computed known answers.
//
// Floating point: every operation is written in the reference's evaluation
// order; build with -ffp-contract=off -fno-fast-math so that no multiply-add is
// contracted (Rust never contracts), which makes the f32 results bit-identical
// to the reference's.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace eqo {

// Orientation (fluid.rs:21-29).
enum Mode : int { AdjustRow = 0, AdjustColumn = 1, Passive = 2 };

// ContainerWall as an integer mask (fluid.rs:10-17): 1 = DefaultWall, 0 = NoWall.
static const uint8_t kWall = 1;

// idx! (fluid.rs:31-35): clamp both coordinates into [0, size-1], x fastest.
inline size_t idx(int64_t x, int64_t y, int64_t size) {
  int64_t cx = x < 0 ? 0 : (x > size - 1 ? size - 1 : x);
  int64_t cy = y < 0 ? 0 : (y > size - 1 ? size - 1 : y);
  return (size_t)(cx + cy * size);
}

// Rust's f32::clamp / f64::clamp: `if x < min {x = min}; if x > max {x = max}`;
// NaN passes through unchanged.
template <class T>
inline T rust_clamp(T x, T lo, T hi) {
  if (x < lo) x = lo;
  if (x > hi) x = hi;
  return x;
}

// Rust's saturating `as u32` for floats: NaN -> 0, negatives -> 0, truncation
// toward zero, values >= 2^32 -> u32::MAX.
template <class T>
inline uint32_t rust_as_u32(T v) {
  if (!(v == v)) return 0u;
  if (v <= (T)0) return 0u;
  if (v >= (T)4294967295.0) return 4294967295u;
  return (uint32_t)v;
}

// manage_single_cell_boundary (fluid.rs:133-189).
template <class T>
inline void manage_single_cell_boundary(Mode m, T* x, int64_t size,
                                        const uint8_t* cells, int64_t i,
                                        int64_t j) {
  if (cells[idx(i, j, size)] == kWall) return;
  const int64_t up_j = rust_clamp<int64_t>(j - 1, 0, size - 1);
  const int64_t down_j = rust_clamp<int64_t>(j + 1, 0, size - 1);
  const int64_t left_i = rust_clamp<int64_t>(i - 1, 0, size - 1);
  const int64_t right_i = rust_clamp<int64_t>(i + 1, 0, size - 1);
  switch (m) {
    case AdjustRow:
      if (cells[idx(left_i, j, size)] == kWall) x[idx(i, j, size)] = -x[idx(left_i, j, size)];
      if (cells[idx(right_i, j, size)] == kWall) x[idx(i, j, size)] = -x[idx(right_i, j, size)];
      break;
    case AdjustColumn:
      if (cells[idx(i, down_j, size)] == kWall) x[idx(i, j, size)] = -x[idx(i, down_j, size)];
      if (cells[idx(i, up_j, size)] == kWall) x[idx(i, j, size)] = -x[idx(i, up_j, size)];
      break;
    case Passive:
      x[idx(i, 0, size)] = x[idx(i, 1, size)];
      x[idx(i, size - 1, size)] = x[idx(i, size - 2, size)];
      x[idx(0, j, size)] = x[idx(1, j, size)];
      x[idx(size - 1, j, size)] = x[idx(size - 2, j, size)];
      break;
  }
}

// set_boundaries (fluid.rs:252-272): every cell in j-outer / i-inner order,
// then the four corners as the mean of their two frame neighbours.
template <class T>
inline void set_boundaries(Mode m, T* x, uint32_t usize, const uint8_t* cells) {
  const int64_t size = (int64_t)usize;
  for (int64_t j = 0; j <= size - 1; ++j)
    for (int64_t i = 0; i <= size - 1; ++i)
      manage_single_cell_boundary<T>(m, x, size, cells, i, j);
  const T h = (T)0.5;
  x[idx(0, 0, size)] = h * (x[idx(1, 0, size)] + x[idx(0, 1, size)]);
  x[idx(0, size - 1, size)] = h * (x[idx(1, size - 1, size)] + x[idx(0, size - 2, size)]);
  x[idx(size - 1, 0, size)] = h * (x[idx(size - 2, 0, size)] + x[idx(size - 1, 1, size)]);
  x[idx(size - 1, size - 1, size)] =
      h * (x[idx(size - 2, size - 1, size)] + x[idx(size - 1, size - 2, size)]);
}

// lin_solve (fluid.rs:301-325): `frames` lexicographic Gauss-Seidel sweeps,
// each followed by set_boundaries(orientation).
template <class T>
inline void lin_solve(Mode m, T* x, const T* x0, T a, T c, uint32_t size,
                      int64_t frames, const uint8_t* cells) {
  const T c_recip = (T)1.0 / c;
  const int64_t S = size;
  for (int64_t k = 0; k < frames; ++k) {
    for (int64_t j = 1; j < S - 1; ++j) {
      for (int64_t i = 1; i < S - 1; ++i) {
        const T sum = ((x[idx(i + 1, j, S)] + x[idx(i - 1, j, S)]) + x[idx(i, j + 1, S)]) +
                      x[idx(i, j - 1, S)];
        x[idx(i, j, S)] = (x0[idx(i, j, S)] + a * sum) * c_recip;
      }
    }
    set_boundaries<T>(m, x, size, cells);
  }
}

// diffuse (fluid.rs:276-298): a = dt * diff * (size-2)^2, c = 1 + 4a.
template <class T>
inline void diffuse(Mode m, T* x, const T* x0, T diffusion, uint32_t size,
                    T delta_t, int64_t frames, const uint8_t* cells) {
  const T size_float = (T)(size - 2);
  const T a = ((delta_t * diffusion) * size_float) * size_float;
  lin_solve<T>(m, x, x0, a, (T)1.0 + (T)4.0 * a, size, frames, cells);
}

// project (fluid.rs:330-375). Note the divergence and gradient scale by
// `size` (ghost frame included), not by size-2. Split in its divergence part
// (fluid.rs:339-352), the pressure solve and its gradient part (fluid.rs:
// 364-374) so that a step can be composed with another pressure solve.
template <class T>
inline void project_divergence(T* vx, T* vy, T* p, T* div, uint32_t size,
                               const uint8_t* cells) {
  const int64_t S = size;
  const T sf = (T)size;
  for (int64_t j = 1; j < S - 1; ++j) {
    for (int64_t i = 1; i < S - 1; ++i) {
      const T inner = ((vx[idx(i + 1, j, S)] - vx[idx(i - 1, j, S)]) + vy[idx(i, j + 1, S)]) -
                      vy[idx(i, j - 1, S)];
      div[idx(i, j, S)] = ((T)-0.5 * inner) / sf;
      p[idx(i, j, S)] = (T)0.0;
    }
  }
  set_boundaries<T>(Passive, div, size, cells);
  set_boundaries<T>(Passive, p, size, cells);
}

template <class T>
inline void project_gradient(T* vx, T* vy, const T* p, uint32_t size, const uint8_t* cells) {
  const int64_t S = size;
  const T sf = (T)size;
  for (int64_t j = 1; j < S - 1; ++j) {
    for (int64_t i = 1; i < S - 1; ++i) {
      vx[idx(i, j, S)] = vx[idx(i, j, S)] -
                         ((T)0.5 * (p[idx(i + 1, j, S)] - p[idx(i - 1, j, S)])) * sf;
      vy[idx(i, j, S)] = vy[idx(i, j, S)] -
                         ((T)0.5 * (p[idx(i, j + 1, S)] - p[idx(i, j - 1, S)])) * sf;
    }
  }
  set_boundaries<T>(AdjustRow, vx, size, cells);
  set_boundaries<T>(AdjustColumn, vy, size, cells);
}

template <class T>
inline void project(T* vx, T* vy, T* p, T* div, uint32_t size, int64_t frames,
                    const uint8_t* cells) {
  const int64_t S = size;
  const T sf = (T)size;
  project_divergence<T>(vx, vy, p, div, size, cells);
  lin_solve<T>(Passive, p, div, (T)1.0, (T)4.0, size, frames, cells);
  for (int64_t j = 1; j < S - 1; ++j) {
    for (int64_t i = 1; i < S - 1; ++i) {
      vx[idx(i, j, S)] = vx[idx(i, j, S)] -
                         ((T)0.5 * (p[idx(i + 1, j, S)] - p[idx(i - 1, j, S)])) * sf;
      vy[idx(i, j, S)] = vy[idx(i, j, S)] -
                         ((T)0.5 * (p[idx(i, j + 1, S)] - p[idx(i, j - 1, S)])) * sf;
    }
  }
  set_boundaries<T>(AdjustRow, vx, size, cells);
  set_boundaries<T>(AdjustColumn, vy, size, cells);
}

// advect (fluid.rs:378-432), including the row break: when the clamped
// backtrace reaches size-1 the cell copies its (already updated) left
// neighbour and the remainder of that row keeps its old values.
template <class T>
inline void advect(Mode m, T* d, const T* d0, const T* u, const T* v,
                   uint32_t size, T delta_t, const uint8_t* cells) {
  const int64_t S = size;
  const T dtx = delta_t * (T)(size - 2);
  const T dty = dtx;
  const T sf = (T)size;
  for (int64_t j = 1; j < S - 1; ++j) {
    for (int64_t i = 1; i < S - 1; ++i) {
      T x = (T)i - dtx * u[idx(i, j, S)];
      T y = (T)j - dty * v[idx(i, j, S)];
      x = rust_clamp<T>(x, (T)0.5, sf - (T)1.0);
      y = rust_clamp<T>(y, (T)0.5, sf - (T)1.0);
      const T i0 = std::floor(x);
      const T i1 = i0 + (T)1.0;
      const T j0 = std::floor(y);
      const T j1 = j0 + (T)1.0;
      const T s1 = x - i0;
      const T s0 = (T)1.0 - s1;
      const T t1 = y - j0;
      const T t0 = (T)1.0 - t1;
      const int64_t i0i = rust_as_u32<T>(i0), i1i = rust_as_u32<T>(i1);
      const int64_t j0i = rust_as_u32<T>(j0), j1i = rust_as_u32<T>(j1);
      if (i1 >= sf || j1 >= sf) {
        d[idx(i, j, S)] = d[idx(i - 1, j, S)];
        break;
      }
      d[idx(i, j, S)] = s0 * (t0 * d0[idx(i0i, j0i, S)] + t1 * d0[idx(i0i, j1i, S)]) +
                        s1 * (t0 * d0[idx(i1i, j0i, S)] + t1 * d0[idx(i1i, j1i, S)]);
    }
  }
  set_boundaries<T>(m, d, size, cells);
}

// The six state arrays of Fluid (fluid.rs:52-81), in this fixed order.
enum Field : int { Scratch = 0, Density = 1, VelX = 2, VelY = 3, VelX0 = 4, VelY0 = 5 };

template <class T>
struct State {
  uint32_t size = 0;
  T delta_t = 0, diffusion = 0, viscousity = 0;
  int64_t frames = 0;
  std::vector<T> f[6];
  std::vector<uint8_t> cells;
};

// add_density / add_velocity (fluid.rs:120-131).
template <class T>
inline void add_density(State<T>& s, uint32_t x, uint32_t y, T amount) {
  const size_t k = idx(x, y, s.size);
  s.f[Density][k] += amount;
  s.f[Scratch][k] += amount;
}
template <class T>
inline void add_velocity(State<T>& s, uint32_t x, uint32_t y, T ax, T ay) {
  const size_t k = idx(x, y, s.size);
  s.f[VelX][k] += ax;
  s.f[VelY][k] += ay;
}

// init (fluid.rs:602-606) = init_velocities (542-548), init_density (527-539),
// init_walls (552-570).
template <class T>
inline void init(State<T>& s) {
  const uint32_t S = s.size;
  for (uint32_t j = 0; j < S; ++j)
    for (uint32_t i = 0; i < S; ++i) add_velocity<T>(s, i, j, (T)1.0, (T)1.0);
  for (uint32_t j = 0; j < S; ++j)
    for (uint32_t i = 0; i < S; ++i) add_density<T>(s, i, j, (T)0.0);
  for (uint32_t j = S / 2 - 10; j <= S / 2 + 10; ++j)
    for (uint32_t i = S / 2 - 10; i <= S / 2 + 10; ++i) add_density<T>(s, i, j, (T)0.9);
  for (uint32_t i = 0; i < S; ++i) {
    s.cells[idx(i, 0, S)] = kWall;
    s.cells[idx(i, S - 1, S)] = kWall;
  }
  for (uint32_t j = 0; j < S; ++j) {
    s.cells[idx(0, j, S)] = kWall;
    s.cells[idx(S - 1, j, S)] = kWall;
  }
}

// Fluid::new (fluid.rs:93-110): zeroed arrays, all cells NoWall, then init().
template <class T>
inline void fluid_new(State<T>& s, uint32_t size, T delta_t, int64_t frames,
                      T diffusion, T viscousity) {
  s.size = size;
  s.delta_t = delta_t;
  s.frames = frames;
  s.diffusion = diffusion;
  s.viscousity = viscousity;
  for (auto& a : s.f) a.assign((size_t)size * size, (T)0);
  s.cells.assign((size_t)size * size, 0);
  init<T>(s);
}

// fill_obstacle (fluid.rs:610-619): half-open [x0,x1) x [y0,y1), clamped idx.
inline void fill_obstacle(uint8_t* cells, uint32_t size, int64_t x0, int64_t y0,
                          int64_t x1, int64_t y1) {
  for (int64_t x = x0; x < x1; ++x)
    for (int64_t y = y0; y < y1; ++y) cells[idx(x, y, size)] = kWall;
}

// Rectangle::are_all_points_valid (obstacle.rs:74-87).
inline bool rectangle_valid(int64_t dlx, int64_t dly, int64_t urx, int64_t ury,
                            int64_t size) {
  return dlx != urx && dly != ury && dlx < urx && dly < ury && dlx < size &&
         dly < size && urx < size && ury < size;
}

// step (fluid.rs:437-524) with the reference's array aliasing.
template <class T>
inline void step_arrays(T* scratch, T* density, T* vx, T* vy, T* vx0, T* vy0,
                        const uint8_t* cells, uint32_t size, T dt, int64_t frames,
                        T diffusion, T viscousity) {
  diffuse<T>(AdjustRow, vx0, vx, viscousity, size, dt, frames, cells);
  diffuse<T>(AdjustColumn, vy0, vy, viscousity, size, dt, frames, cells);
  project<T>(vx0, vy0, vx, vy, size, frames, cells);
  advect<T>(AdjustRow, vx, vx0, vx0, vy0, size, dt, cells);
  advect<T>(AdjustColumn, vy, vy0, vx0, vy0, size, dt, cells);
  project<T>(vx, vy, vx0, vy0, size, frames, cells);
  diffuse<T>(Passive, scratch, density, diffusion, size, dt, frames, cells);
  advect<T>(Passive, density, scratch, vx, vy, size, dt, cells);
  std::memcpy(scratch, density, sizeof(T) * (size_t)size * size);
}

template <class T>
inline void step(State<T>& s) {
  step_arrays<T>(s.f[Scratch].data(), s.f[Density].data(), s.f[VelX].data(),
                 s.f[VelY].data(), s.f[VelX0].data(), s.f[VelY0].data(), s.cells.data(),
                 s.size, s.delta_t, s.frames, s.diffusion, s.viscousity);
}

}  // namespace eqo
