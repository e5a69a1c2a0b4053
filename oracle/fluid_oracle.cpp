// ORACLE -- test infrastructure only (see fluid_oracle.hpp for the status of
// its parity pin). A C ABI over the templated restatement so that Python tests
// and the CPU-baseline leg of bench.py can drive it through ctypes.
//
// Field order everywhere: scratch, density, vx, vy, vx0, vy0 (fluid.rs:59-77).
// Mask: one byte per cell, 1 = DefaultWall, 0 = NoWall (fluid.rs:12-17).
#include "fluid_oracle.hpp"
#include "adjoint.hpp"

#include <chrono>

using namespace eqo;

namespace {

template <class T, class S>
void run_frames(T* const f[6], const uint8_t* cells, uint32_t size, T dt,
                int64_t iters, T diff, T visc, int64_t nframes, int64_t nsrc,
                const uint32_t* sx, const uint32_t* sy, const S* sd, const S* su,
                const S* sv) {
  // One frame = the sources of that frame (add_density, then add_velocity,
  // source by source, fluid.rs:120-131) followed by step() (fluid.rs:437).
  const size_t n = (size_t)size * size;
  (void)n;
  for (int64_t fr = 0; fr < nframes; ++fr) {
    for (int64_t s = 0; s < nsrc; ++s) {
      const int64_t q = fr * nsrc + s;
      const size_t k = idx(sx[q], sy[q], size);
      f[Density][k] += (T)sd[q];
      f[Scratch][k] += (T)sd[q];
      f[VelX][k] += (T)su[q];
      f[VelY][k] += (T)sv[q];
    }
    step_arrays<T>(f[Scratch], f[Density], f[VelX], f[VelY], f[VelX0], f[VelY0], cells,
                   size, dt, iters, diff, visc);
  }
}

template <class T>
void fluid_init_arrays(uint32_t size, T* const f[6], uint8_t* cells) {
  State<T> s;
  fluid_new<T>(s, size, (T)0, 0, (T)0, (T)0);
  for (int q = 0; q < 6; ++q) std::memcpy(f[q], s.f[q].data(), sizeof(T) * s.f[q].size());
  std::memcpy(cells, s.cells.data(), s.cells.size());
}

template <class T>
void fluid_reinit(uint32_t size, T* const f[6], uint8_t* cells) {
  // init() applied on top of existing arrays (Fluid::default calls it twice,
  // fluid.rs:83-89).
  State<T> s;
  s.size = size;
  for (int q = 0; q < 6; ++q) s.f[q].assign(f[q], f[q] + (size_t)size * size);
  s.cells.assign(cells, cells + (size_t)size * size);
  init<T>(s);
  for (int q = 0; q < 6; ++q) std::memcpy(f[q], s.f[q].data(), sizeof(T) * s.f[q].size());
  std::memcpy(cells, s.cells.data(), s.cells.size());
}

}  // namespace

extern "C" {

int eqo_abi_version(void) { return 1; }

// ---- f32 (bit-exact restatement of the reference) -------------------------
void eqo_set_boundaries_f32(int mode, float* x, uint32_t size, const uint8_t* cells) {
  set_boundaries<float>((Mode)mode, x, size, cells);
}
void eqo_lin_solve_f32(int mode, float* x, const float* x0, float a, float c,
                       uint32_t size, int64_t iters, const uint8_t* cells) {
  lin_solve<float>((Mode)mode, x, x0, a, c, size, iters, cells);
}
void eqo_diffuse_f32(int mode, float* x, const float* x0, float diff, uint32_t size,
                     float dt, int64_t iters, const uint8_t* cells) {
  diffuse<float>((Mode)mode, x, x0, diff, size, dt, iters, cells);
}
void eqo_project_f32(float* vx, float* vy, float* p, float* div, uint32_t size,
                     int64_t iters, const uint8_t* cells) {
  project<float>(vx, vy, p, div, size, iters, cells);
}
void eqo_advect_f32(int mode, float* d, const float* d0, const float* u, const float* v,
                    uint32_t size, float dt, const uint8_t* cells) {
  advect<float>((Mode)mode, d, d0, u, v, size, dt, cells);
}
void eqo_step_f32(float* const f[6], const uint8_t* cells, uint32_t size, float dt,
                  int64_t iters, float diff, float visc) {
  step_arrays<float>(f[0], f[1], f[2], f[3], f[4], f[5], cells, size, dt, iters, diff, visc);
}
void eqo_run_f32(float* const f[6], const uint8_t* cells, uint32_t size, float dt,
                 int64_t iters, float diff, float visc, int64_t nframes, int64_t nsrc,
                 const uint32_t* sx, const uint32_t* sy, const float* sd, const float* su,
                 const float* sv) {
  run_frames<float, float>(f, cells, size, dt, iters, diff, visc, nframes, nsrc, sx, sy, sd,
                           su, sv);
}
void eqo_new_f32(uint32_t size, float* const f[6], uint8_t* cells) {
  fluid_init_arrays<float>(size, f, cells);
}
void eqo_reinit_f32(uint32_t size, float* const f[6], uint8_t* cells) {
  fluid_reinit<float>(size, f, cells);
}

// ---- f64 ("the reference step built with f64") ---------------------------
void eqo_lin_solve_f64(int mode, double* x, const double* x0, double a, double c,
                       uint32_t size, int64_t iters, const uint8_t* cells) {
  lin_solve<double>((Mode)mode, x, x0, a, c, size, iters, cells);
}
void eqo_step_f64(double* const f[6], const uint8_t* cells, uint32_t size, double dt,
                  int64_t iters, double diff, double visc) {
  step_arrays<double>(f[0], f[1], f[2], f[3], f[4], f[5], cells, size, dt, iters, diff, visc);
}
void eqo_run_f64(double* const f[6], const uint8_t* cells, uint32_t size, double dt,
                 int64_t iters, double diff, double visc, int64_t nframes, int64_t nsrc,
                 const uint32_t* sx, const uint32_t* sy, const float* sd, const float* su,
                 const float* sv) {
  run_frames<double, float>(f, cells, size, dt, iters, diff, visc, nframes, nsrc, sx, sy, sd,
                            su, sv);
}
void eqo_new_f64(uint32_t size, double* const f[6], uint8_t* cells) {
  fluid_init_arrays<double>(size, f, cells);
}
// The phases of the f64 step, for a step composed with another pressure solve.
void eqo_set_boundaries_f64(int mode, double* x, uint32_t size, const uint8_t* cells) {
  set_boundaries<double>((Mode)mode, x, size, cells);
}
void eqo_diffuse_f64(int mode, double* x, const double* x0, double diff, uint32_t size,
                     double dt, int64_t iters, const uint8_t* cells) {
  diffuse<double>((Mode)mode, x, x0, diff, size, dt, iters, cells);
}
void eqo_advect_f64(int mode, double* d, const double* d0, const double* u, const double* v,
                    uint32_t size, double dt, const uint8_t* cells) {
  advect<double>((Mode)mode, d, d0, u, v, size, dt, cells);
}
void eqo_project_div_f64(double* vx, double* vy, double* p, double* div, uint32_t size,
                         const uint8_t* cells) {
  project_divergence<double>(vx, vy, p, div, size, cells);
}
void eqo_project_grad_f64(double* vx, double* vy, const double* p, uint32_t size,
                          const uint8_t* cells) {
  project_gradient<double>(vx, vy, p, size, cells);
}

// ---- adjoint (the f64 tape adjoint the GPU adjoint is checked against) ----
double eqo_adjoint_problem_f64(const uint8_t* cells, uint32_t size, double dt, int64_t iters,
                               double diff, double visc, int64_t nframes,
                               const double* const init[6], const double* src,
                               const double* target, double* g_vx, double* g_vy, double* g_src,
                               uint64_t* sig) {
  return adjoint_problem<double>(cells, size, dt, iters, diff, visc, nframes, init, src, target,
                                 g_vx, g_vy, g_src, sig);
}
void eqo_lin_solve_adj_f64(int mode, double* xb, double* x0b, double a, double c,
                           uint32_t size, int64_t iters, const uint8_t* cells) {
  lin_solve_adj<double>((Mode)mode, xb, x0b, a, c, size, iters, cells);
}
void eqo_set_boundaries_adj_f64(int mode, double* xb, uint32_t size, const uint8_t* cells) {
  set_boundaries_adj<double>((Mode)mode, xb, size, cells);
}
// advect^T in f32: the same discrete choices (row breaks, clamps) as the f32
// forward that recorded d0, u, v.
void eqo_advect_adj_f32(int mode, float* db, float* d0b, float* ub, float* vb, const float* d0,
                        const float* u, const float* v, uint32_t size, float dt,
                        const uint8_t* cells) {
  advect_adj<float>((Mode)mode, db, d0b, ub, vb, d0, u, v, size, dt, cells);
}
void eqo_project_adj_f64(double* vxb, double* vyb, double* pb, double* divb, uint32_t size,
                         int64_t iters, const uint8_t* cells) {
  project_adj<double>(vxb, vyb, pb, divb, size, iters, cells);
}
// The same problem with the f32 forward (the tape the GPU adjoint records).
float eqo_adjoint_problem_f32(const uint8_t* cells, uint32_t size, float dt, int64_t iters,
                              float diff, float visc, int64_t nframes,
                              const float* const init[6], const float* src, const float* target,
                              float* g_vx, float* g_vy, float* g_src, uint64_t* sig) {
  return adjoint_problem<float>(cells, size, dt, iters, diff, visc, nframes, init, src, target,
                                g_vx, g_vy, g_src, sig);
}

// Central differences along one direction (over the initial vx, vy and every
// source field: 2n + nframes*n values) for each of nh step sizes: out[2k] the
// loss at +h[k], out[2k+1] at -h[k]. frozen != 0: the perturbed runs replay
// the unperturbed run's discrete choices (returns its loss); else plain runs
// (returns 0).
double eqo_fd_direction_f64(const uint8_t* cells, uint32_t size, double dt, int64_t iters,
                            double diff, double visc, int64_t nframes,
                            const double* const init[6], const double* src, const double* target,
                            const double* dir, const double* h, int64_t nh, int frozen,
                            double* out) {
  const size_t n = (size_t)size * size, ns = (size_t)nframes * n;
  std::vector<AdvectPath<double>> paths;
  double base = 0.0;
  if (frozen)
    base = forward_path<double>(cells, size, dt, iters, diff, visc, nframes, init, src, target,
                                paths, true);
  std::vector<double> f[6], s(ns);
  for (int64_t k = 0; k < 2 * nh; ++k) {
    const double e = (k & 1) ? -h[k / 2] : h[k / 2];
    for (int q = 0; q < 6; ++q) f[q].assign(init[q], init[q] + n);
    for (size_t c = 0; c < n; ++c) {
      f[VelX][c] += e * dir[c];
      f[VelY][c] += e * dir[n + c];
    }
    for (size_t c = 0; c < ns; ++c) s[c] = src[c] + e * dir[2 * n + c];
    const double* p[6] = {f[0].data(), f[1].data(), f[2].data(), f[3].data(), f[4].data(),
                          f[5].data()};
    out[k] = frozen ? forward_path<double>(cells, size, dt, iters, diff, visc, nframes, p,
                                           s.data(), target, paths, false)
                    : adjoint_problem<double>(cells, size, dt, iters, diff, visc, nframes, p,
                                              s.data(), target, nullptr, nullptr, nullptr,
                                              nullptr);
  }
  return base;
}

// ---- mask / obstacles -----------------------------------------------------
void eqo_fill_obstacle(uint8_t* cells, uint32_t size, int64_t x0, int64_t y0, int64_t x1,
                       int64_t y1) {
  fill_obstacle(cells, size, x0, y0, x1, y1);
}
int eqo_rectangle_valid(int64_t dlx, int64_t dly, int64_t urx, int64_t ury, int64_t size) {
  return rectangle_valid(dlx, dly, urx, ury, size) ? 1 : 0;
}

// Wall-clock of eqo_run_f32 in seconds, measured inside the library so the
// CPU baseline excludes Python overhead.
double eqo_time_run_f32(float* const f[6], const uint8_t* cells, uint32_t size, float dt,
                        int64_t iters, float diff, float visc, int64_t nframes, int64_t nsrc,
                        const uint32_t* sx, const uint32_t* sy, const float* sd,
                        const float* su, const float* sv) {
  const auto t0 = std::chrono::steady_clock::now();
  run_frames<float, float>(f, cells, size, dt, iters, diff, visc, nframes, nsrc, sx, sy, sd,
                           su, sv);
  const auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count();
}

}  // extern "C"
