// Mixed-precision iterative refinement for project's pressure equation
// (fluid.rs:353-362 solves it with a fixed 20 Gauss-Seidel sweeps; the
// precision form solves it to a relative residual instead).
//
// The equation is lin_solve(Passive, p, div, 1, 4) at its fixed point:
//   4 p(i,j) - (p(i-1,j) + p(i+1,j) + p(i,j-1) + p(i,j+1)) = div(i,j)
// on the N x N interior, with set_boundaries(Passive)'s ghost rule: a frame
// neighbour equals the adjacent interior cell where its row / column holds a
// fluid cell (Neumann), else it keeps its stored value (Dirichlet). Obstacles
// do not enter it (the Passive pass ignores them, fluid.rs:252-272).
//
// Refinement: p (FP32) starts at 0; each round computes the FP32 residual
// r = div - A p with FP64 sums (mean and norm), stops when the mean-free norm
// is below rtol times the first one (the mean is in the null space of the
// pure-Neumann operator, so no solver can remove it), else scales r to unit
// RMS, stores it in the low-precision format and runs one multigrid V-cycle
// for the correction e (low-precision storage, FP32 arithmetic), p += s e.
//
// Multigrid: cell-centred, coarsening by 2, red-black Gauss-Seidel smoothing
// with the Neumann rule solved locally (e = (r + sum of inside neighbours) /
// (number of inside neighbours)), bilinear prolongation with reflection at the
// walls, the coarsest level solved by one block in shared memory. The
// right-hand sides of every level are STORED in the low-precision format; a
// coarse cell holds the AVERAGE of its 2 x 2 children's residuals (the sum,
// which the coarse 5-point stencil needs, divided by 4 per level so that the
// stored values stay O(1) in FP16's range), and level l multiplies its stored
// right-hand side by 4^l when it uses it. The corrections e stay FP32: a
// Poisson correction's smooth part exceeds its rough part by up to N^2 / pi^2
// (about 2^19 at N = 2048), more than an FP16 or BF16 significand holds, so a
// low-precision e would round the rough part away.
#pragma once
#include "half.cuh"

namespace eqk {

// One red-black colour of Gauss-Seidel on A e = rs * s4 (level of n x n
// cells, rs stored, s4 = 4^level).
template <class T>
__device__ __forceinline__ void mg_smooth_cell(float* e, const T* r, int n, int pitch, int color,
                                               float s4, int I2, int J) {
  const int I = 2 * I2 + ((J + color) & 1);
  if (I >= n || J >= n) return;
  const size_t q = (size_t)J * pitch + I;
  float sum = 0.0f;
  int nin = 0;
  if (I > 0) { sum += e[q - 1]; ++nin; }
  if (I < n - 1) { sum += e[q + 1]; ++nin; }
  if (J > 0) { sum += e[q - pitch]; ++nin; }
  if (J < n - 1) { sum += e[q + pitch]; ++nin; }
  e[q] = (hl(r, q) * s4 + sum) / (float)nin;
}
template <class T>
__global__ void k_mg_smooth(float* __restrict__ e, const T* __restrict__ r, int n, int pitch,
                            int color, float s4) {
  mg_smooth_cell(e, r, n, pitch, color, s4, (int)(blockIdx.x * blockDim.x + threadIdx.x),
                 (int)(blockIdx.y * blockDim.y + threadIdx.y));
}

// (r * s4 - A e) at one cell.
template <class T>
__device__ __forceinline__ float mg_resid(const float* e, const T* r, int I, int J, int n,
                                          int pitch, float s4) {
  const size_t q = (size_t)J * pitch + I;
  const float c = e[q];
  float sum = 0.0f;
  int nin = 0;
  if (I > 0) { sum += e[q - 1]; ++nin; }
  if (I < n - 1) { sum += e[q + 1]; ++nin; }
  if (J > 0) { sum += e[q - pitch]; ++nin; }
  if (J < n - 1) { sum += e[q + pitch]; ++nin; }
  return hl(r, q) * s4 - ((float)nin * c - sum);
}

// rc = (sum over the 2 x 2 children of the residual) / (4 s4) (the stored
// form of the coarse right-hand side); ec = 0.
template <class T>
__device__ __forceinline__ void mg_restrict_cell(const float* e, const T* r, int n, int pitch,
                                                 float s4, T* rc, float* ec, int nc, int pitchc,
                                                 int I, int J) {
  if (I >= nc || J >= nc) return;
  float s = 0.0f;
#pragma unroll
  for (int b = 0; b < 2; ++b)
#pragma unroll
    for (int a = 0; a < 2; ++a) {
      const int i = 2 * I + a, j = 2 * J + b;
      if (i < n && j < n) s += mg_resid(e, r, i, j, n, pitch, s4);
    }
  hs(rc, (size_t)J * pitchc + I, s / (4.0f * s4));
  ec[(size_t)J * pitchc + I] = 0.0f;
}
template <class T>
__global__ void k_mg_restrict(const float* __restrict__ e, const T* __restrict__ r, int n,
                              int pitch, float s4, T* __restrict__ rc, float* __restrict__ ec,
                              int nc, int pitchc) {
  mg_restrict_cell(e, r, n, pitch, s4, rc, ec, nc, pitchc,
                   (int)(blockIdx.x * blockDim.x + threadIdx.x),
                   (int)(blockIdx.y * blockDim.y + threadIdx.y));
}

// e += bilinear interpolation of the coarse correction (weights 9/16, 3/16,
// 3/16, 1/16; a coarse neighbour beyond the wall reflects to the parent).
__device__ __forceinline__ void mg_prolong_cell(float* e, int n, int pitch, const float* ec, int nc,
                                                int pitchc, int i, int j) {
  if (i >= n || j >= n) return;
  const int I = i >> 1, J = j >> 1;
  int In = I + ((i & 1) ? 1 : -1), Jn = J + ((j & 1) ? 1 : -1);
  if (In < 0 || In >= nc) In = I;
  if (Jn < 0 || Jn >= nc) Jn = J;
  const float v = 0.5625f * ec[(size_t)J * pitchc + I] + 0.1875f * ec[(size_t)J * pitchc + In] +
                  0.1875f * ec[(size_t)Jn * pitchc + I] + 0.0625f * ec[(size_t)Jn * pitchc + In];
  e[(size_t)j * pitch + i] += v;
}
__global__ void k_mg_prolong(float* __restrict__ e, int n, int pitch, const float* __restrict__ ec,
                             int nc, int pitchc) {
  mg_prolong_cell(e, n, pitch, ec, nc, pitchc, (int)(blockIdx.x * blockDim.x + threadIdx.x),
                  (int)(blockIdx.y * blockDim.y + threadIdx.y));
}

// The coarsest level (n <= 32) by one block of 1024 threads in shared memory:
// `iters` red-black sweeps from e = 0, then the mean removed (the pure
// Neumann problem determines e only up to a constant).
template <class T>
__device__ __forceinline__ void mg_coarse_block(float* __restrict__ e, const T* __restrict__ r,
                                                int n, int pitch, float s4, int iters) {
  __shared__ float se[32][33], sr[32][33];
  __shared__ float ssum[32];
  const int I = threadIdx.x & 31, J = threadIdx.x >> 5;
  const bool in = I < n && J < n;
  se[J][I] = 0.0f;
  sr[J][I] = in ? hl(r, (size_t)J * pitch + I) * s4 : 0.0f;
  __syncthreads();
  for (int it = 0; it < iters; ++it) {
    for (int color = 0; color < 2; ++color) {
      if (in && ((I + J) & 1) == color) {
        float sum = 0.0f;
        int nin = 0;
        if (I > 0) { sum += se[J][I - 1]; ++nin; }
        if (I < n - 1) { sum += se[J][I + 1]; ++nin; }
        if (J > 0) { sum += se[J - 1][I]; ++nin; }
        if (J < n - 1) { sum += se[J + 1][I]; ++nin; }
        se[J][I] = (sr[J][I] + sum) / (float)nin;
      }
      __syncthreads();
    }
  }
  float v = in ? se[J][I] : 0.0f;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (I == 0) ssum[J] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.0f;
    for (int w = 0; w < 32; ++w) t += ssum[w];
    ssum[0] = t / (float)(n * n);
  }
  __syncthreads();
  if (in) e[(size_t)J * pitch + I] = se[J][I] - ssum[0];
}
template <class T>
__global__ void __launch_bounds__(1024) k_mg_coarse(float* __restrict__ e, const T* __restrict__ r,
                                                    int n, int pitch, float s4, int iters) {
  mg_coarse_block(e, r, n, pitch, s4, iters);
}

// The levels of a V-cycle from level l0 down, for k_mg_vcycle_small.
constexpr int kMgMaxLevels = 8;
struct MgLevels {
  int count;  // levels l0 .. l0 + count - 1 (the last one the coarsest)
  int l0;
  int n[kMgMaxLevels], pitch[kMgMaxLevels];
  float* e[kMgMaxLevels];
  void* r[kMgMaxLevels];
};

// The V-cycle's small levels (n <= 64) in one block of 1024 threads: the
// same operations in the same order as the launches of the larger levels
// (two red-black smoothing passes, restriction, the coarser levels, bilinear
// prolongation, two passes in the reverse colour order; the coarsest solved
// in shared memory), a block barrier between them. Every pass updates
// independent cells from the same operands, so the result is the launches'.
template <class T>
__global__ void __launch_bounds__(1024) k_mg_vcycle_small(MgLevels V) {
  auto smooth = [&](int k, int color) {
    const int n = V.n[k], h2 = (n + 1) / 2;
    const float s4 = ldexpf(1.0f, 2 * (V.l0 + k));
    for (int q = threadIdx.x; q < h2 * n; q += blockDim.x)
      mg_smooth_cell(V.e[k], static_cast<const T*>(V.r[k]), n, V.pitch[k], color, s4, q % h2,
                     q / h2);
    __syncthreads();
  };
  const int last = V.count - 1;
  for (int k = 0; k < last; ++k) {
    for (int s = 0; s < 2; ++s) {
      smooth(k, 0);
      smooth(k, 1);
    }
    const int n = V.n[k], nc = V.n[k + 1];
    const float s4 = ldexpf(1.0f, 2 * (V.l0 + k));
    for (int q = threadIdx.x; q < nc * nc; q += blockDim.x)
      mg_restrict_cell(V.e[k], static_cast<const T*>(V.r[k]), n, V.pitch[k], s4,
                       static_cast<T*>(V.r[k + 1]), V.e[k + 1], nc, V.pitch[k + 1], q % nc,
                       q / nc);
    __syncthreads();
  }
  mg_coarse_block(V.e[last], static_cast<const T*>(V.r[last]), V.n[last], V.pitch[last],
                  ldexpf(1.0f, 2 * (V.l0 + last)), 64);
  __syncthreads();
  for (int k = last - 1; k >= 0; --k) {
    const int n = V.n[k];
    for (int q = threadIdx.x; q < n * n; q += blockDim.x)
      mg_prolong_cell(V.e[k], n, V.pitch[k], V.e[k + 1], V.n[k + 1], V.pitch[k + 1], q % n,
                      q / n);
    __syncthreads();
    for (int s = 0; s < 2; ++s) {
      smooth(k, 1);
      smooth(k, 0);
    }
  }
}

// ---- refinement on the fine grid (f32 pressure, pitched like the fields) ----

__device__ __forceinline__ void block_add_f64x2(double a, double b, double* out) {
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  __shared__ double pa[32], pb[32];
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    pa[w] = a;
    pb[w] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ta = 0.0, tb = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
      ta += pa[k];
      tb += pb[k];
    }
    atomicAdd(out, ta);
    atomicAdd(out + 1, tb);
  }
}

// The refinement's pressure is a pair of FP32 grids, p = ph + pl (pl the
// low-order part): the residual of an FP32 pressure has a floor near
// eps32 ||A|| ||p||, above a 1e-5 relative target on large grids. The pair is
// read and updated in double-float arithmetic, FP32 operations only: Knuth's
// two-sum, Dekker's fast two-sum and the FMA's exact product, about 48
// significant bits (an error relative to the operands, not to the
// cancelling result, near 2^-47). FP64 appears only in the reductions.
struct DF {
  float h, l;
};
__device__ __forceinline__ DF df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float v = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v))};
}
__device__ __forceinline__ DF df_fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
  const DF s = df_two_sum(a.h, b.h);
  return df_fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ DF df_neg(DF a) { return {-a.h, -a.l}; }
// (s.h + s.l) * e for an FP32 e
__device__ __forceinline__ DF df_mul_f(DF s, float e) {
  const float p = __fmul_rn(s.h, e);
  return df_fast_two_sum(p, __fmaf_rn(s.l, e, __fmaf_rn(s.h, e, -p)));
}
__device__ __forceinline__ DF ir_p(const float* ph, const float* pl, size_t q) {
  return {ph[q], pl[q]};
}
// a double's nearest double-float (the host splits the refinement's scale)
__host__ __device__ inline void df_split(double v, float* h, float* l) {
  *h = (float)v;
  *l = (float)(v - (double)*h);
}

// r = b - A p on the interior (double-float arithmetic, stored FP32), with
// FP64 sums of r and r^2.
__global__ void k_ir_residual(const float* __restrict__ ph, const float* __restrict__ pl,
                              const float* __restrict__ b, int S, int P,
                              const uint8_t* __restrict__ rowfl,
                              const uint8_t* __restrict__ colfl, float* __restrict__ r,
                              double* __restrict__ acc) {
  const int N = S - 2;
  double s1 = 0.0, s2 = 0.0;
  const size_t n = (size_t)N * N;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(k / N) + 1, i = (int)(k % N) + 1;
    const size_t q = (size_t)j * P + i;
    const DF c = ir_p(ph, pl, q);
    const DF L = (i == 1) ? (rowfl[j] ? c : ir_p(ph, pl, q - 1)) : ir_p(ph, pl, q - 1);
    const DF R = (i == N) ? (rowfl[j] ? c : ir_p(ph, pl, q + 1)) : ir_p(ph, pl, q + 1);
    const DF U = (j == 1) ? (colfl[i] ? c : ir_p(ph, pl, q - P)) : ir_p(ph, pl, q - P);
    const DF D = (j == N) ? (colfl[i] ? c : ir_p(ph, pl, q + P)) : ir_p(ph, pl, q + P);
    const DF c4 = {__fmul_rn(4.0f, c.h), __fmul_rn(4.0f, c.l)};  // exact
    const DF Ap = df_add(c4, df_neg(df_add(df_add(df_add(L, R), U), D)));
    const DF res = df_add({b[q], 0.0f}, df_neg(Ap));
    const float rf = __fadd_rn(res.h, res.l);
    r[q] = rf;
    s1 += (double)rf;
    s2 = __fma_rn((double)rf, (double)rf, s2);
  }
  block_add_f64x2(s1, s2, acc);
}

// Level-0 right-hand side: (r - mean) / scale in the storage format.
template <class T>
__global__ void k_ir_scale(const float* __restrict__ r, int S, int P, float mean, float inv_scale,
                           T* __restrict__ r0, int pitch0) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int N = S - 2;
  if (I >= N || J >= N) return;
  hs(r0, (size_t)J * pitch0 + I, (r[(size_t)(J + 1) * P + I + 1] - mean) * inv_scale);
}

// p += scale * e0 on the interior (double-float; scale = sh + sl).
__global__ void k_ir_update(float* __restrict__ ph, float* __restrict__ pl, int S, int P,
                            const float* __restrict__ e0, int pitch0, float sh, float sl) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int N = S - 2;
  if (I >= N || J >= N) return;
  const size_t q = (size_t)(J + 1) * P + I + 1;
  const DF v = df_add(ir_p(ph, pl, q), df_mul_f({sh, sl}, e0[(size_t)J * pitch0 + I]));
  ph[q] = v.h;
  pl[q] = v.l;
}

// Sum of p over the interior (FP64) into acc[0].
__global__ void k_ir_sum(const float* __restrict__ ph, const float* __restrict__ pl, int S, int P,
                         double* __restrict__ acc) {
  const int N = S - 2;
  DF s = {0.0f, 0.0f};
  const size_t n = (size_t)N * N;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(k / N) + 1, i = (int)(k % N) + 1;
    s = df_add(s, ir_p(ph, pl, (size_t)j * P + i));
  }
  block_add_f64x2((double)s.h + (double)s.l, 0.0, acc);
}

// p -= mean(p) on the interior: the pure-Neumann solution's free constant is
// fixed at zero mean.
__global__ void k_ir_center(float* __restrict__ ph, float* __restrict__ pl, int S, int P,
                            const double* __restrict__ acc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int N = S - 2;
  __shared__ DF s_mean;  // the mean, once per block
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    DF m;
    df_split(acc[0] / ((double)N * N), &m.h, &m.l);
    s_mean = m;
  }
  __syncthreads();
  if (i > N || j > N) return;
  const size_t q = (size_t)j * P + i;
  const DF v = df_add(ir_p(ph, pl, q), df_neg(s_mean));
  ph[q] = v.h;
  pl[q] = v.l;
}

// p = 0 on the interior (project's `p[idx] = 0.0`, fluid.rs:349).
__global__ void k_ir_zero(float* __restrict__ ph, float* __restrict__ pl, int S, int P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > S - 2 || j > S - 2) return;
  ph[(size_t)j * P + i] = 0.0f;
  pl[(size_t)j * P + i] = 0.0f;
}

}  // namespace eqk
