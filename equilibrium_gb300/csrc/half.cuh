// The precision form: the six fields of Fluid (fluid.rs:59-77) stored in
// FP16 or BF16 (half the bytes of every field access), every operation
// computed in FP32 on the widened values, results rounded once on store.
// The frame keeps the reference's phases, order and aliasing (fluid.rs:
// 437-524); the pressure solve is replaced by mixed-precision iterative
// refinement to a relative residual (mg.cuh). Grids are pitched row-major:
// cell (i, j) at j * P + i.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "common.cuh"
#include "kernels.cuh"
#include "store.cuh"

namespace eqk {

// f32 <-> storage over a whole pitched grid.
template <class T>
__global__ void k_h_widen(float* __restrict__ dst, const T* __restrict__ src, size_t n) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride)
    dst[q] = hl(src, q);
}
template <class T>
__global__ void k_h_narrow(T* __restrict__ dst, const float* __restrict__ src, size_t n) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride)
    hs(dst, q, src[q]);
}
template <class T>
__global__ void k_h_copy(T* __restrict__ dst, const T* __restrict__ src, size_t n) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride)
    dst[q] = src[q];
}

// add_density / add_velocity (fluid.rs:120-131), serially in array order
// (scalars in TS, velocities in TV).
template <class TS, class TV>
__global__ void k_h_sources(TS* de, TS* sc, TV* vx, TV* vy, int S, int P, int64_t n,
                            const uint32_t* xs, const uint32_t* ys, const float* dd,
                            const float* du, const float* dv) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  for (int64_t s = 0; s < n; ++s) {
    const uint32_t x = xs[s] > (uint32_t)(S - 1) ? (uint32_t)(S - 1) : xs[s];
    const uint32_t y = ys[s] > (uint32_t)(S - 1) ? (uint32_t)(S - 1) : ys[s];
    const size_t q = (size_t)y * P + x;
    hs(de, q, hl(de, q) + dd[s]);
    hs(sc, q, hl(sc, q) + dd[s]);
    hs(vx, q, hl(vx, q) + du[s]);
    hs(vy, q, hl(vy, q) + dv[s]);
  }
}

// set_boundaries (fluid.rs:252-272) on a stored field: the per-cell map of
// k_set_boundaries with the corners from pre-pass values.
template <int MODE, class T>
__device__ __forceinline__ float h_frame_after_pass(const T* x, const uint8_t* rowfl,
                                                    const uint8_t* colfl, int S, int P, int i,
                                                    int j) {
  if (MODE == kPassive) {
    if (j == 0 && colfl[i]) return hl(x, (size_t)1 * P + i);
    if (j == S - 1 && colfl[i]) return hl(x, (size_t)(S - 2) * P + i);
    if (i == 0 && rowfl[j]) return hl(x, (size_t)j * P + 1);
    if (i == S - 1 && rowfl[j]) return hl(x, (size_t)j * P + (S - 2));
  }
  return hl(x, (size_t)j * P + i);
}

template <int MODE, class T>
__global__ void k_h_bnd(T* __restrict__ x, const uint8_t* __restrict__ code,
                        const uint8_t* __restrict__ rowfl, const uint8_t* __restrict__ colfl,
                        int S, int P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= S || j >= S) return;
  const int N = S - 2;
  if (i == 0 && j == 0) {
    auto f = [&](int a, int b) { return h_frame_after_pass<MODE>(x, rowfl, colfl, S, P, a, b); };
    const float c00 = 0.5f * (f(1, 0) + f(0, 1));
    const float c0S = 0.5f * (f(1, S - 1) + f(0, S - 2));
    const float cS0 = 0.5f * (f(S - 2, 0) + f(S - 1, 1));
    const float cSS = 0.5f * (f(S - 2, S - 1) + f(S - 1, S - 2));
    hs(x, 0, c00);
    hs(x, (size_t)(S - 1) * P, c0S);
    hs(x, (size_t)(S - 1), cS0);
    hs(x, (size_t)(S - 1) * P + (S - 1), cSS);
    return;
  }
  if ((i == 0 || i == S - 1) && (j == 0 || j == S - 1)) return;
  if (MODE == kPassive) {
    if (j == 0 || j == S - 1 || i == 0 || i == S - 1)
      hs(x, (size_t)j * P + i, h_frame_after_pass<MODE>(x, rowfl, colfl, S, P, i, j));
    return;
  }
  if (i < 1 || i > N || j < 1 || j > N) return;
  const size_t q = (size_t)j * P + i;
  const uint8_t c = code[q];
  // (negation is exact in every storage format)
  if (MODE == kRow) {
    if (c & kCodeRowRight)
      hs(x, q, -hl(x, q + 1));
    else if (c & kCodeRowLeft)
      hs(x, q, -hl(x, q - 1));
  } else {
    if (c & kCodeColUp)
      hs(x, q, -hl(x, q - P));
    else if (c & kCodeColDown)
      hs(x, q, -hl(x, q + P));
  }
}

// project's divergence (fluid.rs:339-352) from stored velocities: f32 `div`
// (the refinement's right-hand side) and its stored copy in the array the
// reference aliases as div.
template <class T>
__global__ void k_h_divergence(const T* __restrict__ vx, const T* __restrict__ vy,
                               float* __restrict__ div32, T* __restrict__ divs, int S, int P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int N = S - 2;
  if (i > N || j > N) return;
  const size_t q = (size_t)j * P + i;
  const float inner = ((hl(vx, q + 1) - hl(vx, q - 1)) + hl(vy, q + P)) - hl(vy, q - P);
  const float d = (-0.5f * inner) / (float)S;
  div32[q] = d;
  hs(divs, q, d);
}

// project's gradient subtraction (fluid.rs:364-371) with the f32 pressure.
template <class T>
__global__ void k_h_gradient(T* __restrict__ vx, T* __restrict__ vy, const float* __restrict__ p,
                             int S, int P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int N = S - 2;
  if (i > N || j > N) return;
  const size_t q = (size_t)j * P + i;
  const float sf = (float)S;
  hs(vx, q, hl(vx, q) - (0.5f * (p[q + 1] - p[q - 1])) * sf);
  hs(vy, q, hl(vy, q) - (0.5f * (p[q + P] - p[q - P])) * sf);
}

// ||div(v)||_2 over the interior in FP64 (the post-projection divergence).
template <class T>
__global__ void k_h_div_norm(const T* __restrict__ vx, const T* __restrict__ vy, int S, int P,
                             double* __restrict__ out) {
  const int N = S - 2;
  double acc = 0.0;
  const size_t n = (size_t)N * N;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(k / N) + 1, i = (int)(k % N) + 1;
    const size_t q = (size_t)j * P + i;
    // (-0.5 (dvx + dvy) / S)^2 with the constant factor applied per block
    const double d =
        ((double)hl(vx, q + 1) - hl(vx, q - 1)) + ((double)hl(vy, q + P) - hl(vy, q - P));
    acc = __fma_rn(d, d, acc);
  }
  acc *= 0.25 / ((double)S * S);
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  __shared__ double part[32];
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
    atomicAdd(out, t);
  }
}

// advect (fluid.rs:378-432) on stored fields, one block per row: the row's
// first break, then the cells up to it (the break cell copies its left
// neighbour's new value, or the old ghost when it is column 1).
__device__ __forceinline__ float h_bilerp_f(const Backtrace& b, float A, float B, float C,
                                            float D) {
  return b.s0 * (b.t0 * A + b.t1 * B) + b.s1 * (b.t0 * C + b.t1 * D);
}

template <class T, class TU = T>
__global__ void k_h_advect_rows(T* __restrict__ d, const T* __restrict__ d0,
                                const TU* __restrict__ u, const TU* __restrict__ v, int S, int P,
                                float dt0) {
  const int j = blockIdx.x + 1;
  const int N = S - 2;
  __shared__ int s_brk;
  if (threadIdx.x == 0) s_brk = 0x7fffffff;
  __syncthreads();
  const size_t row = (size_t)j * P;
  int mine = 0x7fffffff;
  for (int i = threadIdx.x + 1; i <= N; i += blockDim.x) {
    if (backtrace(i, j, hl(u, row + i), hl(v, row + i), dt0, S).brk) {
      mine = i;
      break;
    }
  }
  if (mine != 0x7fffffff) atomicMin(&s_brk, mine);
  __syncthreads();
  const int brk = s_brk;
  const float ghost = hl(d, row);
  __syncthreads();
  for (int i = threadIdx.x + 1; i <= N && i <= brk; i += blockDim.x) {
    float val;
    if (i == brk && i == 1) {
      val = ghost;
    } else {
      const int ic = (i == brk) ? i - 1 : i;
      const Backtrace b = backtrace(ic, j, hl(u, row + ic), hl(v, row + ic), dt0, S);
      val = h_bilerp_f(b, hl(d0, (size_t)b.j0 * P + b.i0), hl(d0, (size_t)b.j1 * P + b.i0),
                       hl(d0, (size_t)b.j0 * P + b.i1), hl(d0, (size_t)b.j1 * P + b.i1));
    }
    hs(d, row + i, val);
  }
}

// init() (fluid.rs:602-606) on zeroed stored fields: vx = vy = 1, +0.9
// density and scratch on the block [S/2-10, S/2+10]^2 (idx!-clamped).
template <class TS, class TV>
__global__ void k_h_init(TS* sc, TS* de, TV* vx, TV* vy, int S, int P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= S || j >= S) return;
  const int lo = S / 2 - 10, hi = S / 2 + 10;
  auto mult = [&](int c) {
    int m = (c >= lo && c <= hi) ? 1 : 0;
    if (c == S - 1 && hi > S - 1) m += hi - (S - 1);
    return m;
  };
  float dens = 0.0f;
  for (int r = mult(i) * mult(j); r > 0; --r) dens += 0.9f;
  const size_t q = (size_t)j * P + i;
  hs(sc, q, dens);
  hs(de, q, dens);
  hs(vx, q, 1.0f);
  hs(vy, q, 1.0f);
}

}  // namespace eqk
