// Per-cell kernels of the frame step: set_boundaries, project's divergence and
// gradient, advect, sources. Grids are pitched: cell (i, j) of a field lives at
// f[j * P + i], 0 <= i, j < S, P = row pitch in elements (multiple of 32).
#pragma once
#include "common.cuh"

namespace eqk {

// ---------------------------------------------------------------------------
// set_boundaries (fluid.rs:133-189, 252-272) as an order-independent map.
// Velocity modes write fluid cells from wall neighbours (walls are never
// written); Passive writes the frame from the first/last interior row or
// column, but only where that row/column holds a fluid cell. Corners are the
// mean of the two post-pass frame neighbours, computed from pre-pass values.
// ---------------------------------------------------------------------------
template <int MODE>
__device__ __forceinline__ float frame_after_pass(const float* x, const uint8_t* rowfl,
                                                  const uint8_t* colfl, int S, int P, int i,
                                                  int j) {
  // Value of frame cell (i, j) (not a corner) after the per-cell pass.
  if (MODE == kPassive) {
    if (j == 0 && colfl[i]) return x[(size_t)1 * P + i];
    if (j == S - 1 && colfl[i]) return x[(size_t)(S - 2) * P + i];
    if (i == 0 && rowfl[j]) return x[(size_t)j * P + 1];
    if (i == S - 1 && rowfl[j]) return x[(size_t)j * P + (S - 2)];
  }
  return x[(size_t)j * P + i];
}

template <int MODE>
__device__ __forceinline__ void corners(float* x, const uint8_t* rowfl, const uint8_t* colfl,
                                        int S, int P) {
  const float c00 = fmul(0.5f, fadd(frame_after_pass<MODE>(x, rowfl, colfl, S, P, 1, 0),
                                    frame_after_pass<MODE>(x, rowfl, colfl, S, P, 0, 1)));
  const float c0S = fmul(0.5f, fadd(frame_after_pass<MODE>(x, rowfl, colfl, S, P, 1, S - 1),
                                    frame_after_pass<MODE>(x, rowfl, colfl, S, P, 0, S - 2)));
  const float cS0 = fmul(0.5f, fadd(frame_after_pass<MODE>(x, rowfl, colfl, S, P, S - 2, 0),
                                    frame_after_pass<MODE>(x, rowfl, colfl, S, P, S - 1, 1)));
  const float cSS =
      fmul(0.5f, fadd(frame_after_pass<MODE>(x, rowfl, colfl, S, P, S - 2, S - 1),
                      frame_after_pass<MODE>(x, rowfl, colfl, S, P, S - 1, S - 2)));
  x[0] = c00;
  x[(size_t)(S - 1) * P] = c0S;
  x[S - 1] = cS0;
  x[(size_t)(S - 1) * P + (S - 1)] = cSS;
}

template <int MODE>
__global__ void k_set_boundaries(float* __restrict__ x, const uint8_t* __restrict__ code,
                                 const uint8_t* __restrict__ rowfl,
                                 const uint8_t* __restrict__ colfl, int S, int P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= S || j >= S) return;
  const int N = S - 2;
  if (i == 0 && j == 0) {
    corners<MODE>(x, rowfl, colfl, S, P);
    return;
  }
  const bool corner = (i == 0 || i == S - 1) && (j == 0 || j == S - 1);
  if (corner) return;
  if (MODE == kPassive) {
    if (j == 0 || j == S - 1 || i == 0 || i == S - 1)
      x[(size_t)j * P + i] = frame_after_pass<MODE>(x, rowfl, colfl, S, P, i, j);
    return;
  }
  if (i < 1 || i > N || j < 1 || j > N) return;
  const uint8_t c = code[(size_t)j * P + i];
  if (MODE == kRow) {
    if (c & kCodeRowRight)
      x[(size_t)j * P + i] = -x[(size_t)j * P + i + 1];
    else if (c & kCodeRowLeft)
      x[(size_t)j * P + i] = -x[(size_t)j * P + i - 1];
  } else {
    if (c & kCodeColUp)
      x[(size_t)j * P + i] = -x[(size_t)(j - 1) * P + i];
    else if (c & kCodeColDown)
      x[(size_t)j * P + i] = -x[(size_t)(j + 1) * P + i];
  }
}

// ---------------------------------------------------------------------------
// project (fluid.rs:330-375): divergence + zero pressure on the interior ...
// ---------------------------------------------------------------------------
static __global__ void k_divergence(const float* __restrict__ vx, const float* __restrict__ vy,
                             float* __restrict__ p, float* __restrict__ div, int S, int P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int N = S - 2;
  if (i > N || j > N) return;
  const size_t q = (size_t)j * P + i;
  const float inner = fsub(fadd(fsub(vx[q + 1], vx[q - 1]), vy[q + P]), vy[q - P]);
  div[q] = fdiv(fmul(-0.5f, inner), (float)S);
  p[q] = 0.0f;
}

// ... and the gradient subtraction (fluid.rs:364-371), interior incl. walls.
static __global__ void k_gradient(float* __restrict__ vx, float* __restrict__ vy,
                           const float* __restrict__ p, int S, int P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int N = S - 2;
  if (i > N || j > N) return;
  const size_t q = (size_t)j * P + i;
  const float sf = (float)S;
  vx[q] = fsub(vx[q], fmul(fmul(0.5f, fsub(p[q + 1], p[q - 1])), sf));
  vy[q] = fsub(vy[q], fmul(fmul(0.5f, fsub(p[q + P], p[q - P])), sf));
}

// ---------------------------------------------------------------------------
// advect (fluid.rs:378-432), one CTA per interior row j. Pass 1 finds the
// row's first "break" cell (clamped backtrace reached size-1); pass 2 writes
// cells before it by bilinear interpolation, the break cell with its left
// neighbour's new value (the old ghost when it is i = 1) and leaves the cells
// after it untouched.
// ---------------------------------------------------------------------------
struct Backtrace {
  float s0, s1, t0, t1;
  int i0, i1, j0, j1;
  bool brk;
};

__device__ __forceinline__ Backtrace backtrace(int i, int j, float uij, float vij, float dt0,
                                               int S) {
  const float sf = (float)S;
  const float hi = fsub(sf, 1.0f);
  // the backtrace position stays rounded twice in the FMA build too: a fused
  // i - dt0*u moves the sample point by an ulp, which steep fields (the
  // sources' edges) turn into relative errors above 1e-6
  float x = __fsub_rn((float)i, __fmul_rn(dt0, uij));
  float y = __fsub_rn((float)j, __fmul_rn(dt0, vij));
  x = rust_clamp(x, 0.5f, hi);
  y = rust_clamp(y, 0.5f, hi);
  const float fi0 = floorf(x), fj0 = floorf(y);
  const float fi1 = fadd(fi0, 1.0f), fj1 = fadd(fj0, 1.0f);
  Backtrace b;
  b.s1 = fsub(x, fi0);
  b.s0 = fsub(1.0f, b.s1);
  b.t1 = fsub(y, fj0);
  b.t0 = fsub(1.0f, b.t1);
  b.i0 = as_u32_clamped(fi0, S);
  b.i1 = as_u32_clamped(fi1, S);
  b.j0 = as_u32_clamped(fj0, S);
  b.j1 = as_u32_clamped(fj1, S);
  b.brk = (fi1 >= sf) || (fj1 >= sf);
  return b;
}

__device__ __forceinline__ float bilerp(const Backtrace& b, const float* __restrict__ d0,
                                        int P) {
  const float A = d0[(size_t)b.j0 * P + b.i0];
  const float B = d0[(size_t)b.j1 * P + b.i0];
  const float C = d0[(size_t)b.j0 * P + b.i1];
  const float D = d0[(size_t)b.j1 * P + b.i1];
  return fadd(fmul(b.s0, fadd(fmul(b.t0, A), fmul(b.t1, B))),
              fmul(b.s1, fadd(fmul(b.t0, C), fmul(b.t1, D))));
}

static __global__ void k_advect_rows(float* __restrict__ d, const float* __restrict__ d0,
                              const float* __restrict__ u, const float* __restrict__ v,
                              int S, int P, float dt0) {
  const int j = blockIdx.x + 1;
  const int N = S - 2;
  __shared__ int s_brk;
  if (threadIdx.x == 0) s_brk = 0x7fffffff;
  __syncthreads();
  const size_t row = (size_t)j * P;
  int mine = 0x7fffffff;
  for (int i = threadIdx.x + 1; i <= N; i += blockDim.x) {
    const Backtrace b = backtrace(i, j, u[row + i], v[row + i], dt0, S);
    if (b.brk) {
      mine = i;
      break;  // first break among this thread's cells (they ascend)
    }
  }
  if (mine != 0x7fffffff) atomicMin(&s_brk, mine);
  __syncthreads();
  const int brk = s_brk;
  for (int i = threadIdx.x + 1; i <= N && i <= brk; i += blockDim.x) {
    float val;
    if (i == brk) {
      if (i == 1) {
        val = d[row];  // old ghost d[0, j]
      } else {
        const Backtrace b = backtrace(i - 1, j, u[row + i - 1], v[row + i - 1], dt0, S);
        val = bilerp(b, d0, P);
      }
    } else {
      const Backtrace b = backtrace(i, j, u[row + i], v[row + i], dt0, S);
      val = bilerp(b, d0, P);
    }
    d[row + i] = val;
  }
}

// ---------------------------------------------------------------------------
// Sources (add_density / add_velocity, fluid.rs:120-131), applied serially in
// array order so repeated cells accumulate in the reference's order.
// ---------------------------------------------------------------------------
static __global__ void k_sources(float* __restrict__ density, float* __restrict__ scratch,
                          float* __restrict__ vx, float* __restrict__ vy, int S, int P,
                          int64_t n, const uint32_t* __restrict__ xs,
                          const uint32_t* __restrict__ ys, const float* __restrict__ dd,
                          const float* __restrict__ du, const float* __restrict__ dv) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  for (int64_t s = 0; s < n; ++s) {
    const uint32_t x = xs[s] > (uint32_t)(S - 1) ? (uint32_t)(S - 1) : xs[s];
    const uint32_t y = ys[s] > (uint32_t)(S - 1) ? (uint32_t)(S - 1) : ys[s];
    const size_t q = (size_t)y * P + x;
    if (dd) {
      density[q] = fadd(density[q], dd[s]);
      scratch[q] = fadd(scratch[q], dd[s]);
    }
    if (du) vx[q] = fadd(vx[q], du[s]);
    if (dv) vy[q] = fadd(vy[q], dv[s]);
  }
}

// scratch_space = density.clone() (fluid.rs:523) over the whole pitched grid.
static __global__ void k_copy(float* __restrict__ dst, const float* __restrict__ src, size_t n4) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const float4* s = reinterpret_cast<const float4*>(src);
  float4* d = reinterpret_cast<float4*>(dst);
  for (size_t q = t; q < n4; q += stride) d[q] = s[q];
}

// Dense copies of up to six pitched fields, one after another (the staging of
// eq_fluid_read_fields: one contiguous device-to-host copy per field).
struct PackFields {
  const float* src[6];
  int count;
};
static __global__ void k_pack_fields(PackFields f, float* __restrict__ dst, int S, int P) {
  const size_t g = (size_t)S * S, total = g * (size_t)f.count;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < total;
       q += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(q / g);
    const size_t c = q - (size_t)k * g;
    const size_t j = c / S, i = c - j * S;
    dst[q] = f.src[k][j * P + i];
  }
}

}  // namespace eqk
