// The batched form: thousands of independent scenes (each a full Fluid,
// fluid.rs:52-81, of its own size, time step, diffusion, viscosity and sweep
// count) advance one frame per launch of ONE persistent kernel. A thread block
// takes the next scene from a work queue (scenes ordered by decreasing work,
// so the largest start first) and runs that scene's whole Fluid::step
// (fluid.rs:437-524) by itself: per-cell phases spread over its threads, the
// five lin_solves as block-level temporal wavefronts (wave.cuh), block
// barriers between phases. No inter-block communication exists at all, so
// the result of every scene is bit-identical to the plain form's.
#pragma once
#include "common.cuh"
#include "kernels.cuh"
#include "wave.cuh"

namespace eqk {

// One scene of a batch. Fields f = 0..5 (scratch, density, vx, vy, vx0, vy0)
// live at arena + foff + f * fstride in the anti-diagonal layout of wave.cuh
// (cell (i, j) at (i + j) * P + j, fstride = (2S - 1) * P); the boundary codes
// at marena + moff in the same layout ((2S - 1) * P bytes), then rowfl [S],
// then colfl [S].
struct BScene {
  unsigned long long foff, fstride, moff;
  int S, P, K;
  float dt, diff, visc;
  int nsrc, src_off;
};

struct BatchArgs {
  float* arena;
  const uint8_t* marena;
  const BScene* scenes;
  const int* order;  // queue position -> scene index
  int nscenes;
  unsigned* queue;   // this frame's work counter (zeroed before the launch)
  const uint32_t* src_x;
  const uint32_t* src_y;
  const float* src_d;
  const float* src_u;
  const float* src_v;
  float* gscratch;   // per-block carry/edge rows when they do not fit in shared memory
  int nwmax;         // sweeps per wavefront pass (warps per block)
  int cs;            // carry/edge row stride (floats)
  int bufs_in_smem;  // 1: carry/edge rows in shared memory
};

__host__ __device__ inline size_t batch_ring_floats(int nwmax) {
  return (size_t)(nwmax > 1 ? nwmax - 1 : 0) * 32 * kWRS;
}
__host__ __device__ inline size_t batch_bufs_floats(int nwmax, int cs) {
  return (size_t)nwmax * 3 * cs;  // carry (2 rows) + edge (1 row) per warp
}

// ---- per-cell phases over one scene, by the whole block --------------------
// Cells are visited by anti-diagonals (warp = diagonal, lane = row j), so the
// 32 lanes of a warp touch consecutive addresses.

// Visit every cell (i, j) with ilo <= i <= ihi, jlo <= j <= jhi.
template <class F>
__device__ __forceinline__ void dg_for_cells(int ilo, int ihi, int jlo, int jhi, int P, F&& fn) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
  for (int d = ilo + jlo + warp; d <= ihi + jhi; d += nwarp) {
    const int j0 = max(jlo, d - ihi), j1 = min(jhi, d - ilo);
    for (int j = j0 + lane; j <= j1; j += 32) fn(d - j, j, (size_t)d * P + j);
  }
}

__device__ __forceinline__ void blk_sources(const BatchArgs& A, const BScene& sc, float* de,
                                            float* scr, float* vx, float* vy) {
  if (threadIdx.x != 0 || sc.nsrc <= 0) return;
  const int S = sc.S, P = sc.P;
  for (int s = sc.src_off; s < sc.src_off + sc.nsrc; ++s) {  // array order, like k_sources
    const int x = A.src_x[s] > (uint32_t)(S - 1) ? S - 1 : (int)A.src_x[s];
    const int y = A.src_y[s] > (uint32_t)(S - 1) ? S - 1 : (int)A.src_y[s];
    const size_t q = dg_at(x, y, P);
    de[q] = fadd(de[q], A.src_d[s]);
    scr[q] = fadd(scr[q], A.src_d[s]);
    vx[q] = fadd(vx[q], A.src_u[s]);
    vy[q] = fadd(vy[q], A.src_v[s]);
  }
}

// set_boundaries (fluid.rs:252-272): the order-independent per-cell map of
// k_set_boundaries, then the corners from post-pass frame values.
template <int MODE>
__device__ void blk_bnd(float* x, const uint8_t* code, const uint8_t* rowfl,
                        const uint8_t* colfl, int S, int P) {
  const int N = S - 2;
  if (MODE == kPassive) {
    for (int q = threadIdx.x; q < 4 * N; q += blockDim.x) {
      const int side = q / N, k = q - side * N + 1;
      const int i = side == 0 ? k : (side == 1 ? k : (side == 2 ? 0 : S - 1));
      const int j = side == 0 ? 0 : (side == 1 ? S - 1 : k);
      x[dg_at(i, j, P)] = dg_frame_after_pass<kPassive>(x, rowfl, colfl, S, P, i, j);
    }
  } else {
    // neighbours: (i+-1, j) at q +- P, (i, j+-1) at q +- (P + 1)
    dg_for_cells(1, N, 1, N, P, [&](int i, int j, size_t q) {
      const uint8_t c = code[q];
      if (MODE == kRow) {
        if (c & kCodeRowRight)
          x[q] = -x[q + P];
        else if (c & kCodeRowLeft)
          x[q] = -x[q - P];
      } else {
        if (c & kCodeColUp)
          x[q] = -x[q - P - 1];
        else if (c & kCodeColDown)
          x[q] = -x[q + P + 1];
      }
    });
  }
  __syncthreads();
  if (threadIdx.x == 0) dg_corners<MODE>(x, rowfl, colfl, S, P);
  __syncthreads();
}

// project's divergence + zero pressure (fluid.rs:339-352).
__device__ void blk_divergence(const float* vx, const float* vy, float* p, float* div, int S,
                               int P) {
  const int N = S - 2;
  dg_for_cells(1, N, 1, N, P, [&](int i, int j, size_t q) {
    const float inner =
        fsub(fadd(fsub(vx[q + P], vx[q - P]), vy[q + P + 1]), vy[q - P - 1]);
    div[q] = fdiv(fmul(-0.5f, inner), (float)S);
    p[q] = 0.0f;
  });
  __syncthreads();
}

// project's gradient subtraction (fluid.rs:364-371).
__device__ void blk_gradient(float* vx, float* vy, const float* p, int S, int P) {
  const int N = S - 2;
  const float sf = (float)S;
  dg_for_cells(1, N, 1, N, P, [&](int i, int j, size_t q) {
    vx[q] = fsub(vx[q], fmul(fmul(0.5f, fsub(p[q + P], p[q - P])), sf));
    vy[q] = fsub(vy[q], fmul(fmul(0.5f, fsub(p[q + P + 1], p[q - P - 1])), sf));
  });
  __syncthreads();
}

__device__ __forceinline__ float dg_bilerp(const Backtrace& b, const float* __restrict__ d0,
                                           int P) {
  const float A = d0[dg_at(b.i0, b.j0, P)];
  const float B = d0[dg_at(b.i0, b.j1, P)];
  const float C = d0[dg_at(b.i1, b.j0, P)];
  const float D = d0[dg_at(b.i1, b.j1, P)];
  return fadd(fmul(b.s0, fadd(fmul(b.t0, A), fmul(b.t1, B))),
              fmul(b.s1, fadd(fmul(b.t0, C), fmul(b.t1, D))));
}

// advect (fluid.rs:378-432). Pass 1 finds every row's first break (the
// clamped backtrace reached size-1) with an atomic minimum per row; pass 2
// writes the cells before it by bilinear interpolation, the break cell with
// its left neighbour's new value (the old ghost when it is column 1), and
// leaves the cells after it untouched. `brk` is block scratch of >= S ints.
__device__ void blk_advect(float* d, const float* d0, const float* u, const float* v, int S,
                           int P, float dt0, int* brk) {
  const int N = S - 2;
  for (int j = threadIdx.x; j < S; j += blockDim.x) brk[j] = N + 1;
  __syncthreads();
  dg_for_cells(1, N, 1, N, P, [&](int i, int j, size_t q) {
    if (backtrace(i, j, u[q], v[q], dt0, S).brk) atomicMin(&brk[j], i);
  });
  __syncthreads();
  dg_for_cells(1, N, 1, N, P, [&](int i, int j, size_t q) {
    const int bj = brk[j];
    if (i > bj) return;
    float val;
    if (i == bj && i == 1) {
      val = d[q - P];  // d[0, j] before this pass (column 0 is never written here)
    } else {
      const int ic = (i == bj) ? i - 1 : i;
      const size_t qc = (i == bj) ? q - P : q;
      const Backtrace b = backtrace(ic, j, u[qc], v[qc], dt0, S);
      val = dg_bilerp(b, d0, P);
    }
    d[q] = val;
  });
  __syncthreads();
}

// scratch_space = density.clone() (fluid.rs:523) over every cell.
__device__ void blk_copy(float* dst, const float* src, int S, int P) {
  dg_for_cells(0, S - 1, 0, S - 1, P, [&](int i, int j, size_t q) { dst[q] = src[q]; });
  __syncthreads();
}

// diffuse (fluid.rs:276-298): a = ((dt*diff)*sf)*sf, c = 1 + 4a, 1/c in f32.
template <int MODE>
__device__ void blk_diffuse(const WGrid& G, const WBufs& Bf, int K, int nwmax, float dt,
                            float diffusion) {
  const float sf = (float)(G.S - 2);
  const float a = fmul(fmul(fmul(dt, diffusion), sf), sf);
  const float c = fadd(1.0f, fmul(4.0f, a));
  wave_lin_solve<MODE>(G, Bf, K, nwmax, a, fdiv(1.0f, c));
}

// project (fluid.rs:330-375) with p and div as the reference aliases them.
__device__ void blk_project(WGrid G, const WBufs& Bf, int K, int nwmax, float* vx, float* vy,
                            float* p, float* div) {
  const int S = G.S, P = G.P;
  blk_divergence(vx, vy, p, div, S, P);
  blk_bnd<kPassive>(div, G.code, G.rowfl, G.colfl, S, P);
  blk_bnd<kPassive>(p, G.code, G.rowfl, G.colfl, S, P);
  G.x = p;
  G.x0 = div;
  wave_lin_solve<kPassive>(G, Bf, K, nwmax, 1.0f, fdiv(1.0f, 4.0f));
  blk_gradient(vx, vy, p, S, P);
  blk_bnd<kRow>(vx, G.code, G.rowfl, G.colfl, S, P);
  blk_bnd<kCol>(vy, G.code, G.rowfl, G.colfl, S, P);
}

// One Fluid::step of one scene, with the reference's aliasing of its arrays.
__device__ void blk_frame(const BatchArgs& A, const BScene& sc, const WBufs& Bf) {
  float* f[6];
#pragma unroll
  for (int q = 0; q < 6; ++q) f[q] = A.arena + sc.foff + (size_t)q * sc.fstride;
  float *scr = f[0], *de = f[1], *vx = f[2], *vy = f[3], *vx0 = f[4], *vy0 = f[5];
  const uint8_t* code = A.marena + sc.moff;
  WGrid G;
  G.code = code;
  G.rowfl = code + sc.fstride;
  G.colfl = G.rowfl + sc.S;
  G.S = sc.S;
  G.P = sc.P;
  const int S = sc.S, P = sc.P, K = sc.K, nw = A.nwmax;
  const float dt0 = fmul(sc.dt, (float)(S - 2));
  int* brk = reinterpret_cast<int*>(Bf.edge);  // the edge rows are free between solves

  blk_sources(A, sc, de, scr, vx, vy);
  __syncthreads();
  G.x = vx0; G.x0 = vx;
  blk_diffuse<kRow>(G, Bf, K, nw, sc.dt, sc.visc);
  G.x = vy0; G.x0 = vy;
  blk_diffuse<kCol>(G, Bf, K, nw, sc.dt, sc.visc);
  blk_project(G, Bf, K, nw, vx0, vy0, vx, vy);
  blk_advect(vx, vx0, vx0, vy0, S, P, dt0, brk);
  blk_bnd<kRow>(vx, G.code, G.rowfl, G.colfl, S, P);
  blk_advect(vy, vy0, vx0, vy0, S, P, dt0, brk);
  blk_bnd<kCol>(vy, G.code, G.rowfl, G.colfl, S, P);
  blk_project(G, Bf, K, nw, vx, vy, vx0, vy0);
  G.x = scr; G.x0 = de;
  blk_diffuse<kPassive>(G, Bf, K, nw, sc.dt, sc.diff);
  blk_advect(de, scr, vx, vy, S, P, dt0, brk);
  blk_bnd<kPassive>(de, G.code, G.rowfl, G.colfl, S, P);
  blk_copy(scr, de, S, P);
}

// One frame of every scene: persistent blocks draining the scene queue.
__global__ void __launch_bounds__(640, 1) k_batch_frame(BatchArgs A) {
  extern __shared__ __align__(16) float bsm[];
  __shared__ int s_next;
  WBufs Bf;
  Bf.ring = bsm;
  Bf.cs = A.cs;
  float* bufs = A.bufs_in_smem
                    ? bsm + batch_ring_floats(A.nwmax)
                    : A.gscratch + (size_t)blockIdx.x * batch_bufs_floats(A.nwmax, A.cs);
  Bf.carry = bufs;
  Bf.edge = bufs + (size_t)A.nwmax * 2 * A.cs;
  for (;;) {
    if (threadIdx.x == 0) s_next = (int)atomicAdd(A.queue, 1u);
    __syncthreads();
    const int q = s_next;
    __syncthreads();
    if (q >= A.nscenes) break;
    const BScene sc = A.scenes[A.order[q]];
    blk_frame(A, sc, Bf);
  }
}

// A single lin_solve on field `xf` from `x0f` of every scene (a, c shared),
// the same block solver as the frame kernel; used to check the wavefront in
// isolation.
template <int MODE>
__global__ void __launch_bounds__(640, 1) k_batch_lin_solve(BatchArgs A, int xf, int x0f,
                                                            float a, float cr) {
  extern __shared__ __align__(16) float bsm[];
  __shared__ int s_next;
  WBufs Bf;
  Bf.ring = bsm;
  Bf.cs = A.cs;
  float* bufs = A.bufs_in_smem
                    ? bsm + batch_ring_floats(A.nwmax)
                    : A.gscratch + (size_t)blockIdx.x * batch_bufs_floats(A.nwmax, A.cs);
  Bf.carry = bufs;
  Bf.edge = bufs + (size_t)A.nwmax * 2 * A.cs;
  for (;;) {
    if (threadIdx.x == 0) s_next = (int)atomicAdd(A.queue, 1u);
    __syncthreads();
    const int q = s_next;
    __syncthreads();
    if (q >= A.nscenes) break;
    const BScene sc = A.scenes[A.order[q]];
    WGrid G;
    G.x = A.arena + sc.foff + (size_t)xf * sc.fstride;
    G.x0 = A.arena + sc.foff + (size_t)x0f * sc.fstride;
    G.code = A.marena + sc.moff;
    G.rowfl = G.code + sc.fstride;
    G.colfl = G.rowfl + sc.S;
    G.S = sc.S;
    G.P = sc.P;
    wave_lin_solve<MODE>(G, Bf, sc.K, A.nwmax, a, cr);
  }
}

}  // namespace eqk
