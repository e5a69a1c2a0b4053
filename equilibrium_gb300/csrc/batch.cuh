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
#include <type_traits>

#include "common.cuh"
#include "kernels.cuh"
#include "store.cuh"
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
  void* arena;   // fields in the storage format (FP32, FP16 or BF16)
  void* arena2;  // density and scratch (fields 0, 1) when their storage differs
                 // from the velocity fields' (same offsets); else == arena
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
  int nwmax;         // sweeps per wavefront pass (warps per block)
  int cs;            // carry/edge row stride (floats)
  void* stage;       // per-block staging of the wavefront's packed x0 / codes
  unsigned long long stage_stride;  // bytes per block (>= 16 x (dg_size + 3 P), largest scene)
};

// ---- per-cell phases over one scene, by the whole block --------------------
// Cells are visited by anti-diagonals (warp = diagonal, lane = row j), so the
// 32 lanes of a warp touch consecutive addresses. Each lane takes up to kU
// cells of its diagonal per pass and issues all their loads before using
// them (the phases are latency-bound otherwise: one block per scene). Two
// cells a lane keep fewer values live than four (the kernel's 80-register
// cap is shared with the wavefront): 1.3 % faster frames, 8 slower.
constexpr int kU = 2;

// Calls fn(r, i, j, q, ok) for r < kU cells of one diagonal pass; `ok` marks
// the cells that exist. The callers split their work into load and use
// passes over r so that the loads of all kU cells are in flight together.
template <class F>
__device__ __forceinline__ void dg_for_cells(int ilo, int ihi, int jlo, int jhi, int P, F&& fn) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
  for (int d = ilo + jlo + warp; d <= ihi + jhi; d += nwarp) {
    const int j0 = max(jlo, d - ihi), j1 = min(jhi, d - ilo);
    for (int jb = j0 + lane; jb <= j1; jb += 32 * kU) fn(d, jb, j1);
  }
}

template <class STS, class ST>
__device__ __forceinline__ void blk_sources(const BatchArgs& A, const BScene& sc, STS* de,
                                            STS* scr, ST* vx, ST* vy) {
  if (threadIdx.x != 0 || sc.nsrc <= 0) return;
  const int S = sc.S, P = sc.P;
  for (int s = sc.src_off; s < sc.src_off + sc.nsrc; ++s) {  // array order, like k_sources
    const int x = A.src_x[s] > (uint32_t)(S - 1) ? S - 1 : (int)A.src_x[s];
    const int y = A.src_y[s] > (uint32_t)(S - 1) ? S - 1 : (int)A.src_y[s];
    const size_t q = dg_at(x, y, P);
    hs(de, q, fadd(hl(de, q), A.src_d[s]));
    hs(scr, q, fadd(hl(scr, q), A.src_d[s]));
    hs(vx, q, fadd(hl(vx, q), A.src_u[s]));
    hs(vy, q, fadd(hl(vy, q), A.src_v[s]));
  }
}

// set_boundaries (fluid.rs:252-272): the order-independent per-cell map of
// k_set_boundaries, then the corners from post-pass frame values.
template <int MODE, class ST>
__device__ void blk_bnd(ST* __restrict__ x, const uint8_t* __restrict__ code,
                        const uint8_t* rowfl, const uint8_t* colfl, int S, int P) {
  const int N = S - 2;
  if (MODE == kPassive) {
    for (int q = threadIdx.x; q < 4 * N; q += blockDim.x) {
      const int side = q / N, k = q - side * N + 1;
      const int i = side == 0 ? k : (side == 1 ? k : (side == 2 ? 0 : S - 1));
      const int j = side == 0 ? 0 : (side == 1 ? S - 1 : k);
      hs(x, dg_at(i, j, P), dg_frame_after_pass<kPassive>(x, rowfl, colfl, S, P, i, j));
    }
  } else {
    // neighbours: (i+-1, j) at q +- P, (i, j+-1) at q +- (P + 1). Only fluid
    // cells next to a wall are written, from wall cells (never written).
    dg_for_cells(1, N, 1, N, P, [&](int d, int jb, int j1) {
      uint32_t c[kU];
#pragma unroll
      for (int r = 0; r < kU; ++r) {
        const int j = jb + 32 * r;
        c[r] = j <= j1 ? code[(size_t)d * P + j] : 0u;
      }
#pragma unroll
      for (int r = 0; r < kU; ++r) {
        const size_t q = (size_t)d * P + jb + 32 * r;
        // (negation is exact in every storage format)
        if (MODE == kRow) {
          if (c[r] & kCodeRowRight)
            hs(x, q, -hl(x, q + P));
          else if (c[r] & kCodeRowLeft)
            hs(x, q, -hl(x, q - P));
        } else {
          if (c[r] & kCodeColUp)
            hs(x, q, -hl(x, q - P - 1));
          else if (c[r] & kCodeColDown)
            hs(x, q, -hl(x, q + P + 1));
        }
      }
    });
  }
  __syncthreads();
  if (threadIdx.x == 0) dg_corners<MODE, ST>(x, rowfl, colfl, S, P);
  __syncthreads();
}

// project's divergence + zero pressure (fluid.rs:339-352).
// set_boundaries with the mode known at run time.
template <class ST>
__device__ __forceinline__ void blk_bnd_mode(int mode, ST* x, const uint8_t* code,
                                             const uint8_t* rowfl, const uint8_t* colfl, int S,
                                             int P) {
  if (mode == kRow)
    blk_bnd<kRow>(x, code, rowfl, colfl, S, P);
  else if (mode == kCol)
    blk_bnd<kCol>(x, code, rowfl, colfl, S, P);
  else
    blk_bnd<kPassive>(x, code, rowfl, colfl, S, P);
}

template <class ST>
__device__ void blk_divergence(const ST* __restrict__ vx, const ST* __restrict__ vy,
                               ST* __restrict__ p, ST* __restrict__ div, int S, int P) {
  const int N = S - 2;
  dg_for_cells(1, N, 1, N, P, [&](int d, int jb, int j1) {
    float a[kU], b[kU], c[kU], e[kU];
#pragma unroll
    for (int r = 0; r < kU; ++r) {
      const int j = jb + 32 * r;
      const size_t q = (size_t)d * P + (j <= j1 ? j : jb);
      a[r] = hl(vx, q + P);
      b[r] = hl(vx, q - P);
      c[r] = hl(vy, q + P + 1);
      e[r] = hl(vy, q - P - 1);
    }
#pragma unroll
    for (int r = 0; r < kU; ++r) {
      const int j = jb + 32 * r;
      if (j > j1) continue;
      const size_t q = (size_t)d * P + j;
      const float inner = fsub(fadd(fsub(a[r], b[r]), c[r]), e[r]);
      hs(div, q, fdiv(fmul(-0.5f, inner), (float)S));
      hs(p, q, 0.0f);
    }
  });
  __syncthreads();
}

// project's gradient subtraction (fluid.rs:364-371).
template <class ST>
__device__ void blk_gradient(ST* __restrict__ vx, ST* __restrict__ vy,
                             const ST* __restrict__ p, int S, int P) {
  const int N = S - 2;
  const float sf = (float)S;
  dg_for_cells(1, N, 1, N, P, [&](int d, int jb, int j1) {
    float x[kU], y[kU], pr[kU], pl[kU], pd[kU], pu[kU];
#pragma unroll
    for (int r = 0; r < kU; ++r) {
      const int j = jb + 32 * r;
      const size_t q = (size_t)d * P + (j <= j1 ? j : jb);
      x[r] = hl(vx, q);
      y[r] = hl(vy, q);
      pr[r] = hl(p, q + P);
      pl[r] = hl(p, q - P);
      pd[r] = hl(p, q + P + 1);
      pu[r] = hl(p, q - P - 1);
    }
#pragma unroll
    for (int r = 0; r < kU; ++r) {
      const int j = jb + 32 * r;
      if (j > j1) continue;
      const size_t q = (size_t)d * P + j;
      hs(vx, q, fsub(x[r], fmul(fmul(0.5f, fsub(pr[r], pl[r])), sf)));
      hs(vy, q, fsub(y[r], fmul(fmul(0.5f, fsub(pd[r], pu[r])), sf)));
    }
  });
  __syncthreads();
}

template <class ST>
__device__ __forceinline__ float dg_bilerp(const Backtrace& b, const ST* __restrict__ d0,
                                           int P) {
  const float A = hl(d0, dg_at(b.i0, b.j0, P));
  const float B = hl(d0, dg_at(b.i0, b.j1, P));
  const float C = hl(d0, dg_at(b.i1, b.j0, P));
  const float D = hl(d0, dg_at(b.i1, b.j1, P));
  return fadd(fmul(b.s0, fadd(fmul(b.t0, A), fmul(b.t1, B))),
              fmul(b.s1, fadd(fmul(b.t0, C), fmul(b.t1, D))));
}

// advect's first pass (fluid.rs:400-423): every row's first break (the clamped
// backtrace reached size-1), as an atomic minimum per row. `brk` is block
// scratch of >= S ints. A frame's two velocity advects share u, v and so
// share this pass.
template <class ST>
__device__ void blk_advect_breaks(const ST* __restrict__ u, const ST* __restrict__ v,
                                  int S, int P, float dt0, int* brk) {
  const int N = S - 2;
  for (int j = threadIdx.x; j < S; j += blockDim.x) brk[j] = N + 1;
  __syncthreads();
  dg_for_cells(1, N, 1, N, P, [&](int d, int jb, int j1) {
    float uu[kU], vv[kU];
#pragma unroll
    for (int r = 0; r < kU; ++r) {
      const int j = jb + 32 * r;
      const size_t q = (size_t)d * P + (j <= j1 ? j : jb);
      uu[r] = hl(u, q);
      vv[r] = hl(v, q);
    }
#pragma unroll
    for (int r = 0; r < kU; ++r) {
      const int j = jb + 32 * r;
      if (j <= j1 && backtrace(d - j, j, uu[r], vv[r], dt0, S).brk) atomicMin(&brk[j], d - j);
    }
  });
  __syncthreads();
}

// advect's second pass (fluid.rs:378-432): the cells before the row's break
// by bilinear interpolation, the break cell with its left neighbour's new
// value (the old ghost when it is column 1); the cells after it untouched.
template <class SD, class ST>
__device__ void blk_advect_write(SD* __restrict__ d, const SD* __restrict__ d0,
                                 const ST* __restrict__ u, const ST* __restrict__ v,
                                 int S, int P, float dt0, const int* brk) {
  const int N = S - 2;
  dg_for_cells(1, N, 1, N, P, [&](int dd, int jb, int j1) {
    float uu[kU], vv[kU];
    int bj[kU];
#pragma unroll
    for (int r = 0; r < kU; ++r) {
      const int j = jb + 32 * r;
      const int jj = j <= j1 ? j : jb;
      const int i = dd - jj;
      bj[r] = brk[jj];
      // the break cell copies its left neighbour's value: backtrace (i-1, j)
      const size_t qc = (size_t)dd * P + jj - (i == bj[r] ? P : 0);
      uu[r] = hl(u, qc);
      vv[r] = hl(v, qc);
    }
    Backtrace bt[kU];
#pragma unroll
    for (int r = 0; r < kU; ++r) {
      const int j = jb + 32 * r;
      const int jj = j <= j1 ? j : jb;
      const int i = dd - jj;
      bt[r] = backtrace(i == bj[r] ? i - 1 : i, jj, uu[r], vv[r], dt0, S);
    }
    float val[kU];
#pragma unroll
    for (int r = 0; r < kU; ++r) val[r] = dg_bilerp(bt[r], d0, P);
#pragma unroll
    for (int r = 0; r < kU; ++r) {
      const int j = jb + 32 * r;
      const int i = dd - j;
      if (j > j1 || i > bj[r]) continue;
      const size_t q = (size_t)dd * P + j;
      if (i == bj[r] && i == 1) val[r] = hl(d, q - P);  // d[0, j]: column 0 is never written here
      hs(d, q, val[r]);
    }
  });
  __syncthreads();
}

// scratch_space = density.clone() (fluid.rs:523) over every cell.
template <class ST>
__device__ void blk_copy(ST* __restrict__ dst, const ST* __restrict__ src, int S, int P) {
  dg_for_cells(0, S - 1, 0, S - 1, P, [&](int d, int jb, int j1) {
    ST t[kU];
#pragma unroll
    for (int r = 0; r < kU; ++r) {
      const int j = jb + 32 * r;
      t[r] = src[(size_t)d * P + (j <= j1 ? j : jb)];
    }
#pragma unroll
    for (int r = 0; r < kU; ++r) {
      const int j = jb + 32 * r;
      if (j <= j1) dst[(size_t)d * P + j] = t[r];
    }
  });
  __syncthreads();
}

// ---- operation lists ---------------------------------------------------------
// A launch runs a short list of operations on every scene; one frame
// (Fluid::step, fluid.rs:437-524, with the reference's aliasing of the six
// arrays) is the list built by batch_frame_ops. The scene descriptor is kept
// in shared memory and re-read after every operation, so nothing but the
// operation index is live across a wavefront solve.
enum : int {
  kOpSources = 0,   // add_density / add_velocity of the scene's sources
  kOpDiffuse,       // f[0] = x, f[1] = x0, a = 0: viscosity, 1: diffusion, 2: `c0` given
  kOpLinSolve,      // f[0] = x, f[1] = x0, coefficients a, c given
  kOpDivergence,    // f = vx, vy, p, div: div + p = 0, bnd(Passive) of div and p
  kOpGradient,      // f = vx, vy, p: gradient subtraction, bnd(Row) vx, bnd(Col) vy
  kOpAdvectBreaks,  // f[0] = u, f[1] = v: every row's first break
  kOpAdvectWrite,   // f = d, d0, u, v (breaks of u, v computed before), then bnd(mode) d
  kOpBnd,           // f[0]
  kOpCopy,          // f[0] = f[1]
};

struct BOp {
  int kind, mode;
  int f[4];
  int coef;    // kOpDiffuse: 0 viscosity, 1 diffusion, 2 use `a` as the diffusion
  float a, c;  // kOpLinSolve coefficients (kOpDiffuse with coef 2: a = diffusion)
};

constexpr int kMaxOps = 16;
struct BOpList {
  int n;
  BOp op[kMaxOps];
};

template <class ST>
__device__ __forceinline__ ST* bfield(const BatchArgs& A, const BScene& sc, int f) {
  return static_cast<ST*>(A.arena) + sc.foff + (size_t)f * sc.fstride;
}
// density (1) and scratch (0) in their own storage format (arena2 only when
// it differs from the velocity fields')
template <class STS, class ST>
__device__ __forceinline__ STS* bscalar(const BatchArgs& A, const BScene& sc, int f) {
  if constexpr (std::is_same<ST, STS>::value) return bfield<ST>(A, sc, f);
  return static_cast<STS*>(A.arena2) + sc.foff + (size_t)f * sc.fstride;
}

// One operation on the scene in shared memory. ST: the velocity fields'
// storage; STS: density and scratch's (fields 0 and 1; the op list never
// mixes the two kinds in one solve, copy or advected pair).
template <class ST, class STS>
__device__ __forceinline__ void blk_op(const BatchArgs& A, const BScene* ssc, const BOp& op,
                                       const WBufs& Bf, int* brk) {
  const BScene& sc = *ssc;
  constexpr bool kApart = !std::is_same<ST, STS>::value;
  const int S = sc.S, P = sc.P;
  const uint8_t* code = A.marena + sc.moff;
  const uint8_t* rowfl = code + sc.fstride;
  const uint8_t* colfl = rowfl + S;
  const float dt0 = fmul(sc.dt, (float)(S - 2));
  WGrid<ST> G;
  G.code = code;
  G.rowfl = rowfl;
  G.colfl = colfl;
  G.stage = static_cast<char*>(A.stage) + (size_t)blockIdx.x * A.stage_stride;
  G.S = S;
  G.P = P;
  switch (op.kind) {
    case kOpSources:
      blk_sources(A, sc, bscalar<STS, ST>(A, sc, 1), bscalar<STS, ST>(A, sc, 0), bfield<ST>(A, sc, 2), bfield<ST>(A, sc, 3));
      __syncthreads();
      break;
    case kOpDiffuse:
    case kOpLinSolve: {
      float a, cr;
      if (op.kind == kOpDiffuse) {
        // diffuse (fluid.rs:276-298): a = ((dt*diff)*sf)*sf, c = 1 + 4a
        const float dif = op.coef == 0 ? sc.visc : (op.coef == 1 ? sc.diff : op.a);
        const float sf = (float)(S - 2);
        a = fmul(fmul(fmul(sc.dt, dif), sf), sf);
        cr = fdiv(1.0f, fadd(1.0f, fmul(4.0f, a)));
      } else {
        a = op.a;
        cr = fdiv(1.0f, op.c);
      }
      if (kApart && op.f[0] < 2) {  // density diffusion: the scalar fields
        WGrid<STS> H;
        H.code = code;
        H.rowfl = rowfl;
        H.colfl = colfl;
        H.stage = G.stage;
        H.S = S;
        H.P = P;
        H.x = bscalar<STS, ST>(A, sc, op.f[0]);
        H.x0 = bscalar<STS, ST>(A, sc, op.f[1]);
        if (op.mode == kRow)
          wave_lin_solve<kRow, STS>(H, Bf, sc.K, A.nwmax, a, cr);
        else if (op.mode == kCol)
          wave_lin_solve<kCol, STS>(H, Bf, sc.K, A.nwmax, a, cr);
        else
          wave_lin_solve<kPassive, STS>(H, Bf, sc.K, A.nwmax, a, cr);
        break;
      }
      G.x = bfield<ST>(A, sc, op.f[0]);
      G.x0 = bfield<ST>(A, sc, op.f[1]);
      if (op.mode == kRow)
        wave_lin_solve<kRow, ST>(G, Bf, sc.K, A.nwmax, a, cr);
      else if (op.mode == kCol)
        wave_lin_solve<kCol, ST>(G, Bf, sc.K, A.nwmax, a, cr);
      else
        wave_lin_solve<kPassive, ST>(G, Bf, sc.K, A.nwmax, a, cr);
      break;
    }
    case kOpDivergence: {
      ST* p = bfield<ST>(A, sc, op.f[2]);
      ST* div = bfield<ST>(A, sc, op.f[3]);
      blk_divergence(bfield<ST>(A, sc, op.f[0]), bfield<ST>(A, sc, op.f[1]), p, div, S, P);
      blk_bnd<kPassive>(div, code, rowfl, colfl, S, P);
      blk_bnd<kPassive>(p, code, rowfl, colfl, S, P);
      break;
    }
    case kOpGradient: {
      ST* vx = bfield<ST>(A, sc, op.f[0]);
      ST* vy = bfield<ST>(A, sc, op.f[1]);
      blk_gradient(vx, vy, bfield<ST>(A, sc, op.f[2]), S, P);
      blk_bnd<kRow>(vx, code, rowfl, colfl, S, P);
      blk_bnd<kCol>(vy, code, rowfl, colfl, S, P);
      break;
    }
    case kOpAdvectBreaks:
      blk_advect_breaks(bfield<ST>(A, sc, op.f[0]), bfield<ST>(A, sc, op.f[1]), S, P, dt0, brk);
      break;
    case kOpAdvectWrite: {
      if (kApart && op.f[0] < 2) {  // density advected from scratch
        STS* d = bscalar<STS, ST>(A, sc, op.f[0]);
        blk_advect_write(d, bscalar<STS, ST>(A, sc, op.f[1]), bfield<ST>(A, sc, op.f[2]),
                         bfield<ST>(A, sc, op.f[3]), S, P, dt0, brk);
        blk_bnd_mode(op.mode, d, code, rowfl, colfl, S, P);
        break;
      }
      ST* d = bfield<ST>(A, sc, op.f[0]);
      blk_advect_write(d, bfield<ST>(A, sc, op.f[1]), bfield<ST>(A, sc, op.f[2]),
                       bfield<ST>(A, sc, op.f[3]), S, P, dt0, brk);
      blk_bnd_mode(op.mode, d, code, rowfl, colfl, S, P);
      break;
    }
    case kOpBnd:
      if (kApart && op.f[0] < 2)
        blk_bnd_mode(op.mode, bscalar<STS, ST>(A, sc, op.f[0]), code, rowfl, colfl, S, P);
      else
        blk_bnd_mode(op.mode, bfield<ST>(A, sc, op.f[0]), code, rowfl, colfl, S, P);
      break;
    case kOpCopy:
      if (kApart && op.f[0] < 2)
        blk_copy(bscalar<STS, ST>(A, sc, op.f[0]), bscalar<STS, ST>(A, sc, op.f[1]), S, P);
      else
        blk_copy(bfield<ST>(A, sc, op.f[0]), bfield<ST>(A, sc, op.f[1]), S, P);
      break;
    default:
      break;
  }
}

// Shared-memory layout of a batch block (offsets in floats).
__device__ __forceinline__ WBufs batch_bufs(const BatchArgs& A) {
  WBufs Bf;
  Bf.cs = A.cs;
  Bf.ring = 0;
  Bf.carry = A.nwmax * 32 * kWRS;
  Bf.edge = Bf.carry + A.nwmax * 2 * A.cs;
  return Bf;
}

// The operation list on every scene: persistent blocks draining the scene
// queue (one launch = one frame when L is the frame's list). ST: the velocity
// fields' storage, STS: density and scratch's.
template <class ST, class STS = ST>
__global__ void __launch_bounds__(672, 1) k_batch_run(BatchArgs A, BOpList L) {
  extern __shared__ __align__(16) float bsm[];
  __shared__ int s_next;
  __shared__ BScene s_sc;
  const WBufs Bf = batch_bufs(A);
  int* brk = reinterpret_cast<int*>(bsm + Bf.edge);  // edge rows are free between solves
  for (;;) {
    if (threadIdx.x == 0) {
      const int q = (int)atomicAdd(A.queue, 1u);
      s_next = q;
      if (q < A.nscenes) s_sc = A.scenes[A.order[q]];
    }
    __syncthreads();
    const int q = s_next;
    if (q >= A.nscenes) break;
    for (int k = 0; k < L.n; ++k) blk_op<ST, STS>(A, &s_sc, L.op[k], Bf, brk);
    __syncthreads();
  }
}

// One field of every scene, dense (size x size, row-major) and in scene
// order, from the arena's anti-diagonal layout: block s copies scene s to
// out + doff[s].
template <class ST>
__global__ void k_batch_gather_dense(const ST* __restrict__ arena, const BScene* __restrict__ sc,
                                     const unsigned long long* __restrict__ doff, int field,
                                     float* __restrict__ out) {
  const BScene d = sc[blockIdx.x];
  const ST* src = arena + d.foff + (size_t)field * d.fstride;
  float* dst = out + doff[blockIdx.x];
  const int S = d.S, P = d.P;
  const size_t n = (size_t)S * S;
  for (size_t q = threadIdx.x; q < n; q += blockDim.x) {
    const int j = (int)(q / S), i = (int)(q - (size_t)j * S);
    dst[q] = hl(src, dg_at(i, j, P));
  }
}

// The frame kernel's instances are compiled in batch_kernels.cu (one
// translation unit per storage format, built in parallel); every other
// includer only declares them.
#ifndef EQ_BATCH_KERNELS_TU
extern template __global__ void k_batch_run<float, float>(BatchArgs, BOpList);
extern template __global__ void k_batch_run<__half, __half>(BatchArgs, BOpList);
extern template __global__ void k_batch_run<__nv_bfloat16, __nv_bfloat16>(BatchArgs, BOpList);
extern template __global__ void k_batch_run<float, __half>(BatchArgs, BOpList);
#endif

}  // namespace eqk
