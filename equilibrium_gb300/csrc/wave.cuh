// lin_solve (fluid.rs:301-325) for ONE grid inside ONE thread block: a
// temporal wavefront in which warp w performs Gauss-Seidel sweep w of a pass,
// bit-exactly.
//
// Geometry. A task is (strip t, sweep k); lane l of the warp of sweep k owns
// row  j = 32 t + l - 2 k - 2  (strips skewed by two rows per sweep, so a
// task only depends on (t, k-1) and (t-1, k)) and at step tau of the task
// updates column  i = tau + 1 - l  (lane l lags lane l-1 by one column, so the
// value (i, j-1) of the same sweep is lane l-1's previous result). The sweep-k
// value of an interior cell is
//   G(i,j) = (x0 + a*(((R + L) + D) + U)) * (1/c)
// with L = G(i-1, j) (own register), U = G(i, j-1) (shuffle from lane l-1;
// lane 0 reads the previous strip's lane 31 from a per-warp edge row),
// R = W(k-1)[i+1, j], D = W(k-1)[i, j+1], where W(k) is the grid after sweep k
// AND its set_boundaries. A cell that the sweep does not update (frame rows,
// ghost columns, rows outside the grid) passes its W(k-1) value on as G.
//
// Hand-off between sweeps. Lane l writes W(k)[i-1, j] at step tau (one step
// late: its post-boundary value may need G(i, j) or G(i-1, j+1)). Warp k+1
// reads W(k) rows j and j+1 of lane l at the SAME step index, so the data
// travel through a two-chunk shared-memory ring per warp, indexed by step
// (slot = tau mod 2Q; the lane stride 2Q+1 keeps the 32 lanes on 32 banks).
// The two rows of warp k+1's lanes 0 and 1 come from warp k's PREVIOUS strip
// (its lanes 30 and 31): those lanes also write a per-warp "carry" row pair
// indexed by column. Warp 0 reads W(-1) = x directly from global memory and
// the last warp writes the final sweep straight into x (in place: every read
// of W(-1) happens before the last sweep overwrites that cell; a lane reads
// its own row's column i+1 before writing column i-1).
//
// Boundary fix-ups (set_boundaries after every sweep, fluid.rs:252-272,
// fused): AdjustRow takes -G(i+1) (right wall wins) else -G(i-1); AdjustColumn
// takes -G(i, j-1) (up wall wins) else -G(i, j+1) (lane l+1's value, by
// shuffle). Lane 31's "down" neighbour lives in the next strip, whose lane 0
// writes the fix-up into the carry row (or into x for the last sweep) before
// anything reads it. Passive copies row 1 / row N into the frame rows and
// columns 1 / N into the ghost columns where that row / column holds a fluid
// cell. Corners are computed once after the last sweep: no sweep reads them.
//
// Schedule. All warps advance in lockstep, one chunk of Q steps per
// __syncthreads: at super-step s warp w processes chunk g = s - w of its task
// stream, so what warp w wrote at super-step s is read by warp w+1 at s+1.
// No flags, no spin waits: the only synchronisation is the block barrier.
#pragma once
#include "common.cuh"
#include "kernels.cuh"
#include "store.cuh"

namespace eqk {

constexpr int kWQ = 16;            // steps per chunk
constexpr int kWRS = 2 * kWQ + 1;  // ring lane stride (floats)

// Anti-diagonal ("skewed") grid layout: cell (i, j) of an S x S grid lives at
// (i + j) * P + j, P = S rounded up to 32, 2S - 1 diagonals. A wavefront step
// touches cells (tau + 1 - l, j0 + l) of one anti-diagonal, which are
// consecutive in memory, so every per-lane stream (x0, codes, the first
// sweep's reads and the last sweep's writes) is a coalesced access.
__host__ __device__ inline size_t dg_at(int i, int j, int P) { return (size_t)(i + j) * P + j; }
__host__ __device__ inline size_t dg_size(int S, int P) { return (size_t)(2 * S - 1) * P; }

// set_boundaries' corners (fluid.rs:254-271) on a diagonal-layout grid, from
// the post-pass values of the frame (the rest of the pass is done).
template <int MODE, class ST>
__device__ __forceinline__ float dg_frame_after_pass(const ST* x, const uint8_t* rowfl,
                                                     const uint8_t* colfl, int S, int P, int i,
                                                     int j) {
  if (MODE == kPassive) {
    if (j == 0 && colfl[i]) return hl(x, dg_at(i, 1, P));
    if (j == S - 1 && colfl[i]) return hl(x, dg_at(i, S - 2, P));
    if (i == 0 && rowfl[j]) return hl(x, dg_at(1, j, P));
    if (i == S - 1 && rowfl[j]) return hl(x, dg_at(S - 2, j, P));
  }
  return hl(x, dg_at(i, j, P));
}

template <int MODE, class ST>
__device__ __forceinline__ void dg_corners(ST* x, const uint8_t* rowfl, const uint8_t* colfl,
                                           int S, int P) {
  auto f = [&](int i, int j) { return dg_frame_after_pass<MODE>(x, rowfl, colfl, S, P, i, j); };
  const float c00 = fmul(0.5f, fadd(f(1, 0), f(0, 1)));
  const float c0S = fmul(0.5f, fadd(f(1, S - 1), f(0, S - 2)));
  const float cS0 = fmul(0.5f, fadd(f(S - 2, 0), f(S - 1, 1)));
  const float cSS = fmul(0.5f, fadd(f(S - 2, S - 1), f(S - 1, S - 2)));
  hs(x, dg_at(0, 0, P), c00);
  hs(x, dg_at(0, S - 1, P), c0S);
  hs(x, dg_at(S - 1, 0, P), cS0);
  hs(x, dg_at(S - 1, S - 1, P), cSS);
}

// Shared-memory accesses through 32-bit shared-window addresses (half the
// registers of generic pointers; ptxas folds the per-step offsets).
__device__ __forceinline__ float lds_f32(uint32_t a) {
  float v;
  asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ void sts_f32(uint32_t a, float v) {
  asm volatile("st.shared.f32 [%0], %1;" ::"r"(a), "f"(v) : "memory");
}
// A load only where `on` (else 0), and a store only where `on`: the
// predicate sits inside the instruction, so the lanes that skip it take no
// branch around it.
__device__ __forceinline__ float lds_f32_if(uint32_t a, bool on) {
  float v;
  asm volatile(
      "{ .reg .pred q; setp.ne.b32 q, %2, 0; mov.f32 %0, 0f00000000; @q ld.shared.f32 %0, [%1]; }"
      : "=f"(v)
      : "r"(a), "r"((int)on)
      : "memory");
  return v;
}
__device__ __forceinline__ void sts_f32_if(uint32_t a, float v, bool on) {
  asm volatile("{ .reg .pred q; setp.ne.b32 q, %2, 0; @q st.shared.f32 [%0], %1; }" ::"r"(a), "f"(v),
               "r"((int)on)
               : "memory");
}

// One scene grid as the block solver sees it (diagonal layout; fields in
// storage format ST, arithmetic in FP32).
template <class ST>
struct WGrid {
  ST* x;
  const ST* x0;
  const uint8_t* code;   // boundary codes, diagonal layout
  const uint8_t* rowfl;  // [S]
  const uint8_t* colfl;  // [S]
  void* stage;           // the block's staging: (2 S + 2) P 16-byte packed words, see WPack
  int S, P;
};

// x0 and the boundary codes of W consecutive cells of a row (columns i ..
// i+W-1) in one 16-byte word, so that a lane loads a group of W steps'
// operands in one load instead of 2 W (each global load of a sweep
// warp delays the shared-memory loads issued after it): FP32 as two values
// and their codes, 16-bit formats as four (bits | code << 16). The raw bits
// are kept, so the values are those of the field; columns outside the grid
// hold zeros.
template <class ST>
struct WPack;
template <>
struct WPack<float> {
  static constexpr int W = 2;
  // the word of cell (i, j): cells (i + w, j) at (i + w + j) P + j
  static __device__ __forceinline__ uint4 make(const float* x0, const uint8_t* code, int i, int j,
                                               int S, int P) {
    uint32_t v[2], c = 0u;
#pragma unroll
    for (int w = 0; w < 2; ++w) {
      const bool ok = i + w >= 0 && i + w <= S - 1;
      const size_t q = ok ? (size_t)(i + w + j) * P + j : 0;
      v[w] = ok ? __float_as_uint(x0[q]) : 0u;
      c |= (ok ? (uint32_t)code[q] : 0u) << (8 * w);
    }
    return make_uint4(v[0], v[1], c, 0u);
  }
  static __device__ __forceinline__ float x(const uint4& e, int w) {
    return __uint_as_float(w == 0 ? e.x : e.y);
  }
  static __device__ __forceinline__ uint32_t c(const uint4& e, int w) {
    return (e.z >> (8 * w)) & 0xffu;
  }
};
template <class H>
struct Bits16;
template <>
struct Bits16<__half> {
  static __device__ __forceinline__ unsigned short get(__half v) { return __half_as_ushort(v); }
  static __device__ __forceinline__ float widen(unsigned short b) {
    return __half2float(__ushort_as_half(b));
  }
};
template <>
struct Bits16<__nv_bfloat16> {
  static __device__ __forceinline__ unsigned short get(__nv_bfloat16 v) {
    return __bfloat16_as_ushort(v);
  }
  static __device__ __forceinline__ float widen(unsigned short b) {
    return __bfloat162float(__ushort_as_bfloat16(b));
  }
};
template <class H>
struct WPack16 {
  static constexpr int W = 4;
  static __device__ __forceinline__ uint4 make(const H* x0, const uint8_t* code, int i, int j,
                                               int S, int P) {
    uint32_t v[4];
#pragma unroll
    for (int w = 0; w < 4; ++w) {
      const bool ok = i + w >= 0 && i + w <= S - 1;
      const size_t q = ok ? (size_t)(i + w + j) * P + j : 0;
      v[w] = ok ? ((uint32_t)Bits16<H>::get(x0[q]) | ((uint32_t)code[q] << 16)) : 0u;
    }
    return make_uint4(v[0], v[1], v[2], v[3]);
  }
  static __device__ __forceinline__ float x(const uint4& e, int w) {
    const uint32_t v = w == 0 ? e.x : (w == 1 ? e.y : (w == 2 ? e.z : e.w));
    return Bits16<H>::widen((unsigned short)(v & 0xffffu));
  }
  static __device__ __forceinline__ uint32_t c(const uint4& e, int w) {
    const uint32_t v = w == 0 ? e.x : (w == 1 ? e.y : (w == 2 ? e.z : e.w));
    return v >> 16;
  }
};
template <>
struct WPack<__half> : WPack16<__half> {};
template <>
struct WPack<__nv_bfloat16> : WPack16<__nv_bfloat16> {};

// Block-private buffers, all in the block's dynamic shared memory, given as
// float offsets from its start: the rings [nwmax][32][kWRS] (ring[w] is
// written by warp w: the loader warp 0 or sweep warp w), the carry rows
// [nwmax][2][cs] (carry[w] is written by warp w) and the sweep warps' edge
// rows [nwmax][cs].
struct WBufs {
  int ring, carry, edge;
  int cs;  // row stride of carry / edge, >= S
};

__host__ __device__ inline size_t wave_smem_floats(int nwmax, int cs) {
  return (size_t)nwmax * 32 * kWRS + (size_t)nwmax * 3 * cs;
}

// Strips per pass: every sweep k < nw must cover rows 0..S-1, and lane 31 of
// the last strip must never hold an interior row (its fix-up would need a
// strip that does not exist): 32 (B-1) + 29 - 2 (nw-1) >= S - 1.
__host__ __device__ inline int wave_strips(int S, int nw) { return (S + 2 * nw - 1) / 32 + 1; }
__host__ __device__ inline int wave_chunks(int S) { return (S + 31 + kWQ - 1) / kWQ; }

// Steps per load group (x0 / codes prefetched one group ahead): one packed
// word. Two-step groups for FP32 keep fewer values live than two words of a
// four-step group (fewer spills under the 80-register cap; 3 % faster).
template <class ST>
__host__ __device__ constexpr int wave_group() { return WPack<ST>::W; }
static_assert(kWQ % WPack<float>::W == 0 && kWQ % WPack<__half>::W == 0,
              "a chunk holds whole load groups");

struct WLaneState {
  float g1, g2, u1, rm1;
  float h0, h1;  // carry columns 0 / 1 of lanes 30 / 31, written at the task's end
  uint32_t c1;
};

// Per-task, per-lane constants. Grid rows of the diagonal layout are given as
// a base with column i at base[i * P]; shared rows are 32-bit shared-window
// byte addresses, column- or slot-indexed with stride 4 bytes.
template <class ST>
struct WTask {
  ST* gout;        // last sweep: x row j, global
  ST* gfix;           // last sweep: x row j-1 (AdjustColumn fix-up), global
  const uint4* pkrow;  // packed x0 / codes of row j: columns i .. i+W-1 at [i * P]
  uint32_t sr, sd;    // other sweeps: R / D source (ring lane, slot-indexed, or carry row)
  uint32_t sout;      // other sweeps: this lane's ring row (slot-indexed)
  uint32_t scarry;    // lanes 30/31 of a non-last sweep: carry row (0 = none)
  uint32_t sfix;      // non-last sweep, lane 0: carry row 1 (column-indexed)
  uint32_t sedge;     // this warp's edge row (column-indexed)
  bool rring, dring;  // R / D source indexed by ring slot (else by column)
  bool valid, interior, top, bot, rowfl;
};

// x0 and codes of columns ib..ib+W-1 of this lane's row, one packed load
// (EDGE: only when the word holds a column inside the grid; else zeros).
// Plain (coherent) loads: the block wrote the staging at the solve's start.
template <bool EDGE, class ST>
__device__ __forceinline__ void wave_prefetch(const WTask<ST>& T, int ib, int S, int P,
                                              float (&x)[wave_group<ST>()],
                                              uint32_t (&c)[wave_group<ST>()]) {
  constexpr int W = WPack<ST>::W;
  uint4 e = make_uint4(0u, 0u, 0u, 0u);
  if (!EDGE || (ib + W - 1 >= 0 && ib <= S - 1)) e = T.pkrow[(ptrdiff_t)ib * P];
#pragma unroll
  for (int w = 0; w < W; ++w) {
    x[w] = WPack<ST>::x(e, w);
    c[w] = WPack<ST>::c(e, w);
  }
}

template <int MODE, bool EDGE, bool LAST, class ST>
__device__ __forceinline__ void wave_chunk(const WTask<ST>& T, WLaneState& st, int lane, int tau0,
                                           int half, int S, int P, float a, float cr,
                                           bool next_in_task, bool next_edge) {
  const unsigned FULL = 0xffffffffu;
  const int N = S - 2;
  const int ib = tau0 + 1 - lane;  // column at q = 0
  // R / D / out streams at q = 0
  const uint32_t sR = T.sr + 4u * (uint32_t)(T.rring ? half : ib + 1);
  const uint32_t sD = T.sd + 4u * (uint32_t)(T.dring ? half : ib);
  ST* gO = LAST ? T.gout + (ptrdiff_t)(ib - 1) * P : nullptr;
  const uint32_t sO = T.sout + 4u * (uint32_t)half;
  constexpr int kWG = wave_group<ST>();
  float xa[kWG];
  uint32_t ca[kWG];
  wave_prefetch<EDGE>(T, ib, S, P, xa, ca);

#pragma unroll
  for (int q0 = 0; q0 < kWQ; q0 += kWG) {
    float Xv[kWG];
    uint32_t Cv[kWG];
#pragma unroll
    for (int r = 0; r < kWG; ++r) {
      Xv[r] = xa[r];
      Cv[r] = ca[r];
    }
    // This group's shared-memory operands first, then the next group's x0 /
    // codes: a warp's shared loads return in order behind its global loads,
    // so a shared load issued after the prefetch would wait for it; issued
    // before, the prefetch overlaps this group's arithmetic instead.
    float Rv[kWG], Dv[kWG], Ev[kWG];
#pragma unroll
    for (int r = 0; r < kWG; ++r) {
      const int q = q0 + r;
      const int i = ib + q;
      if (EDGE) {
        const bool okR = T.rring || (i + 1 >= 0 && i + 1 <= S - 1);
        const bool okD = T.dring || (i >= 0 && i <= S - 1);
        const bool okI = (i >= 0 && i <= S - 1);
        Rv[r] = lds_f32_if(sR + 4u * q, okR);
        Dv[r] = lds_f32_if(sD + 4u * q, okD);
        Ev[r] = lds_f32_if(T.sedge + 4u * (uint32_t)i, lane == 0 && okI);
      } else {
        Rv[r] = lds_f32(sR + 4u * q);
        Dv[r] = lds_f32(sD + 4u * q);
        Ev[r] = lds_f32(T.sedge + 4u * (uint32_t)i);
      }
    }
    if (q0 + kWG < kWQ) wave_prefetch<EDGE>(T, ib + q0 + kWG, S, P, xa, ca);
#pragma unroll
    for (int r = 0; r < kWG; ++r) {
      const int q = q0 + r;
      const int i = ib + q;
      float U = __shfl_up_sync(FULL, st.g1, 1);
      if (lane == 0) U = Ev[r];
      const float R = Rv[r];
      const float gc = fmul(fadd(Xv[r], fmul(a, fadd(fadd(fadd(R, st.g1), Dv[r]), U))), cr);
      const bool act = EDGE ? (T.interior && i >= 1 && i <= N) : T.interior;
      const float g = act ? gc : st.rm1;
      const float gdn = __shfl_down_sync(FULL, g, 1);

      // post-boundary value of column i-1
      const uint32_t c1 = st.c1;
      float val;
      if (MODE == kRow) {
        val = (c1 & kCodeRowRight) ? -g : ((c1 & kCodeRowLeft) ? -st.g2 : st.g1);
      } else if (MODE == kCol) {
        val = (c1 & kCodeColUp) ? -st.u1 : ((c1 & kCodeColDown) ? -gdn : st.g1);
      } else {
        const bool cf = (c1 & kCodeColFluid) != 0;
        val = (T.top && cf) ? gdn : ((T.bot && cf) ? st.u1 : st.g1);
        if (EDGE && T.interior) {
          if (i - 1 == 0) val = T.rowfl ? g : st.g1;
          if (i - 1 == S - 1) val = T.rowfl ? st.g2 : st.g1;
        }
      }
      const bool colok = EDGE ? (i - 1 >= 0 && i - 1 <= S - 1) : true;
      if (LAST) {
        if (T.valid && colok) hs(gO, (ptrdiff_t)q * P, val);
      } else {
        sts_f32_if(sO + 4u * q, val, colok);
        if (EDGE && tau0 < 2 * kWQ) {
          // Columns 0 / 1 of the carry rows are produced in chunk 1, the
          // super-step in which the next warp still reads the previous strip's
          // columns 0 / 1; they are held back and written when the task ends.
          if (T.scarry && colok) {
            if (i - 1 == 0) st.h0 = val;
            if (i - 1 == 1) st.h1 = val;
          }
        } else {
          sts_f32_if(T.scarry + 4u * (uint32_t)(i - 1), val, T.scarry && colok);
        }
      }
      sts_f32_if(T.sedge + 4u * (uint32_t)i, g,
                 lane == 31 && (EDGE ? (i >= 0 && i <= S - 1) : true));
      // (a lane whose row lies outside the grid reads a clamped row's code)
      const bool fixc = MODE == kCol && lane == 0 && T.valid && (Cv[r] & kCodeAboveDown) &&
                        (EDGE ? (i >= 1 && i <= N) : true);
      if (LAST) {
        if (fixc) hs(T.gfix, (ptrdiff_t)i * P, -g);
      } else if (MODE == kCol) {
        sts_f32_if(T.sfix + 4u * (uint32_t)i, -g, fixc);
      }

      st.g2 = st.g1;
      st.g1 = g;
      st.u1 = U;
      st.rm1 = R;
      st.c1 = Cv[r];
    }
  }
}

template <int MODE, bool LAST, class ST>
__device__ __forceinline__ void wave_chunk_any(const WTask<ST>& T, WLaneState& st, int lane, int c,
                                               int NCH, int half, int S, int P, float a,
                                               float cr) {
  const int N = S - 2;
  const int tau0 = c * kWQ;
  const bool fast = (tau0 >= 32) && (tau0 + kWQ <= N);
  const bool next_in_task = c + 1 < NCH;
  const bool next_edge = !((tau0 + kWQ >= 32) && (tau0 + 2 * kWQ <= N));
  if (fast)
    wave_chunk<MODE, false, LAST, ST>(T, st, lane, tau0, half, S, P, a, cr, next_in_task,
                                      next_edge);
  else
    wave_chunk<MODE, true, LAST, ST>(T, st, lane, tau0, half, S, P, a, cr, next_in_task,
                                     next_edge);
}

// `K` sweeps of lin_solve on grid G by the whole block (blockDim.x = 32 *
// (nwmax + 1): a loader warp and one warp per sweep of a pass), passes of at
// most nwmax sweeps. Ends with a block barrier; the result (corners included)
// is in G.x.
template <int MODE, class ST>
__device__ __noinline__ void wave_lin_solve(const WGrid<ST> G, const WBufs Bf, int K, int nwmax,
                                            float a, float cr) {
  if (K <= 0) return;
  extern __shared__ __align__(16) float wave_smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;  // warp 0: loader
  const int S = G.S, P = G.P, N = S - 2;
  const int NCH = wave_chunks(S);
  const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(wave_smem);
  const uint32_t ring = sbase + 4u * Bf.ring;
  const uint32_t carry = sbase + 4u * Bf.carry;
  const uint32_t edge = sbase + 4u * Bf.edge;
  const uint32_t cs4 = 4u * Bf.cs;
  constexpr uint32_t kLane4 = 4u * kWRS, kWarp4 = 32u * 4u * kWRS;
  // x0 and the codes of every row into the block's staging, packed: the word
  // of cell (i, j), i = -(W-1) .. S-1, at (i + W - 1 + j) P + j (the diagonal
  // layout shifted by W - 1 columns; warp = anti-diagonal, lane = row)
  constexpr int W = WPack<ST>::W;
  uint4* const pk = static_cast<uint4*>(G.stage);
  for (int d = warp; d <= 2 * S - 2 + (W - 1); d += (int)(blockDim.x >> 5)) {
    const int j0 = max(0, d - (S - 1) - (W - 1)), j1 = min(d, S - 1);
    for (int j = j0 + lane; j <= j1; j += 32) {
      pk[(size_t)d * P + j] = WPack<ST>::make(G.x0, G.code, d - (W - 1) - j, j, S, P);
    }
  }
  __syncthreads();
  for (int k0 = 0; k0 < K; k0 += nwmax) {
    const int nw = min(nwmax, K - k0);
    const int B = wave_strips(S, nw);
    const int ntask = B * NCH;
    const int nsup = ntask + nw;
    if (warp == 0) {
      // ---- loader: W(-1) = x into ring 0 (and carry 0 for lanes 30/31), row
      // j = 32 t + l, column tau - l at step tau; loads one chunk ahead.
      float xs[kWQ];
      float h0 = 0.0f, h1 = 0.0f;
      auto load_chunk = [&](int gg) {
        const int t = gg / NCH, c = gg - t * NCH;
        const int j = 32 * t + lane;
        const bool rowok = j >= 0 && j <= S - 1;
        const int jc = rowok ? j : 0;
        const ST* base = G.x + (size_t)jc * P + jc;
#pragma unroll
        for (int q = 0; q < kWQ; ++q) {
          const int is = c * kWQ + q - lane;
          xs[q] = (rowok && is >= 0 && is <= S - 1) ? hl(base, (ptrdiff_t)is * P) : 0.0f;
        }
      };
      load_chunk(0);
      for (int s = 0; s < nsup; ++s) {
        if (s < ntask) {
          const int t = s / NCH, c = s - t * NCH;
          const int tau0 = c * kWQ;
          const uint32_t sO = ring + (uint32_t)lane * kLane4 + 4u * (uint32_t)((s & 1) * kWQ);
          const uint32_t sC = carry + (uint32_t)(lane - 30) * cs4;
#pragma unroll
          for (int q = 0; q < kWQ; ++q) {
            sts_f32(sO + 4u * q, xs[q]);
            const int is = tau0 + q - lane;
            const bool carried = lane >= 30 && is >= 0 && is <= S - 1;
            if (tau0 < 2 * kWQ) {  // held back: see the sweep warps' carry rows
              if (carried && is == 0) h0 = xs[q];
              if (carried && is == 1) h1 = xs[q];
            } else {
              sts_f32_if(sC + 4u * (uint32_t)is, xs[q], carried);
            }
          }
          if (c == NCH - 1 && lane >= 30) {
            sts_f32(sC, h0);
            if (lane == 30) sts_f32(sC + 4u, h1);
          }
          if (s + 1 < ntask) load_chunk(s + 1);
        }
        __syncthreads();
      }
    } else {
      // ---- sweep warp w performs sweep w-1 of the pass
      const int sw = warp - 1;
      const bool last = (sw == nw - 1);
      WLaneState st;
      st.g1 = st.g2 = st.u1 = st.rm1 = st.h0 = st.h1 = 0.0f;
      st.c1 = 0u;
      WTask<ST> T;
      for (int s = 0; s < nsup; ++s) {
        const int g = s - warp;
        if (sw < nw && g >= 0 && g < ntask) {
          const int t = g / NCH, c = g - t * NCH;
          if (c == 0) {
            // ---- task set-up
            const int j = 32 * t + lane - 2 * sw - 2;
            T.valid = (j >= 0 && j <= S - 1);
            T.interior = (j >= 1 && j <= N);
            T.top = (j == 0);
            T.bot = (j == S - 1);
            const int jc = j < 0 ? 0 : (j > S - 1 ? S - 1 : j);
            T.rowfl = T.interior && G.rowfl[jc];
            const uint32_t ringIn = ring + (uint32_t)(warp - 1) * kWarp4;
            const uint32_t carryIn = carry + (uint32_t)(warp - 1) * 2u * cs4;
            // row j of a diagonal-layout grid: column i at base[i * P]
            const size_t rowJ = (size_t)jc * P + jc;
            T.rring = lane >= 2;
            T.dring = lane >= 1;
            T.sr = T.rring ? ringIn + (uint32_t)(lane - 2) * kLane4 : carryIn + (uint32_t)lane * cs4;
            T.sd = T.dring ? ringIn + (uint32_t)(lane - 1) * kLane4 : carryIn + cs4;
            T.pkrow = pk + (size_t)(W - 1) * P + rowJ;
            T.sedge = edge + (uint32_t)sw * cs4;
            T.gout = G.x + rowJ;
            const int ja = jc > 0 ? jc - 1 : 0;
            T.gfix = G.x + (size_t)ja * P + ja;
            const uint32_t carryOut = carry + (uint32_t)warp * 2u * cs4;
            T.sout = ring + (uint32_t)warp * kWarp4 + (uint32_t)lane * kLane4;
            T.scarry = (!last && lane >= 30) ? carryOut + (uint32_t)(lane - 30) * cs4 : 0u;
            T.sfix = carryOut + cs4;
            // Lanes 0 and 1 start inside the row: their history (G(0) for
            // lane 0, W(k-1)[i, j] for the first step) comes from column 0 / 1
            // of their carry row.
            st.g1 = st.g2 = st.u1 = st.rm1 = 0.0f;
            st.c1 = 0u;
            if (lane == 0) {
              st.g1 = lds_f32(T.sr);
              st.rm1 = lds_f32(T.sr + 4u);
            } else if (lane == 1) {
              st.rm1 = lds_f32(T.sr);
            }
          }
          const int half = (g & 1) * kWQ;
          if (last)
            wave_chunk_any<MODE, true, ST>(T, st, lane, c, NCH, half, S, P, a, cr);
          else
            wave_chunk_any<MODE, false, ST>(T, st, lane, c, NCH, half, S, P, a, cr);
          if (c == NCH - 1 && T.scarry) {
            sts_f32(T.scarry, st.h0);
            if (lane == 30) sts_f32(T.scarry + 4u, st.h1);
          }
        }
        __syncthreads();
      }
    }
  }
  if (threadIdx.x == 0) dg_corners<MODE, ST>(G.x, G.rowfl, G.colfl, S, P);
  __syncthreads();
}

}  // namespace eqk
