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
template <int MODE>
__device__ __forceinline__ float dg_frame_after_pass(const float* x, const uint8_t* rowfl,
                                                     const uint8_t* colfl, int S, int P, int i,
                                                     int j) {
  if (MODE == kPassive) {
    if (j == 0 && colfl[i]) return x[dg_at(i, 1, P)];
    if (j == S - 1 && colfl[i]) return x[dg_at(i, S - 2, P)];
    if (i == 0 && rowfl[j]) return x[dg_at(1, j, P)];
    if (i == S - 1 && rowfl[j]) return x[dg_at(S - 2, j, P)];
  }
  return x[dg_at(i, j, P)];
}

template <int MODE>
__device__ __forceinline__ void dg_corners(float* x, const uint8_t* rowfl, const uint8_t* colfl,
                                           int S, int P) {
  auto f = [&](int i, int j) { return dg_frame_after_pass<MODE>(x, rowfl, colfl, S, P, i, j); };
  const float c00 = fmul(0.5f, fadd(f(1, 0), f(0, 1)));
  const float c0S = fmul(0.5f, fadd(f(1, S - 1), f(0, S - 2)));
  const float cS0 = fmul(0.5f, fadd(f(S - 2, 0), f(S - 1, 1)));
  const float cSS = fmul(0.5f, fadd(f(S - 2, S - 1), f(S - 1, S - 2)));
  x[dg_at(0, 0, P)] = c00;
  x[dg_at(0, S - 1, P)] = c0S;
  x[dg_at(S - 1, 0, P)] = cS0;
  x[dg_at(S - 1, S - 1, P)] = cSS;
}

// One scene grid as the block solver sees it (diagonal layout).
struct WGrid {
  float* x;
  const float* x0;
  const uint8_t* code;   // boundary codes, diagonal layout
  const uint8_t* rowfl;  // [S]
  const uint8_t* colfl;  // [S]
  int S, P;
};

// Block-private buffers (generic pointers: shared memory when they fit).
struct WBufs {
  float* ring;   // [nwmax-1][32][kWRS]  (shared)
  float* carry;  // [nwmax][2][cs]; carry[w] (w >= 1) is written by warp w-1
  float* edge;   // [nwmax][cs]
  int cs;        // row stride of carry / edge, >= S
};

// Strips per pass: every sweep k < nw must cover rows 0..S-1, and lane 31 of
// the last strip must never hold an interior row (its fix-up would need a
// strip that does not exist): 32 (B-1) + 29 - 2 (nw-1) >= S - 1.
__host__ __device__ inline int wave_strips(int S, int nw) { return (S + 2 * nw - 1) / 32 + 1; }
__host__ __device__ inline int wave_chunks(int S) { return (S + 31 + kWQ - 1) / kWQ; }

struct WLaneState {
  float g1, g2, u1, rm1;
  float h0, h1;  // carry columns 0 / 1 of lanes 30 / 31, written at the task's end
  uint32_t c1;
};

// Per-task, per-lane constants. Every stream is (base, stride): the element
// for column i sits at base[i * stride] (column-indexed rows: stride 1;
// diagonal-layout grid rows: stride P, base shifted by the row) or, for ring
// lanes, at base[slot].
struct WTask {
  const float* rsrc;  // R: x row (first sweep), carry row, or ring lane
  const float* dsrc;  // D: x row j+1 (first sweep), carry row 1, or ring lane
  int rstr, dstr;     // 0 = ring (slot-indexed), else column stride
  const float* x0row;
  const uint8_t* crow;
  float* out;  // ring lane (slot-indexed, ostr 0) or x row (column-indexed)
  int ostr;
  bool outok;
  float* carryout;  // lanes 30/31 of a non-last warp: column-indexed carry row
  float* fixrow;    // lane 0 (AdjustColumn): the row above, column-indexed
  int fstr;
  float* edge;      // this warp's edge row
  int P;
  bool valid, interior, top, bot, rowfl;
};

template <int MODE, bool EDGE>
__device__ __forceinline__ void wave_chunk(const WTask& T, WLaneState& st, int lane, int c,
                                           int half, int S, float a, float cr) {
  const unsigned FULL = 0xffffffffu;
  const int N = S - 2;
  const int P = T.P;
  const int tau0 = c * kWQ;
  const int ib = tau0 + 1 - lane;  // column at q = 0
  const float* pR = T.rstr ? T.rsrc + (ptrdiff_t)(ib + 1) * T.rstr : T.rsrc + half;
  const int sR = T.rstr ? T.rstr : 1;
  const float* pD = T.dstr ? T.dsrc + (ptrdiff_t)ib * T.dstr : T.dsrc + half;
  const int sD = T.dstr ? T.dstr : 1;
  float* pO = T.ostr ? T.out + (ptrdiff_t)(ib - 1) * T.ostr : T.out + half;
  const int sO = T.ostr ? T.ostr : 1;
  const float* pX = T.x0row + (ptrdiff_t)ib * P;
  const uint8_t* pC = T.crow + (ptrdiff_t)ib * P;
  float* pF = T.fixrow + (ptrdiff_t)ib * T.fstr;

  constexpr int kG = 4;  // steps whose loads are issued together
#pragma unroll
  for (int q0 = 0; q0 < kWQ; q0 += kG) {
    float Rv[kG], Dv[kG], Xv[kG], Ev[kG];
    uint32_t Cv[kG];
    // Loads of the group first. Safe: x0 and the codes are read-only, the
    // edge columns lane 31 overwrites in this chunk are below the ones lane 0
    // reads, and a lane's writes of its own row / the row below trail its reads.
#pragma unroll
    for (int r = 0; r < kG; ++r) {
      const int q = q0 + r;
      const int i = ib + q;
      if (EDGE) {
        const bool okR = !T.rstr || (i + 1 >= 0 && i + 1 <= S - 1);
        const bool okD = !T.dstr || (i >= 0 && i <= S - 1);
        const bool okI = (i >= 0 && i <= S - 1);
        Rv[r] = okR ? pR[(ptrdiff_t)q * sR] : 0.0f;
        Dv[r] = okD ? pD[(ptrdiff_t)q * sD] : 0.0f;
        Xv[r] = okI ? pX[(ptrdiff_t)q * P] : 0.0f;
        Cv[r] = okI ? (uint32_t)pC[(ptrdiff_t)q * P] : 0u;
        Ev[r] = (lane == 0 && okI) ? T.edge[i] : 0.0f;
      } else {
        Rv[r] = pR[(ptrdiff_t)q * sR];
        Dv[r] = pD[(ptrdiff_t)q * sD];
        Xv[r] = pX[(ptrdiff_t)q * P];
        Cv[r] = pC[(ptrdiff_t)q * P];
        Ev[r] = T.edge[i];
      }
    }
#pragma unroll
    for (int r = 0; r < kG; ++r) {
      const int q = q0 + r;
      const int i = ib + q;
      float U = __shfl_up_sync(FULL, st.g1, 1);
      if (lane == 0) U = Ev[r];
      const float R = Rv[r];
      const float gc = fmul(fadd(Xv[r], fmul(a, fadd(fadd(fadd(R, st.g1), Dv[r]), U))), cr);
      const bool act = EDGE ? (T.interior && i >= 1 && i <= N) : T.interior;
      const float g = act ? gc : st.rm1;
      const float gd = __shfl_down_sync(FULL, g, 1);

      // post-boundary value of column i-1
      const uint32_t c1 = st.c1;
      float val;
      if (MODE == kRow) {
        val = (c1 & kCodeRowRight) ? -g : ((c1 & kCodeRowLeft) ? -st.g2 : st.g1);
      } else if (MODE == kCol) {
        val = (c1 & kCodeColUp) ? -st.u1 : ((c1 & kCodeColDown) ? -gd : st.g1);
      } else {
        const bool cf = (c1 & kCodeColFluid) != 0;
        val = (T.top && cf) ? gd : ((T.bot && cf) ? st.u1 : st.g1);
        if (EDGE && T.interior) {
          if (i - 1 == 0) val = T.rowfl ? g : st.g1;
          if (i - 1 == S - 1) val = T.rowfl ? st.g2 : st.g1;
        }
      }
      const bool colok = EDGE ? (i - 1 >= 0 && i - 1 <= S - 1) : true;
      if (T.outok && colok) pO[(ptrdiff_t)q * sO] = val;
      if (T.carryout && colok) {
        // Columns 0 / 1 of the carry rows are produced in chunk 1, the super-step
        // in which the next warp still reads the previous strip's columns 0 / 1;
        // they are held back and written when the task ends.
        if (EDGE && tau0 < 2 * kWQ) {
          if (i - 1 == 0) st.h0 = val;
          if (i - 1 == 1) st.h1 = val;
        } else {
          T.carryout[i - 1] = val;
        }
      }
      if (lane == 31 && (EDGE ? (i >= 0 && i <= S - 1) : true)) T.edge[i] = g;
      // (a lane whose row lies outside the grid reads a clamped row's code)
      if (MODE == kCol && lane == 0 && T.valid && (Cv[r] & kCodeAboveDown) &&
          (EDGE ? (i >= 1 && i <= N) : true))
        pF[(ptrdiff_t)q * T.fstr] = -g;

      st.g2 = st.g1;
      st.g1 = g;
      st.u1 = U;
      st.rm1 = R;
      st.c1 = Cv[r];
    }
  }
}

// `K` sweeps of lin_solve on grid G by the whole block (blockDim.x = 32 *
// nwmax), passes of at most nwmax sweeps. Ends with a block barrier; the
// result (corners included) is in G.x.
template <int MODE>
__device__ __noinline__ void wave_lin_solve(const WGrid G, const WBufs Bf, int K, int nwmax,
                                            float a, float cr) {
  if (K <= 0) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int S = G.S, P = G.P, N = S - 2;
  const int NCH = wave_chunks(S);
  for (int k0 = 0; k0 < K; k0 += nwmax) {
    const int nw = min(nwmax, K - k0);
    const int B = wave_strips(S, nw);
    const int ntask = B * NCH;
    const int nsup = ntask + nw - 1;
    const bool first = (warp == 0), last = (warp == nw - 1);
    WLaneState st{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0u};
    WTask T;
    T.P = P;
    for (int s = 0; s < nsup; ++s) {
      const int g = s - warp;
      if (warp < nw && g >= 0 && g < ntask) {
        const int t = g / NCH, c = g - t * NCH;
        if (c == 0) {
          // ---- task set-up
          const int j = 32 * t + lane - 2 * warp - 2;
          T.valid = (j >= 0 && j <= S - 1);
          T.interior = (j >= 1 && j <= N);
          T.top = (j == 0);
          T.bot = (j == S - 1);
          const int jc = j < 0 ? 0 : (j > S - 1 ? S - 1 : j);
          const int jd = j + 1 < 0 ? 0 : (j + 1 > S - 1 ? S - 1 : j + 1);
          T.rowfl = T.interior && G.rowfl[jc];
          float* ringIn = Bf.ring + (size_t)(warp - 1) * 32 * kWRS;
          float* carryIn = Bf.carry + (size_t)warp * 2 * Bf.cs;
          // row j of a diagonal-layout grid: column i at base[i * P]
          const size_t rowJ = (size_t)jc * P + jc, rowD = (size_t)jd * P + jd;
          if (first) {
            T.rsrc = G.x + rowJ;
            T.dsrc = G.x + rowD;
            T.rstr = T.dstr = P;
          } else {
            T.rstr = lane >= 2 ? 0 : 1;
            T.dstr = lane >= 1 ? 0 : 1;
            T.rsrc = lane >= 2 ? ringIn + (lane - 2) * kWRS : carryIn + (size_t)lane * Bf.cs;
            T.dsrc = lane >= 1 ? ringIn + (lane - 1) * kWRS : carryIn + Bf.cs;
          }
          T.x0row = G.x0 + rowJ;
          T.crow = G.code + rowJ;
          T.edge = Bf.edge + (size_t)warp * Bf.cs;
          if (last) {
            T.out = G.x + rowJ;
            T.ostr = P;
            T.outok = T.valid;
            T.carryout = nullptr;
            const int ja = jc > 0 ? jc - 1 : 0;
            T.fixrow = G.x + (size_t)ja * P + ja;
            T.fstr = P;
          } else {
            float* carryOut = Bf.carry + (size_t)(warp + 1) * 2 * Bf.cs;
            T.out = Bf.ring + (size_t)warp * 32 * kWRS + lane * kWRS;
            T.ostr = 0;
            T.outok = true;
            T.carryout = (lane >= 30) ? carryOut + (size_t)(lane - 30) * Bf.cs : nullptr;
            T.fixrow = carryOut + Bf.cs;
            T.fstr = 1;
          }
          // Lanes 0 and 1 start inside the row: their history (G(0) for lane
          // 0, W(k-1)[i, j] for the first step) comes from column 0 / 1 of
          // their column-indexed R source.
          st.g1 = st.g2 = st.u1 = st.rm1 = 0.0f;
          st.c1 = 0u;
          if (lane == 0) {
            st.g1 = T.rsrc[0];
            st.rm1 = T.rsrc[T.rstr];
          } else if (lane == 1) {
            st.rm1 = T.rsrc[0];
          }
        }
        const int half = (g & 1) * kWQ;
        const int tau0 = c * kWQ;
        const bool fast = (tau0 >= 32) && (tau0 + kWQ <= N);
        if (fast)
          wave_chunk<MODE, false>(T, st, lane, c, half, S, a, cr);
        else
          wave_chunk<MODE, true>(T, st, lane, c, half, S, a, cr);
        if (c == NCH - 1 && T.carryout) {
          T.carryout[0] = st.h0;
          if (lane == 30) T.carryout[1] = st.h1;
        }
      }
      __syncthreads();
    }
  }
  if (threadIdx.x == 0) dg_corners<MODE>(G.x, G.rowfl, G.colfl, S, P);
  __syncthreads();
}

}  // namespace eqk
