// lin_solve (fluid.rs:301-325) as ONE persistent launch that pipelines all of
// the reference's lexicographic Gauss-Seidel sweeps as a temporal wavefront,
// bit-exactly.
//
// Decomposition. A task is (strip b, sweep k): one warp, lane l owns row
//   j = 32*b + l - 2*k - 2
// (strips are skewed by two rows per sweep so that every dependency of a task
// points to (b, k-1) or (b-1, k) -- never to a later strip), and walks the
// row's columns one per step with lane l lagging lane l-1 by one step:
//   step tau: lane l updates column i = tau + 1 - l.
// The sweep-k value of (i, j) is
//   (x0 + a*(((R + L) + D) + U)) * (1/c)
// with L = own previous result (register), U = lane l-1's previous result
// (shuffle; lane 0 reads strip b-1's published last row), R = (i+1, j) from
// sweep k-1 after its set_boundaries (staged in shared memory) and D = (i, j+1),
// which is exactly what lane l+1 staged as its R (shuffle).
//
// Sequence-tagged buffers. Sweep k writes W(k) into one of two grids of 64-bit
// words (value | tag << 32, tag = tag0 + 1 + k) and reads W(k-1) from the
// other; W(-1) is the caller's x tagged tag0, and the last sweep writes plain
// floats straight into x. A consumer copies a 16-column slot of its row into
// shared memory (cp.async, L2) two chunks ahead and validates every tag it
// will use; a stale tag means the producer has not stored yet, and only that
// slot is copied again (bounded, with back-off). No flags and no fences sit on
// the data path, so no warp ever stalls on a release.
//
// set_boundaries after each sweep is fused into the write: W(k) holds the
// post-boundary value of every cell, while the raw values that later cells of
// the SAME sweep need (L, U) travel in registers and shuffles. A cell whose
// post-boundary value is minus a neighbour's raw value of the same sweep is
// stored one step late (once that neighbour is known); the Column-mode case
// whose neighbour lives in the next strip is stored by that strip's lane 0.
// Every ghost-frame cell except the corners is rewritten each sweep (with its
// Passive copy where the row / column has a fluid cell, like the reference's
// loop over fluid cells, and with its carried value otherwise) so that every
// value a reader uses carries the current tag. Corners, which no sweep reads,
// are computed once after the last sweep.
//
// Work order: task indices come from an atomic ticket in topological order,
// so a task only waits for tasks that already hold a ticket (no co-residency
// assumption). A wait that exceeds the spin budget sets the device error word
// and returns; every wait also watches that word, so the grid drains.
#pragma once
#include "common.cuh"

namespace eqk {

struct LinSolveArgs {
  float* x;                    // out: W(K-1) (plain floats); W(-1) lives in wt[0]
  unsigned long long* wt[2];   // tagged grids: W(k) in wt[(k + 1) & 1]
  const float* x0;
  const uint8_t* code;
  const uint8_t* rowfl;
  const uint8_t* colfl;
  unsigned long long* edge;    // [ntasks][P] tagged raw last-row values
  unsigned* ticket;            // zeroed by the host before every launch
  unsigned* done;              // zeroed by the host before every launch
  int* err;                    // device error word
  long long spin_limit;
  unsigned tag0;               // tag of W(-1)
  int S, P, K, B;
  float a, c_recip;
};

constexpr int kLsQ = 16;     // steps per chunk = columns per slot
constexpr int kLsRing = 64;  // columns kept per row in shared memory (4 slots)

__device__ __forceinline__ unsigned long long pack_tag(float v, unsigned tag) {
  return (unsigned long long)__float_as_uint(v) | ((unsigned long long)tag << 32);
}
__device__ __forceinline__ float tag_val(unsigned long long w) {
  return __uint_as_float((unsigned)(w & 0xffffffffull));
}
__device__ __forceinline__ unsigned tag_of(unsigned long long w) { return (unsigned)(w >> 32); }
__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// W(-1) = x tagged tag0, over the whole pitched grid.
__global__ void k_ls_tag_init(unsigned long long* __restrict__ w, const float* __restrict__ x,
                              size_t n, unsigned tag0) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride)
    w[q] = pack_tag(x[q], tag0);
}

// Shared staging of one task: each lane's own row of W(k-1), x0 and codes as a
// ring of kLsRing columns (slot = column & 63); lane 31 also stages the row
// below its own, lane 0 the previous strip's published last row.
struct LsSmem {
  unsigned long long R[32][kLsRing];
  float X[32][kLsRing];
  unsigned long long D[kLsRing];
  unsigned long long E[kLsRing];
  uint8_t C[32][kLsRing];
};

template <int MODE>
__global__ void __launch_bounds__(32) k_lin_solve(LinSolveArgs A) {
  __shared__ __align__(16) LsSmem sm;
  const int lane = threadIdx.x;
  const unsigned FULL = 0xffffffffu;
  unsigned t = 0;
  if (lane == 0) t = atomicAdd(A.ticket, 1u);
  t = __shfl_sync(FULL, t, 0);
  const int K = A.K, S = A.S, P = A.P, N = S - 2;
  if (t >= (unsigned)(A.B * K)) {  // counters not reset: never index past the tasks
    if (lane == 0) atomicExch(A.err, 5 /* EQ_ERR_STATE */);
    return;
  }
  const int b = (int)(t / (unsigned)K), k = (int)(t % (unsigned)K);
  const int j = 32 * b + lane - 2 * k - 2;
  const unsigned tagIn = A.tag0 + (unsigned)k;  // tag of W(k-1)
  const unsigned tagOut = tagIn + 1u;
  const bool last = (k == K - 1);

  const unsigned long long* Win = (k & 1) ? A.wt[1] : A.wt[0];
  unsigned long long* Wout = (k & 1) ? A.wt[0] : A.wt[1];

  const bool interior = (j >= 1 && j <= N);
  const bool frame = (j == 0 || j == S - 1);
  const int jc = (interior || frame) ? j : 0;
  const int jd = (jc + 1 < S) ? jc + 1 : S - 1;
  const unsigned long long* rowIn = Win + (size_t)jc * P;
  const unsigned long long* rowDn = Win + (size_t)jd * P;
  const float* rowX0 = A.x0 + (size_t)jc * P;
  const uint8_t* rowCode = A.code + (size_t)jc * P;
  const size_t outRow = (size_t)jc * P;
  const size_t aboveRow = (size_t)(jc > 0 ? jc - 1 : 0) * P;
  const unsigned long long* edgeIn = A.edge + (size_t)(b > 0 ? (b - 1) * K + k : 0) * P;
  unsigned long long* edgeOut = A.edge + (size_t)(b * K + k) * P;
  const bool rowHasFluid = interior && A.rowfl[j];
  const bool firstRow = (j == 1), lastRow = (j == N);
  const float a = A.a, cr = A.c_recip;
  const int T = N + 32;  // steps: lane 31 stores its last column at step N+31
  const int nchunks = (T + kLsQ - 1) / kLsQ;

  // Stores of this sweep: tagged into Wout, or plain into x for the last sweep.
  float* const xout = A.x;
#define EQ_LS_PUT(q, v)                                          \
  do {                                                           \
    if (last)                                                    \
      __stcg(xout + (q), (v));                                   \
    else                                                         \
      st_relaxed_u64(Wout + (q), pack_tag((v), tagOut));         \
  } while (0)

  // Lane l reads columns [16c+1-l, 16c+17-l] in chunk c. Its copy stream is cut
  // into 16-column slots starting at base = floor4(2-l): slot n covers
  // [base+16n, base+16n+16) and is needed by chunk n-1 at the latest.
  const int base = ((2 - lane) >= 0) ? ((2 - lane) & ~3) : -(((lane - 2) + 3) & ~3);
  const bool loadD = (lane == 31) && (interior || frame);
  const bool loadE = (lane == 0) && (b > 0);
  // Tags that must be current: every column of an interior row (its ghost
  // columns are rewritten each sweep) and columns 1..N of a frame row.

  auto issue_slot = [&](int n, bool rOnly, bool mine) {
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const int col = base + 16 * n + 4 * s;
      const bool ok = mine && (n >= 0) && col >= 0 && col <= S - 1 && col + 4 <= P;
      const int cc = ok ? col : 0;
      const int slot = cc & (kLsRing - 1);
      cp_async16(&sm.R[lane][slot], rowIn + cc, ok);
      cp_async16(&sm.R[lane][slot + 2], rowIn + cc + 2, ok);
      cp_async16(&sm.D[slot], rowDn + cc, ok && loadD);
      cp_async16(&sm.D[slot + 2], rowDn + cc + 2, ok && loadD);
      cp_async16(&sm.E[slot], edgeIn + cc, ok && loadE);
      cp_async16(&sm.E[slot + 2], edgeIn + cc + 2, ok && loadE);
      if (!rOnly) {
        cp_async16(&sm.X[lane][slot], rowX0 + cc, ok);
        cp_async4(&sm.C[lane][slot], rowCode + cc, ok);
      }
    }
    cp_async_commit();
  };
  // Is any tag that chunk c uses stale? (R at i+1, lane 31's D and lane 0's E
  // at i, plus x[0, j] / x[1, j] that the first columns read.)
  auto chunk_stale = [&](int c) -> bool {
    unsigned bad = 0u;
    const int c0 = c * kLsQ;
#pragma unroll
    for (int q = 0; q < kLsQ; ++q) {
      const int i = c0 + q + 1 - lane;
      const int cr = i + 1;
      const bool useR = interior ? (cr >= 0 && cr <= S - 1) : (frame && cr >= 1 && cr <= N);
      if (useR) bad |= tag_of(sm.R[lane][cr & (kLsRing - 1)]) ^ tagIn;
      const bool inCol = (i >= 1 && i <= N);
      if (loadD && inCol) bad |= tag_of(sm.D[i & (kLsRing - 1)]) ^ tagIn;
      if (loadE && inCol) bad |= tag_of(sm.E[i & (kLsRing - 1)]) ^ tagOut;
    }
    // Lanes 0 and 1 meet column 1 before any step of theirs loaded x[0, j] /
    // x[1, j] as R; both sit in slot 0 for them (base = 0).
    if (c == 0 && lane <= 1) {
      if (interior) bad |= tag_of(sm.R[lane][0]) ^ tagIn;
      if (interior || frame) bad |= tag_of(sm.R[lane][1]) ^ tagIn;
    }
    return bad != 0u;
  };
  // Copy the slots of chunk c again (stale lanes only) until it validates.
  auto settle_chunk = [&](int c, bool bad) -> bool {
    long long tries = 0;
    unsigned ns = 32;
    while (__any_sync(FULL, bad)) {
      if (++tries > A.spin_limit) {
        if (lane == 0) atomicExch(A.err, 3 /* EQ_ERR_TIMEOUT */);
        return false;
      }
      if ((tries & 63) == 0 && __any_sync(FULL, ld_relaxed_i32(A.err) != 0)) return false;
      __nanosleep(ns);
      ns = ns < 512 ? ns * 2 : 512;
      issue_slot(c, true, bad);
      issue_slot(c + 1, true, bad);
      cp_async_wait<0>();
      bad = chunk_stale(c);
    }
    return true;
  };

  issue_slot(0, false, true);
  issue_slot(1, false, true);

  float g1 = 0.f, g2 = 0.f, u1 = 0.f, Rprev = 0.f;
  uint8_t code1 = 0;
  const bool ghostRowLane = (MODE == kPassive) && (firstRow || lastRow);
  const size_t ghostRow = firstRow ? 0 : (size_t)(S - 1) * P;

  for (int c = 0; c < nchunks; ++c) {
    issue_slot(c + 2, false, true);
    cp_async_wait<1>();  // slots <= c+1 have landed
    const int c0 = c * kLsQ;
    if (c0 >= 33 && c0 + kLsQ <= N) {
      // ---- fast chunk: every lane's columns lie in [3, N]. Values are
      // validated as they are consumed; the chunk's results are stored only
      // once every tag checked, so a stale copy is simply redone.
      const float s_g1 = g1, s_g2 = g2, s_u1 = u1, s_Rprev = Rprev;
      float gv[kLsQ], uv[kLsQ];
      long long tries = 0;
      unsigned ns = 32;
      while (true) {
        unsigned bad = 0u;
#pragma unroll
        for (int q = 0; q < kLsQ; ++q) {
          const int i = c0 + q + 1 - lane;
          const int si = i & (kLsRing - 1);
          const unsigned long long Rw = sm.R[lane][(i + 1) & (kLsRing - 1)];
          if (interior || (frame && i + 1 <= N)) bad |= tag_of(Rw) ^ tagIn;
          const float R = tag_val(Rw);
          const float X = sm.X[lane][si];
          float D = __shfl_down_sync(FULL, R, 1);  // lane l+1's R is x[i, j+1]
          if (lane == 31) {
            const unsigned long long Dw = sm.D[si];
            if (loadD) bad |= tag_of(Dw) ^ tagIn;
            D = tag_val(Dw);
          }
          float U = __shfl_up_sync(FULL, g1, 1);  // lane l-1's G(i, j-1)
          if (lane == 0) {
            const unsigned long long Ew = sm.E[si];
            if (loadE) bad |= tag_of(Ew) ^ tagOut;
            U = tag_val(Ew);
          }
          const float gc = fmul(fadd(X, fmul(a, fadd(fadd(fadd(R, g1), D), U))), cr);
          const float g = interior ? gc : Rprev;  // frame lanes pass x[i, j] on
          g2 = g1;
          g1 = g;
          u1 = U;
          Rprev = R;
          gv[q] = g;
          uv[q] = U;
        }
        if (!__any_sync(FULL, bad != 0u)) break;
        // a producer has not stored yet: restore, copy again, recompute
        g1 = s_g1;
        g2 = s_g2;
        u1 = s_u1;
        Rprev = s_Rprev;
        if (++tries > A.spin_limit) {
          if (lane == 0) atomicExch(A.err, 3 /* EQ_ERR_TIMEOUT */);
          cp_async_wait<0>();
          return;
        }
        if ((tries & 63) == 0 && __any_sync(FULL, ld_relaxed_i32(A.err) != 0)) {
          cp_async_wait<0>();
          return;
        }
        __nanosleep(ns);
        ns = ns < 512 ? ns * 2 : 512;
        issue_slot(c, true, bad != 0u);
        issue_slot(c + 1, true, bad != 0u);
        cp_async_wait<0>();
      }
      // ---- the chunk's stores: column i-1 of each step, post-boundary value
#pragma unroll
      for (int q = 0; q < kLsQ; ++q) {
        const int i = c0 + q + 1 - lane;
        const int is = i - 1;
        const float gi = gv[q];                                       // G(i)
        const float gs = q > 0 ? gv[q - 1] : s_g1;                    // G(i-1)
        const float gp = q > 1 ? gv[q - 2] : (q == 1 ? s_g1 : s_g2);  // G(i-2)
        const float us = q > 0 ? uv[q - 1] : s_u1;                    // U at i-1
        const uint8_t cs = sm.C[lane][is & (kLsRing - 1)];            // code(i-1, j)
        const uint8_t ci = sm.C[lane][i & (kLsRing - 1)];             // code(i, j)
        const float gdown = __shfl_down_sync(FULL, gi, 1);            // G(i-1, j+1)
        float val = gs;
        bool keep = true;
        if (MODE == kRow) {
          val = (cs & kCodeRowRight) ? -gi : ((cs & kCodeRowLeft) ? -gp : gs);
        } else if (MODE == kCol) {
          const bool dn = (cs & kCodeColDown) != 0;
          val = (cs & kCodeColUp) ? -us : (dn ? -gdown : gs);
          keep = !(dn && !(cs & kCodeColUp) && lane == 31);  // strip b+1 stores it
        }
        if (interior && keep) EQ_LS_PUT(outRow + is, val);
        if (ghostRowLane && (cs & kCodeColFluid)) EQ_LS_PUT(ghostRow + is, gs);
        const bool cfi = (MODE == kPassive) && ((ci & kCodeColFluid) != 0);
        if (frame && !cfi) EQ_LS_PUT(outRow + i, gi);
        if (MODE == kCol && lane == 0 && (interior || frame) && (ci & kCodeAboveDown))
          EQ_LS_PUT(aboveRow + i, -gi);
        if (lane == 31) st_relaxed_u64(edgeOut + i, pack_tag(gi, tagOut));
      }
      code1 = sm.C[lane][(c0 + kLsQ - lane) & (kLsRing - 1)];
      continue;
    }

    // ---- general chunk (row ends): validate everything, then compute + store
    if (!settle_chunk(c, chunk_stale(c))) {
      cp_async_wait<0>();
      return;
    }
    if (c == 0) Rprev = tag_val(sm.R[lane][1]);
    const float L0 = tag_val(sm.R[lane][0]);  // x[0, j] of W(k-1), used at column 1
#pragma unroll 4
    for (int q = 0; q < kLsQ; ++q) {
      const int i = c0 + q + 1 - lane;
      const int si = i & (kLsRing - 1);
      const float R = tag_val(sm.R[lane][(i + 1) & (kLsRing - 1)]);
      const float X = sm.X[lane][si];
      const uint8_t C = sm.C[lane][si];
      const float Dl = tag_val(sm.D[si]);
      const float El = tag_val(sm.E[si]);
      float D = __shfl_down_sync(FULL, R, 1);  // lane l+1's R is x[i, j+1]
      if (lane == 31) D = Dl;
      float U = __shfl_up_sync(FULL, g1, 1);  // lane l-1's G(i, j-1)
      if (lane == 0) U = El;
      const float L = (i == 1) ? L0 : g1;
      const float gc = fmul(fadd(X, fmul(a, fadd(fadd(fadd(R, L), D), U))), cr);
      const bool act = interior && i >= 1 && i <= N;
      const float g = act ? gc : Rprev;  // frame lanes / column N+1 pass x[i, j] on
      const float gdown = __shfl_down_sync(FULL, g, 1);  // G(i-1, j+1)
      const bool inCol = (i >= 1 && i <= N);

      // delayed store of column i-1 with its post-boundary value
      const int is = i - 1;
      const bool st = interior && is >= 1 && is <= N;
      float val = g1;
      bool keep = true;
      if (MODE == kRow) {
        val = (code1 & kCodeRowRight) ? -g : ((code1 & kCodeRowLeft) ? -g2 : g1);
      } else if (MODE == kCol) {
        const bool dn = (code1 & kCodeColDown) != 0;
        val = (code1 & kCodeColUp) ? -u1 : (dn ? -gdown : g1);
        keep = !(dn && !(code1 & kCodeColUp) && lane == 31);  // strip b+1 stores it
      }
      if (st && keep) EQ_LS_PUT(outRow + is, val);
      // ghost columns of this row: Passive copy where the row has fluid, else carried
      const bool pasRow = (MODE == kPassive) && rowHasFluid;
      if (st && is == 1) EQ_LS_PUT(outRow, pasRow ? g1 : g2);
      if (st && is == N) EQ_LS_PUT(outRow + (S - 1), pasRow ? g1 : g);
      // ghost rows: Passive copy from row 1 / row N where the column has fluid ...
      const bool cf1 = (MODE == kPassive) && ((code1 & kCodeColFluid) != 0);
      if (st && firstRow && cf1) EQ_LS_PUT(is, g1);
      if (st && lastRow && cf1) EQ_LS_PUT((size_t)(S - 1) * P + is, g1);
      // ... else the frame lane carries its value
      const bool cf = (MODE == kPassive) && ((C & kCodeColFluid) != 0);
      if (frame && inCol && !cf) EQ_LS_PUT(outRow + i, g);
      if (MODE == kCol && lane == 0 && (interior || frame) && inCol && (C & kCodeAboveDown))
        EQ_LS_PUT(aboveRow + i, -g);
      if (lane == 31 && inCol) st_relaxed_u64(edgeOut + i, pack_tag(g, tagOut));

      g2 = (i == 1) ? L : g1;
      g1 = g;
      u1 = U;
      code1 = C;
      Rprev = R;
    }
  }
  cp_async_wait<0>();

  // ---- completion; the last task computes the corners (no sweep reads them)
  __syncwarp();
  unsigned prev = 0;
  if (lane == 0) {
    __threadfence();
    prev = atom_add_acq_rel_u32(A.done, 1u);
  }
  prev = __shfl_sync(FULL, prev, 0);
  const unsigned ntasks = (unsigned)(A.B * A.K);
  if (prev == ntasks - 1) {
    __threadfence();
    if (lane == 0) corners<MODE>(A.x, A.rowfl, A.colfl, S, P);
  }
}

#undef EQ_LS_PUT

}  // namespace eqk
