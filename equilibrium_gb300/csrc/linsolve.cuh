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
// (shuffle; lane 0 reads strip b-1's published last row), and R = (i+1, j),
// D = (i, j+1) from sweep k-1 after its set_boundaries.
//
// Buffers. Sweep k reads W(k-1) and writes W(k), alternating between the
// caller's x and a spare grid so that no value is overwritten while a reader
// of the previous sweep may still need it. The final sweep lands in x.
//
// set_boundaries after each sweep is fused into the write: W(k) holds the
// post-boundary value of every cell, while the raw values that later cells of
// the SAME sweep need (L, U) travel in registers and shuffles. A cell whose
// post-boundary value is minus a neighbour's raw value of the same sweep is
// stored one step late (once that neighbour is known); the Column-mode case
// whose neighbour lives in the next strip is stored by that strip's lane 0.
// Passive mode stores the ghost-frame copies (only where the row / column has
// a fluid cell, like the reference's loop over fluid cells). Corners, which no
// sweep reads, are computed once after the last sweep.
//
// Synchronisation. Each task publishes how many of its steps are complete
// (release); a task waits (acquire, bounded spin) for progress of (b, k-1)
// and (b-1, k). Task indices come from an atomic ticket in topological order,
// so a task only ever waits for tasks that already hold a ticket: no
// co-residency assumption. On a spin budget overrun the task sets the device
// error word and returns; all waits watch that word, so the grid drains.
#pragma once
#include "common.cuh"

namespace eqk {

struct LinSolveArgs {
  float* x;        // in: initial guess (W(-1) when K is even), out: result
  float* spare;    // second buffer, holds a copy of the input on entry
  const float* x0;
  const uint8_t* code;
  const uint8_t* rowfl;
  const uint8_t* colfl;
  float* edge;                    // [ntasks][P] raw last-row values
  unsigned long long* progress;   // [ntasks], zero on entry, reset on exit
  unsigned* ticket;               // zero on entry, reset on exit
  unsigned* done;                 // zero on entry, reset on exit
  int* err;                       // device error word
  long long spin_limit;
  int S, P, K, B;
  float a, c_recip;
};

constexpr int kLsQ = 16;  // steps per chunk (one wait + one batch of loads)

__device__ __forceinline__ bool ls_wait(const unsigned long long* p, unsigned long long target,
                                        long long limit, int* err) {
  long long n = 0;
  while (true) {
    if (ld_acquire_u64(p) >= target) return true;
    if (++n > limit) {
      atomicExch(err, 3 /* EQ_ERR_TIMEOUT */);
      return false;
    }
    if ((n & 255) == 0 && ld_relaxed_i32(err) != 0) return false;
  }
}

template <int MODE>
__global__ void __launch_bounds__(32) k_lin_solve(LinSolveArgs A) {
  const int lane = threadIdx.x;
  const unsigned FULL = 0xffffffffu;
  unsigned t = 0;
  if (lane == 0) t = atomicAdd(A.ticket, 1u);
  t = __shfl_sync(FULL, t, 0);
  const int K = A.K, S = A.S, P = A.P, N = S - 2;
  const int b = (int)(t / (unsigned)K), k = (int)(t % (unsigned)K);
  const int j = 32 * b + lane - 2 * k - 2;

  // W(k) = x when (K-1-k) is even; W(k-1) is the other buffer.
  float* Wout = (((K - 1 - k) & 1) == 0) ? A.x : A.spare;
  const float* Win = (((K - 1 - k) & 1) == 0) ? A.spare : A.x;

  const bool interior = (j >= 1 && j <= N);
  const bool frame = (j == 0 || j == S - 1);
  const int jc = (interior || frame) ? j : 0;
  const float* rowIn = Win + (size_t)jc * P;
  const float* rowDn = Win + (size_t)(jc + 1 < S ? jc + 1 : S - 1) * P;
  const float* rowX0 = A.x0 + (size_t)jc * P;
  const uint8_t* rowCode = A.code + (size_t)jc * P;
  float* rowOut = Wout + (size_t)jc * P;
  float* rowAbove = Wout + (size_t)(jc > 0 ? jc - 1 : 0) * P;
  const float* edgeIn = A.edge + (size_t)(b > 0 ? (b - 1) * K + k : 0) * P;
  float* edgeOut = A.edge + (size_t)(b * K + k) * P;
  unsigned long long* progOwn = A.progress + (b * K + k);
  const unsigned long long* progSweep = A.progress + (k > 0 ? b * K + k - 1 : 0);
  const unsigned long long* progStrip = A.progress + (b > 0 ? (b - 1) * K + k : 0);
  const bool rowHasFluid = interior && A.rowfl[j];
  const bool firstRow = (j == 1), lastRow = (j == N);
  float* frameTop = Wout;                       // row 0
  float* frameBot = Wout + (size_t)(S - 1) * P;  // row S-1
  const float a = A.a, cr = A.c_recip;
  const int T = N + 32;  // steps: lane 31 stores its last column at step N+31

  float g1 = 0.f, g2 = 0.f, u1 = 0.f;  // G(i-1), G(i-2), U at i-1
  uint8_t code1 = 0;                    // code(i-1, j)
  bool ok = true;

  for (int c0 = 0; c0 < T; c0 += kLsQ) {
    // ---- wait for the producers of this chunk's inputs
    if (lane == 0) {
      if (k > 0) {
        const unsigned long long need = (unsigned long long)min(c0 + kLsQ, T);
        ok = ls_wait(progSweep, need, A.spin_limit, A.err);
      }
      if (ok && b > 0) {
        const unsigned long long need = (unsigned long long)min(c0 + kLsQ + 33, T);
        ok = ls_wait(progStrip, need, A.spin_limit, A.err);
      }
    }
    ok = __shfl_sync(FULL, ok ? 1 : 0, 0) != 0;
    if (!ok) return;

    // ---- loads for the chunk (independent of the recurrence: issued together)
    float Rv[kLsQ], Dv[kLsQ], Xv[kLsQ], Ev[kLsQ], Lv = 0.f;
    uint8_t Cv[kLsQ];
#pragma unroll
    for (int q = 0; q < kLsQ; ++q) {
      const int i = c0 + q + 1 - lane;
      Rv[q] = 0.f;
      Dv[q] = 0.f;
      Xv[q] = 0.f;
      Ev[q] = 0.f;
      Cv[q] = 0;
      if (interior) {
        if (i >= 1 && i <= N + 1) Rv[q] = __ldcg(rowIn + (i + 1 <= S - 1 ? i + 1 : S - 1));
        if (i >= 1 && i <= N) {
          Dv[q] = __ldcg(rowDn + i);
          Xv[q] = __ldg(rowX0 + i);
          Cv[q] = __ldg(rowCode + i);
        }
        if (i == 1) Lv = __ldcg(rowIn);
      } else if (frame) {
        if (i >= 1 && i <= N) {
          Rv[q] = __ldcg(rowIn + i);
          Cv[q] = __ldg(rowCode + i);
        }
      }
      if (lane == 0 && b > 0 && i >= 1 && i <= N) Ev[q] = __ldcg(edgeIn + i);
    }

    // ---- the recurrence
#pragma unroll
    for (int q = 0; q < kLsQ; ++q) {
      const int i = c0 + q + 1 - lane;
      float U = __shfl_up_sync(FULL, g1, 1);
      if (lane == 0) U = Ev[q];
      float g;
      if (interior) {
        if (i >= 1 && i <= N) {
          const float L = (i == 1) ? Lv : g1;
          const float sum = fadd(fadd(fadd(Rv[q], L), Dv[q]), U);
          g = fmul(fadd(Xv[q], fmul(a, sum)), cr);
        } else {
          g = Rv[q];  // i == N+1: the ghost x[S-1, j] (Row-mode reflection source)
        }
      } else {
        g = Rv[q];  // frame lane: passes x[i, 0] / x[i, S-1] along
      }
      const float gdown = __shfl_down_sync(FULL, g, 1);  // lane l+1: G(i-1, j+1)

      // delayed store of column i-1 (post-boundary value)
      const int is = i - 1;
      if (interior && is >= 1 && is <= N) {
        float val = g1;
        bool store = true;
        if (MODE == kRow) {
          if (code1 & kCodeRowRight)
            val = -g;
          else if (code1 & kCodeRowLeft)
            val = -g2;
        } else if (MODE == kCol) {
          if (code1 & kCodeColUp) {
            val = -u1;
          } else if (code1 & kCodeColDown) {
            val = -gdown;
            store = (lane != 31);  // the next strip's lane 0 stores it
          }
        }
        if (store) __stcg(rowOut + is, val);
        if (MODE == kPassive) {
          if (is == 1 && rowHasFluid) __stcg(rowOut, g1);
          if (is == N && rowHasFluid) __stcg(rowOut + (S - 1), g1);
          if (firstRow && A.colfl[is]) __stcg(frameTop + is, g1);
          if (lastRow && A.colfl[is]) __stcg(frameBot + is, g1);
        }
      }
      // lane 0 stores the Column-mode reflection of the previous strip's last row
      if (MODE == kCol && lane == 0 && (interior || frame) && i >= 1 && i <= N &&
          (Cv[q] & kCodeAboveDown))
        __stcg(rowAbove + i, -g);
      // lane 31 publishes its raw row for strip b+1's lane 0
      if (lane == 31 && i >= 1 && i <= N) __stcg(edgeOut + i, g);

      // shift the per-lane history
      if (i == 1) g1 = Lv;  // so that G(i-2) is the left ghost at column 2
      g2 = g1;
      g1 = g;
      u1 = U;
      code1 = Cv[q];
    }

    // ---- publish progress: steps < c0+Q of this task are complete
    __syncwarp();
    if (lane == 0) {
      __threadfence();
      st_release_u64(progOwn, (unsigned long long)min(c0 + kLsQ, T));
    }
  }

  // ---- completion; the last task computes the corners and resets the counters
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
    for (unsigned q = lane; q < ntasks; q += 32) A.progress[q] = 0ull;
    if (lane == 0) {
      *A.ticket = 0u;
      *A.done = 0u;
    }
  }
}

}  // namespace eqk
