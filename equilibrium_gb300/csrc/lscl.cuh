// lin_solve (fluid.rs:301-325) over a thread-block cluster, bit-exactly: the
// K lexicographic Gauss-Seidel sweeps as one temporal wavefront on
// anti-diagonals, sweep k updating diagonal d = t + 2 - L k (- m r, below) at
// step t.
//
// The sweep-k value of interior cell (i, j) is
//   raw_k(i, j) = (x0 + a*(((R + L) + D) + U)) * (1/c)
// with L = raw_k(i-1, j) and U = raw_k(i, j-1) (this sweep, one diagonal
// back) and R = post_{k-1}(i+1, j), D = post_{k-1}(i, j+1) (the previous
// sweep after its set_boundaries, one diagonal ahead). set_boundaries is read
// as a gather: a fluid cell that the velocity modes overwrite is minus its
// wall neighbour's raw value (the frame's initial value for a frame wall);
// a Passive frame cell is the adjacent interior cell's raw value where its
// row / column holds a fluid cell, else its initial value; every other cell
// is its raw value (sweep -1: the initial x). Reads reach two diagonals
// ahead, hence a lag L of at least three diagonals per sweep. The last sweep's raw
// values are written back and the caller's set_boundaries pass makes them
// the reference's array (corners included).
//
// Block r of the cluster owns positions j in [1 + rJ, (r + 1)J] of every
// diagonal, with its strip of x0, of the initial x and of the codes (one
// position below, two above) staged in shared memory, and the band of raw
// values in a ring of R = L K + 8 diagonals per sweep parity; the strip-edge
// values it computes are pushed into the neighbours' halos through
// distributed shared memory. A warp owns one sweep and the 32 positions of
// its block's strip (requires J <= 32 and K <= 32); the same sweep's
// neighbour values of the previous step travel in registers and shuffles.
// The final values replace x0 in shared memory and are stored after the last
// step.
//
// Synchronisation. With a lag of L = 2m + 3 diagonals per sweep and block r
// running m steps behind block r-1 (sweep k of block r updates diagonal
// t + 2 - L k - m r at step t), every value a warp reads from another warp or
// block was written at least m + 1 steps earlier, so one cluster barrier
// every m + 1 steps orders all of them (a value from the same warp's previous
// step comes in a register or a shuffle); no ring row is rewritten before its
// last read. m = 0 is a barrier per step.
#pragma once
#include <cooperative_groups.h>

#include "common.cuh"

namespace eqk {

constexpr uint8_t kSpecial = 128u;  // staged-code bit: the cell needs the boundary gathers

struct LsClArgs {
  float* x;            // in: initial x; out: last sweep's raw interior values
  const float* x0;
  const uint8_t* code;  // pitched boundary codes
  const uint8_t* rowfl;
  const uint8_t* colfl;
  int S, P, K, R;
  int m;  // a cluster barrier every m + 1 steps; lag 2m + 3, skew m per block
  float a, cr;
  const uint8_t* strip;  // the streamed form's strip-ordered codes (lscs.cuh)
};

struct LsClLayout {  // byte offsets in one block's shared memory
  size_t ring, x0, xi, code, flags, total;
};
__host__ __device__ inline int ls_cl_rows(int K, int m) { return (2 * m + 3) * K + 8; }
__host__ __device__ inline LsClLayout ls_cl_layout(int S, int K, int C, int m) {
  const size_t J = (size_t)((S - 2 + C - 1) / C), W = J + 3, R = (size_t)ls_cl_rows(K, m),
               D = (size_t)(2 * S - 1);
  LsClLayout L;
  L.ring = 0;                        // 2 R W floats
  L.x0 = 2 * R * W * 4;              // D J floats (then the final values)
  L.xi = L.x0 + D * J * 4;           // D W floats
  L.code = L.xi + D * W * 4;         // D W bytes
  L.flags = L.code + ((D * W + 15) / 16) * 16;
  L.total = L.flags + 2 * (size_t)S;
  return L;
}

template <int MODE>
__global__ void __launch_bounds__(1024, 1) k_ls_cl(LsClArgs A) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ __align__(16) unsigned char ls_cl_smem[];
  const int S = A.S, P = A.P, K = A.K, N = S - 2, D0 = 2 * N, R = A.R, m = A.m;
  const int Lg = 2 * m + 3, sig = m;
  const int C = (int)cluster.num_blocks(), r = (int)cluster.block_rank();
  const int J = (N + C - 1) / C, W = J + 3, nd = 2 * S - 1;
  const int jb = 1 + r * J, je = min(N, jb + J - 1);
  const LsClLayout lay = ls_cl_layout(S, K, C, m);
  float* const Y0 = reinterpret_cast<float*>(ls_cl_smem + lay.ring);
  float* const Y1 = Y0 + (size_t)R * W;
  float* const X0 = reinterpret_cast<float*>(ls_cl_smem + lay.x0);
  float* const XI = reinterpret_cast<float*>(ls_cl_smem + lay.xi);
  uint8_t* const CS = ls_cl_smem + lay.code;
  uint8_t* const rowfl = ls_cl_smem + lay.flags;
  uint8_t* const colfl = rowfl + S;
  // stage x0 (own positions), the initial x and the codes (jb-1 .. je+2)
  for (int e = threadIdx.x; e < nd * W; e += blockDim.x) {
    const int d = e / W, k = e - d * W, j = jb - 1 + k, i = d - j;
    const bool in = j >= 0 && j < S && i >= 0 && i < S;
    const size_t q = (size_t)j * P + i;
    XI[e] = in ? A.x[q] : 0.0f;
    CS[e] = in ? A.code[q] : (uint8_t)0;
    if (k >= 1 && k <= J) X0[(size_t)d * J + (k - 1)] = (in && j <= je) ? A.x0[q] : 0.0f;
  }
  for (int e = threadIdx.x; e < S; e += blockDim.x) {
    rowfl[e] = A.rowfl[e];
    colfl[e] = A.colfl[e];
  }
  __syncthreads();
  // kSpecial on an own interior cell whose update needs more than plain reads
  // of its four neighbours: a neighbour on the frame, or (velocity modes) an
  // R or D neighbour that set_boundaries overwrites
  for (int e = threadIdx.x; e < nd * J; e += blockDim.x) {
    const int d = e / J, jj = jb + (e - d * J), i = d - jj, cc = jj - jb + 1;
    if (jj > je || i < 1 || i > N) continue;
    const uint8_t wm = (MODE == kRow) ? kCodeRowMask : (MODE == kCol) ? kCodeColMask : 0;
    bool sp = i == 1 || jj == 1 || i == N || jj == N;
    if (wm && ((CS[(d + 1) * W + cc] & wm) || (CS[(d + 1) * W + cc + 1] & wm))) sp = true;
    if (sp) CS[d * W + cc] |= kSpecial;
  }
  float* const Y0lo = r > 0 ? cluster.map_shared_rank(Y0, r - 1) : nullptr;
  float* const Y0hi = r < C - 1 ? cluster.map_shared_rank(Y0, r + 1) : nullptr;
  const int nsteps = (D0 - 2) + Lg * (K - 1) + sig * (C - 1) + 1;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k = warp;  // this warp's sweep (one 32-position chunk: J <= 32)
  const int j = jb + lane;
  const bool jok = k < K && j <= je;
  const int col = j - jb + 1;  // column of position j in ring rows, XI and CS
  float* const Yc = (k & 1) ? Y1 : Y0;
  const float* const Yp = (k & 1) ? Y0 : Y1;
  const size_t boff = (k & 1) ? (size_t)R * W : 0;
  // my first two positions are the lower neighbour's je+1, je+2 (columns
  // J+1, J+2 there); my last one the upper neighbour's jb-1 (column 0)
  float* const plo = (jok && j <= jb + 1 && Y0lo) ? Y0lo + boff + (J + 1 + (j - jb)) : nullptr;
  float* const phi = (jok && j == je && Y0hi) ? Y0hi + boff : nullptr;
  const float a = A.a, cr = A.cr;
  const int RW = R * W;
  // ring row of diagonal t + 2 - Lg k - sig r at step t (negative: no row until valid)
  const int dstart = 2 - Lg * k - sig * r;
  int o0 = ((dstart % R + R) % R) * W;
  // the value of frame cell (fi, fj) after sweep k-1's set_boundaries
  auto frame_post = [&](int fi, int fj, int km, const float* yp, int orow_adj, int col_adj,
                        int dg, int colf) -> float {
    if (MODE == kPassive && km >= 0) {
      const bool written = (fj == 0 || fj == S - 1) ? colfl[fi] != 0 : rowfl[fj] != 0;
      if (written) return yp[orow_adj + col_adj];
    }
    return XI[dg * W + colf];
  };
  // the value of interior cell (ci, cj) (on diagonal dg, at ring row orow and
  // column cc) after sweep k-1's set_boundaries; rows +-1 around it
  auto interior_post = [&](int ci, int cj, int dg, int orow, int cc, int orow_p1, int orow_m1)
      -> float {
    if (k == 0) return XI[dg * W + cc];
    const uint8_t cd = CS[dg * W + cc];
    int si = -1, sj = -1, so = 0, sc = 0;
    if (MODE == kRow) {
      if (cd & kCodeRowRight) { si = ci + 1; sj = cj; so = orow_p1; sc = cc; }
      else if (cd & kCodeRowLeft) { si = ci - 1; sj = cj; so = orow_m1; sc = cc; }
    } else if (MODE == kCol) {
      if (cd & kCodeColUp) { si = ci; sj = cj - 1; so = orow_m1; sc = cc - 1; }
      else if (cd & kCodeColDown) { si = ci; sj = cj + 1; so = orow_p1; sc = cc + 1; }
    }
    if (si < 0) return Yp[orow + cc];
    const bool fr = si == 0 || sj == 0 || si == S - 1 || sj == S - 1;
    const int sdg = si + sj;
    return -(fr ? XI[sdg * W + sc] : Yp[so + sc]);
  };
  cluster.sync();  // staging done; every block runs before any remote store
  // This sweep's previous-step values travel in registers: L = (i-1, j) is
  // this lane's own last result, U = (i, j-1) lane l-1's (a shuffle; lane 0
  // reads the lower block's pushed value, written m + 1 or more steps ago).
  // So no step needs a warp-level memory fence between the barriers.
  float prev = 0.0f;
  // per-step offsets, advanced incrementally (negative until the warp's
  // first diagonal; nothing is read before its cell is valid)
  int i = dstart - j;                        // column of this lane's cell
  int cso = dstart * W + col;                // its staged code
  int x0o = dstart * J + (j - jb);           // its staged x0
  int cnt = m;                               // steps until the next barrier
  const unsigned Nu = (unsigned)N;
  for (int t = 0; t < nsteps; ++t, ++i, cso += W, x0o += J) {
    const float up = __shfl_up_sync(0xffffffffu, prev, 1);
    if (jok && (unsigned)(i - 1) < Nu) {
      const int op1 = o0 + W == RW ? 0 : o0 + W;
      const int om1 = o0 == 0 ? RW - W : o0 - W;
      const float Ur = lane > 0 ? up : Yc[om1 + col - 1];
      float L, U, Rv, Dv;
      if (!(CS[cso] & kSpecial)) {
        // the common case: plain reads (R, D: the previous sweep at d+1, or
        // the initial x for the first sweep)
        L = prev;
        U = Ur;
        if (k > 0) {
          Rv = Yp[op1 + col];
          Dv = Yp[op1 + col + 1];
        } else {
          Rv = XI[cso + W];
          Dv = XI[cso + W + 1];
        }
      } else {
        const int d = i + j;
        const int op2 = op1 + W == RW ? 0 : op1 + W;
        // L = (i-1, j), U = (i, j-1): this sweep, diagonal d-1
        L = (i > 1) ? prev : frame_post(0, j, k - 1, Yp, o0, col, d - 1, col);
        U = (j > 1) ? Ur : frame_post(i, 0, k - 1, Yp, o0, col, d - 1, col - 1);
        // R = (i+1, j), D = (i, j+1): sweep k-1 after its bnd, diagonal d+1
        Rv = (i < N) ? interior_post(i + 1, j, d + 1, op1, col, op2, o0)
                     : frame_post(S - 1, j, k - 1, Yp, o0, col, d + 1, col);
        Dv = (j < N) ? interior_post(i, j + 1, d + 1, op1, col + 1, op2, o0)
                     : frame_post(i, S - 1, k - 1, Yp, o0, col, d + 1, col + 1);
      }
      const float sum = fadd(fadd(fadd(Rv, L), Dv), U);
      const float v = fmul(fadd(X0[x0o], fmul(a, sum)), cr);
      Yc[o0 + col] = v;
      if (plo) plo[o0] = v;
      if (phi) phi[o0] = v;
      if (k == K - 1) X0[x0o] = v;  // x0 of this cell is no longer read
      prev = v;
    }
    o0 = o0 + W == RW ? 0 : o0 + W;
    if (--cnt < 0 || t == nsteps - 1) {
      cluster.sync();  // also the last step: no remote store may follow a block's exit
      cnt = m;
    }
  }
  // the last sweep's raw values back to x (own positions, interior)
  for (int e = threadIdx.x; e < nd * J; e += blockDim.x) {
    const int d = e / J, jj = jb + (e - d * J), i = d - jj;
    if (jj <= je && i >= 1 && i <= N) A.x[(size_t)jj * P + i] = X0[e];
  }
}

}  // namespace eqk
