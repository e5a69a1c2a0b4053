// Adjoint (reverse-mode derivative) kernels of the frame step
// (fluid.rs:437-524). Every phase of step() is linear in the six arrays except
// advect's dependence on the velocity it backtraces with; the adjoint of a
// frame is the list of transposed phases in reverse order, each at the forward
// state it was applied to (fluid.rs's f32 forward, recomputed from a
// checkpoint, is the tape).
//
// Layout. Adjoint grids use the anti-diagonal layout (cell (i, j) at
// (i + j) * P + j), so that a Gauss-Seidel wavefront step touches consecutive
// addresses; the tape (forward fields) stays in the forward's pitched layout.
// Arithmetic is plain FP32 (these kernels are checked against an FP64 tape
// adjoint with a tolerance, not bit for bit).
//
// set_boundaries^T (fluid.rs:133-189, 252-272 transposed). The forward writes
// some cells from one source each: corners from two frame cells (0.5 each,
// last), Passive frame cells from the adjacent interior cell where that row /
// column holds a fluid cell, and in the velocity modes fluid cells next to a
// wall from minus that wall (right / up wins). No written cell is a source, so
// the transpose is a gather: a written cell's adjoint becomes 0, a source
// collects its writers' adjoints (negated in the velocity modes), corners
// first.
//
// lin_solve^T (fluid.rs:301-325 transposed). The K (sweep; set_boundaries)
// pairs are undone in reverse: set_boundaries^T, then the sweep transposed,
// which visits the interior in reverse lexicographic order. Its gather form:
//   y_s(q) = xbin_s(q) + alpha * (y_s(i+1, j) + y_s(i, j+1))
//   xbout_s(q) = alpha * (y_s(i-1, j) + y_s(i, j-1))        (interior q)
//   x0b(q) += (1/c) * sum_s y_s(q),   alpha = a / c,
// only interior cells counting as neighbours; a frame cell collects
// alpha * y_s of the interior cell that reads it. With xbin_s =
// set_boundaries^T(xbout_{s-1}) folded in, y_s depends on y_s one diagonal
// "behind" and on y_{s-1} at most two diagonals "ahead", so all K reverse sweeps
// run as ONE temporal wavefront inside one thread block: at step t, sweep s
// updates anti-diagonal d = 2N - t + 3s (a lag of three diagonals per sweep;
// y_s lives in the buffer of s's parity), one __syncthreads per step. The
// band of live diagonals stays in shared memory where it fits.
#pragma once
#include <cooperative_groups.h>

#include "common.cuh"
#include "kernels.cuh"
#include "wave.cuh"

namespace eqk {

__device__ __forceinline__ bool is_frame(int i, int j, int S) {
  return i == 0 || j == 0 || i == S - 1 || j == S - 1;
}

// The share of a corner's adjoint that set_boundaries^T hands to frame cell
// (i, j) (the forward's corner = 0.5 * (two adjacent frame cells)).
__device__ __forceinline__ float corner_share(const float* z, int S, int P, int i, int j) {
  float e = 0.0f;
  const int L = S - 1;
  if ((i == 1 && j == 0) || (i == 0 && j == 1)) e += 0.5f * z[dg_at(0, 0, P)];
  if ((i == 1 && j == L) || (i == 0 && j == L - 1)) e += 0.5f * z[dg_at(0, L, P)];
  if ((i == L - 1 && j == 0) || (i == L && j == 1)) e += 0.5f * z[dg_at(L, 0, P)];
  if ((i == L - 1 && j == L) || (i == L && j == L - 1)) e += 0.5f * z[dg_at(L, L, P)];
  return e;
}

// out = set_boundaries^T(z) for MODE, over the whole grid (out != z).
template <int MODE>
__global__ void k_adj_bnd(const float* __restrict__ z, float* __restrict__ out,
                          const uint8_t* __restrict__ code, const uint8_t* __restrict__ rowfl,
                          const uint8_t* __restrict__ colfl, int S, int P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= S || j >= S) return;
  const int N = S - 2;
  const size_t q = dg_at(i, j, P);
  const bool frame = is_frame(i, j, S);
  if (frame && (i == 0 || i == S - 1) && (j == 0 || j == S - 1)) {
    out[q] = 0.0f;  // a corner: handed to its two frame neighbours
    return;
  }
  auto zc = [&](int a, int b) {  // frame cell value after the corners' shares
    return z[dg_at(a, b, P)] + corner_share(z, S, P, a, b);
  };
  if (MODE == kPassive) {
    if (frame) {
      const bool written = (j == 0 || j == S - 1) ? colfl[i] != 0 : rowfl[j] != 0;
      out[q] = written ? 0.0f : zc(i, j);
    } else {
      float v = z[q];
      if (j == 1 && colfl[i]) v += zc(i, 0);
      if (j == N && colfl[i]) v += zc(i, S - 1);
      if (i == 1 && rowfl[j]) v += zc(0, j);
      if (i == N && rowfl[j]) v += zc(S - 1, j);
      out[q] = v;
    }
    return;
  }
  const uint8_t c = frame ? (uint8_t)kCodeWall : code[q];
  const uint8_t wmask = (MODE == kRow) ? kCodeRowMask : kCodeColMask;
  if (c & wmask) {
    out[q] = 0.0f;  // a fluid cell the pass overwrote
    return;
  }
  float v = frame ? zc(i, j) : z[q];
  if (c & kCodeWall) {
    auto inner = [&](int a, int b) { return a >= 1 && a <= N && b >= 1 && b <= N; };
    if (MODE == kRow) {
      if (inner(i - 1, j) && (code[dg_at(i - 1, j, P)] & kCodeRowRight)) v -= z[dg_at(i - 1, j, P)];
      if (inner(i + 1, j) && (code[dg_at(i + 1, j, P)] & kCodeRowLeft)) v -= z[dg_at(i + 1, j, P)];
    } else {
      if (inner(i, j + 1) && (code[dg_at(i, j + 1, P)] & kCodeColUp)) v -= z[dg_at(i, j + 1, P)];
      if (inner(i, j - 1) && (code[dg_at(i, j - 1, P)] & kCodeColDown)) v -= z[dg_at(i, j - 1, P)];
    }
  }
  out[q] = v;
}

struct GsAdjArgs {
  const float* B;   // set_boundaries^T of the incoming adjoint (interior read)
  float* Y0;        // y_s for even s (global form; anti-diagonal, pitch P)
  float* Y1;        // y_s for odd s
  float* Ysum;      // sum over sweeps of y_s (interior); zero on entry unless in shared memory
  float* yK;        // out: y of the last sweep (interior)
  const uint8_t* code;
  const uint8_t* rowfl;
  const uint8_t* colfl;
  int S, P, K;
  int R;            // diagonals kept in shared memory (STORE > 0)
  int m;            // cluster form: a barrier every m + 1 steps (see k_gs_adj_cl)
  float alpha;
};

// Where the wavefront keeps y and its running sum: 0 = global memory (any
// size), 1 = y in a shared-memory ring of R = 3K + 4 anti-diagonals (the band
// the active sweeps touch: every value is read at most 3 steps after it is
// written and the active diagonals span 3(K-1) + 4), the sum in global memory;
// 2 = both in shared memory (3 R S floats), the sum stored once per cell when
// its last sweep retires it.
__host__ __device__ inline size_t gs_adj_smem_bytes(int store, int S, int K) {
  const size_t R = (size_t)(3 * K + 4);
  return store == 2 ? 3 * R * S * 4 : store == 1 ? 2 * R * S * 4 : 0;
}

// The K transposed sweeps as one temporal wavefront in one block (see the
// file comment). Tasks are (sweep s, 32-cell chunk c of the positions j),
// dealt to the warps once: warp w owns tasks w, w + nwarps, ... of the list
// ordered s-fastest, and at each step runs those whose sweep is active.
// Values outside the interior count as 0 (explicit tests, so a reused ring
// slot needs no clearing).
template <int MODE, int STORE>
__global__ void __launch_bounds__(1024, 1) k_gs_adj(GsAdjArgs A) {
  extern __shared__ float gs_smem[];
  const int S = A.S, P = A.P, K = A.K, N = S - 2, D0 = 2 * N, R = A.R;
  const int nsteps = (D0 - 2) + 3 * (K - 1) + 1;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  const int ntask = K * ((N + 31) >> 5);
  const int s0 = warp % K, c0 = warp / K, ds = nwarps % K, dc = nwarps / K;
  const float al = A.alpha;
  const int st = STORE ? S : P;  // elements per diagonal
  float* const Y0 = STORE ? gs_smem : A.Y0;
  float* const Y1 = STORE ? gs_smem + (size_t)R * S : A.Y1;
  float* const Ysm = gs_smem + 2 * (size_t)R * S;  // STORE == 2
  int tb = STORE ? D0 % R : 0;  // ring slot of diagonal D0 - t
  for (int t = 0; t < nsteps; ++t) {
    const int x = t - D0 + 2;
    const int slo = x > 0 ? (x + 2) / 3 : 0;
    const int shi = min(t / 3, K - 1);
    int s = s0, c = c0;
    for (int id = warp; id < ntask; id += nwarps) {
      const int sc = s, cc = c;
      s += ds;
      c += dc;
      if (s >= K) {
        s -= K;
        ++c;
      }
      if (sc < slo || sc > shi) continue;
      const int d = D0 - t + 3 * sc;
      const int j = 1 + (cc << 5) + lane;
      if (j < d - N || j > d - 1 || j > N) continue;
      const int i = d - j;
      float* __restrict__ Yc = (sc & 1) ? Y1 : Y0;
      const float* __restrict__ Yp = (sc & 1) ? Y0 : Y1;
      // row offsets of diagonals d+1, d, d-1, d-2
      size_t op1, o0, om1, om2;
      if (STORE) {
        int r0 = tb + 3 * sc;  // 3 sc < R
        if (r0 >= R) r0 -= R;
        o0 = (size_t)r0 * st;
        op1 = (size_t)(r0 + 1 == R ? 0 : r0 + 1) * st;
        om1 = (size_t)(r0 == 0 ? R - 1 : r0 - 1) * st;
        om2 = (size_t)(r0 >= 2 ? r0 - 2 : r0 + R - 2) * st;
      } else {
        o0 = (size_t)d * st;
        op1 = o0 + st;
        om1 = o0 - st;
        om2 = o0 - 2 * st;
      }
      float v = al * ((i + 1 <= N ? Yc[op1 + j] : 0.0f) + (j + 1 <= N ? Yc[op1 + j + 1] : 0.0f));
      const size_t q = dg_at(i, j, P);
      if (sc == 0) {
        v += A.B[q];
      } else {
        const uint8_t cd = A.code[q];
        const bool written = (MODE == kRow)   ? (cd & kCodeRowMask) != 0
                             : (MODE == kCol) ? (cd & kCodeColMask) != 0
                                              : false;
        if (!written)
          v += al * ((i - 1 >= 1 ? Yp[om1 + j] : 0.0f) + (j - 1 >= 1 ? Yp[om1 + j - 1] : 0.0f));
        if (MODE == kPassive) {
          if (i == 1 || i == N || j == 1 || j == N) {
            const int n = (j == 1 && A.colfl[i]) + (j == N && A.colfl[i]) +
                          (i == 1 && A.rowfl[j]) + (i == N && A.rowfl[j]);
            v += al * (float)n * Yp[o0 + j];
          }
        } else if (cd & kCodeWall) {
          if (MODE == kRow) {
            if (i - 1 >= 1 && (A.code[dg_at(i - 1, j, P)] & kCodeRowRight))
              v -= al * ((i - 2 >= 1 ? Yp[om2 + j] : 0.0f) + (j - 1 >= 1 ? Yp[om2 + j - 1] : 0.0f));
            if (i + 1 <= N && (A.code[dg_at(i + 1, j, P)] & kCodeRowLeft))
              v -= al * (Yp[o0 + j] + (j - 1 >= 1 ? Yp[o0 + j - 1] : 0.0f));
          } else {
            if (j + 1 <= N && (A.code[dg_at(i, j + 1, P)] & kCodeColUp))
              v -= al * ((i - 1 >= 1 ? Yp[o0 + j + 1] : 0.0f) + Yp[o0 + j]);
            if (j - 1 >= 1 && (A.code[dg_at(i, j - 1, P)] & kCodeColDown))
              v -= al * ((i - 1 >= 1 ? Yp[om2 + j - 1] : 0.0f) + (j - 2 >= 1 ? Yp[om2 + j - 2] : 0.0f));
          }
        }
      }
      Yc[o0 + j] = v;
      if (STORE == 2) {
        const float sum = (sc == 0) ? v : Ysm[o0 + j] + v;
        Ysm[o0 + j] = sum;
        if (sc == K - 1) A.Ysum[q] = sum;
      } else {
        A.Ysum[q] += v;
      }
      if (sc == K - 1) A.yK[q] = v;
    }
    if (STORE && --tb < 0) tb += R;
    __syncthreads();
  }
}

// The same wavefront spread over a thread-block cluster of C blocks (one SM
// each): block r owns the positions j in [1 + r J, (r + 1) J] of every
// anti-diagonal (J = ceil(N / C)). Its shared memory holds, for its strip,
// y and its sum in a ring of R = 3K + 4 diagonals, the incoming adjoint B of
// every diagonal, and the boundary codes with one position of halo either
// side, all staged once at the start, so that a step touches no global
// memory except the final stores. The ring rows carry a halo too (positions
// jb-2, jb-1 and je+1): whoever computes a strip's first or last two
// positions also stores them into the neighbour block's halo through
// distributed shared memory, so every read is local and no remote load sits
// on a step's critical path. One cluster barrier per step orders every write,
// local or remote, before the next step's reads, in all blocks.
struct GsClLayout {  // byte offsets in one block's shared memory
  size_t ring, b, code, flags, total;
};
// Ring rows of the cluster form: the band a step touches, stretched by the
// schedule of barrier interval m + 1 (lag 2m + 3 per sweep).
__host__ __device__ inline int gs_cl_rows(int K, int m) { return (2 * m + 3) * K + 8; }
__host__ __device__ inline GsClLayout gs_cl_layout(int S, int K, int C, int m) {
  const size_t J = (size_t)((S - 2 + C - 1) / C), R = (size_t)gs_cl_rows(K, m),
               D = (size_t)(2 * S - 1);
  GsClLayout L;
  L.ring = 0;                                          // 3 R (J + 3) floats (Y0, Y1, sum)
  L.b = 3 * R * (J + 3) * 4;                           // D J floats
  L.code = L.b + D * J * 4;                            // D (J + 2) bytes
  L.flags = L.code + ((D * (J + 2) + 15) / 16) * 16;  // rowfl, colfl: 2 S bytes
  L.total = L.flags + 2 * (size_t)S;
  return L;
}

template <int MODE>
__global__ void __launch_bounds__(1024, 1) k_gs_adj_cl(GsAdjArgs A) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ __align__(16) unsigned char gs_cl_smem[];
  const int S = A.S, P = A.P, K = A.K, N = S - 2, D0 = 2 * N, R = A.R;
  const int C = (int)cluster.num_blocks(), r = (int)cluster.block_rank();
  const int J = (N + C - 1) / C, JC = J + 2, W = J + 3;
  const int jb = 1 + r * J, je = min(N, jb + J - 1);
  const GsClLayout lay = gs_cl_layout(S, K, C, A.m);
  float* const Y0 = reinterpret_cast<float*>(gs_cl_smem + lay.ring);
  float* const Y1 = Y0 + (size_t)R * W;
  float* const Ysm = Y0 + 2 * (size_t)R * W;
  // the neighbours' rings (for the halo stores)
  float* const Y0lo = r > 0 ? cluster.map_shared_rank(Y0, r - 1) : nullptr;
  float* const Y0hi = r < C - 1 ? cluster.map_shared_rank(Y0, r + 1) : nullptr;
  float* const Bs = reinterpret_cast<float*>(gs_cl_smem + lay.b);
  uint8_t* const Cs = gs_cl_smem + lay.code;
  uint8_t* const rowfl = gs_cl_smem + lay.flags;
  uint8_t* const colfl = rowfl + S;
  // stage B (own positions) and the codes (positions jb-1 .. je+1) of every diagonal
  const int nd = 2 * S - 1;
  for (int e = threadIdx.x; e < nd * JC; e += blockDim.x) {
    const int d = e / JC, k = e - d * JC, j = jb - 1 + k;
    const bool in = j >= 0 && j < S && d - j >= 0 && d - j < S;
    Cs[e] = in ? A.code[(size_t)d * P + j] : (uint8_t)0;
    if (k >= 1 && k <= J) Bs[(size_t)d * J + (k - 1)] = (in && j <= je) ? A.B[(size_t)d * P + j] : 0.0f;
  }
  for (int e = threadIdx.x; e < S; e += blockDim.x) {
    rowfl[e] = A.rowfl[e];
    colfl[e] = A.colfl[e];
  }
  auto code_at = [&](int d, int jj) { return Cs[d * JC + (jj - jb + 1)]; };
  const int nsteps = (D0 - 2) + 3 * (K - 1) + 1;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  const int ntask = K * ((J + 31) >> 5);
  const int s0 = warp % K, c0 = warp / K, ds = nwarps % K, dc = nwarps / K;
  const float al = A.alpha;
  // y at (ring slot, position j in [jb-2, je+1]) of buffer `buf`
  auto yat = [&](const float* buf, int slot, int jj) -> float {
    return buf[slot * W + (jj - jb + 2)];
  };
  int tb = D0 % R;  // ring slot of diagonal D0 - t
  cluster.sync();   // staging done; every block of the cluster runs before any remote read
  if (ntask <= nwarps) {
    // One task per warp (the usual shape): the warp's sweep and positions are
    // fixed. With m > 0 the schedule stretches: sweep s of block r updates
    // diagonal D0 - t + (2m + 3) s + m (C - 1 - r) at step t (upper blocks
    // ahead, since this sweep reads position j + 1), so every value from
    // another warp or block is at least m + 1 steps old and one cluster
    // barrier every m + 1 steps orders them. This sweep's previous-step
    // values travel in registers: (i+1, j) is this lane's last result,
    // (i, j+1) lane l+1's (a shuffle; the strip's last position reads the
    // upper block's pushed value).
    const int m = A.m, Lg = 2 * m + 3;
    const int s = warp % K, j = jb + ((warp / K) << 5) + lane;
    const bool jok = warp < ntask && j <= je;
    float* const Yc = ((s & 1) ? Y1 : Y0) + (j - jb + 2);
    const float* const Yp = ((s & 1) ? Y0 : Y1) + (j - jb + 2);
    float* const Ys = Ysm + (j - jb + 2);
    const size_t boff = (s & 1) ? (size_t)R * W : 0;
    float* const plo = (jok && j == jb && Y0lo) ? Y0lo + boff + J + 2 : nullptr;
    float* const phi = (jok && j >= je - 1 && Y0hi) ? Y0hi + boff + (j - je + 1) : nullptr;
    const bool jp1 = j + 1 <= N, jm1 = j - 1 >= 1, jm2 = j - 2 >= 1, jlast = j == je;
    const int RW = R * W;
    const int dtop = D0 + Lg * s + m * (C - 1 - r);  // this warp's diagonal at step 0
    const int nst = (D0 - 2) + Lg * (K - 1) + m * (C - 1) + 1;
    int o0 = (dtop % R) * W;
    int i = dtop - j;
    int bo = dtop * J + (j - jb);
    const unsigned Nu = (unsigned)N;
    float prev = 0.0f;
    int cnt = m;
    // The last sweep's results go to global memory one step late, after the
    // next barrier, so that no barrier's release waits for an L2 write.
    size_t pend_q = 0;
    float pend_v = 0.0f, pend_sum = 0.0f;
    bool pend = false;
    for (int t = 0; t < nst; ++t, --i, bo -= J) {
      if (pend) {
        A.Ysum[pend_q] = pend_sum;
        A.yK[pend_q] = pend_v;
        pend = false;
      }
      const float dn = __shfl_down_sync(0xffffffffu, prev, 1);
      if (jok && (unsigned)(i - 1) < Nu) {
        const int d = i + j;
        const int op1 = o0 + W == RW ? 0 : o0 + W;
        const int om1 = o0 == 0 ? RW - W : o0 - W;
        const float yr = i < N ? prev : 0.0f;                          // (i+1, j)
        const float yd = jp1 ? (jlast ? Yc[op1 + 1] : dn) : 0.0f;       // (i, j+1)
        float v = al * (yr + yd);
        if (s == 0) {
          v += Bs[bo];
        } else {
          const uint8_t cd = code_at(d, j);
          const bool written = (MODE == kRow)   ? (cd & kCodeRowMask) != 0
                               : (MODE == kCol) ? (cd & kCodeColMask) != 0
                                                : false;
          if (!written) v += al * ((i > 1 ? Yp[om1] : 0.0f) + (jm1 ? Yp[om1 - 1] : 0.0f));
          if (MODE == kPassive) {
            if (i == 1 || i == N || j == 1 || j == N) {
              const int n = (j == 1 && colfl[i]) + (j == N && colfl[i]) + (i == 1 && rowfl[j]) +
                            (i == N && rowfl[j]);
              v += al * (float)n * Yp[o0];
            }
          } else if (cd & kCodeWall) {
            const int om2 = om1 == 0 ? RW - W : om1 - W;
            if (MODE == kRow) {
              if (i > 1 && (code_at(d - 1, j) & kCodeRowRight))
                v -= al * ((i > 2 ? Yp[om2] : 0.0f) + (jm1 ? Yp[om2 - 1] : 0.0f));
              if (i < N && (code_at(d + 1, j) & kCodeRowLeft))
                v -= al * (Yp[o0] + (jm1 ? Yp[o0 - 1] : 0.0f));
            } else {
              if (jp1 && (code_at(d + 1, j + 1) & kCodeColUp))
                v -= al * ((i > 1 ? Yp[o0 + 1] : 0.0f) + Yp[o0]);
              if (jm1 && (code_at(d - 1, j - 1) & kCodeColDown))
                v -= al * ((i > 1 ? Yp[om2 - 1] : 0.0f) + (jm2 ? Yp[om2 - 2] : 0.0f));
            }
          }
        }
        Yc[o0] = v;
        if (plo) plo[o0] = v;
        if (phi) phi[o0] = v;
        const float sum = (s == 0) ? v : Ys[o0] + v;
        Ys[o0] = sum;
        if (s == K - 1) {
          pend_q = dg_at(i, j, P);
          pend_v = v;
          pend_sum = sum;
          pend = true;
        }
        prev = v;
      }
      o0 = o0 == 0 ? RW - W : o0 - W;
      if (--cnt < 0 || t == nst - 1) {
        cluster.sync();  // also the last step: no remote store may follow a block's exit
        cnt = m;
      }
    }
    if (pend) {
      A.Ysum[pend_q] = pend_sum;
      A.yK[pend_q] = pend_v;
    }
    return;
  }
  for (int t = 0; t < nsteps; ++t) {
    const int x = t - D0 + 2;
    const int slo = x > 0 ? (x + 2) / 3 : 0;
    const int shi = min(t / 3, K - 1);
    int s = s0, c = c0;
    for (int id = warp; id < ntask; id += nwarps) {
      const int sc = s, cc = c;
      s += ds;
      c += dc;
      if (s >= K) {
        s -= K;
        ++c;
      }
      if (sc < slo || sc > shi) continue;
      const int d = D0 - t + 3 * sc;
      const int j = jb + (cc << 5) + lane;
      if (j > je || j < d - N || j > d - 1) continue;
      const int i = d - j;
      float* Yc = (sc & 1) ? Y1 : Y0;
      float* Yp = (sc & 1) ? Y0 : Y1;
      int r0 = tb + 3 * sc;
      if (r0 >= R) r0 -= R;
      const int rp1 = r0 + 1 == R ? 0 : r0 + 1;
      const int rm1 = r0 == 0 ? R - 1 : r0 - 1;
      const int rm2 = r0 >= 2 ? r0 - 2 : r0 + R - 2;
      float v = al * ((i + 1 <= N ? yat(Yc, rp1, j) : 0.0f) + (j + 1 <= N ? yat(Yc, rp1, j + 1) : 0.0f));
      if (sc == 0) {
        v += Bs[(size_t)d * J + (j - jb)];
      } else {
        const uint8_t cd = code_at(d, j);
        const bool written = (MODE == kRow)   ? (cd & kCodeRowMask) != 0
                             : (MODE == kCol) ? (cd & kCodeColMask) != 0
                                              : false;
        if (!written)
          v += al * ((i - 1 >= 1 ? yat(Yp, rm1, j) : 0.0f) + (j - 1 >= 1 ? yat(Yp, rm1, j - 1) : 0.0f));
        if (MODE == kPassive) {
          if (i == 1 || i == N || j == 1 || j == N) {
            const int n = (j == 1 && colfl[i]) + (j == N && colfl[i]) + (i == 1 && rowfl[j]) +
                          (i == N && rowfl[j]);
            v += al * (float)n * yat(Yp, r0, j);
          }
        } else if (cd & kCodeWall) {
          // (i-1, j) lies on diagonal d-1, (i+1, j) and (i, j+1) on d+1, (i, j-1) on d-1
          if (MODE == kRow) {
            if (i - 1 >= 1 && (code_at(d - 1, j) & kCodeRowRight))
              v -= al * ((i - 2 >= 1 ? yat(Yp, rm2, j) : 0.0f) + (j - 1 >= 1 ? yat(Yp, rm2, j - 1) : 0.0f));
            if (i + 1 <= N && (code_at(d + 1, j) & kCodeRowLeft))
              v -= al * (yat(Yp, r0, j) + (j - 1 >= 1 ? yat(Yp, r0, j - 1) : 0.0f));
          } else {
            if (j + 1 <= N && (code_at(d + 1, j + 1) & kCodeColUp))
              v -= al * ((i - 1 >= 1 ? yat(Yp, r0, j + 1) : 0.0f) + yat(Yp, r0, j));
            if (j - 1 >= 1 && (code_at(d - 1, j - 1) & kCodeColDown))
              v -= al * ((i - 1 >= 1 ? yat(Yp, rm2, j - 1) : 0.0f) + (j - 2 >= 1 ? yat(Yp, rm2, j - 2) : 0.0f));
          }
        }
      }
      const int lo = r0 * W + (j - jb + 2);
      Yc[lo] = v;
      // halo copies: my first position is the lower neighbour's je+1 (index
      // J+2 there), my last two its upper neighbour's jb-1, jb-2 (1, 0)
      const size_t boff = (sc & 1) ? (size_t)R * W : 0;
      if (j == jb && Y0lo) Y0lo[boff + r0 * W + J + 2] = v;
      if (j >= je - 1 && Y0hi) Y0hi[boff + r0 * W + (j - je + 1)] = v;
      const float sum = (sc == 0) ? v : Ysm[lo] + v;
      Ysm[lo] = sum;
      if (sc == K - 1) {
        const size_t q = dg_at(i, j, P);
        A.Ysum[q] = sum;
        A.yK[q] = v;
      }
    }
    if (--tb < 0) tb += R;
    cluster.sync();
  }
}

// After the wavefront: the adjoint of x before the solve (out, whole grid) and
// x0b += (1/c) * sum_s y_s. `bt` is set_boundaries^T of the incoming adjoint
// (what frame cells keep), yK the last sweep's y.
template <int MODE>
__global__ void k_gs_adj_out(float* __restrict__ out, const float* __restrict__ bt,
                             const float* __restrict__ yK, const float* __restrict__ ysum,
                             float* __restrict__ x0b, const uint8_t* __restrict__ code,
                             const uint8_t* __restrict__ rowfl, const uint8_t* __restrict__ colfl,
                             int S, int P, float alpha, float cr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= S || j >= S) return;
  const size_t q = dg_at(i, j, P);
  const int N = S - 2;
  if (!is_frame(i, j, S)) {
    out[q] = alpha * (yK[q - P] + yK[q - P - 1]);
    x0b[q] += cr * ysum[q];
    return;
  }
  if ((i == 0 || i == S - 1) && (j == 0 || j == S - 1)) {
    out[q] = bt[q];
    return;
  }
  // the interior cell that reads this frame cell
  const int ci = (i == 0) ? 1 : (i == S - 1) ? N : i;
  const int cj = (j == 0) ? 1 : (j == S - 1) ? N : j;
  const size_t cq = dg_at(ci, cj, P);
  if (MODE == kPassive) {
    const bool written = (j == 0 || j == S - 1) ? colfl[i] != 0 : rowfl[j] != 0;
    out[q] = written ? alpha * yK[cq] : bt[q] + alpha * ysum[cq];
    return;
  }
  float v = bt[q] + alpha * ysum[cq];
  const uint8_t c = code[cq];
  const bool take = (MODE == kRow) ? ((i == 0 && (c & kCodeRowLeft)) || (i == S - 1 && (c & kCodeRowRight)))
                                   : ((j == 0 && (c & kCodeColUp)) || (j == S - 1 && (c & kCodeColDown)));
  if (take)  // every sweep but the last handed the reading cell's xbout here
    v -= alpha * ((ysum[cq - P] - yK[cq - P]) + (ysum[cq - P - 1] - yK[cq - P - 1]));
  out[q] = v;
}

// advect^T (fluid.rs:378-432 transposed), one block per interior row j, after
// set_boundaries^T of db: replay the row's backtraces to find its break; the
// break cell hands its adjoint to its left neighbour (the old ghost for i = 1);
// cells before it scatter into d0b (transposed bilinear) and, unless clamped,
// into ub / vb (the interpolant's derivative w.r.t. the backtrace) and become
// 0; cells after it keep theirs. d0, u, v: the forward's fields (pitched, Pp).
// The scatter targets may alias each other: every add is atomic.
__global__ void k_adv_adj_rows(float* __restrict__ db, float* d0b, float* ub, float* vb,
                               const float* __restrict__ d0, const float* __restrict__ u,
                               const float* __restrict__ v, int S, int Pp, int P, float dt0) {
  const int j = blockIdx.x + 1;
  const int N = S - 2;
  __shared__ int s_brk;
  if (threadIdx.x == 0) s_brk = 0x7fffffff;
  __syncthreads();
  const size_t row = (size_t)j * Pp;
  int mine = 0x7fffffff;
  for (int i = threadIdx.x + 1; i <= N; i += blockDim.x) {
    if (backtrace(i, j, u[row + i], v[row + i], dt0, S).brk) {
      mine = i;
      break;
    }
  }
  if (mine != 0x7fffffff) atomicMin(&s_brk, mine);
  __syncthreads();
  const int brk = s_brk;
  if (threadIdx.x == 0 && brk <= N) {
    const float g = db[dg_at(brk, j, P)];
    db[dg_at(brk, j, P)] = 0.0f;
    db[dg_at(brk - 1, j, P)] += g;
  }
  __syncthreads();
  const float hi = fsub((float)S, 1.0f);
  for (int i = threadIdx.x + 1; i <= N && i < brk; i += blockDim.x) {
    const size_t q = dg_at(i, j, P);
    const float g = db[q];
    db[q] = 0.0f;
    if (g == 0.0f) continue;
    const float ui = u[row + i], vi = v[row + i];
    const Backtrace b = backtrace(i, j, ui, vi, dt0, S);
    const float A = d0[(size_t)b.j0 * Pp + b.i0], B = d0[(size_t)b.j1 * Pp + b.i0];
    const float C = d0[(size_t)b.j0 * Pp + b.i1], D = d0[(size_t)b.j1 * Pp + b.i1];
    atomicAdd(d0b + dg_at(b.i0, b.j0, P), b.s0 * b.t0 * g);
    atomicAdd(d0b + dg_at(b.i0, b.j1, P), b.s0 * b.t1 * g);
    atomicAdd(d0b + dg_at(b.i1, b.j0, P), b.s1 * b.t0 * g);
    atomicAdd(d0b + dg_at(b.i1, b.j1, P), b.s1 * b.t1 * g);
    const float xr = fsub((float)i, fmul(dt0, ui)), yr = fsub((float)j, fmul(dt0, vi));
    if (!(xr < 0.5f || xr > hi))
      atomicAdd(ub + q, -dt0 * g * ((b.t0 * C + b.t1 * D) - (b.t0 * A + b.t1 * B)));
    if (!(yr < 0.5f || yr > hi))
      atomicAdd(vb + q, -dt0 * g * (b.s0 * (B - A) + b.s1 * (D - C)));
  }
}

// project's gradient subtraction transposed (fluid.rs:364-371): the pressure
// adjoint gathers the interior velocity adjoints that read it.
__global__ void k_grad_adj(const float* __restrict__ vxb, const float* __restrict__ vyb,
                           float* __restrict__ pb, int S, int P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= S || j >= S) return;
  const int N = S - 2;
  auto inner = [&](int a, int b) { return a >= 1 && a <= N && b >= 1 && b <= N; };
  const float h = 0.5f * (float)S;
  float v = 0.0f;
  if (inner(i - 1, j)) v -= vxb[dg_at(i - 1, j, P)];
  if (inner(i + 1, j)) v += vxb[dg_at(i + 1, j, P)];
  if (inner(i, j - 1)) v -= vyb[dg_at(i, j - 1, P)];
  if (inner(i, j + 1)) v += vyb[dg_at(i, j + 1, P)];
  pb[dg_at(i, j, P)] += h * v;
}

// project's divergence transposed (fluid.rs:340-351): the velocity adjoints
// gather w = -0.5 * divb / size of the interior cells that read them.
__global__ void k_div_adj(float* __restrict__ vxb, float* __restrict__ vyb,
                          const float* __restrict__ divb, int S, int P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= S || j >= S) return;
  const int N = S - 2;
  auto inner = [&](int a, int b) { return a >= 1 && a <= N && b >= 1 && b <= N; };
  const float k = -0.5f / (float)S;
  float gx = 0.0f, gy = 0.0f;
  if (inner(i - 1, j)) gx += divb[dg_at(i - 1, j, P)];
  if (inner(i + 1, j)) gx -= divb[dg_at(i + 1, j, P)];
  if (inner(i, j - 1)) gy += divb[dg_at(i, j - 1, P)];
  if (inner(i, j + 1)) gy -= divb[dg_at(i, j + 1, P)];
  const size_t q = dg_at(i, j, P);
  vxb[q] += k * gx;
  vyb[q] += k * gy;
}

// Interior of a and b set to 0 (project overwrote p and div there).
__global__ void k_zero_interior2(float* __restrict__ a, float* __restrict__ b, int S, int P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > S - 2 || j > S - 2) return;
  a[dg_at(i, j, P)] = 0.0f;
  b[dg_at(i, j, P)] = 0.0f;
}

// scratch = density.clone() transposed: db += sb; sb = 0 (whole grid).
__global__ void k_adj_clone(float* __restrict__ db, float* __restrict__ sb, int S, int P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= S || j >= S) return;
  const size_t q = dg_at(i, j, P);
  db[q] += sb[q];
  sb[q] = 0.0f;
}

// Layout moves: dense S x S (x fastest) <-> anti-diagonal; with `b`, the
// dense output is a + b (the source field's adjoint: density + scratch).
__global__ void k_diag_to_dense(const float* __restrict__ a, const float* __restrict__ b,
                                float* __restrict__ out, int S, int P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= S || j >= S) return;
  const size_t q = dg_at(i, j, P);
  out[(size_t)j * S + i] = b ? a[q] + b[q] : a[q];
}
__global__ void k_dense_to_diag(const float* __restrict__ in, float* __restrict__ out, int S,
                                int P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= S || j >= S) return;
  out[dg_at(i, j, P)] = in[(size_t)j * S + i];
}
__global__ void k_code_to_diag(const uint8_t* __restrict__ in, int Pp, uint8_t* __restrict__ out,
                               int S, int P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= S || j >= S) return;
  out[dg_at(i, j, P)] = in[(size_t)j * Pp + i];
}

// The per-frame source field added to density and scratch at every cell
// (add_density at each cell, fluid.rs:120-124), pitched grids, dense source.
__global__ void k_add_src(float* __restrict__ de, float* __restrict__ sc,
                          const float* __restrict__ src, int S, int Pp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= S || j >= S) return;
  const size_t q = (size_t)j * Pp + i;
  const float s = src[(size_t)j * S + i];
  de[q] = fadd(de[q], s);
  sc[q] = fadd(sc[q], s);
}

// loss = 0.5 * sum over the interior of (density - target)^2 (FP64 sum) and
// its adjoint w.r.t. density (anti-diagonal, zero outside the interior).
__global__ void k_l2_loss(const float* __restrict__ de, int Pp, const float* __restrict__ target,
                          float* __restrict__ adj, int S, int P, double* __restrict__ loss) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  double part = 0.0;
  if (i < S && j < S) {
    float e = 0.0f;
    if (!is_frame(i, j, S)) {
      e = de[(size_t)j * Pp + i] - target[(size_t)j * S + i];
      part = 0.5 * (double)e * (double)e;
    }
    adj[dg_at(i, j, P)] = e;
  }
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0 && part != 0.0) atomicAdd(loss, part);
}

}  // namespace eqk
