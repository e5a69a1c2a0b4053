// lin_solve (fluid.rs:301-325) over a thread-block cluster for grids whose
// strips do not fit in shared memory whole: the temporal wavefront of
// lscl.cuh (same schedule, same arithmetic, bit-exact) with x0, the initial x
// and the codes streamed through rings instead of staged up front.
//
// Schedule (as lscl.cuh). Sweep k of block r updates diagonal
// d = t + 2 - L k - m r at step t, L = 2m + 3; one cluster barrier every
// m + 1 steps orders every cross-warp and cross-block value.
//
// Streaming. A loader warp (warp K) issues, at step t, asynchronous copies of
// diagonal e = t + (2m + 6) - m r into ring row e mod R: the initial x of
// positions jb-1 .. je+2, x0 of the block's own positions, and the codes of
// the same positions from a strip-ordered copy in which kSpecial is already
// set (k_ls_cs_codes). It commits one copy group per barrier interval and,
// before each barrier, waits for the previous interval's group, so a row is
// readable two intervals after it was issued; the first sweep first reads
// diagonal e (as its d + 2) 2m + 2 steps after the issue. The last sweep
// reads down to diagonal t + 1 - L (K-1) - m r, and the rings' R = L K + 8
// rows (m <= 3) keep every row until its last read has passed a barrier
// before the copy that overwrites it is issued. The rings share the value
// ring's row index and width (padded to a multiple of 4), so a diagonal's
// offset is the same in all of them.
//
// Positions. A warp owns one sweep and H positions per lane: lane l holds
// positions jb + l + 32h, h < H (J <= 32 H). The same sweep's previous-step
// values travel in registers and shuffles: U of position (h, l) is (h, l-1)'s
// previous value, (h-1, 31)'s for l = 0, h > 0, and for (0, 0) the lower
// block's pushed halo value.
//
// The last sweep writes its raw values of interior cells straight to x. The
// staged initial x is read at the block's own positions, at je + 1 (the
// upper neighbour's first position, which that block, m steps behind,
// writes later) and on the frame (never written); the lower halo column is
// read only at the frame, its other values arriving by the neighbour's push.
// Every copy that is read lands before its cell's write (checked on the CPU
// with these step formulas), and the caller's set_boundaries pass then makes
// x the reference's array.
#pragma once
#include <cooperative_groups.h>

#include "common.cuh"
#include "lscl.cuh"

namespace eqk {

// Ring row width (floats / bytes) for strips of J positions: J + 3 columns
// (one below, two above), padded to a multiple of 4.
__host__ __device__ inline int ls_cs_width(int J) { return ((J + 3 + 3) / 4) * 4; }

struct LsCsLayout {  // byte offsets in one block's shared memory
  size_t ring, xi, x0, code, flags, total;
};
__host__ __device__ inline LsCsLayout ls_cs_layout(int S, int K, int C, int m) {
  const size_t J = (size_t)((S - 2 + C - 1) / C), W = (size_t)ls_cs_width((int)J),
               R = (size_t)ls_cl_rows(K, m);
  LsCsLayout L;
  L.ring = 0;                     // 2 R W floats: the values, per sweep parity
  L.xi = L.ring + 2 * R * W * 4;  // R W floats: the initial x
  L.x0 = L.xi + R * W * 4;        // R J floats: x0 of own positions
  L.code = L.x0 + R * J * 4;      // R W bytes: codes (+ kSpecial)
  L.flags = L.code + ((R * W + 15) / 16) * 16;
  L.total = L.flags + 2 * (size_t)S;
  return L;
}

// Bytes of one mode's strip-ordered codes: (2S - 1) diagonals x C strips x W.
__host__ __device__ inline size_t ls_cs_strip_bytes(int S, int C, int J) {
  return (size_t)(2 * S - 1) * C * ls_cs_width(J);
}

// The codes of every block strip, diagonal by diagonal ([e][r][c]: position
// jb(r) - 1 + c of diagonal e, 0 outside the grid), with kSpecial set on own
// interior cells whose update needs more than plain reads of their four
// neighbours: a neighbour on the frame, or (velocity modes) an R or D
// neighbour that set_boundaries overwrites.
template <int MODE>
__global__ void k_ls_cs_codes(uint8_t* __restrict__ strip, const uint8_t* __restrict__ code, int S,
                              int P, int C, int J) {
  const int N = S - 2, W = ls_cs_width(J);
  const size_t total = (size_t)(2 * S - 1) * C * W;
  const uint8_t wm = (MODE == kRow) ? kCodeRowMask : (MODE == kCol) ? kCodeColMask : 0;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < total;
       q += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(q % W);
    const size_t er = q / W;
    const int r = (int)(er % C), e = (int)(er / C);
    const int jb = 1 + r * J, je = min(N, jb + J - 1);
    const int j = jb - 1 + c, i = e - j;
    uint8_t v = 0;
    if (c < J + 3 && j >= 0 && j < S && i >= 0 && i < S) {
      v = code[(size_t)j * P + i];
      if (c >= 1 && c <= J && j <= je && i >= 1 && i <= N) {
        bool sp = i == 1 || j == 1 || i == N || j == N;
        if (wm && ((code[(size_t)j * P + i + 1] & wm) || (code[(size_t)(j + 1) * P + i] & wm)))
          sp = true;
        if (sp) v |= kSpecial;
      }
    }
    strip[q] = v;
  }
}

template <int MODE, int H>
__global__ void __launch_bounds__(1024, 1) k_ls_cs(LsClArgs A) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ __align__(16) unsigned char ls_cs_smem[];
  const int S = A.S, P = A.P, K = A.K, N = S - 2, D0 = 2 * N, R = A.R, m = A.m;
  const int Lg = 2 * m + 3, sig = m, lead = 2 * m + 6;
  const int C = (int)cluster.num_blocks(), r = (int)cluster.block_rank();
  const int J = (N + C - 1) / C, W = ls_cs_width(J);
  const int jb = 1 + r * J, je = min(N, jb + J - 1);
  const LsCsLayout lay = ls_cs_layout(S, K, C, m);
  float* const Y0 = reinterpret_cast<float*>(ls_cs_smem + lay.ring);
  float* const Y1 = Y0 + (size_t)R * W;
  float* const XI = reinterpret_cast<float*>(ls_cs_smem + lay.xi);
  float* const X0 = reinterpret_cast<float*>(ls_cs_smem + lay.x0);
  uint8_t* const CS = ls_cs_smem + lay.code;
  uint8_t* const rowfl = ls_cs_smem + lay.flags;
  uint8_t* const colfl = rowfl + S;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int RW = R * W;
  const int nd = 2 * S - 1;
  for (int e = threadIdx.x; e < S; e += blockDim.x) {
    rowfl[e] = A.rowfl[e];
    colfl[e] = A.colfl[e];
  }
  // ---- the loader warp: issue the copies of diagonal e (zeros outside)
  auto stage = [&](int e) {
    if (e < 0 || e >= nd) return;
    const int row = e % R;
    float* const xr = XI + (size_t)row * W;
    float* const x0r = X0 + (size_t)row * J;
    for (int c = lane; c < J + 3; c += 32) {
      const int j = jb - 1 + c, i = e - j;
      const bool in = j >= 0 && j < S && i >= 0 && i < S;
      const size_t q = in ? (size_t)j * P + i : 0;
      if (in)
        cp_async4(&xr[c], A.x + q, true);
      else
        xr[c] = 0.0f;
      if (c >= 1 && c <= J) {
        if (in && j <= je)
          cp_async4(&x0r[c - 1], A.x0 + q, true);
        else
          x0r[c - 1] = 0.0f;
      }
    }
    const uint8_t* src = A.strip + ((size_t)e * C + r) * W;
    uint8_t* const crw = CS + (size_t)row * W;
    for (int w = lane; w < W / 4; w += 32) cp_async4(crw + 4 * w, src + 4 * w, true);
  };
  if (warp == K) {
    for (int t = -lead; t < 0; ++t) stage(t + lead - sig * r);
    cp_async_commit();
    cp_async_wait<0>();
  }
  float* const Y0lo = r > 0 ? cluster.map_shared_rank(Y0, r - 1) : nullptr;
  float* const Y0hi = r < C - 1 ? cluster.map_shared_rank(Y0, r + 1) : nullptr;
  const int nsteps = (D0 - 2) + Lg * (K - 1) + sig * (C - 1) + 1;
  const int k = warp;  // this warp's sweep (warp K: the loader)
  const bool sweeper = k < K;
  float* const Yc = (k & 1) ? Y1 : Y0;
  const float* const Yp = (k & 1) ? Y0 : Y1;
  const size_t boff = (k & 1) ? (size_t)R * W : 0;
  int jj[H], col[H];
  bool jok[H];
  float* plo[H];
  float* phi[H];
#pragma unroll
  for (int h = 0; h < H; ++h) {
    jj[h] = jb + lane + 32 * h;
    col[h] = jj[h] - jb + 1;  // column of the position in ring rows
    jok[h] = sweeper && jj[h] <= je;
    // the first two positions are the lower neighbour's je+1, je+2 (columns
    // J+1, J+2 there); the last one the upper neighbour's jb-1 (column 0)
    plo[h] = (jok[h] && jj[h] <= jb + 1 && Y0lo) ? Y0lo + boff + (J + 1 + (jj[h] - jb)) : nullptr;
    phi[h] = (jok[h] && jj[h] == je && Y0hi) ? Y0hi + boff : nullptr;
  }
  const float a = A.a, cr = A.cr;
  // ring row of diagonal t + 2 - Lg k - sig r at step t
  const int dstart = 2 - Lg * k - sig * r;
  int o0 = ((dstart % R + R) % R) * W;
  int xo = (o0 / W) * J;  // the same row in the x0 ring
  // the value of frame cell (fi, fj) after sweep k-1's set_boundaries; xoff:
  // its staged initial value
  auto frame_post = [&](int fi, int fj, int km, const float* yp, int orow_adj, int col_adj,
                        int xoff) -> float {
    if (MODE == kPassive && km >= 0) {
      const bool written = (fj == 0 || fj == S - 1) ? colfl[fi] != 0 : rowfl[fj] != 0;
      if (written) return yp[orow_adj + col_adj];
    }
    return XI[xoff];
  };
  // the value of interior cell (ci, cj) (at ring row orow, column cc) after
  // sweep k-1's set_boundaries; rows of the diagonals +-1 around it
  auto interior_post = [&](int ci, int cj, int orow, int cc, int orow_p1, int orow_m1) -> float {
    if (k == 0) return XI[orow + cc];
    const uint8_t cd = CS[orow + cc];
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
    return -(fr ? XI[so + sc] : Yp[so + sc]);
  };
  cluster.sync();  // first rows staged; every block runs before any remote store
  float prev[H];
#pragma unroll
  for (int h = 0; h < H; ++h) prev[h] = 0.0f;
  int i0 = dstart - jj[0];  // column of position h's cell: i0 - 32 h
  int cnt = m;              // steps until the next barrier
  const unsigned Nu = (unsigned)N;
  for (int t = 0; t < nsteps; ++t, ++i0) {
    if (!sweeper) {
      stage(t + lead - sig * r);
    } else {
      float up[H];
#pragma unroll
      for (int h = 0; h < H; ++h) up[h] = __shfl_up_sync(0xffffffffu, prev[h], 1);
      const float x31 = H > 1 ? __shfl_sync(0xffffffffu, prev[0], 31) : 0.0f;
      const int op1 = o0 + W == RW ? 0 : o0 + W;
      const int om1 = o0 == 0 ? RW - W : o0 - W;
#pragma unroll
      for (int h = 0; h < H; ++h) {
        const int i = i0 - 32 * h;
        const int j = jj[h], cl = col[h];
        if (jok[h] && (unsigned)(i - 1) < Nu) {
          const float Ur = lane > 0 ? up[h] : (h == 0 ? Yc[om1 + cl - 1] : x31);
          float L, U, Rv, Dv;
          if (!(CS[o0 + cl] & kSpecial)) {
            // the common case: plain reads (R, D: the previous sweep at d+1,
            // or the initial x for the first sweep)
            L = prev[h];
            U = Ur;
            if (k > 0) {
              Rv = Yp[op1 + cl];
              Dv = Yp[op1 + cl + 1];
            } else {
              Rv = XI[op1 + cl];
              Dv = XI[op1 + cl + 1];
            }
          } else {
            const int op2 = op1 + W == RW ? 0 : op1 + W;
            // L = (i-1, j), U = (i, j-1): this sweep, diagonal d-1
            L = (i > 1) ? prev[h] : frame_post(0, j, k - 1, Yp, o0, cl, om1 + cl);
            U = (j > 1) ? Ur : frame_post(i, 0, k - 1, Yp, o0, cl, om1 + cl - 1);
            // R = (i+1, j), D = (i, j+1): sweep k-1 after its bnd, diagonal d+1
            Rv = (i < N) ? interior_post(i + 1, j, op1, cl, op2, o0)
                         : frame_post(S - 1, j, k - 1, Yp, o0, cl, op1 + cl);
            Dv = (j < N) ? interior_post(i, j + 1, op1, cl + 1, op2, o0)
                         : frame_post(i, S - 1, k - 1, Yp, o0, cl, op1 + cl + 1);
          }
          const float sum = fadd(fadd(fadd(Rv, L), Dv), U);
          const float v = fmul(fadd(X0[xo + cl - 1], fmul(a, sum)), cr);
          Yc[o0 + cl] = v;
          if (plo[h]) plo[h][o0] = v;
          if (phi[h]) phi[h][o0] = v;
          if (k == K - 1) A.x[(size_t)j * P + i] = v;
          prev[h] = v;
        }
      }
    }
    o0 = o0 + W == RW ? 0 : o0 + W;
    xo = xo + J == R * J ? 0 : xo + J;
    if (--cnt < 0 || t == nsteps - 1) {
      if (!sweeper) {  // this interval's copies in flight, the previous one's landed
        cp_async_commit();
        cp_async_wait<1>();
      }
      cluster.sync();  // also the last step: no remote store may follow a block's exit
      cnt = m;
    }
  }
  if (!sweeper) cp_async_wait<0>();
}

}  // namespace eqk
