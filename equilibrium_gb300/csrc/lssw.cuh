// lin_solve (fluid.rs:301-325) as one persistent launch over strips of rows,
// bit-exactly: the strip wavefront.
//
// Decomposition. Block b owns, for every sweep k of the launch, the 32 rows
//   j = j0(b, k) + l,  j0(b, k) = 32 b - 2 k,  l = lane,
// of its sweep warp k (warp K is the copy warp). A sweep's rows shift up by
// two per sweep, so every value a block needs from another block comes from
// block b-1 (never b+1): blocks take their strip from an atomic ticket, wait
// only for lower tickets, and need no co-residency.
//
// Schedule. Sweep warp k works on local diagonal d = tau - kLg k at block step
// tau; lane l updates cell (i, j) = (d - l, j0 + l), so lane l trails lane
// l-1 by one step (Gauss-Seidel order along every row and down every column).
// The sweep-k value of an interior cell is
//   raw(i, j) = (x0 + a*(((R + L) + D) + U)) * (1/c)
// with L = this lane's previous value, U = lane l-1's previous value (a
// shuffle; lane 0: block b-1's row j0 - 1, imported), and R = post(i+1, j),
// D = post(i, j+1) of sweep k-1 after its set_boundaries, read from sweep k-1's
// ring of post values in shared memory (the first sweep reads the initial x
// from a ring of copied rows). post is written one step late: at step d the
// lane knows raw(i, j), raw(i-1, j), raw(i-2, j), raw(i-1, j-1) (last step's
// U) and raw(i-1, j+1) (lane l+1's value, a shuffle), which is everything the
// per-cell boundary code of (i-1, j) can ask for. Frame rows are lanes too
// (their "value" is the frame cell as the sweep sees it); frame columns are
// the steps i = 0 and i = S-1 of each row. The last sweep writes its raw
// interior values to x; the caller's set_boundaries pass (with corners) then
// makes x the reference's array.
//
// Block-to-block values. Lanes 30 and 31 of every sweep warp export, per
// diagonal, lane 31's value and both lanes' post values as 64-bit words
// (value | tag << 32) that block b+1's sweep warp k polls with relaxed loads,
// issued kSwAHI periods ahead, and copies into its own ring (positions -2,
// -1) and lane-0 U ring. Lane 31 cannot finish a post value that needs the
// next block's row (AdjustColumn, wall below); block b+1's lane 0 overwrites
// it in its ring. The tag is the launch's epoch (a device word the last block
// advances), so a captured graph replays without clearing anything.
//
// Staging. The copy warp streams x0 and the codes of the block's rows, and the
// initial x rows the first sweep reads, into shared-memory rings: per row one
// aligned 16-byte chunk (4 columns) per period, issued kSwAH periods before
// its first use. All warps meet at one block barrier per period of kSwQ
// steps; every cross-warp value is written at least one barrier before it is
// read and its slot is reused only after its last read (the schedule is
// checked on the CPU with these formulas).
//
// Safety. Every wait is bounded (spin budget); a timeout sets the device error
// word and the block's abort flag, and all warps leave the period loop at the
// same barrier. The copy warp waits for its copies before exit.
#pragma once
#include "common.cuh"
#include "kernels.cuh"

namespace eqk {

constexpr int kSwQ = 4;      // steps per period (one block barrier per period)
constexpr int kSwLg = 4;     // steps between consecutive sweeps (>= kSwQ)
constexpr int kSwRD = 16;    // diagonals kept per sweep ring
constexpr int kSwRW = 36;    // floats per ring row: positions -2 .. 33
constexpr int kSwPC = 128;   // columns of the x0 / code rings
constexpr int kSwPX = 32;    // columns of the initial-x ring
constexpr int kSwAH = 3;     // a chunk copy is issued kSwAH periods before its use
constexpr int kSwMaxK = 20;  // sweeps per launch
static_assert(kSwLg >= kSwQ, "a ring value must be one barrier old when read");

struct LsSwArgs {
  float* x;  // in: initial x; out: the last sweep's raw interior values
  const float* x0;
  const uint8_t* code;
  const uint8_t* rowfl;
  const uint8_t* colfl;
  unsigned long long* edge;  // [B-1][K][RE][4] tagged exports
  unsigned* ctr;             // [0] ticket, [1] done (zeroed per launch), [2] epoch
  int* err;
  long long spin_limit;
  int S, P, K, B, RE;
  float a, cr;
};

__host__ __device__ inline int ls_sw_strips(int S, int K) { return (S + 2 * (K - 1) + 31) / 32; }
__host__ __device__ inline int ls_sw_records(int S) { return S + 32; }

struct LsSwLayout {  // byte offsets in one block's shared memory
  size_t vr, ui, x0r, cr, xr, total;
};
__host__ __device__ inline LsSwLayout ls_sw_layout(int K) {
  const size_t nrw = 32 + 2 * (size_t)(K - 1);
  LsSwLayout L;
  L.vr = 0;                                                  // K RD RW floats
  L.ui = L.vr + (size_t)K * kSwRD * kSwRW * 4;               // K RD floats
  L.x0r = ((L.ui + (size_t)K * kSwRD * 4) + 15) / 16 * 16;  // nrw PC floats
  L.cr = L.x0r + nrw * kSwPC * 4;                            // nrw PC bytes
  L.xr = L.cr + nrw * kSwPC;                                 // 33 PX floats
  L.total = L.xr + 33 * kSwPX * 4;
  return L;
}

__device__ __forceinline__ unsigned ld_relaxed_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_u64_sw(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long sw_pack(float v, unsigned tag) {
  return (unsigned long long)__float_as_uint(v) | ((unsigned long long)tag << 32);
}

// The Gauss-Seidel update; the FMA build contracts x0 + a*sum.
__device__ __forceinline__ float gs_update(float x0, float a, float sum, float cr) {
#if defined(EQ_FMA) && EQ_FMA
  return __fmul_rn(__fmaf_rn(a, sum, x0), cr);
#else
  return fmul(fadd(x0, fmul(a, sum)), cr);
#endif
}

template <int MODE>
__global__ void __launch_bounds__(32 * (kSwMaxK + 1), 1) k_ls_sw(LsSwArgs A) {
  extern __shared__ __align__(16) unsigned char ls_sw_smem[];
  // abort flags by period parity: set during period cp in s_abort[cp & 1] and
  // read by every thread after that period's barrier (nobody writes that slot
  // again before the next barrier), so all warps leave at the same barrier
  __shared__ int s_b, s_abort[2];
  __shared__ unsigned s_tag;
  const unsigned FULL = 0xffffffffu;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int K = A.K, S = A.S, P = A.P, N = S - 2, B = A.B;
  if (threadIdx.x == 0) {
    s_b = (int)atomicAdd(&A.ctr[0], 1u);
    s_tag = ld_relaxed_u32(&A.ctr[2]) + 1u;
    s_abort[0] = s_abort[1] = 0;
  }
  __syncthreads();
  const int b = s_b;
  const unsigned tag = s_tag;
  if (b >= B) {  // counters not reset: never index past the strips
    if (threadIdx.x == 0) atomicExch(A.err, 5 /* EQ_ERR_STATE */);
    return;
  }
  const LsSwLayout lay = ls_sw_layout(K);
  float* const VR = reinterpret_cast<float*>(ls_sw_smem + lay.vr);
  float* const UI = reinterpret_cast<float*>(ls_sw_smem + lay.ui);
  float* const X0R = reinterpret_cast<float*>(ls_sw_smem + lay.x0r);
  uint8_t* const CR = ls_sw_smem + lay.cr;
  float* const XR = reinterpret_cast<float*>(ls_sw_smem + lay.xr);
  const int nrw = 32 + 2 * (K - 1);
  const int rA = 32 * b - 2 * (K - 1);  // first row of the block's rings
  const int T = S + 32 + kSwLg * (K - 1);
  const int NP = (T + kSwQ - 1) / kSwQ;

  if (warp == K) {
    // ---- the copy warp: x0 / code rows and the first sweep's initial-x rows
    auto issue = [&](int cp) {
      const int u = cp + kSwAH;  // use period
      for (int q = lane; q < nrw; q += 32) {
        const int r = rA + q;
        if (r < 0 || r > S - 1) continue;
        const int dr = 32 * b - r;
        const int kmin = dr > 0 ? (dr + 1) >> 1 : 0;
        const int off = dr - (kSwLg + 2) * kmin;
        const int n = u + ((off + 3) >> 2);
        if (n < 0 || 4 * n >= P) continue;
        const int sc = (4 * n) & (kSwPC - 1);
        cp_async16(&X0R[q * kSwPC + sc], A.x0 + (size_t)r * P + 4 * n, true);
        cp_async4(&CR[q * kSwPC + sc], A.code + (size_t)r * P + 4 * n, true);
      }
      for (int q = lane; q < 33; q += 32) {
        const int r = 32 * b + q;
        if (r > S - 1) continue;
        const int n = u + 1 - ((q + 3) >> 2);
        if (n < 0 || 4 * n >= P) continue;
        cp_async16(&XR[q * kSwPX + ((4 * n) & (kSwPX - 1))], A.x + (size_t)r * P + 4 * n, true);
      }
      cp_async_commit();
    };
    for (int cp = -kSwAH - 1; cp < 0; ++cp) issue(cp);
    cp_async_wait<kSwAH - 1>();  // use periods -1 and 0 have landed
    __syncthreads();
    if (!s_abort[1]) {
      for (int cp = 0; cp < NP; ++cp) {
        issue(cp);
        cp_async_wait<kSwAH - 1>();  // use period cp + 1 has landed
        __syncthreads();
        if (s_abort[cp & 1]) break;
      }
    }
    cp_async_wait<0>();
  } else {
    // ---- sweep warp k
    const int k = warp;
    const int j0 = 32 * b - 2 * k, j = j0 + lane;
    const bool interior = j >= 1 && j <= N, top = j == 0, bot = j == S - 1;
    const bool idle = !(interior || top || bot);
    const bool active = j0 <= S - 1 && j0 + 31 >= 0;
    const bool hasFrame = __any_sync(FULL, top || bot);
    const bool last = k == K - 1;
    float* const VRk = VR + (size_t)k * kSwRD * kSwRW;
    const float* const VRp = VR + (size_t)(k > 0 ? k - 1 : 0) * kSwRD * kSwRW;
    float* const UIk = UI + (size_t)k * kSwRD;
    const int rrow = 2 * (K - 1 - k) + lane;
    const float* const X0row = X0R + rrow * kSwPC;
    const uint8_t* const CRrow = CR + rrow * kSwPC;
    const float* const XRl = XR + lane * kSwPX;
    const float* const XRd = XR + (lane + 1) * kSwPX;
    const float a = A.a, cr = A.cr;
    // per-lane constants: the row's frame columns and its Passive flag
    const float xL = interior ? A.x[(size_t)j * P] : 0.0f;
    const float xR = interior ? A.x[(size_t)j * P + (S - 1)] : 0.0f;
    const bool pasRow = MODE == kPassive && interior && A.rowfl[j] != 0;
    const float* const xFrame = A.x + (bot ? (size_t)(S - 1) * P : 0);
    // imports from block b-1's sweep warp k: lane t < 12 holds word t % 3 of
    // record t / 3 (diagonal offset) of each period
    const int jp = 32 * (b - 1) - 2 * k;
    const bool impOn = b > 0 && jp <= S - 1 && jp + 31 >= 0;
    const unsigned long long* const edgeIn =
        impOn ? A.edge + ((size_t)(b - 1) * K + k) * A.RE * 4 : nullptr;
    unsigned long long* const edgeOut =
        (b < B - 1) ? A.edge + ((size_t)b * K + k) * A.RE * 4 : nullptr;
    const int iq = lane / 3, iw = lane - 3 * (lane / 3);
    auto imp_dd = [&](int u) { return u * kSwQ - kSwLg * k - 1 + iq; };
    auto imp_ok = [&](int u) {
      const int dd = imp_dd(u);
      return impOn && lane < 12 && dd >= -1 && dd <= S - 2;
    };
    auto imp_load = [&](int u) -> unsigned long long {
      return imp_ok(u) ? ld_relaxed_u64(edgeIn + (size_t)(imp_dd(u) + 32) * 4 + iw) : 0ull;
    };
    // check and store the words of use period u (w: loaded earlier); false on timeout
    auto imp_store = [&](int u, unsigned long long w) -> bool {
      const bool need = imp_ok(u);
      bool bad = need && (unsigned)(w >> 32) != tag;
      long long tries = 0;
      unsigned ns = 32;
      while (__any_sync(FULL, bad)) {
        if (++tries > A.spin_limit) {
          if (lane == 0) atomicExch(A.err, 3 /* EQ_ERR_TIMEOUT */);
          return false;
        }
        if ((tries & 63) == 0 && __any_sync(FULL, ld_relaxed_i32(A.err) != 0)) return false;
        __nanosleep(ns);
        ns = ns < 256 ? ns * 2 : 256;
        if (bad) {
          w = ld_relaxed_u64(edgeIn + (size_t)(imp_dd(u) + 32) * 4 + iw);
          bad = (unsigned)(w >> 32) != tag;
        }
      }
      if (need) {
        const int s = imp_dd(u) & (kSwRD - 1);
        const float v = __uint_as_float((unsigned)(w & 0xffffffffull));
        if (iw == 0)
          UIk[s] = v;
        else
          VRk[s * kSwRW + (iw - 1)] = v;
      }
      return true;
    };
    bool ok = true;
    unsigned long long w0 = imp_load(0);
    ok = imp_store(0, w0);  // the prologue: imports of period 0
    w0 = imp_load(1);
    unsigned long long w1 = imp_load(2);
    if (!ok) s_abort[1] = 1;  // the prologue counts as period -1
    __syncthreads();
    const bool go = !s_abort[1];

    float vcur = 0.0f, vprev = 0.0f, uprev = 0.0f;
    unsigned cprev = 0;
    const unsigned actMask =
        MODE == kRow ? (kCodeRowLeft | kCodeRowRight) : MODE == kCol ? (kCodeColUp | kCodeColDown) : 0u;
    for (int cp = 0; go && cp < NP; ++cp) {
      bool fine = imp_store(cp + 1, w0);
      if (!fine) s_abort[cp & 1] = 1;
      w0 = w1;
      w1 = imp_load(cp + 3);
      if (active && fine) {
#pragma unroll
        for (int t = 0; t < kSwQ; ++t) {
          const int d = cp * kSwQ + t - kSwLg * k;
          if (d < 0 || d > S + 31) continue;
          const int i = d - lane;
          float R, D;
          if (k > 0) {
            const float* const row = VRp + ((d - 1) & (kSwRD - 1)) * kSwRW;
            R = row[lane];
            D = row[lane + 1];
          } else {
            R = XRl[(i + 1) & (kSwPX - 1)];
            D = XRd[i & (kSwPX - 1)];
          }
          const float Ui = UIk[(d - 1) & (kSwRD - 1)];
          float U = __shfl_up_sync(FULL, vcur, 1);
          if (lane == 0) U = Ui;
          const int ci = i & (kSwPC - 1);
          const float X0 = X0row[ci];
          const unsigned cd = CRrow[ci];
          const float gs = gs_update(X0, a, fadd(fadd(fadd(R, vcur), D), U), cr);
          const bool fix = MODE == kCol && lane == 0 && (cd & kCodeAboveDown) != 0;
          const bool fastL = idle || top || bot ||
                             (interior && (unsigned)(i - 2) <= (unsigned)(N - 2) &&
                              (cprev & actMask) == 0u && !fix);
          float vnew, post;
          if (__all_sync(FULL, fastL)) {
            vnew = gs;
            post = vcur;
            if (hasFrame) {  // frame-row lanes: the frame cell as the sweep sees it
              const bool fl = top || bot;
              const bool inr = (unsigned)i < (unsigned)S;
              const int ic = min(max(i, 0), S - 1);
              float xf = 0.0f;
              unsigned cf = 0, cfp = 0;
              if (fl) {
                xf = xFrame[ic];
                if (MODE == kPassive) {
                  cf = A.colfl[ic];
                  cfp = A.colfl[min(max(i - 1, 0), S - 1)];
                }
              }
              if (fl) vnew = inr ? ((MODE == kPassive && top && k > 0 && cf) ? D : xf) : vcur;
              if (MODE == kPassive) {
                const float vdown = __shfl_down_sync(FULL, vnew, 1);
                const bool pc = (unsigned)(i - 2) <= (unsigned)(N - 1) && cfp != 0u;
                if (fl) post = pc ? (top ? vdown : uprev) : vcur;
              } else if (fl) {
                post = vcur;
              }
            }
          } else {
            // ---- the general rules, every lane
            vnew = vcur;
            if (interior) {
              if ((unsigned)(i - 1) < (unsigned)N)
                vnew = gs;
              else if (i == 0)
                vnew = (MODE == kPassive && k > 0 && pasRow) ? R : xL;
              else if (i == S - 1)
                vnew = xR;
            } else if (top || bot) {
              if ((unsigned)i < (unsigned)S) {
                const float xf = xFrame[i];
                vnew = (MODE == kPassive && top && k > 0 && A.colfl[i]) ? D : xf;
              }
            } else {
              vnew = 0.0f;
            }
            const float vdown = __shfl_down_sync(FULL, vnew, 1);
            const int im1 = i - 1;
            post = vcur;
            if (interior) {
              if ((unsigned)(im1 - 1) < (unsigned)N) {
                if (MODE == kRow)
                  post = (cprev & kCodeRowRight) ? -vnew : ((cprev & kCodeRowLeft) ? -vprev : vcur);
                else if (MODE == kCol)
                  post = (cprev & kCodeColUp) ? -uprev : ((cprev & kCodeColDown) ? -vdown : vcur);
              } else if (im1 == 0) {
                post = pasRow ? vnew : vcur;
              } else if (im1 == S - 1) {
                post = pasRow ? vprev : vcur;
              }
            } else if (top || bot) {
              if (MODE == kPassive && (unsigned)(im1 - 1) < (unsigned)N && A.colfl[im1])
                post = top ? vdown : uprev;
            } else {
              post = 0.0f;
            }
          }
          float* const wrow = VRk + ((d - 1) & (kSwRD - 1)) * kSwRW;
          wrow[lane + 2] = post;
          if (fix && (interior || bot) && (unsigned)(i - 1) < (unsigned)N) wrow[1] = -vnew;
          if (edgeOut) {
            if (lane == 31) st_relaxed_u64_sw(edgeOut + (size_t)d * 4, sw_pack(vnew, tag));
            if (lane >= 30 && d >= 1)
              st_relaxed_u64_sw(edgeOut + (size_t)(d - 1) * 4 + (lane - 29), sw_pack(post, tag));
          }
          if (last && interior && (unsigned)(i - 1) < (unsigned)N) A.x[(size_t)j * P + i] = vnew;
          vprev = vcur;
          vcur = vnew;
          uprev = U;
          cprev = cd;
        }
      }
      __syncthreads();
      if (s_abort[cp & 1]) break;
    }
  }
  // ---- completion: the last block to finish advances the epoch
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned prev = atom_add_acq_rel_u32(&A.ctr[1], 1u);
    if (prev == (unsigned)B - 1u) atomicAdd(&A.ctr[2], 1u);
  }
}

}  // namespace eqk
