// lin_solve (fluid.rs:301-325) as one persistent launch over strips of rows
// and groups of sweeps, bit-exactly: the strip wavefront.
//
// Decomposition. The launch covers K sweeps. Block (b, g) owns strip b for
// the sweeps k in [g KG, g KG + nk) (sweep group g): its sweep warp kk
// (k = g KG + kk) updates the 32 rows
//   j = j0(b, k) + l,  j0(b, k) = 32 b - 2 k,  l = lane.
// A sweep's rows shift up by two per sweep, so every value a block needs
// from another block comes from block (b-1, g) (the halo of the same sweeps)
// or (b, g-1) (the previous sweep of the first warp): blocks take (b, g) from
// an atomic ticket (b major), wait only for lower tickets and need no
// co-residency.
//
// Schedule. Sweep warp kk works on local diagonal d = tau - kSwLg kk at block
// step tau; lane l updates cell (i, j) = (d - l, j0 + l), so lane l trails lane
// l-1 by one step (Gauss-Seidel order along every row and down every column).
// The sweep-k value of an interior cell is
//   raw(i, j) = (x0 + a*(((R + L) + D) + U)) * (1/c)
// with L = this lane's previous value, U = lane l-1's previous value (a
// shuffle; lane 0: strip b-1's row j0 - 1, imported), and R = post(i+1, j),
// D = post(i, j+1) of sweep k-1 after its set_boundaries, read from sweep k-1's
// ring of post values in shared memory (the group's first sweep reads the
// previous group's exported ring, or for the first group the initial x from a
// ring of copied rows). post is written one step late: at step d the lane
// knows raw(i, j), raw(i-1, j), raw(i-2, j), raw(i-1, j-1) (last step's U) and
// raw(i-1, j+1) (lane l+1's value, a shuffle), everything the boundary code of
// (i-1, j) can ask for. Frame rows are lanes too (their value is the frame
// cell as the sweep sees it); frame columns are the steps i = 0 and i = S-1
// of each row. The last sweep writes its raw interior values to x; the
// caller's set_boundaries pass (with corners) then makes x the reference's
// array.
//
// Steps. Inside a warp's fast range (every grid row of the warp an interior
// row at 2 <= i <= N) a period is straight-line code: the update, the
// interior boundary rule by the cell's code (branch-free selects; AdjustColumn
// takes the lane below by a shuffle), the post store and the lane-0 fix. The
// general rules (frame columns, idle lanes) run only outside that range.
//
// Block-to-block values, as 64-bit words (value | tag << 32) polled with
// relaxed loads issued kSwAHI periods ahead and copied into shared memory:
// * halo: lanes 30 and 31 of sweep warp k export per diagonal
//   [post30, -, uval31, post31] for strip b+1's sweep warp k (its ring
//   positions -2, -1 and lane-0 U ring), imported by that warp at the start
//   of the period that reads them. Lane 31 cannot finish a post value that
//   needs the next strip's row (AdjustColumn, wall below); strip b+1's lane 0
//   overwrites it in its ring.
// * group: the last sweep warp of group g exports its post ring row per
//   diagonal (positions -2 .. 31) for group g+1's first sweep, read by an
//   import warp one period ahead.
// The tag is the launch's epoch (a device word the last block advances), so
// a captured graph replays without clearing anything.
//
// Staging. A copy warp streams x0 and the codes of the block's rows into
// shared-memory rings (and in the first group, which imports nothing from a
// previous group, the group import warp streams the initial x rows its first
// sweep reads): per row one aligned 16-byte chunk (4 columns) per period,
// issued kSwAH periods before its first use. No sweep warp issues a global
// load: a warp's shared-memory loads return in order behind its global loads. All warps meet at one block barrier per
// period of kSwQ steps; every cross-warp value is written at least one
// barrier before it is read and its slot is reused only after its last read
// (the schedule is checked on the CPU with these formulas).
//
// Safety. Every wait is bounded (spin budget); a timeout sets the device error
// word and the block's abort flag, and all warps leave the period loop at the
// same barrier. The copy warp waits for its copies before exit.
#pragma once
#include "common.cuh"
#include "kernels.cuh"

namespace eqk {

constexpr int kSwQ = 4;       // steps per period (one block barrier per period)
constexpr int kSwLg = 4;      // steps between consecutive sweeps (>= kSwQ)
constexpr int kSwRD = 16;     // diagonals kept per sweep ring
constexpr int kSwRW = 36;     // floats per ring row: positions -2 .. 33
constexpr int kSwPC = 128;    // columns of the x0 / code rings
constexpr int kSwPX = 32;     // columns of the initial-x ring
// Row strides of those rings, padded so that the copy warp's per-row chunk
// writes (one row per lane) fall in different banks and the sweep warps'
// reads (row + lane, column - lane) stay conflict-free; the 4 padding columns
// repeat the ring's columns 0 .. 3, so a period's 4 columns are read from one
// base without wrapping.
constexpr int kSwPCS = kSwPC + 4;  // x0 ring row (floats)
constexpr int kSwCCS = kSwPC + 4;  // code ring row (bytes)
constexpr int kSwPXS = kSwPX + 4;  // initial-x ring row (floats)
constexpr int kSwAH = 5;      // a chunk copy is issued kSwAH periods before its use
constexpr int kSwAHI = 1;     // an import load is checked kSwAHI periods after its issue
constexpr int kSwMaxK = 20;   // sweeps per launch
constexpr int kSwMaxKG = 10;  // sweeps per block (its warps' registers hold a period's operands)
constexpr int kSwGrpWords = 36;  // words per group-export record (34 used)
static_assert(kSwLg >= kSwQ, "a ring value must be one barrier old when read");

struct LsSwArgs {
  float* x;  // in: initial x; out: the last sweep's raw interior values
  const float* x0;
  const uint8_t* code;
  const uint8_t* rowfl;
  unsigned long long* edge;  // [B-1][K][RE][4] halo exports
  unsigned long long* gexp;  // [B][G-1][RE+1][kSwGrpWords] group exports
  unsigned* ctr;             // [0] ticket, [1] done (zeroed by each launch's last block), [2] epoch
  int* err;
  long long spin_limit;
  int S, P, K, B, G, KG, RE;
  int slack;  // a block starts once its producers are this many periods ahead
  float a, cr;
};

__host__ __device__ inline int ls_sw_strips(int S, int K) { return (S + 2 * (K - 1) + 31) / 32; }
__host__ __device__ inline int ls_sw_records(int S) { return S + 32; }

struct LsSwLayout {  // byte offsets in one block's shared memory
  size_t vr, ui, vp, x0r, cr, xr, total;
};
__host__ __device__ inline LsSwLayout ls_sw_layout(int KG) {
  const size_t nrw = 32 + 2 * (size_t)(KG - 1);
  LsSwLayout L;
  L.vr = 0;                                        // KG RD RW floats
  L.ui = L.vr + (size_t)KG * kSwRD * kSwRW * 4;     // KG RD floats
  L.vp = L.ui + (size_t)KG * kSwRD * 4;             // RD RW floats
  L.x0r = (L.vp + (size_t)kSwRD * kSwRW * 4 + 15) / 16 * 16;  // nrw PC floats
  L.cr = L.x0r + nrw * kSwPCS * 4;                 // nrw CCS bytes
  L.xr = (L.cr + nrw * kSwCCS + 15) / 16 * 16;     // 33 PXS floats
  L.total = L.xr + 33 * kSwPXS * 4;
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
// Exports: each 64-bit element is one single-copy-atomic word (value | tag).
// A word validates itself by its tag, so no export is ordered against any
// other memory access: no memory clobber, and the compiler may schedule the
// steps' shared-memory traffic across it.
__device__ __forceinline__ void sw_st1(unsigned long long* p, float v, unsigned tag) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p),
               "l"((unsigned long long)__float_as_uint(v) | ((unsigned long long)tag << 32)));
}
// Two words, stored only where `on` (a predicate inside the instruction, so
// that the lanes that export nothing take no branch around it).
__device__ __forceinline__ void sw_st2(unsigned long long* p, float v0, float v1, unsigned tag,
                                       bool on) {
  asm volatile(
      "{ .reg .pred q; setp.ne.b32 q, %3, 0; @q st.relaxed.gpu.global.v2.u64 [%0], {%1, %2}; }" ::"l"(p),
      "l"((unsigned long long)__float_as_uint(v0) | ((unsigned long long)tag << 32)),
      "l"((unsigned long long)__float_as_uint(v1) | ((unsigned long long)tag << 32)), "r"((int)on));
}

// The Gauss-Seidel update; the FMA build contracts x0 + a*sum.
__device__ __forceinline__ float gs_update(float x0, float a, float sum, float cr) {
#if defined(EQ_FMA) && EQ_FMA
  return __fmul_rn(__fmaf_rn(a, sum, x0), cr);
#else
  return fmul(fadd(x0, fmul(a, sum)), cr);
#endif
}

// One sweep warp's state and constants.
struct SwWarp {
  // lane state: the value at the previous step (L), the one before, last
  // step's U and the code of the previous cell
  float vcur, vprev, uprev;
  unsigned cprev;
  // lane constants (cfTop / cfBot: the frame rows' column-flag masks)
  unsigned cfTop, cfBot;
  int lane, j, S, N, k;
  bool interior, top, bot, idle, pasRow;
  float xL, xR, a, cr;
  const float* prev;   // previous sweep's ring (or the previous group's)
  float* own;          // this sweep's ring
  const float* ui;     // lane-0 U ring
  const float* x0row;  // x0 ring row of this lane's row
  const uint8_t* crow;
  const float* xrl;    // first sweep of the first group: initial-x ring rows
  const float* xrd;
  unsigned long long* edgeOut;  // halo export (lanes 30, 31; the base elsewhere, unused)
  bool edgeOn;
  float* xlast;                 // x + j P - lane for the last sweep, else null
  unsigned tag;
};

// The shared-memory operands of step d = dp + q of a sweep warp (dp a
// multiple of kSwQ, q < kSwQ): loaded for a whole period before its first
// step, so that no load waits behind a previous step's ring store. Ring slot
// d % kSwRD holds diagonal d - 1, so a period's slots are consecutive. A
// frame row's x0 ring row holds the frame row of x (its value before the
// sweeps), and every code carries its column's fluid flag.
struct SwOps {
  float R, D, Ui, X0;
  unsigned cd;
};

template <bool FIRSTX>
__device__ __forceinline__ SwOps sw_load(const SwWarp& w, int dp, int q) {
  const int lane = w.lane;
  const int slot = (dp & (kSwRD - 1)) + q;
  SwOps o;
  if (FIRSTX) {
    // a period's 4 columns from one base: the ring's column 0 chunk is also
    // stored past its end (columns kSwPX .. kSwPX + 3)
    o.R = w.xrl[((dp - lane + 1) & (kSwPX - 1)) + q];
    o.D = w.xrd[((dp - lane) & (kSwPX - 1)) + q];
  } else {
    o.R = w.prev[slot * kSwRW + lane];
    o.D = w.prev[slot * kSwRW + lane + 1];
  }
  o.Ui = w.ui[slot];
  const int ci = ((dp - lane) & (kSwPC - 1)) + q;  // column i, the same way
  o.X0 = w.x0row[ci];
  o.cd = w.crow[ci];
  return o;
}

// The frame-row lanes of a step (FRAME warps): the frame cell as the sweep
// sees it (the frame row of x from the x0 ring; Passive, from sweep 1 on, a
// fluid column's top cell takes the previous sweep's cell (i, 1)), and the
// bottom row's post value (Passive: a fluid column's bottom cell takes cell
// (i, S-2) of this sweep, last step's U). A top row's post value is never
// read. The column flag rides in every code (0 in the frame columns), held
// per lane as a mask: cfTop for Passive top-row lanes from sweep 1 on,
// cfBot for Passive bottom-row lanes, 0 elsewhere.
template <int MODE>
__device__ __forceinline__ void sw_frame(const SwWarp& w, const SwOps& o, float& vnew,
                                         float& post) {
  vnew = (w.top || w.bot) ? ((o.cd & w.cfTop) ? o.D : o.X0) : vnew;
  if (MODE == kPassive) post = (w.cprev & w.cfBot) ? w.uprev : post;
}

// Step d = dp + q outside a warp's fast range (its first and last 8 or 9
// periods, which the next strip and the next group wait for): the fast step
// plus the frame columns. Only values that some later update reads have to
// follow the general rules there: an interior row's frame columns i = 0
// (the frame value; Passive fluid rows from sweep 1 on: the previous sweep's
// cell (1, j)) and i = S-1, and the post value of column S-1 (Passive fluid
// rows: cell S-2 as this sweep left it; the codes of frame cells hold no
// boundary rule, so the other modes keep the frame value). A lane before its
// row's column 0 or past column S-1, an idle lane, the post value of column
// 0 and a top frame row's post values are never read: they hold whatever the
// arithmetic gives, and nothing of them reaches x (the last sweep stores
// columns 1 .. N only) or another warp's read.
template <int MODE, bool FRAME>
__device__ __forceinline__ void sw_step_edge(SwWarp& w, int dp, int q, const SwOps& o) {
  const unsigned FULL = 0xffffffffu;
  const int lane = w.lane;
  const int d = dp + q;
  const int i = d - lane;
  const int slot = (dp & (kSwRD - 1)) + q;
  const int S = w.S, N = w.N;
  float U = __shfl_up_sync(FULL, w.vcur, 1);
  U = lane == 0 ? o.Ui : U;
  const float gs = gs_update(o.X0, w.a, fadd(fadd(fadd(o.R, w.vcur), o.D), U), w.cr);
  const bool inI = (unsigned)(i - 1) < (unsigned)N;  // 1 <= i <= N
  const bool fix = MODE == kCol && lane == 0 && (o.cd & kCodeAboveDown) != 0 &&
                   (w.interior || w.bot) && inI;
  const float vL = (MODE == kPassive && w.k > 0 && w.pasRow) ? o.R : w.xL;
  float vnew = i == 0 ? vL : (i == S - 1 ? w.xR : gs);
  float post = w.vcur;
  if (FRAME) sw_frame<MODE>(w, o, vnew, post);
  if (MODE == kRow) {
    const float pr =
        (w.cprev & kCodeRowRight) ? -vnew : ((w.cprev & kCodeRowLeft) ? -w.vprev : w.vcur);
    post = w.interior ? pr : post;
  } else if (MODE == kCol) {
    const float vdown = __shfl_down_sync(FULL, vnew, 1);
    const float pc =
        (w.cprev & kCodeColUp) ? -w.uprev : ((w.cprev & kCodeColDown) ? -vdown : w.vcur);
    post = w.interior ? pc : post;
  } else {
    post = (w.pasRow && i - 1 == S - 1) ? w.vprev : post;
  }
  float* const wrow = w.own + slot * kSwRW;
  wrow[lane + 2] = post;
  if (MODE == kCol && fix) wrow[1] = -vnew;
  // lanes 30, 31: halo record d-1 = [post30, -, uval31, post31]
  sw_st2(w.edgeOut + (size_t)(d - 1) * 4, lane == 31 ? w.vcur : post, post, w.tag,
         w.edgeOn && d >= 1);
  if (w.xlast && w.interior && inI) w.xlast[d] = vnew;
  w.vprev = w.vcur;
  w.vcur = vnew;
  w.uprev = U;
  w.cprev = o.cd;
}

// A step of a fast period: the update, the boundary rule of the interior
// lanes, the post store and the halo export, with no branch, so that the
// compiler schedules a period's kSwQ steps as one straight-line block. Gives
// the bits of the general rules wherever a later read needs them, when every
// interior lane of the warp is at 2 <= i <= N.
template <int MODE, bool FRAME>
__device__ __forceinline__ void sw_step_fast(SwWarp& w, int dp, int q, const SwOps& o) {
  const unsigned FULL = 0xffffffffu;
  const int lane = w.lane;
  const int d = dp + q;
  const int i = d - lane;
  const int slot = (dp & (kSwRD - 1)) + q;
  const int N = w.N;
  float U = __shfl_up_sync(FULL, w.vcur, 1);
  U = lane == 0 ? o.Ui : U;
  const float gs = gs_update(o.X0, w.a, fadd(fadd(fadd(o.R, w.vcur), o.D), U), w.cr);
  // the lane-0 fix of the row above (AdjustColumn, a wall cell under a
  // fluid cell whose rule takes its lower neighbour)
  const bool fix = MODE == kCol && lane == 0 && (o.cd & kCodeAboveDown) != 0 &&
                   (w.interior || w.bot) && (unsigned)(i - 1) < (unsigned)N;
  float vnew = gs, post = w.vcur;
  if (FRAME) sw_frame<MODE>(w, o, vnew, post);  // frame-row lanes
  // set_boundaries' rule for the interior cell (i-1, j) by its code, branch
  // free: AdjustRow takes -raw(i, j) (right wall) or -raw(i-2, j) (left),
  // AdjustColumn -raw(i-1, j-1) (up) or -raw(i-1, j+1) (down, lane l+1)
  if (MODE == kRow) {
    const float pr =
        (w.cprev & kCodeRowRight) ? -vnew : ((w.cprev & kCodeRowLeft) ? -w.vprev : w.vcur);
    post = w.interior ? pr : post;
  } else if (MODE == kCol) {
    const float vdown = __shfl_down_sync(FULL, vnew, 1);
    const float pc =
        (w.cprev & kCodeColUp) ? -w.uprev : ((w.cprev & kCodeColDown) ? -vdown : w.vcur);
    post = w.interior ? pc : post;
  }
  float* const wrow = w.own + slot * kSwRW;
  wrow[lane + 2] = post;
  if (MODE == kCol && fix) wrow[1] = -vnew;
  // lanes 30, 31: halo record d-1 = [post30, -, uval31, post31] (d >= 2 here)
  sw_st2(w.edgeOut + (size_t)(d - 1) * 4, lane == 31 ? w.vcur : post, post, w.tag, w.edgeOn);
  if (w.xlast && w.interior) w.xlast[d] = vnew;  // 1 <= i - 1 < N in the fast range
  w.vprev = w.vcur;
  w.vcur = vnew;
  w.uprev = U;
  w.cprev = o.cd;
}

// A period of a warp's fast range: every operand loaded first, then the
// kSwQ steps.
template <int MODE, bool FIRSTX, bool FRAME>
__device__ __forceinline__ void sw_period_fast(SwWarp& w, int dp) {
  SwOps o[kSwQ];
#pragma unroll
  for (int q = 0; q < kSwQ; ++q) o[q] = sw_load<FIRSTX>(w, dp, q);
#pragma unroll
  for (int q = 0; q < kSwQ; ++q) sw_step_fast<MODE, FRAME>(w, dp, q, o[q]);
}

// A period outside the fast range: every operand loaded first (the loads
// stay inside the rings for any d), then the steps of the warp's diagonals
// 0 .. S + 31.
template <int MODE, bool FIRSTX, bool FRAME>
__device__ __forceinline__ void sw_period_edge(SwWarp& w, int dp) {
  SwOps o[kSwQ];
#pragma unroll
  for (int q = 0; q < kSwQ; ++q) o[q] = sw_load<FIRSTX>(w, dp, q);
#pragma unroll
  for (int q = 0; q < kSwQ; ++q) {
    const int d = dp + q;
    if (d >= 0 && d <= w.S + 31) sw_step_edge<MODE, FRAME>(w, dp, q, o[q]);
  }
}

// Warps of a block: kSwMaxKG sweep warps at most, the copy warp, the group
// import warp, the halo import warp and the group export warp.
constexpr int kSwHelpers = 4;
constexpr int kSwThreads = 32 * (kSwMaxKG + kSwHelpers);
static_assert(12 * kSwMaxKG <= 128, "the halo import warp holds 4 words a lane per period");

// The role of warp w of a block with KG sweep warps (nk of them real): sweep
// kk < KG, or KG (copy), KG + 1 (group import), KG + 2 (halo import), KG + 3
// (group export). Warps w, w + 4, w + 8 issue from the same SM sub-partition.
// With 5 sweeps (the usual block) the two sweeps that must share one get it
// to themselves; otherwise the helpers take warps h .. h+3 (h = min(4, KG))
// and the two heaviest sweeps, the first (it reads the initial x or the
// group import ring) and the last (it writes x in the last group), take
// warps 0 and 1.
__device__ __forceinline__ int sw_role(int w, int KG, int nk) {
  if (KG == 5) {
    // warps w, w + 4, w + 8 share a sub-partition: {0, 4, 8} first sweep,
    // group export, copy; {1, 5} two middle sweeps alone; {2, 6} a sweep and
    // the halo import; {3, 7} the last sweep and the group import
    if (w == 4) return KG + 3;
    if (w == 8) return KG;
    if (w == 6) return KG + 2;
    if (w == 7) return KG + 1;
    const int slot = w == 0 ? 0 : (w == 3 ? 1 : (w == 2 ? 2 : (w == 1 ? 3 : 4)));
    if (slot == 0 || nk < 2) return slot;
    if (slot == 1) return nk - 1;
    return slot <= nk - 1 ? slot - 1 : slot;
  }
  const int h = KG < 4 ? KG : 4;
  // helpers in warp order: group export (light, beside the first sweep and
  // the sweep of slot 4), group import, halo import, copy
  if (w >= h && w < h + kSwHelpers) return KG + ((0x0213 >> (4 * (w - h))) & 0xF);
  const int slot = w < h ? w : w - kSwHelpers;  // sweep slots in warp order
  if (slot == 0 || nk < 2) return slot;
  if (slot == 1) return nk - 1;
  return slot <= nk - 1 ? slot - 1 : slot;
}

template <int MODE>
__global__ void __launch_bounds__(kSwThreads, 1) k_ls_sw(LsSwArgs A) {
  extern __shared__ __align__(16) unsigned char ls_sw_smem[];
  // A warp that gives up a wait (timeout) raises its vote at the period's
  // barrier (__syncthreads_or), and every warp leaves at that barrier. The
  // vote needs no shared-memory flag: a warp with global loads in flight
  // would wait for them before any shared-memory load returns.
  __shared__ int s_t;
  __shared__ unsigned s_tag;
  const unsigned FULL = 0xffffffffu;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int K = A.K, S = A.S, P = A.P, N = S - 2, B = A.B, G = A.G, KG = A.KG;
  if (threadIdx.x == 0) {
    s_t = (int)atomicAdd(&A.ctr[0], 1u);
    s_tag = ld_relaxed_u32(&A.ctr[2]) + 1u;
  }
  __syncthreads();
  const int t = s_t;
  const unsigned tag = s_tag;
  if (t >= B * G) {  // counters not reset: never index past the blocks
    if (threadIdx.x == 0) atomicExch(A.err, 5 /* EQ_ERR_STATE */);
    return;
  }
  const int b = t / G, g = t - (t / G) * G;
  const int kF = g * KG, nk = min(K - kF, KG);
  const int jb = 32 * b - 2 * kF;  // first row of the group's first sweep
  const int nrw = 32 + 2 * (nk - 1);
  const int rA = jb - 2 * (nk - 1);  // first row of the block's rings
  const int T = S + 32 + kSwLg * (nk - 1);
  const int NP = (T + kSwQ - 1) / kSwQ;
  auto rows_active = [&](int k) {  // sweep k's rows of strip b meet the grid
    const int j0 = 32 * b - 2 * k;
    return j0 <= S - 1 && j0 + 31 >= 0;
  };
  const int role = sw_role(warp, KG, nk);
  const LsSwLayout lay = ls_sw_layout(KG);
  float* const VR = reinterpret_cast<float*>(ls_sw_smem + lay.vr);
  float* const UI = reinterpret_cast<float*>(ls_sw_smem + lay.ui);
  float* const VP = reinterpret_cast<float*>(ls_sw_smem + lay.vp);
  float* const X0R = reinterpret_cast<float*>(ls_sw_smem + lay.x0r);
  uint8_t* const CR = ls_sw_smem + lay.cr;
  float* const XR = reinterpret_cast<float*>(ls_sw_smem + lay.xr);
  const unsigned long long* const gexpIn =
      g > 0 ? A.gexp + ((size_t)b * (G - 1) + (g - 1)) * (A.RE + 1) * kSwGrpWords : nullptr;

  // A copy loop: chunk copies issued kSwAH periods before their use period,
  // the use period cp + 1 landed before the barrier that ends period cp.
  auto copy_loop = [&](auto issue) {
    for (int cp = -kSwAH - 1; cp < 0; ++cp) issue(cp);
    cp_async_wait<kSwAH - 1>();  // use periods -1 and 0 have landed
    if (!__syncthreads_or(0)) {
      for (int cp = 0; cp < NP; ++cp) {
        issue(cp);
        cp_async_wait<kSwAH - 1>();  // use period cp + 1 has landed
        if (__syncthreads_or(0)) break;
      }
    }
    cp_async_wait<0>();
  };
  if (role == KG) {
    // ---- the copy warp: x0 / code rows (the frame rows 0 and S-1: x, the
    // frame values the sweeps see). Lane l copies rows l and l + 32 of the
    // rings; row q's 4-column chunk n = u + c(q) is first read in use period u
    // (c(q) from the first sweep that reads the row).
    const float* gx[2];
    const uint8_t* gc[2];
    int cq[2], qs[2];
#pragma unroll
    for (int s2 = 0; s2 < 2; ++s2) {
      const int q = lane + 32 * s2, r = rA + q;
      const bool ok = q < nrw && r >= 0 && r <= S - 1;
      const int dr = jb - r;
      const int kmin = dr > 0 ? (dr + 1) >> 1 : 0;
      cq[s2] = ok ? (dr - (kSwLg + 2) * kmin + 3) >> 2 : -(1 << 28);
      gx[s2] = (r == 0 || r == S - 1 ? A.x : A.x0) + (size_t)(ok ? r : 0) * P;
      gc[s2] = A.code + (size_t)(ok ? r : 0) * P;
      qs[s2] = q;
    }
    copy_loop([&](int cp) {
#pragma unroll
      for (int s2 = 0; s2 < 2; ++s2) {
        const int n = cp + kSwAH + cq[s2];
        if (n >= 0 && 4 * n < P) {
          const int sc = (4 * n) & (kSwPC - 1);
          cp_async16(&X0R[qs[s2] * kSwPCS + sc], gx[s2] + 4 * n, true);
          cp_async4(&CR[qs[s2] * kSwCCS + sc], gc[s2] + 4 * n, true);
          if (sc == 0) {  // the copy past the ring's end (the readers' period base)
            cp_async16(&X0R[qs[s2] * kSwPCS + kSwPC], gx[s2] + 4 * n, true);
            cp_async4(&CR[qs[s2] * kSwCCS + kSwPC], gc[s2] + 4 * n, true);
          }
        }
      }
      cp_async_commit();
    });
  } else if (role == KG + 1 && g == 0) {
    // ---- the first group has no group import: this warp copies the initial
    // x rows its first sweep reads (row q's chunk u + 1 - ceil(q / 4) is first
    // read in use period u)
    const float* gx[2];
    int cq[2], qs[2];
#pragma unroll
    for (int s2 = 0; s2 < 2; ++s2) {
      const int q = lane + 32 * s2, r = jb + q;
      const bool ok = q < 33 && r <= S - 1;
      cq[s2] = ok ? 1 - ((q + 3) >> 2) : -(1 << 28);
      gx[s2] = A.x + (size_t)(ok ? r : 0) * P;
      qs[s2] = q;
    }
    copy_loop([&](int cp) {
#pragma unroll
      for (int s2 = 0; s2 < 2; ++s2) {
        const int n = cp + kSwAH + cq[s2];
        if (n >= 0 && 4 * n < P) {
          const int sc = (4 * n) & (kSwPX - 1);
          cp_async16(&XR[qs[s2] * kSwPXS + sc], gx[s2] + 4 * n, true);
          if (sc == 0) cp_async16(&XR[qs[s2] * kSwPXS + kSwPX], gx[s2] + 4 * n, true);
        }
      }
      cp_async_commit();
    });
  } else if (role == KG + 1) {
    // ---- the group import warp: the previous group's last sweep, per period
    // 4 records x 34 words (positions -2 .. 31) of the diagonals d - 1 the
    // first sweep reads in that period; slot s of lane l is word l + 32 s
    const bool on = g > 0 && rows_active(kF);
    auto rec_of = [&](int u, int s) { return u * kSwQ + (lane + 32 * s) / 34; };
    auto ok_of = [&](int u, int s) {
      const int w = lane + 32 * s, r = rec_of(u, s);
      return on && w < 4 * 34 && r >= 0 && r <= S + 31;
    };
    auto addr_of = [&](int u, int s) {
      const int w = lane + 32 * s;
      return gexpIn + (size_t)rec_of(u, s) * kSwGrpWords + (w % 34);
    };
    auto load = [&](int u, unsigned long long* v) {
#pragma unroll
      for (int s = 0; s < 5; ++s) v[s] = ok_of(u, s) ? ld_relaxed_u64(addr_of(u, s)) : 0ull;
    };
    // spin until the words of use period u carry the launch's tag (bounded);
    // with put, copy them into the previous-sweep ring
    auto settle = [&](int u, unsigned long long* v, bool put) -> bool {
      bool bad = false;
#pragma unroll
      for (int s = 0; s < 5; ++s) bad |= ok_of(u, s) && (unsigned)(v[s] >> 32) != tag;
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
        bad = false;
#pragma unroll
        for (int s = 0; s < 5; ++s) {
          if (ok_of(u, s) && (unsigned)(v[s] >> 32) != tag) {
            v[s] = ld_relaxed_u64(addr_of(u, s));
            bad |= (unsigned)(v[s] >> 32) != tag;
          }
        }
      }
#pragma unroll
      for (int s = 0; s < 5; ++s) {
        if (put && ok_of(u, s)) {
          const int w = lane + 32 * s;
          const int r = rec_of(u, s);  // diagonal r - 1, in slot r
          VP[(r & (kSwRD - 1)) * kSwRW + (w % 34)] =
              __uint_as_float((unsigned)(v[s] & 0xffffffffull));
        }
      }
      return true;
    };
    // loads in flight: wv[q] holds the words of use period cp + 1 + q
    unsigned long long wv[kSwAHI][5];
    load(0, wv[0]);
    bool ok0 = settle(0, wv[0], true);
    // start only once the previous group is A.slack periods ahead, so that
    // the loads issued kSwAHI periods early find their words written
    if (ok0 && on) {
      const int us = min(1 + A.slack, (S + 31) / kSwQ);
      unsigned long long ws[5];
      load(us, ws);
      ok0 = settle(us, ws, false);
    }
#pragma unroll
    for (int q = 0; q < kSwAHI; ++q) load(1 + q, wv[q]);
    if (!__syncthreads_or(!ok0)) {  // the prologue counts as period -1
      for (int cp = 0; cp < NP; ++cp) {
        const bool bad = !settle(cp + 1, wv[0], true);
#pragma unroll
        for (int q = 0; q + 1 < kSwAHI; ++q)
#pragma unroll
          for (int s = 0; s < 5; ++s) wv[q][s] = wv[q + 1][s];
        load(cp + 1 + kSwAHI, wv[kSwAHI - 1]);
        if (__syncthreads_or(bad)) break;
      }
    }
  } else if (role == KG + 2) {
    // ---- the halo import warp: strip b-1's exports for every sweep warp of
    // the block, copied into its rings one period before their use (lane 0's
    // U ring, ring positions -2 and -1). Word w = lane + 32 s of a period is
    // word {0, 2, 3}[t % 3] of record t / 3 (t = w % 12) for sweep w / 12.
    bool hon[4];
    int hdd0[4], hslot0[4], hstr[4];
    const unsigned long long* hin[4];
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const int w = lane + 32 * s, kk = w / 12, tt = w - 12 * (w / 12);
      const int k = kF + kk;
      const int jp = 32 * (b - 1) - 2 * k;  // strip b-1's rows of sweep k (the producer)
      hon[s] = w < 12 * nk && b > 0 && jp <= S - 1 && jp + 31 >= 0;
      const int iwi = tt - 3 * (tt / 3), iw = iwi == 0 ? 0 : iwi + 1;
      hdd0[s] = -kSwLg * kk - 1 + tt / 3;  // diagonal of period u: u kSwQ + hdd0
      // U ring slot base (word 2) or ring position -2 / -1 (words 0 / 3)
      hslot0[s] = iw == 2 ? (int)(lay.ui / 4) + kk * kSwRD
                          : (int)(lay.vr / 4) + kk * kSwRD * kSwRW + (iw == 0 ? 0 : 1);
      hstr[s] = iw == 2 ? 1 : kSwRW;
      hin[s] = hon[s] ? A.edge + ((size_t)(b - 1) * K + k) * A.RE * 4 + iw : nullptr;
    }
    auto ok_of = [&](int u, int s) {
      const int dd = u * kSwQ + hdd0[s];
      return hon[s] && dd >= -1 && dd <= S - 2;
    };
    auto addr_of = [&](int u, int s) { return hin[s] + (size_t)(u * kSwQ + hdd0[s] + 32) * 4; };
    auto load = [&](int u, unsigned long long* v) {
#pragma unroll
      for (int s = 0; s < 4; ++s) v[s] = ok_of(u, s) ? ld_relaxed_u64(addr_of(u, s)) : 0ull;
    };
    float* const smf = reinterpret_cast<float*>(ls_sw_smem);
    // spin until the words of use period u carry the launch's tag (bounded);
    // with put, copy them into the rings (diagonal dd lives in slot dd + 1)
    auto settle = [&](int u, unsigned long long* v, bool put) -> bool {
      bool bad = false;
#pragma unroll
      for (int s = 0; s < 4; ++s) bad |= ok_of(u, s) && (unsigned)(v[s] >> 32) != tag;
      long long tries = 0;
      unsigned ns = 0;  // re-poll at once, then back off
      while (__any_sync(FULL, bad)) {
        if (++tries > A.spin_limit) {
          if (lane == 0) atomicExch(A.err, 3 /* EQ_ERR_TIMEOUT */);
          return false;
        }
        if ((tries & 63) == 0 && __any_sync(FULL, ld_relaxed_i32(A.err) != 0)) return false;
        if (ns) __nanosleep(ns);
        ns = tries < 4 ? 0u : (ns < 32 ? 32u : (ns < 256 ? ns * 2 : 256u));
        bad = false;
#pragma unroll
        for (int s = 0; s < 4; ++s) {
          if (ok_of(u, s) && (unsigned)(v[s] >> 32) != tag) {
            v[s] = ld_relaxed_u64(addr_of(u, s));
            bad |= (unsigned)(v[s] >> 32) != tag;
          }
        }
      }
#pragma unroll
      for (int s = 0; s < 4; ++s) {
        if (put && ok_of(u, s)) {
          const int slot = (u * kSwQ + hdd0[s] + 1) & (kSwRD - 1);
          smf[hslot0[s] + slot * hstr[s]] = __uint_as_float((unsigned)(v[s] & 0xffffffffull));
        }
      }
      return true;
    };
    unsigned long long hv[kSwAHI][4];  // hv[q]: the words of use period cp + 1 + q
    load(0, hv[0]);
    bool ok0 = settle(0, hv[0], true);  // the prologue: imports of period 0
    // start only once strip b-1 is A.slack periods ahead, so that the loads
    // issued kSwAHI periods early find their words written
    if (ok0 && A.slack > 0) {
      unsigned long long ws[4];
      load(1 + A.slack, ws);
      ok0 = settle(1 + A.slack, ws, false);
    }
#pragma unroll
    for (int q = 0; q < kSwAHI; ++q) load(1 + q, hv[q]);
    if (!__syncthreads_or(!ok0)) {  // the prologue counts as period -1
      for (int cp = 0; cp < NP; ++cp) {
        const bool bad = !settle(cp + 1, hv[0], true);
#pragma unroll
        for (int q = 0; q + 1 < kSwAHI; ++q)
#pragma unroll
          for (int s = 0; s < 4; ++s) hv[q][s] = hv[q + 1][s];
        load(cp + 1 + kSwAHI, hv[kSwAHI - 1]);
        if (__syncthreads_or(bad)) break;
      }
    }
  } else if (role == KG + 3) {
    // ---- the group export warp: the group's last sweep (kk = nk - 1) leaves
    // its ring row of diagonal d - 1 complete (positions -2 .. 31, with the
    // imported halo and any lane-0 fix) at the end of the period that holds
    // step d; this warp stores it as record d (word p + 2 = position p) for
    // group g+1's import warp during the next period (the ring keeps it for
    // kSwRD steps).
    const int kx = nk - 1, k = kF + kx;
    const bool on = g < G - 1 && (rows_active(k) || rows_active(k + 1));
    unsigned long long* const out =
        on ? A.gexp + ((size_t)b * (G - 1) + g) * (A.RE + 1) * kSwGrpWords : nullptr;
    const float* const ring = VR + (size_t)kx * kSwRD * kSwRW;
    auto export_period = [&](int p) {  // the records of period p
#pragma unroll
      for (int s = 0; s < 5; ++s) {
        const int w = lane + 32 * s;  // word w % 34 of record q = w / 34
        const int q = w / 34, word = w - 34 * (w / 34);
        const int d = p * kSwQ - kSwLg * kx + q;
        if (w < 4 * 34 && d >= 0 && d <= S + 31)
          sw_st1(out + (size_t)d * kSwGrpWords + word, ring[(d & (kSwRD - 1)) * kSwRW + word], tag);
      }
    };
    int done = -1;  // the last period whose records are out
    if (!__syncthreads_or(0)) {  // the prologue counts as period -1
      for (int cp = 0; cp < NP; ++cp) {
        if (on && cp > 0) export_period(cp - 1);
        done = cp - 1;
        if (__syncthreads_or(0)) break;
      }
      if (on && done == NP - 2) export_period(NP - 1);  // after the last barrier
    }
  } else {
    // ---- sweep warp kk (k = kF + kk); warps past nk only meet the barriers
    const int kk = role, k = kF + kk;
    const bool real = kk < nk;
    const bool exportGroup = real && g < G - 1 && kk == nk - 1;
    const bool runs = real && (rows_active(k) || (exportGroup && rows_active(k + 1)));
    SwWarp W;
    W.lane = lane;
    W.S = S;
    W.N = N;
    W.k = k;
    const int j0 = jb - 2 * kk;
    W.j = j0 + lane;
    W.interior = W.j >= 1 && W.j <= N;
    W.top = W.j == 0;
    W.bot = W.j == S - 1;
    W.idle = !(W.interior || W.top || W.bot);
    const bool hasFrame = __any_sync(FULL, W.top || W.bot);
    W.pasRow = MODE == kPassive && W.interior && A.rowfl[W.j] != 0;
    W.cfTop = (MODE == kPassive && W.top && k > 0) ? kCodeColFluid : 0u;
    W.cfBot = (MODE == kPassive && W.bot) ? kCodeColFluid : 0u;
    W.xL = W.interior ? A.x[(size_t)W.j * P] : 0.0f;
    W.xR = W.interior ? A.x[(size_t)W.j * P + (S - 1)] : 0.0f;
    W.a = A.a;
    W.cr = A.cr;
    const int kr = real ? kk : 0;
    W.own = VR + (size_t)kr * kSwRD * kSwRW;
    W.prev = kk > 0 ? VR + (size_t)(kk - 1) * kSwRD * kSwRW : VP;
    W.ui = UI + (size_t)kr * kSwRD;
    const int rrow = 2 * (nk - 1 - kr) + lane;
    W.x0row = X0R + (real ? rrow : 0) * kSwPCS;
    W.crow = CR + (real ? rrow : 0) * kSwCCS;
    W.xrl = XR + lane * kSwPXS;
    W.xrd = XR + (lane + 1) * kSwPXS;
    W.edgeOn = real && b < B - 1 && lane >= 30;
    W.edgeOut = W.edgeOn ? A.edge + ((size_t)b * K + k) * A.RE * 4 + (lane == 30 ? 0 : 2) : A.edge;
    W.xlast = (real && k == K - 1) ? A.x + (size_t)max(W.j, 0) * P - lane : nullptr;
    W.tag = tag;
    W.vcur = W.vprev = W.uprev = 0.0f;
    W.cprev = 0u;
    const bool firstX = g == 0 && kk == 0;
    // fast range: every interior lane at 2 <= i <= N
    const int lA = max(0, 1 - j0), lB = min(31, N - j0);
    const int dF0 = lA <= lB ? lB + 2 : 1 << 30, dF1 = lA <= lB ? lA + N : -(1 << 30);
    if (!__syncthreads_or(0)) {  // the prologue counts as period -1
      for (int cp = 0; cp < NP; ++cp) {
        if (runs) {
          const int dp = cp * kSwQ - kSwLg * kk;
          if (dp >= dF0 && dp + kSwQ - 1 <= dF1) {
            if (firstX) {
              if (hasFrame)
                sw_period_fast<MODE, true, true>(W, dp);
              else
                sw_period_fast<MODE, true, false>(W, dp);
            } else if (hasFrame) {
              sw_period_fast<MODE, false, true>(W, dp);
            } else {
              sw_period_fast<MODE, false, false>(W, dp);
            }
          } else if (firstX) {
            if (hasFrame)
              sw_period_edge<MODE, true, true>(W, dp);
            else
              sw_period_edge<MODE, true, false>(W, dp);
          } else if (hasFrame) {
            sw_period_edge<MODE, false, true>(W, dp);
          } else {
            sw_period_edge<MODE, false, false>(W, dp);
          }
        }
        if (__syncthreads_or(0)) break;
      }
    }
  }
  // ---- completion: the last block to finish (every block has taken its
  // ticket) resets the ticket and done counters for the next launch on the
  // stream and advances the epoch
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned prev = atom_add_acq_rel_u32(&A.ctr[1], 1u);
    if (prev == (unsigned)(B * G) - 1u) {
      atomicExch(&A.ctr[0], 0u);
      atomicExch(&A.ctr[1], 0u);
      atomicAdd(&A.ctr[2], 1u);
    }
  }
}

}  // namespace eqk
