// C ABI (include/eqfluid.h) and host orchestration of the sm_103a frame step.
//
// One handle = one scene: the six pitched f32 grids of Fluid (fluid.rs:59-77),
// a spare grid for lin_solve's double buffering, the wall mask with its
// derived per-cell boundary codes, and the lin_solve wavefront's sync state.
// Every launch goes to the handle's own stream; nothing here falls back to
// the CPU -- if a CUDA call fails the entry point reports EQ_ERR_CUDA.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/eqfluid.h"
#include "common.cuh"
#include "kernels.cuh"
#include "linsolve.cuh"
#include "lscl.cuh"
#include "lscs.cuh"
#include "lssw.cuh"

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

#define EQ_CUDA(call)                                                                   \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return fail(EQ_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));     \
  } while (0)

constexpr int kMaxSweepsPerLaunch = 64;
constexpr int kSwMaxGroups = 5;  // sweep groups per strip of the strip wavefront
constexpr int kSwStaticSmem = 1024;  // reserved beside its dynamic shared memory
constexpr long long kDefaultSpinLimit = 1ll << 22;

}  // namespace

struct eq_fluid {
  int device = 0;
  cudaStream_t stream = nullptr;
  uint32_t S = 0;
  int P = 0;  // row pitch (elements)
  float dt = 0.f, diff = 0.f, visc = 0.f;
  int64_t frames = 0;
  int32_t has_perlin_noise = 0;

  float* block = nullptr;  // the 6 grids
  float* field[6] = {};
  uint8_t* cells = nullptr;  // pitched mask, 1 = wall
  uint8_t* code = nullptr;   // pitched boundary codes
  uint8_t* rowfl = nullptr;  // [S] row has a fluid cell
  uint8_t* colfl = nullptr;  // [S] column has a fluid cell
  std::vector<uint8_t> host_cells;  // authoritative mirror of cells_type
  bool mask_dirty = true;

  // lin_solve wavefront state
  int B = 0;  // strips for kMaxSweepsPerLaunch
  unsigned long long* wt = nullptr;    // 2 sequence-tagged grids
  unsigned long long* edge = nullptr;  // tagged last rows [B*64][P]
  unsigned* counters = nullptr;        // [0] ticket, [1] done
  uint32_t tag = 1;                    // next W(-1) tag (monotonic)
  int* err = nullptr;

  // Concurrent phases of one step: two side streams (the vy diffusion and the
  // density diffusion run beside the vx diffusion and the velocity pipeline),
  // fork / join events, and the side solves' own wavefront state (slots 1, 2;
  // slot 0 is wt / edge / counters / tag above). `cur` / `cur_slot` are the
  // stream and slot the launch helpers use (the main stream and slot 0
  // outside launch_step's side branches). `concurrent`: which diffusions run
  // on a side stream (EQ_CONC_* bits).
  int concurrent = EQ_CONC_VY | EQ_CONC_DENSITY;
  cudaStream_t cur = nullptr;
  int cur_slot = 0;
  cudaStream_t side[2] = {};
  cudaEvent_t fork_ev = nullptr;
  cudaEvent_t join_ev[2] = {};
  unsigned long long* xwt[2] = {};
  unsigned long long* xedge[2] = {};
  unsigned* xcounters[2] = {};
  uint32_t xtag[2] = {1, 1};
  long long spin_limit = kDefaultSpinLimit;

  // dense staging of eq_fluid_read_fields (grown on demand)
  float* d_pack = nullptr;
  size_t d_pack_cap = 0;  // floats
  // eq_fluid_read_fields_async: two staging buffers used in turn, copied to
  // the host on their own stream while the next step runs
  float* d_apack[2] = {};
  size_t d_apack_cap = 0;  // floats, each
  int apack_next = 0;
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t apack_ev[2] = {}, acopy_ev[2] = {};

  // source staging
  uint8_t* d_src = nullptr;
  size_t d_src_cap = 0;
  uint8_t* h_src = nullptr;  // pinned
  size_t h_src_cap = 0;
  cudaEvent_t src_ev = nullptr;

  uint64_t launches = 0;

  // optional kernel timing (event pairs around each wavefront launch)
  bool profiling = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ls_events;

  // around the step: noise counter, rendered image, captured frame loop
  unsigned long long* noise_counter = nullptr;
  void* rgba = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int64_t gframes = -1, gK = -1;
  bool gnoise = false;
  uint64_t gseed = 0;
  float gdt = 0.f, gdiff = 0.f, gvisc = 0.f;
  uint64_t glaunches = 0;
  bool graph_mode = false;  // lin_solve clears its tagged buffers (graph replay)

  // lin_solve form: 0 auto (the cluster wavefront where it applies), 1 the
  // multi-block wavefront always, 2 the cluster wavefront where it applies
  int solver = 0;
  int64_t cl_K = -1;  // sweep count the cluster check below was made for
  int cl_blocks = 0;  // blocks per cluster for cl_K, 0 = not applicable
  int cl_m = 0;       // its barrier interval - 1 (lscl.cuh)
  int cl_kind = 0;    // 1: strips staged whole (k_ls_cl), 2: streamed (k_ls_cs)
  int cl_H = 1;       // positions per lane of the streamed form
  // the streamed form's strip-ordered codes, one copy per mode (lscs.cuh),
  // rebuilt with the mask; allocated where the streamed form can apply
  uint8_t* cs_strip = nullptr;
  int cs_C = 0, cs_J = 0;
  int cl_mmax = -1;   // cap on cl_m; -1: 2 for N >= 192, else 1 (the fastest, measured)
  // the strip wavefront (lssw.cuh), one set per stream slot: tagged exports
  // [strips-1][sweeps][records][4] and counters (ticket, done, epoch)
  unsigned long long* sw_edge[3] = {};
  unsigned long long* sw_gexp[3] = {};  // group exports [strips][groups-1][records+1][36]
  unsigned* sw_ctr[3] = {};
  int sw_groups = 0;  // sweep groups per strip (0: by size and by what runs beside)
  bool sw_pair = false;  // step(): the vx diffusion runs beside the vy diffusion
  int sw_slack = 0;   // periods a block's producers must be ahead before it starts

  size_t grid_elems() const { return (size_t)P * S; }
};

namespace {

int strips_for(int S, int K) { return (S + 2 * K + 31) / 32; }

int select_device(const eq_fluid* h) {
  EQ_CUDA(cudaSetDevice(h->device));
  return EQ_OK;
}

int check_field(int f) { return (f >= 0 && f < 6) ? EQ_OK : fail(EQ_ERR_ARG, "field index out of range"); }

int check_mode(int m) {
  return (m >= 0 && m <= 2) ? EQ_OK : fail(EQ_ERR_ARG, "mode out of range");
}

// Derives the per-cell boundary codes (pitched, P per row) and the row /
// column "has a fluid cell" flags from a dense size*size wall mask.
void derive_codes(const std::vector<uint8_t>& m, int S, int P, uint8_t* code, uint8_t* rowfl,
                  uint8_t* colfl) {
  const int N = S - 2;
  auto wall = [&](int i, int j) { return m[(size_t)j * S + i] != 0; };
  std::memset(code, 0, (size_t)P * S);
  std::memset(rowfl, 0, S);
  std::memset(colfl, 0, S);
  for (int j = 0; j < S; ++j) {
    for (int i = 0; i < S; ++i) {
      uint8_t c = 0;
      const bool w = wall(i, j);
      if (w) c |= eqk::kCodeWall;
      if (!w && i >= 1 && i <= N && j >= 1 && j <= N) {
        rowfl[j] = 1;
        colfl[i] = 1;
        if (wall(i + 1, j))
          c |= eqk::kCodeRowRight;
        else if (wall(i - 1, j))
          c |= eqk::kCodeRowLeft;
        if (wall(i, j - 1))
          c |= eqk::kCodeColUp;
        else if (wall(i, j + 1))
          c |= eqk::kCodeColDown;
      }
      // (i, j-1) has kCodeColDown: it is fluid, (i, j-2) is not a wall, (i, j) is.
      if (j >= 2 && j - 1 <= N && i >= 1 && i <= N && w && !wall(i, j - 1) &&
          !wall(i, j - 2))
        c |= eqk::kCodeAboveDown;
      code[(size_t)j * P + i] |= c;
    }
  }
  for (int j = 0; j < S; ++j)
    for (int i = 0; i < S; ++i)
      if (colfl[i]) code[(size_t)j * P + i] |= eqk::kCodeColFluid;
}

// Uploads the mask and its derived codes / flags when the mask changed.
int upload_mask(eq_fluid* h) {
  if (!h->mask_dirty) return EQ_OK;
  const int S = (int)h->S, P = h->P;
  const std::vector<uint8_t>& m = h->host_cells;
  std::vector<uint8_t> code((size_t)P * S, 0), cellsP((size_t)P * S, 0), rowfl(S, 0),
      colfl(S, 0);
  for (int j = 0; j < S; ++j)
    for (int i = 0; i < S; ++i) cellsP[(size_t)j * P + i] = m[(size_t)j * S + i] ? 1 : 0;
  derive_codes(m, S, P, code.data(), rowfl.data(), colfl.data());
  EQ_CUDA(cudaMemcpyAsync(h->cells, cellsP.data(), cellsP.size(), cudaMemcpyHostToDevice,
                          h->stream));
  EQ_CUDA(cudaMemcpyAsync(h->code, code.data(), code.size(), cudaMemcpyHostToDevice,
                          h->stream));
  EQ_CUDA(cudaMemcpyAsync(h->rowfl, rowfl.data(), S, cudaMemcpyHostToDevice, h->stream));
  EQ_CUDA(cudaMemcpyAsync(h->colfl, colfl.data(), S, cudaMemcpyHostToDevice, h->stream));
  if (h->cs_strip) {  // the streamed cluster solver's strip-ordered codes, per mode
    const size_t sb = eqk::ls_cs_strip_bytes(S, h->cs_C, h->cs_J);
    const int blocks = (int)std::min<size_t>((sb + 255) / 256, 152 * 8);
    eqk::k_ls_cs_codes<eqk::kRow><<<blocks, 256, 0, h->stream>>>(h->cs_strip, h->code, S, P,
                                                                  h->cs_C, h->cs_J);
    eqk::k_ls_cs_codes<eqk::kCol><<<blocks, 256, 0, h->stream>>>(h->cs_strip + sb, h->code, S,
                                                                  P, h->cs_C, h->cs_J);
    eqk::k_ls_cs_codes<eqk::kPassive><<<blocks, 256, 0, h->stream>>>(
        h->cs_strip + 2 * sb, h->code, S, P, h->cs_C, h->cs_J);
    h->launches += 3;
    EQ_CUDA(cudaGetLastError());
  }
  // The staging vectors are pageable: the async copies above are staged
  // synchronously, but wait anyway before they go out of scope.
  EQ_CUDA(cudaStreamSynchronize(h->stream));
  h->mask_dirty = false;
  return EQ_OK;
}

int check_launch(eq_fluid* h) {
  h->launches++;
  EQ_CUDA(cudaGetLastError());
  return EQ_OK;
}

dim3 grid2d(int nx, int ny, dim3 blk) {
  return dim3((nx + blk.x - 1) / blk.x, (ny + blk.y - 1) / blk.y);
}

int launch_bnd(eq_fluid* h, int mode, float* x) {
  const dim3 blk(32, 8);
  const dim3 grd = grid2d((int)h->S, (int)h->S, blk);
  switch (mode) {
    case eqk::kRow:
      eqk::k_set_boundaries<eqk::kRow><<<grd, blk, 0, h->cur>>>(x, h->code, h->rowfl, h->colfl, (int)h->S, h->P);
      break;
    case eqk::kCol:
      eqk::k_set_boundaries<eqk::kCol><<<grd, blk, 0, h->cur>>>(x, h->code, h->rowfl, h->colfl, (int)h->S, h->P);
      break;
    default:
      eqk::k_set_boundaries<eqk::kPassive><<<grd, blk, 0, h->cur>>>(x, h->code, h->rowfl, h->colfl, (int)h->S, h->P);
      break;
  }
  return check_launch(h);
}

// Blocks per cluster for the cluster wavefront (lscl.cuh) at this size and
// sweep count, or 0 where it does not apply: one warp per sweep (K <= 32),
// strips of 16 to 32 positions, the staged strip and band within the opt-in
// shared memory, and a device that can hold the cluster.
// Raises the dynamic shared memory limit and allows 16-block clusters for a
// set of cluster kernels, once per device (bit `set` of a per-device mask).
bool raise_cluster_attrs(int device, int set, const void* const* fns, int nfn, int optin) {
  static std::atomic<uint64_t> raised[4];
  const uint64_t bit = device < 64 ? (1ull << device) : 0ull;
  if (bit && (raised[set].load() & bit)) return true;
  for (int q = 0; q < nfn; ++q)
    if (cudaFuncSetAttribute(fns[q], cudaFuncAttributeMaxDynamicSharedMemorySize, optin) !=
            cudaSuccess ||
        cudaFuncSetAttribute(fns[q], cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
            cudaSuccess) {
      cudaGetLastError();
      return false;
    }
  raised[set].fetch_or(bit);
  return true;
}

// Blocks per cluster of the cluster wavefront for K sweeps (0: it does not
// apply). Strips of J <= 32 positions whose x0, initial x and codes fit in
// shared memory whole use k_ls_cl (lscl.cuh); otherwise strips of J <= 64
// stream them (k_ls_cs, lscs.cuh). Either needs a cluster of C <= 16 blocks
// that can be resident.
int cluster_blocks(eq_fluid* h, int64_t K) {
  if (h->cl_K == K) return h->cl_blocks;
  h->cl_K = K;
  h->cl_blocks = 0;
  h->cl_kind = 0;
  const int S = (int)h->S, N = S - 2;
  if (K < 1 || K > 32 || N < 32) return 0;
  const int C = std::min(16, (N + 31) / 32), J = (N + C - 1) / C;
  if (C < 2 || J > 64 || J < 16 || (C - 1) * J >= N) return 0;
  int optin = 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device) !=
      cudaSuccess)
    return 0;
  const int mcap = h->cl_mmax >= 0 ? h->cl_mmax : (N >= 192 ? 2 : 1);
  int kind = 0, m = 0, H = 1;
  size_t bytes = 0;
  if (J <= 32) {  // the longest barrier interval whose strips still fit whole
    m = mcap;
    while (m > 0 && eqk::ls_cl_layout(S, (int)K, C, m).total > (size_t)optin) --m;
    bytes = eqk::ls_cl_layout(S, (int)K, C, m).total;
    if (bytes <= (size_t)optin) kind = 1;
  }
  if (!kind && h->cs_strip && h->cs_C == C && h->cs_J == J && K <= 31) {
    // the streamed rings' bound holds for m <= 3; 3 is the fastest measured
    m = h->cl_mmax >= 0 ? std::min(h->cl_mmax, 3) : 3;
    while (m > 0 && eqk::ls_cs_layout(S, (int)K, C, m).total > (size_t)optin) --m;
    bytes = eqk::ls_cs_layout(S, (int)K, C, m).total;
    if (bytes <= (size_t)optin) {
      kind = 2;
      H = J > 32 ? 2 : 1;
    }
  }
  if (!kind) return 0;
  const void* fns[3];
  int set = 0;
  if (kind == 1) {
    fns[0] = (const void*)eqk::k_ls_cl<eqk::kRow>;
    fns[1] = (const void*)eqk::k_ls_cl<eqk::kCol>;
    fns[2] = (const void*)eqk::k_ls_cl<eqk::kPassive>;
  } else if (H == 1) {
    set = 1;
    fns[0] = (const void*)eqk::k_ls_cs<eqk::kRow, 1>;
    fns[1] = (const void*)eqk::k_ls_cs<eqk::kCol, 1>;
    fns[2] = (const void*)eqk::k_ls_cs<eqk::kPassive, 1>;
  } else {
    set = 2;
    fns[0] = (const void*)eqk::k_ls_cs<eqk::kRow, 2>;
    fns[1] = (const void*)eqk::k_ls_cs<eqk::kCol, 2>;
    fns[2] = (const void*)eqk::k_ls_cs<eqk::kPassive, 2>;
  }
  if (!raise_cluster_attrs(h->device, set, fns, 3, optin)) return 0;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(C);
  cfg.blockDim = dim3(32 * (unsigned)(kind == 1 ? K : K + 1));
  cfg.dynamicSmemBytes = bytes;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int nclusters = 0;
  if (cudaOccupancyMaxActiveClusters(&nclusters, fns[2], &cfg) == cudaSuccess && nclusters >= 1) {
    h->cl_blocks = C;
    h->cl_kind = kind;
    h->cl_H = H;
    h->cl_m = m;
  }
  cudaGetLastError();
  return h->cl_blocks;
}

// lin_solve by the cluster wavefront, then set_boundaries of the last sweep.
int launch_lin_solve_cluster(eq_fluid* h, int mode, float* x, const float* x0, float a,
                             float c_recip, int C) {
  const int S = (int)h->S;
  const int K = (int)h->frames;
  const bool streamed = h->cl_kind == 2;
  eqk::LsClArgs A;
  A.x = x;
  A.x0 = x0;
  A.code = h->code;
  A.rowfl = h->rowfl;
  A.colfl = h->colfl;
  A.S = S;
  A.P = h->P;
  A.K = K;
  A.m = h->cl_m;
  A.R = eqk::ls_cl_rows(K, A.m);
  A.a = a;
  A.cr = c_recip;
  A.strip = streamed ? h->cs_strip + (size_t)mode * eqk::ls_cs_strip_bytes(S, h->cs_C, h->cs_J)
                     : nullptr;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(C);
  cfg.blockDim = dim3(32 * (unsigned)(streamed ? K + 1 : K));
  cfg.dynamicSmemBytes = streamed ? eqk::ls_cs_layout(S, K, C, A.m).total
                                  : eqk::ls_cl_layout(S, K, C, A.m).total;
  cfg.stream = h->cur;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  if (h->profiling) {
    EQ_CUDA(cudaEventCreate(&ev0));
    EQ_CUDA(cudaEventCreate(&ev1));
    EQ_CUDA(cudaEventRecord(ev0, h->cur));
  }
  if (!streamed) {
    switch (mode) {
      case eqk::kRow:
        EQ_CUDA(cudaLaunchKernelEx(&cfg, eqk::k_ls_cl<eqk::kRow>, A));
        break;
      case eqk::kCol:
        EQ_CUDA(cudaLaunchKernelEx(&cfg, eqk::k_ls_cl<eqk::kCol>, A));
        break;
      default:
        EQ_CUDA(cudaLaunchKernelEx(&cfg, eqk::k_ls_cl<eqk::kPassive>, A));
        break;
    }
  } else if (h->cl_H == 1) {
    switch (mode) {
      case eqk::kRow:
        EQ_CUDA(cudaLaunchKernelEx(&cfg, eqk::k_ls_cs<eqk::kRow, 1>, A));
        break;
      case eqk::kCol:
        EQ_CUDA(cudaLaunchKernelEx(&cfg, eqk::k_ls_cs<eqk::kCol, 1>, A));
        break;
      default:
        EQ_CUDA(cudaLaunchKernelEx(&cfg, eqk::k_ls_cs<eqk::kPassive, 1>, A));
        break;
    }
  } else {
    switch (mode) {
      case eqk::kRow:
        EQ_CUDA(cudaLaunchKernelEx(&cfg, eqk::k_ls_cs<eqk::kRow, 2>, A));
        break;
      case eqk::kCol:
        EQ_CUDA(cudaLaunchKernelEx(&cfg, eqk::k_ls_cs<eqk::kCol, 2>, A));
        break;
      default:
        EQ_CUDA(cudaLaunchKernelEx(&cfg, eqk::k_ls_cs<eqk::kPassive, 2>, A));
        break;
    }
  }
  int rc = check_launch(h);
  if (rc) return rc;
  if (h->profiling) {
    EQ_CUDA(cudaEventRecord(ev1, h->cur));
    h->ls_events.emplace_back(ev0, ev1);
  }
  return launch_bnd(h, mode, x);
}

// Sweep groups of the strip wavefront for K sweeps on this grid: blocks of
// one strip share its sweeps so that about one block per SM works on a solve.
// The two velocity diffusions that step() runs side by side (the critical
// path) take the fewest groups, so that both fit the SMs at once; the density
// diffusion beside them (lower stream priority, needed only at the frame's
// end) keeps about one block per SM (N = 1024, 20 sweeps: 1.91 ms a step,
// against 1.98 with one block per SM for all three and 1.94 with the fewest).
int sw_groups_for(const eq_fluid* h, int K) {
  int G = h->sw_groups;
  if (G <= 0) {
    const int B = eqk::ls_sw_strips((int)h->S, K);
    G = (h->sw_pair || h->cur_slot == 1)
            ? 1
            : std::max(1, std::min(kSwMaxGroups, 152 / std::max(B, 1)));
  }
  G = std::min(G, std::min(K, kSwMaxGroups));
  G = std::max(G, (K + eqk::kSwMaxKG - 1) / eqk::kSwMaxKG);  // at most kSwMaxKG sweeps a block
  const int KG = (K + G - 1) / G;
  return (K + KG - 1) / KG;  // groups that hold a sweep
}

// Whether the strip wavefront's shared memory fits for the sweep groups of
// this grid (its rings grow with the sweeps a block holds, not with the size).
bool sw_fits(const eq_fluid* h) {
  int optin = 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device) !=
      cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  const int K = (int)std::min<int64_t>(eqk::kSwMaxK, std::max<int64_t>(h->frames, 1));
  const int G = sw_groups_for(h, K);
  return eqk::ls_sw_layout((K + G - 1) / G).total <= (size_t)(optin - kSwStaticSmem);
}

// lin_solve by the strip wavefront (lssw.cuh), kSwMaxK sweeps per launch,
// each launch finished by set_boundaries of its last sweep.
int launch_lin_solve_sw(eq_fluid* h, int mode, float* x, const float* x0, float a,
                        float c_recip) {
  static std::atomic<uint64_t> raised{0};
  const uint64_t bit = h->device < 64 ? (1ull << h->device) : 0ull;
  if (!bit || !(raised.load() & bit)) {
    int optin = 0;
    EQ_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device));
    const int dyn = optin - kSwStaticSmem;  // room for the kernel's static shared words
    EQ_CUDA(cudaFuncSetAttribute(eqk::k_ls_sw<eqk::kRow>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, dyn));
    EQ_CUDA(cudaFuncSetAttribute(eqk::k_ls_sw<eqk::kCol>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, dyn));
    EQ_CUDA(cudaFuncSetAttribute(eqk::k_ls_sw<eqk::kPassive>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, dyn));
    raised.fetch_or(bit);
  }
  const int S = (int)h->S;
  const int sl = h->cur_slot;
  for (int64_t done = 0; done < h->frames; done += eqk::kSwMaxK) {
    const int Kc = (int)std::min<int64_t>(eqk::kSwMaxK, h->frames - done);
    const int G = sw_groups_for(h, Kc);
    const int KG = (Kc + G - 1) / G;
    eqk::LsSwArgs A;  // its ticket / done counters are zero (reset by the last launch's last block)
    A.x = x;
    A.x0 = x0;
    A.code = h->code;
    A.rowfl = h->rowfl;
    A.edge = h->sw_edge[sl];
    A.gexp = h->sw_gexp[sl];
    A.ctr = h->sw_ctr[sl];
    A.err = h->err;
    A.spin_limit = h->spin_limit;
    A.S = S;
    A.P = h->P;
    A.K = Kc;
    A.B = eqk::ls_sw_strips(S, Kc);
    A.G = G;
    A.KG = KG;
    A.RE = eqk::ls_sw_records(S);
    A.slack = h->sw_slack;
    A.a = a;
    A.cr = c_recip;
    const size_t smem = eqk::ls_sw_layout(KG).total;
    const dim3 grid((unsigned)(A.B * G)), block(32u * (unsigned)(KG + eqk::kSwHelpers));
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    if (h->profiling) {
      EQ_CUDA(cudaEventCreate(&ev0));
      EQ_CUDA(cudaEventCreate(&ev1));
      EQ_CUDA(cudaEventRecord(ev0, h->cur));
    }
    switch (mode) {
      case eqk::kRow:
        eqk::k_ls_sw<eqk::kRow><<<grid, block, smem, h->cur>>>(A);
        break;
      case eqk::kCol:
        eqk::k_ls_sw<eqk::kCol><<<grid, block, smem, h->cur>>>(A);
        break;
      default:
        eqk::k_ls_sw<eqk::kPassive><<<grid, block, smem, h->cur>>>(A);
        break;
    }
    int rc = check_launch(h);
    if (rc) return rc;
    if (h->profiling) {
      EQ_CUDA(cudaEventRecord(ev1, h->cur));
      h->ls_events.emplace_back(ev0, ev1);
    }
    if ((rc = launch_bnd(h, mode, x))) return rc;
  }
  return EQ_OK;
}

// lin_solve (fluid.rs:301-325) on device grids.
int launch_lin_solve(eq_fluid* h, int mode, float* x, const float* x0, float a, float c) {
  const int64_t K = h->frames;
  if (K <= 0) return EQ_OK;
  const float c_recip = 1.0f / c;  // fluid.rs:311, IEEE f32 division
  // the strip wavefront's bulk copies read x, x0 and the codes from 16-byte
  // aligned rows (a handle's fields and codes always are)
  const bool aligned16 = (((uintptr_t)x | (uintptr_t)x0 | (uintptr_t)h->code) & 15u) == 0;
  // The strip wavefront is the fastest kernel at every measured size (N = 128
  // to 1024, alone and in step()); it runs wherever its shared memory fits.
  if ((h->solver == 0 || h->solver == 3) && aligned16 && sw_fits(h))
    return launch_lin_solve_sw(h, mode, x, x0, a, c_recip);
  if (h->solver != 1) {
    // Otherwise (and with solver 4): the staged cluster form where it
    // applies. The streamed one is slower alone than the multi-block
    // wavefront but holds only C SMs, so it takes the side-stream solves of
    // step() (beside the multi-block solve of the critical path); solver 2
    // uses it for every solve.
    const int C = cluster_blocks(h, K);
    if (C > 0 && (h->cl_kind == 1 || h->cur_slot != 0 || h->solver == 2))
      return launch_lin_solve_cluster(h, mode, x, x0, a, c_recip, C);
  }
  const int S = (int)h->S;
  // this solve's wavefront state (slot 0 on the main stream, 1 / 2 on the side streams)
  const int sl = h->cur_slot;
  unsigned long long* const wt = sl ? h->xwt[sl - 1] : h->wt;
  unsigned long long* const edge = sl ? h->xedge[sl - 1] : h->edge;
  unsigned* const counters = sl ? h->xcounters[sl - 1] : h->counters;
  uint32_t& tag = sl ? h->xtag[sl - 1] : h->tag;
  for (int64_t done = 0; done < K; done += kMaxSweepsPerLaunch) {
    const int Kc = (int)std::min<int64_t>(kMaxSweepsPerLaunch, K - done);
    if (h->graph_mode) {
      // A captured frame replays with the same tags: clear what a previous
      // replay left so that no stale word carries a current tag.
      EQ_CUDA(cudaMemsetAsync(wt, 0, 2 * h->grid_elems() * 8, h->cur));
      EQ_CUDA(cudaMemsetAsync(edge, 0, (size_t)h->B * kMaxSweepsPerLaunch * h->P * 8,
                              h->cur));
    }
    if (tag > 0xF0000000u) {  // tags would wrap: restart from clean buffers
      EQ_CUDA(cudaMemsetAsync(wt, 0, 2 * h->grid_elems() * 8, h->cur));
      EQ_CUDA(cudaMemsetAsync(edge, 0, (size_t)h->B * kMaxSweepsPerLaunch * h->P * 8,
                              h->cur));
      tag = 1;
    }
    EQ_CUDA(cudaMemsetAsync(counters, 0, 2 * sizeof(unsigned), h->cur));
    {
      const size_t n = h->grid_elems();
      const int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 8);
      eqk::k_ls_tag_init<<<blocks, 256, 0, h->cur>>>(wt, x, n, tag);
      int rc0 = check_launch(h);
      if (rc0) return rc0;
    }
    eqk::LinSolveArgs A;
    A.x = x;
    A.wt[0] = wt;
    A.wt[1] = wt + h->grid_elems();
    A.tag0 = tag;
    tag += (uint32_t)Kc + 1u;
    A.x0 = x0;
    A.code = h->code;
    A.rowfl = h->rowfl;
    A.colfl = h->colfl;
    A.edge = edge;
    A.ticket = counters;
    A.done = counters + 1;
    A.err = h->err;
    A.spin_limit = h->spin_limit;
    A.S = S;
    A.P = h->P;
    A.K = Kc;
    A.B = strips_for(S, Kc);
    A.a = a;
    A.c_recip = c_recip;
    const unsigned ntasks = (unsigned)(A.B * Kc);
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    if (h->profiling) {
      EQ_CUDA(cudaEventCreate(&ev0));
      EQ_CUDA(cudaEventCreate(&ev1));
      EQ_CUDA(cudaEventRecord(ev0, h->cur));
    }
    switch (mode) {
      case eqk::kRow:
        eqk::k_lin_solve<eqk::kRow><<<ntasks, 32, 0, h->cur>>>(A);
        break;
      case eqk::kCol:
        eqk::k_lin_solve<eqk::kCol><<<ntasks, 32, 0, h->cur>>>(A);
        break;
      default:
        eqk::k_lin_solve<eqk::kPassive><<<ntasks, 32, 0, h->cur>>>(A);
        break;
    }
    int rc = check_launch(h);
    if (rc) return rc;
    if (h->profiling) {
      EQ_CUDA(cudaEventRecord(ev1, h->cur));
      h->ls_events.emplace_back(ev0, ev1);
    }
  }
  return EQ_OK;
}

// diffuse (fluid.rs:276-298).
int launch_diffuse(eq_fluid* h, int mode, float* x, const float* x0, float diffusion) {
  const float sf = (float)(h->S - 2);
  const float a = ((h->dt * diffusion) * sf) * sf;
  const float c = 1.0f + 4.0f * a;
  return launch_lin_solve(h, mode, x, x0, a, c);
}

// project (fluid.rs:330-375).
int launch_project(eq_fluid* h, float* vx, float* vy, float* p, float* div) {
  const int S = (int)h->S, N = S - 2;
  const dim3 blk(32, 8);
  const dim3 grd = grid2d(N, N, blk);
  eqk::k_divergence<<<grd, blk, 0, h->cur>>>(vx, vy, p, div, S, h->P);
  int rc = check_launch(h);
  if (rc) return rc;
  if ((rc = launch_bnd(h, eqk::kPassive, div))) return rc;
  if ((rc = launch_bnd(h, eqk::kPassive, p))) return rc;
  if ((rc = launch_lin_solve(h, eqk::kPassive, p, div, 1.0f, 4.0f))) return rc;
  eqk::k_gradient<<<grd, blk, 0, h->cur>>>(vx, vy, p, S, h->P);
  if ((rc = check_launch(h))) return rc;
  if ((rc = launch_bnd(h, eqk::kRow, vx))) return rc;
  return launch_bnd(h, eqk::kCol, vy);
}

// advect (fluid.rs:378-432).
int launch_advect(eq_fluid* h, int mode, float* d, const float* d0, const float* u,
                  const float* v) {
  const int S = (int)h->S, N = S - 2;
  const float dt0 = h->dt * (float)(h->S - 2);
  const int threads = std::min(256, ((N + 31) / 32) * 32);
  eqk::k_advect_rows<<<N, threads, 0, h->cur>>>(d, d0, u, v, S, h->P, dt0);
  int rc = check_launch(h);
  if (rc) return rc;
  return launch_bnd(h, mode, d);
}

int launch_copy(eq_fluid* h, float* dst, const float* src) {
  const size_t n4 = h->grid_elems() / 4;
  const int threads = 256;
  const int blocks = (int)std::min<size_t>((n4 + threads - 1) / threads, 152 * 16);
  eqk::k_copy<<<blocks, threads, 0, h->cur>>>(dst, src, n4);
  return check_launch(h);
}

// step (fluid.rs:437-524), with the reference's aliasing of the six arrays.
// One frame (fluid.rs:437-524). With a tape, the fields each advect reads are
// saved into it on the way (vx0, vy0 after the first project, vx, vy after
// the second, scratch after the density diffusion: 5 pitched grids).
int launch_step(eq_fluid* h, float* tape = nullptr) {
  int rc = upload_mask(h);
  if (rc) return rc;
  float* sc = h->field[EQ_FIELD_SCRATCH];
  float* de = h->field[EQ_FIELD_DENSITY];
  float* vx = h->field[EQ_FIELD_VX];
  float* vy = h->field[EQ_FIELD_VY];
  float* vx0 = h->field[EQ_FIELD_VX0];
  float* vy0 = h->field[EQ_FIELD_VY0];
  const size_t G = h->grid_elems(), GB = G * sizeof(float);
  auto save = [&](int slot, const float* f) -> int {
    if (tape)
      EQ_CUDA(cudaMemcpyAsync(tape + (size_t)slot * G, f, GB, cudaMemcpyDeviceToDevice,
                              h->stream));
    return EQ_OK;
  };
  if (!h->concurrent) {
    if ((rc = launch_diffuse(h, eqk::kRow, vx0, vx, h->visc))) return rc;
    if ((rc = launch_diffuse(h, eqk::kCol, vy0, vy, h->visc))) return rc;
    if ((rc = launch_project(h, vx0, vy0, vx, vy))) return rc;
    if ((rc = save(0, vx0)) || (rc = save(1, vy0))) return rc;
    if ((rc = launch_advect(h, eqk::kRow, vx, vx0, vx0, vy0))) return rc;
    if ((rc = launch_advect(h, eqk::kCol, vy, vy0, vx0, vy0))) return rc;
    if ((rc = launch_project(h, vx, vy, vx0, vy0))) return rc;
    if ((rc = save(2, vx)) || (rc = save(3, vy))) return rc;
    if ((rc = launch_diffuse(h, eqk::kPassive, sc, de, h->diff))) return rc;
    if ((rc = save(4, sc))) return rc;
    if ((rc = launch_advect(h, eqk::kPassive, de, sc, vx, vy))) return rc;
    return launch_copy(h, sc, de);
  }
  // The same phases with the independent ones side by side (every solve is
  // latency-bound and leaves most of the GPU idle): diffuse(vy0 <- vy) and
  // diffuse(scratch <- density) touch nothing the vx diffusion or the
  // velocity pipeline reads or writes until their joins, so the results are
  // those of the sequence above, bit for bit.
  const bool sideVy = (h->concurrent & EQ_CONC_VY) != 0;
  const bool sideDe = (h->concurrent & EQ_CONC_DENSITY) != 0;
  EQ_CUDA(cudaEventRecord(h->fork_ev, h->stream));
  auto on = [&](cudaStream_t st, int slot) {
    h->cur = st;
    h->cur_slot = slot;
  };
  // the critical path's solve first, then the side solves
  h->sw_pair = sideVy;
  rc = launch_diffuse(h, eqk::kRow, vx0, vx, h->visc);
  h->sw_pair = false;
  if (rc) return rc;
  if (sideVy) {
    EQ_CUDA(cudaStreamWaitEvent(h->side[0], h->fork_ev, 0));
    on(h->side[0], 1);
    rc = launch_diffuse(h, eqk::kCol, vy0, vy, h->visc);
    if (!rc && cudaEventRecord(h->join_ev[0], h->side[0]) != cudaSuccess) rc = EQ_ERR_CUDA;
    on(h->stream, 0);
    if (rc) return rc == EQ_ERR_CUDA ? fail(EQ_ERR_CUDA, "side stream event") : rc;
  }
  if (sideDe) {
    EQ_CUDA(cudaStreamWaitEvent(h->side[1], h->fork_ev, 0));
    on(h->side[1], 2);
    rc = launch_diffuse(h, eqk::kPassive, sc, de, h->diff);
    if (!rc && cudaEventRecord(h->join_ev[1], h->side[1]) != cudaSuccess) rc = EQ_ERR_CUDA;
    on(h->stream, 0);
    if (rc) return rc == EQ_ERR_CUDA ? fail(EQ_ERR_CUDA, "side stream event") : rc;
  }
  if (sideVy)
    EQ_CUDA(cudaStreamWaitEvent(h->stream, h->join_ev[0], 0));
  else if ((rc = launch_diffuse(h, eqk::kCol, vy0, vy, h->visc)))
    return rc;
  if ((rc = launch_project(h, vx0, vy0, vx, vy))) return rc;
  if ((rc = save(0, vx0)) || (rc = save(1, vy0))) return rc;
  if ((rc = launch_advect(h, eqk::kRow, vx, vx0, vx0, vy0))) return rc;
  if ((rc = launch_advect(h, eqk::kCol, vy, vy0, vx0, vy0))) return rc;
  if ((rc = launch_project(h, vx, vy, vx0, vy0))) return rc;
  if ((rc = save(2, vx)) || (rc = save(3, vy))) return rc;
  if (sideDe)
    EQ_CUDA(cudaStreamWaitEvent(h->stream, h->join_ev[1], 0));
  else if ((rc = launch_diffuse(h, eqk::kPassive, sc, de, h->diff)))
    return rc;
  if ((rc = save(4, sc))) return rc;
  if ((rc = launch_advect(h, eqk::kPassive, de, sc, vx, vy))) return rc;
  return launch_copy(h, sc, de);
}

int ensure_src_capacity(eq_fluid* h, size_t bytes) {
  if (bytes <= h->d_src_cap && bytes <= h->h_src_cap) return EQ_OK;
  size_t cap = std::max<size_t>(bytes, 4096);
  if (h->src_ev) EQ_CUDA(cudaEventSynchronize(h->src_ev));
  if (h->d_src) cudaFree(h->d_src);
  if (h->h_src) cudaFreeHost(h->h_src);
  h->d_src = nullptr;
  h->h_src = nullptr;
  h->d_src_cap = h->h_src_cap = 0;
  if (cudaMalloc(&h->d_src, cap) != cudaSuccess) return fail(EQ_ERR_OOM, "cudaMalloc (sources)");
  if (cudaMallocHost(&h->h_src, cap) != cudaSuccess)
    return fail(EQ_ERR_OOM, "cudaMallocHost (sources)");
  h->d_src_cap = h->h_src_cap = cap;
  return EQ_OK;
}

void free_handle(eq_fluid* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (int k = 0; k < 2; ++k)
    if (h->side[k]) cudaStreamSynchronize(h->side[k]);
  for (auto& e : h->ls_events) {
    cudaEventDestroy(e.first);
    cudaEventDestroy(e.second);
  }
  if (h->gexec) cudaGraphExecDestroy(h->gexec);
  if (h->graph) cudaGraphDestroy(h->graph);
  cudaFree(h->noise_counter);
  cudaFree(h->rgba);
  cudaFree(h->block);
  cudaFree(h->cells);
  cudaFree(h->code);
  cudaFree(h->cs_strip);
  cudaFree(h->rowfl);
  cudaFree(h->colfl);
  cudaFree(h->edge);
  cudaFree(h->wt);
  cudaFree(h->counters);
  for (int k = 0; k < 2; ++k) {
    cudaFree(h->xedge[k]);
    cudaFree(h->xwt[k]);
    cudaFree(h->xcounters[k]);
    if (h->side[k]) cudaStreamDestroy(h->side[k]);
    if (h->join_ev[k]) cudaEventDestroy(h->join_ev[k]);
  }
  if (h->fork_ev) cudaEventDestroy(h->fork_ev);
  for (int k = 0; k < 3; ++k) {
    cudaFree(h->sw_edge[k]);
    cudaFree(h->sw_gexp[k]);
    cudaFree(h->sw_ctr[k]);
  }
  cudaFree(h->err);
  cudaFree(h->d_pack);
  for (int k = 0; k < 2; ++k) {
    cudaFree(h->d_apack[k]);
    if (h->apack_ev[k]) cudaEventDestroy(h->apack_ev[k]);
    if (h->acopy_ev[k]) cudaEventDestroy(h->acopy_ev[k]);
  }
  if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
  cudaFree(h->d_src);
  if (h->h_src) cudaFreeHost(h->h_src);
  if (h->src_ev) cudaEventDestroy(h->src_ev);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

int alloc_handle(uint32_t size, int device, eq_fluid** out) {
  if (device < 0) {
    EQ_CUDA(cudaGetDevice(&device));
  }
  EQ_CUDA(cudaSetDevice(device));
  eq_fluid* h = new eq_fluid();
  h->device = device;
  h->S = size;
  h->P = (int)(((size + 31u) / 32u) * 32u);
  auto bail = [&](int code, const char* what) {
    free_handle(h);
    return fail(code, what);
  };
  // Stream priorities: the main stream and the vy side stream carry the
  // step's critical path (both feed the first project); the density side
  // stream is only joined before the last advect, so its blocks are
  // dispatched after theirs.
  int prio_low = 0, prio_high = 0;
  if (cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high) != cudaSuccess) {
    cudaGetLastError();
    prio_low = prio_high = 0;
  }
  if (cudaStreamCreateWithPriority(&h->stream, cudaStreamNonBlocking, prio_high) != cudaSuccess)
    return bail(EQ_ERR_CUDA, "cudaStreamCreate");
  if (cudaEventCreateWithFlags(&h->src_ev, cudaEventDisableTiming) != cudaSuccess)
    return bail(EQ_ERR_CUDA, "cudaEventCreate");
  const size_t g = h->grid_elems();
  if (cudaMalloc(&h->block, 6 * g * sizeof(float)) != cudaSuccess)
    return bail(EQ_ERR_OOM, "cudaMalloc (grids)");
  for (int f = 0; f < 6; ++f) h->field[f] = h->block + f * g;
  if (cudaMalloc(&h->cells, g) != cudaSuccess || cudaMalloc(&h->code, g) != cudaSuccess ||
      cudaMalloc(&h->rowfl, size) != cudaSuccess || cudaMalloc(&h->colfl, size) != cudaSuccess)
    return bail(EQ_ERR_OOM, "cudaMalloc (mask)");
  {
    // strips of the cluster wavefront: 16-64 positions per block, at most 16
    // blocks; grids from N = 128 may need the streamed form (lscs.cuh)
    const int N = (int)size - 2;
    const int C = std::min(16, (N + 31) / 32), J = C > 0 ? (N + C - 1) / C : 0;
    if (N >= 128 && C >= 2 && J >= 16 && J <= 64 && (C - 1) * J < N) {
      h->cs_C = C;
      h->cs_J = J;
      if (cudaMalloc(&h->cs_strip, 3 * eqk::ls_cs_strip_bytes((int)size, C, J)) != cudaSuccess)
        return bail(EQ_ERR_OOM, "cudaMalloc (cluster strip codes)");
    }
  }
  h->B = strips_for((int)size, kMaxSweepsPerLaunch);
  const size_t ntasks = (size_t)h->B * kMaxSweepsPerLaunch;
  if (cudaMalloc(&h->edge, ntasks * h->P * 8) != cudaSuccess ||
      cudaMalloc(&h->wt, 2 * g * 8) != cudaSuccess ||
      cudaMalloc(&h->counters, 2 * sizeof(unsigned)) != cudaSuccess ||
      cudaMalloc(&h->err, sizeof(int)) != cudaSuccess)
    return bail(EQ_ERR_OOM, "cudaMalloc (wavefront state)");
  if (cudaMemsetAsync(h->block, 0, 6 * g * sizeof(float), h->stream) != cudaSuccess ||
      cudaMemsetAsync(h->wt, 0, 2 * g * 8, h->stream) != cudaSuccess ||
      cudaMemsetAsync(h->edge, 0, ntasks * h->P * 8, h->stream) != cudaSuccess ||
      cudaMemsetAsync(h->counters, 0, 2 * sizeof(unsigned), h->stream) != cudaSuccess ||
      cudaMemsetAsync(h->err, 0, sizeof(int), h->stream) != cudaSuccess)
    return bail(EQ_ERR_CUDA, "cudaMemsetAsync");
  h->cur = h->stream;
  if (cudaEventCreateWithFlags(&h->fork_ev, cudaEventDisableTiming) != cudaSuccess)
    return bail(EQ_ERR_CUDA, "cudaEventCreate");
  for (int k = 0; k < 2; ++k) {
    if (cudaStreamCreateWithPriority(&h->side[k], cudaStreamNonBlocking,
                                     k == 0 ? prio_high : prio_low) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->join_ev[k], cudaEventDisableTiming) != cudaSuccess)
      return bail(EQ_ERR_CUDA, "cudaStreamCreate (side streams)");
    if (cudaMalloc(&h->xedge[k], ntasks * h->P * 8) != cudaSuccess ||
        cudaMalloc(&h->xwt[k], 2 * g * 8) != cudaSuccess ||
        cudaMalloc(&h->xcounters[k], 2 * sizeof(unsigned)) != cudaSuccess)
      return bail(EQ_ERR_OOM, "cudaMalloc (side wavefront state)");
    if (cudaMemsetAsync(h->xwt[k], 0, 2 * g * 8, h->stream) != cudaSuccess ||
        cudaMemsetAsync(h->xedge[k], 0, ntasks * h->P * 8, h->stream) != cudaSuccess ||
        cudaMemsetAsync(h->xcounters[k], 0, 2 * sizeof(unsigned), h->stream) != cudaSuccess)
      return bail(EQ_ERR_CUDA, "cudaMemsetAsync");
  }
  {
    // strip wavefront exports for the longest launch (kSwMaxK sweeps), per slot
    const int Bs = eqk::ls_sw_strips((int)size, eqk::kSwMaxK);
    const size_t words =
        (size_t)std::max(Bs - 1, 1) * eqk::kSwMaxK * eqk::ls_sw_records((int)size) * 4;
    const size_t gwords = (size_t)Bs * (kSwMaxGroups - 1) *
                          (eqk::ls_sw_records((int)size) + 1) * eqk::kSwGrpWords;
    for (int k = 0; k < 3; ++k) {
      if (cudaMalloc(&h->sw_edge[k], words * 8) != cudaSuccess ||
          cudaMalloc(&h->sw_gexp[k], gwords * 8) != cudaSuccess ||
          cudaMalloc(&h->sw_ctr[k], 4 * sizeof(unsigned)) != cudaSuccess)
        return bail(EQ_ERR_OOM, "cudaMalloc (strip wavefront state)");
      if (cudaMemsetAsync(h->sw_edge[k], 0, words * 8, h->stream) != cudaSuccess ||
          cudaMemsetAsync(h->sw_gexp[k], 0, gwords * 8, h->stream) != cudaSuccess ||
          cudaMemsetAsync(h->sw_ctr[k], 0, 4 * sizeof(unsigned), h->stream) != cudaSuccess)
        return bail(EQ_ERR_CUDA, "cudaMemsetAsync");
    }
  }
  h->host_cells.assign((size_t)size * size, 0);
  *out = h;
  return EQ_OK;
}

// init() (fluid.rs:602-606) applied to the current state: computed on the
// host (it is O(size^2) set-up, not the hot path) and written back.
int apply_init(eq_fluid* h) {
  const uint32_t S = h->S;
  const size_t n = (size_t)S * S;
  std::vector<float> f[6];
  for (int q = 0; q < 6; ++q) {
    f[q].resize(n);
    int rc = eq_fluid_read_field(h, q, f[q].data(), n);
    if (rc) return rc;
  }
  auto idx = [&](int64_t x, int64_t y) {
    const int64_t s = S;
    x = x < 0 ? 0 : (x > s - 1 ? s - 1 : x);
    y = y < 0 ? 0 : (y > s - 1 ? s - 1 : y);
    return (size_t)(x + y * s);
  };
  for (uint32_t j = 0; j < S; ++j)
    for (uint32_t i = 0; i < S; ++i) {
      f[EQ_FIELD_VX][idx(i, j)] += 1.0f;
      f[EQ_FIELD_VY][idx(i, j)] += 1.0f;
    }
  for (uint32_t j = 0; j < S; ++j)
    for (uint32_t i = 0; i < S; ++i) {
      f[EQ_FIELD_DENSITY][idx(i, j)] += 0.0f;
      f[EQ_FIELD_SCRATCH][idx(i, j)] += 0.0f;
    }
  for (uint32_t j = S / 2 - 10; j <= S / 2 + 10; ++j)
    for (uint32_t i = S / 2 - 10; i <= S / 2 + 10; ++i) {
      f[EQ_FIELD_DENSITY][idx(i, j)] += 0.9f;
      f[EQ_FIELD_SCRATCH][idx(i, j)] += 0.9f;
    }
  for (uint32_t i = 0; i < S; ++i) {
    h->host_cells[idx(i, 0)] = 1;
    h->host_cells[idx(i, S - 1)] = 1;
  }
  for (uint32_t j = 0; j < S; ++j) {
    h->host_cells[idx(0, j)] = 1;
    h->host_cells[idx(S - 1, j)] = 1;
  }
  h->mask_dirty = true;
  for (int q = 0; q < 6; ++q) {
    int rc = eq_fluid_write_field(h, q, f[q].data(), n);
    if (rc) return rc;
  }
  EQ_CUDA(cudaStreamSynchronize(h->stream));
  return upload_mask(h);
}

int read_err_word(eq_fluid* h) {
  int e = 0;
  EQ_CUDA(cudaMemcpyAsync(&e, h->err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  EQ_CUDA(cudaStreamSynchronize(h->stream));
  if (e != 0) {
    // Leave the wavefront state clean for the next launch.
    EQ_CUDA(cudaMemsetAsync(h->counters, 0, 2 * sizeof(unsigned), h->stream));
    for (int k = 0; k < 2; ++k)
      EQ_CUDA(cudaMemsetAsync(h->xcounters[k], 0, 2 * sizeof(unsigned), h->stream));
    for (int k = 0; k < 3; ++k)
      EQ_CUDA(cudaMemsetAsync(h->sw_ctr[k], 0, 2 * sizeof(unsigned), h->stream));
    EQ_CUDA(cudaMemsetAsync(h->err, 0, sizeof(int), h->stream));
    EQ_CUDA(cudaStreamSynchronize(h->stream));
    if (e == EQ_ERR_TIMEOUT)
      return fail(EQ_ERR_TIMEOUT, "lin_solve: a bounded inter-block wait ran out");
    return fail(EQ_ERR_STATE, "device error word set");
  }
  return EQ_OK;
}

}  // namespace

extern "C" {

int eq_abi_version(void) { return EQ_ABI_VERSION; }

const char* eq_last_error(void) { return g_last_error.c_str(); }

int eq_fluid_new(const eq_fluid_configs* fluid, const eq_simulation_configs* sim, int device,
                 eq_fluid** out) {
  if (!fluid || !sim || !out) return fail(EQ_ERR_ARG, "null argument");
  *out = nullptr;
  if (sim->size < 20) return fail(EQ_ERR_ARG, "size must be >= 20 (fluid.rs:534 underflows)");
  if (sim->size > 65536) return fail(EQ_ERR_ARG, "size too large");
  if (sim->frames < 0) return fail(EQ_ERR_ARG, "frames must be >= 0");
  eq_fluid* h = nullptr;
  int rc = alloc_handle(sim->size, device, &h);
  if (rc) return rc;
  h->dt = sim->delta_t;
  h->frames = sim->frames;
  h->diff = fluid->diffusion;
  h->visc = fluid->viscousity;
  h->has_perlin_noise = fluid->has_perlin_noise;
  if ((rc = apply_init(h))) {
    free_handle(h);
    return rc;
  }
  *out = h;
  return EQ_OK;
}

int eq_fluid_default(int device, eq_fluid** out) {
  // configs.rs:14-22 and 50-60.
  eq_simulation_configs sim{0.02f, 16, 128};
  eq_fluid_configs fl{0.0f, 0.001f, 1};
  int rc = eq_fluid_new(&fl, &sim, device, out);
  if (rc) return rc;
  rc = apply_init(*out);  // Default calls init() a second time (fluid.rs:86)
  if (rc) {
    free_handle(*out);
    *out = nullptr;
  }
  return rc;
}

int eq_fluid_init(eq_fluid* h) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  int rc = select_device(h);
  if (rc) return rc;
  return apply_init(h);
}

int eq_fluid_clone(const eq_fluid* src, eq_fluid** out) {
  if (!src || !out) return fail(EQ_ERR_ARG, "null argument");
  *out = nullptr;
  eq_fluid* h = nullptr;
  int rc = alloc_handle(src->S, src->device, &h);
  if (rc) return rc;
  h->dt = src->dt;
  h->frames = src->frames;
  h->diff = src->diff;
  h->visc = src->visc;
  h->has_perlin_noise = src->has_perlin_noise;
  h->spin_limit = src->spin_limit;
  h->host_cells = src->host_cells;
  h->mask_dirty = true;
  // Order the copy after the source's pending work.
  cudaEvent_t ev;
  if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventRecord(ev, src->stream) != cudaSuccess ||
      cudaStreamWaitEvent(h->stream, ev, 0) != cudaSuccess) {
    free_handle(h);
    return fail(EQ_ERR_CUDA, "clone: event");
  }
  cudaEventDestroy(ev);
  if (cudaMemcpyAsync(h->block, src->block, 6 * h->grid_elems() * sizeof(float),
                      cudaMemcpyDeviceToDevice, h->stream) != cudaSuccess) {
    free_handle(h);
    return fail(EQ_ERR_CUDA, "clone: copy");
  }
  if ((rc = upload_mask(h))) {
    free_handle(h);
    return rc;
  }
  *out = h;
  return EQ_OK;
}

int eq_fluid_free(eq_fluid* h) {
  free_handle(h);
  return EQ_OK;
}

int eq_fluid_get_configs(const eq_fluid* h, eq_fluid_configs* fluid,
                         eq_simulation_configs* sim) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  if (fluid) {
    fluid->diffusion = h->diff;
    fluid->viscousity = h->visc;
    fluid->has_perlin_noise = h->has_perlin_noise;
  }
  if (sim) {
    sim->delta_t = h->dt;
    sim->frames = h->frames;
    sim->size = h->S;
  }
  return EQ_OK;
}

int eq_fluid_set_configs(eq_fluid* h, const eq_fluid_configs* fluid,
                         const eq_simulation_configs* sim) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  if (sim) {
    if (sim->size != h->S) return fail(EQ_ERR_ARG, "size cannot change");
    if (sim->frames < 0) return fail(EQ_ERR_ARG, "frames must be >= 0");
    h->dt = sim->delta_t;
    h->frames = sim->frames;
  }
  if (fluid) {
    h->diff = fluid->diffusion;
    h->visc = fluid->viscousity;
    h->has_perlin_noise = fluid->has_perlin_noise;
  }
  return EQ_OK;
}

int eq_fluid_step(eq_fluid* h) { return eq_fluid_step_n(h, 1); }

int eq_fluid_step_n(eq_fluid* h, int64_t nframes) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  if (nframes < 0) return fail(EQ_ERR_ARG, "nframes must be >= 0");
  int rc = select_device(h);
  if (rc) return rc;
  for (int64_t f = 0; f < nframes; ++f)
    if ((rc = launch_step(h))) return rc;
  return EQ_OK;
}

int eq_fluid_synchronize(eq_fluid* h) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  int rc = select_device(h);
  if (rc) return rc;
  EQ_CUDA(cudaStreamSynchronize(h->stream));
  for (int k = 0; k < 2; ++k)  // joined into the main stream by every step; an
    EQ_CUDA(cudaStreamSynchronize(h->side[k]));  // aborted step may have left work
  if (h->copy_stream) EQ_CUDA(cudaStreamSynchronize(h->copy_stream));  // async read-backs
  return read_err_word(h);
}

int eq_fluid_add_sources(eq_fluid* h, int64_t n, const uint32_t* x, const uint32_t* y,
                         const float* density, const float* vx, const float* vy) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  if (n < 0) return fail(EQ_ERR_ARG, "n must be >= 0");
  if (n == 0) return EQ_OK;
  if (!x || !y) return fail(EQ_ERR_ARG, "null coordinates");
  int rc = select_device(h);
  if (rc) return rc;
  const size_t bytes = (size_t)n * (2 * sizeof(uint32_t) + 3 * sizeof(float));
  if ((rc = ensure_src_capacity(h, bytes))) return rc;
  EQ_CUDA(cudaEventSynchronize(h->src_ev));  // previous upload has consumed the staging
  uint8_t* p = h->h_src;
  std::memcpy(p, x, n * sizeof(uint32_t));
  std::memcpy(p + n * 4, y, n * sizeof(uint32_t));
  float* fd = reinterpret_cast<float*>(p + n * 8);
  float* fu = fd + n;
  float* fv = fu + n;
  for (int64_t s = 0; s < n; ++s) {
    fd[s] = density ? density[s] : 0.0f;
    fu[s] = vx ? vx[s] : 0.0f;
    fv[s] = vy ? vy[s] : 0.0f;
  }
  EQ_CUDA(cudaMemcpyAsync(h->d_src, h->h_src, bytes, cudaMemcpyHostToDevice, h->stream));
  EQ_CUDA(cudaEventRecord(h->src_ev, h->stream));
  const uint32_t* dx = reinterpret_cast<const uint32_t*>(h->d_src);
  const uint32_t* dy = dx + n;
  const float* dd = reinterpret_cast<const float*>(h->d_src + n * 8);
  eqk::k_sources<<<1, 1, 0, h->stream>>>(
      h->field[EQ_FIELD_DENSITY], h->field[EQ_FIELD_SCRATCH], h->field[EQ_FIELD_VX],
      h->field[EQ_FIELD_VY], (int)h->S, h->P, n, dx, dy, density ? dd : nullptr,
      vx ? dd + n : nullptr, vy ? dd + 2 * n : nullptr);
  return check_launch(h);
}

int eq_fluid_add_density(eq_fluid* h, uint32_t x, uint32_t y, float amount) {
  return eq_fluid_add_sources(h, 1, &x, &y, &amount, nullptr, nullptr);
}

int eq_fluid_add_velocity(eq_fluid* h, uint32_t x, uint32_t y, float amount_x,
                          float amount_y) {
  return eq_fluid_add_sources(h, 1, &x, &y, nullptr, &amount_x, &amount_y);
}

int eq_fluid_run_device_sources(eq_fluid* h, int64_t nframes, int64_t nsrc,
                                const uint32_t* d_x, const uint32_t* d_y,
                                const float* d_density, const float* d_vx,
                                const float* d_vy) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  if (nframes < 0 || nsrc < 0) return fail(EQ_ERR_ARG, "negative count");
  if (nsrc > 0 && (!d_x || !d_y)) return fail(EQ_ERR_ARG, "null coordinates");
  int rc = select_device(h);
  if (rc) return rc;
  for (int64_t f = 0; f < nframes; ++f) {
    if (nsrc > 0) {
      const int64_t o = f * nsrc;
      eqk::k_sources<<<1, 1, 0, h->stream>>>(
          h->field[EQ_FIELD_DENSITY], h->field[EQ_FIELD_SCRATCH], h->field[EQ_FIELD_VX],
          h->field[EQ_FIELD_VY], (int)h->S, h->P, nsrc, d_x + o, d_y + o,
          d_density ? d_density + o : nullptr, d_vx ? d_vx + o : nullptr,
          d_vy ? d_vy + o : nullptr);
      if ((rc = check_launch(h))) return rc;
    }
    if ((rc = launch_step(h))) return rc;
  }
  return EQ_OK;
}

int eq_rectangle_check(int64_t dl_x, int64_t dl_y, int64_t ur_x, int64_t ur_y,
                       uint32_t size) {
  const int64_t s = size;
  const bool ok = dl_x != ur_x && dl_y != ur_y && dl_x < ur_x && dl_y < ur_y && dl_x < s &&
                  dl_y < s && ur_x < s && ur_y < s;
  return ok ? EQ_OK : fail(EQ_ERR_ARG, "Invalid input for Rectangle");
}

int eq_fluid_fill_obstacle(eq_fluid* h, int64_t x0, int64_t y0, int64_t x1, int64_t y1) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  const int64_t S = h->S;
  for (int64_t x = x0; x < x1; ++x)
    for (int64_t y = y0; y < y1; ++y) {
      const int64_t cx = x < 0 ? 0 : (x > S - 1 ? S - 1 : x);
      const int64_t cy = y < 0 ? 0 : (y > S - 1 ? S - 1 : y);
      h->host_cells[(size_t)(cx + cy * S)] = 1;
    }
  h->mask_dirty = true;
  return EQ_OK;
}

static int field_copy(eq_fluid* h, int field, void* host, uint64_t n, bool to_host,
                      bool sync) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  int rc = check_field(field);
  if (rc) return rc;
  if (n != (uint64_t)h->S * h->S) return fail(EQ_ERR_ARG, "element count must be size*size");
  if (!host) return fail(EQ_ERR_ARG, "null host buffer");
  if ((rc = select_device(h))) return rc;
  const size_t w = (size_t)h->S * sizeof(float);
  if (to_host)
    EQ_CUDA(cudaMemcpy2DAsync(host, w, h->field[field], (size_t)h->P * sizeof(float), w, h->S,
                              cudaMemcpyDeviceToHost, h->stream));
  else
    EQ_CUDA(cudaMemcpy2DAsync(h->field[field], (size_t)h->P * sizeof(float), host, w, w, h->S,
                              cudaMemcpyHostToDevice, h->stream));
  if (sync) EQ_CUDA(cudaStreamSynchronize(h->stream));
  return EQ_OK;
}

int eq_fluid_read_field(eq_fluid* h, int field, float* host, uint64_t n) {
  int rc = field_copy(h, field, host, n, true, true);
  if (rc) return rc;
  return read_err_word(h);
}
int eq_fluid_write_field(eq_fluid* h, int field, const float* host, uint64_t n) {
  return field_copy(h, field, const_cast<float*>(host), n, false, true);
}
int eq_fluid_read_field_async(eq_fluid* h, int field, float* host, uint64_t n) {
  return field_copy(h, field, host, n, true, false);
}

int eq_fluid_read_fields(eq_fluid* h, int count, const int* fields, float* const* host,
                         uint64_t n) {
  if (!h || !fields || !host) return fail(EQ_ERR_ARG, "null argument");
  if (count < 1 || count > 6) return fail(EQ_ERR_ARG, "count must be 1..6");
  const size_t g = (size_t)h->S * h->S;
  if (n != g) return fail(EQ_ERR_ARG, "element count must be size*size");
  int rc;
  for (int k = 0; k < count; ++k) {
    if ((rc = check_field(fields[k]))) return rc;
    if (!host[k]) return fail(EQ_ERR_ARG, "null host buffer");
  }
  if ((rc = select_device(h))) return rc;
  if (h->d_pack_cap < (size_t)count * g) {
    EQ_CUDA(cudaStreamSynchronize(h->stream));
    cudaFree(h->d_pack);
    h->d_pack = nullptr;
    h->d_pack_cap = 0;
    if (cudaMalloc(&h->d_pack, (size_t)count * g * sizeof(float)) != cudaSuccess)
      return fail(EQ_ERR_OOM, "cudaMalloc (read staging)");
    h->d_pack_cap = (size_t)count * g;
  }
  eqk::PackFields pf;
  pf.count = count;
  for (int k = 0; k < count; ++k) pf.src[k] = h->field[fields[k]];
  const int blocks = (int)std::min<size_t>((g * count + 255) / 256, 152 * 8);
  eqk::k_pack_fields<<<blocks, 256, 0, h->stream>>>(pf, h->d_pack, (int)h->S, h->P);
  if ((rc = check_launch(h))) return rc;
  for (int k = 0; k < count; ++k)
    EQ_CUDA(cudaMemcpyAsync(host[k], h->d_pack + (size_t)k * g, g * sizeof(float),
                            cudaMemcpyDeviceToHost, h->stream));
  return read_err_word(h);  // synchronises the stream
}
int eq_fluid_read_fields_async(eq_fluid* h, int count, const int* fields, float* const* host,
                               uint64_t n) {
  if (!h || !fields || !host) return fail(EQ_ERR_ARG, "null argument");
  if (count < 1 || count > 6) return fail(EQ_ERR_ARG, "count must be 1..6");
  const size_t g = (size_t)h->S * h->S;
  if (n != g) return fail(EQ_ERR_ARG, "element count must be size*size");
  int rc;
  for (int k = 0; k < count; ++k) {
    if ((rc = check_field(fields[k]))) return rc;
    if (!host[k]) return fail(EQ_ERR_ARG, "null host buffer");
  }
  if ((rc = select_device(h))) return rc;
  if (!h->copy_stream) {
    if (cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking) != cudaSuccess)
      return fail(EQ_ERR_CUDA, "cudaStreamCreate (read-back)");
    for (int k = 0; k < 2; ++k)
      if (cudaEventCreateWithFlags(&h->apack_ev[k], cudaEventDisableTiming) != cudaSuccess ||
          cudaEventCreateWithFlags(&h->acopy_ev[k], cudaEventDisableTiming) != cudaSuccess)
        return fail(EQ_ERR_CUDA, "cudaEventCreate (read-back)");
  }
  if (h->d_apack_cap < (size_t)count * g) {
    EQ_CUDA(cudaStreamSynchronize(h->stream));
    EQ_CUDA(cudaStreamSynchronize(h->copy_stream));
    for (int k = 0; k < 2; ++k) {
      cudaFree(h->d_apack[k]);
      h->d_apack[k] = nullptr;
    }
    h->d_apack_cap = 0;
    for (int k = 0; k < 2; ++k)
      if (cudaMalloc(&h->d_apack[k], (size_t)count * g * sizeof(float)) != cudaSuccess)
        return fail(EQ_ERR_OOM, "cudaMalloc (read-back staging)");
    h->d_apack_cap = (size_t)count * g;
    for (int k = 0; k < 2; ++k) EQ_CUDA(cudaEventRecord(h->acopy_ev[k], h->copy_stream));
  }
  const int slot = h->apack_next;
  h->apack_next ^= 1;
  // the packing reuses this buffer only after its previous copy is done
  EQ_CUDA(cudaStreamWaitEvent(h->stream, h->acopy_ev[slot], 0));
  eqk::PackFields pf;
  pf.count = count;
  for (int k = 0; k < count; ++k) pf.src[k] = h->field[fields[k]];
  const int blocks = (int)std::min<size_t>((g * count + 255) / 256, 152 * 8);
  eqk::k_pack_fields<<<blocks, 256, 0, h->stream>>>(pf, h->d_apack[slot], (int)h->S, h->P);
  if ((rc = check_launch(h))) return rc;
  EQ_CUDA(cudaEventRecord(h->apack_ev[slot], h->stream));
  EQ_CUDA(cudaStreamWaitEvent(h->copy_stream, h->apack_ev[slot], 0));
  for (int k = 0; k < count; ++k)
    EQ_CUDA(cudaMemcpyAsync(host[k], h->d_apack[slot] + (size_t)k * g, g * sizeof(float),
                            cudaMemcpyDeviceToHost, h->copy_stream));
  EQ_CUDA(cudaEventRecord(h->acopy_ev[slot], h->copy_stream));
  return EQ_OK;
}

int eq_fluid_write_field_async(eq_fluid* h, int field, const float* host, uint64_t n) {
  return field_copy(h, field, const_cast<float*>(host), n, false, false);
}

int eq_fluid_read_cells(eq_fluid* h, uint8_t* host, uint64_t n) {
  if (!h || !host) return fail(EQ_ERR_ARG, "null argument");
  if (n != (uint64_t)h->S * h->S) return fail(EQ_ERR_ARG, "element count must be size*size");
  std::memcpy(host, h->host_cells.data(), n);
  return EQ_OK;
}

int eq_fluid_write_cells(eq_fluid* h, const uint8_t* host, uint64_t n) {
  if (!h || !host) return fail(EQ_ERR_ARG, "null argument");
  const uint32_t S = h->S;
  if (n != (uint64_t)S * S) return fail(EQ_ERR_ARG, "element count must be size*size");
  for (uint32_t i = 0; i < S; ++i)
    if (!host[i] || !host[(size_t)(S - 1) * S + i] || !host[(size_t)i * S] ||
        !host[(size_t)i * S + S - 1])
      return fail(EQ_ERR_ARG, "the ghost frame must stay DefaultWall");
  for (uint64_t q = 0; q < n; ++q) h->host_cells[q] = host[q] ? 1 : 0;
  h->mask_dirty = true;
  return EQ_OK;
}

int eq_fluid_set_boundaries(eq_fluid* h, int mode, int field) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  int rc;
  if ((rc = check_mode(mode)) || (rc = check_field(field)) || (rc = select_device(h)) ||
      (rc = upload_mask(h)))
    return rc;
  return launch_bnd(h, mode, h->field[field]);
}

int eq_fluid_lin_solve(eq_fluid* h, int mode, int x_field, int x0_field, float a, float c) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  int rc;
  if ((rc = check_mode(mode)) || (rc = check_field(x_field)) || (rc = check_field(x0_field)))
    return rc;
  if (x_field == x0_field) return fail(EQ_ERR_ARG, "x and x0 must differ");
  if ((rc = select_device(h)) || (rc = upload_mask(h))) return rc;
  return launch_lin_solve(h, mode, h->field[x_field], h->field[x0_field], a, c);
}

int eq_fluid_diffuse(eq_fluid* h, int mode, int x_field, int x0_field, float diffusion) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  int rc;
  if ((rc = check_mode(mode)) || (rc = check_field(x_field)) || (rc = check_field(x0_field)))
    return rc;
  if (x_field == x0_field) return fail(EQ_ERR_ARG, "x and x0 must differ");
  if ((rc = select_device(h)) || (rc = upload_mask(h))) return rc;
  return launch_diffuse(h, mode, h->field[x_field], h->field[x0_field], diffusion);
}

int eq_fluid_project(eq_fluid* h, int vx_field, int vy_field, int p_field, int div_field) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  int rc;
  if ((rc = check_field(vx_field)) || (rc = check_field(vy_field)) ||
      (rc = check_field(p_field)) || (rc = check_field(div_field)))
    return rc;
  const int f[4] = {vx_field, vy_field, p_field, div_field};
  for (int a = 0; a < 4; ++a)
    for (int b = a + 1; b < 4; ++b)
      if (f[a] == f[b]) return fail(EQ_ERR_ARG, "project fields must be distinct");
  if ((rc = select_device(h)) || (rc = upload_mask(h))) return rc;
  return launch_project(h, h->field[vx_field], h->field[vy_field], h->field[p_field],
                        h->field[div_field]);
}

int eq_fluid_advect(eq_fluid* h, int mode, int d_field, int d0_field, int u_field,
                    int v_field) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  int rc;
  if ((rc = check_mode(mode)) || (rc = check_field(d_field)) || (rc = check_field(d0_field)) ||
      (rc = check_field(u_field)) || (rc = check_field(v_field)))
    return rc;
  if (d_field == d0_field || d_field == u_field || d_field == v_field)
    return fail(EQ_ERR_ARG, "advect destination must differ from its inputs");
  if ((rc = select_device(h)) || (rc = upload_mask(h))) return rc;
  return launch_advect(h, mode, h->field[d_field], h->field[d0_field], h->field[u_field],
                       h->field[v_field]);
}

int eq_fluid_device_field(eq_fluid* h, int field, float** dptr, uint32_t* pitch_elems) {
  if (!h || !dptr) return fail(EQ_ERR_ARG, "null argument");
  int rc = check_field(field);
  if (rc) return rc;
  *dptr = h->field[field];
  if (pitch_elems) *pitch_elems = (uint32_t)h->P;
  return EQ_OK;
}

int eq_fluid_launch_count(const eq_fluid* h, uint64_t* count) {
  if (!h || !count) return fail(EQ_ERR_ARG, "null argument");
  *count = h->launches;
  return EQ_OK;
}

int eq_fluid_get_stream(eq_fluid* h, void** stream) {
  if (!h || !stream) return fail(EQ_ERR_ARG, "null argument");
  *stream = (void*)h->stream;
  return EQ_OK;
}

int eq_fluid_set_profiling(eq_fluid* h, int enable) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  h->profiling = enable != 0;
  return EQ_OK;
}

int eq_fluid_kernel_stats(eq_fluid* h, int kernel, double* total_ms, uint64_t* launches) {
  if (!h || !total_ms || !launches) return fail(EQ_ERR_ARG, "null argument");
  if (kernel != 0) return fail(EQ_ERR_ARG, "unknown kernel id");
  int rc = select_device(h);
  if (rc) return rc;
  EQ_CUDA(cudaStreamSynchronize(h->stream));
  double sum = 0.0;
  for (auto& e : h->ls_events) {
    float ms = 0.f;
    EQ_CUDA(cudaEventElapsedTime(&ms, e.first, e.second));
    sum += ms;
    cudaEventDestroy(e.first);
    cudaEventDestroy(e.second);
  }
  *total_ms = sum;
  *launches = h->ls_events.size();
  h->ls_events.clear();
  return EQ_OK;
}

int eq_fluid_set_concurrency(eq_fluid* h, int mask) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  if (mask < 0 || mask > (EQ_CONC_VY | EQ_CONC_DENSITY))
    return fail(EQ_ERR_ARG, "concurrency mask must be in [0, 3]");
  h->concurrent = mask;
  return EQ_OK;
}

int eq_fluid_set_solver(eq_fluid* h, int solver) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  if (solver < 0 || solver > 4) return fail(EQ_ERR_ARG, "solver must be 0..4");
  h->solver = solver;
  return EQ_OK;
}

int eq_fluid_set_strip_groups(eq_fluid* h, int groups) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  if (groups < 0 || groups > kSwMaxGroups) return fail(EQ_ERR_ARG, "groups must be 0..5");
  h->sw_groups = groups;
  return EQ_OK;
}

int eq_fluid_set_strip_slack(eq_fluid* h, int periods) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  if (periods < 0 || periods > 64) return fail(EQ_ERR_ARG, "periods must be 0..64");
  h->sw_slack = periods;
  return EQ_OK;
}

int eq_fluid_set_cluster_interval(eq_fluid* h, int max_m) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  if (max_m < 0 || max_m > 3) return fail(EQ_ERR_ARG, "max_m must be in [0, 3]");
  h->cl_mmax = max_m;
  h->cl_K = -1;  // re-check
  return EQ_OK;
}

int eq_fluid_get_solver(eq_fluid* h, int* cluster_blocks_out) {
  if (!h || !cluster_blocks_out) return fail(EQ_ERR_ARG, "null argument");
  int rc = select_device(h);
  if (rc) return rc;
  *cluster_blocks_out = h->solver == 1 ? 0 : cluster_blocks(h, h->frames);
  return EQ_OK;
}

int eq_fluid_get_cluster_form(eq_fluid* h, int* form) {
  if (!h || !form) return fail(EQ_ERR_ARG, "null argument");
  int rc = select_device(h);
  if (rc) return rc;
  *form = (h->solver != 1 && cluster_blocks(h, h->frames) > 0) ? h->cl_kind : 0;
  return EQ_OK;
}

int eq_fluid_set_spin_limit(eq_fluid* h, int64_t iterations) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  if (iterations < 1) return fail(EQ_ERR_ARG, "spin limit must be >= 1");
  h->spin_limit = iterations;
  return EQ_OK;
}

}  // extern "C"

// The allocation-free lin_solve entry point and its static scratch, compiled
// in this translation unit (it shares the kernels above).
#include "noalloc.cu"

// The batched form (many scenes per launch).
#include "batch.cu"

// The precision form (half storage, refined pressure).
#include "half.cu"

// Around the step: image, noise, device obstacles, graph-captured frames.
#include "frame.cu"

// The differentiation form (recorded forward, adjoint kernels, backward).
#include "adjoint.cu"
