// lin_solve without any allocation, for callers that cannot allocate device
// memory: a solver embedded in a host application that owns all device memory
// through its own allocator or a fixed budget (a render engine, a framework
// with a caching allocator) and forbids its plugins to call cudaMalloc, and
// frame loops that must not take the device-wide synchronisation a
// cudaMalloc / cudaFree can cause (this entry point synchronises only the
// caller's stream). The caller passes its own device grids; every scratch
// buffer the wavefront needs lives in one file-scope static device array,
// sized for grids of at most kNaMaxSize x kNaMaxSize cells (about 3.2 MB,
// held by every GPU that loads this library until the process exits).
//
// Set-up: the first call on a device (with that device current) looks up the
// array's device address with cudaGetSymbolAddress and clears it; make that
// first call before any stream capture begins. Every call shares the array,
// which keeps the last call's contents, so calls that overlap on the GPU (two
// streams, two threads) race; callers serialise them.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/eqfluid.h"
#include "common.cuh"
#include "kernels.cuh"
#include "linsolve.cuh"

namespace {

constexpr int kNaMaxSize = 258;                       // cells per side incl. ghost frame
constexpr int kNaMaxPitch = 288;                      // row pitch limit (elements)
constexpr int kNaSweeps = 64;                         // sweeps per wavefront launch
constexpr int kNaMaxStrips = (kNaMaxSize + 2 * kNaSweeps + 31) / 32;
constexpr size_t kAlign = 256;
constexpr size_t align_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

constexpr size_t kOffWt = 0;
constexpr size_t kOffEdge =
    align_up(kOffWt + 2ull * kNaMaxPitch * kNaMaxSize * sizeof(unsigned long long));
constexpr size_t kOffCode = align_up(
    kOffEdge + (size_t)kNaMaxStrips * kNaSweeps * kNaMaxPitch * sizeof(unsigned long long));
constexpr size_t kOffRowfl = align_up(kOffCode + (size_t)kNaMaxPitch * kNaMaxSize);
constexpr size_t kOffColfl = align_up(kOffRowfl + kNaMaxSize);
constexpr size_t kOffCnt = align_up(kOffColfl + kNaMaxSize);
constexpr size_t kOffErr = kOffCnt + 2 * sizeof(unsigned);
constexpr size_t kNaBytes = align_up(kOffErr + sizeof(int));

// The scratch. In host code this name is only a stand-in for the symbol, not
// a device address: host code uses the address cudaGetSymbolAddress returns.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

constexpr int kMaxDevices = 64;
std::mutex g_na_mutex;
unsigned char* g_na_ptr[kMaxDevices] = {};
uint32_t g_na_tag[kMaxDevices] = {};

// Row / column "has a fluid cell" flags and the frame check (the frame must be
// walls, as init_walls leaves it); one thread per row or column.
__global__ void k_na_flags(const uint8_t* __restrict__ cells, int S, int P,
                           uint8_t* __restrict__ rowfl, uint8_t* __restrict__ colfl,
                           int* __restrict__ err) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2 * S) return;
  const int N = S - 2;
  const bool isRow = t < S;
  const int r = isRow ? t : t - S;
  uint8_t any = 0;
  bool frameOk = true;
  for (int q = 0; q < S; ++q) {
    const int i = isRow ? q : r, j = isRow ? r : q;
    const bool w = cells[(size_t)j * P + i] != 0;
    if (i == 0 || j == 0 || i == S - 1 || j == S - 1) frameOk &= w;
    if (!w && i >= 1 && i <= N && j >= 1 && j <= N) any = 1;
  }
  if (isRow)
    rowfl[r] = any;
  else
    colfl[r] = any;
  if (!frameOk) atomicExch(err, EQ_ERR_ARG);
}

// Per-cell boundary codes (the same derivation the handle path does on the host).
__global__ void k_na_codes(const uint8_t* __restrict__ cells, const uint8_t* __restrict__ colfl,
                           int S, int P, uint8_t* __restrict__ code) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= S || j >= S) return;
  const int N = S - 2;
  auto wall = [&](int x, int y) { return cells[(size_t)y * P + x] != 0; };
  const bool w = wall(i, j);
  uint8_t c = w ? eqk::kCodeWall : 0;
  if (!w && i >= 1 && i <= N && j >= 1 && j <= N) {
    if (wall(i + 1, j))
      c |= eqk::kCodeRowRight;
    else if (wall(i - 1, j))
      c |= eqk::kCodeRowLeft;
    if (wall(i, j - 1))
      c |= eqk::kCodeColUp;
    else if (wall(i, j + 1))
      c |= eqk::kCodeColDown;
  }
  if (j >= 2 && j - 1 <= N && i >= 1 && i <= N && w && !wall(i, j - 1) && !wall(i, j - 2))
    c |= eqk::kCodeAboveDown;
  if (colfl[i]) c |= eqk::kCodeColFluid;
  code[(size_t)j * P + i] = c;
}

}  // namespace

extern "C" int eq_lin_solve_noalloc(int mode, float* x, const float* x0, const uint8_t* cells,
                                    uint32_t size, uint32_t pitch, int64_t iters, float a,
                                    float c, void* stream_handle) {
  if (mode < 0 || mode > 2 || !x || !x0 || !cells) return EQ_ERR_ARG;
  if (size < 3 || size > (uint32_t)kNaMaxSize) return EQ_ERR_ARG;
  if (pitch < size || pitch > (uint32_t)kNaMaxPitch || (pitch % 4) != 0) return EQ_ERR_ARG;
  if (((uintptr_t)x | (uintptr_t)x0 | (uintptr_t)cells) & 15u) return EQ_ERR_ARG;
  if (x == x0 || iters < 0) return EQ_ERR_ARG;
  if (iters == 0) return EQ_OK;
  cudaStream_t stream = (cudaStream_t)stream_handle;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return EQ_ERR_CUDA;

  std::lock_guard<std::mutex> lock(g_na_mutex);
  if (!g_na_ptr[dev]) {  // once per device, with that device current
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return EQ_ERR_CUDA;
    if (cudaMemsetAsync(p, 0, kNaBytes, stream) != cudaSuccess) return EQ_ERR_CUDA;
    g_na_ptr[dev] = static_cast<unsigned char*>(p);
    g_na_tag[dev] = 1;
  }
  unsigned char* base = g_na_ptr[dev];
  unsigned long long* wt = reinterpret_cast<unsigned long long*>(base + kOffWt);
  unsigned long long* edge = reinterpret_cast<unsigned long long*>(base + kOffEdge);
  uint8_t* code = base + kOffCode;
  uint8_t* rowfl = base + kOffRowfl;
  uint8_t* colfl = base + kOffColfl;
  unsigned* cnt = reinterpret_cast<unsigned*>(base + kOffCnt);
  int* err = reinterpret_cast<int*>(base + kOffErr);
  const int S = (int)size, P = (int)pitch;
  const size_t g = (size_t)P * S;

  if (cudaMemsetAsync(err, 0, sizeof(int), stream) != cudaSuccess) return EQ_ERR_CUDA;
  k_na_flags<<<(2 * S + 127) / 128, 128, 0, stream>>>(cells, S, P, rowfl, colfl, err);
  k_na_codes<<<dim3((S + 127) / 128, S), 128, 0, stream>>>(cells, colfl, S, P, code);
  if (cudaGetLastError() != cudaSuccess) return EQ_ERR_CUDA;
  // The frame check's verdict before anything writes x: a mask whose frame is
  // not all walls returns EQ_ERR_ARG with x untouched.
  int herr = 0;  // the device error word, read into this stack variable
  if (cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
      cudaStreamSynchronize(stream) != cudaSuccess)
    return EQ_ERR_CUDA;
  if (herr != 0) return herr;

  const float c_recip = 1.0f / c;
  for (int64_t done = 0; done < iters; done += kNaSweeps) {
    const int Kc = (int)((iters - done) < kNaSweeps ? (iters - done) : kNaSweeps);
    if (g_na_tag[dev] > 0xF0000000u) {
      // tags would wrap: clear the whole tagged region (the grids and edge
      // rows of every size and pitch an earlier call used), not just this
      // call's part of it
      if (cudaMemsetAsync(base + kOffWt, 0, kOffCode - kOffWt, stream) != cudaSuccess)
        return EQ_ERR_CUDA;
      g_na_tag[dev] = 1;
    }
    if (cudaMemsetAsync(cnt, 0, 2 * sizeof(unsigned), stream) != cudaSuccess) return EQ_ERR_CUDA;
    eqk::k_ls_tag_init<<<(int)((g + 255) / 256), 256, 0, stream>>>(wt, x, g, g_na_tag[dev]);
    eqk::LinSolveArgs A;
    A.x = x;
    A.wt[0] = wt;
    A.wt[1] = wt + g;
    A.x0 = x0;
    A.code = code;
    A.rowfl = rowfl;
    A.colfl = colfl;
    A.edge = edge;
    A.ticket = cnt;
    A.done = cnt + 1;
    A.err = err;
    A.spin_limit = 1ll << 22;
    A.tag0 = g_na_tag[dev];
    A.S = S;
    A.P = P;
    A.K = Kc;
    A.B = (S + 2 * Kc + 31) / 32;
    A.a = a;
    A.c_recip = c_recip;
    g_na_tag[dev] += (uint32_t)Kc + 1u;
    const unsigned ntasks = (unsigned)(A.B * Kc);
    if (mode == eqk::kRow)
      eqk::k_lin_solve<eqk::kRow><<<ntasks, 32, 0, stream>>>(A);
    else if (mode == eqk::kCol)
      eqk::k_lin_solve<eqk::kCol><<<ntasks, 32, 0, stream>>>(A);
    else
      eqk::k_lin_solve<eqk::kPassive><<<ntasks, 32, 0, stream>>>(A);
    if (cudaGetLastError() != cudaSuccess) return EQ_ERR_CUDA;
  }
  if (cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
      cudaStreamSynchronize(stream) != cudaSuccess)
    return EQ_ERR_CUDA;
  return herr == 0 ? EQ_OK : herr;
}
