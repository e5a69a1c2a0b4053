// Host side of the batched form (include/eqfluid.h, "batches of scenes").
// Compiled in the same translation unit as eqfluid.cu (it shares the kernels,
// the error helpers and the boundary-code derivation).
//
// Device layout. All scenes' fields live in one f32 arena: scene s owns six
// grids in the anti-diagonal layout of wave.cuh (cell (i, j) at
// (i + j) * P + j, P = size rounded up to 32, 2 size - 1 diagonals; every grid
// starts on a 128-byte boundary) at consecutive offsets; the boundary codes
// (same layout), row and column "has a fluid cell" flags live in one byte
// arena. Host reads and writes convert to and from the dense layout. A scene table and a
// queue order (scenes sorted by decreasing size^2 x sweeps, largest first)
// feed the persistent frame kernel. One launch = one frame of every scene;
// eq_batch_step captures a whole sequence of frames (counter reset + one
// launch per frame) into a CUDA graph and replays it.
#include "batch.cuh"

struct eq_batch {
  int device = 0;
  int storage = 0;   // 0 FP32 (bit-exact), EQ_STORE_F16, EQ_STORE_BF16, EQ_STORE_F16_SCALARS
  size_t esize = 4;  // bytes per stored cell value (velocity fields)
  size_t esize2 = 4; // bytes per stored cell value of density and scratch
  cudaStream_t stream = nullptr;
  int64_t n = 0;
  std::vector<eqk::BScene> desc;
  std::vector<std::vector<uint8_t>> masks;  // dense size*size, 1 = DefaultWall
  struct Src {
    std::vector<uint32_t> x, y;
    std::vector<float> d, u, v;
  };
  std::vector<Src> src;
  bool mask_dirty = true, src_dirty = true;
  int smax = 0;

  void* arena = nullptr;
  void* arena2 = nullptr;  // density and scratch when stored apart (== arena otherwise)
  size_t arena_elems = 0;
  uint8_t* marena = nullptr;
  size_t marena_bytes = 0;
  eqk::BScene* d_desc = nullptr;
  int* d_order = nullptr;
  unsigned* d_queue = nullptr;
  int64_t queue_cap = 0;
  uint32_t* d_sx = nullptr;
  uint32_t* d_sy = nullptr;
  float* d_sval = nullptr;  // d, u, v (3 x total)
  int64_t src_cap = 0;

  // eq_batch_read_fields: every scene's dense field (device staging) and the
  // scenes' offsets in it, allocated on first use
  float* d_dense = nullptr;
  unsigned long long* d_doff = nullptr;
  uint64_t dense_total = 0;

  int nwmax = 20;  // sweeps per wavefront pass = warps per block
  int bps = 1;     // blocks per SM
  // the wavefront's per-block staging of packed x0 / codes (16 bytes a cell
  // of the largest scene's diagonal layout, 3 diagonals more), grown to the
  // launch's blocks
  void* d_stage = nullptr;
  size_t stage_stride = 0;
  int stage_blocks = 0;
  int num_sms = 0;
  size_t max_smem_block = 0, max_smem_sm = 0;

  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int64_t gframes = -1;
  int gnw = 0, gbps = 0;
  uint64_t launches = 0;
};

namespace {

void batch_drop_graph(eq_batch* b) {
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->gexec = nullptr;
  b->graph = nullptr;
  b->gframes = -1;
}

void batch_free(eq_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  batch_drop_graph(b);
  if (b->arena2 && b->arena2 != b->arena) cudaFree(b->arena2);
  cudaFree(b->arena);
  cudaFree(b->d_stage);
  cudaFree(b->d_dense);
  cudaFree(b->d_doff);
  cudaFree(b->marena);
  cudaFree(b->d_desc);
  cudaFree(b->d_order);
  cudaFree(b->d_queue);
  cudaFree(b->d_sx);
  cudaFree(b->d_sy);
  cudaFree(b->d_sval);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

// Fluid::new state (fluid.rs:93-110 then init(), fluid.rs:602-606) of every
// scene: zeros, vx = vy = 0 + 1, density = scratch = 0 + 0 (+ 0.9 on the
// block [size/2-10, size/2+10]^2). The arenas were zeroed before; density and
// scratch live in arena2 (== arena unless stored apart).
template <class ST, class STS>
__global__ void k_batch_init(ST* arena, STS* arena2, const eqk::BScene* scenes, int64_t n) {
  for (int64_t s = blockIdx.x; s < n; s += gridDim.x) {
    const eqk::BScene sc = scenes[s];
    const int S = sc.S, P = sc.P;
    const int lo = S / 2 - 10, hi = S / 2 + 10;
    ST* f = arena + sc.foff;
    STS* g = arena2 + sc.foff;
    const size_t cells = (size_t)S * S;
    // idx! clamps the block's coordinates into the grid (fluid.rs:31-35), so for
    // size 20 the last column / row receives the 0.9 twice (the corner 4x).
    auto mult = [&](int c) {
      int m = (c >= lo && c <= hi) ? 1 : 0;
      if (c == S - 1 && hi > S - 1) m += hi - (S - 1);
      return m;
    };
    for (size_t q = threadIdx.x; q < cells; q += blockDim.x) {
      const int j = (int)(q / S), i = (int)(q - (size_t)j * S);
      float dens = eqk::fadd(0.0f, 0.0f);
      for (int r = mult(i) * mult(j); r > 0; --r) dens = eqk::fadd(dens, 0.9f);
      const float vel = eqk::fadd(0.0f, 1.0f);
      const size_t a = eqk::dg_at(i, j, P);
      eqk::hs(g, a, dens);
      eqk::hs(g, sc.fstride + a, dens);
      eqk::hs(f, 2 * sc.fstride + a, vel);
      eqk::hs(f, 3 * sc.fstride + a, vel);
    }
  }
}

int batch_upload_masks(eq_batch* b) {
  if (!b->mask_dirty) return EQ_OK;
  std::vector<uint8_t> host(b->marena_bytes, 0), rowmajor;
  for (int64_t s = 0; s < b->n; ++s) {
    const eqk::BScene& sc = b->desc[s];
    const int S = sc.S, P = sc.P;
    uint8_t* code = host.data() + sc.moff;
    rowmajor.assign((size_t)P * S, 0);
    derive_codes(b->masks[s], S, P, rowmajor.data(), code + sc.fstride, code + sc.fstride + S);
    for (int j = 0; j < S; ++j)
      for (int i = 0; i < S; ++i) code[eqk::dg_at(i, j, P)] = rowmajor[(size_t)j * P + i];
  }
  EQ_CUDA(cudaMemcpyAsync(b->marena, host.data(), host.size(), cudaMemcpyHostToDevice,
                          b->stream));
  EQ_CUDA(cudaStreamSynchronize(b->stream));
  b->mask_dirty = false;
  return EQ_OK;
}

int batch_upload_sources(eq_batch* b) {
  if (!b->src_dirty) return EQ_OK;
  int64_t total = 0;
  for (int64_t s = 0; s < b->n; ++s) {
    b->desc[s].src_off = (int)total;
    b->desc[s].nsrc = (int)b->src[s].x.size();
    total += (int64_t)b->src[s].x.size();
  }
  if (total > b->src_cap) {
    EQ_CUDA(cudaStreamSynchronize(b->stream));
    cudaFree(b->d_sx);
    cudaFree(b->d_sy);
    cudaFree(b->d_sval);
    b->d_sx = b->d_sy = nullptr;
    b->d_sval = nullptr;
    b->src_cap = 0;
    if (cudaMalloc(&b->d_sx, total * 4) != cudaSuccess ||
        cudaMalloc(&b->d_sy, total * 4) != cudaSuccess ||
        cudaMalloc(&b->d_sval, total * 3 * sizeof(float)) != cudaSuccess)
      return fail(EQ_ERR_OOM, "cudaMalloc (batch sources)");
    b->src_cap = total;
  }
  if (total > 0) {
    std::vector<uint32_t> xs, ys;
    std::vector<float> vals(3 * b->src_cap);  // d | u | v, each src_cap long
    xs.reserve(total);
    ys.reserve(total);
    int64_t o = 0;
    for (int64_t s = 0; s < b->n; ++s) {
      const auto& S = b->src[s];
      for (size_t q = 0; q < S.x.size(); ++q, ++o) {
        xs.push_back(S.x[q]);
        ys.push_back(S.y[q]);
        vals[o] = S.d[q];
        vals[b->src_cap + o] = S.u[q];
        vals[2 * b->src_cap + o] = S.v[q];
      }
    }
    EQ_CUDA(cudaMemcpyAsync(b->d_sx, xs.data(), total * 4, cudaMemcpyHostToDevice, b->stream));
    EQ_CUDA(cudaMemcpyAsync(b->d_sy, ys.data(), total * 4, cudaMemcpyHostToDevice, b->stream));
    EQ_CUDA(cudaMemcpyAsync(b->d_sval, vals.data(), vals.size() * 4, cudaMemcpyHostToDevice,
                            b->stream));
  }
  EQ_CUDA(cudaMemcpyAsync(b->d_desc, b->desc.data(), b->n * sizeof(eqk::BScene),
                          cudaMemcpyHostToDevice, b->stream));
  EQ_CUDA(cudaStreamSynchronize(b->stream));
  b->src_dirty = false;
  batch_drop_graph(b);  // the graph's kernel arguments point at the old arrays
  return EQ_OK;
}

int batch_cs(const eq_batch* b) { return ((b->smax + 3) / 4) * 4; }

// Launch shape for the current tuning: blocks, threads and dynamic shared
// memory (the wavefront's ring, carry and edge rows).
struct BLaunch {
  int blocks, threads;
  size_t smem;
};

size_t batch_smem_budget(const eq_batch* b, int bps) {
  // per-block budget with bps blocks per SM (1 KB per block is reserved)
  return std::min(b->max_smem_block, b->max_smem_sm / (size_t)bps - 1024);
}

size_t batch_smem_bytes(const eq_batch* b, int nw) {
  return eqk::wave_smem_floats(nw, batch_cs(b)) * sizeof(float);
}

int batch_launch_shape(eq_batch* b, BLaunch* L) {
  L->threads = 32 * (b->nwmax + 1);  // + the wavefront's loader warp
  L->smem = batch_smem_bytes(b, b->nwmax);
  if (L->smem > batch_smem_budget(b, b->bps))
    return fail(EQ_ERR_ARG, "the wavefront buffers do not fit in shared memory at this tuning");
  L->blocks = (int)std::min<int64_t>(b->n, (int64_t)b->num_sms * b->bps);
  if (L->blocks < 1) L->blocks = 1;
  if (L->blocks > b->stage_blocks) {  // staging for every block of the launch
    size_t stride = 256;
    for (const eqk::BScene& d : b->desc)
      stride = std::max<size_t>(stride, ((d.fstride + 3 * (size_t)d.P) * 16 + 255) / 256 * 256);
    EQ_CUDA(cudaStreamSynchronize(b->stream));
    batch_drop_graph(b);  // the graph's kernel arguments point at the old staging
    cudaFree(b->d_stage);
    b->d_stage = nullptr;
    b->stage_blocks = 0;
    if (cudaMalloc(&b->d_stage, stride * (size_t)L->blocks) != cudaSuccess) {
      b->d_stage = nullptr;
      return fail(EQ_ERR_OOM, "cudaMalloc (wavefront staging)");
    }
    b->stage_stride = stride;
    b->stage_blocks = L->blocks;
  }
  EQ_CUDA(cudaFuncSetAttribute(eqk::k_batch_run<float>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L->smem));
  EQ_CUDA(cudaFuncSetAttribute(eqk::k_batch_run<__half>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L->smem));
  EQ_CUDA(cudaFuncSetAttribute(eqk::k_batch_run<__nv_bfloat16>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L->smem));
  EQ_CUDA(cudaFuncSetAttribute(eqk::k_batch_run<float, __half>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L->smem));
  return EQ_OK;
}

// The operation list of one frame: Fluid::step (fluid.rs:437-524) with the
// reference's aliasing (project's p and div are the other pair of velocity
// arrays), preceded by the scene's sources.
eqk::BOpList batch_frame_ops() {
  eqk::BOpList L;
  L.n = 0;
  auto add = [&](int kind, int mode, int f0, int f1, int f2, int f3, int coef, float a,
                 float c) {
    eqk::BOp& o = L.op[L.n++];
    o.kind = kind;
    o.mode = mode;
    o.f[0] = f0;
    o.f[1] = f1;
    o.f[2] = f2;
    o.f[3] = f3;
    o.coef = coef;
    o.a = a;
    o.c = c;
  };
  const int SC = EQ_FIELD_SCRATCH, DE = EQ_FIELD_DENSITY, VX = EQ_FIELD_VX, VY = EQ_FIELD_VY,
            VX0 = EQ_FIELD_VX0, VY0 = EQ_FIELD_VY0;
  add(eqk::kOpSources, 0, 0, 0, 0, 0, 0, 0.f, 0.f);
  add(eqk::kOpDiffuse, eqk::kRow, VX0, VX, 0, 0, 0, 0.f, 0.f);  // diffuse(1, vx0, vx, visc)
  add(eqk::kOpDiffuse, eqk::kCol, VY0, VY, 0, 0, 0, 0.f, 0.f);  // diffuse(2, vy0, vy, visc)
  add(eqk::kOpDivergence, 0, VX0, VY0, VX, VY, 0, 0.f, 0.f);   // project(vx0, vy0, vx, vy)
  add(eqk::kOpLinSolve, eqk::kPassive, VX, VY, 0, 0, 0, 1.0f, 4.0f);
  add(eqk::kOpGradient, 0, VX0, VY0, VX, 0, 0, 0.f, 0.f);
  add(eqk::kOpAdvectBreaks, 0, VX0, VY0, 0, 0, 0, 0.f, 0.f);     // u = vx0, v = vy0 (both)
  add(eqk::kOpAdvectWrite, eqk::kRow, VX, VX0, VX0, VY0, 0, 0.f, 0.f);
  add(eqk::kOpAdvectWrite, eqk::kCol, VY, VY0, VX0, VY0, 0, 0.f, 0.f);
  add(eqk::kOpDivergence, 0, VX, VY, VX0, VY0, 0, 0.f, 0.f);     // project(vx, vy, vx0, vy0)
  add(eqk::kOpLinSolve, eqk::kPassive, VX0, VY0, 0, 0, 0, 1.0f, 4.0f);
  add(eqk::kOpGradient, 0, VX, VY, VX0, 0, 0, 0.f, 0.f);
  add(eqk::kOpDiffuse, eqk::kPassive, SC, DE, 0, 0, 1, 0.f, 0.f);  // diffuse(0, s, d, diff)
  add(eqk::kOpAdvectBreaks, 0, VX, VY, 0, 0, 0, 0.f, 0.f);
  add(eqk::kOpAdvectWrite, eqk::kPassive, DE, SC, VX, VY, 0, 0.f, 0.f);
  add(eqk::kOpCopy, 0, SC, DE, 0, 0, 0, 0.f, 0.f);  // scratch = density.clone()
  return L;
}

eqk::BatchArgs batch_args(eq_batch* b, const BLaunch& L, unsigned* queue) {
  (void)L;
  eqk::BatchArgs A;
  A.arena = b->arena;
  A.arena2 = b->arena2;
  A.marena = b->marena;
  A.scenes = b->d_desc;
  A.order = b->d_order;
  A.nscenes = (int)b->n;
  A.queue = queue;
  A.src_x = b->d_sx;
  A.src_y = b->d_sy;
  A.src_d = b->d_sval;
  A.src_u = b->d_sval ? b->d_sval + b->src_cap : nullptr;
  A.src_v = b->d_sval ? b->d_sval + 2 * b->src_cap : nullptr;
  A.nwmax = b->nwmax;
  A.cs = batch_cs(b);
  A.stage = b->d_stage;
  A.stage_stride = b->stage_stride;
  return A;
}

int batch_prepare(eq_batch* b) {
  int rc;
  if ((rc = batch_upload_masks(b))) return rc;
  return batch_upload_sources(b);
}

int batch_ensure_queue(eq_batch* b, int64_t n) {
  if (n <= b->queue_cap) return EQ_OK;
  EQ_CUDA(cudaStreamSynchronize(b->stream));
  batch_drop_graph(b);
  cudaFree(b->d_queue);
  b->d_queue = nullptr;
  b->queue_cap = 0;
  const int64_t cap = std::max<int64_t>(n, 256);
  if (cudaMalloc(&b->d_queue, cap * sizeof(unsigned)) != cudaSuccess)
    return fail(EQ_ERR_OOM, "cudaMalloc (batch queue)");
  b->queue_cap = cap;
  return EQ_OK;
}

void batch_launch_run(eq_batch* b, const BLaunch& L, const eqk::BatchArgs& A,
                      const eqk::BOpList& ops) {
  if (b->storage == EQ_STORE_F16_SCALARS)
    eqk::k_batch_run<float, __half><<<L.blocks, L.threads, L.smem, b->stream>>>(A, ops);
  else if (b->storage == EQ_STORE_F16)
    eqk::k_batch_run<__half><<<L.blocks, L.threads, L.smem, b->stream>>>(A, ops);
  else if (b->storage == EQ_STORE_BF16)
    eqk::k_batch_run<__nv_bfloat16><<<L.blocks, L.threads, L.smem, b->stream>>>(A, ops);
  else
    eqk::k_batch_run<float><<<L.blocks, L.threads, L.smem, b->stream>>>(A, ops);
}

// Enqueue `nframes` frame launches (counter reset first) on the batch stream.
int batch_enqueue_frames(eq_batch* b, const BLaunch& L, int64_t nframes) {
  EQ_CUDA(cudaMemsetAsync(b->d_queue, 0, nframes * sizeof(unsigned), b->stream));
  const eqk::BOpList ops = batch_frame_ops();
  for (int64_t f = 0; f < nframes; ++f) {
    eqk::BatchArgs A = batch_args(b, L, b->d_queue + f);
    batch_launch_run(b, L, A, ops);
    EQ_CUDA(cudaGetLastError());
  }
  return EQ_OK;
}

// One launch of an operation list on every scene (the single-phase entries).
int batch_run_ops(eq_batch* b, const eqk::BOpList& ops) {
  int rc;
  if ((rc = batch_prepare(b)) || (rc = batch_ensure_queue(b, 1))) return rc;
  BLaunch L;
  if ((rc = batch_launch_shape(b, &L))) return rc;
  EQ_CUDA(cudaMemsetAsync(b->d_queue, 0, sizeof(unsigned), b->stream));
  const eqk::BatchArgs A = batch_args(b, L, b->d_queue);
  batch_launch_run(b, L, A, ops);
  b->launches++;
  EQ_CUDA(cudaGetLastError());
  return EQ_OK;
}

eqk::BOp batch_op(int kind, int mode, int f0, int f1, int f2, int f3, int coef, float a,
                  float c) {
  eqk::BOp o;
  o.kind = kind;
  o.mode = mode;
  o.f[0] = f0;
  o.f[1] = f1;
  o.f[2] = f2;
  o.f[3] = f3;
  o.coef = coef;
  o.a = a;
  o.c = c;
  return o;
}

int batch_check(eq_batch* b) {
  if (!b) return fail(EQ_ERR_ARG, "null batch");
  EQ_CUDA(cudaSetDevice(b->device));
  return EQ_OK;
}

int batch_scene(eq_batch* b, int64_t s) {
  return (s >= 0 && s < b->n) ? EQ_OK : fail(EQ_ERR_ARG, "scene index out of range");
}

}  // namespace

extern "C" {

int eq_batch_new(int64_t nscenes, const eq_scene_desc* scenes, int device, eq_batch** out) {
  return eq_batch_new_storage(nscenes, scenes, 0, device, out);
}

int eq_batch_new_storage(int64_t nscenes, const eq_scene_desc* scenes, int storage, int device,
                         eq_batch** out) {
  if (!out || !scenes) return fail(EQ_ERR_ARG, "null argument");
  if (storage != 0 && storage != EQ_STORE_F16 && storage != EQ_STORE_BF16 &&
      storage != EQ_STORE_F16_SCALARS)
    return fail(EQ_ERR_ARG,
                "storage must be 0 (FP32), EQ_STORE_F16, EQ_STORE_BF16 or EQ_STORE_F16_SCALARS");
  *out = nullptr;
  if (nscenes <= 0) return fail(EQ_ERR_ARG, "nscenes must be > 0");
  if (nscenes > (int64_t)1 << 30) return fail(EQ_ERR_ARG, "too many scenes");
  for (int64_t s = 0; s < nscenes; ++s) {
    if (scenes[s].size < 20) return fail(EQ_ERR_ARG, "size must be >= 20 (fluid.rs:534 underflows)");
    if (scenes[s].size > 16384) return fail(EQ_ERR_ARG, "batched scene size must be <= 16384");
    if (scenes[s].frames < 0 || scenes[s].frames > (int64_t)1 << 30)
      return fail(EQ_ERR_ARG, "frames out of range");
  }
  if (device < 0) EQ_CUDA(cudaGetDevice(&device));
  EQ_CUDA(cudaSetDevice(device));
  eq_batch* b = new eq_batch();
  b->device = device;
  b->n = nscenes;
  b->storage = storage;
  b->esize = (storage == 0 || storage == EQ_STORE_F16_SCALARS) ? 4 : 2;
  b->esize2 = storage == 0 ? 4 : 2;
  auto bail = [&](int code, const char* what) {
    batch_free(b);
    return fail(code, what);
  };
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess)
    return bail(EQ_ERR_CUDA, "cudaGetDeviceProperties");
  b->num_sms = prop.multiProcessorCount;
  b->max_smem_block = prop.sharedMemPerBlockOptin;
  b->max_smem_sm = prop.sharedMemPerMultiprocessor;
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(EQ_ERR_CUDA, "cudaStreamCreate");
  b->desc.resize(nscenes);
  b->masks.resize(nscenes);
  b->src.resize(nscenes);
  size_t foff = 0, moff = 0;
  for (int64_t s = 0; s < nscenes; ++s) {
    eqk::BScene& d = b->desc[s];
    const uint32_t S = scenes[s].size;
    d.S = (int)S;
    d.P = (int)(((S + 31u) / 32u) * 32u);
    d.K = (int)scenes[s].frames;
    d.dt = scenes[s].delta_t;
    d.diff = scenes[s].diffusion;
    d.visc = scenes[s].viscousity;
    d.nsrc = 0;
    d.src_off = 0;
    d.fstride = eqk::dg_size((int)S, d.P);
    d.foff = foff;
    foff += 6 * d.fstride;
    d.moff = moff;
    moff += (d.fstride + 2 * S + 127) / 128 * 128;
    b->smax = std::max(b->smax, (int)S);
    // init_walls (fluid.rs:552-570): the frame is DefaultWall
    std::vector<uint8_t>& m = b->masks[s];
    m.assign((size_t)S * S, 0);
    for (uint32_t i = 0; i < S; ++i) {
      m[i] = m[(size_t)(S - 1) * S + i] = 1;
      m[(size_t)i * S] = m[(size_t)i * S + S - 1] = 1;
    }
  }
  b->arena_elems = foff;
  b->marena_bytes = moff;
  if (cudaMalloc(&b->arena, foff * b->esize) != cudaSuccess)
    return bail(EQ_ERR_OOM, "cudaMalloc (batch fields)");
  if (cudaMemsetAsync(b->arena, 0, foff * b->esize, b->stream) != cudaSuccess)
    return bail(EQ_ERR_CUDA, "cudaMemsetAsync (batch fields)");
  b->arena2 = b->arena;
  if (storage == EQ_STORE_F16_SCALARS) {  // density and scratch apart, same offsets
    if (cudaMalloc(&b->arena2, foff * b->esize2) != cudaSuccess) {
      b->arena2 = nullptr;
      return bail(EQ_ERR_OOM, "cudaMalloc (batch scalar fields)");
    }
    if (cudaMemsetAsync(b->arena2, 0, foff * b->esize2, b->stream) != cudaSuccess)
      return bail(EQ_ERR_CUDA, "cudaMemsetAsync (batch scalar fields)");
  }
  if (cudaMalloc(&b->marena, moff) != cudaSuccess ||
      cudaMalloc(&b->d_desc, nscenes * sizeof(eqk::BScene)) != cudaSuccess ||
      cudaMalloc(&b->d_order, nscenes * sizeof(int)) != cudaSuccess)
    return bail(EQ_ERR_OOM, "cudaMalloc (batch tables)");
  // Largest work first (longest-processing-time order for the scene queue).
  std::vector<int> order(nscenes);
  for (int64_t s = 0; s < nscenes; ++s) order[s] = (int)s;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    const double wx = (double)b->desc[x].S * b->desc[x].S * (1.0 + b->desc[x].K);
    const double wy = (double)b->desc[y].S * b->desc[y].S * (1.0 + b->desc[y].K);
    return wx > wy;
  });
  if (cudaMemcpy(b->d_order, order.data(), nscenes * sizeof(int), cudaMemcpyHostToDevice) !=
          cudaSuccess ||
      cudaMemcpy(b->d_desc, b->desc.data(), nscenes * sizeof(eqk::BScene),
                 cudaMemcpyHostToDevice) != cudaSuccess)
    return bail(EQ_ERR_CUDA, "cudaMemcpy (batch tables)");
  int kmax = 1;
  for (int64_t s = 0; s < nscenes; ++s) kmax = std::max(kmax, b->desc[s].K);
  b->bps = 1;
  b->nwmax = std::min(kmax, 20);
  while (b->nwmax > 1 && batch_smem_bytes(b, b->nwmax) > batch_smem_budget(b, 1)) b->nwmax--;
  if (batch_smem_bytes(b, b->nwmax) > batch_smem_budget(b, 1))
    return bail(EQ_ERR_ARG, "the largest scene is too large for the block wavefront");
  {
    const int blocks = (int)std::min<int64_t>(nscenes, 4096);
    if (storage == EQ_STORE_F16)
      k_batch_init<<<blocks, 256, 0, b->stream>>>(static_cast<__half*>(b->arena), static_cast<__half*>(b->arena2), b->d_desc, nscenes);
    else if (storage == EQ_STORE_BF16)
      k_batch_init<<<blocks, 256, 0, b->stream>>>(static_cast<__nv_bfloat16*>(b->arena), static_cast<__nv_bfloat16*>(b->arena2), b->d_desc, nscenes);
    else if (storage == EQ_STORE_F16_SCALARS)
      k_batch_init<<<blocks, 256, 0, b->stream>>>(static_cast<float*>(b->arena), static_cast<__half*>(b->arena2), b->d_desc, nscenes);
    else
      k_batch_init<<<blocks, 256, 0, b->stream>>>(static_cast<float*>(b->arena), static_cast<float*>(b->arena2), b->d_desc, nscenes);
    if (cudaGetLastError() != cudaSuccess) return bail(EQ_ERR_CUDA, "k_batch_init");
    b->launches++;
  }
  if (cudaStreamSynchronize(b->stream) != cudaSuccess) return bail(EQ_ERR_CUDA, "init");
  *out = b;
  return EQ_OK;
}

int eq_batch_free(eq_batch* b) {
  batch_free(b);
  return EQ_OK;
}

int eq_batch_scene_count(const eq_batch* b, int64_t* n) {
  if (!b || !n) return fail(EQ_ERR_ARG, "null argument");
  *n = b->n;
  return EQ_OK;
}

int eq_batch_cell_count(const eq_batch* b, uint64_t* interior_cells) {
  if (!b || !interior_cells) return fail(EQ_ERR_ARG, "null argument");
  uint64_t c = 0;
  for (const auto& d : b->desc) c += (uint64_t)(d.S - 2) * (uint64_t)(d.S - 2);
  *interior_cells = c;
  return EQ_OK;
}

int eq_batch_fill_obstacle(eq_batch* b, int64_t scene, int64_t x0, int64_t y0, int64_t x1,
                           int64_t y1) {
  int rc;
  if ((rc = batch_check(b)) || (rc = batch_scene(b, scene))) return rc;
  const int64_t S = b->desc[scene].S;
  std::vector<uint8_t>& m = b->masks[scene];
  for (int64_t x = x0; x < x1; ++x)
    for (int64_t y = y0; y < y1; ++y) {
      const int64_t cx = x < 0 ? 0 : (x > S - 1 ? S - 1 : x);
      const int64_t cy = y < 0 ? 0 : (y > S - 1 ? S - 1 : y);
      m[(size_t)(cx + cy * S)] = 1;
    }
  b->mask_dirty = true;
  return EQ_OK;
}

int eq_batch_read_cells(eq_batch* b, int64_t scene, uint8_t* host, uint64_t n) {
  int rc;
  if ((rc = batch_check(b)) || (rc = batch_scene(b, scene))) return rc;
  if (!host) return fail(EQ_ERR_ARG, "null host buffer");
  if (n != b->masks[scene].size()) return fail(EQ_ERR_ARG, "element count must be size*size");
  std::memcpy(host, b->masks[scene].data(), n);
  return EQ_OK;
}

int eq_batch_set_sources(eq_batch* b, int64_t scene, int64_t n, const uint32_t* x,
                         const uint32_t* y, const float* density, const float* vx,
                         const float* vy) {
  int rc;
  if ((rc = batch_check(b)) || (rc = batch_scene(b, scene))) return rc;
  if (n < 0) return fail(EQ_ERR_ARG, "n must be >= 0");
  if (n > 0 && (!x || !y)) return fail(EQ_ERR_ARG, "null coordinates");
  auto& S = b->src[scene];
  S.x.assign(x, x + n);
  S.y.assign(y, y + n);
  S.d.assign(n, 0.0f);
  S.u.assign(n, 0.0f);
  S.v.assign(n, 0.0f);
  for (int64_t q = 0; q < n; ++q) {
    if (density) S.d[q] = density[q];
    if (vx) S.u[q] = vx[q];
    if (vy) S.v[q] = vy[q];
  }
  b->src_dirty = true;
  return EQ_OK;
}

static int batch_field_copy(eq_batch* b, int64_t scene, int field, void* host, uint64_t n,
                            bool to_host) {
  int rc;
  if ((rc = batch_check(b)) || (rc = batch_scene(b, scene)) || (rc = check_field(field)))
    return rc;
  const eqk::BScene& d = b->desc[scene];
  const int S = d.S, P = d.P;
  if (n != (uint64_t)S * S) return fail(EQ_ERR_ARG, "element count must be size*size");
  if (!host) return fail(EQ_ERR_ARG, "null host buffer");
  // density (1) and scratch (0) live in arena2 in their own format
  const bool scalar = field < 2;
  const size_t es = scalar ? b->esize2 : b->esize;
  const int fmt = es == 4 ? 0 : (b->storage == EQ_STORE_BF16 ? EQ_STORE_BF16 : EQ_STORE_F16);
  uint8_t* dev = static_cast<uint8_t*>(scalar ? b->arena2 : b->arena) +
                 (d.foff + (size_t)field * d.fstride) * es;
  std::vector<uint8_t> diag(d.fstride * es, 0);
  float* dense = static_cast<float*>(host);
  auto get = [&](size_t q) -> float {
    if (fmt == EQ_STORE_F16) return __half2float(reinterpret_cast<const __half*>(diag.data())[q]);
    if (fmt == EQ_STORE_BF16)
      return __bfloat162float(reinterpret_cast<const __nv_bfloat16*>(diag.data())[q]);
    return reinterpret_cast<const float*>(diag.data())[q];
  };
  auto put = [&](size_t q, float v) {
    if (fmt == EQ_STORE_F16)
      reinterpret_cast<__half*>(diag.data())[q] = __float2half_rn(v);
    else if (fmt == EQ_STORE_BF16)
      reinterpret_cast<__nv_bfloat16*>(diag.data())[q] = __float2bfloat16_rn(v);
    else
      reinterpret_cast<float*>(diag.data())[q] = v;
  };
  if (to_host) {
    EQ_CUDA(cudaMemcpyAsync(diag.data(), dev, diag.size(), cudaMemcpyDeviceToHost, b->stream));
    EQ_CUDA(cudaStreamSynchronize(b->stream));
    for (int j = 0; j < S; ++j)
      for (int i = 0; i < S; ++i) dense[(size_t)j * S + i] = get(eqk::dg_at(i, j, P));
  } else {
    for (int j = 0; j < S; ++j)
      for (int i = 0; i < S; ++i) put(eqk::dg_at(i, j, P), dense[(size_t)j * S + i]);
    EQ_CUDA(cudaMemcpyAsync(dev, diag.data(), diag.size(), cudaMemcpyHostToDevice, b->stream));
    EQ_CUDA(cudaStreamSynchronize(b->stream));
  }
  return EQ_OK;
}

int eq_batch_read_field(eq_batch* b, int64_t scene, int field, float* host, uint64_t n) {
  return batch_field_copy(b, scene, field, host, n, true);
}

int eq_batch_write_field(eq_batch* b, int64_t scene, int field, const float* host,
                         uint64_t n) {
  return batch_field_copy(b, scene, field, const_cast<float*>(host), n, false);
}

int eq_batch_read_fields(eq_batch* b, int field, float* host, uint64_t n) {
  int rc;
  if ((rc = batch_check(b)) || (rc = check_field(field))) return rc;
  if (!host) return fail(EQ_ERR_ARG, "null host buffer");
  if (!b->d_doff) {
    std::vector<unsigned long long> off(b->n);
    uint64_t t = 0;
    for (int64_t s = 0; s < b->n; ++s) {
      off[s] = t;
      t += (uint64_t)b->desc[s].S * b->desc[s].S;
    }
    if (cudaMalloc(&b->d_doff, b->n * sizeof(unsigned long long)) != cudaSuccess) {
      b->d_doff = nullptr;
      return fail(EQ_ERR_OOM, "cudaMalloc (dense offsets)");
    }
    if (cudaMalloc(&b->d_dense, t * sizeof(float)) != cudaSuccess) {
      cudaFree(b->d_doff);
      b->d_doff = nullptr;
      b->d_dense = nullptr;
      return fail(EQ_ERR_OOM, "cudaMalloc (dense staging)");
    }
    EQ_CUDA(cudaMemcpy(b->d_doff, off.data(), b->n * sizeof(unsigned long long),
                       cudaMemcpyHostToDevice));
    b->dense_total = t;
  }
  if (n != b->dense_total) return fail(EQ_ERR_ARG, "element count must be the sum of size*size");
  // density (1) and scratch (0) live in arena2 in their own format
  const bool scalar = field < 2;
  const void* arena = scalar ? b->arena2 : b->arena;
  const bool half = (scalar ? b->esize2 : b->esize) == 2;
  const unsigned blocks = (unsigned)b->n;
  if (!half)
    eqk::k_batch_gather_dense<<<blocks, 256, 0, b->stream>>>(
        static_cast<const float*>(arena), b->d_desc, b->d_doff, field, b->d_dense);
  else if (b->storage == EQ_STORE_BF16)
    eqk::k_batch_gather_dense<<<blocks, 256, 0, b->stream>>>(
        static_cast<const __nv_bfloat16*>(arena), b->d_desc, b->d_doff, field, b->d_dense);
  else
    eqk::k_batch_gather_dense<<<blocks, 256, 0, b->stream>>>(
        static_cast<const __half*>(arena), b->d_desc, b->d_doff, field, b->d_dense);
  EQ_CUDA(cudaGetLastError());
  b->launches++;
  EQ_CUDA(cudaMemcpyAsync(host, b->d_dense, n * sizeof(float), cudaMemcpyDeviceToHost, b->stream));
  EQ_CUDA(cudaStreamSynchronize(b->stream));
  return EQ_OK;
}

int eq_batch_set_tuning(eq_batch* b, int sweeps_per_pass, int blocks_per_sm) {
  int rc;
  if ((rc = batch_check(b))) return rc;
  if (sweeps_per_pass < 1 || sweeps_per_pass > 20)
    return fail(EQ_ERR_ARG, "sweeps_per_pass must be in [1, 20]");
  if (blocks_per_sm < 1 || blocks_per_sm > 4) return fail(EQ_ERR_ARG, "blocks_per_sm must be in [1, 4]");
  if ((sweeps_per_pass + 1) * 32 * blocks_per_sm > 1344)
    return fail(EQ_ERR_ARG, "more threads per SM than the kernel's register budget allows");
  const int onw = b->nwmax, obps = b->bps;
  b->nwmax = sweeps_per_pass;
  b->bps = blocks_per_sm;
  BLaunch L;
  if ((rc = batch_launch_shape(b, &L))) {
    b->nwmax = onw;
    b->bps = obps;
    return rc;
  }
  int active = 0;
  EQ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&active, eqk::k_batch_run<float>, L.threads,
                                                        L.smem));
  if (active < blocks_per_sm) {
    b->nwmax = onw;
    b->bps = obps;
    return fail(EQ_ERR_ARG, "that many blocks per SM do not fit (registers or shared memory)");
  }
  return EQ_OK;
}

int eq_batch_get_tuning(const eq_batch* b, int* sweeps_per_pass, int* blocks_per_sm) {
  if (!b) return fail(EQ_ERR_ARG, "null batch");
  if (sweeps_per_pass) *sweeps_per_pass = b->nwmax;
  if (blocks_per_sm) *blocks_per_sm = b->bps;
  return EQ_OK;
}

int eq_batch_step(eq_batch* b, int64_t nframes) {
  int rc;
  if ((rc = batch_check(b))) return rc;
  if (nframes < 0) return fail(EQ_ERR_ARG, "nframes must be >= 0");
  if (nframes == 0) return EQ_OK;
  if ((rc = batch_prepare(b)) || (rc = batch_ensure_queue(b, nframes))) return rc;
  BLaunch L;
  if ((rc = batch_launch_shape(b, &L))) return rc;
  if (!b->gexec || b->gframes != nframes || b->gnw != b->nwmax || b->gbps != b->bps) {
    batch_drop_graph(b);
    EQ_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    rc = batch_enqueue_frames(b, L, nframes);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return fail(EQ_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
    b->graph = g;
    EQ_CUDA(cudaGraphInstantiate(&b->gexec, b->graph, 0));
    b->gframes = nframes;
    b->gnw = b->nwmax;
    b->gbps = b->bps;
  }
  EQ_CUDA(cudaGraphLaunch(b->gexec, b->stream));
  b->launches += (uint64_t)nframes;  // one frame kernel per replayed frame
  return EQ_OK;
}

int eq_batch_step_eager(eq_batch* b, int64_t nframes) {
  int rc;
  if ((rc = batch_check(b))) return rc;
  if (nframes < 0) return fail(EQ_ERR_ARG, "nframes must be >= 0");
  if (nframes == 0) return EQ_OK;
  if ((rc = batch_prepare(b)) || (rc = batch_ensure_queue(b, nframes))) return rc;
  BLaunch L;
  if ((rc = batch_launch_shape(b, &L))) return rc;
  if ((rc = batch_enqueue_frames(b, L, nframes))) return rc;
  b->launches += (uint64_t)nframes;
  return EQ_OK;
}

int eq_batch_lin_solve(eq_batch* b, int mode, int x_field, int x0_field, float a, float c) {
  int rc;
  if ((rc = batch_check(b)) || (rc = check_mode(mode)) || (rc = check_field(x_field)) ||
      (rc = check_field(x0_field)))
    return rc;
  if (x_field == x0_field) return fail(EQ_ERR_ARG, "x and x0 must differ");
  eqk::BOpList L;
  L.n = 1;
  L.op[0] = batch_op(eqk::kOpLinSolve, mode, x_field, x0_field, 0, 0, 0, a, c);
  return batch_run_ops(b, L);
}

int eq_batch_diffuse(eq_batch* b, int mode, int x_field, int x0_field, float diffusion) {
  int rc;
  if ((rc = batch_check(b)) || (rc = check_mode(mode)) || (rc = check_field(x_field)) ||
      (rc = check_field(x0_field)))
    return rc;
  if (x_field == x0_field) return fail(EQ_ERR_ARG, "x and x0 must differ");
  eqk::BOpList L;
  L.n = 1;
  L.op[0] = batch_op(eqk::kOpDiffuse, mode, x_field, x0_field, 0, 0, 2, diffusion, 0.f);
  return batch_run_ops(b, L);
}

int eq_batch_project(eq_batch* b, int vx_field, int vy_field, int p_field, int div_field) {
  int rc;
  if ((rc = batch_check(b)) || (rc = check_field(vx_field)) || (rc = check_field(vy_field)) ||
      (rc = check_field(p_field)) || (rc = check_field(div_field)))
    return rc;
  const int f[4] = {vx_field, vy_field, p_field, div_field};
  for (int x = 0; x < 4; ++x)
    for (int y = x + 1; y < 4; ++y)
      if (f[x] == f[y]) return fail(EQ_ERR_ARG, "project fields must be distinct");
  eqk::BOpList L;
  L.n = 3;
  L.op[0] = batch_op(eqk::kOpDivergence, 0, vx_field, vy_field, p_field, div_field, 0, 0.f, 0.f);
  L.op[1] = batch_op(eqk::kOpLinSolve, eqk::kPassive, p_field, div_field, 0, 0, 0, 1.0f, 4.0f);
  L.op[2] = batch_op(eqk::kOpGradient, 0, vx_field, vy_field, p_field, 0, 0, 0.f, 0.f);
  return batch_run_ops(b, L);
}

int eq_batch_advect(eq_batch* b, int mode, int d_field, int d0_field, int u_field,
                    int v_field) {
  int rc;
  if ((rc = batch_check(b)) || (rc = check_mode(mode)) || (rc = check_field(d_field)) ||
      (rc = check_field(d0_field)) || (rc = check_field(u_field)) || (rc = check_field(v_field)))
    return rc;
  if (d_field == d0_field || d_field == u_field || d_field == v_field)
    return fail(EQ_ERR_ARG, "advect destination must differ from its inputs");
  eqk::BOpList L;
  L.n = 2;
  L.op[0] = batch_op(eqk::kOpAdvectBreaks, 0, u_field, v_field, 0, 0, 0, 0.f, 0.f);
  L.op[1] = batch_op(eqk::kOpAdvectWrite, mode, d_field, d0_field, u_field, v_field, 0, 0.f, 0.f);
  return batch_run_ops(b, L);
}

int eq_batch_set_boundaries(eq_batch* b, int mode, int field) {
  int rc;
  if ((rc = batch_check(b)) || (rc = check_mode(mode)) || (rc = check_field(field))) return rc;
  eqk::BOpList L;
  L.n = 1;
  L.op[0] = batch_op(eqk::kOpBnd, mode, field, 0, 0, 0, 0, 0.f, 0.f);
  return batch_run_ops(b, L);
}

int eq_batch_synchronize(eq_batch* b) {
  int rc;
  if ((rc = batch_check(b))) return rc;
  EQ_CUDA(cudaStreamSynchronize(b->stream));
  return EQ_OK;
}

int eq_batch_get_stream(eq_batch* b, void** stream) {
  if (!b || !stream) return fail(EQ_ERR_ARG, "null argument");
  *stream = (void*)b->stream;
  return EQ_OK;
}

int eq_batch_launch_count(const eq_batch* b, uint64_t* count) {
  if (!b || !count) return fail(EQ_ERR_ARG, "null argument");
  *count = b->launches;
  return EQ_OK;
}

// Autotuner: times `trial_frames` frames for each candidate (sweeps per pass,
// blocks per SM) from a snapshot of the state, restores the snapshot after
// every trial, and keeps the fastest. Writes the per-candidate times (ms per
// frame, 0 for a candidate that does not fit) to `ms_out` when given
// (capacity `cap`) and the candidate count to `ncand`.
int eq_batch_autotune(eq_batch* b, int trial_frames, double* ms_out, int cap, int* ncand) {
  int rc;
  if ((rc = batch_check(b))) return rc;
  if (trial_frames < 1) return fail(EQ_ERR_ARG, "trial_frames must be >= 1");
  if ((rc = batch_prepare(b)) || (rc = batch_ensure_queue(b, trial_frames))) return rc;
  int kmax = 1;
  for (const auto& d : b->desc) kmax = std::max(kmax, d.K);
  std::vector<std::pair<int, int>> cand;
  for (int nw : {20, 16, 10, 8, 5, 4}) {
    const int w = std::min(nw, kmax);
    for (int bps : {1, 2}) {
      if ((w + 1) * 32 * bps > 1344) continue;
      if (std::find(cand.begin(), cand.end(), std::make_pair(w, bps)) == cand.end())
        cand.emplace_back(w, bps);
    }
  }
  void* snap = nullptr;
  void* snap2 = nullptr;  // density and scratch when stored apart
  const bool apart = b->arena2 != b->arena;
  if (cudaMalloc(&snap, b->arena_elems * b->esize) != cudaSuccess)
    return fail(EQ_ERR_OOM, "cudaMalloc (autotune snapshot)");
  if (apart && cudaMalloc(&snap2, b->arena_elems * b->esize2) != cudaSuccess) {
    cudaFree(snap);
    return fail(EQ_ERR_OOM, "cudaMalloc (autotune snapshot)");
  }
  EQ_CUDA(cudaMemcpyAsync(snap, b->arena, b->arena_elems * b->esize, cudaMemcpyDeviceToDevice,
                          b->stream));
  if (apart)
    EQ_CUDA(cudaMemcpyAsync(snap2, b->arena2, b->arena_elems * b->esize2,
                            cudaMemcpyDeviceToDevice, b->stream));
  const int onw = b->nwmax, obps = b->bps;
  int best = -1;
  double best_ms = 0.0;
  cudaEvent_t e0, e1;
  EQ_CUDA(cudaEventCreate(&e0));
  EQ_CUDA(cudaEventCreate(&e1));
  for (size_t q = 0; q < cand.size(); ++q) {
    double ms = 0.0;
    if (eq_batch_set_tuning(b, cand[q].first, cand[q].second) == EQ_OK) {
      BLaunch L;
      if ((rc = batch_launch_shape(b, &L))) break;
      // one untimed frame (first-touch, module load), then the timed frames
      if ((rc = batch_enqueue_frames(b, L, 1))) break;
      EQ_CUDA(cudaEventRecord(e0, b->stream));
      if ((rc = batch_enqueue_frames(b, L, trial_frames))) break;
      EQ_CUDA(cudaEventRecord(e1, b->stream));
      EQ_CUDA(cudaEventSynchronize(e1));
      float t = 0.f;
      EQ_CUDA(cudaEventElapsedTime(&t, e0, e1));
      ms = (double)t / trial_frames;
      EQ_CUDA(cudaMemcpyAsync(b->arena, snap, b->arena_elems * b->esize,
                              cudaMemcpyDeviceToDevice, b->stream));
      if (apart)
        EQ_CUDA(cudaMemcpyAsync(b->arena2, snap2, b->arena_elems * b->esize2,
                                cudaMemcpyDeviceToDevice, b->stream));
      if (best < 0 || ms < best_ms) {
        best = (int)q;
        best_ms = ms;
      }
    }
    if (ms_out && (int)q < cap) ms_out[q] = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamSynchronize(b->stream);
  cudaFree(snap);
  cudaFree(snap2);
  if (rc) return rc;
  if (ncand) *ncand = (int)cand.size();
  if (best < 0) {
    b->nwmax = onw;
    b->bps = obps;
    return fail(EQ_ERR_STATE, "no autotune candidate fits");
  }
  b->nwmax = cand[best].first;
  b->bps = cand[best].second;
  return EQ_OK;
}

}  // extern "C"
