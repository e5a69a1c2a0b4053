// Host side of the differentiation form (include/eqfluid.h, "adjoint"): a
// recorded forward run of a plain handle (sources added each frame, then
// step()), checkpoints every C frames, and backward(): segment by segment from
// the last, the segment's frames are recomputed from their checkpoint with the
// fields each advect reads saved (the tape), then undone frame by frame with
// the adjoint kernels. Compiled in the same translation unit as eqfluid.cu (it
// drives the plain handle's launches).
#include <atomic>

#include "adjoint.cuh"

struct eq_grad {
  eq_fluid* h = nullptr;
  int64_t max_frames = 0, every = 8, nframes = 0;
  bool recorded = false, seeded = false;
  // what the recorded run used (backward refuses if the handle changed)
  float dt = 0.f, diff = 0.f, visc = 0.f;
  int64_t K = 0;
  std::vector<uint8_t> cells;
  size_t grid = 0;              // floats per pitched grid
  size_t dn = 0;                // floats per anti-diagonal grid
  size_t nn = 0;                // S * S
  float* ckpt = nullptr;        // nseg x 6 pitched grids
  float* final_state = nullptr; // 6 pitched grids
  float* tape = nullptr;        // every x 5 pitched grids (vx0, vy0, vx, vy, sc)
  int64_t tape_seg = -1;        // the segment whose frames the tape holds
  float* src = nullptr;         // max_frames x S x S dense
  bool have_src = false;
  float* adj = nullptr;         // the six adjoint grids (anti-diagonal)
  float* work = nullptr;        // tmp, Y0, Y1, Ysum, yK (anti-diagonal)
  float* xwork = nullptr;       // two more such sets, for backward's side streams
  // The stream and work set the adjoint launches use: the handle's stream
  // and `work`, except inside adj_step's side branches (the handle's side
  // streams with a set of xwork each), forked from and joined to the stream
  // by afork / ajoin.
  cudaStream_t cs = nullptr;
  float* cw = nullptr;
  cudaEvent_t afork = nullptr;
  cudaEvent_t ajoin[2] = {};
  float* phase = nullptr;       // 4 anti-diagonal grids for the per-phase entry points
  uint8_t* dcode = nullptr;     // boundary codes, anti-diagonal
  float* dense = nullptr;       // 12 x S x S staging
  float* gsrc = nullptr;        // max_frames x S x S (host-pointer backward)
  float* pstage = nullptr;      // 3 pitched grids (per-phase advect inputs)
  double* d_loss = nullptr;
  uint64_t launches = 0;
  bool profiling = false;  // event pairs around every adjoint wavefront launch
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> gs_events;
  int gs_store = 0;   // where the adjoint wavefront keeps its band (see gs_adj_smem_bytes)
  int gs_force = -1;  // cap on gs_store (tests of the other forms)
  int gs_cluster = 8; // blocks per cluster (gs_store == 3)
  int gs_m = 0;       // its barrier interval - 1
  int gs_mmax = -1;   // cap on gs_m; -1: 2 for N >= 192, else 1 (the fastest, measured)
};

namespace {

constexpr int kTapeFields = 5;  // vx0, vy0 (after project 1), vx, vy (after project 2), sc

float* gadj(eq_grad* g, int f) { return g->adj + (size_t)f * g->dn; }
float* gtmp(eq_grad* g) { return g->cw; }

int gcheck(eq_grad* g) {
  g->launches++;
  EQ_CUDA(cudaGetLastError());
  return EQ_OK;
}

dim3 gblk() { return dim3(32, 8); }
dim3 ggrd(const eq_grad* g) { return grid2d((int)g->h->S, (int)g->h->S, gblk()); }

int grad_codes(eq_grad* g) {
  eq_fluid* h = g->h;
  int rc = upload_mask(h);
  if (rc) return rc;
  eqk::k_code_to_diag<<<ggrd(g), gblk(), 0, h->stream>>>(h->code, h->P, g->dcode, (int)h->S, h->P);
  return gcheck(g);
}

// x = set_boundaries^T(x) (through the tmp grid).
int adj_bnd(eq_grad* g, int mode, float* x) {
  eq_fluid* h = g->h;
  const int S = (int)h->S, P = h->P;
  float* t = gtmp(g);
  switch (mode) {
    case eqk::kRow:
      eqk::k_adj_bnd<eqk::kRow><<<ggrd(g), gblk(), 0, g->cs>>>(x, t, g->dcode, h->rowfl, h->colfl, S, P);
      break;
    case eqk::kCol:
      eqk::k_adj_bnd<eqk::kCol><<<ggrd(g), gblk(), 0, g->cs>>>(x, t, g->dcode, h->rowfl, h->colfl, S, P);
      break;
    default:
      eqk::k_adj_bnd<eqk::kPassive><<<ggrd(g), gblk(), 0, g->cs>>>(x, t, g->dcode, h->rowfl, h->colfl, S, P);
      break;
  }
  int rc = gcheck(g);
  if (rc) return rc;
  EQ_CUDA(cudaMemcpyAsync(x, t, g->dn * sizeof(float), cudaMemcpyDeviceToDevice, g->cs));
  return EQ_OK;
}

// Threads of one cluster block: a warp per (sweep, 32-position chunk) task,
// at most 32 warps.
int gs_cl_threads(int S, int K, int C) {
  const int J = (S - 2 + C - 1) / C;
  return 32 * std::min(32, K * ((J + 31) / 32));
}

template <int MODE>
int launch_gs_adj(eq_grad* g, const eqk::GsAdjArgs& A) {
  const int store = g->gs_store;
  const size_t smem = eqk::gs_adj_smem_bytes(store, A.S, A.K);
  cudaStream_t s = g->cs;
  if (store == 3) {  // a cluster of g->gs_cluster blocks
    cudaEvent_t c0 = nullptr, c1 = nullptr;
    if (g->profiling) {
      EQ_CUDA(cudaEventCreate(&c0));
      EQ_CUDA(cudaEventCreate(&c1));
      EQ_CUDA(cudaEventRecord(c0, s));
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(g->gs_cluster);
    cfg.blockDim = dim3(gs_cl_threads(A.S, A.K, g->gs_cluster));
    cfg.dynamicSmemBytes = eqk::gs_cl_layout(A.S, A.K, g->gs_cluster, A.m).total;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = g->gs_cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    EQ_CUDA(cudaLaunchKernelEx(&cfg, eqk::k_gs_adj_cl<MODE>, A));
    int rc = gcheck(g);
    if (rc) return rc;
    if (g->profiling) {
      EQ_CUDA(cudaEventRecord(c1, s));
      g->gs_events.emplace_back(c0, c1);
    }
    return EQ_OK;
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (g->profiling) {
    EQ_CUDA(cudaEventCreate(&e0));
    EQ_CUDA(cudaEventCreate(&e1));
    EQ_CUDA(cudaEventRecord(e0, s));
  }
  if (store == 2)
    eqk::k_gs_adj<MODE, 2><<<1, 1024, smem, s>>>(A);
  else if (store == 1)
    eqk::k_gs_adj<MODE, 1><<<1, 1024, smem, s>>>(A);
  else
    eqk::k_gs_adj<MODE, 0><<<1, 1024, 0, s>>>(A);
  int rc = gcheck(g);
  if (rc) return rc;
  if (g->profiling) {
    EQ_CUDA(cudaEventRecord(e1, s));
    g->gs_events.emplace_back(e0, e1);
  }
  return EQ_OK;
}

// The storage form of the wavefront for this size and sweep count: a cluster
// when every block keeps >= 16 positions, its share fits and the device can
// hold the cluster, else one block with shared memory where the band fits
// (the kernels' attributes are raised once).
int pick_gs_store(eq_grad* g, int S, int K) {
  // kernel attributes are per device: one bit per device once they are raised
  static std::atomic<uint64_t> raised{0};
  int dev = g->h->device, optin = 0;
  EQ_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  const uint64_t bit = dev < 64 ? (1ull << dev) : 0ull;
  if (!bit || !(raised.load() & bit)) {
    auto raise = [&](const void* fn) {
      return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    };
    auto nonportable = [&](const void* fn) {
      return cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    };
    if (raise((const void*)eqk::k_gs_adj<eqk::kRow, 1>) != cudaSuccess ||
        raise((const void*)eqk::k_gs_adj<eqk::kRow, 2>) != cudaSuccess ||
        raise((const void*)eqk::k_gs_adj<eqk::kCol, 1>) != cudaSuccess ||
        raise((const void*)eqk::k_gs_adj<eqk::kCol, 2>) != cudaSuccess ||
        raise((const void*)eqk::k_gs_adj<eqk::kPassive, 1>) != cudaSuccess ||
        raise((const void*)eqk::k_gs_adj<eqk::kPassive, 2>) != cudaSuccess ||
        raise((const void*)eqk::k_gs_adj_cl<eqk::kRow>) != cudaSuccess ||
        raise((const void*)eqk::k_gs_adj_cl<eqk::kCol>) != cudaSuccess ||
        raise((const void*)eqk::k_gs_adj_cl<eqk::kPassive>) != cudaSuccess ||
        nonportable((const void*)eqk::k_gs_adj_cl<eqk::kRow>) != cudaSuccess ||
        nonportable((const void*)eqk::k_gs_adj_cl<eqk::kCol>) != cudaSuccess ||
        nonportable((const void*)eqk::k_gs_adj_cl<eqk::kPassive>) != cudaSuccess)
      return fail(EQ_ERR_CUDA, "cudaFuncSetAttribute (adjoint wavefront)");
    raised.fetch_or(bit);
  }
  bool ok[4];
  ok[0] = true;
  ok[1] = eqk::gs_adj_smem_bytes(1, S, K) <= (size_t)optin;
  ok[2] = eqk::gs_adj_smem_bytes(2, S, K) <= (size_t)optin;
  ok[3] = false;
  const int C = (S - 2) >= 384 ? 16 : 8;
  // the barrier interval: m + 1 steps where every warp has one task (the
  // streamlined path) and the stretched band fits, else a barrier per step
  const int J = (S - 2 + C - 1) / C;
  const int mcap = g->gs_mmax >= 0 ? g->gs_mmax : (S - 2 >= 192 ? 2 : 1);
  int m = (K * ((J + 31) / 32) <= 32) ? mcap : 0;
  while (m > 0 && eqk::gs_cl_layout(S, K, C, m).total > (size_t)optin) --m;
  g->gs_m = m;
  const size_t cl_bytes = eqk::gs_cl_layout(S, K, C, m).total;
  if ((S - 2) / C >= 16 && cl_bytes <= (size_t)optin) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(C);
    cfg.blockDim = dim3(gs_cl_threads(S, K, C));
    cfg.dynamicSmemBytes = cl_bytes;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    ok[3] = cudaOccupancyMaxActiveClusters(&nclusters, eqk::k_gs_adj_cl<eqk::kRow>, &cfg) ==
                cudaSuccess &&
            nclusters >= 1;
    cudaGetLastError();  // a refused query leaves the single-block forms
  }
  const int cap = g->gs_force >= 0 ? g->gs_force : 3;
  int store = 0;
  for (int k = cap; k >= 0; --k)
    if (ok[k]) {
      store = k;
      break;
    }
  g->gs_store = store;
  g->gs_cluster = C;
  return EQ_OK;
}

// lin_solve^T: xb (adjoint after the solve) -> adjoint before it; x0b += ...
int adj_lin_solve(eq_grad* g, int mode, float* xb, float* x0b, float a, float c) {
  eq_fluid* h = g->h;
  const int64_t K = h->frames;
  if (K <= 0) return EQ_OK;
  if (K > (1 << 20)) return fail(EQ_ERR_ARG, "too many sweeps for the adjoint");
  const int S = (int)h->S, P = h->P;
  float* t = gtmp(g);
  float* Y0 = g->cw + g->dn;
  float* Y1 = g->cw + 2 * g->dn;
  float* Ys = g->cw + 3 * g->dn;
  float* yK = g->cw + 4 * g->dn;
  const float cr = 1.0f / c, alpha = a * cr;
  int rc;
  if ((rc = pick_gs_store(g, S, (int)K))) return rc;
  switch (mode) {
    case eqk::kRow:
      eqk::k_adj_bnd<eqk::kRow><<<ggrd(g), gblk(), 0, g->cs>>>(xb, t, g->dcode, h->rowfl, h->colfl, S, P);
      break;
    case eqk::kCol:
      eqk::k_adj_bnd<eqk::kCol><<<ggrd(g), gblk(), 0, g->cs>>>(xb, t, g->dcode, h->rowfl, h->colfl, S, P);
      break;
    default:
      eqk::k_adj_bnd<eqk::kPassive><<<ggrd(g), gblk(), 0, g->cs>>>(xb, t, g->dcode, h->rowfl, h->colfl, S, P);
      break;
  }
  if ((rc = gcheck(g))) return rc;
  // Ghost positions of Ysum and yK stay 0 (never written); their interior is
  // rewritten by every solve except Ysum accumulated in global memory.
  if (g->gs_store < 2) EQ_CUDA(cudaMemsetAsync(Y0, 0, 3 * g->dn * sizeof(float), g->cs));
  eqk::GsAdjArgs A;
  A.B = t;
  A.Y0 = Y0;
  A.Y1 = Y1;
  A.Ysum = Ys;
  A.yK = yK;
  A.code = g->dcode;
  A.rowfl = h->rowfl;
  A.colfl = h->colfl;
  A.S = S;
  A.P = P;
  A.K = (int)K;
  A.m = g->gs_store == 3 ? g->gs_m : 0;
  A.R = g->gs_store == 3 ? eqk::gs_cl_rows((int)K, A.m) : (int)(3 * K + 4);
  A.alpha = alpha;
  switch (mode) {
    case eqk::kRow:
      if ((rc = launch_gs_adj<eqk::kRow>(g, A))) return rc;
      eqk::k_gs_adj_out<eqk::kRow><<<ggrd(g), gblk(), 0, g->cs>>>(xb, t, yK, Ys, x0b, g->dcode, h->rowfl, h->colfl, S, P, alpha, cr);
      break;
    case eqk::kCol:
      if ((rc = launch_gs_adj<eqk::kCol>(g, A))) return rc;
      eqk::k_gs_adj_out<eqk::kCol><<<ggrd(g), gblk(), 0, g->cs>>>(xb, t, yK, Ys, x0b, g->dcode, h->rowfl, h->colfl, S, P, alpha, cr);
      break;
    default:
      if ((rc = launch_gs_adj<eqk::kPassive>(g, A))) return rc;
      eqk::k_gs_adj_out<eqk::kPassive><<<ggrd(g), gblk(), 0, g->cs>>>(xb, t, yK, Ys, x0b, g->dcode, h->rowfl, h->colfl, S, P, alpha, cr);
      break;
  }
  return gcheck(g);
}

// advect^T at the forward state (d0, u, v pitched).
int adj_advect(eq_grad* g, int mode, float* db, float* d0b, float* ub, float* vb,
               const float* d0, const float* u, const float* v) {
  eq_fluid* h = g->h;
  int rc = adj_bnd(g, mode, db);
  if (rc) return rc;
  const int S = (int)h->S, N = S - 2;
  const float dt0 = h->dt * (float)(h->S - 2);
  const int threads = std::min(256, ((N + 31) / 32) * 32);
  eqk::k_adv_adj_rows<<<N, threads, 0, g->cs>>>(db, d0b, ub, vb, d0, u, v, S, h->P, h->P, dt0);
  return gcheck(g);
}

// project^T with p and div the aliased arrays (fluid.rs:330-375 transposed).
int adj_project(eq_grad* g, float* vxb, float* vyb, float* pb, float* divb) {
  eq_fluid* h = g->h;
  const int S = (int)h->S, P = h->P;
  int rc;
  if ((rc = adj_bnd(g, eqk::kCol, vyb)) || (rc = adj_bnd(g, eqk::kRow, vxb))) return rc;
  eqk::k_grad_adj<<<ggrd(g), gblk(), 0, g->cs>>>(vxb, vyb, pb, S, P);
  if ((rc = gcheck(g))) return rc;
  if ((rc = adj_lin_solve(g, eqk::kPassive, pb, divb, 1.0f, 4.0f))) return rc;
  if ((rc = adj_bnd(g, eqk::kPassive, pb)) || (rc = adj_bnd(g, eqk::kPassive, divb))) return rc;
  eqk::k_div_adj<<<ggrd(g), gblk(), 0, g->cs>>>(vxb, vyb, divb, S, P);
  if ((rc = gcheck(g))) return rc;
  const dim3 gi = grid2d(S - 2, S - 2, gblk());
  eqk::k_zero_interior2<<<gi, gblk(), 0, g->cs>>>(pb, divb, S, P);
  return gcheck(g);
}

// step^T (fluid.rs:437-524 transposed) at the frame's tape.
int adj_step(eq_grad* g, const float* tp) {
  eq_fluid* h = g->h;
  const int S = (int)h->S, P = h->P;
  const size_t G = g->grid;
  const float* t_vx0 = tp;
  const float* t_vy0 = tp + G;
  const float* t_vx = tp + 2 * G;
  const float* t_vy = tp + 3 * G;
  const float* t_sc = tp + 4 * G;
  float* scb = gadj(g, EQ_FIELD_SCRATCH);
  float* deb = gadj(g, EQ_FIELD_DENSITY);
  float* vxb = gadj(g, EQ_FIELD_VX);
  float* vyb = gadj(g, EQ_FIELD_VY);
  float* vx0b = gadj(g, EQ_FIELD_VX0);
  float* vy0b = gadj(g, EQ_FIELD_VY0);
  const float sf = (float)(S - 2);
  const float ad = ((h->dt * h->diff) * sf) * sf;
  const float av = ((h->dt * h->visc) * sf) * sf;
  int rc;
  eqk::k_adj_clone<<<ggrd(g), gblk(), 0, g->cs>>>(deb, scb, S, P);
  if ((rc = gcheck(g))) return rc;
  if ((rc = adj_advect(g, eqk::kPassive, deb, scb, vxb, vyb, t_sc, t_vx, t_vy))) return rc;
  // From here the density's diffusion^T (scb, deb) and the velocity chain
  // (vxb, vyb, vx0b, vy0b) touch disjoint grids, and so do the last two
  // diffusions^T: with the handle's concurrency on they run on its side
  // streams, each with its own work set, joined at the end of the frame.
  const bool side = h->concurrent != 0;
  cudaStream_t mst = h->stream;
  auto on = [&](cudaStream_t st, float* w) {
    g->cs = st;
    g->cw = w;
  };
  auto fork = [&](int k) -> int {
    EQ_CUDA(cudaEventRecord(g->afork, mst));
    EQ_CUDA(cudaStreamWaitEvent(h->side[k], g->afork, 0));
    on(h->side[k], g->xwork + (size_t)k * 5 * g->dn);
    return EQ_OK;
  };
  auto join = [&](int k) -> int {
    EQ_CUDA(cudaEventRecord(g->ajoin[k], h->side[k]));
    on(mst, g->work);
    return EQ_OK;
  };
  if (side) {
    if ((rc = fork(1))) return rc;
    rc = adj_lin_solve(g, eqk::kPassive, scb, deb, ad, 1.0f + 4.0f * ad);
    const int rj = join(1);
    if (rc || (rc = rj)) return rc;
  } else if ((rc = adj_lin_solve(g, eqk::kPassive, scb, deb, ad, 1.0f + 4.0f * ad))) {
    return rc;
  }
  if ((rc = adj_project(g, vxb, vyb, vx0b, vy0b))) return rc;
  if ((rc = adj_advect(g, eqk::kCol, vyb, vy0b, vx0b, vy0b, t_vy0, t_vx0, t_vy0))) return rc;
  if ((rc = adj_advect(g, eqk::kRow, vxb, vx0b, vx0b, vy0b, t_vx0, t_vx0, t_vy0))) return rc;
  if ((rc = adj_project(g, vx0b, vy0b, vxb, vyb))) return rc;
  if (side) {
    if ((rc = fork(0))) return rc;
    rc = adj_lin_solve(g, eqk::kCol, vy0b, vyb, av, 1.0f + 4.0f * av);
    const int rj = join(0);
    if (rc || (rc = rj)) return rc;
  } else if ((rc = adj_lin_solve(g, eqk::kCol, vy0b, vyb, av, 1.0f + 4.0f * av))) {
    return rc;
  }
  if ((rc = adj_lin_solve(g, eqk::kRow, vx0b, vxb, av, 1.0f + 4.0f * av))) return rc;
  if (side) {
    EQ_CUDA(cudaStreamWaitEvent(mst, g->ajoin[0], 0));
    EQ_CUDA(cudaStreamWaitEvent(mst, g->ajoin[1], 0));
  }
  return EQ_OK;
}

// The forward step with the fields each advect reads saved into tp (the
// plain step, its independent diffusions on side streams as configured).
int step_taped(eq_grad* g, float* tp) { return launch_step(g->h, tp); }

int add_frame_source(eq_grad* g, int64_t f) {
  if (!g->have_src) return EQ_OK;
  eq_fluid* h = g->h;
  eqk::k_add_src<<<ggrd(g), gblk(), 0, h->stream>>>(h->field[EQ_FIELD_DENSITY],
                                                      h->field[EQ_FIELD_SCRATCH],
                                                      g->src + (size_t)f * g->nn, (int)h->S, h->P);
  return gcheck(g);
}

int copy_state(eq_grad* g, float* dst, const float* src) {
  EQ_CUDA(cudaMemcpyAsync(dst, src, 6 * g->grid * sizeof(float), cudaMemcpyDeviceToDevice,
                          g->h->stream));
  return EQ_OK;
}

int unchanged(eq_grad* g) {
  eq_fluid* h = g->h;
  if (h->dt != g->dt || h->diff != g->diff || h->visc != g->visc || h->frames != g->K ||
      h->host_cells != g->cells)
    return fail(EQ_ERR_STATE, "the handle's configs or mask changed since the recorded forward");
  return EQ_OK;
}

int run_forward(eq_grad* g, int64_t nframes) {
  eq_fluid* h = g->h;
  int rc;
  if ((rc = select_device(h)) || (rc = grad_codes(g))) return rc;
  g->dt = h->dt;
  g->diff = h->diff;
  g->visc = h->visc;
  g->K = h->frames;
  g->cells = h->host_cells;
  // The last segment's frames keep their tape as they run: backward starts
  // there without recomputing it.
  const int64_t last = (nframes - 1) / g->every;
  const size_t tstride = (size_t)kTapeFields * g->grid;
  for (int64_t f = 0; f < nframes; ++f) {
    if (f % g->every == 0)
      if ((rc = copy_state(g, g->ckpt + (size_t)(f / g->every) * 6 * g->grid, h->block))) return rc;
    if ((rc = add_frame_source(g, f))) return rc;
    rc = (f / g->every == last) ? step_taped(g, g->tape + (size_t)(f - last * g->every) * tstride)
                                : launch_step(h);
    if (rc) return rc;
  }
  g->tape_seg = last;
  if ((rc = copy_state(g, g->final_state, h->block))) return rc;
  g->nframes = nframes;
  g->recorded = true;
  g->seeded = false;
  EQ_CUDA(cudaStreamSynchronize(h->stream));
  return read_err_word(h);
}

int check_n(uint64_t n, uint64_t want, const char* what) {
  return n == want ? EQ_OK : fail(EQ_ERR_ARG, std::string(what) + ": wrong element count");
}

int to_diag(eq_grad* g, const float* dense, float* diag) {
  eqk::k_dense_to_diag<<<ggrd(g), gblk(), 0, g->h->stream>>>(dense, diag, (int)g->h->S, g->h->P);
  return gcheck(g);
}
int to_dense(eq_grad* g, const float* a, const float* b, float* dense) {
  eqk::k_diag_to_dense<<<ggrd(g), gblk(), 0, g->h->stream>>>(a, b, dense, (int)g->h->S, g->h->P);
  return gcheck(g);
}

int run_backward(eq_grad* g, const float* d_adj_final, float* d_grad_init, float* d_grad_src) {
  eq_fluid* h = g->h;
  int rc;
  if (!g->recorded) return fail(EQ_ERR_STATE, "backward before a recorded forward");
  if (!d_adj_final && !g->seeded)
    return fail(EQ_ERR_STATE, "no adjoint of the final state (pass one or call l2_loss)");
  if ((rc = select_device(h)) || (rc = unchanged(g)) || (rc = grad_codes(g))) return rc;
  if (d_adj_final)
    for (int f = 0; f < 6; ++f)
      if ((rc = to_diag(g, d_adj_final + (size_t)f * g->nn, gadj(g, f)))) return rc;
  const int64_t nseg = (g->nframes + g->every - 1) / g->every;
  const size_t tstride = (size_t)kTapeFields * g->grid;
  for (int64_t seg = nseg - 1; seg >= 0; --seg) {
    const int64_t f0 = seg * g->every, f1 = std::min(f0 + g->every, g->nframes);
    if (g->tape_seg != seg) {  // recompute the segment from its checkpoint
      g->tape_seg = -1;
      if ((rc = copy_state(g, h->block, g->ckpt + (size_t)seg * 6 * g->grid))) return rc;
      for (int64_t f = f0; f < f1; ++f)
        if ((rc = add_frame_source(g, f)) ||
            (rc = step_taped(g, g->tape + (size_t)(f - f0) * tstride)))
          return rc;
      g->tape_seg = seg;
    }
    for (int64_t f = f1 - 1; f >= f0; --f) {
      if ((rc = adj_step(g, g->tape + (size_t)(f - f0) * tstride))) return rc;
      if (d_grad_src && (rc = to_dense(g, gadj(g, EQ_FIELD_DENSITY), gadj(g, EQ_FIELD_SCRATCH),
                                      d_grad_src + (size_t)f * g->nn)))
        return rc;
    }
  }
  if (d_grad_init)
    for (int f = 0; f < 6; ++f)
      if ((rc = to_dense(g, gadj(g, f), nullptr, d_grad_init + (size_t)f * g->nn))) return rc;
  if ((rc = copy_state(g, h->block, g->final_state))) return rc;
  g->seeded = false;
  return EQ_OK;
}

void free_grad(eq_grad* g) {
  if (!g) return;
  if (g->h) cudaSetDevice(g->h->device);
  for (auto& e : g->gs_events) {
    cudaEventDestroy(e.first);
    cudaEventDestroy(e.second);
  }
  cudaFree(g->ckpt);
  cudaFree(g->final_state);
  cudaFree(g->tape);
  cudaFree(g->src);
  cudaFree(g->adj);
  cudaFree(g->work);
  cudaFree(g->xwork);
  if (g->afork) cudaEventDestroy(g->afork);
  for (cudaEvent_t e : g->ajoin)
    if (e) cudaEventDestroy(e);
  cudaFree(g->phase);
  cudaFree(g->dcode);
  cudaFree(g->dense);
  cudaFree(g->gsrc);
  cudaFree(g->pstage);
  cudaFree(g->d_loss);
  delete g;
}

// Per-phase entry points: host S x S arrays in, through the anti-diagonal
// phase grids, back out.
int phase_in(eq_grad* g, const float* host, int slot) {
  eq_fluid* h = g->h;
  float* d = g->dense + (size_t)slot * g->nn;
  EQ_CUDA(cudaMemcpyAsync(d, host, g->nn * sizeof(float), cudaMemcpyHostToDevice, h->stream));
  return to_diag(g, d, g->phase + (size_t)slot * g->dn);
}
int phase_out(eq_grad* g, float* host, int slot) {
  eq_fluid* h = g->h;
  float* d = g->dense + (size_t)slot * g->nn;
  int rc = to_dense(g, g->phase + (size_t)slot * g->dn, nullptr, d);
  if (rc) return rc;
  EQ_CUDA(cudaMemcpyAsync(host, d, g->nn * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
  return EQ_OK;
}
int phase_begin(eq_grad* g, uint64_t n) {
  if (!g) return fail(EQ_ERR_ARG, "null handle");
  int rc;
  if ((rc = check_n(n, g->nn, "array")) || (rc = select_device(g->h)) || (rc = grad_codes(g)))
    return rc;
  return EQ_OK;
}
int phase_end(eq_grad* g) {
  EQ_CUDA(cudaStreamSynchronize(g->h->stream));
  return EQ_OK;
}

}  // namespace

extern "C" {

int eq_grad_new(eq_fluid* h, int64_t max_frames, int64_t checkpoint_every, eq_grad** out) {
  if (!h || !out) return fail(EQ_ERR_ARG, "null argument");
  if (max_frames < 1) return fail(EQ_ERR_ARG, "max_frames must be >= 1");
  if (checkpoint_every < 1) return fail(EQ_ERR_ARG, "checkpoint_every must be >= 1");
  if (h->S < 8) return fail(EQ_ERR_ARG, "the adjoint needs size >= 8");
  int rc = select_device(h);
  if (rc) return rc;
  eq_grad* g = new eq_grad();
  g->h = h;
  g->max_frames = max_frames;
  g->every = std::min(checkpoint_every, max_frames);
  g->grid = h->grid_elems();
  g->dn = eqk::dg_size((int)h->S, h->P);
  g->nn = (size_t)h->S * h->S;
  const int64_t nseg = (max_frames + g->every - 1) / g->every;
  auto bail = [&](const char* what) {
    free_grad(g);
    return fail(EQ_ERR_OOM, what);
  };
  const size_t F = sizeof(float);
  if (cudaMalloc(&g->ckpt, (size_t)nseg * 6 * g->grid * F) != cudaSuccess ||
      cudaMalloc(&g->final_state, 6 * g->grid * F) != cudaSuccess ||
      cudaMalloc(&g->tape, (size_t)g->every * kTapeFields * g->grid * F) != cudaSuccess)
    return bail("cudaMalloc (checkpoints, tape)");
  if (cudaMalloc(&g->src, (size_t)max_frames * g->nn * F) != cudaSuccess ||
      cudaMalloc(&g->adj, 6 * g->dn * F) != cudaSuccess ||
      cudaMalloc(&g->work, 5 * g->dn * F) != cudaSuccess ||
      cudaMalloc(&g->xwork, 10 * g->dn * F) != cudaSuccess ||
      cudaMalloc(&g->phase, 4 * g->dn * F) != cudaSuccess ||
      cudaMalloc(&g->dcode, g->dn) != cudaSuccess ||
      cudaMalloc(&g->dense, 12 * g->nn * F) != cudaSuccess ||
      cudaMalloc(&g->pstage, 3 * g->grid * F) != cudaSuccess ||
      cudaMalloc(&g->d_loss, sizeof(double)) != cudaSuccess)
    return bail("cudaMalloc (adjoint state)");
  cudaStream_t s = h->stream;
  if (cudaMemsetAsync(g->adj, 0, 6 * g->dn * F, s) != cudaSuccess ||
      cudaMemsetAsync(g->work, 0, 5 * g->dn * F, s) != cudaSuccess ||
      cudaMemsetAsync(g->xwork, 0, 10 * g->dn * F, s) != cudaSuccess ||
      cudaMemsetAsync(g->phase, 0, 4 * g->dn * F, s) != cudaSuccess ||
      cudaMemsetAsync(g->pstage, 0, 3 * g->grid * F, s) != cudaSuccess) {
    free_grad(g);
    return fail(EQ_ERR_CUDA, "cudaMemsetAsync");
  }
  g->cs = h->stream;
  g->cw = g->work;
  if (cudaEventCreateWithFlags(&g->afork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&g->ajoin[0], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&g->ajoin[1], cudaEventDisableTiming) != cudaSuccess) {
    free_grad(g);
    return fail(EQ_ERR_CUDA, "cudaEventCreate");
  }
  *out = g;
  return EQ_OK;
}

int eq_grad_free(eq_grad* g) {
  free_grad(g);
  return EQ_OK;
}

int eq_grad_forward_device(eq_grad* g, int64_t nframes, const float* d_src) {
  if (!g) return fail(EQ_ERR_ARG, "null handle");
  if (nframes < 1 || nframes > g->max_frames)
    return fail(EQ_ERR_ARG, "nframes must be in [1, max_frames]");
  int rc = select_device(g->h);
  if (rc) return rc;
  g->have_src = d_src != nullptr;
  if (d_src)
    EQ_CUDA(cudaMemcpyAsync(g->src, d_src, (size_t)nframes * g->nn * sizeof(float),
                            cudaMemcpyDeviceToDevice, g->h->stream));
  return run_forward(g, nframes);
}

int eq_grad_forward(eq_grad* g, int64_t nframes, const float* src, uint64_t n) {
  if (!g) return fail(EQ_ERR_ARG, "null handle");
  if (nframes < 1 || nframes > g->max_frames)
    return fail(EQ_ERR_ARG, "nframes must be in [1, max_frames]");
  int rc;
  if (src && (rc = check_n(n, (uint64_t)nframes * g->nn, "src"))) return rc;
  if ((rc = select_device(g->h))) return rc;
  g->have_src = src != nullptr;
  if (src)
    EQ_CUDA(cudaMemcpyAsync(g->src, src, (size_t)nframes * g->nn * sizeof(float),
                            cudaMemcpyHostToDevice, g->h->stream));
  return run_forward(g, nframes);
}

int eq_grad_l2_loss(eq_grad* g, const float* target, uint64_t n, double* loss,
                    float* adj_density) {
  if (!g || !target || !loss) return fail(EQ_ERR_ARG, "null argument");
  if (!g->recorded) return fail(EQ_ERR_STATE, "l2_loss before a recorded forward");
  int rc;
  if ((rc = check_n(n, g->nn, "target")) || (rc = select_device(g->h))) return rc;
  eq_fluid* h = g->h;
  EQ_CUDA(cudaMemcpyAsync(g->dense, target, g->nn * sizeof(float), cudaMemcpyHostToDevice,
                          h->stream));
  EQ_CUDA(cudaMemsetAsync(g->adj, 0, 6 * g->dn * sizeof(float), h->stream));
  EQ_CUDA(cudaMemsetAsync(g->d_loss, 0, sizeof(double), h->stream));
  eqk::k_l2_loss<<<ggrd(g), gblk(), 0, h->stream>>>(
      g->final_state + (size_t)EQ_FIELD_DENSITY * g->grid, h->P, g->dense,
      gadj(g, EQ_FIELD_DENSITY), (int)h->S, h->P, g->d_loss);
  if ((rc = gcheck(g))) return rc;
  EQ_CUDA(cudaMemcpyAsync(loss, g->d_loss, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  if (adj_density) {
    if ((rc = to_dense(g, gadj(g, EQ_FIELD_DENSITY), nullptr, g->dense + g->nn))) return rc;
    EQ_CUDA(cudaMemcpyAsync(adj_density, g->dense + g->nn, g->nn * sizeof(float),
                            cudaMemcpyDeviceToHost, h->stream));
  }
  EQ_CUDA(cudaStreamSynchronize(h->stream));
  g->seeded = true;
  return EQ_OK;
}

int eq_grad_backward_device(eq_grad* g, const float* d_adj_final, float* d_grad_init,
                            float* d_grad_src) {
  if (!g) return fail(EQ_ERR_ARG, "null handle");
  int rc = run_backward(g, d_adj_final, d_grad_init, d_grad_src);
  if (rc) return rc;
  EQ_CUDA(cudaStreamSynchronize(g->h->stream));
  return read_err_word(g->h);
}

int eq_grad_backward(eq_grad* g, const float* adj_final, uint64_t n_adj, float* grad_init,
                     uint64_t n_init, float* grad_src, uint64_t n_src) {
  if (!g) return fail(EQ_ERR_ARG, "null handle");
  int rc;
  if (adj_final && (rc = check_n(n_adj, 6 * g->nn, "adj_final"))) return rc;
  if (grad_init && (rc = check_n(n_init, 6 * g->nn, "grad_init"))) return rc;
  if (grad_src && (rc = check_n(n_src, (uint64_t)g->nframes * g->nn, "grad_src"))) return rc;
  if ((rc = select_device(g->h))) return rc;
  eq_fluid* h = g->h;
  if (grad_src && !g->gsrc) {
    if (cudaMalloc(&g->gsrc, (size_t)g->max_frames * g->nn * sizeof(float)) != cudaSuccess)
      return fail(EQ_ERR_OOM, "cudaMalloc (source gradients)");
  }
  if (adj_final)
    EQ_CUDA(cudaMemcpyAsync(g->dense, adj_final, 6 * g->nn * sizeof(float),
                            cudaMemcpyHostToDevice, h->stream));
  if ((rc = run_backward(g, adj_final ? g->dense : nullptr, grad_init ? g->dense + 6 * g->nn : nullptr,
                         grad_src ? g->gsrc : nullptr)))
    return rc;
  if (grad_init)
    EQ_CUDA(cudaMemcpyAsync(grad_init, g->dense + 6 * g->nn, 6 * g->nn * sizeof(float),
                            cudaMemcpyDeviceToHost, h->stream));
  if (grad_src)
    EQ_CUDA(cudaMemcpyAsync(grad_src, g->gsrc, (size_t)g->nframes * g->nn * sizeof(float),
                            cudaMemcpyDeviceToHost, h->stream));
  EQ_CUDA(cudaStreamSynchronize(h->stream));
  return read_err_word(h);
}

int eq_grad_frames(const eq_grad* g, int64_t* recorded) {
  if (!g || !recorded) return fail(EQ_ERR_ARG, "null argument");
  *recorded = g->recorded ? g->nframes : 0;
  return EQ_OK;
}

int eq_grad_launch_count(const eq_grad* g, uint64_t* count) {
  if (!g || !count) return fail(EQ_ERR_ARG, "null argument");
  *count = g->launches;
  return EQ_OK;
}

int eq_grad_set_profiling(eq_grad* g, int enable) {
  if (!g) return fail(EQ_ERR_ARG, "null handle");
  g->profiling = enable != 0;
  return EQ_OK;
}

int eq_grad_kernel_stats(eq_grad* g, double* total_ms, uint64_t* launches) {
  if (!g || !total_ms || !launches) return fail(EQ_ERR_ARG, "null argument");
  int rc = select_device(g->h);
  if (rc) return rc;
  EQ_CUDA(cudaStreamSynchronize(g->h->stream));
  double sum = 0.0;
  for (auto& e : g->gs_events) {
    float ms = 0.f;
    EQ_CUDA(cudaEventElapsedTime(&ms, e.first, e.second));
    sum += ms;
    cudaEventDestroy(e.first);
    cudaEventDestroy(e.second);
  }
  *total_ms = sum;
  *launches = g->gs_events.size();
  g->gs_events.clear();
  return EQ_OK;
}

int eq_grad_set_wavefront_storage(eq_grad* g, int max_store) {
  if (!g) return fail(EQ_ERR_ARG, "null handle");
  if (max_store < -1 || max_store > 3) return fail(EQ_ERR_ARG, "max_store must be in [-1, 3]");
  g->gs_force = max_store;
  return EQ_OK;
}

int eq_grad_set_cluster_interval(eq_grad* g, int max_m) {
  if (!g) return fail(EQ_ERR_ARG, "null handle");
  if (max_m < 0 || max_m > 3) return fail(EQ_ERR_ARG, "max_m must be in [0, 3]");
  g->gs_mmax = max_m;
  return EQ_OK;
}

int eq_grad_get_wavefront_storage(const eq_grad* g, int* store, int* cluster_blocks) {
  if (!g || !store || !cluster_blocks) return fail(EQ_ERR_ARG, "null argument");
  *store = g->gs_store;
  *cluster_blocks = g->gs_store == 3 ? g->gs_cluster : 1;
  return EQ_OK;
}

int eq_grad_set_boundaries_adj(eq_grad* g, int mode, float* xb, uint64_t n) {
  int rc;
  if ((rc = check_mode(mode)) || (rc = phase_begin(g, n))) return rc;
  if (!xb) return fail(EQ_ERR_ARG, "null array");
  if ((rc = phase_in(g, xb, 0)) || (rc = adj_bnd(g, mode, g->phase)) || (rc = phase_out(g, xb, 0)))
    return rc;
  return phase_end(g);
}

int eq_grad_lin_solve_adj(eq_grad* g, int mode, float* xb, float* x0b, float a, float c,
                          uint64_t n) {
  int rc;
  if ((rc = check_mode(mode)) || (rc = phase_begin(g, n))) return rc;
  if (!xb || !x0b) return fail(EQ_ERR_ARG, "null array");
  if ((rc = phase_in(g, xb, 0)) || (rc = phase_in(g, x0b, 1))) return rc;
  if ((rc = adj_lin_solve(g, mode, g->phase, g->phase + g->dn, a, c))) return rc;
  if ((rc = phase_out(g, xb, 0)) || (rc = phase_out(g, x0b, 1))) return rc;
  return phase_end(g);
}

int eq_grad_advect_adj(eq_grad* g, int mode, float* db, float* d0b, float* ub, float* vb,
                       const float* d0, const float* u, const float* v, uint64_t n) {
  int rc;
  if ((rc = check_mode(mode)) || (rc = phase_begin(g, n))) return rc;
  if (!db || !d0b || !ub || !vb || !d0 || !u || !v) return fail(EQ_ERR_ARG, "null array");
  eq_fluid* h = g->h;
  const size_t w = (size_t)h->S * sizeof(float);
  const float* in[3] = {d0, u, v};
  for (int k = 0; k < 3; ++k)
    EQ_CUDA(cudaMemcpy2DAsync(g->pstage + k * g->grid, (size_t)h->P * sizeof(float), in[k], w, w,
                              h->S, cudaMemcpyHostToDevice, h->stream));
  float* io[4] = {db, d0b, ub, vb};
  for (int k = 0; k < 4; ++k)
    if ((rc = phase_in(g, io[k], k))) return rc;
  if ((rc = adj_advect(g, mode, g->phase, g->phase + g->dn, g->phase + 2 * g->dn,
                       g->phase + 3 * g->dn, g->pstage, g->pstage + g->grid,
                       g->pstage + 2 * g->grid)))
    return rc;
  for (int k = 0; k < 4; ++k)
    if ((rc = phase_out(g, io[k], k))) return rc;
  return phase_end(g);
}

int eq_grad_project_adj(eq_grad* g, float* vxb, float* vyb, float* pb, float* divb,
                        uint64_t n) {
  int rc;
  if ((rc = phase_begin(g, n))) return rc;
  if (!vxb || !vyb || !pb || !divb) return fail(EQ_ERR_ARG, "null array");
  float* io[4] = {vxb, vyb, pb, divb};
  for (int k = 0; k < 4; ++k)
    if ((rc = phase_in(g, io[k], k))) return rc;
  if ((rc = adj_project(g, g->phase, g->phase + g->dn, g->phase + 2 * g->dn, g->phase + 3 * g->dn)))
    return rc;
  for (int k = 0; k < 4; ++k)
    if ((rc = phase_out(g, io[k], k))) return rc;
  return phase_end(g);
}

}  // extern "C"
