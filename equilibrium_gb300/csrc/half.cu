// Host side of the precision form (include/eqfluid.h, "half-storage fluid").
// Compiled in the same translation unit as eqfluid.cu: the diffusion solves
// reuse the plain handle's lin_solve wavefront on FP32 staging grids (the
// reference's lexicographic Gauss-Seidel, 20 sweeps in FP32 arithmetic), the
// pressure solves run mixed-precision refinement (mg.cuh).
#include "mg.cuh"

struct eq_hfluid {
  eq_fluid* plain = nullptr;  // stream, mask, codes, lin_solve state, FP32 staging grids
  int storage = EQ_STORE_F16;
  void* f[6] = {};            // stored fields (2 bytes per cell), pitched like the plain grids
  void* fblock = nullptr;
  float* p32 = nullptr;       // pressure (FP32, pitched, with ghosts)
  float* plo = nullptr;       // its low-order part during refinement (p = p32 + plo)
  float* b32 = nullptr;       // right-hand side: project's div (FP32)
  float* r32 = nullptr;       // fine residual (FP32)
  double* d_acc = nullptr;    // FP64 reduction slots
  double* h_acc = nullptr;    // pinned
  struct Level {
    int n, pitch;
    void* e;  // FP32 correction
    void* r;  // right-hand side in the storage format (scaled by 4^-level)
  };
  std::vector<Level> lv;
  void* lvblock = nullptr;
  double rtol = 1e-5;
  int max_ir = 30;
  eq_hstats stats{};
  std::vector<uint32_t> sx, sy;
  std::vector<float> sd, su, sv;
  uint8_t* d_src = nullptr;
  size_t d_src_cap = 0;
};

namespace {

dim3 h_grid(int nx, int ny) { return dim3((nx + 31) / 32, (ny + 7) / 8); }
const dim3 kHBlk(32, 8);

int h_check(eq_hfluid* h) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  EQ_CUDA(cudaSetDevice(h->plain->device));
  return EQ_OK;
}

void hfree(eq_hfluid* h) {
  if (!h) return;
  if (h->plain) {
    cudaSetDevice(h->plain->device);
    cudaStreamSynchronize(h->plain->stream);
  }
  cudaFree(h->fblock);
  cudaFree(h->p32);
  cudaFree(h->plo);
  cudaFree(h->b32);
  cudaFree(h->r32);
  cudaFree(h->d_acc);
  cudaFree(h->lvblock);
  cudaFree(h->d_src);
  if (h->h_acc) cudaFreeHost(h->h_acc);
  free_handle(h->plain);
  delete h;
}

template <class T>
int h_bnd(eq_hfluid* h, int mode, T* x) {
  eq_fluid* pl = h->plain;
  const int S = (int)pl->S;
  const dim3 g = h_grid(S, S);
  if (mode == eqk::kRow)
    eqk::k_h_bnd<eqk::kRow, T><<<g, kHBlk, 0, pl->stream>>>(x, pl->code, pl->rowfl, pl->colfl, S, pl->P);
  else if (mode == eqk::kCol)
    eqk::k_h_bnd<eqk::kCol, T><<<g, kHBlk, 0, pl->stream>>>(x, pl->code, pl->rowfl, pl->colfl, S, pl->P);
  else
    eqk::k_h_bnd<eqk::kPassive, T><<<g, kHBlk, 0, pl->stream>>>(x, pl->code, pl->rowfl, pl->colfl, S, pl->P);
  return check_launch(pl);
}

int h_blocks(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 152 * 8); }

// diffuse (fluid.rs:276-298): the stored x (initial guess) and x0 widened
// into two of the plain handle's FP32 grids (2 stage and 2 stage + 1: one
// pair per diffusion that may run at the same time), the reference's
// lin_solve there on the plain handle's current stream, x narrowed back.
template <class T>
int h_diffuse(eq_hfluid* h, int mode, T* x, const T* x0, float diffusion, int stage = 0) {
  eq_fluid* pl = h->plain;
  const size_t n = pl->grid_elems();
  float* xs = pl->field[2 * stage];
  float* x0s = pl->field[2 * stage + 1];
  cudaStream_t st = pl->cur;
  eqk::k_h_widen<T><<<h_blocks(n), 256, 0, st>>>(xs, x, n);
  eqk::k_h_widen<T><<<h_blocks(n), 256, 0, st>>>(x0s, x0, n);
  int rc = check_launch(pl);
  if (rc) return rc;
  if ((rc = launch_diffuse(pl, mode, xs, x0s, diffusion))) return rc;
  eqk::k_h_narrow<T><<<h_blocks(n), 256, 0, st>>>(x, xs, n);
  return check_launch(pl);
}

template <class T>
void h_vcycle(eq_hfluid* h, size_t l) {
  cudaStream_t st = h->plain->stream;
  const auto& L = h->lv[l];
  float* e = static_cast<float*>(L.e);
  T* r = static_cast<T*>(L.r);
  const float s4 = std::ldexp(1.0f, 2 * (int)l);  // 4^l
  if (l + 1 == h->lv.size()) {
    h->plain->launches += 1;
    eqk::k_mg_coarse<T><<<1, 1024, 0, st>>>(e, r, L.n, L.pitch, s4, 64);
    return;
  }
  if (L.n <= 64 && h->lv.size() - l <= (size_t)eqk::kMgMaxLevels) {
    // this level and the coarser ones in one block
    eqk::MgLevels V;
    V.count = (int)(h->lv.size() - l);
    V.l0 = (int)l;
    for (int k = 0; k < V.count; ++k) {
      V.n[k] = h->lv[l + k].n;
      V.pitch[k] = h->lv[l + k].pitch;
      V.e[k] = static_cast<float*>(h->lv[l + k].e);
      V.r[k] = h->lv[l + k].r;
    }
    h->plain->launches += 1;
    eqk::k_mg_vcycle_small<T><<<1, 1024, 0, st>>>(V);
    return;
  }
  h->plain->launches += 10;
  const dim3 gs = h_grid((L.n + 1) / 2, L.n);
  for (int s = 0; s < 2; ++s) {
    eqk::k_mg_smooth<T><<<gs, kHBlk, 0, st>>>(e, r, L.n, L.pitch, 0, s4);
    eqk::k_mg_smooth<T><<<gs, kHBlk, 0, st>>>(e, r, L.n, L.pitch, 1, s4);
  }
  const auto& C = h->lv[l + 1];
  eqk::k_mg_restrict<T><<<h_grid(C.n, C.n), kHBlk, 0, st>>>(
      e, r, L.n, L.pitch, s4, static_cast<T*>(C.r), static_cast<float*>(C.e), C.n, C.pitch);
  h_vcycle<T>(h, l + 1);
  eqk::k_mg_prolong<<<h_grid(L.n, L.n), kHBlk, 0, st>>>(e, L.n, L.pitch,
                                                       static_cast<const float*>(C.e), C.n,
                                                       C.pitch);
  for (int s = 0; s < 2; ++s) {
    eqk::k_mg_smooth<T><<<gs, kHBlk, 0, st>>>(e, r, L.n, L.pitch, 1, s4);
    eqk::k_mg_smooth<T><<<gs, kHBlk, 0, st>>>(e, r, L.n, L.pitch, 0, s4);
  }
}

// project (fluid.rs:330-375) with the pressure solved by mixed-precision
// refinement; p and div are the stored arrays the reference aliases.
template <class T>
int h_project(eq_hfluid* h, int which, T* vx, T* vy, T* ps, T* divs) {
  eq_fluid* pl = h->plain;
  cudaStream_t st = pl->stream;
  const int S = (int)pl->S, P = pl->P, N = S - 2;
  const size_t n = pl->grid_elems();
  int rc;
  // pre-projection divergence (statistics)
  EQ_CUDA(cudaMemsetAsync(h->d_acc, 0, 4 * sizeof(double), st));
  eqk::k_h_div_norm<T><<<h_blocks((size_t)N * N), 256, 0, st>>>(vx, vy, S, P, h->d_acc + 2);
  eqk::k_h_divergence<T><<<h_grid(N, N), kHBlk, 0, st>>>(vx, vy, h->b32, divs, S, P);
  if ((rc = check_launch(pl))) return rc;
  if ((rc = h_bnd<T>(h, eqk::kPassive, divs))) return rc;
  // p: the stored array's values (its frame is the Dirichlet value where a
  // row / column has no fluid cell), interior zeroed
  eqk::k_h_widen<T><<<h_blocks(n), 256, 0, st>>>(h->p32, ps, n);
  eqk::k_ir_zero<<<h_grid(N, N), kHBlk, 0, st>>>(h->p32, h->plo, S, P);
  if ((rc = check_launch(pl))) return rc;
  const auto& L0 = h->lv[0];
  double bnorm = 0.0, rel = 0.0, prev = 0.0;
  int it = 0, slow = 0;
  for (;; ++it) {
    EQ_CUDA(cudaMemsetAsync(h->d_acc, 0, 2 * sizeof(double), st));
    eqk::k_ir_residual<<<h_blocks((size_t)N * N), 256, 0, st>>>(
        h->p32, h->plo, h->b32, S, P, pl->rowfl, pl->colfl, h->r32, h->d_acc);
    if ((rc = check_launch(pl))) return rc;
    EQ_CUDA(cudaMemcpyAsync(h->h_acc, h->d_acc, 4 * sizeof(double), cudaMemcpyDeviceToHost, st));
    EQ_CUDA(cudaStreamSynchronize(st));
    const double cnt = (double)N * N;
    const double mean = h->h_acc[0] / cnt;
    const double rn = std::sqrt(std::max(0.0, h->h_acc[1] - cnt * mean * mean));
    if (it == 0) {
      bnorm = rn;
      h->stats.div_norm_before[which] = std::sqrt(h->h_acc[2]);
    }
    rel = bnorm > 0.0 ? rn / bnorm : 0.0;
    if (rel <= h->rtol || it >= h->max_ir || rn == 0.0) break;
    // The pressure is held as p32 + plo (FP32 pairs) and the residual and
    // the update are computed in FP64, so the residual floor is far below
    // rtol; still stop once two rounds in a row gain less than a factor 2.
    if (it > 0) slow = (rel > 0.5 * prev) ? slow + 1 : 0;
    if (slow >= 2) break;
    prev = rel;
    const double scale = rn / std::sqrt(cnt);
    eqk::k_ir_scale<T><<<h_grid(N, N), kHBlk, 0, st>>>(h->r32, S, P, (float)mean,
                                                       (float)(1.0 / scale),
                                                       static_cast<T*>(L0.r), L0.pitch);
    EQ_CUDA(cudaMemsetAsync(L0.e, 0, (size_t)L0.pitch * L0.n * sizeof(float), st));
    h_vcycle<T>(h, 0);
    float sh, sl;
    eqk::df_split(scale, &sh, &sl);
    eqk::k_ir_update<<<h_grid(N, N), kHBlk, 0, st>>>(h->p32, h->plo, S, P,
                                                     static_cast<const float*>(L0.e), L0.pitch,
                                                     sh, sl);
    if ((rc = check_launch(pl))) return rc;
  }
  h->stats.ir_iterations[which] = it;
  h->stats.rel_residual[which] = rel;
  // zero-mean pressure where every frame neighbour is a Neumann copy (the
  // operator's null space; a Dirichlet frame would fix the constant itself)
  {
    bool neumann = true;
    const std::vector<uint8_t>& m = pl->host_cells;
    for (int k = 1; k <= N && neumann; ++k) {
      bool rf = false, cf = false;
      for (int q = 1; q <= N; ++q) {
        rf = rf || !m[(size_t)k * S + q];
        cf = cf || !m[(size_t)q * S + k];
      }
      neumann = rf && cf;
    }
    if (neumann) {
      EQ_CUDA(cudaMemsetAsync(h->d_acc, 0, 2 * sizeof(double), st));
      eqk::k_ir_sum<<<h_blocks((size_t)N * N), 256, 0, st>>>(h->p32, h->plo, S, P, h->d_acc);
      eqk::k_ir_center<<<h_grid(N, N), kHBlk, 0, st>>>(h->p32, h->plo, S, P, h->d_acc);
      if ((rc = check_launch(pl))) return rc;
    }
  }
  // p's frame by set_boundaries(Passive) (+ corners), stored into p's array
  eqk::k_set_boundaries<eqk::kPassive><<<h_grid(S, S), kHBlk, 0, st>>>(h->p32, pl->code, pl->rowfl,
                                                                      pl->colfl, S, P);
  eqk::k_h_narrow<T><<<h_blocks(n), 256, 0, st>>>(ps, h->p32, n);
  eqk::k_h_gradient<T><<<h_grid(N, N), kHBlk, 0, st>>>(vx, vy, h->p32, S, P);
  if ((rc = check_launch(pl))) return rc;
  if ((rc = h_bnd<T>(h, eqk::kRow, vx)) || (rc = h_bnd<T>(h, eqk::kCol, vy))) return rc;
  EQ_CUDA(cudaMemsetAsync(h->d_acc + 3, 0, sizeof(double), st));
  eqk::k_h_div_norm<T><<<h_blocks((size_t)N * N), 256, 0, st>>>(vx, vy, S, P, h->d_acc + 3);
  EQ_CUDA(cudaMemcpyAsync(h->h_acc + 3, h->d_acc + 3, sizeof(double), cudaMemcpyDeviceToHost, st));
  EQ_CUDA(cudaStreamSynchronize(st));
  h->stats.div_norm[which] = std::sqrt(h->h_acc[3]);
  return check_launch(pl);
}

template <class T, class TU>
int h_advect(eq_hfluid* h, int mode, T* d, const T* d0, const TU* u, const TU* v) {
  eq_fluid* pl = h->plain;
  const int S = (int)pl->S, N = S - 2;
  const float dt0 = pl->dt * (float)(S - 2);
  const int threads = std::min(256, ((N + 31) / 32) * 32);
  eqk::k_h_advect_rows<T, TU><<<N, threads, 0, pl->stream>>>(d, d0, u, v, S, pl->P, dt0);
  int rc = check_launch(pl);
  if (rc) return rc;
  return h_bnd<T>(h, mode, d);
}

// One frame with density and scratch stored in TS, the four velocity arrays
// (which project also uses for its pressure and divergence) in TV.
template <class TS, class TV>
int h_step(eq_hfluid* h) {
  eq_fluid* pl = h->plain;
  int rc = upload_mask(pl);
  if (rc) return rc;
  TS* sc = static_cast<TS*>(h->f[EQ_FIELD_SCRATCH]);
  TS* de = static_cast<TS*>(h->f[EQ_FIELD_DENSITY]);
  TV* vx = static_cast<TV*>(h->f[EQ_FIELD_VX]);
  TV* vy = static_cast<TV*>(h->f[EQ_FIELD_VY]);
  TV* vx0 = static_cast<TV*>(h->f[EQ_FIELD_VX0]);
  TV* vy0 = static_cast<TV*>(h->f[EQ_FIELD_VY0]);
  const int64_t ns = (int64_t)h->sx.size();
  if (ns > 0) {
    const size_t bytes = (size_t)ns * 20;
    if (bytes > h->d_src_cap) {
      EQ_CUDA(cudaStreamSynchronize(pl->stream));
      cudaFree(h->d_src);
      h->d_src = nullptr;
      h->d_src_cap = 0;
      if (cudaMalloc(&h->d_src, bytes) != cudaSuccess) return fail(EQ_ERR_OOM, "cudaMalloc (sources)");
      h->d_src_cap = bytes;
    }
    std::vector<uint8_t> buf(bytes);
    std::memcpy(buf.data(), h->sx.data(), ns * 4);
    std::memcpy(buf.data() + ns * 4, h->sy.data(), ns * 4);
    std::memcpy(buf.data() + ns * 8, h->sd.data(), ns * 4);
    std::memcpy(buf.data() + ns * 12, h->su.data(), ns * 4);
    std::memcpy(buf.data() + ns * 16, h->sv.data(), ns * 4);
    EQ_CUDA(cudaMemcpyAsync(h->d_src, buf.data(), bytes, cudaMemcpyHostToDevice, pl->stream));
    const uint32_t* dx = reinterpret_cast<const uint32_t*>(h->d_src);
    const float* dv = reinterpret_cast<const float*>(h->d_src + ns * 8);
    eqk::k_h_sources<TS, TV><<<1, 1, 0, pl->stream>>>(de, sc, vx, vy, (int)pl->S, pl->P, ns, dx,
                                                 dx + ns, dv, dv + ns, dv + 2 * ns);
    if ((rc = check_launch(pl))) return rc;
    EQ_CUDA(cudaStreamSynchronize(pl->stream));  // the staging vector goes out of scope
    h->sx.clear();
    h->sy.clear();
    h->sd.clear();
    h->su.clear();
    h->sv.clear();
  }
  // The vy and the density diffusions run on the plain handle's side
  // streams as its concurrency mask says (their own staging grids and
  // wavefront state; joined before their results are read), the rest on
  // its stream in the reference's order.
  const bool sideVy = (pl->concurrent & EQ_CONC_VY) != 0;
  const bool sideDe = (pl->concurrent & EQ_CONC_DENSITY) != 0;
  auto on = [&](cudaStream_t st, int slot) {
    pl->cur = st;
    pl->cur_slot = slot;
  };
  auto side = [&](int k, int mode, auto* x, const auto* x0, float dif) -> int {
    EQ_CUDA(cudaStreamWaitEvent(pl->side[k], pl->fork_ev, 0));
    on(pl->side[k], k + 1);
    int r = h_diffuse(h, mode, x, x0, dif, k + 1);
    if (!r && cudaEventRecord(pl->join_ev[k], pl->side[k]) != cudaSuccess)
      r = fail(EQ_ERR_CUDA, "side stream event");
    on(pl->stream, 0);
    return r;
  };
  if (sideVy || sideDe) EQ_CUDA(cudaEventRecord(pl->fork_ev, pl->stream));
  if ((rc = h_diffuse<TV>(h, eqk::kRow, vx0, vx, pl->visc))) return rc;
  if (sideVy && (rc = side(0, eqk::kCol, vy0, vy, pl->visc))) return rc;
  if (sideDe && (rc = side(1, eqk::kPassive, sc, de, pl->diff))) return rc;
  if (sideVy)
    EQ_CUDA(cudaStreamWaitEvent(pl->stream, pl->join_ev[0], 0));
  else if ((rc = h_diffuse<TV>(h, eqk::kCol, vy0, vy, pl->visc)))
    return rc;
  if ((rc = h_project<TV>(h, 0, vx0, vy0, vx, vy))) return rc;
  if ((rc = h_advect<TV, TV>(h, eqk::kRow, vx, vx0, vx0, vy0))) return rc;
  if ((rc = h_advect<TV, TV>(h, eqk::kCol, vy, vy0, vx0, vy0))) return rc;
  if ((rc = h_project<TV>(h, 1, vx, vy, vx0, vy0))) return rc;
  if (sideDe)
    EQ_CUDA(cudaStreamWaitEvent(pl->stream, pl->join_ev[1], 0));
  else if ((rc = h_diffuse<TS>(h, eqk::kPassive, sc, de, pl->diff)))
    return rc;
  if ((rc = h_advect<TS, TV>(h, eqk::kPassive, de, sc, vx, vy))) return rc;
  const size_t n = pl->grid_elems();
  eqk::k_h_copy<TS><<<h_blocks(n), 256, 0, pl->stream>>>(sc, de, n);
  return check_launch(pl);
}

template <class TS, class TV>
int h_init(eq_hfluid* h) {
  eq_fluid* pl = h->plain;
  const int S = (int)pl->S;
  eqk::k_h_init<TS, TV><<<h_grid(S, S), kHBlk, 0, pl->stream>>>(
      static_cast<TS*>(h->f[0]), static_cast<TS*>(h->f[1]), static_cast<TV*>(h->f[2]),
      static_cast<TV*>(h->f[3]), S, pl->P);
  return check_launch(pl);
}

}  // namespace

extern "C" {

int eq_hfluid_new(const eq_fluid_configs* fluid, const eq_simulation_configs* sim, int storage,
                  double pressure_rtol, int32_t max_refinements, int device, eq_hfluid** out) {
  if (!fluid || !sim || !out) return fail(EQ_ERR_ARG, "null argument");
  *out = nullptr;
  if (storage != EQ_STORE_F16 && storage != EQ_STORE_BF16 && storage != EQ_STORE_F16_SCALARS)
    return fail(EQ_ERR_ARG,
                "storage must be EQ_STORE_F16, EQ_STORE_BF16 or EQ_STORE_F16_SCALARS");
  if (sim->size < 20) return fail(EQ_ERR_ARG, "size must be >= 20 (fluid.rs:534 underflows)");
  if (sim->size > 32768) return fail(EQ_ERR_ARG, "size too large");
  if (sim->frames < 0) return fail(EQ_ERR_ARG, "frames must be >= 0");
  if (!(pressure_rtol > 0.0) || max_refinements < 1)
    return fail(EQ_ERR_ARG, "pressure_rtol must be > 0 and max_refinements >= 1");
  eq_hfluid* h = new eq_hfluid();
  h->storage = storage;
  h->rtol = pressure_rtol;
  h->max_ir = max_refinements;
  int rc = alloc_handle(sim->size, device, &h->plain);
  if (rc) {
    delete h;
    return rc;
  }
  eq_fluid* pl = h->plain;
  pl->dt = sim->delta_t;
  pl->frames = sim->frames;
  pl->diff = fluid->diffusion;
  pl->visc = fluid->viscousity;
  pl->has_perlin_noise = fluid->has_perlin_noise;
  const uint32_t S = sim->size;
  for (uint32_t i = 0; i < S; ++i) {  // init_walls (fluid.rs:552-570)
    pl->host_cells[i] = pl->host_cells[(size_t)(S - 1) * S + i] = 1;
    pl->host_cells[(size_t)i * S] = pl->host_cells[(size_t)i * S + S - 1] = 1;
  }
  pl->mask_dirty = true;
  const size_t g = pl->grid_elems();
  auto bail = [&](int code, const char* what) {
    hfree(h);
    return fail(code, what);
  };
  const bool mixed = storage == EQ_STORE_F16_SCALARS;
  size_t fbytes = 0;  // scalars 2 bytes a cell; velocities 4 with FP32 velocity storage
  for (int q = 0; q < 6; ++q) fbytes += g * ((mixed && q >= 2) ? 4 : 2);
  if (cudaMalloc(&h->fblock, fbytes) != cudaSuccess ||
      cudaMalloc(&h->p32, g * 4) != cudaSuccess || cudaMalloc(&h->plo, g * 4) != cudaSuccess ||
      cudaMalloc(&h->b32, g * 4) != cudaSuccess ||
      cudaMalloc(&h->r32, g * 4) != cudaSuccess ||
      cudaMalloc(&h->d_acc, 4 * sizeof(double)) != cudaSuccess)
    return bail(EQ_ERR_OOM, "cudaMalloc (half fields)");
  if (cudaMallocHost(&h->h_acc, 4 * sizeof(double)) != cudaSuccess)
    return bail(EQ_ERR_OOM, "cudaMallocHost");
  {
    size_t off = 0;
    for (int q = 0; q < 6; ++q) {
      h->f[q] = static_cast<uint8_t*>(h->fblock) + off;
      off += g * ((mixed && q >= 2) ? 4 : 2);
    }
  }
  if (cudaMemsetAsync(h->fblock, 0, fbytes, pl->stream) != cudaSuccess ||
      cudaMemsetAsync(h->p32, 0, g * 4, pl->stream) != cudaSuccess ||
      cudaMemsetAsync(h->plo, 0, g * 4, pl->stream) != cudaSuccess ||
      cudaMemsetAsync(h->b32, 0, g * 4, pl->stream) != cudaSuccess ||
      cudaMemsetAsync(h->r32, 0, g * 4, pl->stream) != cudaSuccess)
    return bail(EQ_ERR_CUDA, "cudaMemsetAsync");
  // multigrid levels: n, ceil(n/2), ... down to <= 4 cells per side
  size_t bytes = 0;
  for (int n = (int)S - 2;; n = (n + 1) / 2) {
    eq_hfluid::Level L;
    L.n = n;
    L.pitch = ((n + 63) / 64) * 64;
    L.e = L.r = nullptr;
    h->lv.push_back(L);
    bytes += (size_t)L.pitch * n * (4 + (mixed ? 4 : 2));
    if (n <= 4) break;
  }
  if (cudaMalloc(&h->lvblock, bytes) != cudaSuccess) return bail(EQ_ERR_OOM, "cudaMalloc (levels)");
  EQ_CUDA(cudaMemsetAsync(h->lvblock, 0, bytes, pl->stream));
  uint8_t* base = static_cast<uint8_t*>(h->lvblock);
  for (auto& L : h->lv) {
    L.e = base;  // FP32 correction
    base += (size_t)L.pitch * L.n * 4;
    L.r = base;  // right-hand side in the velocity storage format
    base += (size_t)L.pitch * L.n * (mixed ? 4 : 2);
  }
  rc = storage == EQ_STORE_F16    ? h_init<__half, __half>(h)
       : storage == EQ_STORE_BF16 ? h_init<__nv_bfloat16, __nv_bfloat16>(h)
                                  : h_init<__half, float>(h);
  if (rc) {
    hfree(h);
    return rc;
  }
  if (cudaStreamSynchronize(pl->stream) != cudaSuccess) return bail(EQ_ERR_CUDA, "init");
  *out = h;
  return EQ_OK;
}

int eq_hfluid_free(eq_hfluid* h) {
  hfree(h);
  return EQ_OK;
}

int eq_hfluid_fill_obstacle(eq_hfluid* h, int64_t x0, int64_t y0, int64_t x1, int64_t y1) {
  int rc = h_check(h);
  if (rc) return rc;
  return eq_fluid_fill_obstacle(h->plain, x0, y0, x1, y1);
}

int eq_hfluid_add_sources(eq_hfluid* h, int64_t n, const uint32_t* x, const uint32_t* y,
                          const float* density, const float* vx, const float* vy) {
  int rc = h_check(h);
  if (rc) return rc;
  if (n < 0) return fail(EQ_ERR_ARG, "n must be >= 0");
  if (n > 0 && (!x || !y)) return fail(EQ_ERR_ARG, "null coordinates");
  for (int64_t s = 0; s < n; ++s) {
    h->sx.push_back(x[s]);
    h->sy.push_back(y[s]);
    h->sd.push_back(density ? density[s] : 0.0f);
    h->su.push_back(vx ? vx[s] : 0.0f);
    h->sv.push_back(vy ? vy[s] : 0.0f);
  }
  return EQ_OK;
}

int eq_hfluid_step(eq_hfluid* h) {
  int rc = h_check(h);
  if (rc) return rc;
  rc = h->storage == EQ_STORE_F16    ? h_step<__half, __half>(h)
       : h->storage == EQ_STORE_BF16 ? h_step<__nv_bfloat16, __nv_bfloat16>(h)
                                     : h_step<__half, float>(h);
  if (rc) return rc;
  return read_err_word(h->plain);
}

int eq_hfluid_synchronize(eq_hfluid* h) {
  int rc = h_check(h);
  if (rc) return rc;
  EQ_CUDA(cudaStreamSynchronize(h->plain->stream));
  return read_err_word(h->plain);
}

static int hfield_copy(eq_hfluid* h, int field, float* host, uint64_t n, bool to_host) {
  int rc = h_check(h);
  if (rc) return rc;
  if ((rc = check_field(field))) return rc;
  eq_fluid* pl = h->plain;
  if (n != (uint64_t)pl->S * pl->S) return fail(EQ_ERR_ARG, "element count must be size*size");
  if (!host) return fail(EQ_ERR_ARG, "null host buffer");
  const size_t g = pl->grid_elems();
  float* stage = pl->field[2];  // FP32 staging grid of the plain handle
  const size_t w = (size_t)pl->S * sizeof(float);
  const bool f32 = h->storage == EQ_STORE_F16_SCALARS && field >= 2;  // stored in FP32
  if (f32) {
    EQ_CUDA(cudaMemcpy2DAsync(to_host ? (void*)host : h->f[field], to_host ? w : (size_t)pl->P * 4,
                              to_host ? h->f[field] : (void*)host,
                              to_host ? (size_t)pl->P * 4 : w, w, pl->S,
                              to_host ? cudaMemcpyDeviceToHost : cudaMemcpyHostToDevice,
                              pl->stream));
  } else if (to_host) {
    if (h->storage != EQ_STORE_BF16)
      eqk::k_h_widen<__half><<<h_blocks(g), 256, 0, pl->stream>>>(stage, static_cast<__half*>(h->f[field]), g);
    else
      eqk::k_h_widen<__nv_bfloat16><<<h_blocks(g), 256, 0, pl->stream>>>(stage, static_cast<__nv_bfloat16*>(h->f[field]), g);
    if ((rc = check_launch(pl))) return rc;
    EQ_CUDA(cudaMemcpy2DAsync(host, w, stage, (size_t)pl->P * 4, w, pl->S, cudaMemcpyDeviceToHost,
                              pl->stream));
  } else {
    EQ_CUDA(cudaMemcpy2DAsync(stage, (size_t)pl->P * 4, host, w, w, pl->S, cudaMemcpyHostToDevice,
                              pl->stream));
    if (h->storage != EQ_STORE_BF16)
      eqk::k_h_narrow<__half><<<h_blocks(g), 256, 0, pl->stream>>>(static_cast<__half*>(h->f[field]), stage, g);
    else
      eqk::k_h_narrow<__nv_bfloat16><<<h_blocks(g), 256, 0, pl->stream>>>(static_cast<__nv_bfloat16*>(h->f[field]), stage, g);
    if ((rc = check_launch(pl))) return rc;
  }
  EQ_CUDA(cudaStreamSynchronize(pl->stream));
  return EQ_OK;
}

int eq_hfluid_read_field(eq_hfluid* h, int field, float* host, uint64_t n) {
  return hfield_copy(h, field, host, n, true);
}

int eq_hfluid_write_field(eq_hfluid* h, int field, const float* host, uint64_t n) {
  return hfield_copy(h, field, const_cast<float*>(host), n, false);
}

int eq_hfluid_stats(const eq_hfluid* h, eq_hstats* out) {
  if (!h || !out) return fail(EQ_ERR_ARG, "null argument");
  *out = h->stats;
  return EQ_OK;
}

int eq_hfluid_get_stream(eq_hfluid* h, void** stream) {
  if (!h || !stream) return fail(EQ_ERR_ARG, "null argument");
  *stream = (void*)h->plain->stream;
  return EQ_OK;
}

int eq_hfluid_launch_count(const eq_hfluid* h, uint64_t* count) {
  if (!h || !count) return fail(EQ_ERR_ARG, "null argument");
  *count = h->plain->launches;
  return EQ_OK;
}

int eq_hfluid_set_concurrency(eq_hfluid* h, int mask) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  return eq_fluid_set_concurrency(h->plain, mask);
}

int eq_hfluid_set_solver(eq_hfluid* h, int solver) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  return eq_fluid_set_solver(h->plain, solver);
}

}  // extern "C"
