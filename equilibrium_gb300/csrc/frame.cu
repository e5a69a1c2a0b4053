// Host side of the frame's surroundings (include/eqfluid.h, "around the
// step"): the rendered image, the seeded noise impulse, device obstacle
// rasterisation and the graph-captured frame loop. Compiled in the same
// translation unit as eqfluid.cu (it drives the plain handle's step).
#include "frame.cuh"

namespace {

// Improved gradient noise (Perlin 2002, a published algorithm) at (x, y),
// in [-1, 1], with a fixed permutation drawn by SplitMix64 Fisher-Yates.
double gradient_noise_2d(double x, double y) {
  static int perm[512];
  static bool ready = false;
  if (!ready) {
    int p[256];
    for (int k = 0; k < 256; ++k) p[k] = k;
    uint64_t s = 0x5eed0001ull;
    for (int k = 255; k > 0; --k) {
      s += 0x9e3779b97f4a7c15ull;
      uint64_t z = s;
      z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
      z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
      z ^= z >> 31;
      const int r = (int)(z % (uint64_t)(k + 1));
      std::swap(p[k], p[r]);
    }
    for (int k = 0; k < 512; ++k) perm[k] = p[k & 255];
    ready = true;
  }
  auto fade = [](double t) { return t * t * t * (t * (t * 6.0 - 15.0) + 10.0); };
  auto grad = [](int h, double dx, double dy) {
    return ((h & 1) ? -dx : dx) + ((h & 2) ? -dy : dy);
  };
  const double fx = std::floor(x), fy = std::floor(y);
  const int xi = (int)fx & 255, yi = (int)fy & 255;
  const double xf = x - fx, yf = y - fy;
  const double u = fade(xf), v = fade(yf);
  const int aa = perm[perm[xi] + yi], ab = perm[perm[xi] + yi + 1];
  const int ba = perm[perm[xi + 1] + yi], bb = perm[perm[xi + 1] + yi + 1];
  const double x1 = grad(aa, xf, yf) + u * (grad(ba, xf - 1.0, yf) - grad(aa, xf, yf));
  const double x2 = grad(ab, xf, yf - 1.0) + u * (grad(bb, xf - 1.0, yf - 1.0) - grad(ab, xf, yf - 1.0));
  return x1 + v * (x2 - x1);
}

uchar4 rgba(const uint8_t* c) { return make_uchar4(c[0], c[1], c[2], c[3]); }

int launch_noise(eq_fluid* h, uint64_t seed) {
  if (!h->noise_counter) {
    if (cudaMalloc(&h->noise_counter, sizeof(unsigned long long)) != cudaSuccess)
      return fail(EQ_ERR_OOM, "cudaMalloc (noise counter)");
    EQ_CUDA(cudaMemsetAsync(h->noise_counter, 0, sizeof(unsigned long long), h->stream));
  }
  const float angle = (float)(gradient_noise_2d(h->dt, h->dt) * 6.28 * 2.0);
  eqk::k_add_noise<<<1, 1, 0, h->stream>>>(h->field[EQ_FIELD_VX], h->field[EQ_FIELD_VY],
                                           (int)h->S, h->P, angle, seed, h->noise_counter);
  return check_launch(h);
}

void drop_step_graph(eq_fluid* h) {
  if (h->gexec) cudaGraphExecDestroy(h->gexec);
  if (h->graph) cudaGraphDestroy(h->graph);
  h->gexec = nullptr;
  h->graph = nullptr;
  h->gframes = -1;
}

}  // namespace

extern "C" {

double eq_noise_angle(float delta_t) {
  return gradient_noise_2d(delta_t, delta_t) * 6.28 * 2.0;
}

int eq_fluid_add_noise(eq_fluid* h, uint64_t seed) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  int rc = select_device(h);
  if (rc) return rc;
  return launch_noise(h, seed);
}

int eq_fluid_render_rgba_device(eq_fluid* h, const eq_render_colors* colors, void* d_rgba) {
  if (!h || !d_rgba) return fail(EQ_ERR_ARG, "null argument");
  int rc;
  if ((rc = select_device(h)) || (rc = upload_mask(h))) return rc;
  eq_render_colors c = colors ? *colors : eq_render_colors{{208, 88, 157, 220}, {94, 146, 162, 128}, {255, 0, 0, 255}};
  const int S = (int)h->S;
  const dim3 blk(32, 8), grd((S + 31) / 32, (S + 7) / 8);
  eqk::k_colormap<<<grd, blk, 0, h->stream>>>(h->field[EQ_FIELD_DENSITY], h->cells, S, h->P,
                                              rgba(c.fluid), rgba(c.world), rgba(c.obstacles),
                                              static_cast<uchar4*>(d_rgba));
  return check_launch(h);
}

int eq_fluid_render_rgba(eq_fluid* h, const eq_render_colors* colors, uint8_t* host_rgba,
                         uint64_t nbytes) {
  if (!h || !host_rgba) return fail(EQ_ERR_ARG, "null argument");
  if (nbytes != (uint64_t)h->S * h->S * 4) return fail(EQ_ERR_ARG, "nbytes must be size*size*4");
  int rc = select_device(h);
  if (rc) return rc;
  if (!h->rgba) {
    if (cudaMalloc(&h->rgba, nbytes) != cudaSuccess) return fail(EQ_ERR_OOM, "cudaMalloc (image)");
  }
  if ((rc = eq_fluid_render_rgba_device(h, colors, h->rgba))) return rc;
  EQ_CUDA(cudaMemcpyAsync(host_rgba, h->rgba, nbytes, cudaMemcpyDeviceToHost, h->stream));
  EQ_CUDA(cudaStreamSynchronize(h->stream));
  return read_err_word(h);
}

int eq_fluid_fill_obstacle_device(eq_fluid* h, int64_t x0, int64_t y0, int64_t x1, int64_t y1) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  int rc;
  if ((rc = select_device(h)) || (rc = upload_mask(h))) return rc;  // pending host edits first
  if (x0 >= x1 || y0 >= y1) return EQ_OK;  // the reference's loops run zero times
  const int64_t S = h->S;
  auto cl = [&](int64_t v) { return v < 0 ? 0 : (v > S - 1 ? S - 1 : v); };
  const int bx0 = (int)cl(x0), bx1 = (int)cl(x1 - 1), by0 = (int)cl(y0), by1 = (int)cl(y1 - 1);
  for (int y = by0; y <= by1; ++y)  // keep the host mirror of cells_type current
    for (int x = bx0; x <= bx1; ++x) h->host_cells[(size_t)y * S + x] = 1;
  const dim3 blk(32, 8);
  eqk::k_fill_rect<<<dim3((bx1 - bx0 + 32) / 32, (by1 - by0 + 8) / 8), blk, 0, h->stream>>>(
      h->cells, h->P, bx0, by0, bx1, by1);
  if ((rc = check_launch(h))) return rc;
  EQ_CUDA(cudaMemsetAsync(h->rowfl, 0, S, h->stream));
  EQ_CUDA(cudaMemsetAsync(h->colfl, 0, S, h->stream));
  const dim3 g((int)(S + 31) / 32, (int)(S + 7) / 8);
  eqk::k_fluid_flags<<<g, blk, 0, h->stream>>>(h->cells, (int)S, h->P, h->rowfl, h->colfl);
  eqk::k_derive_codes<<<g, blk, 0, h->stream>>>(h->cells, (int)S, h->P, h->colfl, h->code);
  if ((rc = check_launch(h))) return rc;
  h->mask_dirty = false;
  drop_step_graph(h);
  return EQ_OK;
}

int eq_fluid_step_graph(eq_fluid* h, int64_t nframes, int32_t with_noise, uint64_t seed) {
  if (!h) return fail(EQ_ERR_ARG, "null handle");
  if (nframes < 0) return fail(EQ_ERR_ARG, "nframes must be >= 0");
  if (nframes == 0) return EQ_OK;
  int rc;
  if ((rc = select_device(h)) || (rc = upload_mask(h))) return rc;
  if (with_noise && !h->noise_counter) {
    if (cudaMalloc(&h->noise_counter, sizeof(unsigned long long)) != cudaSuccess)
      return fail(EQ_ERR_OOM, "cudaMalloc (noise counter)");
    EQ_CUDA(cudaMemsetAsync(h->noise_counter, 0, sizeof(unsigned long long), h->stream));
  }
  const bool same = h->gexec && h->gframes == nframes && h->gnoise == (with_noise != 0) &&
                    h->gseed == seed && h->gdt == h->dt && h->gdiff == h->diff &&
                    h->gvisc == h->visc && h->gK == h->frames;
  if (!same) {
    drop_step_graph(h);
    const bool prof = h->profiling;
    h->profiling = false;  // no timing events inside a graph
    h->graph_mode = true;  // each lin_solve clears its tagged buffers
    const uint64_t l0 = h->launches;
    EQ_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    rc = EQ_OK;
    for (int64_t f = 0; f < nframes && !rc; ++f) {
      if (with_noise) rc = launch_noise(h, seed);
      if (!rc) rc = launch_step(h);
    }
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    h->graph_mode = false;
    h->profiling = prof;
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return fail(EQ_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
    h->graph = g;
    EQ_CUDA(cudaGraphInstantiate(&h->gexec, h->graph, 0));
    h->gframes = nframes;
    h->gnoise = with_noise != 0;
    h->gseed = seed;
    h->gdt = h->dt;
    h->gdiff = h->diff;
    h->gvisc = h->visc;
    h->gK = h->frames;
    h->glaunches = h->launches - l0;  // captured, not yet executed
    h->launches = l0;
  }
  EQ_CUDA(cudaGraphLaunch(h->gexec, h->stream));
  h->launches += h->glaunches;
  return EQ_OK;
}

}  // extern "C"
