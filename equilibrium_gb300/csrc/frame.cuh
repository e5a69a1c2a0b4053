// The code either side of the hot path: the frame's image (render_image,
// renderer_helpers.rs:115-180), the seeded noise impulse (add_noise,
// fluid.rs:575-599) and obstacle rasterisation with the boundary codes
// derived on the device (fill_obstacle, fluid.rs:610-619).
#pragma once
#include "common.cuh"

namespace eqk {

// Rust's saturating `f32 as u8`: NaN -> 0, below 0 -> 0, above 255 -> 255,
// otherwise truncation toward zero.
__device__ __forceinline__ uint8_t rust_as_u8(float v) {
  if (!(v == v) || v <= 0.0f) return 0;
  if (v >= 255.0f) return 255;
  return (uint8_t)v;
}

// render_image's per-pixel rule: walls in the obstacles colour; a fluid cell
// with non-zero density as ((density * fluid.r) as u8, fluid.g, density as
// u8, 1); everything else in the world colour. RGBA8, x fastest.
__global__ void k_colormap(const float* __restrict__ density, const uint8_t* __restrict__ cells,
                           int S, int P, uchar4 fluid, uchar4 world, uchar4 obstacles,
                           uchar4* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= S || y >= S) return;
  const size_t q = (size_t)y * P + x;
  const float d = density[q];
  uchar4 px;
  if (cells[q]) {
    px = obstacles;
  } else if (d != 0.0f) {
    px = make_uchar4(rust_as_u8(fmul(d, (float)fluid.x)), fluid.y, rust_as_u8(d), 1);
  } else {
    px = world;
  }
  out[(size_t)y * S + x] = px;
}

// SplitMix64 (a published counter-based generator): the noise impulse's cell.
__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// add_noise: a velocity impulse at the centre cell whose value is twice the
// point (rx, ry) rotated about the centre by `angle_deg` degrees (geo's
// rotate_around_point), (rx, ry) uniform over the grid from (seed, frame
// counter). The angle depends only on delta_t and is computed once by the
// host. One thread; the counter advances every call (graph-replay safe).
__global__ void k_add_noise(float* __restrict__ vx, float* __restrict__ vy, int S, int P,
                            float angle_deg, uint64_t seed, unsigned long long* counter) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const unsigned long long frame = (*counter)++;
  const uint64_t r = splitmix64(seed ^ splitmix64(frame));
  const int rx = (int)((r & 0xffffffffull) % (uint64_t)S);
  const int ry = (int)((r >> 32) % (uint64_t)S);
  const float c = (float)(S / 2);
  float sn, cs;
  sincosf(angle_deg * 0.017453292519943295f, &sn, &cs);
  const float ox = (float)rx - c, oy = (float)ry - c;
  const float px = c + (ox * cs - oy * sn);
  const float py = c + (ox * sn + oy * cs);
  const size_t q = (size_t)(S / 2) * P + (S / 2);
  vx[q] = fadd(vx[q], fmul(px, 2.0f));
  vy[q] = fadd(vy[q], fmul(py, 2.0f));
}

// fill_obstacle on the device mask: every (clamp(x), clamp(y)) for x in
// [x0, x1), y in [y0, y1) becomes DefaultWall; that is the clamped box.
__global__ void k_fill_rect(uint8_t* __restrict__ cells, int P, int bx0, int by0, int bx1,
                            int by1) {
  const int x = bx0 + blockIdx.x * blockDim.x + threadIdx.x;
  const int y = by0 + blockIdx.y * blockDim.y + threadIdx.y;
  if (x > bx1 || y > by1) return;
  cells[(size_t)y * P + x] = 1;
}

// Row / column "has a fluid cell" flags (Passive frame rule) from the mask.
__global__ void k_fluid_flags(const uint8_t* __restrict__ cells, int S, int P,
                              uint8_t* __restrict__ rowfl, uint8_t* __restrict__ colfl) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > S - 2 || j > S - 2) return;
  if (!cells[(size_t)j * P + i]) {
    rowfl[j] = 1;  // every writer stores the same value
    colfl[i] = 1;
  }
}

// The per-cell boundary codes (see common.cuh) from the mask and the flags:
// the device form of the host derivation.
__global__ void k_derive_codes(const uint8_t* __restrict__ cells, int S, int P,
                               const uint8_t* __restrict__ colfl, uint8_t* __restrict__ code) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= S || j >= S) return;
  const int N = S - 2;
  auto wall = [&](int a, int b) { return cells[(size_t)b * P + a] != 0; };
  uint8_t c = 0;
  const bool w = wall(i, j);
  if (w) c |= kCodeWall;
  if (!w && i >= 1 && i <= N && j >= 1 && j <= N) {
    if (wall(i + 1, j))
      c |= kCodeRowRight;
    else if (wall(i - 1, j))
      c |= kCodeRowLeft;
    if (wall(i, j - 1))
      c |= kCodeColUp;
    else if (wall(i, j + 1))
      c |= kCodeColDown;
  }
  if (j >= 2 && j - 1 <= N && i >= 1 && i <= N && w && !wall(i, j - 1) && !wall(i, j - 2))
    c |= kCodeAboveDown;
  if (colfl[i]) c |= kCodeColFluid;
  code[(size_t)j * P + i] = c;
}

}  // namespace eqk
