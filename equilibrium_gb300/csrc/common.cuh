// Shared device helpers for the sm_103a stable-fluids kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace eqk {

// Modes (fluid.rs:21-29).
enum : int { kRow = 0, kCol = 1, kPassive = 2 };

// Per-cell boundary code, derived from the wall mask once per mask change.
// set_boundaries (fluid.rs:133-189, 252-272) only ever WRITES fluid cells in
// the velocity modes and only READS wall cells, so it is a per-cell map:
//   AdjustRow:    right wall -> x = -x[i+1] (wins), else left wall -> -x[i-1]
//   AdjustColumn: up wall (j-1) -> x = -x[j-1] (wins), else down (j+1) -> -x[j+1]
enum : uint8_t {
  kCodeWall = 1u,        // DefaultWall
  kCodeRowLeft = 2u,     // AdjustRow takes -x[i-1, j]
  kCodeRowRight = 4u,    // AdjustRow takes -x[i+1, j]
  kCodeColDown = 8u,     // AdjustColumn takes -x[i, j+1]
  kCodeColUp = 16u,      // AdjustColumn takes -x[i, j-1]
  kCodeAboveDown = 32u,  // the cell (i, j-1) has kCodeColDown
  kCodeColFluid = 64u,   // column i holds a fluid cell (Passive frame rule)
};
constexpr uint8_t kCodeRowMask = kCodeRowLeft | kCodeRowRight;
constexpr uint8_t kCodeColMask = kCodeColDown | kCodeColUp;

// Explicitly rounded IEEE operations: never contracted into FMA whatever the
// compiler's --fmad setting, so results match the reference's f32 bit for bit.
// The FMA build (EQ_FMA, compiled with --fmad=true) uses plain operators
// instead, which the compiler may fuse into a*b+c with one rounding.
#if defined(EQ_FMA) && EQ_FMA
__device__ __forceinline__ float fadd(float a, float b) { return a + b; }
__device__ __forceinline__ float fsub(float a, float b) { return a - b; }
__device__ __forceinline__ float fmul(float a, float b) { return a * b; }
#else
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
#endif
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }

// Rust's f32::clamp (NaN passes through).
__device__ __forceinline__ float rust_clamp(float x, float lo, float hi) {
  if (x < lo) x = lo;
  if (x > hi) x = hi;
  return x;
}

// Rust's saturating `f32 as u32`, then idx!'s clamp into [0, S-1].
__device__ __forceinline__ int as_u32_clamped(float v, int S) {
  if (!(v == v)) return 0;
  if (v <= 0.0f) return 0;
  if (v >= (float)(S - 1)) return S - 1;
  return (int)v;  // truncation toward zero, v in (0, S-1)
}

// Memory-model helpers for the inter-block waits.
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ int ld_relaxed_i32(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned atom_add_acq_rel_u32(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;"
               : "=r"(old)
               : "l"(p), "r"(v)
               : "memory");
  return old;
}

// Asynchronous global -> shared copies (L2 only for the 16-byte form, so data
// another block released is read coherently after the acquire).
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, bool pred) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile(
      "{ .reg .pred p; setp.ne.b32 p, %2, 0; @p cp.async.cg.shared.global [%0], [%1], 16; }" ::"r"(s),
      "l"(gmem), "r"((int)pred)
      : "memory");
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem, bool pred) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile(
      "{ .reg .pred p; setp.ne.b32 p, %2, 0; @p cp.async.ca.shared.global [%0], [%1], 4; }" ::"r"(s),
      "l"(gmem), "r"((int)pred)
      : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

}  // namespace eqk
