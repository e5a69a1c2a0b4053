// Storage formats of a field: FP32 (the reference's), FP16 or BF16. Values
// are widened to FP32 on load and rounded (to nearest, ties to even) once on
// store; FP32 storage loads and stores unchanged, so FP32 code paths written
// with these helpers stay bit-identical to plain loads and stores.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

namespace eqk {

template <class ST>
struct Store;
template <>
struct Store<float> {
  static __device__ __forceinline__ float ld(const float* p) { return *p; }
  static __device__ __forceinline__ void st(float* p, float v) { *p = v; }
};
template <>
struct Store<__half> {
  static __device__ __forceinline__ float ld(const __half* p) { return __half2float(*p); }
  static __device__ __forceinline__ void st(__half* p, float v) { *p = __float2half_rn(v); }
};
template <>
struct Store<__nv_bfloat16> {
  static __device__ __forceinline__ float ld(const __nv_bfloat16* p) {
    return __bfloat162float(*p);
  }
  static __device__ __forceinline__ void st(__nv_bfloat16* p, float v) {
    *p = __float2bfloat16_rn(v);
  }
};

template <class ST>
__device__ __forceinline__ float hl(const ST* p, size_t q) {
  return Store<ST>::ld(p + q);
}
template <class ST>
__device__ __forceinline__ void hs(ST* p, size_t q, float v) {
  Store<ST>::st(p + q, v);
}

}  // namespace eqk
