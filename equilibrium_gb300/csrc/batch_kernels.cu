// Instances of the batched frame kernel k_batch_run (batch.cuh). The library
// build compiles this file once per storage format (EQ_BATCH_STORE: 0 FP32,
// 1 FP16, 2 BF16, 3 FP32 velocities with FP16 density / scratch) beside the
// main translation unit, which only declares these instances; the units
// build in parallel.
#define EQ_BATCH_KERNELS_TU
#include "batch.cuh"

#ifndef EQ_BATCH_STORE
#error "EQ_BATCH_STORE (0..3) must be defined"
#endif

namespace eqk {
#if EQ_BATCH_STORE == 0
template __global__ void k_batch_run<float, float>(BatchArgs, BOpList);
#elif EQ_BATCH_STORE == 1
template __global__ void k_batch_run<__half, __half>(BatchArgs, BOpList);
#elif EQ_BATCH_STORE == 2
template __global__ void k_batch_run<__nv_bfloat16, __nv_bfloat16>(BatchArgs, BOpList);
#else
template __global__ void k_batch_run<float, __half>(BatchArgs, BOpList);
#endif
}  // namespace eqk
