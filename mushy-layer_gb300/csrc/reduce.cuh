// reduce.cuh -- deterministic block reductions for the fused residual norms.
// Each block writes one partial (FP64) to a scratch slot; a single-block
// finalize kernel combines the partials in a fixed order, so the same input
// always gives the same bits.
#pragma once
#include "common.cuh"

namespace mlgpu {

constexpr int kBlock = 256;

template <int NORM>
__device__ __forceinline__ double norm_accum(double acc, double v) {
  if (NORM == MLGPU_NORM_MAX) {
    double a = fabs(v);
    // keep NaN sticky: fmax would drop it
    return (a > acc || a != a) ? a : acc;
  } else if (NORM == MLGPU_NORM_L1) {
    return acc + fabs(v);
  } else {
    return acc + v * v;
  }
}

template <int NORM>
__device__ __forceinline__ double norm_combine(double a, double b) {
  if (NORM == MLGPU_NORM_MAX) return (b > a || b != b) ? b : a;
  return a + b;
}

// Block-wide reduction; result valid in thread 0.
template <int NORM>
__device__ __forceinline__ double block_reduce(double v) {
  __shared__ double warp_part[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = norm_combine<NORM>(v, __shfl_down_sync(0xffffffffu, v, o));
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) warp_part[w] = v;
  __syncthreads();
  int nw = (blockDim.x + 31) >> 5;
  if (w == 0) {
    v = lane < nw ? warp_part[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = norm_combine<NORM>(v, __shfl_down_sync(0xffffffffu, v, o));
  }
  return v;
}

// Combine `n` partials into out[0] (norm finished: sqrt for L2).
template <int NORM>
__global__ void finalize_norm_kernel(const double *__restrict__ part, int n,
                                     double *__restrict__ out) {
  double acc = 0.0;
  for (int q = threadIdx.x; q < n; q += blockDim.x) acc = norm_combine<NORM>(acc, part[q]);
  acc = block_reduce<NORM>(acc);
  if (threadIdx.x == 0) out[0] = (NORM == MLGPU_NORM_L2) ? sqrt(acc) : acc;
}

}  // namespace mlgpu
