// launch_f32.cu -- FP32 instantiations of the kernel launchers (inner
// multigrid cycles of the mixed-precision solvers).  FMA contraction is left
// on; the nonlinear closure inside these kernels still runs in FP64.  The
// FAS restriction is in launch_f32_nlr.cu, the linear-operator and transfer
// instantiations and the fused FP32 kernels (tiles, coarse cycle, linearised
// (H, C) cycles) in launch_f32_fast.cu: the units compile in parallel.
#include "launch_impl.cuh"

namespace mlgpu {

template cudaError_t launch_nl_op<float>(const NLArgs<float> &, int, int, const float *,
                                         const float *, float *, float *, double *, int *,
                                         cudaStream_t);
template cudaError_t launch_nl_gsrb<float>(const NLArgs<float> &, float *, const float *, int,
                                           cudaStream_t);
template cudaError_t launch_nl_relax_block<float>(const NLArgs<float> &, float *, const float *,
                                                  int, cudaStream_t);
template cudaError_t launch_nl_lambda<float>(const NLArgs<float> &, float *, cudaStream_t);
}  // namespace mlgpu
