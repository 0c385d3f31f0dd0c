// launch_f32_nlr.cu -- the FP32 instantiation of the nonlinear FAS
// restriction launcher (its own translation unit: it compiles in parallel
// with the other FP32 launchers).  FMA contraction is left on.
#include "launch_impl.cuh"

namespace mlgpu {

template cudaError_t launch_nl_restrict<float>(const NLArgs<float> &, const Geom &, const float *,
                                               const float *, float *, float *, cudaStream_t);

}  // namespace mlgpu
