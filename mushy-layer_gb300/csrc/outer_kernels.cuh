// outer_kernels.cuh -- device-resident outer iteration of a solve.
// The multigrid outer loop (AMRMultiGrid::solveNoInit: cycle, new residual,
// norm, convergence / hang / iteration-limit tests) runs as the body of a
// CUDA-graph WHILE node; this one-thread kernel applies the same tests the
// host loop applies and sets the node's condition, so a whole solve is one
// graph launch with no host round trip per iteration.
#pragma once
#include <cuda_runtime.h>
#include "common.cuh"

namespace mlgpu {

struct OuterDev {
  double norm0, norm, prev;
  int iter, status, parity, cont;
  int fault;  // set by a kernel whose bounded wait ran out; ends the loop
  double hist[64];
};

// exit status of a solve that a device-side wait timeout ended
constexpr int kStatusDeviceFault = 16;

struct OuterCfg {
  double tolerance, hang, norm_thresh;
  int max_iter;
};

#ifdef MLGPU_FP64_UNIT  // defined once, in launch_f64.cu
// the host loop's tests after one outer iteration with residual norm `norm`
__device__ __forceinline__ void outer_decide_step(OuterDev *st, double norm, const OuterCfg &c,
                                                  cudaGraphConditionalHandle h) {
  int iter = st->iter + 1;
  st->iter = iter;
  st->norm = norm;
  if (iter < 64) st->hist[iter] = norm;
  st->parity ^= 1;
  int status = 0;
  if (st->fault) {
    status = kStatusDeviceFault;
  } else if (!isfinite(norm)) {
    status = 8;
  } else if (norm > (1.0 - c.hang) * st->prev && norm > c.tolerance * st->norm0) {
    status = 2;
  } else {
    st->prev = norm;
  }
  st->status = status;
  int cont = norm > c.tolerance * st->norm0 && st->norm0 > c.norm_thresh && iter < c.max_iter &&
             status == 0;
  st->cont = cont;
  cudaGraphSetConditional(h, cont ? 1u : 0u);
}

__global__ void outer_decide_kernel(OuterDev *st, const double *__restrict__ norm_in, OuterCfg c,
                                    cudaGraphConditionalHandle h) {
  outer_decide_step(st, norm_in[0], c, h);
}
#endif

}  // namespace mlgpu
