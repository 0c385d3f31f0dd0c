// launch_f32.cu -- FP32 instantiations of the kernel launchers (inner
// multigrid cycles of the mixed-precision solvers).  FMA contraction is left
// on; the nonlinear closure inside these kernels still runs in FP64.
#define MLGPU_FP32_UNIT 1
#include "launch_impl.cuh"
#include "tile_fast_kernels.cuh"

namespace mlgpu {

template cudaError_t launch_nl_op<float>(const NLArgs<float> &, int, int, const float *,
                                         const float *, float *, float *, double *, cudaStream_t);
template cudaError_t launch_nl_gsrb<float>(const NLArgs<float> &, float *, const float *, int,
                                           cudaStream_t);
template cudaError_t launch_nl_relax_block<float>(const NLArgs<float> &, float *, const float *,
                                                  int, cudaStream_t);
template cudaError_t launch_nl_restrict<float>(const NLArgs<float> &, const Geom &, const float *,
                                               const float *, float *, float *, cudaStream_t);
template cudaError_t launch_nl_lambda<float>(const NLArgs<float> &, float *, cudaStream_t);
template cudaError_t launch_vc_op<float>(const VCArgs<float> &, int, int, const float *,
                                         const float *, float *, int, double *, cudaStream_t);
template cudaError_t launch_vc_gsrb<float>(const VCArgs<float> &, float *, const float *, int,
                                           cudaStream_t);
template cudaError_t launch_vc_gsrb_zero<float>(const VCArgs<float> &, float *, const float *,
                                                cudaStream_t);
template cudaError_t launch_vc_relax_block<float>(const VCArgs<float> &, float *, const float *,
                                                  int, int, cudaStream_t);
template cudaError_t launch_vc_restrict<float>(const VCArgs<float> &, const Geom &, const float *,
                                               const float *, float *, float *, cudaStream_t);
template cudaError_t launch_vc_lambda<float>(const VCArgs<float> &, float *, cudaStream_t);
template cudaError_t launch_restrict_avg<float>(const Geom &, int, const float *, float *,
                                                cudaStream_t);
template cudaError_t launch_prolong<float>(const Geom &, const BCD &, int, int, float *,
                                           const float *, const float *, cudaStream_t);
template cudaError_t launch_coarsen_faces<float>(const Geom &, int, int, const float *, float *,
                                                 cudaStream_t);
template cudaError_t launch_axpby<float>(long long, float, const float *, float, float *,
                                         cudaStream_t);
template cudaError_t launch_norm_partial<float>(long long, const float *, int, double *,
                                                cudaStream_t);
template cudaError_t launch_convert<float, double>(long long, float *, const double *,
                                                  cudaStream_t);
template cudaError_t launch_convert<float, float>(long long, float *, const float *, cudaStream_t);

}  // namespace mlgpu

namespace mlgpu {
template cudaError_t launch_vc_block_cycle<float>(const VCBlockCycle<float> &, cudaStream_t);
template cudaError_t launch_vc_tile_smooth<float>(const TileSmooth<float> &, cudaStream_t);

cudaError_t launch_vc_tile_fast(const TileFast &P, cudaStream_t s) {
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(vc_tile_fast_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kMaxDynSmem);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  size_t bytes = tile_fast_smem_bytes(P.halo);
  if (bytes > kMaxDynSmem) return cudaErrorInvalidValue;
  dim3 grid((P.G.n0 + kTileX - 1) / kTileX, (P.G.n1 + kTileY - 1) / kTileY);
  vc_tile_fast_kernel<<<grid, dim3(kTileTX, kTileTY), bytes, s>>>(P);
  return cudaGetLastError();
}

cudaError_t launch_fast_coefs(const VCArgs<double> &A, float *cx, float *cy, float *lam,
                              float *diag, cudaStream_t s) {
  if (A.G.dim != 2) return cudaErrorInvalidValue;
  long long n = A.G.nface(0) > A.G.ncell ? A.G.nface(0) : A.G.ncell;
  if (A.G.nface(1) > n) n = A.G.nface(1);
  fast_coefs_kernel<2><<<blocks_for(n), kBlock, 0, s>>>(A, cx, cy, lam, diag);
  return cudaGetLastError();
}
}
