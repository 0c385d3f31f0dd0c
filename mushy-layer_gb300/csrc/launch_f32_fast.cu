// launch_f32_fast.cu -- FP32 instantiations of the linear-operator, transfer
// and vector launchers, and the launchers of the fused FP32 kernels of the
// mixed-precision solvers: the 2D tile smoother and coarse cycle of the
// linear operators, the linearised (H, C) cycles (FMA contraction on).
#define MLGPU_FP32_UNIT 1
#include "launch_impl.cuh"
#include "tile_fast_kernels.cuh"
#include "cycle_fast_kernels.cuh"
#include "hcm_kernels.cuh"

namespace mlgpu {
template cudaError_t launch_vc_op<float>(const VCArgs<float> &, int, int, const float *,
                                         const float *, float *, int, double *, int *,
                                         cudaStream_t);
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
template cudaError_t launch_norm_partial<float>(long long, const float *, int, double *, int *,
                                                cudaStream_t);
template cudaError_t launch_convert<float, double>(long long, float *, const double *,
                                                  cudaStream_t);
template cudaError_t launch_convert<float, float>(long long, float *, const float *, cudaStream_t);

template cudaError_t launch_vc_block_cycle<float>(const VCBlockCycle<float> &, cudaStream_t);
template cudaError_t launch_vc_tile_smooth<float>(const TileSmooth<float> &, cudaStream_t);

cudaError_t launch_vc_tile_fast(const TileFast &P, cudaStream_t s) {
  if (P.G.dim != 2 || P.halo < 0 || P.halo > kTFMaxHalo) return cudaErrorInvalidValue;
  if (P.halo < P.n_half + (P.rc ? 1 : 0)) return cudaErrorInvalidValue;
  const int te = tile_fast_edge(P.halo);
  dim3 grid((P.G.n0 + te - 1) / te, (P.G.n1 + te - 1) / te);
  vc_tile_fast_kernel<<<grid, dim3(kTFThreadsX, kTFThreadsY), 0, s>>>(P);
  return cudaGetLastError();
}

cudaError_t launch_vc_cycle_fast(const CycFast &P, cudaStream_t s) {
  if (P.nlev < 2 || P.nlev > kFastCycLevels || P.G[0].dim != 2 || !P.pack) return cudaErrorInvalidValue;
  if (P.G[0].ncell > kFastCycCells || (P.off[P.nlev] & 3)) return cudaErrorInvalidValue;
  const int quads = (P.G[0].n0 / 2) * (P.G[0].n1 / 2);
  if (quads > kFastCycThreads) return cudaErrorInvalidValue;
  size_t bytes = cyc_fast_smem_bytes(P);
  if (bytes > kMaxDynSmem) return cudaErrorInvalidValue;
  // raise the dynamic shared-memory limit only as far as needed: the kernel
  // also has static shared memory (level table, barrier), and static +
  // dynamic must stay within the per-block opt-in maximum
  static size_t attr_bytes = 48 * 1024;
  if (bytes > attr_bytes) {
    cudaError_t e = cudaFuncSetAttribute(vc_cycle_fast_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return e;
    attr_bytes = bytes;
  }
  int threads = (quads + 31) / 32 * 32;
  if (threads < 64) threads = 64;
  vc_cycle_fast_kernel<<<1, threads, bytes, s>>>(P);
  return cudaGetLastError();
}

cudaError_t launch_cyc_pack(const Geom &G, const BCD &bc, const FastCoefs &K, float *level,
                            cudaStream_t s) {
  if (G.dim != 2 || G.ncell > 65535) return cudaErrorInvalidValue;
  cyc_pack_kernel<<<blocks_for(cyc_pad((int)G.ncell)), kBlock, 0, s>>>(G, bc, K, level);
  return cudaGetLastError();
}

cudaError_t launch_hcm_gsrb(const HCMArgs &A, float *e, const float *r, int pass,
                            cudaStream_t s) {
  const int nb = blocks_for(colour_threads(A.G));
  MLGPU_DIM_SWITCH(A.G.dim, (hcm_gsrb_kernel<DIM><<<nb, kBlock, 0, s>>>(A, e, r, pass)));
  return cudaGetLastError();
}

cudaError_t launch_hcm_relax_block(const HCMArgs &A, float *e, const float *r, int sweeps,
                                   cudaStream_t s) {
  long long nt = colour_threads(A.G);
  int threads = (int)((nt + 31) / 32 * 32);
  if (threads > 1024) threads = 1024;
  if (threads < 64) threads = 64;
  MLGPU_DIM_SWITCH(A.G.dim, (hcm_relax_block_kernel<DIM><<<1, threads, 0, s>>>(A, e, r, sweeps)));
  return cudaGetLastError();
}

cudaError_t launch_hcm_restrict(const HCMArgs &A, const Geom &C, const float *e, const float *r,
                                float *rc, cudaStream_t s) {
  MLGPU_DIM_SWITCH(A.G.dim, (hcm_restrict_kernel<DIM><<<blocks_for(C.ncell), kBlock, 0, s>>>(A, C, e, r, rc)));
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
