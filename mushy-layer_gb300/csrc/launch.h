// launch.h -- host launchers of the sm_103a kernels.  Each precision is
// instantiated in its own translation units: the FP64 units (launch_f64.cu,
// launch_f64_nlc.cu for the cached-closure (H, C) kernels, launch_f64_adj.cu
// for the Jacobian / adjoint kernels, compiled in parallel) use --fmad=false
// so FP64 keeps the reference's unfused evaluation (bitwise parity with the
// CPU restatement), launch_f32.cu has FMA contraction on.
#pragma once
#include <cuda_runtime.h>
#include "common.cuh"

namespace mlgpu {

template <class T> struct NLArgs;
template <class T> struct VCArgs;

// Grid size for grid-stride kernels: enough blocks to cover n work items, at
// most 16 resident blocks per SM on the 152 SMs of a GB300.
constexpr int kMaxBlocks = 152 * 16;
inline int blocks_for(long long n) {
  long long b = (n + 255) / 256;
  if (b < 1) b = 1;
  if (b > kMaxBlocks) b = kMaxBlocks;
  return (int)b;
}

// scratch for fused norms: kMaxBlocks partials + 1 result slot
constexpr size_t kNormScratchDoubles = kMaxBlocks + 8;

template <class T>
cudaError_t launch_nl_op(const NLArgs<T> &A, int mode, int norm, const T *phi, const T *rhs, T *out,
                         T *copy, double *part, int *nparts, cudaStream_t s);
template <class T>
cudaError_t launch_nl_gsrb(const NLArgs<T> &A, T *phi, const T *rhs, int pass, cudaStream_t s);
template <class T>
cudaError_t launch_nl_relax_block(const NLArgs<T> &A, T *phi, const T *rhs, int sweeps,
                                  cudaStream_t s);
template <class T>
cudaError_t launch_nl_restrict(const NLArgs<T> &A, const Geom &C, const T *phi, const T *rhs,
                               T *res_c, T *phi_c, cudaStream_t s);
template <class T>
cudaError_t launch_nl_lambda(const NLArgs<T> &A, T *lam, cudaStream_t s);

template <class T>
cudaError_t launch_vc_op(const VCArgs<T> &A, int mode, int norm, const T *phi, const T *rhs, T *out,
                         int homog, double *part, int *nparts, cudaStream_t s);
template <class T, class E>
cudaError_t launch_vc_update_residual(const VCArgs<T> &A, int norm, const T *phi, const E *e,
                                      const T *rhs, T *out_phi, T *res, E *res_inner,
                                      double *part, int *nparts, cudaStream_t s,
                                      const int *par = nullptr);
template <class T>
cudaError_t launch_vc_gsrb(const VCArgs<T> &A, T *phi, const T *rhs, int pass, cudaStream_t s);
template <class T>
cudaError_t launch_vc_gsrb_zero(const VCArgs<T> &A, T *phi, const T *rhs, cudaStream_t s);
template <class T>
cudaError_t launch_vc_relax_block(const VCArgs<T> &A, T *phi, const T *rhs, int sweeps,
                                  int zero_first, cudaStream_t s);
template <class T>
cudaError_t launch_vc_restrict(const VCArgs<T> &A, const Geom &C, const T *phi, const T *rhs,
                               T *res_c, T *zero_c, cudaStream_t s);
template <class T>
cudaError_t launch_vc_lambda(const VCArgs<T> &A, T *lam, cudaStream_t s);
template <class T> struct VCBlockCycle;
template <class T>
cudaError_t launch_vc_block_cycle(const VCBlockCycle<T> &P, cudaStream_t s);
// levels at or below this many cells run inside one thread block
constexpr long long kBlockCycleCells = 256;
template <class T> struct TileSmooth;
template <class T>
cudaError_t launch_vc_tile_smooth(const TileSmooth<T> &P, cudaStream_t s);
// largest halo a tile launch may use for element size `elem` (shared memory)
int tile_max_halo(size_t elem);
struct TileFast;
cudaError_t launch_vc_tile_fast(const TileFast &P, cudaStream_t s);
struct HCMArgs;
cudaError_t launch_hcm_gsrb(const HCMArgs &A, float *e, const float *r, int pass, cudaStream_t s);
cudaError_t launch_hcm_relax_block(const HCMArgs &A, float *e, const float *r, int sweeps,
                                   cudaStream_t s);
cudaError_t launch_hcm_restrict(const HCMArgs &A, const Geom &C, const float *e, const float *r,
                                float *rc, cudaStream_t s);
struct CycFast;
cudaError_t launch_vc_cycle_fast(const CycFast &P, cudaStream_t s);
struct FastCoefs;
cudaError_t launch_cyc_pack(const Geom &G, const BCD &bc, const FastCoefs &K, float *level,
                            cudaStream_t s);
cudaError_t launch_fast_coefs(const VCArgs<double> &A, float *cx, float *cy, float *lam,
                              float *diag, cudaStream_t s);

template <class T>
cudaError_t launch_restrict_avg(const Geom &F, int ncomp, const T *fine, T *coarse, cudaStream_t s);
template <class T>
cudaError_t launch_prolong(const Geom &F, const BCD &bc, int ncomp, int kind, T *fine, const T *a,
                           const T *b, cudaStream_t s);
template <class T>
cudaError_t launch_coarsen_faces(const Geom &F, int ncomp, int d, const T *ff, T *cf,
                                 cudaStream_t s);
template <class T>
cudaError_t launch_axpby(long long n, T a, const T *x, T b, T *y, cudaStream_t s);
template <class T>
cudaError_t launch_norm_partial(long long n, const T *x, int norm, double *part, int *nparts,
                                cudaStream_t s);
template <class D, class S>
cudaError_t launch_convert(long long n, D *dst, const S *src, cudaStream_t s);

// Every launcher that writes fused-norm partials (one per block) stores the
// number it wrote in *nparts (when part is non-null); the finalize call is
// given that count, so a launch and the combine of its partials cannot
// disagree about the grid.
cudaError_t launch_finalize_norm(int norm, const double *part, int nparts, double *out,
                                 cudaStream_t s);

}  // namespace mlgpu
