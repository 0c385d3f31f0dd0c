// launch_impl.cuh -- definitions of the launchers declared in launch.h.
// Included by one translation unit per precision, which instantiates them.
#pragma once
#include "launch.h"
#include "nl_kernels.cuh"
#include "vc_kernels.cuh"
#include "misc_kernels.cuh"
#include "cycle_kernels.cuh"
#include "tile_kernels.cuh"
#include "outer_kernels.cuh"

namespace mlgpu {

constexpr size_t kMaxDynSmem = 227 * 1024;

template <class T>
cudaError_t launch_vc_tile_smooth(const TileSmooth<T> &P, cudaStream_t s) {
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(vc_tile_smooth_kernel<T>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kMaxDynSmem);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  size_t bytes = tile_smem_bytes(P.halo, sizeof(T));
  if (bytes > kMaxDynSmem) return cudaErrorInvalidValue;
  const Geom &G = P.A.G;
  dim3 grid((G.n0 + kTileX - 1) / kTileX, (G.n1 + kTileY - 1) / kTileY);
  vc_tile_smooth_kernel<T><<<grid, dim3(kTileTX, kTileTY), bytes, s>>>(P);
  return cudaGetLastError();
}

#define MLGPU_DIM_SWITCH(dim, ...) \
  do {                              \
    if ((dim) == 3) {               \
      constexpr int DIM = 3;        \
      __VA_ARGS__;                  \
    } else {                        \
      constexpr int DIM = 2;        \
      __VA_ARGS__;                  \
    }                               \
  } while (0)

#define MLGPU_NORM_SWITCH(norm, ...)           \
  do {                                         \
    switch (norm) {                            \
      case MLGPU_NORM_MAX: {                   \
        constexpr int NORM = MLGPU_NORM_MAX;   \
        __VA_ARGS__;                           \
      } break;                                 \
      case MLGPU_NORM_L1: {                    \
        constexpr int NORM = MLGPU_NORM_L1;    \
        __VA_ARGS__;                           \
      } break;                                 \
      case MLGPU_NORM_L2: {                    \
        constexpr int NORM = MLGPU_NORM_L2;    \
        __VA_ARGS__;                           \
      } break;                                 \
      default: {                               \
        constexpr int NORM = -1;               \
        __VA_ARGS__;                           \
      } break;                                 \
    }                                          \
  } while (0)

template <class T>
cudaError_t launch_nl_op(const NLArgs<T> &A, int mode, int norm, const T *phi, const T *rhs, T *out,
                         T *copy, double *part, int *nparts, cudaStream_t s) {
  int nb = blocks_for(A.G.ncell);
  if (nparts) *nparts = (part && norm >= 0) ? nb : 0;
  MLGPU_DIM_SWITCH(A.G.dim, MLGPU_NORM_SWITCH(norm, {
    switch (mode) {
      case NL_RESIDUAL:
        nl_op_kernel<T, DIM, NL_RESIDUAL, NORM><<<nb, kBlock, 0, s>>>(A, phi, rhs, out, copy, part);
        break;
      case NL_APPLY:
        nl_op_kernel<T, DIM, NL_APPLY, NORM><<<nb, kBlock, 0, s>>>(A, phi, rhs, out, copy, part);
        break;
      case NL_APPLY_PLUS:
        nl_op_kernel<T, DIM, NL_APPLY_PLUS, NORM><<<nb, kBlock, 0, s>>>(A, phi, rhs, out, copy, part);
        break;
      default:
        nl_op_kernel<T, DIM, NL_JACOBI, NORM><<<nb, kBlock, 0, s>>>(A, phi, rhs, out, copy, part);
        break;
    }
  }));
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_nl_gsrb(const NLArgs<T> &A, T *phi, const T *rhs, int pass, cudaStream_t s) {
  int nb = blocks_for(colour_threads(A.G));
  MLGPU_DIM_SWITCH(A.G.dim, (nl_gsrb_kernel<T, DIM><<<nb, kBlock, 0, s>>>(A, phi, rhs, pass)));
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_nl_relax_block(const NLArgs<T> &A, T *phi, const T *rhs, int sweeps,
                                  cudaStream_t s) {
  long long nt = colour_threads(A.G);
  int threads = (int)((nt + 31) / 32 * 32);
  if (threads > 1024) threads = 1024;
  if (threads < 32) threads = 32;
  MLGPU_DIM_SWITCH(A.G.dim, (nl_relax_block_kernel<T, DIM><<<1, threads, 0, s>>>(A, phi, rhs, sweeps)));
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_nl_restrict(const NLArgs<T> &A, const Geom &C, const T *phi, const T *rhs,
                               T *res_c, T *phi_c, cudaStream_t s) {
  int nb = blocks_for(C.ncell);
  MLGPU_DIM_SWITCH(A.G.dim, (nl_restrict_kernel<T, DIM><<<nb, kBlock, 0, s>>>(A, C, phi, rhs, res_c, phi_c)));
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_nl_lambda(const NLArgs<T> &A, T *lam, cudaStream_t s) {
  int nb = blocks_for(A.G.ncell);
  MLGPU_DIM_SWITCH(A.G.dim, (nl_lambda_kernel<T, DIM><<<nb, kBlock, 0, s>>>(A, lam)));
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_vc_op(const VCArgs<T> &A, int mode, int norm, const T *phi, const T *rhs, T *out,
                         int homog, double *part, int *nparts, cudaStream_t s) {
  int nb = blocks_for(A.G.ncell);
  if (nparts) *nparts = (part && norm >= 0) ? nb : 0;
  MLGPU_DIM_SWITCH(A.G.dim, MLGPU_NORM_SWITCH(norm, {
    switch (mode) {
      case VC_RESIDUAL:
        vc_op_kernel<T, DIM, VC_RESIDUAL, NORM><<<nb, kBlock, 0, s>>>(A, phi, rhs, out, homog, part);
        break;
      case VC_APPLY:
        vc_op_kernel<T, DIM, VC_APPLY, NORM><<<nb, kBlock, 0, s>>>(A, phi, rhs, out, homog, part);
        break;
      default:
        vc_op_kernel<T, DIM, VC_JACOBI, NORM><<<nb, kBlock, 0, s>>>(A, phi, rhs, out, homog, part);
        break;
    }
  }));
  return cudaGetLastError();
}

template <class T, class E>
cudaError_t launch_vc_update_residual(const VCArgs<T> &A, int norm, const T *phi, const E *e,
                                      const T *rhs, T *out_phi, T *res, E *res_inner,
                                      double *part, int *nparts, cudaStream_t s,
                                      const int *par) {
  int nb = blocks_for(A.G.ncell);
  if (nparts) *nparts = nb;
  if (norm < 0) norm = MLGPU_NORM_MAX;
  MLGPU_DIM_SWITCH(A.G.dim, MLGPU_NORM_SWITCH(norm, {
    if (NORM >= 0)
      vc_update_residual_kernel<T, E, DIM, (NORM < 0 ? 0 : NORM)>
          <<<nb, kBlock, 0, s>>>(A, phi, e, rhs, out_phi, res, res_inner, part, par);
  }));
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_vc_gsrb(const VCArgs<T> &A, T *phi, const T *rhs, int pass, cudaStream_t s) {
  int nb = blocks_for(colour_threads(A.G));
  MLGPU_DIM_SWITCH(A.G.dim, (vc_gsrb_kernel<T, DIM><<<nb, kBlock, 0, s>>>(A, phi, rhs, pass)));
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_vc_gsrb_zero(const VCArgs<T> &A, T *phi, const T *rhs, cudaStream_t s) {
  int nb = blocks_for(A.G.ncell);
  MLGPU_DIM_SWITCH(A.G.dim, (vc_gsrb_zero_kernel<T, DIM><<<nb, kBlock, 0, s>>>(A, phi, rhs)));
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_vc_relax_block(const VCArgs<T> &A, T *phi, const T *rhs, int sweeps,
                                  int zero_first, cudaStream_t s) {
  long long nt = colour_threads(A.G);
  int threads = (int)((nt + 31) / 32 * 32);
  if (threads > 1024) threads = 1024;
  if (threads < 32) threads = 32;
  MLGPU_DIM_SWITCH(A.G.dim, (vc_relax_block_kernel<T, DIM><<<1, threads, 0, s>>>(A, phi, rhs, sweeps, zero_first)));
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_vc_restrict(const VCArgs<T> &A, const Geom &C, const T *phi, const T *rhs,
                               T *res_c, T *zero_c, cudaStream_t s) {
  int nb = blocks_for(C.ncell);
  MLGPU_DIM_SWITCH(A.G.dim, (vc_restrict_kernel<T, DIM><<<nb, kBlock, 0, s>>>(A, C, phi, rhs, res_c, zero_c)));
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_vc_lambda(const VCArgs<T> &A, T *lam, cudaStream_t s) {
  int nb = blocks_for(A.G.ncell);
  MLGPU_DIM_SWITCH(A.G.dim, (vc_lambda_kernel<T, DIM><<<nb, kBlock, 0, s>>>(A, lam)));
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_vc_block_cycle(const VCBlockCycle<T> &P, cudaStream_t s) {
  long long nt = colour_threads(P.A[0].G);
  int threads = (int)((nt + 31) / 32 * 32);
  if (threads > 256) threads = 256;  // __launch_bounds__ of the kernel
  if (threads < 64) threads = 64;
  size_t bytes = block_cycle_smem_bytes(P);
  if (bytes > 48 * 1024) return cudaErrorInvalidValue;  // levels above kBlockCycleCells
  MLGPU_DIM_SWITCH(P.A[0].G.dim, (vc_block_cycle_kernel<T, DIM><<<1, threads, bytes, s>>>(P)));
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_restrict_avg(const Geom &F, int ncomp, const T *fine, T *coarse, cudaStream_t s) {
  Geom C = coarsen_geom(F);
  int nb = blocks_for(C.ncell * ncomp);
  MLGPU_DIM_SWITCH(F.dim, (restrict_avg_kernel<T, DIM><<<nb, kBlock, 0, s>>>(F, C, ncomp, fine, coarse)));
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_prolong(const Geom &F, const BCD &bc, int ncomp, int kind, T *fine, const T *a,
                           const T *b, cudaStream_t s) {
  Geom C = coarsen_geom(F);
  int nb = blocks_for(F.ncell * ncomp);
  MLGPU_DIM_SWITCH(F.dim, {
    if (kind == MLGPU_PROLONG_LINEAR)
      prolong_kernel<T, DIM, MLGPU_PROLONG_LINEAR><<<nb, kBlock, 0, s>>>(F, C, bc, ncomp, fine, a, b);
    else
      prolong_kernel<T, DIM, MLGPU_PROLONG_CONSTANT><<<nb, kBlock, 0, s>>>(F, C, bc, ncomp, fine, a, b);
  });
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_coarsen_faces(const Geom &F, int ncomp, int d, const T *ff, T *cf,
                                 cudaStream_t s) {
  Geom C = coarsen_geom(F);
  int nb = blocks_for(C.nface(d) * ncomp);
  MLGPU_DIM_SWITCH(F.dim, (coarsen_faces_kernel<T, DIM><<<nb, kBlock, 0, s>>>(F, C, ncomp, d, ff, cf)));
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_axpby(long long n, T a, const T *x, T b, T *y, cudaStream_t s) {
  axpby_kernel<T><<<blocks_for(n), kBlock, 0, s>>>(n, a, x, b, y);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_norm_partial(long long n, const T *x, int norm, double *part, int *nparts,
                                cudaStream_t s) {
  int nb = blocks_for(n);
  if (nparts) *nparts = norm >= 0 ? nb : 0;
  MLGPU_NORM_SWITCH(norm, {
    if (NORM >= 0) norm_partial_kernel<T, (NORM < 0 ? 0 : NORM)><<<nb, kBlock, 0, s>>>(n, x, part);
  });
  return cudaGetLastError();
}

template <class D, class S>
cudaError_t launch_convert(long long n, D *dst, const S *src, cudaStream_t s) {
  convert_kernel<D, S><<<blocks_for(n), kBlock, 0, s>>>(n, dst, src);
  return cudaGetLastError();
}

}  // namespace mlgpu
