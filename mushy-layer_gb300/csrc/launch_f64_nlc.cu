// launch_f64_nlc.cu -- launchers of the cached-closure kernels of the (H, C)
// FAS path (nl_cached_kernels.cuh), a unit of their own so that the
// library's units compile in parallel.  Built with --fmad=false, as
// launch_f64.cu.
#define MLGPU_NLC_UNIT 1
#include "launch_impl.cuh"
#include "nl_cached_kernels.cuh"

namespace mlgpu {

cudaError_t launch_nlc_closure(const NLArgs<double> &A, const double *phi, double *tcl,
                               cudaStream_t s, int lean) {
  const int nb = nlc_blocks(A.G.ncell);
  const ClosureLean P = make_closure_lean(A.cp);
  if (lean) {
    MLGPU_DIM_SWITCH(A.G.dim, (nlc_closure_kernel<DIM, true><<<nb, kNLCBlock, 0, s>>>(A, P, phi, tcl)));
  } else {
    MLGPU_DIM_SWITCH(A.G.dim, (nlc_closure_kernel<DIM, false><<<nb, kNLCBlock, 0, s>>>(A, P, phi, tcl)));
  }
  return cudaGetLastError();
}

cudaError_t launch_nlc_gsrb(const NLArgs<double> &A, double *phi, const double *rhs, double *tcl,
                            const double *lam, int pass, cudaStream_t s) {
  const int nb = nlc_blocks(colour_threads(A.G));
  MLGPU_DIM_SWITCH(A.G.dim, (nlc_gsrb_kernel<DIM><<<nb, kNLCBlock, 0, s>>>(A, phi, rhs, tcl, lam, pass)));
  return cudaGetLastError();
}

cudaError_t launch_nlc_relax_block(const NLArgs<double> &A, double *phi, const double *rhs,
                                   double *tcl, const double *lam, int sweeps, int init,
                                   cudaStream_t s) {
  // one warp per colour cell, at most 32 warps
  long long nt = colour_threads(A.G);
  int threads = (int)(32 * (nt < 32 ? (nt < 1 ? 1 : nt) : 32));
  MLGPU_DIM_SWITCH(A.G.dim, (nlc_relax_block_kernel<DIM><<<1, threads, 0, s>>>(A, phi, rhs, tcl, lam, sweeps, init)));
  return cudaGetLastError();
}

cudaError_t launch_nlc_op(const NLArgs<double> &A, int mode, int norm, const double *phi,
                          const double *tcl, const double *rhs, double *out, double *copy,
                          double *part, int *nparts, cudaStream_t s, double *part_max) {
  const int nb = nlc_blocks(A.G.ncell);
  if (nparts) *nparts = (part && mode == NL_RESIDUAL && norm >= 0) ? nb : 0;
  if (mode == NL_RESIDUAL) {
    if (part_max && norm >= 0) {
      MLGPU_DIM_SWITCH(A.G.dim, MLGPU_NORM_SWITCH(norm, (nlc_op_kernel<DIM, NL_RESIDUAL, NORM, true><<<nb, kNLCBlock, 0, s>>>(A, phi, tcl, rhs, out, copy, part, part_max))));
    } else {
      MLGPU_DIM_SWITCH(A.G.dim, MLGPU_NORM_SWITCH(norm, (nlc_op_kernel<DIM, NL_RESIDUAL, NORM, false><<<nb, kNLCBlock, 0, s>>>(A, phi, tcl, rhs, out, copy, part, nullptr))));
    }
  } else if (mode == NL_APPLY_PLUS) {
    MLGPU_DIM_SWITCH(A.G.dim, (nlc_op_kernel<DIM, NL_APPLY_PLUS, -1, false><<<nb, kNLCBlock, 0, s>>>(A, phi, tcl, rhs, out, copy, part, nullptr)));
  } else {
    return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_nlc_bsum(const NLArgs<double> &A, double *sb, cudaStream_t s) {
  MLGPU_DIM_SWITCH(A.G.dim, (nlc_bsum_kernel<DIM><<<nlc_blocks(A.G.ncell), kNLCBlock, 0, s>>>(A, sb)));
  return cudaGetLastError();
}

cudaError_t launch_nlc_res_lean(const NLArgs<double> &A, const double *phi, const double *tcl,
                                const double *sb, const double *rhs, double *out, double *part,
                                double *part_max, int *nparts, cudaStream_t s) {
  const int nb = nlc_blocks(A.G.ncell);
  if (nparts) *nparts = nb;
  MLGPU_DIM_SWITCH(A.G.dim, (nlc_res_lean_kernel<DIM><<<nb, kNLCBlock, 0, s>>>(A, phi, tcl, sb, rhs, out, part, part_max)));
  return cudaGetLastError();
}

cudaError_t launch_nlc_restrict(const NLArgs<double> &A, const Geom &C, const double *phi,
                                const double *tcl, const double *rhs, double *res_c,
                                double *phi_c, cudaStream_t s) {
  MLGPU_DIM_SWITCH(A.G.dim, (nlc_restrict_kernel<DIM><<<nlc_blocks(C.ncell), kNLCBlock, 0, s>>>(A, C, phi, tcl, rhs, res_c, phi_c)));
  return cudaGetLastError();
}

}  // namespace mlgpu
