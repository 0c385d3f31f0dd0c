// launch_f64_adj.cu -- FP64 launchers of the Jacobian / adjoint kernels
// (adjoint_kernels.cuh), a unit of their own so that the library's units
// compile in parallel.  Built with --fmad=false, as launch_f64.cu.
#define MLGPU_ADJ_UNIT 1
#include "launch_impl.cuh"
#include "adjoint_kernels.cuh"

namespace mlgpu {

cudaError_t launch_adj_jac(const Geom &G, const ClosureParams &cp, const double *u, double *J,
                           cudaStream_t s) {
  adj_jac_kernel<double><<<blocks_for(G.ncell), kBlock, 0, s>>>(G, cp, u, J);
  return cudaGetLastError();
}
cudaError_t launch_porosity_jac(const Geom &G, const ClosureParams &cp, const double *u,
                                double *dp, cudaStream_t s) {
  porosity_jac_kernel<<<blocks_for(G.ncell), kBlock, 0, s>>>(G, cp, u, dp);
  return cudaGetLastError();
}
#define MLGPU_TR_SWITCH(tr, ...) \
  do {                            \
    if (tr) {                     \
      constexpr bool TR = true;   \
      __VA_ARGS__;                \
    } else {                      \
      constexpr bool TR = false;  \
      __VA_ARGS__;                \
    }                             \
  } while (0)

cudaError_t launch_adj_op(const AdjArgs<double> &A, int mode, int norm, const double *y,
                          const double *g, double *out, double *part, int *nparts,
                          cudaStream_t s, bool tr) {
  const int nb = blocks_for(A.G.ncell);
  if (nparts) *nparts = (part && mode == ADJ_RESIDUAL && norm >= 0) ? nb : 0;
  if (mode == ADJ_RESIDUAL && norm >= 0) {
    if (!part) return cudaErrorInvalidValue;
    MLGPU_TR_SWITCH(tr, MLGPU_DIM_SWITCH(A.G.dim, MLGPU_NORM_SWITCH(norm, (adj_op_kernel<double, DIM, ADJ_RESIDUAL, NORM, TR><<<nb, kBlock, 0, s>>>(A, y, g, out, part)))));
  } else if (mode == ADJ_RESIDUAL) {
    MLGPU_TR_SWITCH(tr, MLGPU_DIM_SWITCH(A.G.dim, (adj_op_kernel<double, DIM, ADJ_RESIDUAL, -1, TR><<<nb, kBlock, 0, s>>>(A, y, g, out, part))));
  } else {
    MLGPU_TR_SWITCH(tr, MLGPU_DIM_SWITCH(A.G.dim, (adj_op_kernel<double, DIM, ADJ_APPLY, -1, TR><<<nb, kBlock, 0, s>>>(A, y, g, out, part))));
  }
  return cudaGetLastError();
}
cudaError_t launch_adj_gsrb(const AdjArgs<double> &A, double *y, const double *g, int pass,
                            cudaStream_t s, bool tr) {
  MLGPU_TR_SWITCH(tr, MLGPU_DIM_SWITCH(A.G.dim, (adj_gsrb_kernel<double, DIM, TR><<<blocks_for(colour_threads(A.G)), kBlock, 0, s>>>(A, y, g, pass))));
  return cudaGetLastError();
}
cudaError_t launch_adj_relax_block(const AdjArgs<double> &A, double *y, const double *g,
                                   int sweeps, int zero, cudaStream_t s, bool tr) {
  MLGPU_TR_SWITCH(tr, MLGPU_DIM_SWITCH(A.G.dim, (adj_relax_block_kernel<double, DIM, TR><<<1, 1024, 0, s>>>(A, y, g, sweeps, zero))));
  return cudaGetLastError();
}
cudaError_t launch_adj_minv(const AdjArgs<double> &A, const double *zero, double *Minv,
                            double *D, cudaStream_t s) {
  MLGPU_DIM_SWITCH(A.G.dim, (adj_minv_kernel<double, DIM><<<blocks_for(A.G.ncell), kBlock, 0, s>>>(A, zero, Minv, D)));
  return cudaGetLastError();
}
cudaError_t launch_adj_bottom_direct(const AdjArgs<double> &A, double *y, const double *g,
                                     cudaStream_t s, bool tr) {
  if (2 * A.G.ncell > kAdjDirectMax) return cudaErrorInvalidValue;
  MLGPU_TR_SWITCH(tr, MLGPU_DIM_SWITCH(A.G.dim, (adj_bottom_direct_kernel<double, DIM, TR><<<1, kAdjDirectMax, 0, s>>>(A, y, g))));
  return cudaGetLastError();
}
cudaError_t launch_adj_restrict(const AdjArgs<double> &A, const Geom &C, const double *y,
                                const double *g, double *gc, cudaStream_t s, bool tr) {
  MLGPU_TR_SWITCH(tr, MLGPU_DIM_SWITCH(A.G.dim, (adj_restrict_kernel<double, DIM, TR><<<blocks_for(C.ncell), kBlock, 0, s>>>(A, C, y, g, gc))));
  return cudaGetLastError();
}
cudaError_t launch_adj_bc_grad(const AdjArgs<double> &A, const double *y, double *out,
                               cudaStream_t s) {
  MLGPU_DIM_SWITCH(A.G.dim, (adj_bc_grad_kernel<double, DIM><<<6, kBlock, 0, s>>>(A, y, out)));
  return cudaGetLastError();
}

}  // namespace mlgpu
