// launch_f64.cu -- FP64 instantiations of the kernel launchers.  Built with
// --fmad=false: every FP64 product and sum is rounded separately, as in the
// reference's Fortran, so FP64 results match the CPU restatement bit for bit.
#define MLGPU_FP64_UNIT 1
#include "launch_impl.cuh"
#include "outer_fast_kernels.cuh"
#include "hcm_kernels.cuh"
#include "bicgstab_kernels.cuh"

namespace mlgpu {

template <class S>
cudaError_t launch_vc_bicgstab(const VCArgs<double> &A, S *e, const S *rhs, double *ws,
                               int imax, int remove_mean, cudaStream_t s) {
  MLGPU_DIM_SWITCH(A.G.dim, (vc_bicgstab_kernel<S, DIM><<<1, kBiCGThreads, 0, s>>>(A, e, rhs, ws, imax, remove_mean)));
  return cudaGetLastError();
}
template cudaError_t launch_vc_bicgstab<double>(const VCArgs<double> &, double *, const double *,
                                                double *, int, int, cudaStream_t);
template cudaError_t launch_vc_bicgstab<float>(const VCArgs<double> &, float *, const float *,
                                               double *, int, int, cudaStream_t);

template cudaError_t launch_nl_op<double>(const NLArgs<double> &, int, int, const double *,
                                          const double *, double *, double *, double *, int *,
                                          cudaStream_t);
template cudaError_t launch_nl_gsrb<double>(const NLArgs<double> &, double *, const double *, int,
                                            cudaStream_t);
template cudaError_t launch_nl_relax_block<double>(const NLArgs<double> &, double *,
                                                   const double *, int, cudaStream_t);
template cudaError_t launch_nl_restrict<double>(const NLArgs<double> &, const Geom &,
                                                const double *, const double *, double *,
                                                double *, cudaStream_t);
template cudaError_t launch_nl_lambda<double>(const NLArgs<double> &, double *, cudaStream_t);
template cudaError_t launch_vc_op<double>(const VCArgs<double> &, int, int, const double *,
                                          const double *, double *, int, double *, int *,
                                          cudaStream_t);
template cudaError_t launch_vc_update_residual<double, double>(const VCArgs<double> &, int,
                                                               const double *, const double *,
                                                               const double *, double *,
                                                               double *, double *, double *,
                                                               int *, cudaStream_t, const int *);
template cudaError_t launch_vc_update_residual<double, float>(const VCArgs<double> &, int,
                                                              const double *, const float *,
                                                              const double *, double *, double *,
                                                              float *, double *, int *,
                                                              cudaStream_t, const int *);

cudaError_t launch_vc_outer_fast(const OuterFast &P, int norm, cudaStream_t s) {
  if (P.G.dim != 2 || !P.count || !P.part || !P.res_inner) return cudaErrorInvalidValue;
  long long tiles = (long long)((P.G.n0 + kOTX - 1) / kOTX) * ((P.G.n1 + kOTY - 1) / kOTY);
  int grid = (int)(tiles < kMaxBlocks ? tiles : kMaxBlocks);
  MLGPU_NORM_SWITCH(norm, (vc_outer_fast_kernel<NORM><<<grid, kOTThreads, 0, s>>>(P)));
  return cudaGetLastError();
}

cudaError_t launch_hcm_jac(const Geom &G, const ClosureParams &cp, const double *u, float *J,
                           cudaStream_t s) {
  hcm_jac_kernel<<<blocks_for(G.ncell), kBlock, 0, s>>>(G, cp, u, J);
  return cudaGetLastError();
}

cudaError_t launch_hcm_update(long long n, double *u, const float *e, cudaStream_t s) {
  hcm_update_kernel<<<blocks_for(n), kBlock, 0, s>>>(n, u, e);
  return cudaGetLastError();
}

cudaError_t launch_outer_coefs(const VCArgs<double> &A, double *cx, double *cy, double *diag,
                               cudaStream_t s) {
  if (A.G.dim != 2) return cudaErrorInvalidValue;
  long long n = A.G.nface(0) > A.G.ncell ? A.G.nface(0) : A.G.ncell;
  if (A.G.nface(1) > n) n = A.G.nface(1);
  outer_coefs_kernel<<<blocks_for(n), kBlock, 0, s>>>(A, cx, cy, diag);
  return cudaGetLastError();
}

cudaError_t launch_outer_decide(OuterDev *st, const double *norm, const OuterCfg &c,
                                cudaGraphConditionalHandle h, cudaStream_t s) {
  outer_decide_kernel<<<1, 1, 0, s>>>(st, norm, c, h);
  return cudaGetLastError();
}
template cudaError_t launch_vc_gsrb<double>(const VCArgs<double> &, double *, const double *, int,
                                            cudaStream_t);
template cudaError_t launch_vc_gsrb_zero<double>(const VCArgs<double> &, double *, const double *,
                                                 cudaStream_t);
template cudaError_t launch_vc_relax_block<double>(const VCArgs<double> &, double *,
                                                   const double *, int, int, cudaStream_t);
template cudaError_t launch_vc_restrict<double>(const VCArgs<double> &, const Geom &,
                                                const double *, const double *, double *,
                                                double *, cudaStream_t);
template cudaError_t launch_vc_lambda<double>(const VCArgs<double> &, double *, cudaStream_t);
template cudaError_t launch_restrict_avg<double>(const Geom &, int, const double *, double *,
                                                 cudaStream_t);
template cudaError_t launch_prolong<double>(const Geom &, const BCD &, int, int, double *,
                                            const double *, const double *, cudaStream_t);
template cudaError_t launch_coarsen_faces<double>(const Geom &, int, int, const double *, double *,
                                                  cudaStream_t);
template cudaError_t launch_axpby<double>(long long, double, const double *, double, double *,
                                          cudaStream_t);
template cudaError_t launch_norm_partial<double>(long long, const double *, int, double *, int *,
                                                 cudaStream_t);
template cudaError_t launch_convert<double, float>(long long, double *, const float *,
                                                   cudaStream_t);
template cudaError_t launch_convert<double, double>(long long, double *, const double *,
                                                    cudaStream_t);

cudaError_t launch_finalize_norm(int norm, const double *part, int nparts, double *out,
                                 cudaStream_t s) {
  // nparts comes from the launch that wrote the partials; 0 means it wrote none
  if (nparts < 1 || nparts > kMaxBlocks) return cudaErrorInvalidValue;
  switch (norm) {
    case MLGPU_NORM_L1:
      finalize_norm_kernel<MLGPU_NORM_L1><<<1, 1024, 0, s>>>(part, nparts, out);
      break;
    case MLGPU_NORM_L2:
      finalize_norm_kernel<MLGPU_NORM_L2><<<1, 1024, 0, s>>>(part, nparts, out);
      break;
    default:
      finalize_norm_kernel<MLGPU_NORM_MAX><<<1, 1024, 0, s>>>(part, nparts, out);
      break;
  }
  return cudaGetLastError();
}

// full closure / MAC helpers are FP64-only and live in this unit too
cudaError_t launch_closure_full(long long n, const ClosureParams &p, const double *HC, double *T,
                                double *por, double *Cl, double *Cs, double *Hs, double *He,
                                double *Hl, cudaStream_t s) {
  closure_full_kernel<<<blocks_for(n), kBlock, 0, s>>>(n, p, HC, T, por, Cl, Cs, Hs, He, Hl);
  return cudaGetLastError();
}
cudaError_t launch_closure_tcl(long long n, const ClosureParams &p, const double *HC, double *TCl,
                               cudaStream_t s) {
  closure_tcl_kernel<<<blocks_for(n), kBlock, 0, s>>>(n, p, HC, TCl);
  return cudaGetLastError();
}

cudaError_t launch_add_dt_src(long long n, double *out, const double *src, double dt,
                              cudaStream_t s) {
  add_dt_src_kernel<<<blocks_for(n), kBlock, 0, s>>>(n, out, src, dt);
  return cudaGetLastError();
}
cudaError_t launch_scale_by_a(long long n, const double *x, const double *a, double *out,
                              cudaStream_t s) {
  scale_by_a_kernel<<<blocks_for(n), kBlock, 0, s>>>(n, x, a, out);
  return cudaGetLastError();
}

cudaError_t launch_closure_tcl_lean(long long n, const ClosureParams &p, const double *HC,
                                   double *TCl, cudaStream_t s) {
  closure_tcl_lean_kernel<<<blocks_for(n), kBlock, 0, s>>>(n, make_closure_lean(p), HC, TCl);
  return cudaGetLastError();
}
cudaError_t launch_face_geomean(const Geom &G, int d, const double *cell, double *face,
                                cudaStream_t s) {
  face_geomean_kernel<<<blocks_for(G.nface(d)), kBlock, 0, s>>>(G, d, cell, face);
  return cudaGetLastError();
}
cudaError_t launch_mac_div(const Geom &G, const double *u0, const double *u1, const double *u2,
                           double *div, cudaStream_t s) {
  mac_div_kernel<<<blocks_for(G.ncell), kBlock, 0, s>>>(G, u0, u1, u2, div);
  return cudaGetLastError();
}
cudaError_t launch_mac_correct(const Geom &G, const BCD &bc, int d, const double *phi,
                               const double *scale, double *u, cudaStream_t s) {
  mac_correct_kernel<<<blocks_for(G.nface(d)), kBlock, 0, s>>>(G, bc, d, phi, scale, u);
  return cudaGetLastError();
}
cudaError_t launch_be_rhs(long long n, const double *phi_old, const double *a, const double *src,
                          double dt, double *rhs, cudaStream_t s) {
  be_rhs_kernel<<<blocks_for(n), kBlock, 0, s>>>(n, phi_old, a, src, dt, rhs);
  return cudaGetLastError();
}

// ---- adjoint
cudaError_t launch_mac_grad_t(const Geom &G, const BCD &bc, const double *const y[3],
                              const double *const scale[3], double *r, cudaStream_t s) {
  mac_grad_t_kernel<<<blocks_for(G.ncell), kBlock, 0, s>>>(G, bc, y[0], y[1], y[2], scale[0],
                                                           scale[1], scale[2], r);
  return cudaGetLastError();
}
cudaError_t launch_mac_div_t(const Geom &G, int d, const double *q, const double *ubar,
                             double *out, cudaStream_t s) {
  mac_div_t_kernel<<<blocks_for(G.nface(d)), kBlock, 0, s>>>(G, d, q, ubar, out);
  return cudaGetLastError();
}
cudaError_t launch_mac_pi_bar(const Geom &G, const BCD &bc, int d, const double *phi,
                              const double *usb, double *pib, cudaStream_t s) {
  mac_pi_bar_kernel<<<blocks_for(G.nface(d)), kBlock, 0, s>>>(G, bc, d, phi, usb, pib);
  return cudaGetLastError();
}
cudaError_t launch_be_adj(long long n, const double *mu, const double *a, double dt,
                          double *old_bar, double *src_bar, cudaStream_t s) {
  be_adj_kernel<<<blocks_for(n), kBlock, 0, s>>>(n, mu, a, dt, old_bar, src_bar);
  return cudaGetLastError();
}

}  // namespace mlgpu

namespace mlgpu {
template cudaError_t launch_vc_block_cycle<double>(const VCBlockCycle<double> &, cudaStream_t);
template cudaError_t launch_vc_tile_smooth<double>(const TileSmooth<double> &, cudaStream_t);

int tile_max_halo(size_t elem) {
  int h = 0;
  while (tile_smem_bytes(h + 1, elem) <= kMaxDynSmem) h++;
  return h;
}
}
