// capi_internal.h -- declarations shared by the C-ABI units (capi.cu,
// solver.cu): descriptor conversion and the FP64-only launchers.
#pragma once
#include "launch.h"
#include "nl_kernels.cuh"
#include "vc_kernels.cuh"
#include "cycle_kernels.cuh"
#include "tile_kernels.cuh"
#include "tile_fast_kernels.cuh"
#include "cycle_fast_kernels.cuh"
#include "outer_kernels.cuh"
#include "outer_fast_kernels.cuh"
#include "nl_cached_kernels.cuh"
#include "hcm_kernels.cuh"
#include "adjoint_kernels.cuh"
#include "bicgstab_kernels.cuh"
#include "lin_lean_kernels.cuh"
#include "vc_lean_kernels.cuh"

namespace mlgpu {

bool valid_grid(const mlgpu_grid *g);
bool valid_vcop(const mlgpu_vcop *op);
bool valid_bc(const mlgpu_bc &b, int dim, bool temperature_h);
bool valid_nl_bcs(const mlgpu_nlop &op);
bool valid_adjoint_op(const mlgpu_nlop *op);
AdjArgs<double> make_adj_args(const mlgpu_nlop &op, const double *phi, const double *J);
template <class T> NLArgs<T> make_nl_args(const mlgpu_nlop &op);
template <class T> VCArgs<T> make_vc_args(const mlgpu_vcop &op);
int status_of(cudaError_t e);
int finish_norm(int norm_type, double *part, int nparts, double *host_out, cudaStream_t s);

cudaError_t launch_closure_full(long long n, const ClosureParams &p, const double *HC, double *T,
                                double *por, double *Cl, double *Cs, double *Hs, double *He,
                                double *Hl, cudaStream_t s);
cudaError_t launch_closure_tcl(long long n, const ClosureParams &p, const double *HC, double *TCl,
                               cudaStream_t s);
// TGA pieces: out += dt src; out = a x (a null: a == 1)
cudaError_t launch_add_dt_src(long long n, double *out, const double *src, double dt,
                              cudaStream_t s);
cudaError_t launch_scale_by_a(long long n, const double *x, const double *a, double *out,
                              cudaStream_t s);
cudaError_t launch_closure_tcl_lean(long long n, const ClosureParams &p, const double *HC,
                                   double *TCl, cudaStream_t s);
cudaError_t launch_face_geomean(const Geom &G, int d, const double *cell, double *face,
                                cudaStream_t s);
cudaError_t launch_mac_div(const Geom &G, const double *u0, const double *u1, const double *u2,
                           double *div, cudaStream_t s);
cudaError_t launch_mac_correct(const Geom &G, const BCD &bc, int d, const double *phi,
                               const double *scale, double *u, cudaStream_t s);
cudaError_t launch_be_rhs(long long n, const double *phi_old, const double *a, const double *src,
                          double dt, double *rhs, cudaStream_t s);
cudaError_t launch_vc_outer_fast(const OuterFast &P, int norm, cudaStream_t s);
// adjoint (adjoint_kernels.cuh, misc_kernels.cuh)
cudaError_t launch_mac_grad_t(const Geom &G, const BCD &bc, const double *const y[3],
                              const double *const scale[3], double *r, cudaStream_t s);
cudaError_t launch_mac_div_t(const Geom &G, int d, const double *q, const double *ubar,
                             double *out, cudaStream_t s);
cudaError_t launch_mac_pi_bar(const Geom &G, const BCD &bc, int d, const double *phi,
                              const double *usb, double *pib, cudaStream_t s);
cudaError_t launch_be_adj(long long n, const double *mu, const double *a, double dt,
                          double *old_bar, double *src_bar, cudaStream_t s);
cudaError_t launch_adj_jac(const Geom &G, const ClosureParams &cp, const double *u, double *J,
                           cudaStream_t s);
cudaError_t launch_porosity_jac(const Geom &G, const ClosureParams &cp, const double *u,
                                double *dp, cudaStream_t s);
// tr: A^T (the adjoint) or A (the linearised operator of a Newton step)
cudaError_t launch_adj_op(const AdjArgs<double> &A, int mode, int norm, const double *y,
                          const double *g, double *out, double *part, int *nparts,
                          cudaStream_t s, bool tr = true);
cudaError_t launch_adj_gsrb(const AdjArgs<double> &A, double *y, const double *g, int pass,
                            cudaStream_t s, bool tr = true);
cudaError_t launch_adj_relax_block(const AdjArgs<double> &A, double *y, const double *g,
                                   int sweeps, int zero, cudaStream_t s, bool tr = true);
cudaError_t launch_adj_restrict(const AdjArgs<double> &A, const Geom &C, const double *y,
                                const double *g, double *gc, cudaStream_t s, bool tr = true);
cudaError_t launch_adj_bottom_direct(const AdjArgs<double> &A, double *y, const double *g,
                                     cudaStream_t s, bool tr = true);
// inverse diagonal blocks of A^T per cell (`zero`: a zero field of the level)
cudaError_t launch_adj_minv(const AdjArgs<double> &A, const double *zero, double *Minv,
                            double *D, cudaStream_t s);
cudaError_t launch_adj_bc_grad(const AdjArgs<double> &A, const double *y, double *out,
                               cudaStream_t s);
cudaError_t launch_outer_coefs(const VCArgs<double> &A, double *cx, double *cy, double *diag,
                               cudaStream_t s);
// mixed-precision nonlinear solve: FP64 closure Jacobian (stored FP32), u += e
cudaError_t launch_hcm_jac(const Geom &G, const ClosureParams &cp, const double *u, float *J,
                           cudaStream_t s);
cudaError_t launch_hcm_update(long long n, double *u, const float *e, cudaStream_t s);
// BiCGStab bottom solve of L e = rhs on one level (FP64 arithmetic, storage S)
template <class S>
cudaError_t launch_vc_bicgstab(const VCArgs<double> &A, S *e, const S *rhs, double *ws,
                               int imax, int remove_mean, cudaStream_t s);
// FP32 Jacobian cycles of the mixed-precision Newton solve (launch_f32_adj.cu)
cudaError_t launch_adj_jac(const Geom &G, const ClosureParams &cp, const double *u, float *J,
                           cudaStream_t s);
cudaError_t launch_adj_op(const AdjArgs<float> &A, int mode, int norm, const float *y,
                          const float *g, float *out, double *part, int *nparts, cudaStream_t s,
                          bool tr);
cudaError_t launch_adj_gsrb(const AdjArgs<float> &A, float *y, const float *g, int pass,
                            cudaStream_t s, bool tr);
cudaError_t launch_adj_relax_block(const AdjArgs<float> &A, float *y, const float *g, int sweeps,
                                   int zero, cudaStream_t s, bool tr);
cudaError_t launch_adj_minv(const AdjArgs<float> &A, const float *zero, float *Minv, float *D,
                            cudaStream_t s);
// lean cycles of the Newton step (lin_lean_kernels.cuh); T = float or double;
// fine-level arrays colour-split, the coarse level's split when csplit
// vec: the vector-load kernel where the level's rows allow it (the same bits)
template <class T>
cudaError_t launch_lean_gsrb(const LinLeanT<T> &P, int pass, cudaStream_t s, int vec = 0);
// red: the red half's residual only (after a black half sweep); black: the
// black half's prolongation only (before a red half sweep); vec: the red
// residual and restriction by vector groups where the rows allow it (the
// same per-cell bits)
template <class T>
cudaError_t launch_lean_residual(const LinLeanT<T> &P, int split, int red, int norm,
                                 double *part, int *nparts, cudaStream_t s, int vec = 0);
template <class T>
cudaError_t launch_lean_restrict(const LinLeanT<T> &P, const Geom &C, int csplit, int red, T *gc,
                                 T *xc, T *wc, cudaStream_t s, int vec = 0);
template <class T>
cudaError_t launch_lean_prolong(const LinLeanT<T> &P, const Geom &C, int csplit, int black,
                                int kind, const T *xc, cudaStream_t s);
// lean cycles of the linear operator on 3D levels (vc_lean_kernels.cuh; T =
// float for the mixed solve, double for the comparison path): diag and 1/diag
// to the split layout (once per solver), red/black half sweep (zero: the
// other colour's e is zero), residual restriction (red: the red children
// only) with the coarse e zeroed, black-only prolongation, and the FP64 outer
// step with a lean level 0 (e, res_inner split, in the cycles' precision E)
template <class T>
cudaError_t launch_vcl_diag(const VCArgs<T> &A, T *idg, T *dg, cudaStream_t s);
template <class T>
cudaError_t launch_vcl_gsrb(const VCLeanT<T> &P, int pass, int zero, cudaStream_t s,
                            int vec = 1);
template <class T>
cudaError_t launch_vcl_restrict(const VCLeanT<T> &P, const Geom &C, int csplit, int red, T *rc,
                                T *ec, cudaStream_t s);
template <class T>
cudaError_t launch_vcl_prolong(const VCLeanT<T> &P, const Geom &C, const BCD &bc, int csplit,
                               int black, int kind, const T *ec, cudaStream_t s);
template <class E>
cudaError_t launch_vcl_outer(const VCArgs<double> &A, int norm, const double *phi, const E *e,
                             const double *rhs, double *out_phi, E *res_inner, double *part,
                             int *nparts, cudaStream_t s, const int *par = nullptr);
// per-cell face sums P of a smoothed level (natural layout), once per solver
template <class T>
cudaError_t launch_lean_psum(const AdjArgs<T> &A, T *P, cudaStream_t s);
// J, K, D of a smoothed level from the state u and P, in the split layout
template <class T>
cudaError_t launch_lean_state(const AdjArgs<T> &A, const double *u, const T *P, T *Js, T *Ks,
                              T *Ds, cudaStream_t s);
template <class T, class S>
cudaError_t launch_lean_pack(const Geom &G, int split, int ncomp, const S *src, T *dst,
                             cudaStream_t s);
// clip: the regime clipping of the update, or null for u = u_old + scale e
template <class T>
cudaError_t launch_lean_step(const Geom &G, int split, const StepClip *clip, double *u,
                             const double *u_old, double scale, const T *e, cudaStream_t s);
cudaError_t launch_adj_bottom_direct(const AdjArgs<float> &A, float *y, const float *g,
                                     cudaStream_t s, bool tr);
cudaError_t launch_adj_restrict(const AdjArgs<float> &A, const Geom &C, const float *y,
                                const float *g, float *gc, cudaStream_t s, bool tr);
// FP64 nonlinear kernels over the per-level (T, C_l) cache
// lean: t_cl_lean (the lean Newton paths' closure) instead of t_cl
cudaError_t launch_nlc_closure(const NLArgs<double> &A, const double *phi, double *tcl,
                               cudaStream_t s, int lean = 0);
cudaError_t launch_nlc_gsrb(const NLArgs<double> &A, double *phi, const double *rhs, double *tcl,
                            const double *lam, int pass, cudaStream_t s);
cudaError_t launch_nlc_relax_block(const NLArgs<double> &A, double *phi, const double *rhs,
                                   double *tcl, const double *lam, int sweeps, int init,
                                   cudaStream_t s);
// the lean Newton paths' residual rhs - N(phi) over the cache, with its L2
// (part) and max (part_max) norm partials; sb: every cell's face sum per
// component (launch_nlc_bsum, once per solver)
cudaError_t launch_nlc_bsum(const NLArgs<double> &A, double *sb, cudaStream_t s);
cudaError_t launch_nlc_res_lean(const NLArgs<double> &A, const double *phi, const double *tcl,
                                const double *sb, const double *rhs, double *out, double *part,
                                double *part_max, int *nparts, cudaStream_t s);
// part_max: with a norm, the max-norm partials too (same count)
cudaError_t launch_nlc_op(const NLArgs<double> &A, int mode, int norm, const double *phi,
                          const double *tcl, const double *rhs, double *out, double *copy,
                          double *part, int *nparts, cudaStream_t s,
                          double *part_max = nullptr);
cudaError_t launch_nlc_restrict(const NLArgs<double> &A, const Geom &C, const double *phi,
                                const double *tcl, const double *rhs, double *res_c,
                                double *phi_c, cudaStream_t s);
cudaError_t launch_outer_decide(OuterDev *st, const double *norm, const OuterCfg &c,
                                cudaGraphConditionalHandle h, cudaStream_t s);

}  // namespace mlgpu
