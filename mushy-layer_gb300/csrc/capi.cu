// capi.cu -- extern "C" entry points of include/mlgpu.h (kernel level).
// Each call validates its arguments, converts the POD descriptors into
// kernel arguments and launches on the caller's stream.  No entry point
// allocates device memory; reductions use the caller's workspace.
#include <cstring>
#include "capi_internal.h"

namespace mlgpu {

bool valid_grid(const mlgpu_grid *g) {
  if (!g) return false;
  if (g->dim != 2 && g->dim != 3) return false;
  for (int d = 0; d < g->dim; d++)
    if (g->n[d] < 1) return false;
  if (g->dim == 2 && g->n[2] != 1) return false;
  if (!(g->dx > 0)) return false;
  // 32-bit index arithmetic in the kernels: two components of the box plus
  // one face layer must stay below 2^31 entries
  long long cells = (long long)g->n[0] * g->n[1] * g->n[2];
  if (2 * (cells + (long long)g->n[0] * g->n[1] + (long long)g->n[1] * g->n[2] +
           (long long)g->n[0] * g->n[2]) >= (1LL << 31))
    return false;
  return true;
}

template <class T>
NLArgs<T> make_nl_args(const mlgpu_nlop &op) {
  NLArgs<T> A;
  A.G = make_geom(op.grid);
  A.cp = make_cp(op.params);
  A.phi_bc = make_bcd(op.phi_bc);
  A.dbc = make_dbcd(op.derived_bc, op.nlbc, op.grid.dx);
  A.nlbc = make_nlbcd(op.phi_bc, op.nlbc, op.grid.dx);
  A.apply_dbc = op.apply_derived_bc;
  double dxinv = 1.0 / (op.grid.dx * op.grid.dx);
  A.alpha = (T)op.alpha;
  A.beta = (T)op.beta;
  A.dxinv = (T)dxinv;
  A.dx = (T)op.grid.dx;
  A.a = (const T *)op.aCoef;
  for (int d = 0; d < 3; d++) A.b[d] = (const T *)op.bCoef[d];
  return A;
}
template NLArgs<double> make_nl_args<double>(const mlgpu_nlop &);
template NLArgs<float> make_nl_args<float>(const mlgpu_nlop &);

template <class T>
VCArgs<T> make_vc_args(const mlgpu_vcop &op) {
  VCArgs<T> A;
  A.G = make_geom(op.grid);
  A.bc = make_bcd(op.bc);
  double dxinv = 1.0 / (op.grid.dx * op.grid.dx);
  A.alpha = (T)op.alpha;
  A.beta = (T)op.beta;
  A.dxinv = (T)dxinv;
  A.dx = (T)op.grid.dx;
  A.a = (const T *)op.aCoef;
  A.c = (const T *)op.cCoef;
  for (int d = 0; d < 3; d++) A.b[d] = (const T *)op.bCoef[d];
  A.lam = nullptr;
  return A;
}
template VCArgs<double> make_vc_args<double>(const mlgpu_vcop &);
template VCArgs<float> make_vc_args<float>(const mlgpu_vcop &);

int status_of(cudaError_t e) { return e == cudaSuccess ? MLGPU_OK : MLGPU_ERR_CUDA; }

// BC types: Neumann/Dirichlet everywhere, temperature conditions only on
// component 0 of a nonlinear operator's (H, C) condition
bool valid_bc(const mlgpu_bc &b, int dim, bool temperature_h) {
  for (int d = 0; d < dim; d++)
    for (int s = 0; s < 2; s++)
      for (int c = 0; c < 2; c++) {
        const int t = b.type[d][s][c];
        if (t == MLGPU_BC_NEUMANN || t == MLGPU_BC_DIRICHLET) continue;
        if (temperature_h && c == 0 && is_temperature_bc(t)) continue;
        return false;
      }
  return true;
}

// derived conditions: Neumann/Dirichlet, and the mixed temperature condition
// on comp 0 (T) only
static bool valid_derived_bc(const mlgpu_bc &b, int dim) {
  for (int d = 0; d < dim; d++)
    for (int s = 0; s < 2; s++)
      for (int c = 0; c < 2; c++) {
        const int t = b.type[d][s][c];
        if (t == MLGPU_BC_NEUMANN || t == MLGPU_BC_DIRICHLET) continue;
        if (c == 0 && t == MLGPU_BC_MIXED_TEMPERATURE_SALINITY) continue;
        return false;
      }
  return true;
}

bool valid_nl_bcs(const mlgpu_nlop &op) {
  if (!valid_bc(op.phi_bc, op.grid.dim, true) || !valid_derived_bc(op.derived_bc, op.grid.dim))
    return false;
  const mlgpu_nlbc &n = op.nlbc;
  if (n.method != MLGPU_NLBC_PICARD && n.method != MLGPU_NLBC_NEWTON) return false;
  if (n.max_iter < 0 || !(n.dx >= 0)) return false;
  // a Robin denominator a/dx - b/2 of zero has no ghost value
  const double dxb = n.dx > 0 ? n.dx : op.grid.dx;
  for (int d = 0; d < op.grid.dim; d++)
    for (int s = 0; s < 2; s++) {
      const bool robin_h = op.phi_bc.type[d][s][0] == MLGPU_BC_TEMPERATURE_FLUX_RADIATION;
      const bool robin_t = op.apply_derived_bc &&
                           op.derived_bc.type[d][s][0] == MLGPU_BC_MIXED_TEMPERATURE_SALINITY;
      if ((robin_h || robin_t) && !(n.a[d][s] / dxb - n.b[d][s] / 2 != 0)) return false;
    }
  return true;
}

static bool valid_nlop(const mlgpu_nlop *op) {
  if (!op || !valid_grid(&op->grid)) return false;
  if (!valid_nl_bcs(*op)) return false;
  if (op->dtype != MLGPU_F64 && op->dtype != MLGPU_F32) return false;
  for (int d = 0; d < op->grid.dim; d++)
    if (!op->bCoef[d]) return false;
  return true;
}

bool valid_vcop(const mlgpu_vcop *op) {
  if (!op || !valid_grid(&op->grid)) return false;
  if (!valid_bc(op->bc, op->grid.dim, false)) return false;
  if (op->dtype != MLGPU_F64 && op->dtype != MLGPU_F32) return false;
  for (int d = 0; d < op->grid.dim; d++)
    if (!op->bCoef[d]) return false;
  return true;
}

// the adjoint differentiates the linear wall rules only
bool valid_adjoint_op(const mlgpu_nlop *op) {
  if (!valid_nlop(op) || op->dtype != MLGPU_F64) return false;
  for (int d = 0; d < 3; d++)
    for (int s = 0; s < 2; s++)
      if (is_temperature_bc(op->phi_bc.type[d][s][0])) return false;
  return true;
}

AdjArgs<double> make_adj_args(const mlgpu_nlop &op, const double *phi, const double *J) {
  NLArgs<double> N = make_nl_args<double>(op);
  AdjArgs<double> A;
  A.G = N.G;
  A.cp = N.cp;
  A.phi_bc = N.phi_bc;
  A.dbc = N.dbc;
  A.apply_dbc = N.apply_dbc;
  A.alpha = N.alpha;
  A.beta = N.beta;
  A.dxinv = N.dxinv;
  A.dx = N.dx;
  A.a = N.a;
  for (int d = 0; d < 3; d++) A.b[d] = N.b[d];
  A.J = J;
  A.u = phi;
  return A;
}

static bool coarsenable(const mlgpu_grid &g) {
  for (int d = 0; d < g.dim; d++)
    if (g.n[d] % 2) return false;
  return true;
}

// finish a fused norm: combine partials and copy the result to the host
int finish_norm(int norm_type, double *part, int nparts, double *host_out, cudaStream_t s) {
  double *res = part + kMaxBlocks;
  cudaError_t e = launch_finalize_norm(norm_type, part, nparts, res, s);
  if (e != cudaSuccess) return MLGPU_ERR_CUDA;
  e = cudaMemcpyAsync(host_out, res, sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return MLGPU_ERR_CUDA;
  e = cudaStreamSynchronize(s);
  return status_of(e);
}

}  // namespace mlgpu

using namespace mlgpu;

extern "C" {

const char *mlgpu_status_string(int status) {
  switch (status) {
    case MLGPU_OK: return "ok";
    case MLGPU_ERR_ARG: return "invalid argument";
    case MLGPU_ERR_CUDA: return "CUDA runtime error";
    case MLGPU_ERR_NAN: return "NaN or Inf in residual";
    case MLGPU_ERR_NOT_CONVERGED: return "not converged";
    case MLGPU_ERR_WORKSPACE: return "workspace too small or misaligned";
    case MLGPU_ERR_HANG: return "solver hung (residual stopped decreasing)";
    case MLGPU_ERR_SCRATCH: return "request exceeds the fixed scratch area";
    default: return "unknown status";
  }
}

int mlgpu_version(void) { return 1; }

size_t mlgpu_norm_workspace_bytes(void) { return kNormScratchDoubles * sizeof(double); }

int mlgpu_closure(const mlgpu_grid *g, const mlgpu_params *p, const double *HC, double *T,
                  double *por, double *Cl, double *Cs, double *Hs, double *He, double *Hl,
                  void *stream) {
  if (!valid_grid(g) || !p || !HC) return MLGPU_ERR_ARG;
  Geom G = make_geom(*g);
  return status_of(launch_closure_full(G.ncell, make_cp(*p), HC, T, por, Cl, Cs, Hs, He, Hl,
                                       (cudaStream_t)stream));
}

int mlgpu_closure_tcl(const mlgpu_grid *g, const mlgpu_params *p, const double *HC,
                      double *TCl, void *stream) {
  if (!valid_grid(g) || !p || !HC || !TCl) return MLGPU_ERR_ARG;
  Geom G = make_geom(*g);
  return status_of(launch_closure_tcl(G.ncell, make_cp(*p), HC, TCl, (cudaStream_t)stream));
}

int mlgpu_closure_tcl_lean(const mlgpu_grid *g, const mlgpu_params *p, const double *HC,
                           double *TCl, void *stream) {
  if (!valid_grid(g) || !p || !HC || !TCl) return MLGPU_ERR_ARG;
  Geom G = make_geom(*g);
  return status_of(
      launch_closure_tcl_lean(G.ncell, make_cp(*p), HC, TCl, (cudaStream_t)stream));
}

int mlgpu_device_alloc(size_t bytes, void **ptr) {
  if (!ptr) return MLGPU_ERR_ARG;
  *ptr = nullptr;
  if (bytes == 0) return MLGPU_OK;
  return status_of(cudaMalloc(ptr, bytes));
}

int mlgpu_device_free(void *ptr) { return ptr ? status_of(cudaFree(ptr)) : MLGPU_OK; }

int mlgpu_memcpy(void *dst, const void *src, size_t bytes, int kind, void *stream) {
  if ((!dst || !src) && bytes) return MLGPU_ERR_ARG;
  cudaMemcpyKind k = kind == 0   ? cudaMemcpyHostToDevice
                     : kind == 1 ? cudaMemcpyDeviceToHost
                     : kind == 2 ? cudaMemcpyDeviceToDevice
                                 : cudaMemcpyDefault;
  if (kind < 0 || kind > 2) return MLGPU_ERR_ARG;
  if (!bytes) return MLGPU_OK;
  return status_of(cudaMemcpyAsync(dst, src, bytes, k, (cudaStream_t)stream));
}

int mlgpu_memset_zero(void *ptr, size_t bytes, void *stream) {
  if (!ptr && bytes) return MLGPU_ERR_ARG;
  if (!bytes) return MLGPU_OK;
  return status_of(cudaMemsetAsync(ptr, 0, bytes, (cudaStream_t)stream));
}

int mlgpu_stream_synchronize(void *stream) {
  return status_of(cudaStreamSynchronize((cudaStream_t)stream));
}

int mlgpu_closure_jacobian(const mlgpu_grid *g, const mlgpu_params *p, const double *HC,
                           double *J, void *stream) {
  if (!valid_grid(g) || !p || !HC || !J) return MLGPU_ERR_ARG;
  return status_of(launch_adj_jac(make_geom(*g), make_cp(*p), HC, J, (cudaStream_t)stream));
}

int mlgpu_porosity_jacobian(const mlgpu_grid *g, const mlgpu_params *p, const double *HC,
                            double *dpor, void *stream) {
  if (!valid_grid(g) || !p || !HC || !dpor) return MLGPU_ERR_ARG;
  return status_of(
      launch_porosity_jac(make_geom(*g), make_cp(*p), HC, dpor, (cudaStream_t)stream));
}

int mlgpu_hc_adjoint_apply(const mlgpu_nlop *op, const double *phi, const double *J,
                           const double *y, const double *g, double *out, void *stream) {
  if (!valid_adjoint_op(op) || !phi || !J || !y || !out) return MLGPU_ERR_ARG;
  return status_of(launch_adj_op(make_adj_args(*op, phi, J), g ? ADJ_RESIDUAL : ADJ_APPLY, -1,
                                 y, g, out, nullptr, nullptr, (cudaStream_t)stream));
}

int mlgpu_hc_adjoint_gsrb_pass(const mlgpu_nlop *op, const double *phi, const double *J,
                               double *y, const double *g, int pass, void *stream) {
  if (!valid_adjoint_op(op) || !phi || !J || !y || !g || (pass != 0 && pass != 1))
    return MLGPU_ERR_ARG;
  return status_of(launch_adj_gsrb(make_adj_args(*op, phi, J), y, g, pass, (cudaStream_t)stream));
}

int mlgpu_hc_linearized_apply(const mlgpu_nlop *op, const double *phi, const double *J,
                              const double *x, const double *r, double *out, void *stream) {
  if (!valid_adjoint_op(op) || !phi || !J || !x || !out) return MLGPU_ERR_ARG;
  return status_of(launch_adj_op(make_adj_args(*op, phi, J), r ? ADJ_RESIDUAL : ADJ_APPLY, -1, x,
                                 r, out, nullptr, nullptr, (cudaStream_t)stream, false));
}

int mlgpu_hc_linearized_gsrb_pass(const mlgpu_nlop *op, const double *phi, const double *J,
                                  double *x, const double *r, int pass, void *stream) {
  if (!valid_adjoint_op(op) || !phi || !J || !x || !r || (pass != 0 && pass != 1))
    return MLGPU_ERR_ARG;
  return status_of(
      launch_adj_gsrb(make_adj_args(*op, phi, J), x, r, pass, (cudaStream_t)stream, false));
}

int mlgpu_hc_adjoint_restrict(const mlgpu_nlop *op, const double *phi, const double *J,
                              const double *y, const double *g, double *gc, void *stream) {
  if (!valid_adjoint_op(op) || !phi || !J || !y || !g || !gc || !coarsenable(op->grid))
    return MLGPU_ERR_ARG;
  mlgpu_grid cg = op->grid;
  for (int d = 0; d < cg.dim; d++) cg.n[d] /= 2;
  cg.dx *= 2;
  return status_of(launch_adj_restrict(make_adj_args(*op, phi, J), make_geom(cg), y, g, gc,
                                       (cudaStream_t)stream));
}

int mlgpu_nl_residual(const mlgpu_nlop *op, void *res, const void *phi, const void *rhs,
                      int norm_type, double *norm, void *ws, size_t ws_bytes, void *stream) {
  if (!valid_nlop(op) || !res || !phi || !rhs) return MLGPU_ERR_ARG;
  if (norm_type > MLGPU_NORM_L2) return MLGPU_ERR_ARG;
  bool want = norm_type >= 0;
  if (want && (!norm || !ws)) return MLGPU_ERR_ARG;
  if (want && ws_bytes < mlgpu_norm_workspace_bytes()) return MLGPU_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  double *part = want ? (double *)ws : nullptr;
  int nt = want ? norm_type : -1, nparts = 0;
  cudaError_t e;
  if (op->dtype == MLGPU_F64)
    e = launch_nl_op<double>(make_nl_args<double>(*op), NL_RESIDUAL, nt, (const double *)phi,
                             (const double *)rhs, (double *)res, nullptr, part, &nparts, s);
  else
    e = launch_nl_op<float>(make_nl_args<float>(*op), NL_RESIDUAL, nt, (const float *)phi,
                            (const float *)rhs, (float *)res, nullptr, part, &nparts, s);
  if (e != cudaSuccess) return MLGPU_ERR_CUDA;
  if (!want) return MLGPU_OK;
  return finish_norm(norm_type, part, nparts, norm, s);
}

int mlgpu_nl_apply(const mlgpu_nlop *op, void *lhs, const void *phi, void *stream) {
  if (!valid_nlop(op) || !lhs || !phi) return MLGPU_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e;
  if (op->dtype == MLGPU_F64)
    e = launch_nl_op<double>(make_nl_args<double>(*op), NL_APPLY, -1, (const double *)phi,
                             nullptr, (double *)lhs, nullptr, nullptr, nullptr, s);
  else
    e = launch_nl_op<float>(make_nl_args<float>(*op), NL_APPLY, -1, (const float *)phi, nullptr,
                            (float *)lhs, nullptr, nullptr, nullptr, s);
  return status_of(e);
}

int mlgpu_nl_gsrb_pass(const mlgpu_nlop *op, void *phi, const void *rhs, int pass,
                       void *stream) {
  if (!valid_nlop(op) || !phi || !rhs || (pass != 0 && pass != 1)) return MLGPU_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e;
  if (op->dtype == MLGPU_F64)
    e = launch_nl_gsrb<double>(make_nl_args<double>(*op), (double *)phi, (const double *)rhs,
                               pass, s);
  else
    e = launch_nl_gsrb<float>(make_nl_args<float>(*op), (float *)phi, (const float *)rhs, pass, s);
  return status_of(e);
}

int mlgpu_nl_relax(const mlgpu_nlop *op, void *phi, const void *rhs, int n, void *stream) {
  if (n < 0) return MLGPU_ERR_ARG;
  for (int i = 0; i < n; i++)
    for (int pass = 0; pass < 2; pass++) {
      int rc = mlgpu_nl_gsrb_pass(op, phi, rhs, pass, stream);
      if (rc) return rc;
    }
  return MLGPU_OK;
}

int mlgpu_nl_jacobi(const mlgpu_nlop *op, void *phi, const void *rhs, void *tmp,
                    void *stream) {
  if (!valid_nlop(op) || !phi || !rhs || !tmp || tmp == phi) return MLGPU_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  long long n = 2 * make_geom(op->grid).ncell;
  cudaError_t e;
  size_t bytes;
  if (op->dtype == MLGPU_F64) {
    e = launch_nl_op<double>(make_nl_args<double>(*op), NL_JACOBI, -1, (const double *)phi,
                             (const double *)rhs, (double *)tmp, nullptr, nullptr, nullptr, s);
    bytes = n * sizeof(double);
  } else {
    e = launch_nl_op<float>(make_nl_args<float>(*op), NL_JACOBI, -1, (const float *)phi,
                            (const float *)rhs, (float *)tmp, nullptr, nullptr, nullptr, s);
    bytes = n * sizeof(float);
  }
  if (e != cudaSuccess) return MLGPU_ERR_CUDA;
  return status_of(cudaMemcpyAsync(phi, tmp, bytes, cudaMemcpyDeviceToDevice, s));
}

int mlgpu_nl_lambda(const mlgpu_nlop *op, void *lam, void *stream) {
  if (!valid_nlop(op) || !lam) return MLGPU_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (op->dtype == MLGPU_F64)
    return status_of(launch_nl_lambda<double>(make_nl_args<double>(*op), (double *)lam, s));
  return status_of(launch_nl_lambda<float>(make_nl_args<float>(*op), (float *)lam, s));
}

int mlgpu_nl_restrict_residual(const mlgpu_nlop *op, void *res_c, const void *phi,
                               const void *rhs, void *stream) {
  if (!valid_nlop(op) || !res_c || !phi || !rhs || !coarsenable(op->grid)) return MLGPU_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  Geom C = coarsen_geom(make_geom(op->grid));
  if (op->dtype == MLGPU_F64)
    return status_of(launch_nl_restrict<double>(make_nl_args<double>(*op), C, (const double *)phi,
                                                (const double *)rhs, (double *)res_c, nullptr, s));
  return status_of(launch_nl_restrict<float>(make_nl_args<float>(*op), C, (const float *)phi,
                                             (const float *)rhs, (float *)res_c, nullptr, s));
}

int mlgpu_restrict_average(const mlgpu_grid *g, int ncomp, int dtype, void *coarse,
                           const void *fine, void *stream) {
  if (!valid_grid(g) || ncomp < 1 || !coarse || !fine || !coarsenable(*g)) return MLGPU_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  Geom F = make_geom(*g);
  if (dtype == MLGPU_F64)
    return status_of(launch_restrict_avg<double>(F, ncomp, (const double *)fine, (double *)coarse, s));
  if (dtype == MLGPU_F32)
    return status_of(launch_restrict_avg<float>(F, ncomp, (const float *)fine, (float *)coarse, s));
  return MLGPU_ERR_ARG;
}

int mlgpu_prolong_increment(const mlgpu_grid *g, const mlgpu_bc *bc, int ncomp, int dtype,
                            int kind, void *fine, const void *coarse, void *stream) {
  if (!valid_grid(g) || !bc || ncomp < 1 || ncomp > 2 || !fine || !coarse || !coarsenable(*g))
    return MLGPU_ERR_ARG;
  if (kind != MLGPU_PROLONG_CONSTANT && kind != MLGPU_PROLONG_LINEAR) return MLGPU_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  Geom F = make_geom(*g);
  BCD b = make_bcd(*bc);
  if (dtype == MLGPU_F64)
    return status_of(launch_prolong<double>(F, b, ncomp, kind, (double *)fine,
                                            (const double *)coarse, nullptr, s));
  if (dtype == MLGPU_F32)
    return status_of(launch_prolong<float>(F, b, ncomp, kind, (float *)fine, (const float *)coarse,
                                           nullptr, s));
  return MLGPU_ERR_ARG;
}

int mlgpu_coarsen_faces(const mlgpu_grid *g, int ncomp, int dtype, int dir, void *cf,
                        const void *ff, void *stream) {
  if (!valid_grid(g) || ncomp < 1 || dir < 0 || dir >= g->dim || !cf || !ff || !coarsenable(*g))
    return MLGPU_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  Geom F = make_geom(*g);
  if (dtype == MLGPU_F64)
    return status_of(launch_coarsen_faces<double>(F, ncomp, dir, (const double *)ff, (double *)cf, s));
  if (dtype == MLGPU_F32)
    return status_of(launch_coarsen_faces<float>(F, ncomp, dir, (const float *)ff, (float *)cf, s));
  return MLGPU_ERR_ARG;
}

int mlgpu_face_geomean(const mlgpu_grid *g, const double *cell, double *faces[3], void *stream) {
  if (!valid_grid(g) || !cell || !faces) return MLGPU_ERR_ARG;
  Geom G = make_geom(*g);
  for (int d = 0; d < g->dim; d++) {
    if (!faces[d]) return MLGPU_ERR_ARG;
    cudaError_t e = launch_face_geomean(G, d, cell, faces[d], (cudaStream_t)stream);
    if (e != cudaSuccess) return MLGPU_ERR_CUDA;
  }
  return MLGPU_OK;
}

int mlgpu_vc_residual(const mlgpu_vcop *op, void *res, const void *phi, const void *rhs,
                      int homogeneous, int norm_type, double *norm, void *ws, size_t ws_bytes,
                      void *stream) {
  if (!valid_vcop(op) || !res || !phi || !rhs) return MLGPU_ERR_ARG;
  if (norm_type > MLGPU_NORM_L2) return MLGPU_ERR_ARG;
  bool want = norm_type >= 0;
  if (want && (!norm || !ws)) return MLGPU_ERR_ARG;
  if (want && ws_bytes < mlgpu_norm_workspace_bytes()) return MLGPU_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  double *part = want ? (double *)ws : nullptr;
  int nt = want ? norm_type : -1, nparts = 0;
  cudaError_t e;
  if (op->dtype == MLGPU_F64)
    e = launch_vc_op<double>(make_vc_args<double>(*op), VC_RESIDUAL, nt, (const double *)phi,
                             (const double *)rhs, (double *)res, homogeneous, part, &nparts, s);
  else
    e = launch_vc_op<float>(make_vc_args<float>(*op), VC_RESIDUAL, nt, (const float *)phi,
                            (const float *)rhs, (float *)res, homogeneous, part, &nparts, s);
  if (e != cudaSuccess) return MLGPU_ERR_CUDA;
  if (!want) return MLGPU_OK;
  return finish_norm(norm_type, part, nparts, norm, s);
}

int mlgpu_vc_apply(const mlgpu_vcop *op, void *lhs, const void *phi, int homogeneous,
                   void *stream) {
  if (!valid_vcop(op) || !lhs || !phi) return MLGPU_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (op->dtype == MLGPU_F64)
    return status_of(launch_vc_op<double>(make_vc_args<double>(*op), VC_APPLY, -1,
                                          (const double *)phi, nullptr, (double *)lhs,
                                          homogeneous, nullptr, nullptr, s));
  return status_of(launch_vc_op<float>(make_vc_args<float>(*op), VC_APPLY, -1, (const float *)phi,
                                       nullptr, (float *)lhs, homogeneous, nullptr, nullptr, s));
}

int mlgpu_vc_gsrb_pass(const mlgpu_vcop *op, void *phi, const void *rhs, int pass,
                       void *stream) {
  if (!valid_vcop(op) || !phi || !rhs || (pass != 0 && pass != 1)) return MLGPU_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (op->dtype == MLGPU_F64)
    return status_of(launch_vc_gsrb<double>(make_vc_args<double>(*op), (double *)phi,
                                            (const double *)rhs, pass, s));
  return status_of(
      launch_vc_gsrb<float>(make_vc_args<float>(*op), (float *)phi, (const float *)rhs, pass, s));
}

int mlgpu_vc_relax(const mlgpu_vcop *op, void *phi, const void *rhs, int n, void *stream) {
  if (n < 0) return MLGPU_ERR_ARG;
  for (int i = 0; i < n; i++)
    for (int pass = 0; pass < 2; pass++) {
      int rc = mlgpu_vc_gsrb_pass(op, phi, rhs, pass, stream);
      if (rc) return rc;
    }
  return MLGPU_OK;
}

int mlgpu_vc_jacobi(const mlgpu_vcop *op, void *phi, const void *rhs, void *tmp, void *stream) {
  if (!valid_vcop(op) || !phi || !rhs || !tmp || tmp == phi) return MLGPU_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  long long n = make_geom(op->grid).ncell;
  cudaError_t e;
  size_t bytes;
  if (op->dtype == MLGPU_F64) {
    e = launch_vc_op<double>(make_vc_args<double>(*op), VC_JACOBI, -1, (const double *)phi,
                             (const double *)rhs, (double *)tmp, 1, nullptr, nullptr, s);
    bytes = n * sizeof(double);
  } else {
    e = launch_vc_op<float>(make_vc_args<float>(*op), VC_JACOBI, -1, (const float *)phi,
                            (const float *)rhs, (float *)tmp, 1, nullptr, nullptr, s);
    bytes = n * sizeof(float);
  }
  if (e != cudaSuccess) return MLGPU_ERR_CUDA;
  return status_of(cudaMemcpyAsync(phi, tmp, bytes, cudaMemcpyDeviceToDevice, s));
}

int mlgpu_vc_lambda(const mlgpu_vcop *op, void *lam, void *stream) {
  if (!valid_vcop(op) || !lam) return MLGPU_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (op->dtype == MLGPU_F64)
    return status_of(launch_vc_lambda<double>(make_vc_args<double>(*op), (double *)lam, s));
  return status_of(launch_vc_lambda<float>(make_vc_args<float>(*op), (float *)lam, s));
}

int mlgpu_vc_restrict_residual(const mlgpu_vcop *op, void *res_c, const void *phi,
                               const void *rhs, void *stream) {
  if (!valid_vcop(op) || !res_c || !phi || !rhs || !coarsenable(op->grid)) return MLGPU_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  Geom C = coarsen_geom(make_geom(op->grid));
  if (op->dtype == MLGPU_F64)
    return status_of(launch_vc_restrict<double>(make_vc_args<double>(*op), C, (const double *)phi,
                                                (const double *)rhs, (double *)res_c, nullptr, s));
  return status_of(launch_vc_restrict<float>(make_vc_args<float>(*op), C, (const float *)phi,
                                             (const float *)rhs, (float *)res_c, nullptr, s));
}

int mlgpu_mac_divergence(const mlgpu_grid *g, double *div, const double *u[3], void *stream) {
  if (!valid_grid(g) || !div || !u) return MLGPU_ERR_ARG;
  for (int d = 0; d < g->dim; d++)
    if (!u[d]) return MLGPU_ERR_ARG;
  return status_of(launch_mac_div(make_geom(*g), u[0], u[1], g->dim == 3 ? u[2] : nullptr, div,
                                  (cudaStream_t)stream));
}

int mlgpu_mac_correct(const mlgpu_grid *g, const mlgpu_bc *bc, const double *phi,
                      const double *scale[3], double *u[3], void *stream) {
  if (!valid_grid(g) || !bc || !phi || !u) return MLGPU_ERR_ARG;
  Geom G = make_geom(*g);
  BCD b = make_bcd(*bc);
  for (int d = 0; d < g->dim; d++) {
    if (!u[d]) return MLGPU_ERR_ARG;
    cudaError_t e = launch_mac_correct(G, b, d, phi, scale ? scale[d] : nullptr, u[d],
                                       (cudaStream_t)stream);
    if (e != cudaSuccess) return MLGPU_ERR_CUDA;
  }
  return MLGPU_OK;
}

int mlgpu_axpby(size_t n, int dtype, double a, const void *x, double b, void *y, void *stream) {
  if (!x || !y) return MLGPU_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == MLGPU_F64)
    return status_of(launch_axpby<double>((long long)n, a, (const double *)x, b, (double *)y, s));
  if (dtype == MLGPU_F32)
    return status_of(
        launch_axpby<float>((long long)n, (float)a, (const float *)x, (float)b, (float *)y, s));
  return MLGPU_ERR_ARG;
}

int mlgpu_norm(size_t n, int dtype, const void *x, int norm_type, double *out, void *ws,
               size_t ws_bytes, void *stream) {
  if (!x || !out || !ws || norm_type < 0 || norm_type > MLGPU_NORM_L2) return MLGPU_ERR_ARG;
  if (ws_bytes < mlgpu_norm_workspace_bytes()) return MLGPU_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  double *part = (double *)ws;
  int nparts = 0;
  cudaError_t e;
  if (dtype == MLGPU_F64)
    e = launch_norm_partial<double>((long long)n, (const double *)x, norm_type, part, &nparts, s);
  else if (dtype == MLGPU_F32)
    e = launch_norm_partial<float>((long long)n, (const float *)x, norm_type, part, &nparts, s);
  else
    return MLGPU_ERR_ARG;
  if (e != cudaSuccess) return MLGPU_ERR_CUDA;
  return finish_norm(norm_type, part, nparts, out, s);
}

int mlgpu_convert(size_t n, int dd, void *dst, int ds, const void *src, void *stream) {
  if (!dst || !src) return MLGPU_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  long long m = (long long)n;
  if (dd == MLGPU_F64 && ds == MLGPU_F32)
    return status_of(launch_convert<double, float>(m, (double *)dst, (const float *)src, s));
  if (dd == MLGPU_F32 && ds == MLGPU_F64)
    return status_of(launch_convert<float, double>(m, (float *)dst, (const double *)src, s));
  if (dd == MLGPU_F64 && ds == MLGPU_F64)
    return status_of(launch_convert<double, double>(m, (double *)dst, (const double *)src, s));
  if (dd == MLGPU_F32 && ds == MLGPU_F32)
    return status_of(launch_convert<float, float>(m, (float *)dst, (const float *)src, s));
  return MLGPU_ERR_ARG;
}

}  // extern "C"
