/*
 * mlgpu.hpp -- C++ host classes over the C ABI of mlgpu.h, mirroring the
 * reference's level-operator interface for this path:
 *
 *   NLMultiCompOp    AMRNonLinearMultiCompOp (src/AMRNonLinearMultiCompOp.H)
 *   ProjectionOp     AMRProjectionOp         (src/AMRProjectionOp.h)
 *   DarcyBrinkmanOp  DarcyBrinkmanOp         (src/DarcyBrinkmanOp.H)
 *   AMRFASMultiGrid  / AMRMultiGrid          the drivers' role (Chombo)
 *   AdjointMultiGrid the transposed-Jacobian solver (no reference counterpart)
 *
 * Method names and argument meaning follow the reference (residual, applyOp,
 * relax, levelGSRB, levelJacobi, restrictResidual, restrictR,
 * prolongIncrement, createCoarser, setAlphaAndBeta, MGnewOp).  Fields are
 * DeviceField: one box in device memory, [comp][k][j][i], no ghost cells
 * (ghost values are produced in registers from the boundary descriptors).
 * Errors that the reference handles with MayDay::Error / Abort throw
 * mlgpu::Error; a solve that stops above its tolerance is not an error and
 * reports through its mlgpu_solve_stats, as the reference's exit status.
 *
 * Header-only; links against libmlgpu.so alone (device memory through the
 * library's helpers, no CUDA runtime of the caller's own).  Streams are
 * passed as void* (cudaStream_t); nullptr is the legacy default stream.
 */
#ifndef MLGPU_HPP_
#define MLGPU_HPP_

#include <cstddef>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>

#include "mlgpu.h"

namespace mlgpu {

class Error : public std::runtime_error {
 public:
  Error(int status, const std::string &what)
      : std::runtime_error(what + ": " + mlgpu_status_string(status)), status_(status) {}
  int status() const { return status_; }

 private:
  int status_;
};

inline void check(int rc, const char *what) {
  if (rc != MLGPU_OK) throw Error(rc, what);
}

inline size_t cells(const mlgpu_grid &g) { return (size_t)g.n[0] * g.n[1] * g.n[2]; }
inline size_t faces(const mlgpu_grid &g, int d) {
  size_t m = 1;
  for (int e = 0; e < 3; e++) m *= (size_t)(g.n[e] + (e == d ? 1 : 0));
  return m;
}
// createCoarser's test: every extent even (coarsen by 2)
inline bool coarsenable(const mlgpu_grid &g) {
  for (int d = 0; d < g.dim; d++)
    if (g.n[d] < 2 || g.n[d] % 2) return false;
  return true;
}
inline mlgpu_grid coarsened(const mlgpu_grid &g) {
  mlgpu_grid c = g;
  for (int d = 0; d < g.dim; d++) c.n[d] = g.n[d] / 2;
  c.dx = g.dx * 2;
  return c;
}
inline size_t elem_size(int dtype) { return dtype == MLGPU_F32 ? 4 : 8; }

// One box of device data owned by the object: `ncomp` components of
// `count_per_comp` values each (cells by default, faces for coefficients).
class DeviceField {
 public:
  DeviceField(const mlgpu_grid &g, int ncomp, int dtype = MLGPU_F64, size_t count_per_comp = 0)
      : grid_(g), ncomp_(ncomp), dtype_(dtype),
        count_(count_per_comp ? count_per_comp : cells(g)) {
    check(mlgpu_device_alloc(bytes(), &ptr_), "DeviceField");
  }
  ~DeviceField() {
    if (ptr_) mlgpu_device_free(ptr_);
  }
  DeviceField(const DeviceField &) = delete;
  DeviceField &operator=(const DeviceField &) = delete;
  DeviceField(DeviceField &&o) noexcept
      : grid_(o.grid_), ncomp_(o.ncomp_), dtype_(o.dtype_), count_(o.count_), ptr_(o.ptr_) {
    o.ptr_ = nullptr;
  }

  void *data() { return ptr_; }
  const void *data() const { return ptr_; }
  const mlgpu_grid &grid() const { return grid_; }
  int ncomp() const { return ncomp_; }
  int dtype() const { return dtype_; }
  size_t size() const { return count_ * (size_t)ncomp_; }
  size_t bytes() const { return size() * elem_size(dtype_); }

  void upload(const void *host, void *stream = nullptr) {
    check(mlgpu_memcpy(ptr_, host, bytes(), 0, stream), "DeviceField::upload");
  }
  void download(void *host, void *stream = nullptr) const {
    check(mlgpu_memcpy(host, ptr_, bytes(), 1, stream), "DeviceField::download");
    check(mlgpu_stream_synchronize(stream), "DeviceField::download");
  }
  void copyFrom(const DeviceField &o, void *stream = nullptr) {
    if (o.bytes() != bytes()) throw Error(MLGPU_ERR_ARG, "DeviceField::copyFrom");
    check(mlgpu_memcpy(ptr_, o.ptr_, bytes(), 2, stream), "DeviceField::copyFrom");
  }
  void setToZero(void *stream = nullptr) {
    check(mlgpu_memset_zero(ptr_, bytes(), stream), "DeviceField::setToZero");
  }

 private:
  mlgpu_grid grid_;
  int ncomp_, dtype_;
  size_t count_;
  void *ptr_ = nullptr;
};

// Scratch for fused norms, allocated on first use (an operator that never
// asks for a norm holds no device memory of its own).
class NormScratch {
 public:
  void *data() { return get().data(); }
  size_t bytes() { return get().bytes(); }

 private:
  DeviceField &get() {
    if (!f_) {
      mlgpu_grid g = {2, {1, 1, 1}, 1.0, {0, 0, 0}};
      f_.reset(new DeviceField(g, 1, MLGPU_F64, mlgpu_norm_workspace_bytes() / 8 + 1));
    }
    return *f_;
  }
  std::unique_ptr<DeviceField> f_;
};

// ------------------------------------------------- AMRNonLinearMultiCompOp
class NLMultiCompOp {
 public:
  // `desc` holds device pointers to the coefficients (owned by the caller)
  explicit NLMultiCompOp(const mlgpu_nlop &desc, void *stream = nullptr) : d_(desc), s_(stream) {}

  const mlgpu_nlop &desc() const { return d_; }
  void *stream() const { return s_; }

  // residualI: lhs = rhs - L(phi); returns the norm when norm_type >= 0
  double residual(DeviceField &lhs, const DeviceField &phi, const DeviceField &rhs,
                  int norm_type = -1) {
    double nrm = 0;
    check(mlgpu_nl_residual(&d_, lhs.data(), phi.data(), rhs.data(), norm_type,
                            norm_type >= 0 ? &nrm : nullptr, norm_type >= 0 ? ws_.data() : nullptr,
                            norm_type >= 0 ? ws_.bytes() : 0, s_),
          "NLMultiCompOp::residual");
    return nrm;
  }
  void applyOp(DeviceField &lhs, const DeviceField &phi) {
    check(mlgpu_nl_apply(&d_, lhs.data(), phi.data(), s_), "NLMultiCompOp::applyOp");
  }
  void relax(DeviceField &phi, const DeviceField &rhs, int iterations) {
    check(mlgpu_nl_relax(&d_, phi.data(), rhs.data(), iterations, s_), "NLMultiCompOp::relax");
  }
  void levelGSRB(DeviceField &phi, const DeviceField &rhs) {
    for (int pass = 0; pass < 2; pass++)
      check(mlgpu_nl_gsrb_pass(&d_, phi.data(), rhs.data(), pass, s_), "NLMultiCompOp::levelGSRB");
  }
  void levelJacobi(DeviceField &phi, const DeviceField &rhs) {
    DeviceField tmp(phi.grid(), phi.ncomp(), phi.dtype());
    check(mlgpu_nl_jacobi(&d_, phi.data(), rhs.data(), tmp.data(), s_),
          "NLMultiCompOp::levelJacobi");
    check(mlgpu_stream_synchronize(s_), "NLMultiCompOp::levelJacobi");
  }
  // resetLambda as an explicit field
  void computeLambda(DeviceField &lambda) {
    check(mlgpu_nl_lambda(&d_, lambda.data(), s_), "NLMultiCompOp::computeLambda");
  }
  // FAS restrictResidual: resC = average of (rhs - L(phi)) on the coarse box
  void restrictResidual(DeviceField &resC, const DeviceField &phi, const DeviceField &rhs) {
    check(mlgpu_nl_restrict_residual(&d_, resC.data(), phi.data(), rhs.data(), s_),
          "NLMultiCompOp::restrictResidual");
  }
  void restrictR(DeviceField &phiC, const DeviceField &phiF) {
    check(mlgpu_restrict_average(&d_.grid, 2, d_.dtype, phiC.data(), phiF.data(), s_),
          "NLMultiCompOp::restrictR");
  }
  void prolongIncrement(DeviceField &phi, const DeviceField &corrC,
                        int kind = MLGPU_PROLONG_LINEAR) {
    check(mlgpu_prolong_increment(&d_.grid, &d_.phi_bc, 2, d_.dtype, kind, phi.data(),
                                  corrC.data(), s_),
          "NLMultiCompOp::prolongIncrement");
  }
  void setAlphaAndBeta(double alpha, double beta) {
    d_.alpha = alpha;
    d_.beta = beta;
  }
  // a field on the box coarsened by 2, or nullptr when it cannot be coarsened
  std::unique_ptr<DeviceField> createCoarser(const DeviceField &fine) const {
    if (!coarsenable(fine.grid())) return nullptr;
    return std::unique_ptr<DeviceField>(
        new DeviceField(coarsened(fine.grid()), fine.ncomp(), fine.dtype()));
  }
  // MGnewOp: the operator one level coarser with its coefficients averaged
  // (cells over 2^D, faces over 2^(D-1)); nullptr at the coarsening limit
  std::unique_ptr<NLMultiCompOp> MGnewOp() const {
    if (!coarsenable(d_.grid)) return nullptr;
    std::unique_ptr<NLMultiCompOp> c(new NLMultiCompOp(d_, s_));
    const mlgpu_grid cg = coarsened(d_.grid);
    c->d_.grid = cg;
    if (d_.aCoef) {
      c->own_a_.reset(new DeviceField(cg, 2, d_.dtype));
      check(mlgpu_restrict_average(&d_.grid, 2, d_.dtype, c->own_a_->data(), d_.aCoef, s_),
            "NLMultiCompOp::MGnewOp");
      c->d_.aCoef = c->own_a_->data();
    }
    for (int d = 0; d < 3; d++) {
      c->d_.bCoef[d] = nullptr;
      if (d >= d_.grid.dim) continue;
      c->own_b_[d].reset(new DeviceField(cg, 2, d_.dtype, faces(cg, d)));
      check(mlgpu_coarsen_faces(&d_.grid, 2, d_.dtype, d, c->own_b_[d]->data(), d_.bCoef[d], s_),
            "NLMultiCompOp::MGnewOp");
      c->d_.bCoef[d] = c->own_b_[d]->data();
    }
    return c;
  }

 private:
  mlgpu_nlop d_;
  void *s_;
  NormScratch ws_;
  std::unique_ptr<DeviceField> own_a_, own_b_[3];  // coefficients of an MGnewOp level
};

// ----------------------------------- AMRProjectionOp / DarcyBrinkmanOp
class VCOp {
 public:
  explicit VCOp(const mlgpu_vcop &desc, void *stream = nullptr) : d_(desc), s_(stream) {}
  virtual ~VCOp() = default;

  const mlgpu_vcop &desc() const { return d_; }
  void *stream() const { return s_; }

  double residual(DeviceField &lhs, const DeviceField &phi, const DeviceField &rhs,
                  bool homogeneous = false, int norm_type = -1) {
    double nrm = 0;
    check(mlgpu_vc_residual(&d_, lhs.data(), phi.data(), rhs.data(), homogeneous ? 1 : 0,
                            norm_type, norm_type >= 0 ? &nrm : nullptr,
                            norm_type >= 0 ? ws_.data() : nullptr,
                            norm_type >= 0 ? ws_.bytes() : 0, s_),
          "VCOp::residual");
    return nrm;
  }
  void applyOp(DeviceField &lhs, const DeviceField &phi, bool homogeneous = false) {
    check(mlgpu_vc_apply(&d_, lhs.data(), phi.data(), homogeneous ? 1 : 0, s_), "VCOp::applyOp");
  }
  void relax(DeviceField &phi, const DeviceField &rhs, int iterations) {
    check(mlgpu_vc_relax(&d_, phi.data(), rhs.data(), iterations, s_), "VCOp::relax");
  }
  void levelGSRB(DeviceField &phi, const DeviceField &rhs) {
    for (int pass = 0; pass < 2; pass++)
      check(mlgpu_vc_gsrb_pass(&d_, phi.data(), rhs.data(), pass, s_), "VCOp::levelGSRB");
  }
  void levelJacobi(DeviceField &phi, const DeviceField &rhs) {
    DeviceField tmp(phi.grid(), phi.ncomp(), phi.dtype());
    check(mlgpu_vc_jacobi(&d_, phi.data(), rhs.data(), tmp.data(), s_), "VCOp::levelJacobi");
    check(mlgpu_stream_synchronize(s_), "VCOp::levelJacobi");
  }
  void computeLambda(DeviceField &lambda) {
    check(mlgpu_vc_lambda(&d_, lambda.data(), s_), "VCOp::computeLambda");
  }
  void restrictResidual(DeviceField &resC, const DeviceField &phi, const DeviceField &rhs) {
    check(mlgpu_vc_restrict_residual(&d_, resC.data(), phi.data(), rhs.data(), s_),
          "VCOp::restrictResidual");
  }
  void restrictR(DeviceField &phiC, const DeviceField &phiF) {
    check(mlgpu_restrict_average(&d_.grid, 1, d_.dtype, phiC.data(), phiF.data(), s_),
          "VCOp::restrictR");
  }
  // AMRProjectionOp::prolongIncrement is piecewise constant (src/AMRProjectionOp.cpp:67-98)
  void prolongIncrement(DeviceField &phi, const DeviceField &corrC,
                        int kind = MLGPU_PROLONG_CONSTANT) {
    check(mlgpu_prolong_increment(&d_.grid, &d_.bc, 1, d_.dtype, kind, phi.data(), corrC.data(),
                                  s_),
          "VCOp::prolongIncrement");
  }
  void setAlphaAndBeta(double alpha, double beta) {
    d_.alpha = alpha;
    d_.beta = beta;
  }
  std::unique_ptr<DeviceField> createCoarser(const DeviceField &fine) const {
    if (!coarsenable(fine.grid())) return nullptr;
    return std::unique_ptr<DeviceField>(
        new DeviceField(coarsened(fine.grid()), fine.ncomp(), fine.dtype()));
  }
  // MGnewOp (AMRProjectionOpFactory / DarcyBrinkmanOpFactory): the operator
  // one level coarser, a and c averaged over 2^D cells, the faces over
  // 2^(D-1); nullptr at the coarsening limit
  std::unique_ptr<VCOp> MGnewOp() const {
    if (!coarsenable(d_.grid)) return nullptr;
    std::unique_ptr<VCOp> c(new VCOp(d_, s_));
    const mlgpu_grid cg = coarsened(d_.grid);
    c->d_.grid = cg;
    const void *cell[2] = {d_.aCoef, d_.cCoef};
    const void **dst[2] = {&c->d_.aCoef, &c->d_.cCoef};
    for (int m = 0; m < 2; m++) {
      if (!cell[m]) continue;
      c->own_cell_[m].reset(new DeviceField(cg, 1, d_.dtype));
      check(mlgpu_restrict_average(&d_.grid, 1, d_.dtype, c->own_cell_[m]->data(), cell[m], s_),
            "VCOp::MGnewOp");
      *dst[m] = c->own_cell_[m]->data();
    }
    for (int d = 0; d < 3; d++) {
      c->d_.bCoef[d] = nullptr;
      if (d >= d_.grid.dim) continue;
      c->own_b_[d].reset(new DeviceField(cg, 1, d_.dtype, faces(cg, d)));
      check(mlgpu_coarsen_faces(&d_.grid, 1, d_.dtype, d, c->own_b_[d]->data(), d_.bCoef[d], s_),
            "VCOp::MGnewOp");
      c->d_.bCoef[d] = c->own_b_[d]->data();
    }
    return c;
  }

 protected:
  mlgpu_vcop d_;
  void *s_;
  NormScratch ws_;
  std::unique_ptr<DeviceField> own_cell_[2], own_b_[3];  // coefficients of an MGnewOp level
};

// alpha = 0, bCoef = -Pi_face, beta = 1, cCoef = NULL (srcSubcycle/Projector.cpp:2942-2973)
class ProjectionOp : public VCOp {
 public:
  using VCOp::VCOp;
};

// (alpha a - beta c - beta div b grad) u = rho per velocity component
class DarcyBrinkmanOp : public VCOp {
 public:
  using VCOp::VCOp;
};

// ------------------------------------------------------------- drivers
class Solver {
 public:
  Solver(const Solver &) = delete;
  Solver &operator=(const Solver &) = delete;
  virtual ~Solver() {
    if (h_) mlgpu_solver_destroy(h_);
  }
  mlgpu_solver *handle() { return h_; }
  // solve in place: phi holds the initial guess
  mlgpu_solve_stats solve(DeviceField &phi, const DeviceField &rhs) {
    mlgpu_solve_stats st;
    int rc = mlgpu_solver_solve(h_, (double *)phi.data(), (const double *)rhs.data(), &st);
    tolerate(rc, "Solver::solve");
    return st;
  }
  void setAlphaAndBeta(double alpha, double beta) {
    check(mlgpu_solver_set_alpha_beta(h_, alpha, beta), "Solver::setAlphaAndBeta");
  }

 protected:
  Solver() = default;
  // non-convergence and stagnation are reported by the stats, not thrown
  static void tolerate(int rc, const char *what) {
    if (rc != MLGPU_OK && rc != MLGPU_ERR_NOT_CONVERGED && rc != MLGPU_ERR_HANG) check(rc, what);
  }
  void make_workspace(size_t bytes) {
    mlgpu_grid g = {2, {1, 1, 1}, 1.0, {0, 0, 0}};
    ws_.reset(new DeviceField(g, 1, MLGPU_F64, bytes / 8 + 64));
  }
  // mlgpu_hc_tga_step on solver h with its two-field scratch
  static mlgpu_solve_stats tga_step(mlgpu_solver *h, DeviceField &phi_new,
                                    const DeviceField &phi_old, double dt, const DeviceField *src,
                                    const DeviceField *aCoef, const char *what) {
    DeviceField scratch(phi_old.grid(), 2 * phi_old.ncomp(), phi_old.dtype());
    mlgpu_solve_stats st;
    int rc = mlgpu_hc_tga_step(h, (double *)phi_new.data(), (const double *)phi_old.data(),
                               src ? (const double *)src->data() : nullptr,
                               aCoef ? (const double *)aCoef->data() : nullptr, dt,
                               (double *)scratch.data(), &st);
    tolerate(rc, what);
    return st;
  }
  // the workspace must be 256-byte aligned, which every device allocation
  // made through the library (cudaMalloc) is
  void *ws() { return ws_->data(); }
  size_t ws_bytes() const { return ws_->bytes(); }

  mlgpu_solver *h_ = nullptr;
  std::unique_ptr<DeviceField> ws_;
};

inline mlgpu_mg_options default_options(bool hc) {
  mlgpu_mg_options o;
  mlgpu_mg_default_options(&o, hc ? 1 : 0);
  return o;
}

// FAS multigrid for NLMultiCompOp (AMRFASMultiGrid's role)
class AMRFASMultiGrid : public Solver {
 public:
  explicit AMRFASMultiGrid(const NLMultiCompOp &op, const mlgpu_mg_options &o = default_options(true)) {
    size_t bytes = 0;
    check(mlgpu_hc_solver_workspace(&op.desc(), &o, &bytes), "AMRFASMultiGrid");
    make_workspace(bytes);
    check(mlgpu_hc_solver_create(&op.desc(), &o, ws(), ws_bytes(), op.stream(), &h_),
          "AMRFASMultiGrid");
  }
  // LevelBackwardEuler::updateSoln: (a - dt L) phi_new = a phi_old + dt src
  mlgpu_solve_stats backwardEuler(DeviceField &phi_new, const DeviceField &phi_old, double dt,
                                  const DeviceField *src = nullptr,
                                  const DeviceField *aCoef = nullptr) {
    DeviceField scratch(phi_old.grid(), phi_old.ncomp(), phi_old.dtype());
    mlgpu_solve_stats st;
    int rc = mlgpu_hc_backward_euler(h_, (double *)phi_new.data(), (const double *)phi_old.data(),
                                     src ? (const double *)src->data() : nullptr,
                                     aCoef ? (const double *)aCoef->data() : nullptr, dt,
                                     (double *)scratch.data(), &st);
    tolerate(rc, "AMRFASMultiGrid::backwardEuler");
    return st;
  }
  // LevelTGA::updateSoln: (a - mu1 dt L) psi = (a + mu3 dt L) phi_old + dt src,
  // (a - mu2 dt L) phi_new = a psi (mlgpu_hc_tga_step, FAS solves)
  mlgpu_solve_stats tgaStep(DeviceField &phi_new, const DeviceField &phi_old, double dt,
                            const DeviceField *src = nullptr, const DeviceField *aCoef = nullptr) {
    return tga_step(h_, phi_new, phi_old, dt, src, aCoef, "AMRFASMultiGrid::tgaStep");
  }
};

// linear multigrid for ProjectionOp / DarcyBrinkmanOp (AMRMultiGrid's role)
class AMRMultiGrid : public Solver {
 public:
  explicit AMRMultiGrid(const VCOp &op, const mlgpu_mg_options &o = default_options(false))
      : grid_(op.desc().grid), bc_(op.desc().bc) {
    size_t bytes = 0;
    check(mlgpu_vc_solver_workspace(&op.desc(), &o, &bytes), "AMRMultiGrid");
    make_workspace(bytes);
    check(mlgpu_vc_solver_create(&op.desc(), &o, ws(), ws_bytes(), op.stream(), &h_),
          "AMRMultiGrid");
  }
  // Projector::levelMacProject: u -= Pi grad phi with div(Pi grad phi) = div u
  mlgpu_solve_stats levelMacProject(DeviceField *u[3], const DeviceField *pi_face[3],
                                    DeviceField &phi) {
    DeviceField scratch(grid_, 1);
    double *uu[3] = {nullptr, nullptr, nullptr};
    const double *pp[3] = {nullptr, nullptr, nullptr};
    for (int d = 0; d < grid_.dim; d++) {
      uu[d] = (double *)u[d]->data();
      if (pi_face) pp[d] = (const double *)pi_face[d]->data();
    }
    mlgpu_solve_stats st;
    int rc = mlgpu_mac_project(h_, &grid_, &bc_, uu, pi_face ? pp : nullptr,
                               (double *)phi.data(), (double *)scratch.data(), &st);
    tolerate(rc, "AMRMultiGrid::levelMacProject");
    return st;
  }

 private:
  mlgpu_grid grid_;
  mlgpu_bc bc_;
};

// transposed-Jacobian multigrid (adjoint solves) and Newton steps
class AdjointMultiGrid : public Solver {
 public:
  explicit AdjointMultiGrid(const NLMultiCompOp &op, const mlgpu_mg_options &o = default_options(true)) {
    size_t bytes = 0;
    check(mlgpu_hc_adjoint_workspace(&op.desc(), &o, &bytes), "AdjointMultiGrid");
    make_workspace(bytes);
    check(mlgpu_hc_adjoint_create(&op.desc(), &o, ws(), ws_bytes(), op.stream(), &h_),
          "AdjointMultiGrid");
  }
  // A^T y = g with A = dN/dphi at phi (y: initial guess in, solution out)
  mlgpu_solve_stats adjointSolve(const DeviceField &phi, const DeviceField &g, DeviceField &y) {
    mlgpu_solve_stats st;
    int rc = mlgpu_hc_adjoint_solve(h_, (const double *)phi.data(), (const double *)g.data(),
                                    (double *)y.data(), &st);
    tolerate(rc, "AdjointMultiGrid::adjointSolve");
    return st;
  }
  // N(phi) = rhs by Newton steps on the Jacobian hierarchy
  mlgpu_solve_stats newtonSolve(DeviceField &phi, const DeviceField &rhs) {
    mlgpu_solve_stats st;
    int rc = mlgpu_hc_newton_solve(h_, (double *)phi.data(), (const double *)rhs.data(), &st);
    tolerate(rc, "AdjointMultiGrid::newtonSolve");
    return st;
  }
  // the TGA step with Newton's solves (mlgpu_hc_tga_step on this solver)
  mlgpu_solve_stats tgaStep(DeviceField &phi_new, const DeviceField &phi_old, double dt,
                            const DeviceField *src = nullptr, const DeviceField *aCoef = nullptr) {
    return tga_step(h_, phi_new, phi_old, dt, src, aCoef, "AdjointMultiGrid::tgaStep");
  }
  // adjoint of AMRFASMultiGrid::backwardEuler: A^T mu = phi_new_bar, then
  // phi_old_bar = a mu, src_bar = dt mu and the wall-value gradient
  // (bc_grad[(dir * 2 + side) * 2 + comp]); outputs may be null
  mlgpu_solve_stats backwardEulerAdjoint(const DeviceField &phi_new,
                                         const DeviceField &phi_new_bar, double dt,
                                         DeviceField &mu, DeviceField *phi_old_bar,
                                         DeviceField *src_bar, double bc_grad[12] = nullptr,
                                         const DeviceField *aCoef = nullptr) {
    mlgpu_solve_stats st;
    int rc = mlgpu_hc_backward_euler_adjoint(
        h_, (const double *)phi_new.data(), (const double *)phi_new_bar.data(),
        aCoef ? (const double *)aCoef->data() : nullptr, dt, (double *)mu.data(),
        phi_old_bar ? (double *)phi_old_bar->data() : nullptr,
        src_bar ? (double *)src_bar->data() : nullptr, bc_grad, &st);
    tolerate(rc, "AdjointMultiGrid::backwardEulerAdjoint");
    return st;
  }
};

// adjoint of AMRMultiGrid::levelMacProject on the solver `mg` that ran the
// forward: ustar_bar = ubar - D^T q with D Pi G q = G^T (Pi ubar), and
// pi_bar = -ustar_bar (G p) when pi_bar is given (p: the forward pressure)
inline mlgpu_solve_stats macProjectAdjoint(AMRMultiGrid &mg, const mlgpu_grid &grid,
                                           const mlgpu_bc &bc, const DeviceField *ubar[3],
                                           const DeviceField *pi_face[3], const DeviceField &p,
                                           DeviceField *ustar_bar[3], DeviceField *pi_bar[3],
                                           DeviceField &q) {
  DeviceField scratch(grid, 1);
  const double *ub[3] = {nullptr, nullptr, nullptr}, *pf[3] = {nullptr, nullptr, nullptr};
  double *us[3] = {nullptr, nullptr, nullptr}, *pb[3] = {nullptr, nullptr, nullptr};
  for (int d = 0; d < grid.dim; d++) {
    ub[d] = (const double *)ubar[d]->data();
    us[d] = (double *)ustar_bar[d]->data();
    if (pi_face) pf[d] = (const double *)pi_face[d]->data();
    if (pi_bar) pb[d] = (double *)pi_bar[d]->data();
  }
  mlgpu_solve_stats st;
  int rc = mlgpu_mac_project_adjoint(mg.handle(), &grid, &bc, ub, pi_face ? pf : nullptr,
                                     (const double *)p.data(), us, pi_bar ? pb : nullptr,
                                     (double *)q.data(), (double *)scratch.data(), &st);
  if (rc != MLGPU_OK && rc != MLGPU_ERR_NOT_CONVERGED && rc != MLGPU_ERR_HANG)
    check(rc, "macProjectAdjoint");
  return st;
}

}  // namespace mlgpu

#endif /* MLGPU_HPP_ */
