// oracle.cpp -- CPU FP64 restatement of mushy-layer's elliptic/closure hot
// path.  TEST INFRASTRUCTURE ONLY: the CUDA product never links, loads or
// calls this file; tests and the CPU-baseline leg of the benchmark use it as
// the checker.
//
// It follows the reference's data model literally: every field is a FAB with
// one ghost layer; operators fill ghosts (periodic exchange, then physical BC
// functions), compute the closure over the ghosted box, apply the derived
// variable BC and then run the Fortran loop nests.  Expressions keep the
// Fortran evaluation order (left to right, no contraction; build with
// -ffp-contract=off) so that FP64 results can be compared bit for bit.
//
// Reference files restated (paths inside the mushy-layer project):
//   src/EnthalpyVariablesF.ChF        closure kernels
//   src/phaseDiagram.cpp              closure driver
//   src/AMRNonLinearMultiCompOpF.ChF  nonlinear op kernels
//   src/AMRNonLinearMultiCompOp.cpp   op call sequence, lambda, MGnewOp
//   src/DarcyBrinkmanOpF.ChF / .cpp   linear op with c term
//   src/AMRProjectionOp.cpp, AMRProjectionOpF.ChF   projection op, prolong
//   src/CellToEdge2F.ChF, util/DivergenceF.ChF, util/Gradient.cpp
//   BCutil/BCFuncF.ChF, BCutil/BCFunctions.cpp, BCutil/PhysBCUtil.cpp
// The multigrid drivers restate Chombo's AMRMultiGrid / AMRFASMultiGrid /
// RelaxSolver (Chombo fork c00e7b62, not in the reference tree); parity at
// the driver level is unpinned.
//
// Pins: the closure reproduces the reference's own plotfile output bit for
// bit (tests/test_golden.py); the operators, wall conditions and solvers
// reproduce the analytic answers of the reference's physics tests: steady
// Robin conduction (test/diffusiveGrowth), Poiseuille-Brinkman flow
// (test/poiseuilleFlow) and the directional-solidification mushy layer of
// test/testDiffusiveSolidification.py (second-order convergence).

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/mlgpu.h"

namespace {

// ------------------------------------------------------------------ FAB
struct Fab {
  int nc = 0;
  int n[3] = {1, 1, 1};
  int g[3] = {0, 0, 0};
  int s[3] = {0, 0, 0};  // strides of the ghosted box
  std::vector<double> v;
  Fab() {}
  Fab(const mlgpu_grid &gr, int ncomp) { define(gr, ncomp); }
  void define(const mlgpu_grid &gr, int ncomp) {
    nc = ncomp;
    for (int d = 0; d < 3; d++) {
      n[d] = gr.n[d];
      g[d] = (d < gr.dim) ? 1 : 0;
    }
    s[0] = 1;
    s[1] = n[0] + 2 * g[0];
    s[2] = s[1] * (n[1] + 2 * g[1]);
    v.assign((size_t)nc * s[2] * (n[2] + 2 * g[2]), 0.0);
  }
  size_t plane() const { return (size_t)s[2] * (n[2] + 2 * g[2]); }
  double &operator()(int i, int j, int k, int c) {
    return v[(size_t)c * plane() + (size_t)(i + g[0]) + (size_t)(j + g[1]) * s[1] +
             (size_t)(k + g[2]) * s[2]];
  }
  double operator()(int i, int j, int k, int c) const {
    return v[(size_t)c * plane() + (size_t)(i + g[0]) + (size_t)(j + g[1]) * s[1] +
             (size_t)(k + g[2]) * s[2]];
  }
  void load(const double *dense) {
    for (int c = 0; c < nc; c++)
      for (int k = 0; k < n[2]; k++)
        for (int j = 0; j < n[1]; j++)
          for (int i = 0; i < n[0]; i++)
            (*this)(i, j, k, c) = dense[(((size_t)c * n[2] + k) * n[1] + j) * n[0] + i];
  }
  void store(double *dense) const {
    for (int c = 0; c < nc; c++)
      for (int k = 0; k < n[2]; k++)
        for (int j = 0; j < n[1]; j++)
          for (int i = 0; i < n[0]; i++)
            dense[(((size_t)c * n[2] + k) * n[1] + j) * n[0] + i] = (*this)(i, j, k, c);
  }
};

inline size_t ncells(const mlgpu_grid &g) { return (size_t)g.n[0] * g.n[1] * g.n[2]; }
inline size_t nfaces(const mlgpu_grid &g, int d) {
  size_t m = 1;
  for (int e = 0; e < 3; e++) m *= (size_t)(g.n[e] + (e == d ? 1 : 0));
  return m;
}
// face index of face (i,j,k) in direction d (face i sits between cells i-1, i)
inline size_t fidx(const mlgpu_grid &g, int d, int i, int j, int k, int c) {
  int m0 = g.n[0] + (d == 0), m1 = g.n[1] + (d == 1), m2 = g.n[2] + (d == 2);
  return (((size_t)c * m2 + k) * m1 + j) * m0 + i;
}

mlgpu_grid coarsen_grid(const mlgpu_grid &f) {
  mlgpu_grid c = f;
  for (int d = 0; d < f.dim; d++) c.n[d] = f.n[d] / 2;
  c.dx = f.dx * 2;
  return c;
}

// ------------------------------------------------------ BC functions
// Periodic exchange of the face ghosts (trimmed-edge copier: corners are
// not exchanged).
void exchange(Fab &f, const mlgpu_grid &gr) {
  for (int d = 0; d < gr.dim; d++) {
    if (!gr.periodic[d]) continue;
    int lo[3] = {0, 0, 0}, hi[3] = {f.n[0] - 1, f.n[1] - 1, f.n[2] - 1};
    for (int c = 0; c < f.nc; c++)
      for (int k = lo[2]; k <= hi[2]; k++)
        for (int j = lo[1]; j <= hi[1]; j++)
          for (int i = lo[0]; i <= hi[0]; i++) {
            int idx[3] = {i, j, k};
            if (idx[d] != 0 && idx[d] != f.n[d] - 1) continue;
            if (idx[d] == f.n[d] - 1) {
              int t[3] = {i, j, k};
              t[d] = -1;
              f(t[0], t[1], t[2], c) = f(i, j, k, c);
            }
            if (idx[d] == 0) {
              int t[3] = {i, j, k};
              t[d] = f.n[d];
              f(t[0], t[1], t[2], c) = f(i, j, k, c);
            }
          }
  }
}

// MixedBCTemperatureSalinity on the derived T (BCutil/PhysBCUtil.cpp:764-800):
// T_g = (T_i (a/m_dx + b/2) + F - b T_ref) / (a/m_dx - b/2), the radiation
// constants a, b, T_ref of [dir][side] and the condition's spacing m_dx.
// p1 = a/dx + b/2, bt = b T_ref, p2 = a/dx - b/2; g = p1 / p2 is the ghost's
// derivative in the interior value, f = 1 / p2 in F.
struct MixedT {
  double p1, bt, p2, g, f;
};
MixedT mixed_t(const mlgpu_nlbc &nb, double grid_dx, int d, int side) {
  const double dx = nb.dx > 0 ? nb.dx : grid_dx;
  MixedT m;
  m.p1 = nb.a[d][side] / dx + nb.b[d][side] / 2;
  m.bt = nb.b[d][side] * nb.T_ref[d][side];
  m.p2 = nb.a[d][side] / dx - nb.b[d][side] / 2;
  m.g = m.p1 / m.p2;
  m.f = 1.0 / m.p2;
  return m;
}

// DIRIBC order 1 (BCutil/BCFuncF.ChF:14-57) and NEUMBC (:63-95) on the ghost
// row adjacent to the valid box (adjCellBox, BCFunctions.cpp:101-161); with
// `nb`, the derived state's mixed temperature condition on comp 0 (its
// homogeneous form g T_i is the linearised rule).
void physbc(Fab &f, const mlgpu_grid &gr, const mlgpu_bc &bc, bool homogeneous,
            const mlgpu_nlbc *nb = nullptr) {
  for (int d = 0; d < gr.dim; d++) {
    if (gr.periodic[d]) continue;
    for (int side = 0; side < 2; side++) {
      int isign = side == 0 ? -1 : 1;
      for (int c = 0; c < f.nc; c++) {
        int type = bc.type[d][side][c];
        double val = homogeneous ? 0.0 : bc.value[d][side][c];
        const bool mixed = nb && c == 0 && type == MLGPU_BC_MIXED_TEMPERATURE_SALINITY;
        const MixedT mt = mixed ? mixed_t(*nb, gr.dx, d, side) : MixedT{0, 0, 0, 0, 0};
        int lo[3] = {0, 0, 0}, hi[3] = {f.n[0] - 1, f.n[1] - 1, f.n[2] - 1};
        lo[d] = hi[d] = (side == 0) ? -1 : f.n[d];
        for (int k = lo[2]; k <= hi[2]; k++)
          for (int j = lo[1]; j <= hi[1]; j++)
            for (int i = lo[0]; i <= hi[0]; i++) {
              int t[3] = {i, j, k};
              t[d] -= isign;
              double phi1 = f(t[0], t[1], t[2], c);
              if (mixed)
                f(i, j, k, c) = homogeneous ? mt.g * phi1 : (phi1 * mt.p1 + val - mt.bt) / mt.p2;
              else if (type == MLGPU_BC_DIRICHLET)
                f(i, j, k, c) = 2 * val - phi1;
              else
                f(i, j, k, c) = phi1 + (isign * gr.dx) * val;
            }
      }
    }
  }
}

// a derived-condition wall's share of the diagonal face sum (the ghost's
// homogeneous rule g T_i gives the face term b (g - 1) T_i): 2b Dirichlet,
// 0 Neumann, (1 - g) b for the mixed temperature condition
double dbc_wall_diag(const mlgpu_nlop &op, int d, int side, int c, double bf) {
  const int t = op.derived_bc.type[d][side][c];
  if (t == MLGPU_BC_DIRICHLET) return 2 * bf;
  if (t == MLGPU_BC_MIXED_TEMPERATURE_SALINITY && c == 0)
    return (1.0 - mixed_t(op.nlbc, op.grid.dx, d, side).g) * bf;
  return 0.0;
}

void fill_ghosts(Fab &f, const mlgpu_grid &gr, const mlgpu_bc &bc, bool homogeneous) {
  exchange(f, gr);
  physbc(f, gr, bc, homogeneous);
}

// Homogeneous ghost fill including edges and corners, direction by
// direction over the already-extended ranges; used for the coarse correction
// read by the prolongation.
void fill_ghosts_full_homog(Fab &f, const mlgpu_grid &gr, const mlgpu_bc &bc) {
  for (int d = 0; d < gr.dim; d++) {
    int lo[3], hi[3];
    for (int e = 0; e < 3; e++) {
      lo[e] = (e < d) ? -f.g[e] : 0;
      hi[e] = (e < d) ? f.n[e] - 1 + f.g[e] : f.n[e] - 1;
    }
    for (int side = 0; side < 2; side++) {
      int gl[3] = {lo[0], lo[1], lo[2]}, gh[3] = {hi[0], hi[1], hi[2]};
      gl[d] = gh[d] = (side == 0) ? -1 : f.n[d];
      for (int c = 0; c < f.nc; c++)
        for (int k = gl[2]; k <= gh[2]; k++)
          for (int j = gl[1]; j <= gh[1]; j++)
            for (int i = gl[0]; i <= gh[0]; i++) {
              int t[3] = {i, j, k};
              if (gr.periodic[d]) {
                t[d] = (side == 0) ? f.n[d] - 1 : 0;
                f(i, j, k, c) = f(t[0], t[1], t[2], c);
              } else {
                t[d] = (side == 0) ? 0 : f.n[d] - 1;
                double v = f(t[0], t[1], t[2], c);
                f(i, j, k, c) = (bc.type[d][side][c] == MLGPU_BC_DIRICHLET) ? -v : v;
              }
            }
    }
  }
}

// ------------------------------------------------------------ closure
// CALCULATE_BOUNDING_ENERGY (src/EnthalpyVariablesF.ChF:657-698)
inline void bounding_energy(double C, const mlgpu_params &p, double &Hs, double &He,
                            double &Hl) {
  const double CR = p.compositionRatio, k = p.waterDistributionCoeff,
               cp = p.specificHeatRatio, St = p.stefan, te = p.thetaEutectic,
               Te = p.ThetaEutectic;
  if (C < -CR)
    Hs = 0.0;
  else
    Hs = cp * ((-C - CR) / k);
  if (Hs < 0.0) Hs = 0.0;
  Hs = Hs + te * cp;
  double pe = (CR + C) / (CR + Te);
  He = pe * (St + te * (1 - cp)) + cp * te;
  Hl = St - C + te + Te;
}

// CALCULATEPOROSITYMUSH (src/EnthalpyVariablesF.ChF:103-150), clamps C >= -CR.
inline double porosity_mush(double C, double H, const mlgpu_params &p) {
  const double CR = p.compositionRatio, k = p.waterDistributionCoeff,
               cp = p.specificHeatRatio, St = p.stefan;
  double validC = (C >= -CR) ? C : -CR;
  if (St == 0) return 1;
  double a = CR * (cp - 1) + St * (k - 1);
  double b = CR * (1 - 2 * cp) + H * (1 - k) - validC * (cp - 1) - k * St;
  double c = (CR + validC) * cp + k * H;
  return (-b - std::sqrt(b * b - 4 * a * c)) / (2 * a);
}

// CALCULATE_T_CL (src/EnthalpyVariablesF.ChF:419-467)
inline void t_cl(double H, double C, const mlgpu_params &p, double &T, double &Cl) {
  double Hs, He, Hl;
  bounding_energy(C, p, Hs, He, Hl);
  const double CR = p.compositionRatio, k = p.waterDistributionCoeff;
  if (H <= Hs) {
    T = H / p.specificHeatRatio;
    Cl = p.ThetaEutectic;
  } else if (H > Hs && H <= He) {
    T = p.thetaEutectic;
    Cl = p.ThetaEutectic;
  } else if (H > He && H < Hl) {
    double por = porosity_mush(C, H, p);
    T = -(C + CR * (1 - por)) / (por + k * (1 - por));
    Cl = (C + CR * (1 - por)) / (por + k * (1 - por));
  } else if (H >= Hl) {
    T = H - p.stefan;
    Cl = C;
  } else {
    // NaN input.  This departs from the reference: CALCULATE_T_CL takes no
    // branch for a NaN and leaves T and C_l as they were in the output
    // array.  Here both become NaN (T = H, C_l = C), so a poisoned state
    // stays poisoned and the solvers' NaN detection sees it; the device
    // closure does the same.
    T = H;
    Cl = C;
  }
}

// Derivative of t_cl, J = {dT/dH, dT/dC, dC_l/dH, dC_l/dC} (no counterpart in
// the reference: the linearisation used by the mixed-precision nonlinear
// solve).  Regimes as t_cl; in the mush the porosity root of
// a por^2 + b por + c = 0 is differentiated implicitly, C clamped at -CR.
inline void t_cl_jac(double H, double C, const mlgpu_params &p, double J[4]) {
  double Hs, He, Hl;
  bounding_energy(C, p, Hs, He, Hl);
  const double CR = p.compositionRatio, k = p.waterDistributionCoeff,
               cp = p.specificHeatRatio, St = p.stefan;
  J[0] = J[1] = J[2] = J[3] = 0.0;
  if (H <= Hs) {
    J[0] = 1.0 / cp;
  } else if (H > Hs && H <= He) {
  } else if (H > He && H < Hl) {
    double por = 1.0, dpH = 0.0, dpC = 0.0;
    if (St != 0) {
      const bool clamp = !(C >= -CR);
      const double vC = clamp ? -CR : C;
      const double a = CR * (cp - 1) + St * (k - 1);
      const double b = CR * (1 - 2 * cp) + H * (1 - k) - vC * (cp - 1) - k * St;
      const double c = (CR + vC) * cp + k * H;
      const double sD = std::sqrt(b * b - 4 * a * c);
      por = (-b - sD) / (2 * a);
      const double dbH = 1 - k, dbC = clamp ? 0.0 : -(cp - 1), dcH = k, dcC = clamp ? 0.0 : cp;
      dpH = (-dbH - (b * dbH - 2 * a * dcH) / sD) / (2 * a);
      dpC = (-dbC - (b * dbC - 2 * a * dcC) / sD) / (2 * a);
    }
    const double num = C + CR * (1 - por), den = por + k * (1 - por);
    const double dcl = (-CR * den - num * (1 - k)) / (den * den);
    J[2] = dcl * dpH;
    J[3] = 1.0 / den + dcl * dpC;
    J[0] = -J[2];
    J[1] = -J[3];
  } else if (H >= Hl) {
    J[0] = 1.0;
    J[3] = 1.0;
  }
}

// ------------------------------------ nonlinear temperature conditions
// computeTemperature (src/phaseDiagram.cpp:225-258) as called by
// MushyLayerParams::computeTemperature (src/MushyLayerParams.cpp:1312-1321):
// bounding energies of computeBoundingEnergy (:326-341, H_s with
// std::max(0, (-C - CR)/k)) and the unclamped root of
// computePorosityMushyLayer (:298-324).
double pd_temperature(double H, double C, const mlgpu_params &p) {
  const double CR = p.compositionRatio, k = p.waterDistributionCoeff,
               cp = p.specificHeatRatio, St = p.stefan, te = p.thetaEutectic,
               Te = p.ThetaEutectic;
  const double zero = 0.0;
  const double H_s = cp * (te + std::max(zero, (-C - CR) / k));
  const double chi_e = (CR + C) / (Te + CR);
  const double H_e = chi_e * (St + te * (1 - cp)) + cp * te;
  const double H_l = St - C + te + Te;
  if (H <= H_s) return H / cp;
  if (H > H_s && H <= H_e) return te;
  if (H > H_e && H < H_l) {
    double por;
    if (St == 0) {
      por = 1;
    } else {
      double a = CR * (cp - 1) + St * (k - 1);
      double b = CR * (1 - 2 * cp) + H * (1 - k) - C * (cp - 1) - k * St;
      double c = (C + CR) * cp + k * H;
      por = (-b - std::sqrt(b * b - 4 * a * c)) / (2 * a);
    }
    return -(C + CR * (1 - por)) / (por + k * (1 - por));
  }
  return H - St;
}

// NonlinearTemperatureBCRobin (BCutil/NonlinearBC.H:63-122)
struct RobinTemperatureBC {
  mlgpu_params params;
  double dx, a, b, F, T_ref;
  // computeResidual (:88-116)
  double residual(double H_ghost, double C_ghost, double T_interior) const {
    double T_ghost = pd_temperature(H_ghost, C_ghost, params);
    double predicted = (T_interior * a / dx + F + b * T_interior / 2 - T_ref * b) / (a / dx - b / 2);
    double r = predicted - T_ghost;
    if (std::fabs(r) > 10.0) r = 0.0;
    return r;
  }
};

// NonlinearBCSolverPicard::solve (BCutil/NonlinearBC.H:194-233)
void solve_picard(const RobinTemperatureBC &R, const mlgpu_nlbc &nb, double &H_ghost,
                  double T_interior, double C_ghost) {
  double r = R.residual(H_ghost, C_ghost, T_interior);
  H_ghost = H_ghost + nb.relax_coeff * r;
  int iter = 0;
  while (std::fabs(r) > nb.max_residual && iter < nb.max_iter) {
    r = R.residual(H_ghost, C_ghost, T_interior);
    H_ghost = H_ghost + nb.relax_coeff * r;
    iter++;
  }
}

// NonlinearBCSolverNewton::solve (BCutil/NonlinearBC.H:259-301)
void solve_newton(const RobinTemperatureBC &R, const mlgpu_nlbc &nb, double &H_ghost,
                  double T_interior, double C_ghost) {
  double dH = 0.01;
  double r_old = nb.max_residual * 10, r_new = nb.max_residual * 10;
  int iter = 0;
  while (std::fabs(r_old) > nb.max_residual && iter < nb.max_iter) {
    r_old = R.residual(H_ghost, C_ghost, T_interior);
    r_new = R.residual(H_ghost + dH, C_ghost, T_interior);
    if (std::fabs(r_new - r_old) < nb.max_residual) {
      H_ghost = H_ghost + r_old;
      dH = 2 * dH;
    } else {
      H_ghost = H_ghost - r_old * (dH) / (r_new - r_old);
    }
    iter++;
  }
}

// AdvectDiffuseScalarBC temperature branch for the enthalpy component
// (BCutil/PhysBCUtil.cpp:590-722): Robin coefficients by condition type,
// then per ghost cell of the face row either the interior enthalpy (below the
// no-flux limit along the next direction) or the solved ghost enthalpy, with
// the interior concentration as ghost concentration.  The spacing is the one
// the condition object was built with (PhysBCUtil m_dx).
void temperature_bc(Fab &f, const mlgpu_nlop &op, int d, int side) {
  const int type = op.phi_bc.type[d][side][0];
  const double value = op.phi_bc.value[d][side][0];
  const mlgpu_nlbc &nb = op.nlbc;
  RobinTemperatureBC R;
  R.params = op.params;
  R.dx = nb.dx > 0 ? nb.dx : op.grid.dx;
  R.a = 0.0;
  R.b = 0.0;
  R.F = 0.0;
  R.T_ref = 0.0;
  if (type == MLGPU_BC_FIXED_TEMPERATURE) {
    R.T_ref = value;
    R.b = 1.0;
  } else if (type == MLGPU_BC_TEMPERATURE_FLUX) {
    R.F = value;
    R.a = 1.0;
  } else {
    R.a = nb.a[d][side];
    R.b = nb.b[d][side];
    R.F = value;
    R.T_ref = nb.T_ref[d][side];
  }
  const int isign = side == 0 ? -1 : 1;
  const int perp = (d == op.grid.dim - 1) ? 0 : d + 1;
  int lo[3] = {0, 0, 0}, hi[3] = {f.n[0] - 1, f.n[1] - 1, f.n[2] - 1};
  lo[d] = hi[d] = (side == 0) ? -1 : f.n[d];
  for (int k = lo[2]; k <= hi[2]; k++)
    for (int j = lo[1]; j <= hi[1]; j++)
      for (int i = lo[0]; i <= hi[0]; i++) {
        int iv[3] = {i, j, k};
        iv[d] -= isign;
        const double H_i = f(iv[0], iv[1], iv[2], 0), C_i = f(iv[0], iv[1], iv[2], 1);
        const double face_pos = R.dx * (iv[perp] + 0.5);
        if (face_pos < nb.no_flux_limit[d][side]) {
          f(i, j, k, 0) = H_i;
          continue;
        }
        const double T_i = pd_temperature(H_i, C_i, op.params);
        double H_g = H_i;
        if (nb.method == MLGPU_NLBC_NEWTON)
          solve_newton(R, nb, H_g, T_i, C_i);
        else
          solve_picard(R, nb, H_g, T_i, C_i);
        f(i, j, k, 0) = H_g;
      }
}

// CALCULATEPOROSITY/CL/CS/T (src/EnthalpyVariablesF.ChF:13-284) for one cell.
inline void full_closure(double H, double C, const mlgpu_params &p, double &T,
                         double &por, double &Cl, double &Cs, double &Hs, double &He,
                         double &Hl) {
  bounding_energy(C, p, Hs, He, Hl);
  const double CR = p.compositionRatio, k = p.waterDistributionCoeff,
               cp = p.specificHeatRatio, St = p.stefan, te = p.thetaEutectic,
               Te = p.ThetaEutectic;
  if (H <= Hs) {
    por = 0;
    Cl = Te;
    Cs = C;
    T = H / cp;
  } else if (H > Hs && H <= He) {
    por = (H - te * cp) / (St + te * (1 - cp));
    Cl = Te;
    double pm = porosity_mush(C, H, p);  // CALCULATECS uses the mush root here
    Cs = C / (1 - pm);
    T = te;
  } else if (H > He && H < Hl) {
    double pm = porosity_mush(C, H, p);
    por = pm;
    Cl = (C + CR * (1 - pm)) / (pm + k * (1 - pm));
    Cs = (C * k - CR * pm) / (pm + k * (1 - pm));
    T = -(C + CR * (1 - pm)) / (pm + k * (1 - pm));
  } else if (H >= Hl) {
    por = 1;
    Cl = C;
    Cs = 0;
    T = H - St;
  } else {
    por = H; Cl = H; Cs = H; T = H;
  }
}

// computeDiffusedVar (src/AMRNonLinearMultiCompOp.cpp:57-98): closure over
// the whole ghosted box, then the derived-variable BC.
void diffused_var(Fab &out, const Fab &phi, const mlgpu_nlop &op) {
  out.define(op.grid, 2);
  int lo[3], hi[3];
  for (int d = 0; d < 3; d++) {
    lo[d] = -phi.g[d];
    hi[d] = phi.n[d] - 1 + phi.g[d];
  }
  for (int k = lo[2]; k <= hi[2]; k++)
    for (int j = lo[1]; j <= hi[1]; j++)
      for (int i = lo[0]; i <= hi[0]; i++) {
        double T, Cl;
        t_cl(phi(i, j, k, 0), phi(i, j, k, 1), op.params, T, Cl);
        out(i, j, k, 0) = T;
        out(i, j, k, 1) = Cl;
      }
  if (op.apply_derived_bc) physbc(out, op.grid, op.derived_bc, false, &op.nlbc);
}

// --------------------------------------------------- face coefficients
struct Faces {
  const double *b[3] = {nullptr, nullptr, nullptr};
  mlgpu_grid g;
  double operator()(int d, int i, int j, int k, int c) const {
    return b[d][fidx(g, d, i, j, k, c)];
  }
};

// Flat Fortran sum over directions:
// b0(i+1)(p(i+1)-p0) - b0(i)(p0-p(i-1)) + b1(j+1)(..) - b1(j)(..) [+ b2 ..]
inline double flux_sum(const Faces &B, const Fab &pl, int i, int j, int k, int c,
                       int dim) {
  double p0 = pl(i, j, k, c);
  double s = B(0, i + 1, j, k, c) * (pl(i + 1, j, k, c) - p0) -
             B(0, i, j, k, c) * (p0 - pl(i - 1, j, k, c));
  s = s + B(1, i, j + 1, k, c) * (pl(i, j + 1, k, c) - p0);
  s = s - B(1, i, j, k, c) * (p0 - pl(i, j - 1, k, c));
  if (dim == 3) {
    s = s + B(2, i, j, k + 1, c) * (pl(i, j, k + 1, c) - p0);
    s = s - B(2, i, j, k, c) * (p0 - pl(i, j, k - 1, c));
  }
  return s;
}

// resetLambda (AMRNonLinearMultiCompOp.cpp:540-573 / DarcyBrinkmanOp.cpp:
// 265-296): lambda = a*alpha [+ (-beta) c] + sum_d scale*beta*(b_hi + b_lo),
// then 1/lambda.
inline double lambda_at(const Faces &B, const double *a, const double *cc,
                        double alpha, double beta, double scale, size_t cell, int i,
                        int j, int k, int c, int dim) {
  double l = (a ? a[cell] : 1.0) * alpha;
  if (cc) l = l + (-beta) * cc[cell];
  for (int d = 0; d < dim; d++) {
    int ip = i + (d == 0), jp = j + (d == 1), kp = k + (d == 2);
    double sumVal = B(d, ip, jp, kp, c) + B(d, i, j, k, c);
    l = l + scale * beta * sumVal;
  }
  return 1.0 / l;
}

inline size_t cidx(const mlgpu_grid &g, int i, int j, int k, int c) {
  return (((size_t)c * g.n[2] + k) * g.n[1] + j) * g.n[0] + i;
}

Faces make_faces(const mlgpu_grid &g, const void *const b[3]) {
  Faces F;
  F.g = g;
  for (int d = 0; d < 3; d++) F.b[d] = (const double *)b[d];
  return F;
}

// -------------------------------------------------- nonlinear operator
struct NLCtx {
  const mlgpu_nlop &op;
  Faces B;
  const double *a;
  double dxinv, scale;
  int nc = 2;
  explicit NLCtx(const mlgpu_nlop &o) : op(o) {
    B = make_faces(o.grid, o.bCoef);
    a = (const double *)o.aCoef;
    dxinv = 1.0 / (o.grid.dx * o.grid.dx);
    scale = 1.0 / (o.grid.dx * o.grid.dx);
  }
  // L(phi) at a cell given phi and the diffused variable (NLVCCOMPUTEOP)
  double lofphi(const Fab &phi, const Fab &pl, int i, int j, int k, int c) const {
    size_t cell = cidx(op.grid, i, j, k, c);
    double av = a ? a[cell] : 1.0;
    return op.alpha * av * phi(i, j, k, c) -
           op.beta * flux_sum(B, pl, i, j, k, c, op.grid.dim) * dxinv;
  }
};

// (H, C) ghosts: exchange, the linear conditions, then the temperature
// conditions on H where phi_bc comp 0 names one (they read interior cells only)
void nl_fill_ghosts(Fab &phi, const mlgpu_nlop &op) {
  fill_ghosts(phi, op.grid, op.phi_bc, false);
  for (int d = 0; d < op.grid.dim; d++) {
    if (op.grid.periodic[d]) continue;
    for (int side = 0; side < 2; side++) {
      int t = op.phi_bc.type[d][side][0];
      if (t == MLGPU_BC_FIXED_TEMPERATURE || t == MLGPU_BC_TEMPERATURE_FLUX ||
          t == MLGPU_BC_TEMPERATURE_FLUX_RADIATION)
        temperature_bc(phi, op, d, side);
    }
  }
}

void nl_prepare(Fab &phi, Fab &pl, const mlgpu_nlop &op, const double *phid) {
  phi.define(op.grid, 2);
  phi.load(phid);
  nl_fill_ghosts(phi, op);
  diffused_var(pl, phi, op);
}

template <class F>
void for_cells(const mlgpu_grid &g, F f) {
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < g.n[2]; k++)
    for (int j = 0; j < g.n[1]; j++)
      for (int i = 0; i < g.n[0]; i++) f(i, j, k);
}

// one red/black pass: NONLINEARSMOOTHING (F.ChF:50-198) with lambda inline
void nl_gsrb_pass_fab(Fab &phi, const double *rhs, const mlgpu_nlop &op, int pass) {
  NLCtx X(op);
  nl_fill_ghosts(phi, op);
  Fab pl;
  diffused_var(pl, phi, op);
  const mlgpu_grid &g = op.grid;
  for (int c = 0; c < 2; c++) {
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < g.n[2]; k++)
      for (int j = 0; j < g.n[1]; j++) {
        int imin = std::abs((j + k + pass) % 2);
        for (int i = imin; i < g.n[0]; i += 2) {
          size_t cell = cidx(g, i, j, k, c);
          double lam = lambda_at(X.B, X.a, nullptr, op.alpha, op.beta, X.scale, cell,
                                 i, j, k, c, g.dim);
          double lof = X.lofphi(phi, pl, i, j, k, c);
          phi(i, j, k, c) = phi(i, j, k, c) - lam * (lof - rhs[cell]);
        }
      }
  }
}

// ------------------------------------------------------ linear operator
struct VCCtx {
  const mlgpu_vcop &op;
  Faces B;
  const double *a, *cc;
  double dxinv, scale;
  explicit VCCtx(const mlgpu_vcop &o) : op(o) {
    B = make_faces(o.grid, o.bCoef);
    a = (const double *)o.aCoef;
    cc = (const double *)o.cCoef;
    dxinv = 1.0 / (o.grid.dx * o.grid.dx);
    scale = 1.0 / (o.grid.dx * o.grid.dx);
  }
  // DBCOMPUTEOP (F.ChF:182-274); without c it is the VC Poisson operator
  double lofphi(const Fab &phi, int i, int j, int k) const {
    size_t cell = cidx(op.grid, i, j, k, 0);
    double av = a ? a[cell] : 1.0;
    double v = op.alpha * av * phi(i, j, k, 0);
    if (cc) v = v - op.beta * cc[cell] * phi(i, j, k, 0);
    return v - op.beta * flux_sum(B, phi, i, j, k, 0, op.grid.dim) * dxinv;
  }
};

void vc_gsrb_pass_fab(Fab &phi, const double *rhs, const mlgpu_vcop &op, int pass) {
  VCCtx X(op);
  fill_ghosts(phi, op.grid, op.bc, true);  // levelGSRB: homogeneous BCs
  const mlgpu_grid &g = op.grid;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < g.n[2]; k++)
    for (int j = 0; j < g.n[1]; j++) {
      int imin = std::abs((j + k + pass) % 2);
      for (int i = imin; i < g.n[0]; i += 2) {
        size_t cell = cidx(g, i, j, k, 0);
        double lam = lambda_at(X.B, X.a, X.cc, op.alpha, op.beta, X.scale, cell, i, j,
                               k, 0, g.dim);
        double lof = X.lofphi(phi, i, j, k);
        phi(i, j, k, 0) = phi(i, j, k, 0) - lam * (lof - rhs[cell]);
      }
    }
}

// ------------------------------------------------------------ transfers
// RESTRICT / RESTRICTRESNLVC accumulation order: fine cells of a coarse cell
// in Fortran loop order (k, j outer; i fastest), each scaled by 1/2^D.
template <class F>
void restrict_loop(const mlgpu_grid &fg, int ncomp, double *coarse, F fine_val) {
  mlgpu_grid cg = coarsen_grid(fg);
  double denom = fg.dim == 3 ? 8.0 : 4.0;
  int r2 = fg.dim == 3 ? 2 : 1;
  for (int c = 0; c < ncomp; c++) {
#pragma omp parallel for collapse(2) schedule(static)
    for (int K = 0; K < cg.n[2]; K++)
      for (int J = 0; J < cg.n[1]; J++)
        for (int I = 0; I < cg.n[0]; I++) {
          double acc = 0.0;
          for (int kk = 0; kk < r2; kk++)
            for (int jj = 0; jj < 2; jj++)
              for (int ii = 0; ii < 2; ii++)
                acc = acc + fine_val(2 * I + ii, 2 * J + jj, r2 == 2 ? 2 * K + kk : 0, c) / denom;
          coarse[cidx(cg, I, J, K, c)] = acc;
        }
  }
}

void prolong_fab(const mlgpu_grid &fg, const mlgpu_bc &bc, int ncomp, int kind,
                 double *fine, const double *coarse) {
  mlgpu_grid cg = coarsen_grid(fg);
  Fab C(cg, ncomp);
  C.load(coarse);
  fill_ghosts_full_homog(C, cg, bc);
  int dim = fg.dim;
  double den = 1.0 / (dim == 3 ? 64.0 : 16.0);
  double fx1 = 3.0 * den, fx2 = 9.0 * den, fx3 = 27.0 * den, f0 = 1.0 * den;
  for (int c = 0; c < ncomp; c++) {
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < fg.n[2]; k++)
      for (int j = 0; j < fg.n[1]; j++)
        for (int i = 0; i < fg.n[0]; i++) {
          int ic = i / 2, jc = j / 2, kc = (dim == 3) ? k / 2 : 0;
          double &p = fine[cidx(fg, i, j, k, c)];
          if (kind == MLGPU_PROLONG_CONSTANT) {
            p = p + C(ic, jc, kc, c);
            continue;
          }
          int o1 = 2 * (i % 2) - 1, o2 = 2 * (j % 2) - 1, o3 = (dim == 3) ? 2 * (k % 2) - 1 : 0;
          if (dim == 2) {
            p = p + fx2 * C(ic, jc, kc, c) + f0 * C(ic + o1, jc + o2, kc, c);
            p = p + fx1 * (C(ic + o1, jc, kc, c) + C(ic, jc + o2, kc, c));
          } else {
            p = p + fx3 * C(ic, jc, kc, c) + f0 * C(ic + o1, jc + o2, kc + o3, c);
            p = p + fx2 * (C(ic + o1, jc, kc, c) + C(ic, jc + o2, kc, c) + C(ic, jc, kc + o3, c));
            p = p + fx1 * (C(ic + o1, jc + o2, kc, c) + C(ic, jc + o2, kc + o3, c) +
                           C(ic + o1, jc, kc + o3, c));
          }
        }
  }
}

// CoarseAverageFace (arithmetic): sum of the 2^(D-1) covered fine faces in
// Fortran order, times 1/2^(D-1).
void coarsen_faces(const mlgpu_grid &fg, int ncomp, int d, double *cf, const double *ff) {
  mlgpu_grid cg = coarsen_grid(fg);
  int dim = fg.dim;
  double refScale = dim == 3 ? 0.25 : 0.5;
  int m[3];
  for (int e = 0; e < 3; e++) m[e] = cg.n[e] + (e == d);
  for (int c = 0; c < ncomp; c++)
    for (int K = 0; K < m[2]; K++)
      for (int J = 0; J < m[1]; J++)
        for (int I = 0; I < m[0]; I++) {
          int r[3] = {2, 2, dim == 3 ? 2 : 1};
          r[d] = 1;
          double sum = 0.0;
          for (int kk = 0; kk < r[2]; kk++)
            for (int jj = 0; jj < r[1]; jj++)
              for (int ii = 0; ii < r[0]; ii++) {
                int fi = 2 * I + ii, fj = 2 * J + jj, fk = (dim == 3) ? 2 * K + kk : 0;
                sum = sum + ff[fidx(fg, d, fi, fj, fk, c)];
              }
          cf[fidx(cg, d, I, J, K, c)] = sum * refScale;
        }
}

double norm_of(const double *x, size_t n, int type) {
  double r = 0;
  if (type == MLGPU_NORM_MAX) {
    // a NaN stays in the maximum (std::max would drop it and report a
    // poisoned field as converged), so every solver reads it as non-finite
    for (size_t i = 0; i < n; i++) {
      const double a = std::fabs(x[i]);
      if (a > r || a != a) r = a;
    }
    return r;
  }
  if (type == MLGPU_NORM_L1) {
    for (size_t i = 0; i < n; i++) r += std::fabs(x[i]);
    return r;
  }
  for (size_t i = 0; i < n; i++) r += x[i] * x[i];
  return std::sqrt(r);
}

bool has_nan(const double *x, size_t n) {
  for (size_t i = 0; i < n; i++)
    if (!std::isfinite(x[i])) return true;
  return false;
}

}  // namespace

// ====================================================================== C ABI
extern "C" {

// host threads of the OpenMP loops (the timed CPU baseline runs at 1 and at
// all cores); returns the count now in effect
int orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

int orc_closure(const mlgpu_grid *g, const mlgpu_params *p, const double *HC, double *T,
                double *por, double *Cl, double *Cs, double *Hs, double *He,
                double *Hl) {
  size_t n = ncells(*g);
#pragma omp parallel for schedule(static)
  for (size_t q = 0; q < n; q++) {
    double t, po, cl, cs, hs, he, hl;
    full_closure(HC[q], HC[n + q], *p, t, po, cl, cs, hs, he, hl);
    if (T) T[q] = t;
    if (por) por[q] = po;
    if (Cl) Cl[q] = cl;
    if (Cs) Cs[q] = cs;
    if (Hs) Hs[q] = hs;
    if (He) He[q] = he;
    if (Hl) Hl[q] = hl;
  }
  return 0;
}

int orc_closure_tcl(const mlgpu_grid *g, const mlgpu_params *p, const double *HC,
                    double *TCl) {
  size_t n = ncells(*g);
#pragma omp parallel for schedule(static)
  for (size_t q = 0; q < n; q++) t_cl(HC[q], HC[n + q], *p, TCl[q], TCl[n + q]);
  return 0;
}

// J[4][cells] = d(T, C_l)/d(H, C) of every cell
// d porosity/d(H, C) of the full closure (no counterpart in the reference):
// eutectic 1/(St + te (1 - cp)) in H, the mush root differentiated
// implicitly (C clamped at -CR), zero elsewhere
int orc_porosity_jac(const mlgpu_grid *g, const mlgpu_params *p, const double *HC, double *dp) {
  size_t n = ncells(*g);
  const double CR = p->compositionRatio, k = p->waterDistributionCoeff,
               cp = p->specificHeatRatio, St = p->stefan, te = p->thetaEutectic;
  for (size_t q = 0; q < n; q++) {
    double H = HC[q], C = HC[q + n], Hs, He, Hl;
    bounding_energy(C, *p, Hs, He, Hl);
    double d0 = 0.0, d1 = 0.0;
    if (H <= Hs) {
    } else if (H > Hs && H <= He) {
      d0 = 1.0 / (St + te * (1 - cp));
    } else if (H > He && H < Hl) {
      if (St != 0) {
        const bool clamp = !(C >= -CR);
        const double vC = clamp ? -CR : C;
        const double a = CR * (cp - 1) + St * (k - 1);
        const double b = CR * (1 - 2 * cp) + H * (1 - k) - vC * (cp - 1) - k * St;
        const double c = (CR + vC) * cp + k * H;
        const double sD = std::sqrt(b * b - 4 * a * c);
        const double dbH = 1 - k, dbC = clamp ? 0.0 : -(cp - 1), dcH = k, dcC = clamp ? 0.0 : cp;
        d0 = (-dbH - (b * dbH - 2 * a * dcH) / sD) / (2 * a);
        d1 = (-dbC - (b * dbC - 2 * a * dcC) / sD) / (2 * a);
      }
    }
    dp[q] = d0;
    dp[q + n] = d1;
  }
  return 0;
}

int orc_closure_jac(const mlgpu_grid *g, const mlgpu_params *p, const double *HC, double *J) {
  size_t n = ncells(*g);
#pragma omp parallel for schedule(static)
  for (size_t q = 0; q < n; q++) {
    double j4[4];
    t_cl_jac(HC[q], HC[n + q], *p, j4);
    for (int m = 0; m < 4; m++) J[m * n + q] = j4[m];
  }
  return 0;
}

int orc_nl_residual(const mlgpu_nlop *op, double *res, const double *phid,
                    const double *rhs) {
  Fab phi, pl;
  nl_prepare(phi, pl, *op, phid);
  NLCtx X(*op);
  for (int c = 0; c < 2; c++)
    for_cells(op->grid, [&](int i, int j, int k) {
      size_t cell = cidx(op->grid, i, j, k, c);
      res[cell] = rhs[cell] - X.lofphi(phi, pl, i, j, k, c);
    });
  return 0;
}

int orc_nl_apply(const mlgpu_nlop *op, double *lhs, const double *phid) {
  Fab phi, pl;
  nl_prepare(phi, pl, *op, phid);
  NLCtx X(*op);
  for (int c = 0; c < 2; c++)
    for_cells(op->grid, [&](int i, int j, int k) {
      lhs[cidx(op->grid, i, j, k, c)] = X.lofphi(phi, pl, i, j, k, c);
    });
  return 0;
}

int orc_nl_gsrb_pass(const mlgpu_nlop *op, double *phid, const double *rhs, int pass) {
  Fab phi(op->grid, 2);
  phi.load(phid);
  nl_gsrb_pass_fab(phi, rhs, *op, pass);
  phi.store(phid);
  return 0;
}

int orc_nl_relax(const mlgpu_nlop *op, double *phid, const double *rhs, int n) {
  Fab phi(op->grid, 2);
  phi.load(phid);
  for (int s = 0; s < n; s++) {
    nl_gsrb_pass_fab(phi, rhs, *op, 0);
    nl_gsrb_pass_fab(phi, rhs, *op, 1);
  }
  phi.store(phid);
  return 0;
}

int orc_nl_lambda(const mlgpu_nlop *op, double *lam) {
  NLCtx X(*op);
  for (int c = 0; c < 2; c++)
    for_cells(op->grid, [&](int i, int j, int k) {
      size_t cell = cidx(op->grid, i, j, k, c);
      lam[cell] = lambda_at(X.B, X.a, nullptr, op->alpha, op->beta, X.scale, cell, i, j,
                            k, c, op->grid.dim);
    });
  return 0;
}

// levelJacobi (AMRNonLinearMultiCompOp.cpp:1077-1101): phi + 0.5*(r*lambda)
int orc_nl_jacobi(const mlgpu_nlop *op, double *phid, const double *rhs) {
  size_t n = 2 * ncells(op->grid);
  std::vector<double> r(n), lam(n);
  orc_nl_residual(op, r.data(), phid, rhs);
  orc_nl_lambda(op, lam.data());
  for (size_t q = 0; q < n; q++) phid[q] = phid[q] + 0.5 * (r[q] * lam[q]);
  return 0;
}

int orc_nl_restrict_residual(const mlgpu_nlop *op, double *resc, const double *phid,
                             const double *rhs) {
  Fab phi, pl;
  nl_prepare(phi, pl, *op, phid);
  NLCtx X(*op);
  restrict_loop(op->grid, 2, resc, [&](int i, int j, int k, int c) {
    return rhs[cidx(op->grid, i, j, k, c)] - X.lofphi(phi, pl, i, j, k, c);
  });
  return 0;
}

int orc_restrict_average(const mlgpu_grid *g, int ncomp, double *coarse,
                         const double *fine) {
  restrict_loop(*g, ncomp, coarse, [&](int i, int j, int k, int c) {
    return fine[cidx(*g, i, j, k, c)];
  });
  return 0;
}

int orc_prolong_increment(const mlgpu_grid *g, const mlgpu_bc *bc, int ncomp, int kind,
                          double *fine, const double *coarse) {
  prolong_fab(*g, *bc, ncomp, kind, fine, coarse);
  return 0;
}

int orc_coarsen_faces(const mlgpu_grid *g, int ncomp, int dir, double *cf,
                      const double *ff) {
  coarsen_faces(*g, ncomp, dir, cf, ff);
  return 0;
}

// CELLTOEDGEGEOMETRIC (src/CellToEdge2F.ChF): edge = sqrt(|c(i-1) c(i)|);
// cell ghosts: periodic wrap, else zero-gradient copy.
int orc_face_geomean(const mlgpu_grid *g, const double *cell, double *faces[3]) {
  Fab c(*g, 1);
  c.load(cell);
  mlgpu_bc bc;
  memset(&bc, 0, sizeof(bc));
  fill_ghosts(c, *g, bc, true);
  for (int d = 0; d < g->dim; d++) {
    int m[3];
    for (int e = 0; e < 3; e++) m[e] = g->n[e] + (e == d);
    for (int k = 0; k < m[2]; k++)
      for (int j = 0; j < m[1]; j++)
        for (int i = 0; i < m[0]; i++) {
          int ii = i - (d == 0), jj = j - (d == 1), kk = k - (d == 2);
          faces[d][fidx(*g, d, i, j, k, 0)] =
              std::sqrt(std::fabs(c(ii, jj, kk, 0) * c(i, j, k, 0)));
        }
  }
  return 0;
}

int orc_vc_residual(const mlgpu_vcop *op, double *res, const double *phid,
                    const double *rhs, int homogeneous) {
  Fab phi(op->grid, 1);
  phi.load(phid);
  fill_ghosts(phi, op->grid, op->bc, homogeneous != 0);
  VCCtx X(*op);
  for_cells(op->grid, [&](int i, int j, int k) {
    size_t cell = cidx(op->grid, i, j, k, 0);
    res[cell] = rhs[cell] - X.lofphi(phi, i, j, k);
  });
  return 0;
}

int orc_vc_apply(const mlgpu_vcop *op, double *lhs, const double *phid, int homogeneous) {
  Fab phi(op->grid, 1);
  phi.load(phid);
  fill_ghosts(phi, op->grid, op->bc, homogeneous != 0);
  VCCtx X(*op);
  for_cells(op->grid, [&](int i, int j, int k) {
    lhs[cidx(op->grid, i, j, k, 0)] = X.lofphi(phi, i, j, k);
  });
  return 0;
}

int orc_vc_gsrb_pass(const mlgpu_vcop *op, double *phid, const double *rhs, int pass) {
  Fab phi(op->grid, 1);
  phi.load(phid);
  vc_gsrb_pass_fab(phi, rhs, *op, pass);
  phi.store(phid);
  return 0;
}

int orc_vc_relax(const mlgpu_vcop *op, double *phid, const double *rhs, int n) {
  Fab phi(op->grid, 1);
  phi.load(phid);
  for (int s = 0; s < n; s++) {
    vc_gsrb_pass_fab(phi, rhs, *op, 0);
    vc_gsrb_pass_fab(phi, rhs, *op, 1);
  }
  phi.store(phid);
  return 0;
}

int orc_vc_lambda(const mlgpu_vcop *op, double *lam) {
  VCCtx X(*op);
  for_cells(op->grid, [&](int i, int j, int k) {
    size_t cell = cidx(op->grid, i, j, k, 0);
    lam[cell] = lambda_at(X.B, X.a, X.cc, op->alpha, op->beta, X.scale, cell, i, j, k, 0,
                          op->grid.dim);
  });
  return 0;
}

// DarcyBrinkmanOp::levelJacobi (DarcyBrinkmanOp.cpp:699-720): homogeneous residual
int orc_vc_jacobi(const mlgpu_vcop *op, double *phid, const double *rhs) {
  size_t n = ncells(op->grid);
  std::vector<double> r(n), lam(n);
  orc_vc_residual(op, r.data(), phid, rhs, 1);
  orc_vc_lambda(op, lam.data());
  for (size_t q = 0; q < n; q++) phid[q] = phid[q] + 0.5 * (r[q] * lam[q]);
  return 0;
}

int orc_vc_restrict_residual(const mlgpu_vcop *op, double *resc, const double *phid,
                             const double *rhs) {
  Fab phi(op->grid, 1);
  phi.load(phid);
  fill_ghosts(phi, op->grid, op->bc, true);
  VCCtx X(*op);
  restrict_loop(op->grid, 1, resc, [&](int i, int j, int k, int) {
    return rhs[cidx(op->grid, i, j, k, 0)] - X.lofphi(phi, i, j, k);
  });
  return 0;
}

// DIVERGENCE (util/DivergenceF.ChF): div += (u(i+e_d) - u(i)) / dx per dir
int orc_mac_divergence(const mlgpu_grid *g, double *div, const double *u[3]) {
  double one_on_dx = 1.0 / g->dx;
  for_cells(*g, [&](int i, int j, int k) {
    double v = 0.0;
    for (int d = 0; d < g->dim; d++) {
      int ip = i + (d == 0), jp = j + (d == 1), kp = k + (d == 2);
      v = v + one_on_dx * (u[d][fidx(*g, d, ip, jp, kp, 0)] - u[d][fidx(*g, d, i, j, k, 0)]);
    }
    div[cidx(*g, i, j, k, 0)] = v;
  });
  return 0;
}

// levelGradientMAC + correction loop (srcSubcycle/Projector.cpp:942-968):
// grad = (phi(i) - phi(i-e_d)) / dx on faces, u -= scale * grad
int orc_mac_correct(const mlgpu_grid *g, const mlgpu_bc *bc, const double *phid,
                    const double *scale[3], double *u[3]) {
  Fab phi(*g, 1);
  phi.load(phid);
  fill_ghosts(phi, *g, *bc, false);
  for (int d = 0; d < g->dim; d++) {
    int m[3];
    for (int e = 0; e < 3; e++) m[e] = g->n[e] + (e == d);
    for (int k = 0; k < m[2]; k++)
      for (int j = 0; j < m[1]; j++)
        for (int i = 0; i < m[0]; i++) {
          int ii = i - (d == 0), jj = j - (d == 1), kk = k - (d == 2);
          size_t f = fidx(*g, d, i, j, k, 0);
          double grad = (phi(i, j, k, 0) - phi(ii, jj, kk, 0)) / g->dx;
          if (scale && scale[d]) grad = grad * scale[d][f];
          u[d][f] = u[d][f] - grad;
        }
  }
  return 0;
}

double orc_norm(size_t n, const double *x, int type) { return norm_of(x, n, type); }

}  // extern "C"

// ========================================================== solver drivers
namespace {

struct Level {
  mlgpu_grid g;
  std::vector<double> a, c, b[3];
  std::vector<double> u, f, r, e, uold;  // scratch
};

int mg_depth(const mlgpu_grid &g, int max_coarse) {
  // MGnewOp returns nullptr when !coarsenable(2^depth * s_maxCoarse)
  int depth = 0;
  while (true) {
    long c = (long)(1L << (depth + 1)) * max_coarse;
    bool ok = true;
    for (int d = 0; d < g.dim; d++)
      if (g.n[d] % c != 0) ok = false;
    if (!ok) break;
    depth++;
  }
  return depth;  // number of coarser levels
}

void build_levels(std::vector<Level> &L, const mlgpu_grid &g0, int ncomp, const double *a0,
                  const double *c0, const void *const b0[3], int max_coarse) {
  int depth = mg_depth(g0, max_coarse);
  L.resize(depth + 1);
  L[0].g = g0;
  size_t n0 = ncells(g0) * ncomp;
  if (a0) L[0].a.assign(a0, a0 + n0);
  if (c0) L[0].c.assign(c0, c0 + n0);
  for (int d = 0; d < g0.dim; d++) {
    const double *bb = (const double *)b0[d];
    L[0].b[d].assign(bb, bb + nfaces(g0, d) * ncomp);
  }
  for (int l = 1; l <= depth; l++) {
    L[l].g = coarsen_grid(L[l - 1].g);
    size_t nc = ncells(L[l].g) * ncomp;
    if (a0) {
      L[l].a.assign(nc, 0);
      orc_restrict_average(&L[l - 1].g, ncomp, L[l].a.data(), L[l - 1].a.data());
    }
    if (c0) {
      L[l].c.assign(nc, 0);
      orc_restrict_average(&L[l - 1].g, ncomp, L[l].c.data(), L[l - 1].c.data());
    }
    for (int d = 0; d < g0.dim; d++) {
      L[l].b[d].assign(nfaces(L[l].g, d) * ncomp, 0);
      coarsen_faces(L[l - 1].g, ncomp, d, L[l].b[d].data(), L[l - 1].b[d].data());
    }
  }
  for (auto &lv : L) {
    size_t n = ncells(lv.g) * ncomp;
    lv.u.assign(n, 0);
    lv.f.assign(n, 0);
    lv.r.assign(n, 0);
    lv.e.assign(n, 0);
    lv.uold.assign(n, 0);
  }
}

void vec_axpy(std::vector<double> &y, double a, const std::vector<double> &x) {
  for (size_t q = 0; q < y.size(); q++) y[q] = y[q] + a * x[q];
}

// ---- nonlinear FAS
struct HCSolver {
  mlgpu_nlop op0;
  mlgpu_mg_options o;
  std::vector<Level> L;
  double updates = 0;

  mlgpu_nlop op_at(int l) {
    mlgpu_nlop op = op0;
    op.grid = L[l].g;
    op.aCoef = L[l].a.empty() ? nullptr : L[l].a.data();
    for (int d = 0; d < 3; d++) op.bCoef[d] = d < op.grid.dim ? L[l].b[d].data() : nullptr;
    return op;
  }
  size_t cells(int l) { return ncells(L[l].g); }

  void relax(int l, double *u, const double *f, int n) {
    mlgpu_nlop op = op_at(l);
    for (int s = 0; s < n; s++) {
      if (o.relax_mode == MLGPU_RELAX_JACOBI)
        orc_nl_jacobi(&op, u, f);
      else {
        orc_nl_gsrb_pass(&op, u, f, 0);
        orc_nl_gsrb_pass(&op, u, f, 1);
      }
      updates += cells(l);
    }
  }

  // FAS V-cycle on level l (restated AMRFASMultiGrid cycle)
  void cycle(int l, double *u, const double *f) {
    int last = (int)L.size() - 1;
    if (l == last) {
      relax(l, u, f, o.bottom_max_iter);
      return;
    }
    relax(l, u, f, o.num_smooth_down);
    mlgpu_nlop op = op_at(l), opc = op_at(l + 1);
    Level &C = L[l + 1];
    orc_restrict_average(&L[l].g, 2, C.u.data(), u);          // restrictR
    orc_nl_restrict_residual(&op, C.r.data(), u, f);           // restrictResidual
    updates += cells(l);
    orc_nl_apply(&opc, C.f.data(), C.u.data());                // N_c(R u)
    updates += cells(l + 1);
    for (size_t q = 0; q < C.f.size(); q++) C.f[q] = C.f[q] + C.r[q];
    C.uold = C.u;
    for (int m = 0; m < o.num_mg; m++) cycle(l + 1, C.u.data(), C.f.data());
    for (size_t q = 0; q < C.e.size(); q++) C.e[q] = C.u[q] - C.uold[q];
    orc_prolong_increment(&L[l].g, &op0.phi_bc, 2, o.prolong, u, C.e.data());
    relax(l, u, f, o.num_smooth_up);
  }
};

// BiCGStab bottom-solver settings (relative tolerance, restart threshold,
// restarts); the device kernel uses the same ones
constexpr double kBiCGEps = 1e-6, kBiCGHang = 1e-8;
constexpr int kBiCGRestarts = 5;

struct VCSolver {
  mlgpu_vcop op0;
  mlgpu_mg_options o;
  std::vector<Level> L;
  double updates = 0;
  mlgpu_vcop op_at(int l) {
    mlgpu_vcop op = op0;
    op.grid = L[l].g;
    op.aCoef = L[l].a.empty() ? nullptr : L[l].a.data();
    op.cCoef = L[l].c.empty() ? nullptr : L[l].c.data();
    for (int d = 0; d < 3; d++) op.bCoef[d] = d < op.grid.dim ? L[l].b[d].data() : nullptr;
    return op;
  }
  size_t cells(int l) { return ncells(L[l].g); }
  void relax(int l, double *e, const double *r, int n) {
    mlgpu_vcop op = op_at(l);
    for (int s = 0; s < n; s++) {
      if (o.relax_mode == MLGPU_RELAX_JACOBI)
        orc_vc_jacobi(&op, e, r);
      else {
        orc_vc_gsrb_pass(&op, e, r, 0);
        orc_vc_gsrb_pass(&op, e, r, 1);
      }
      updates += cells(l);
    }
  }
  // Dot product in the device's fixed order: 32 lane sums (lane l takes the
  // cells q = l mod 32 in increasing q), then a halving tree over the lanes.
  static double lane_dot(const std::vector<double> &a, const std::vector<double> &b) {
    double part[32] = {0.0};
    for (size_t q = 0; q < a.size(); q++) part[q & 31] = part[q & 31] + a[q] * b[q];
    for (int w = 16; w > 0; w >>= 1)
      for (int l = 0; l < w; l++) part[l] = part[l] + part[l + w];
    return part[0];
  }
  // the operator's preconditioner (DarcyBrinkmanOp::preCond,
  // src/DarcyBrinkmanOp.cpp:89-121): x = lambda y, then two red/black sweeps
  // of L x = y, homogeneous walls
  void precond(const mlgpu_vcop &op, const std::vector<double> &lam, const std::vector<double> &y,
               std::vector<double> &x) {
    for (size_t q = 0; q < y.size(); q++) x[q] = y[q] * lam[q];
    for (int s = 0; s < 2; s++) {
      orc_vc_gsrb_pass(&op, x.data(), y.data(), 0);
      orc_vc_gsrb_pass(&op, x.data(), y.data(), 1);
    }
  }
  // BiCGStab bottom solve of L e = r (the reference's default bottom solver
  // of the MAC projection and velocity solves, srcSubcycle/Projector.cpp:
  // 3012-3020, 2976-2986; Chombo's BiCGStabSolver, absent from the tree).
  // Restated from van der Vorst's right-preconditioned BiCGStab with the
  // operator's preCond: relative tolerance 1e-6 of the initial residual (L2
  // norm), at most bottom_max_iter iterations, a restart from the true
  // residual when an iteration gains less than 1e-8 (at most 5), and an exit
  // on breakdown (rho or <r~, v> zero).
  void bicgstab(int l, double *e, const double *rhs) {
    const mlgpu_vcop op = op_at(l);
    const size_t n = cells(l);
    std::vector<double> lam(n), r(n), rt(n), x(n, 0.0), p(n, 0.0), v(n, 0.0), ph(n), s(n),
        sh(n), t(n), tmp(n);
    orc_vc_lambda(&op, lam.data());
    auto residual = [&]() {  // r = rhs - L(e), homogeneous
      orc_vc_apply(&op, tmp.data(), e, 1);
      for (size_t q = 0; q < n; q++) r[q] = rhs[q] - tmp[q];
    };
    residual();
    rt = r;
    const double norm0 = std::sqrt(lane_dot(r, r));
    double norm = norm0, rho0 = 0.0, rho1 = 0.0, alpha = 0.0, omega = 0.0;
    bool init = true;
    int restarts = 0;
    for (int it = 0; it < o.bottom_max_iter && norm > kBiCGEps * norm0 && restarts <= kBiCGRestarts;
         it++) {
      rho1 = rho0;
      rho0 = lane_dot(rt, r);
      if (rho0 == 0.0) break;
      if (init) {
        p = r;
        init = false;
      } else {
        const double beta = (rho0 / rho1) * (alpha / omega);
        for (size_t q = 0; q < n; q++) p[q] = r[q] + beta * (p[q] - omega * v[q]);
      }
      precond(op, lam, p, ph);
      orc_vc_apply(&op, v.data(), ph.data(), 1);
      const double m = lane_dot(rt, v);
      if (m == 0.0) break;
      alpha = rho0 / m;
      for (size_t q = 0; q < n; q++) {
        s[q] = r[q] - alpha * v[q];
        x[q] = x[q] + alpha * ph[q];
      }
      const double snorm = std::sqrt(lane_dot(s, s));
      if (snorm <= kBiCGEps * norm0) {
        norm = snorm;
        break;
      }
      precond(op, lam, s, sh);
      orc_vc_apply(&op, t.data(), sh.data(), 1);
      const double tt = lane_dot(t, t);
      omega = tt > 0.0 ? lane_dot(t, s) / tt : 0.0;
      for (size_t q = 0; q < n; q++) {
        x[q] = x[q] + omega * sh[q];
        r[q] = s[q] - omega * t[q];
      }
      const double prev = norm;
      norm = std::sqrt(lane_dot(r, r));
      if (omega == 0.0 || norm > (1.0 - kBiCGHang) * prev) {
        // restart from the true residual of e + x
        for (size_t q = 0; q < n; q++) {
          e[q] = e[q] + x[q];
          x[q] = 0.0;
        }
        residual();
        rt = r;
        norm = std::sqrt(lane_dot(r, r));
        init = true;
        restarts++;
      }
    }
    for (size_t q = 0; q < n; q++) e[q] = e[q] + x[q];
    // counted as the relaxation bottom is (bottom_max_iter updates per cell)
    updates += (double)o.bottom_max_iter * n;
  }
  // MultiGrid::cycle (homogeneous correction form)
  void cycle(int l, double *e, const double *r) {
    int last = (int)L.size() - 1;
    if (l == last) {
      if (o.bottom_solver == MLGPU_BOTTOM_BICGSTAB)
        bicgstab(l, e, r);
      else
        relax(l, e, r, o.bottom_max_iter);
      return;
    }
    relax(l, e, r, o.num_smooth_down);
    mlgpu_vcop op = op_at(l);
    Level &C = L[l + 1];
    orc_vc_restrict_residual(&op, C.r.data(), e, r);
    updates += cells(l);
    std::fill(C.e.begin(), C.e.end(), 0.0);
    for (int m = 0; m < o.num_mg; m++) cycle(l + 1, C.e.data(), C.r.data());
    orc_prolong_increment(&L[l].g, &op0.bc, 1, o.prolong, e, C.e.data());
    relax(l, e, r, o.num_smooth_up);
  }
};

// outer loop shared by both solvers (AMRMultiGrid::solveNoInit semantics)
template <class Res, class Iter>
int outer_loop(const mlgpu_mg_options &o, mlgpu_solve_stats *st, Res residual_norm,
               Iter iterate) {
  double norm0 = residual_norm();
  st->initial_norm = norm0;
  st->norm_history[0] = norm0;
  st->iterations = 0;
  st->cycles = 0;
  st->exit_status = 0;
  if (!std::isfinite(norm0)) {
    st->exit_status = 8;
    st->final_norm = norm0;
    return MLGPU_ERR_NAN;
  }
  double norm = norm0, prev = norm0;
  int iter = 0;
  while (norm > o.tolerance * norm0 && norm0 > o.norm_thresh && iter < o.max_iter) {
    iterate();
    iter++;
    norm = residual_norm();
    if (iter < 64) st->norm_history[iter] = norm;
    if (!std::isfinite(norm)) {
      st->exit_status = 8;
      break;
    }
    if (norm > (1.0 - o.hang) * prev && norm > o.tolerance * norm0) {
      st->exit_status = 2;
      break;
    }
    prev = norm;
  }
  st->iterations = iter;
  st->final_norm = norm;
  if (st->exit_status == 0 && norm > o.tolerance * norm0 && norm0 > o.norm_thresh)
    st->exit_status = 4;
  if (st->exit_status == 8) return MLGPU_ERR_NAN;
  if (st->exit_status == 2) return MLGPU_ERR_HANG;
  if (st->exit_status == 4) return MLGPU_ERR_NOT_CONVERGED;
  return MLGPU_OK;
}

}  // namespace

extern "C" {

void orc_mg_default_options(mlgpu_mg_options *o, int hc) {
  memset(o, 0, sizeof(*o));
  // HCMultigrid defaults (srcSubcycle/MushyLayerSubcycleUtils.cpp:668-678)
  // or projection defaults (srcSubcycle/Projector.cpp:44-64)
  o->num_smooth_down = hc ? 1 : 2;
  o->num_smooth_up = 4;
  o->num_mg = 1;
  o->max_iter = hc ? 10 : 20;
  o->tolerance = hc ? 1e-10 : 1e-15;
  o->hang = hc ? 1e-10 : 1e-15;
  o->norm_thresh = hc ? 1e-10 : 1e-30;
  o->relax_mode = MLGPU_RELAX_GSRB;
  o->bottom_solver = MLGPU_BOTTOM_RELAX;
  o->bottom_max_iter = hc ? 40 : 20;
  o->max_coarse = 2;
  o->prolong = hc ? MLGPU_PROLONG_LINEAR : MLGPU_PROLONG_CONSTANT;
  o->precision = MLGPU_PREC_F64;
  o->inner_cycles = 0;
  o->norm_type = MLGPU_NORM_MAX;
  o->use_graph = 0;
  o->fuse_levels = 1;
}

int orc_mg_depth(const mlgpu_grid *g, int max_coarse) { return mg_depth(*g, max_coarse); }

double orc_pd_temperature(double H, double C, const mlgpu_params *p) {
  return pd_temperature(H, C, *p);
}

int orc_hc_solve(const mlgpu_nlop *op, const mlgpu_mg_options *o, double *phi,
                 const double *rhs, mlgpu_solve_stats *st) {
  HCSolver S;
  S.op0 = *op;
  // the temperature condition object keeps the level's spacing on the
  // coarser multigrid levels (PhysBCUtil m_dx)
  if (!(S.op0.nlbc.dx > 0)) S.op0.nlbc.dx = op->grid.dx;
  S.o = *o;
  build_levels(S.L, op->grid, 2, (const double *)op->aCoef, nullptr, op->bCoef,
               o->max_coarse);
  memset(st, 0, sizeof(*st));
  st->levels = (int)S.L.size();
  size_t n = 2 * ncells(op->grid);
  std::vector<double> r(n);
  auto resnorm = [&]() {
    orc_nl_residual(op, r.data(), phi, rhs);
    S.updates += ncells(op->grid);
    return norm_of(r.data(), n, o->norm_type);
  };
  int cycles = 0;
  auto iterate = [&]() {
    S.cycle(0, phi, rhs);
    cycles++;
  };
  int rc = outer_loop(*o, st, resnorm, iterate);
  st->cycles = cycles;
  st->cell_updates = S.updates;
  return rc;
}

int orc_vc_solve(const mlgpu_vcop *op, const mlgpu_mg_options *o, double *phi,
                 const double *rhs, mlgpu_solve_stats *st);

// Projector::levelMacProject (srcSubcycle/Projector.cpp:858-982):
// div -> solve div(Pi grad phi) = div u -> u -= Pi grad phi
int orc_mac_project(const mlgpu_vcop *op, const mlgpu_mg_options *o, const mlgpu_bc *phi_bc,
                    double *u[3], const double *pi[3], double *phi, mlgpu_solve_stats *st) {
  std::vector<double> rhs(ncells(op->grid));
  const double *uc[3] = {u[0], u[1], u[2]};
  orc_mac_divergence(&op->grid, rhs.data(), uc);
  int rc = orc_vc_solve(op, o, phi, rhs.data(), st);
  orc_mac_correct(&op->grid, phi_bc, phi, pi, u);
  return rc;
}

// LevelBackwardEuler::updateSoln: rhs = phi_old * a + dt * src, alpha = 1,
// beta = -dt, FAS solve for phi_new
int orc_hc_solve(const mlgpu_nlop *op, const mlgpu_mg_options *o, double *phi,
                 const double *rhs, mlgpu_solve_stats *st);
int orc_hc_backward_euler(const mlgpu_nlop *op, const mlgpu_mg_options *o, double *phi_new,
                          const double *phi_old, const double *src, const double *a, double dt,
                          mlgpu_solve_stats *st) {
  size_t n = 2 * ncells(op->grid);
  std::vector<double> rhs(n);
  for (size_t q = 0; q < n; q++) {
    double v = a ? phi_old[q] * a[q] : phi_old[q];
    if (src) v = v + dt * src[q];
    rhs[q] = v;
  }
  mlgpu_nlop be = *op;
  be.alpha = 1.0;
  be.beta = -dt;
  return orc_hc_solve(&be, o, phi_new, rhs.data(), st);
}

// mlgpu_hc_tga_step restated (the TGA scheme of Twizell, Gumel & Arigu
// 1996 as Chombo's LevelTGA drives it; Chombo is not in the reference tree):
// R = (a + mu3 dt L) phi_old + dt src by the operator with alpha 1, beta
// mu3 dt; (a - mu1 dt L) psi = R from psi = phi_old; (a - mu2 dt L) phi_new
// = a psi from phi_new = psi.  st: the second solve's, with the iterations,
// cycles and cell updates of both
int orc_hc_newton_solve(const mlgpu_nlop *op, const mlgpu_mg_options *o, double *phi,
                        const double *rhs, mlgpu_solve_stats *st);
}  // extern "C"

template <class Solve>
static int tga_step(const mlgpu_nlop *op, Solve solve, double *phi_new, const double *phi_old,
                    const double *src, const double *a, double dt, mlgpu_solve_stats *st) {
  const double at = 2.0 - std::sqrt(2.0) - 1e-12;
  const double d = std::sqrt(at * at - 4.0 * at + 2.0);
  const double mu1 = 0.5 * (at - d), mu2 = 0.5 * (at + d), mu3 = 1.0 - at;
  const size_t n = 2 * ncells(op->grid);
  std::vector<double> R(n), psi(phi_old, phi_old + n);
  mlgpu_nlop opR = *op;
  opR.alpha = 1.0;
  opR.beta = mu3 * dt;
  orc_nl_apply(&opR, R.data(), phi_old);
  if (src)
    for (size_t q = 0; q < n; q++) R[q] = R[q] + dt * src[q];
  mlgpu_nlop s1 = *op;
  s1.alpha = 1.0;
  s1.beta = -mu1 * dt;
  mlgpu_solve_stats st1;
  const int rc1 = solve(&s1, psi.data(), R.data(), &st1);
  if (rc1 != MLGPU_OK && rc1 != MLGPU_ERR_NOT_CONVERGED && rc1 != MLGPU_ERR_HANG) return rc1;
  for (size_t q = 0; q < n; q++) {
    R[q] = a ? psi[q] * a[q] : psi[q];
    phi_new[q] = psi[q];
  }
  mlgpu_nlop s2 = *op;
  s2.alpha = 1.0;
  s2.beta = -mu2 * dt;
  const int rc2 = solve(&s2, phi_new, R.data(), st);
  st->iterations += st1.iterations;
  st->cycles += st1.cycles;
  st->cell_updates += st1.cell_updates;
  return rc2 == MLGPU_OK ? rc1 : rc2;
}

extern "C" {

int orc_hc_tga_step(const mlgpu_nlop *op, const mlgpu_mg_options *o, double *phi_new,
                    const double *phi_old, const double *src, const double *a, double dt,
                    mlgpu_solve_stats *st) {
  return tga_step(
      op,
      [o](const mlgpu_nlop *x, double *u, const double *r, mlgpu_solve_stats *s) {
        return orc_hc_solve(x, o, u, r, s);
      },
      phi_new, phi_old, src, a, dt, st);
}

// the same step with Newton solves (orc_hc_newton_solve)
int orc_hc_tga_step_newton(const mlgpu_nlop *op, const mlgpu_mg_options *o, double *phi_new,
                           const double *phi_old, const double *src, const double *a,
                           double dt, mlgpu_solve_stats *st) {
  return tga_step(
      op,
      [o](const mlgpu_nlop *x, double *u, const double *r, mlgpu_solve_stats *s) {
        return orc_hc_newton_solve(x, o, u, r, s);
      },
      phi_new, phi_old, src, a, dt, st);
}

int orc_vc_solve(const mlgpu_vcop *op, const mlgpu_mg_options *o, double *phi,
                 const double *rhs, mlgpu_solve_stats *st) {
  VCSolver S;
  S.op0 = *op;
  S.o = *o;
  build_levels(S.L, op->grid, 1, (const double *)op->aCoef, (const double *)op->cCoef,
               op->bCoef, o->max_coarse);
  memset(st, 0, sizeof(*st));
  st->levels = (int)S.L.size();
  size_t n = ncells(op->grid);
  std::vector<double> r(n), e(n);
  auto resnorm = [&]() {
    orc_vc_residual(op, r.data(), phi, rhs, 0);
    S.updates += n;
    return norm_of(r.data(), n, o->norm_type);
  };
  int cycles = 0;
  auto iterate = [&]() {
    std::fill(e.begin(), e.end(), 0.0);
    for (int m = 0; m < std::max(1, o->inner_cycles); m++) {
      S.cycle(0, e.data(), r.data());
      cycles++;
    }
    for (size_t q = 0; q < n; q++) phi[q] = phi[q] + e[q];
  };
  int rc = outer_loop(*o, st, resnorm, iterate);
  st->cycles = cycles;
  st->cell_updates = S.updates;
  return rc;
}

}  // extern "C"

// ================================================================ adjoint
// Discrete adjoint of the nonlinear operator (no counterpart in the
// reference).  With f = (T, C_l) of (H, C) and J = df/d(H, C) (t_cl_jac), the
// Jacobian of N(phi) = alpha a phi - beta dxinv sum_f b_f (f_nb - f) is
//   A x = alpha a x - beta dxinv sum_f b_f (J_nb x_nb - J x)
// with the wall ghost of J x from the condition N uses: the derived
// condition's homogeneous rule on J x, or J_g S x with J_g the Jacobian at the
// (H, C)-condition ghost state and S its homogeneous signs.  Its transpose,
// per cell, is alpha a y - beta dxinv (J^T w + e) with
//   w = sum_f b_f (y_g - y),  y_g = neighbour, derived-rule ghost of y, or 0
//   e = sum over (H, C)-condition faces of S J_g^T (b_f y).
// The functions below restate that, and A itself, on ghosted FABs.
namespace {

struct AdjCtx {
  const mlgpu_nlop &op;
  Faces B;
  const double *a, *J, *u;
  double dxinv;
  size_t n;
  AdjCtx(const mlgpu_nlop &o, const double *phi, const double *Jd) : op(o), J(Jd), u(phi) {
    B = make_faces(o.grid, o.bCoef);
    a = (const double *)o.aCoef;
    dxinv = 1.0 / (o.grid.dx * o.grid.dx);
    n = ncells(o.grid);
  }
  double jac(size_t q, int m) const { return J[m * n + q]; }
};

// ghosts of the adjoint variable: periodic copies; the derived condition's
// homogeneous rule when N applies it; zero under the (H, C) condition
void adj_fill(Fab &y, const mlgpu_nlop &op) {
  exchange(y, op.grid);
  if (op.apply_derived_bc) {
    physbc(y, op.grid, op.derived_bc, true, &op.nlbc);
    return;
  }
  for (int d = 0; d < op.grid.dim; d++) {
    if (op.grid.periodic[d]) continue;
    for (int side = 0; side < 2; side++) {
      int lo[3] = {0, 0, 0}, hi[3] = {y.n[0] - 1, y.n[1] - 1, y.n[2] - 1};
      lo[d] = hi[d] = side == 0 ? -1 : y.n[d];
      for (int c = 0; c < 2; c++)
        for (int k = lo[2]; k <= hi[2]; k++)
          for (int j = lo[1]; j <= hi[1]; j++)
            for (int i = lo[0]; i <= hi[0]; i++) y(i, j, k, c) = 0.0;
    }
  }
}

// Jacobian at the (H, C)-condition ghost state across (d, side) of cell q
void ghost_jac(const AdjCtx &X, size_t q, int d, int side, double Jg[4]) {
  const mlgpu_bc &bc = X.op.phi_bc;
  double st[2];
  for (int c = 0; c < 2; c++) {
    double interior = X.u[c * X.n + q];
    double val = bc.value[d][side][c];
    if (bc.type[d][side][c] == MLGPU_BC_DIRICHLET)
      st[c] = 2 * val - interior;
    else
      st[c] = interior + ((side == 0 ? -1 : 1) * X.op.grid.dx) * val;
  }
  t_cl_jac(st[0], st[1], X.op.params, Jg);
}

// (A^T y) of cell (i,j,k); M = its 2x2 diagonal block (row-major) if asked
void adj_row(const AdjCtx &X, const Fab &y, int i, int j, int k, double out[2], double *M) {
  const mlgpu_grid &g = X.op.grid;
  const size_t q = cidx(g, i, j, k, 0);
  const double y0[2] = {y(i, j, k, 0), y(i, j, k, 1)};
  double w[2], P[2], ex[2] = {0.0, 0.0}, Xm[4] = {0.0, 0.0, 0.0, 0.0};
  bool any_phi = false;
  const int at[3] = {i, j, k};
  for (int c = 0; c < 2; c++) {
    // w_c = sum over faces of (b_nb y_nb - b y0): the neighbour's row reads
    // its own face coefficient, which differs from this cell's only across a
    // periodic seam (face n for cell n-1, face 0 for cell 0)
    double s = 0.0;
    for (int d = 0; d < g.dim; d++)
      for (int side = 1; side >= 0; side--) {
        int fi[3] = {i, j, k}, nbc[3] = {i, j, k};
        if (side) fi[d] += 1;
        nbc[d] += side ? 1 : -1;
        double bf = X.B(d, fi[0], fi[1], fi[2], c);
        double yn = y(nbc[0], nbc[1], nbc[2], c);
        double t;
        bool seam = g.periodic[d] && (nbc[d] < 0 || nbc[d] >= g.n[d]);
        if (seam && g.n[d] == 1) {
          t = 0.0;
        } else if (seam) {
          int fs[3] = {i, j, k};
          fs[d] = side ? 0 : g.n[d];
          double bn = X.B(d, fs[0], fs[1], fs[2], c);
          t = side ? bn * yn - bf * y0[c] : bf * y0[c] - bn * yn;
        } else {
          t = side ? bf * (yn - y0[c]) : bf * (y0[c] - yn);
        }
        if (side)
          s = d == 0 ? t : s + t;
        else
          s = s - t;
      }
    w[c] = s;
    // d w_c / d y_c = -P_c
    double p = 0.0;
    for (int d = 0; d < g.dim; d++)
      for (int side = 1; side >= 0; side--) {
        int fi[3] = {i, j, k};
        if (side) fi[d] += 1;
        double bf = X.B(d, fi[0], fi[1], fi[2], c);
        int nb = at[d] + (side ? 1 : -1);
        double dp;
        if (nb >= 0 && nb < g.n[d])
          dp = bf;
        else if (g.periodic[d])
          dp = g.n[d] == 1 ? 0.0 : bf;
        else if (X.op.apply_derived_bc)
          dp = dbc_wall_diag(X.op, d, side, c, bf);
        else {
          dp = bf;
          any_phi = true;
        }
        p = p + dp;
      }
    P[c] = p;
  }
  if (any_phi) {
    for (int d = 0; d < g.dim; d++) {
      if (g.periodic[d]) continue;
      for (int side = 0; side < 2; side++) {
        if (side ? at[d] != g.n[d] - 1 : at[d] != 0) continue;
        int fi[3] = {i, j, k};
        if (side) fi[d] += 1;
        const double b0 = X.B(d, fi[0], fi[1], fi[2], 0), b1 = X.B(d, fi[0], fi[1], fi[2], 1);
        double Jg[4];
        ghost_jac(X, q, d, side, Jg);
        for (int c = 0; c < 2; c++) {
          double sc = X.op.phi_bc.type[d][side][c] == MLGPU_BC_DIRICHLET ? -1.0 : 1.0;
          double g0 = Jg[c], g1 = Jg[2 + c];
          ex[c] = ex[c] + sc * (g0 * (b0 * y0[0]) + g1 * (b1 * y0[1]));
          Xm[2 * c + 0] = Xm[2 * c + 0] + sc * (g0 * b0);
          Xm[2 * c + 1] = Xm[2 * c + 1] + sc * (g1 * b1);
        }
      }
    }
  }
  for (int c = 0; c < 2; c++) {
    double t = X.jac(q, c) * w[0] + X.jac(q, 2 + c) * w[1];
    if (any_phi) t = t + ex[c];
    double av = X.a ? X.a[q + c * X.n] : 1.0;
    out[c] = X.op.alpha * av * y0[c] - X.op.beta * t * X.dxinv;
    if (M)
      for (int cp = 0; cp < 2; cp++) {
        double v = X.op.beta * X.dxinv * (X.jac(q, 2 * cp + c) * P[cp] - Xm[2 * c + cp]);
        if (cp == c) v = X.op.alpha * av + v;
        M[2 * c + cp] = v;
      }
  }
}

void adj_load(Fab &y, const mlgpu_nlop &op, const double *yd) {
  y.define(op.grid, 2);
  y.load(yd);
  adj_fill(y, op);
}

// inverse of every cell's diagonal block M of A^T, {M3, -M1, -M2, M0}/det
// (the driver's smoother stores it once per state)
void adj_minv(const AdjCtx &X, double *Minv) {
  const mlgpu_grid &gr = X.op.grid;
  Fab z;
  std::vector<double> zero(2 * X.n, 0.0);
  adj_load(z, X.op, zero.data());
  for (int k = 0; k < gr.n[2]; k++)
    for (int j = 0; j < gr.n[1]; j++)
      for (int i = 0; i < gr.n[0]; i++) {
        double out[2], M[4];
        adj_row(X, z, i, j, k, out, M);
        size_t q = cidx(gr, i, j, k, 0);
        double det = M[0] * M[3] - M[1] * M[2];
        Minv[q] = M[3] / det;
        Minv[q + X.n] = -M[1] / det;
        Minv[q + 2 * X.n] = -M[2] / det;
        Minv[q + 3 * X.n] = M[0] / det;
      }
}

// one red/black pass of the block smoother: each cell of the colour solves
// its two rows exactly, y += M^-1 (g - A^T y); with Minv given the stored
// inverse is applied, else M is formed and inverted inline
void adj_gsrb_pass_fab(Fab &y, const AdjCtx &X, const double *g, int pass,
                       const double *Minv = nullptr) {
  const mlgpu_grid &gr = X.op.grid;
  adj_fill(y, X.op);
  for (int k = 0; k < gr.n[2]; k++)
    for (int j = 0; j < gr.n[1]; j++) {
      int imin = std::abs((j + k + pass) % 2);
      for (int i = imin; i < gr.n[0]; i += 2) {
        size_t q = cidx(gr, i, j, k, 0);
        double y0 = y(i, j, k, 0), y1 = y(i, j, k, 1);
        if (Minv) {
          double out[2];
          adj_row(X, y, i, j, k, out, nullptr);
          double r0 = g[q] - out[0], r1 = g[q + X.n] - out[1];
          double m0 = Minv[q], m1 = Minv[q + X.n], m2 = Minv[q + 2 * X.n], m3 = Minv[q + 3 * X.n];
          y(i, j, k, 0) = y0 + (m0 * r0 + m1 * r1);
          y(i, j, k, 1) = y1 + (m2 * r0 + m3 * r1);
          continue;
        }
        double out[2], M[4];
        adj_row(X, y, i, j, k, out, M);
        double r0 = g[q] - out[0], r1 = g[q + X.n] - out[1];
        double det = M[0] * M[3] - M[1] * M[2];
        y(i, j, k, 0) = y0 + (M[3] * r0 - M[1] * r1) / det;
        y(i, j, k, 1) = y1 + (M[0] * r1 - M[2] * r0) / det;
      }
    }
}

// A x (the linearised operator) on ghosted FABs of J x
void lin_apply(const AdjCtx &X, const double *xd, double *out) {
  const mlgpu_nlop &op = X.op;
  const mlgpu_grid &g = op.grid;
  Fab x(g, 2), jx(g, 2);
  x.load(xd);
  for (int k = 0; k < g.n[2]; k++)
    for (int j = 0; j < g.n[1]; j++)
      for (int i = 0; i < g.n[0]; i++) {
        size_t q = cidx(g, i, j, k, 0);
        double x0 = x(i, j, k, 0), x1 = x(i, j, k, 1);
        jx(i, j, k, 0) = X.jac(q, 0) * x0 + X.jac(q, 1) * x1;
        jx(i, j, k, 1) = X.jac(q, 2) * x0 + X.jac(q, 3) * x1;
      }
  exchange(jx, g);
  if (op.apply_derived_bc) {
    physbc(jx, g, op.derived_bc, true, &op.nlbc);
  } else {
    for (int d = 0; d < g.dim; d++) {
      if (g.periodic[d]) continue;
      for (int side = 0; side < 2; side++) {
        int lo[3] = {0, 0, 0}, hi[3] = {g.n[0] - 1, g.n[1] - 1, g.n[2] - 1};
        lo[d] = hi[d] = side == 0 ? 0 : g.n[d] - 1;
        for (int k = lo[2]; k <= hi[2]; k++)
          for (int j = lo[1]; j <= hi[1]; j++)
            for (int i = lo[0]; i <= hi[0]; i++) {
              size_t q = cidx(g, i, j, k, 0);
              double Jg[4];
              ghost_jac(X, q, d, side, Jg);
              double s0 = op.phi_bc.type[d][side][0] == MLGPU_BC_DIRICHLET ? -1.0 : 1.0;
              double s1 = op.phi_bc.type[d][side][1] == MLGPU_BC_DIRICHLET ? -1.0 : 1.0;
              double e0 = s0 * x(i, j, k, 0), e1 = s1 * x(i, j, k, 1);
              int t[3] = {i, j, k};
              t[d] += side == 0 ? -1 : 1;
              jx(t[0], t[1], t[2], 0) = Jg[0] * e0 + Jg[1] * e1;
              jx(t[0], t[1], t[2], 1) = Jg[2] * e0 + Jg[3] * e1;
            }
      }
    }
  }
  for (int c = 0; c < 2; c++)
    for (int k = 0; k < g.n[2]; k++)
      for (int j = 0; j < g.n[1]; j++)
        for (int i = 0; i < g.n[0]; i++) {
          size_t q = cidx(g, i, j, k, c);
          double av = X.a ? X.a[q] : 1.0;
          out[q] = op.alpha * av * x(i, j, k, c) -
                   op.beta * flux_sum(X.B, jx, i, j, k, c, g.dim) * X.dxinv;
        }
}

// one red/black pass of the block smoother on A x = r (the Newton step's
// linear solve): out and the diagonal block D of each colour cell from J x
// with its ghosts, x += D^-1 (r - A x)
// With Minv (the stored inverse of A^T's diagonal blocks) its transpose is
// applied instead of forming D.
void lin_gsrb_pass(const AdjCtx &X, double *xd, const double *r, int pass,
                   const double *Minv = nullptr) {
  const mlgpu_nlop &op = X.op;
  const mlgpu_grid &g = op.grid;
  std::vector<double> out(2 * X.n);
  lin_apply(X, xd, out.data());
  for (int k = 0; k < g.n[2]; k++)
    for (int j = 0; j < g.n[1]; j++) {
      int imin = std::abs((j + k + pass) % 2);
      for (int i = imin; i < g.n[0]; i += 2) {
        const size_t q = cidx(g, i, j, k, 0);
        if (Minv) {
          double r0 = r[q] - out[q], r1 = r[q + X.n] - out[q + X.n];
          double m0 = Minv[q], m1 = Minv[q + X.n], m2 = Minv[q + 2 * X.n], m3 = Minv[q + 3 * X.n];
          double x0 = xd[q], x1 = xd[q + X.n];
          xd[q] = x0 + (m0 * r0 + m2 * r1);
          xd[q + X.n] = x1 + (m1 * r0 + m3 * r1);
          continue;
        }
        const int at[3] = {i, j, k};
        double P[2], Y[4] = {0.0, 0.0, 0.0, 0.0}, M[4];
        for (int c = 0; c < 2; c++) {
          double p = 0.0;
          for (int d = 0; d < g.dim; d++)
            for (int side = 1; side >= 0; side--) {
              int fi[3] = {i, j, k};
              if (side) fi[d] += 1;
              double bf = X.B(d, fi[0], fi[1], fi[2], c);
              int nb = at[d] + (side ? 1 : -1);
              double dp;
              if (nb >= 0 && nb < g.n[d])
                dp = bf;
              else if (g.periodic[d])
                dp = g.n[d] == 1 ? 0.0 : bf;
              else if (op.apply_derived_bc)
                dp = dbc_wall_diag(op, d, side, c, bf);
              else {
                double Jg[4];
                ghost_jac(X, q, d, side, Jg);
                double s0 = op.phi_bc.type[d][side][0] == MLGPU_BC_DIRICHLET ? -1.0 : 1.0;
                double s1 = op.phi_bc.type[d][side][1] == MLGPU_BC_DIRICHLET ? -1.0 : 1.0;
                dp = bf;
                Y[2 * c + 0] = Y[2 * c + 0] + bf * (Jg[2 * c] * s0);
                Y[2 * c + 1] = Y[2 * c + 1] + bf * (Jg[2 * c + 1] * s1);
              }
              p = p + dp;
            }
          P[c] = p;
          double av = X.a ? X.a[q + c * X.n] : 1.0;
          for (int cp = 0; cp < 2; cp++) {
            double v = op.beta * X.dxinv * (P[c] * X.jac(q, 2 * c + cp) - Y[2 * c + cp]);
            if (cp == c) v = op.alpha * av + v;
            M[2 * c + cp] = v;
          }
        }
        double r0 = r[q] - out[q], r1 = r[q + X.n] - out[q + X.n];
        double det = M[0] * M[3] - M[1] * M[2];
        double x0 = xd[q], x1 = xd[q + X.n];
        xd[q] = x0 + (M[3] * r0 - M[1] * r1) / det;
        xd[q + X.n] = x1 + (M[0] * r1 - M[2] * r0) / det;
      }
    }
}

// ---- multigrid for A^T y = g (the device driver restated)
struct AdjLevelO {
  mlgpu_grid g;
  std::vector<double> a, b[3], u, J, y, gg, r, Minv;
};

struct AdjSolver {
  mlgpu_nlop op0;
  mlgpu_mg_options o;
  std::vector<AdjLevelO> L;
  double updates = 0;
  bool tr = true;  // cycles on A^T (adjoint) or on A (Newton's linear solve)

  mlgpu_nlop op_at(int l) {
    mlgpu_nlop op = op0;
    op.grid = L[l].g;
    op.aCoef = L[l].a.empty() ? nullptr : L[l].a.data();
    for (int d = 0; d < 3; d++) op.bCoef[d] = d < op.grid.dim ? L[l].b[d].data() : nullptr;
    return op;
  }
  void build(const double *phi) {
    std::vector<Level> LL;
    build_levels(LL, op0.grid, 2, (const double *)op0.aCoef, nullptr, op0.bCoef, o.max_coarse);
    L.assign(LL.size(), AdjLevelO());
    for (size_t l = 0; l < LL.size(); l++) {
      L[l].g = LL[l].g;
      L[l].a = LL[l].a;
      for (int d = 0; d < 3; d++) L[l].b[d] = LL[l].b[d];
      size_t n = 2 * ncells(L[l].g);
      L[l].u.assign(n, 0);
      L[l].J.assign(2 * n, 0);
      L[l].y.assign(n, 0);
      L[l].gg.assign(n, 0);
      L[l].r.assign(n, 0);
    }
    std::copy(phi, phi + L[0].u.size(), L[0].u.begin());
    refresh();
  }
  // coarse states averaged from level 0's, J and the inverse blocks per level
  void refresh() {
    for (size_t l = 1; l < L.size(); l++)
      orc_restrict_average(&L[l - 1].g, 2, L[l].u.data(), L[l - 1].u.data());
    for (auto &lv : L) orc_closure_jac(&lv.g, &op0.params, lv.u.data(), lv.J.data());
    for (size_t l = 0; l < L.size(); l++) {
      L[l].Minv.assign(2 * L[l].u.size(), 0.0);
      mlgpu_nlop op = op_at((int)l);
      AdjCtx X(op, L[l].u.data(), L[l].J.data());
      adj_minv(X, L[l].Minv.data());
    }
  }
  void smooth(int l, int n) {
    mlgpu_nlop op = op_at(l);
    AdjCtx X(op, L[l].u.data(), L[l].J.data());
    Fab y;
    y.define(op.grid, 2);
    y.load(L[l].y.data());
    if (!tr) {
      for (int s = 0; s < n; s++) {
        lin_gsrb_pass(X, L[l].y.data(), L[l].gg.data(), 0, L[l].Minv.data());
        lin_gsrb_pass(X, L[l].y.data(), L[l].gg.data(), 1, L[l].Minv.data());
      }
      return;
    }
    for (int s = 0; s < n; s++) {
      adj_gsrb_pass_fab(y, X, L[l].gg.data(), 0, L[l].Minv.data());
      adj_gsrb_pass_fab(y, X, L[l].gg.data(), 1, L[l].Minv.data());
    }
    y.store(L[l].y.data());
  }
  // exact bottom solve (at most 32 unknowns): columns A^T e_k, Gaussian
  // elimination with partial pivoting (first largest |pivot|), back
  // substitution -- the device's operation order
  void direct(int l) {
    mlgpu_nlop op = op_at(l);
    AdjCtx X(op, L[l].u.data(), L[l].J.data());
    const size_t nc = ncells(L[l].g);
    const int n = (int)(2 * nc);
    std::vector<double> M((size_t)n * (n + 1));
    auto at = [&](int r, int c) -> double & { return M[(size_t)r * (n + 1) + c]; };
    std::vector<double> e(n, 0.0), col(n);
    for (int k = 0; k < n; k++) {
      std::fill(e.begin(), e.end(), 0.0);
      e[k] = 1.0;
      if (tr) {
        Fab y;
        adj_load(y, op, e.data());
        for (int kk = 0; kk < L[l].g.n[2]; kk++)
          for (int j = 0; j < L[l].g.n[1]; j++)
            for (int i = 0; i < L[l].g.n[0]; i++) {
              double o2[2];
              adj_row(X, y, i, j, kk, o2, nullptr);
              size_t q = cidx(L[l].g, i, j, kk, 0);
              col[q] = o2[0];
              col[q + nc] = o2[1];
            }
      } else {
        lin_apply(X, e.data(), col.data());
      }
      for (int r = 0; r < n; r++) at(r, k) = col[r];
      at(k, n) = L[l].gg[k];
    }
    for (int p = 0; p < n; p++) {
      int best = p;
      double bv = std::fabs(at(p, p));
      for (int r = p + 1; r < n; r++) {
        double v = std::fabs(at(r, p));
        if (v > bv) {
          bv = v;
          best = r;
        }
      }
      if (best != p)
        for (int c = 0; c <= n; c++) std::swap(at(p, c), at(best, c));
      for (int r = p + 1; r < n; r++) {
        double lr = at(r, p) / at(p, p);
        for (int c = p; c <= n; c++) at(r, c) = at(r, c) - lr * at(p, c);
      }
    }
    for (int r = n - 1; r >= 0; r--) {
      double s = at(r, n);
      for (int c = r + 1; c < n; c++) s = s - at(r, c) * L[l].y[c];
      L[l].y[r] = s / at(r, r);
    }
  }

  void cycle(int l) {
    const int last = (int)L.size() - 1;
    if (l > 0) std::fill(L[l].y.begin(), L[l].y.end(), 0.0);
    if (l == last) {
      if (2 * ncells(L[l].g) <= 32)
        direct(l);
      else
        smooth(l, o.bottom_max_iter);
      updates += (double)o.bottom_max_iter * ncells(L[l].g);
      return;
    }
    smooth(l, o.num_smooth_down);
    mlgpu_nlop op = op_at(l);
    if (tr)
      orc_hc_adjoint_restrict_impl(op, L[l].u.data(), L[l].J.data(), L[l].y.data(),
                                   L[l].gg.data(), L[l + 1].gg.data());
    else
      lin_restrict(op, L[l].u.data(), L[l].J.data(), L[l].y.data(), L[l].gg.data(),
                   L[l + 1].gg.data());
    for (int m = 0; m < o.num_mg; m++) cycle(l + 1);
    mlgpu_bc ybc = op0.apply_derived_bc ? op0.derived_bc : op0.phi_bc;
    orc_prolong_increment(&L[l].g, &ybc, 2, o.prolong, L[l].y.data(), L[l + 1].y.data());
    smooth(l, o.num_smooth_up);
    updates += (double)(o.num_smooth_down + o.num_smooth_up + 1) * ncells(L[l].g);
  }
  // 2^D average of g - A y (the children in the device's order)
  static void lin_restrict(const mlgpu_nlop &op, const double *phi, const double *J,
                           const double *yd, const double *g, double *gc) {
    AdjCtx X(op, phi, J);
    std::vector<double> ay(2 * X.n);
    lin_apply(X, yd, ay.data());
    mlgpu_grid cg = coarsen_grid(op.grid);
    const double denom = op.grid.dim == 3 ? 8.0 : 4.0;
    size_t nc = ncells(cg);
    for (int K = 0; K < cg.n[2]; K++)
      for (int J2 = 0; J2 < cg.n[1]; J2++)
        for (int I = 0; I < cg.n[0]; I++) {
          double acc[2] = {0.0, 0.0};
          for (int kk = 0; kk < (op.grid.dim == 3 ? 2 : 1); kk++)
            for (int jj = 0; jj < 2; jj++)
              for (int ii = 0; ii < 2; ii++) {
                int i = 2 * I + ii, j = 2 * J2 + jj, k = op.grid.dim == 3 ? 2 * K + kk : 0;
                size_t q = cidx(op.grid, i, j, k, 0);
                for (int c = 0; c < 2; c++)
                  acc[c] = acc[c] + (g[q + c * X.n] - ay[q + c * X.n]) / denom;
              }
          size_t Q = cidx(cg, I, J2, K, 0);
          gc[Q] = acc[0];
          gc[Q + nc] = acc[1];
        }
  }

  static void orc_hc_adjoint_restrict_impl(const mlgpu_nlop &op, const double *phi,
                                           const double *J, const double *yd, const double *g,
                                           double *gc) {
    AdjCtx X(op, phi, J);
    Fab y;
    adj_load(y, op, yd);
    mlgpu_grid cg = coarsen_grid(op.grid);
    const double denom = op.grid.dim == 3 ? 8.0 : 4.0;
    size_t nc = ncells(cg);
    for (int K = 0; K < cg.n[2]; K++)
      for (int J2 = 0; J2 < cg.n[1]; J2++)
        for (int I = 0; I < cg.n[0]; I++) {
          double acc[2] = {0.0, 0.0};
          for (int kk = 0; kk < (op.grid.dim == 3 ? 2 : 1); kk++)
            for (int jj = 0; jj < 2; jj++)
              for (int ii = 0; ii < 2; ii++) {
                int i = 2 * I + ii, j = 2 * J2 + jj, k = op.grid.dim == 3 ? 2 * K + kk : 0;
                double o2[2];
                adj_row(X, y, i, j, k, o2, nullptr);
                size_t q = cidx(op.grid, i, j, k, 0);
                for (int c = 0; c < 2; c++) acc[c] = acc[c] + (g[q + c * X.n] - o2[c]) / denom;
              }
          size_t Q = cidx(cg, I, J2, K, 0);
          gc[Q] = acc[0];
          gc[Q + nc] = acc[1];
        }
  }
};

}  // namespace

extern "C" {

int orc_hc_adjoint_apply(const mlgpu_nlop *op, const double *phi, const double *J,
                         const double *yd, const double *g, double *out) {
  AdjCtx X(*op, phi, J);
  Fab y;
  adj_load(y, *op, yd);
  const mlgpu_grid &gr = op->grid;
  for (int k = 0; k < gr.n[2]; k++)
    for (int j = 0; j < gr.n[1]; j++)
      for (int i = 0; i < gr.n[0]; i++) {
        double o2[2];
        adj_row(X, y, i, j, k, o2, nullptr);
        size_t q = cidx(gr, i, j, k, 0);
        for (int c = 0; c < 2; c++) out[q + c * X.n] = g ? g[q + c * X.n] - o2[c] : o2[c];
      }
  return 0;
}

int orc_hc_adjoint_gsrb_pass(const mlgpu_nlop *op, const double *phi, const double *J,
                             double *yd, const double *g, int pass) {
  AdjCtx X(*op, phi, J);
  Fab y;
  y.define(op->grid, 2);
  y.load(yd);
  adj_gsrb_pass_fab(y, X, g, pass);
  y.store(yd);
  return 0;
}

int orc_hc_adjoint_restrict(const mlgpu_nlop *op, const double *phi, const double *J,
                            const double *y, const double *g, double *gc) {
  AdjSolver::orc_hc_adjoint_restrict_impl(*op, phi, J, y, g, gc);
  return 0;
}

int orc_hc_linearized_apply(const mlgpu_nlop *op, const double *phi, const double *J,
                            const double *x, double *out) {
  AdjCtx X(*op, phi, J);
  lin_apply(X, x, out);
  return 0;
}

int orc_hc_lin_gsrb_pass(const mlgpu_nlop *op, const double *phi, const double *J, double *x,
                         const double *r, int pass) {
  AdjCtx X(*op, phi, J);
  lin_gsrb_pass(X, x, r, pass);
  return 0;
}

int orc_hc_adjoint_solve(const mlgpu_nlop *op, const mlgpu_mg_options *o, const double *phi,
                         const double *g, double *y, mlgpu_solve_stats *st) {
  AdjSolver S;
  S.op0 = *op;
  if (!(S.op0.nlbc.dx > 0)) S.op0.nlbc.dx = op->grid.dx;
  S.o = *o;
  S.build(phi);
  memset(st, 0, sizeof(*st));
  st->levels = (int)S.L.size();
  size_t n = 2 * ncells(op->grid);
  std::copy(y, y + n, S.L[0].y.begin());
  std::copy(g, g + n, S.L[0].gg.begin());
  mlgpu_nlop op0 = S.op_at(0);
  auto resnorm = [&]() {
    orc_hc_adjoint_apply(&op0, S.L[0].u.data(), S.L[0].J.data(), S.L[0].y.data(),
                         S.L[0].gg.data(), S.L[0].r.data());
    S.updates += ncells(op->grid);
    return norm_of(S.L[0].r.data(), n, o->norm_type);
  };
  int cycles = 0;
  auto iterate = [&]() {
    S.cycle(0);
    cycles++;
  };
  int rc = outer_loop(*o, st, resnorm, iterate);
  st->cycles = cycles;
  st->cell_updates = S.updates;
  std::copy(S.L[0].y.begin(), S.L[0].y.end(), y);
  return rc;
}

// -y^T dN/dv for the wall values, grad[(d * 2 + side) * 2 + c]
int orc_hc_adjoint_bc_gradient(const mlgpu_nlop *op, const double *phi, const double *J,
                               const double *y, double *grad) {
  AdjCtx X(*op, phi, J);
  const mlgpu_grid &g = op->grid;
  for (int q = 0; q < 12; q++) grad[q] = 0.0;
  const mlgpu_bc &bc = op->apply_derived_bc ? op->derived_bc : op->phi_bc;
  for (int d = 0; d < g.dim; d++) {
    if (g.periodic[d]) continue;
    for (int side = 0; side < 2; side++) {
      int lo[3] = {0, 0, 0}, hi[3] = {g.n[0] - 1, g.n[1] - 1, g.n[2] - 1};
      lo[d] = hi[d] = side == 0 ? 0 : g.n[d] - 1;
      double acc[2] = {0.0, 0.0};
      for (int k = lo[2]; k <= hi[2]; k++)
        for (int j = lo[1]; j <= hi[1]; j++)
          for (int i = lo[0]; i <= hi[0]; i++) {
            size_t q = cidx(g, i, j, k, 0);
            int fi[3] = {i, j, k};
            if (side) fi[d] += 1;
            double yb0 = y[q] * X.B(d, fi[0], fi[1], fi[2], 0);
            double yb1 = y[q + X.n] * X.B(d, fi[0], fi[1], fi[2], 1);
            if (op->apply_derived_bc) {
              acc[0] += yb0;
              acc[1] += yb1;
            } else {
              double Jg[4];
              ghost_jac(X, q, d, side, Jg);
              acc[0] += yb0 * Jg[0] + yb1 * Jg[2];
              acc[1] += yb0 * Jg[1] + yb1 * Jg[3];
            }
          }
      for (int c = 0; c < 2; c++) {
        double df = bc.type[d][side][c] == MLGPU_BC_DIRICHLET ? 2.0 : (side ? 1.0 : -1.0) * g.dx;
        if (op->apply_derived_bc && bc.type[d][side][c] == MLGPU_BC_MIXED_TEMPERATURE_SALINITY)
          df = mixed_t(op->nlbc, g.dx, d, side).f;
        grad[(d * 2 + side) * 2 + c] = op->beta * X.dxinv * df * acc[c];
      }
    }
  }
  return 0;
}

// adjoint of orc_hc_backward_euler: A^T mu = phi_new_bar (alpha 1, beta -dt),
// phi_old_bar = a mu, src_bar = dt mu, bc gradient of -mu^T N
int orc_hc_backward_euler_adjoint(const mlgpu_nlop *op, const mlgpu_mg_options *o,
                                  const double *phi_new, const double *phi_new_bar,
                                  const double *a, double dt, double *mu, double *phi_old_bar,
                                  double *src_bar, double *bc_grad, mlgpu_solve_stats *st) {
  mlgpu_nlop be = *op;
  be.alpha = 1.0;
  be.beta = -dt;
  int rc = orc_hc_adjoint_solve(&be, o, phi_new, phi_new_bar, mu, st);
  size_t n = 2 * ncells(op->grid);
  for (size_t q = 0; q < n; q++) {
    if (phi_old_bar) phi_old_bar[q] = a ? a[q] * mu[q] : mu[q];
    if (src_bar) src_bar[q] = dt * mu[q];
  }
  if (bc_grad) {
    std::vector<double> J(2 * n);
    orc_closure_jac(&op->grid, &op->params, phi_new, J.data());
    orc_hc_adjoint_bc_gradient(&be, phi_new, J.data(), mu, bc_grad);
  }
  return rc;
}

// adjoint of orc_mac_project: D Pi G q = G^T (Pi ubar), ustar_bar = ubar - D^T q,
// pi_bar = -ustar_bar (G p)
int orc_mac_project_adjoint(const mlgpu_vcop *op, const mlgpu_mg_options *o,
                            const mlgpu_bc *phi_bc, const double *ubar[3], const double *pi[3],
                            const double *p, double *ustar_bar[3], double *pi_bar[3], double *q,
                            mlgpu_solve_stats *st) {
  const mlgpu_grid &g = op->grid;
  const size_t n = ncells(g);
  std::vector<double> r(n);
  const double one_on_dx = 1.0 / g.dx;
  for (int k = 0; k < g.n[2]; k++)
    for (int j = 0; j < g.n[1]; j++)
      for (int i = 0; i < g.n[0]; i++) {
        const int at[3] = {i, j, k};
        double v = 0.0;
        for (int d = 0; d < g.dim; d++) {
          const int m = g.n[d], a = at[d];
          int f[3] = {i, j, k};
          size_t flo = fidx(g, d, f[0], f[1], f[2], 0);
          f[d] += 1;
          size_t fhi = fidx(g, d, f[0], f[1], f[2], 0);
          auto yv = [&](size_t ff) { return pi && pi[d] ? ubar[d][ff] * pi[d][ff] : ubar[d][ff]; };
          double clo = 1.0, chi = -1.0;
          if (!g.periodic[d]) {
            if (a == 0) clo = phi_bc->type[d][0][0] == MLGPU_BC_DIRICHLET ? 2.0 : 0.0;
            if (a == m - 1) chi = phi_bc->type[d][1][0] == MLGPU_BC_DIRICHLET ? -2.0 : 0.0;
          }
          double t = clo * yv(flo) + chi * yv(fhi);
          if (g.periodic[d]) {
            if (a == 0) {
              f[d] = m;
              t = t + yv(fidx(g, d, f[0], f[1], f[2], 0));
            }
            if (a == m - 1) {
              f[d] = 0;
              t = t - yv(fidx(g, d, f[0], f[1], f[2], 0));
            }
          }
          v = v + t / g.dx;
        }
        r[cidx(g, i, j, k, 0)] = v;
      }
  int rc = orc_vc_solve(op, o, q, r.data(), st);
  for (int d = 0; d < g.dim; d++) {
    int m[3];
    for (int e = 0; e < 3; e++) m[e] = g.n[e] + (e == d);
    for (int k = 0; k < m[2]; k++)
      for (int j = 0; j < m[1]; j++)
        for (int i = 0; i < m[0]; i++) {
          int f[3] = {i, j, k};
          const int b = f[d];
          double dt = 0.0;
          if (b >= 1) {
            int c[3] = {i, j, k};
            c[d] = b - 1;
            dt = dt + one_on_dx * q[cidx(g, c[0], c[1], c[2], 0)];
          }
          if (b <= g.n[d] - 1) dt = dt - one_on_dx * q[cidx(g, i, j, k, 0)];
          size_t ff = fidx(g, d, i, j, k, 0);
          ustar_bar[d][ff] = ubar[d][ff] - dt;
        }
  }
  if (pi_bar) {
    Fab ph(g, 1);
    ph.load(p);
    fill_ghosts(ph, g, *phi_bc, false);
    for (int d = 0; d < g.dim; d++) {
      if (!pi_bar[d]) continue;
      int m[3];
      for (int e = 0; e < 3; e++) m[e] = g.n[e] + (e == d);
      for (int k = 0; k < m[2]; k++)
        for (int j = 0; j < m[1]; j++)
          for (int i = 0; i < m[0]; i++) {
            int ii = i - (d == 0), jj = j - (d == 1), kk = k - (d == 2);
            size_t ff = fidx(g, d, i, j, k, 0);
            double grad = (ph(i, j, k, 0) - ph(ii, jj, kk, 0)) / g.dx;
            pi_bar[d][ff] = -(ustar_bar[d][ff] * grad);
          }
    }
  }
  return rc;
}

}  // extern "C"

// Bounds and regime of (H, C) for the Newton update's clipping
// (step_clip_near restated: FP64 bounds with the constant divisors as
// reciprocals); 0 solid, 1 eutectic, 2 mush, 3 liquid, 4 NaN
static void clip_bounds(double C, const mlgpu_params &p, double B[3]) {
  const double CR = p.compositionRatio, cp = p.specificHeatRatio, St = p.stefan,
               te = p.thetaEutectic, Te = p.ThetaEutectic;
  const double inv_k = 1.0 / p.waterDistributionCoeff, inv_CRTe = 1.0 / (CR + Te);
  double Hs = (C < -CR) ? 0.0 : cp * ((-C - CR) * inv_k);
  if (Hs < 0.0) Hs = 0.0;
  B[0] = Hs + te * cp;
  B[1] = (CR + C) * inv_CRTe * (St + te * (1 - cp)) + cp * te;
  B[2] = St - C + te + Te;
}
static int clip_regime(double H, const double B[3]) {
  if (H <= B[0]) return 0;
  if (H > B[0] && H <= B[1]) return 1;
  if (H > B[1] && H < B[2]) return 2;
  if (H >= B[2]) return 3;
  return 4;
}

// the device Newton's default clip of the update and cap of the forcing term
constexpr double kNewtonClip = 0.1, kNewtonEtaMax = 0.3;

// Newton for N(phi) = rhs on the Jacobian hierarchy (the device's
// mlgpu_hc_newton_solve restated with its default settings): A(u) d =
// rhs - N(u) by V-cycles on A to eta relative (at most 12; eta the
// Eisenstat-Walker forcing term, choice 2, gamma 0.9, alpha 2, safeguarded,
// capped at 0.3, at least 0.5 tolerance |r_0| / |r_k|, and lowered to that
// bound on a converging step (|r_k| / |r_k-1| < 0.1) when it is within a
// factor 10 of the forcing), u = u_old + s d with a
// cell whose H would leave
// its closure regime stopped at the first regime boundary it crosses plus
// kNewtonClip of its overshoot, s halved while the L2 residual grows (at most
// 4 times), stagnation on the L2 merit, three stalled steps below 1e-8 of the
// start end the solve
extern "C" int orc_hc_newton_solve(const mlgpu_nlop *op, const mlgpu_mg_options *o, double *phi,
                                   const double *rhs, mlgpu_solve_stats *st) {
  AdjSolver S;
  S.op0 = *op;
  if (!(S.op0.nlbc.dx > 0)) S.op0.nlbc.dx = op->grid.dx;
  S.o = *o;
  S.tr = false;
  S.build(phi);
  memset(st, 0, sizeof(*st));
  st->levels = (int)S.L.size();
  const size_t n = 2 * ncells(op->grid);
  std::vector<double> r(n), uold(n), lr(n);
  mlgpu_nlop op0 = S.op_at(0);
  auto nl = [&](double &merit) {
    orc_nl_residual(&op0, r.data(), S.L[0].u.data(), rhs);
    merit = norm_of(r.data(), n, MLGPU_NORM_L2);
    return norm_of(r.data(), n, o->norm_type);
  };
  auto lin_norm = [&]() {
    AdjCtx X(op0, S.L[0].u.data(), S.L[0].J.data());
    lin_apply(X, S.L[0].y.data(), lr.data());
    for (size_t q = 0; q < n; q++) lr[q] = S.L[0].gg[q] - lr[q];
    return norm_of(lr.data(), n, o->norm_type);
  };
  double merit;
  const double norm0 = nl(merit);
  double norm = norm0, prev = norm0;
  st->initial_norm = norm0;
  st->norm_history[0] = norm0;
  int iter = 0, status = std::isfinite(norm0) ? 0 : 8, stall = 0, cycles = 0;
  double eta = kNewtonEtaMax;
  while (norm > o->tolerance * norm0 && norm0 > o->norm_thresh && iter < o->max_iter &&
         status == 0) {
    S.refresh();
    std::fill(S.L[0].y.begin(), S.L[0].y.end(), 0.0);
    std::copy(r.begin(), r.end(), S.L[0].gg.begin());
    const double l0 = lin_norm();
    double ln = l0;
    for (int c = 0; c < 12 && ln > eta * l0; c++) {
      S.cycle(0);
      cycles++;
      ln = lin_norm();
    }
    uold = S.L[0].u;
    double scale = 1.0, merit_new = merit, norm_new = norm;
    for (int h = 0; h <= 4; h++) {
      for (size_t q = 0; q < n; q++) S.L[0].u[q] = scale * S.L[0].y[q] + 1.0 * uold[q];
      const size_t nc = n / 2;
      for (size_t q = 0; q < nc; q++) {
        double &h1 = S.L[0].u[q];
        const double c1 = S.L[0].u[nc + q];
        double B0[3], B1[3];
        clip_bounds(uold[nc + q], op->params, B0);
        clip_bounds(c1, op->params, B1);
        const int r0 = clip_regime(uold[q], B0), r1 = clip_regime(h1, B1);
        if (r0 != r1 && r0 < 4 && r1 < 4) {
          const double bnd = B1[r1 > r0 ? r0 : r0 - 1];
          h1 = bnd + (double)(float)kNewtonClip * (h1 - bnd);
        }
      }
      norm_new = nl(merit_new);
      if (std::isfinite(merit_new) && merit_new <= merit) break;
      scale *= 0.5;
    }
    const double merit_prev = merit;
    merit = merit_new;
    norm = norm_new;
    stall = norm >= 0.95 * prev ? stall + 1 : 0;
    iter++;
    if (iter < 64) st->norm_history[iter] = norm;
    if (!std::isfinite(norm) || !std::isfinite(merit))
      status = 8;
    else if (merit > (1.0 - o->hang) * merit_prev && norm > o->tolerance * norm0)
      status = 2;
    if (prev > 0 && std::isfinite(norm)) {
      const double ratio = norm / prev;
      double e = 0.9 * ratio * ratio;
      const double guard = 0.9 * eta * eta;
      if (guard > 0.1) e = std::max(e, guard);
      e = std::min(e, kNewtonEtaMax);
      const double fin = 0.5 * o->tolerance * norm0 / norm;
      eta = std::min(kNewtonEtaMax, std::max(e, fin));
      // finishing step: down to the forcing that ends the solve when that
      // costs at most a tenth more reduction
      if (ratio < 0.1 && fin < eta && fin >= 0.1 * eta) eta = fin;
    }
    prev = norm;
    if (stall >= 3 && norm < 1e-8 * norm0 && status == 0) status = 2;
  }
  std::copy(S.L[0].u.begin(), S.L[0].u.end(), phi);
  st->iterations = iter;
  st->cycles = cycles;
  st->final_norm = norm;
  if (status == 0 && norm > o->tolerance * norm0 && norm0 > o->norm_thresh) status = 4;
  st->exit_status = status;
  if (status == 8) return MLGPU_ERR_NAN;
  if (status == 2) return MLGPU_ERR_HANG;
  if (status == 4) return MLGPU_ERR_NOT_CONVERGED;
  return MLGPU_OK;
}
