// common.cuh -- device-side geometry, boundary conditions and the FP64
// enthalpy closure shared by every sm_103a kernel of the library.
//
// Layout: cell field [comp][k][j][i] (i fastest), no ghost cells stored.
// Face field of direction d: [comp][k][j][i] with n[d]+1 entries along d.
// A stencil that needs a ghost value produces it in registers from the
// interior cell next to the boundary, with the reference's first-order rules
// (BCutil/BCFuncF.ChF:14-95): Dirichlet ghost = 2 v - interior, Neumann
// ghost = interior + s dx g, periodic = wrapped interior.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/mlgpu.h"

namespace mlgpu {

struct Geom {
  int dim;
  int n0, n1, n2;
  int per0, per1, per2;
  double dx;
  long long ncell;  // cells per component
  __host__ __device__ int n(int d) const { return d == 0 ? n0 : (d == 1 ? n1 : n2); }
  __host__ __device__ int per(int d) const { return d == 0 ? per0 : (d == 1 ? per1 : per2); }
  __host__ __device__ long long cell(int i, int j, int k) const {
    return ((long long)k * n1 + j) * n0 + i;
  }
  // face (i,j,k) of direction d sits between cells (i,j,k)-e_d and (i,j,k)
  __host__ __device__ long long face(int d, int i, int j, int k) const {
    if (d == 0) return ((long long)k * n1 + j) * (n0 + 1) + i;
    if (d == 1) return ((long long)k * (n1 + 1) + j) * n0 + i;
    return ((long long)k * n1 + j) * n0 + i;
  }
  __host__ __device__ long long nface(int d) const {
    return (long long)(n0 + (d == 0)) * (n1 + (d == 1)) * (n2 + (d == 2));
  }
};

inline Geom make_geom(const mlgpu_grid &g) {
  Geom G;
  G.dim = g.dim;
  G.n0 = g.n[0];
  G.n1 = g.n[1];
  G.n2 = g.dim == 3 ? g.n[2] : 1;
  G.per0 = g.periodic[0];
  G.per1 = g.periodic[1];
  G.per2 = g.dim == 3 ? g.periodic[2] : 0;
  G.dx = g.dx;
  G.ncell = (long long)G.n0 * G.n1 * G.n2;
  return G;
}

__host__ __device__ inline Geom coarsen_geom(const Geom &f) {
  Geom c = f;
  c.n0 = f.n0 / 2;
  c.n1 = f.n1 / 2;
  c.n2 = f.dim == 3 ? f.n2 / 2 : 1;
  c.dx = f.dx * 2;
  c.ncell = (long long)c.n0 * c.n1 * c.n2;
  return c;
}

// Boundary description in a kernel-argument friendly form.
struct BCD {
  int type[3][2][2];
  double val[3][2][2];
};

inline BCD make_bcd(const mlgpu_bc &b) {
  BCD r;
  for (int d = 0; d < 3; d++)
    for (int s = 0; s < 2; s++)
      for (int c = 0; c < 2; c++) {
        r.type[d][s][c] = b.type[d][s][c];
        r.val[d][s][c] = b.value[d][s][c];
      }
  return r;
}

// Ghost value on side s (0 low, 1 high) of direction d from the interior
// value next to it (DIRIBC order 1 / NEUMBC).
template <class T>
__device__ __forceinline__ T ghost_value(const BCD &bc, int d, int s, int c, T interior,
                                         T dx, bool homogeneous) {
  T v = homogeneous ? T(0) : T(bc.val[d][s][c]);
  if (bc.type[d][s][c] == MLGPU_BC_DIRICHLET) return T(2) * v - interior;
  T isign = s == 0 ? T(-1) : T(1);
  return interior + (isign * dx) * v;
}

// ------------------------------------------------------------ closure (FP64)
struct ClosureParams {
  double CR, k, cp, St, te, Te;
};

inline ClosureParams make_cp(const mlgpu_params &p) {
  ClosureParams c;
  c.CR = p.compositionRatio;
  c.k = p.waterDistributionCoeff;
  c.cp = p.specificHeatRatio;
  c.St = p.stefan;
  c.te = p.thetaEutectic;
  c.Te = p.ThetaEutectic;
  return c;
}

// CALCULATE_BOUNDING_ENERGY (src/EnthalpyVariablesF.ChF:657-698)
__device__ __forceinline__ void bounding_energy(double C, const ClosureParams &p,
                                                double &Hs, double &He, double &Hl) {
  if (C < -p.CR)
    Hs = 0.0;
  else
    Hs = p.cp * ((-C - p.CR) / p.k);
  if (Hs < 0.0) Hs = 0.0;
  Hs = Hs + p.te * p.cp;
  double pe = (p.CR + C) / (p.CR + p.Te);
  He = pe * (p.St + p.te * (1 - p.cp)) + p.cp * p.te;
  Hl = p.St - C + p.te + p.Te;
}

// CALCULATEPOROSITYMUSH (src/EnthalpyVariablesF.ChF:103-150)
__device__ __forceinline__ double porosity_mush(double C, double H, const ClosureParams &p) {
  double validC = (C >= -p.CR) ? C : -p.CR;
  if (p.St == 0) return 1.0;
  double a = p.CR * (p.cp - 1) + p.St * (p.k - 1);
  double b = p.CR * (1 - 2 * p.cp) + H * (1 - p.k) - validC * (p.cp - 1) - p.k * p.St;
  double c = (p.CR + validC) * p.cp + p.k * H;
  return (-b - sqrt(b * b - 4 * a * c)) / (2 * a);
}

// CALCULATE_T_CL (src/EnthalpyVariablesF.ChF:419-467): (H, C) -> (T, C_l)
__device__ __forceinline__ void t_cl(double H, double C, const ClosureParams &p, double &T,
                                     double &Cl) {
  double Hs, He, Hl;
  bounding_energy(C, p, Hs, He, Hl);
  if (H <= Hs) {
    T = H / p.cp;
    Cl = p.Te;
  } else if (H > Hs && H <= He) {
    T = p.te;
    Cl = p.Te;
  } else if (H > He && H < Hl) {
    double por = porosity_mush(C, H, p);
    // T = -(x) / d and C_l = x / d: IEEE division is symmetric in the sign of
    // the numerator, so T is exactly -C_l (one FP64 division instead of two)
    Cl = (C + p.CR * (1 - por)) / (por + p.k * (1 - por));
    T = -Cl;
  } else if (H >= Hl) {
    T = H - p.St;
    Cl = C;
  } else {  // NaN input
    T = H;
    Cl = C;
  }
}

// Derivative of t_cl: J = {dT/dH, dT/dC, dC_l/dH, dC_l/dC}, regime by regime
// (solid T = H/cp; eutectic constant; mush through the porosity root
// a por^2 + b por + c = 0, differentiated implicitly, with C clamped at -CR
// as CALCULATEPOROSITYMUSH does; liquid T = H - St, C_l = C).  Used by the
// linearised inner cycles of the mixed-precision nonlinear solve; it has no
// counterpart in the reference, which only evaluates the closure.
__device__ __forceinline__ void t_cl_jac(double H, double C, const ClosureParams &p, double J[4]) {
  double Hs, He, Hl;
  bounding_energy(C, p, Hs, He, Hl);
  J[0] = J[1] = J[2] = J[3] = 0.0;
  if (H <= Hs) {
    J[0] = 1.0 / p.cp;
  } else if (H > Hs && H <= He) {
    // eutectic: T and C_l fixed
  } else if (H > He && H < Hl) {
    double por = 1.0, dpH = 0.0, dpC = 0.0;
    if (p.St != 0) {
      const bool clamp = !(C >= -p.CR);
      const double validC = clamp ? -p.CR : C;
      const double a = p.CR * (p.cp - 1) + p.St * (p.k - 1);
      const double b = p.CR * (1 - 2 * p.cp) + H * (1 - p.k) - validC * (p.cp - 1) - p.k * p.St;
      const double c = (p.CR + validC) * p.cp + p.k * H;
      const double sD = sqrt(b * b - 4 * a * c);
      por = (-b - sD) / (2 * a);
      const double dbH = 1 - p.k, dbC = clamp ? 0.0 : -(p.cp - 1);
      const double dcH = p.k, dcC = clamp ? 0.0 : p.cp;
      dpH = (-dbH - (b * dbH - 2 * a * dcH) / sD) / (2 * a);
      dpC = (-dbC - (b * dbC - 2 * a * dcC) / sD) / (2 * a);
    }
    const double num = C + p.CR * (1 - por), den = por + p.k * (1 - por);
    const double dCl_dpor = (-p.CR * den - num * (1 - p.k)) / (den * den);
    J[2] = dCl_dpor * dpH;
    J[3] = 1.0 / den + dCl_dpor * dpC;
    J[0] = -J[2];
    J[1] = -J[3];
  } else if (H >= Hl) {
    J[0] = 1.0;
    J[3] = 1.0;
  }
}

// ------------------------------------------------------------ thread helpers
__device__ __forceinline__ long long gtid() {
  return (long long)blockIdx.x * blockDim.x + threadIdx.x;
}
__device__ __forceinline__ long long gstride() { return (long long)gridDim.x * blockDim.x; }

// Index decode in 32-bit unsigned arithmetic (a box holds fewer than 2^31
// cells per component; the library rejects larger boxes): a 64-bit division
// costs ~4x the instructions and dominated the small stencil kernels.
__device__ __forceinline__ void cell_ijk(const Geom &G, long long q, int &i, int &j, int &k) {
  unsigned u = (unsigned)q, n0 = (unsigned)G.n0, n1 = (unsigned)G.n1;
  unsigned t = u / n0;
  i = (int)(u - t * n0);
  unsigned kk = t / n1;
  j = (int)(t - kk * n1);
  k = (int)kk;
}

// Active cells of a red (pass 0) / black (pass 1) half sweep.  The
// reference's parity rule imin = lo + |mod(lo + j + k + pass, 2)| with lo = 0
// selects cells with (i + j + k) % 2 == pass.
__device__ __forceinline__ bool colour_cell(const Geom &G, int pass, long long t, int &i, int &j,
                                            int &k) {
  unsigned half = (unsigned)(G.n0 + 1) / 2u, n1 = (unsigned)G.n1;
  unsigned u = (unsigned)t;
  unsigned row = u / half;
  int h = (int)(u - row * half);
  unsigned kk = row / n1;
  j = (int)(row - kk * n1);
  k = (int)kk;
  int imin = (j + k + pass) & 1;
  i = imin + 2 * h;
  return i < G.n0 && k < G.n2;
}

__host__ __device__ inline long long colour_threads(const Geom &G) {
  return (long long)((G.n0 + 1) / 2) * G.n1 * G.n2;
}

}  // namespace mlgpu
