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

// The derived-variable (T, C_l) conditions: BCD plus, per [dir][side], the
// constants of the MixedBCTemperatureSalinity ghost on T
// (BCutil/PhysBCUtil.cpp:764-800): p1 = a/dx + b/2, bt = b T_ref,
// p2 = a/dx - b/2, the derivative g = p1 / p2 of the ghost with respect to the
// interior value, and f = 1 / p2 with respect to F (the value)
struct DBCD : BCD {
  double rob[3][2][5];  // p1, bt, p2, g, f
};

inline DBCD make_dbcd(const mlgpu_bc &b, const mlgpu_nlbc &nb, double grid_dx) {
  DBCD r;
  static_cast<BCD &>(r) = make_bcd(b);
  const double dx = nb.dx > 0 ? nb.dx : grid_dx;
  for (int d = 0; d < 3; d++)
    for (int s = 0; s < 2; s++) {
      double *o = r.rob[d][s];
      o[0] = o[1] = o[2] = o[3] = o[4] = 0.0;
      if (b.type[d][s][0] != MLGPU_BC_MIXED_TEMPERATURE_SALINITY) continue;
      const double a = nb.a[d][s], bb = nb.b[d][s];
      o[0] = a / dx + bb / 2;
      o[1] = bb * nb.T_ref[d][s];
      o[2] = a / dx - bb / 2;
      o[3] = o[0] / o[2];
      o[4] = 1.0 / o[2];
    }
  return r;
}

// Derived-variable ghost: the mixed temperature condition on comp 0, else
// ghost_value.  Inhomogeneous: (T_i p1 + F - bt) / p2 in the reference's
// order; homogeneous (the linearised operators): g T_i.
template <class T>
__device__ __forceinline__ T ghost_value(const DBCD &bc, int d, int s, int c, T interior,
                                         T dx, bool homogeneous) {
  if (bc.type[d][s][c] == MLGPU_BC_MIXED_TEMPERATURE_SALINITY) {
    const double *r = bc.rob[d][s];
    if (homogeneous) return T(r[3]) * interior;
    return (interior * T(r[0]) + T(bc.val[d][s][c]) - T(r[1])) / T(r[2]);
  }
  return ghost_value<T>(static_cast<const BCD &>(bc), d, s, c, interior, dx, homogeneous);
}

// A derived-condition wall's share of the diagonal face sum: the ghost's
// homogeneous rule g T_i makes the face term b (g - 1) T_i, so the wall adds
// (1 - g) b: 2b Dirichlet, 0 Neumann, (1 - g) b mixed
template <class T>
__device__ __forceinline__ T dbc_wall_diag(const DBCD &bc, int d, int s, int c, T bf) {
  const int t = bc.type[d][s][c];
  if (t == MLGPU_BC_DIRICHLET) return T(2) * bf;
  if (t == MLGPU_BC_MIXED_TEMPERATURE_SALINITY) return T(1.0 - bc.rob[d][s][3]) * bf;
  return T(0);
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
  } else {
    // NaN input (a departure from CALCULATE_T_CL, which takes no branch and
    // leaves the output untouched): T and C_l become NaN so the solvers'
    // NaN detection sees the poisoned state
    T = H;
    Cl = C;
  }
}

// ---- FP32 <-> FP64 conversions on the integer pipe.  GB300 issues the
// hardware conversions on its FP64 pipe (1/64 of the FP32 rate), where a
// kernel that converts a few values per cell spends most of its time.
// FP64 <-> FP32 conversions on the integer pipe.  GB300 runs FP64 work,
// conversions included, at 1/64 of the FP32 rate, and a fallback to the
// hardware conversion for rare inputs is predicated by the compiler, so it
// would still issue on the FP64 pipe for every cell: every case is formed
// from the bit pattern instead.  Results below FP32's normal range flush to a
// signed zero, inf stays inf and NaN a (quiet) NaN.
// f32_trunc: x rounded toward zero (overflow: the largest finite magnitude);
// for decisions with a margin far above an FP32 ulp and for seeds refined in
// FP64.
__device__ __forceinline__ float f32_trunc(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32);
  const unsigned s = hi & 0x80000000u, ex = (hi >> 20) & 0x7ffu;
  const int e = (int)ex - 896;  // FP32 biased exponent
  unsigned r = s | ((unsigned)e << 23) | ((hi & 0xfffffu) << 3) | (unsigned)((b >> 29) & 7u);
  r = e <= 0 ? s : r;
  r = e >= 255 ? (s | 0x7f7fffffu) : r;
  r = ex == 0x7ffu ? (s | 0x7f800000u | ((b << 12) != 0ull ? 0x400000u : 0u)) : r;
  return __uint_as_float(r);
}
// f32_round: x rounded to nearest, ties to even (overflow: inf)
__device__ __forceinline__ float f32_round(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32);
  const unsigned s = hi & 0x80000000u, ex = (hi >> 20) & 0x7ffu;
  const int e = (int)ex - 896;
  unsigned r = ((unsigned)e << 23) | ((hi & 0xfffffu) << 3) | (unsigned)((b >> 29) & 7u);
  const unsigned rem = (unsigned)(b & 0x1fffffffull);  // the 29 dropped bits
  r += (rem > 0x10000000u || (rem == 0x10000000u && (r & 1u))) ? 1u : 0u;  // may carry to inf
  r = e <= 0 ? 0u : r;
  r = e >= 255 ? 0x7f800000u : r;
  r = ex == 0x7ffu ? (0x7f800000u | ((b << 12) != 0ull ? 0x400000u : 0u)) : r;
  return __uint_as_float(s | r);
}
// f64_exact: the FP64 value of f (exact; FP32 subnormals flush to zero)
__device__ __forceinline__ double f64_exact(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  const unsigned long long s = (unsigned long long)(u & 0x80000000u) << 32;
  const unsigned long long m = (unsigned long long)(u & 0x7fffffu) << 29;
  unsigned long long r = s | ((unsigned long long)(e + 896u) << 52) | m;
  r = e == 0u ? s : r;
  r = e == 255u ? (s | 0x7ff0000000000000ull | m) : r;
  return __longlong_as_double((long long)r);
}
// the cycles' precision T from FP64: f32_round for float
template <class T>
__device__ __forceinline__ T narrow_to(double x) {
  if constexpr (sizeof(T) == 4)
    return f32_round(x);
  else
    return x;
}

// ---- lean FP64 closure (the outer loops of the lean Newton paths)
// t_cl with the closure's divisions by constants as products with their
// reciprocals and the two per-cell operations (the porosity root's square
// root, the liquid concentration's quotient) from an FP32 seed refined in
// FP64: the coupled square-root / half-reciprocal-root iteration and the
// reciprocal-then-quotient correction of Markstein ("Computation of
// elementary functions on the IBM RISC System/6000", IBM J. Res. Dev. 34,
// 1990) and Karp & Markstein ("High-precision division and square root",
// ACM TOMS 23, 1997), with FMA residuals.  About half the FP64 pipe
// operations of t_cl per mush cell; within a few ulps of it (the Newton
// residual it feeds targets 1e-10 of the initial), not its bit pattern --
// the reference-order paths keep t_cl.
struct ClosureLean {
  double CR, k, cp, St, te, Te;
  double inv_k, inv_CRTe, He_slope, a, inv_2a, four_a, b0, omk, cpm1, inv_cp;
};

inline ClosureLean make_closure_lean(const ClosureParams &p) {
  ClosureLean L;
  L.CR = p.CR;
  L.k = p.k;
  L.cp = p.cp;
  L.St = p.St;
  L.te = p.te;
  L.Te = p.Te;
  L.inv_k = 1.0 / p.k;
  L.inv_CRTe = 1.0 / (p.CR + p.Te);
  L.He_slope = p.St + p.te * (1 - p.cp);
  L.a = p.CR * (p.cp - 1) + p.St * (p.k - 1);
  L.inv_2a = 1.0 / (2 * L.a);
  L.four_a = 4 * L.a;
  L.b0 = p.CR * (1 - 2 * p.cp) - p.k * p.St;
  L.omk = 1 - p.k;
  L.cpm1 = p.cp - 1;
  L.inv_cp = 1.0 / p.cp;
  return L;
}

// 0 < x < inf with 2^-99 <= x < 2^99, decided on the sign and exponent bits
// (integer pipe): the range where FP32 seeds are normal and the FP64
// refinements below neither overflow nor underflow
__device__ __forceinline__ bool lean_pos_range(double x) {
  const unsigned se = (unsigned)((unsigned long long)__double_as_longlong(x) >> 52);
  return se - 924u < 198u;  // sign 0, biased exponent in [1023 - 99, 1023 + 99)
}
// the same for |x|
__device__ __forceinline__ bool lean_abs_range(double x) {
  const unsigned e = (unsigned)((unsigned long long)__double_as_longlong(x) >> 52) & 0x7ffu;
  return e - 924u < 198u;
}
// |x| < 2^830 (about 7e249) and x not NaN, on the exponent bits
__device__ __forceinline__ bool lean_below_2p830(double x) {
  const unsigned e = (unsigned)((unsigned long long)__double_as_longlong(x) >> 52) & 0x7ffu;
  return e < 1853u;
}

// sqrt(D) for D well inside FP32's normal range (else the library square
// root); the FP32 seed's conversions on the integer pipe
__device__ __forceinline__ double lean_sqrt(double D) {
  if (!lean_pos_range(D)) return sqrt(D);
  const double y = f64_exact(rsqrtf(f32_trunc(D)));  // 1/sqrt(D) to ~2^-22
  double g = D * y, h = 0.5 * y;                      // sqrt(D), 1/(2 sqrt(D))
  const double r = fma(-g, h, 0.5);
  g = fma(g, r, g);
  h = fma(h, r, h);
  const double d = fma(-g, g, D);
  return fma(d, h, g);
}

// num / den for |den| well inside FP32's normal range and a finite quotient
// (else the library division)
__device__ __forceinline__ double lean_div(double num, double den) {
  if (!(lean_abs_range(den) && lean_below_2p830(num))) return num / den;
  double y = f64_exact(__frcp_rn(f32_trunc(den)));  // 1/den to ~2^-23
  y = fma(fma(-den, y, 1.0), y, y);                  // to ~2^-46
  const double q = num * y;
  return fma(fma(-den, q, num), y, q);
}

// 1 / x for |x| well inside FP32's normal range (else the library division):
// the FP32 reciprocal refined by two FMA iterations (~2^-23, 2^-46, then to
// within an ulp)
__device__ __forceinline__ double lean_rcp(double x) {
  if (!lean_abs_range(x)) return 1.0 / x;
  double y = f64_exact(__frcp_rn(f32_trunc(x)));
  y = fma(fma(-x, y, 1.0), y, y);
  return fma(fma(-x, y, 1.0), y, y);
}

// The regime of (H, C) (0 solid, 1 eutectic, 2 mush, 3 liquid, 4 NaN input)
// from FP32 bounds (integer-pipe conversions), re-decided in FP64 within 1e-4
// of a bound; the closure is continuous across its bounds, so a cell an ulp
// from one may take either side
__device__ __forceinline__ int lean_regime(double H, double C, const ClosureLean &p) {
  int reg;
  {
    const float h = f32_trunc(H), c = f32_trunc(C);
    const float CR = (float)p.CR, cpv = (float)p.cp;
    float Hs = (c < -CR) ? 0.f : cpv * ((-c - CR) * (float)p.inv_k);
    if (Hs < 0.f) Hs = 0.f;
    Hs = Hs + (float)p.te * cpv;
    const float He = (CR + c) * (float)p.inv_CRTe * (float)p.He_slope + cpv * (float)p.te;
    const float Hl = (float)p.St - c + (float)p.te + (float)p.Te;
    const float band = 1e-4f;
    if (fabsf(h - Hs) < band * (1.f + fabsf(Hs)) || fabsf(h - He) < band * (1.f + fabsf(He)) ||
        fabsf(h - Hl) < band * (1.f + fabsf(Hl))) {
      double Hs2 = (C < -p.CR) ? 0.0 : p.cp * ((-C - p.CR) * p.inv_k);
      if (Hs2 < 0.0) Hs2 = 0.0;
      Hs2 = Hs2 + p.te * p.cp;
      const double He2 = (p.CR + C) * p.inv_CRTe * p.He_slope + p.cp * p.te;
      const double Hl2 = p.St - C + p.te + p.Te;
      reg = H <= Hs2 ? 0 : (H <= He2 ? 1 : (H < Hl2 ? 2 : (H >= Hl2 ? 3 : 4)));
    } else {
      reg = h <= Hs ? 0 : (h <= He ? 1 : (h < Hl ? 2 : (h >= Hl ? 3 : 4)));
    }
  }
  return reg;
}

__device__ __forceinline__ void t_cl_lean(double H, double C, const ClosureLean &p, double &T,
                                          double &Cl) {
  const int reg = lean_regime(H, C, p);
  if (reg == 0) {
    T = H * p.inv_cp;
    Cl = p.Te;
  } else if (reg == 1) {
    T = p.te;
    Cl = p.Te;
  } else if (reg == 2) {
    double por = 1.0;
    if (p.St != 0) {
      const double vC = (C >= -p.CR) ? C : -p.CR;
      const double b = p.b0 + H * p.omk - vC * p.cpm1;
      const double c = (p.CR + vC) * p.cp + p.k * H;
      por = (-b - lean_sqrt(fma(b, b, -p.four_a * c))) * p.inv_2a;
    }
    Cl = lean_div(C + p.CR * (1 - por), por + p.k * (1 - por));
    T = -Cl;
  } else if (reg == 3) {
    T = H - p.St;
    Cl = C;
  } else {  // NaN input, as t_cl
    T = H;
    Cl = C;
  }
}

// d(T, C_l)/d(H, C) in FP64 for the lean FP64 Newton cycles: t_cl_jac_in's
// expressions in the lean closure's regime, with the constant divisors as
// reciprocals and the per-cell divisors (sqrt(disc), den) as one refined
// reciprocal each (lean_sqrt, lean_rcp) -- a Jacobian to within a few ulps of
// t_cl_jac's (the Newton iteration's fixed point is the residual's alone)
__device__ __forceinline__ void t_cl_jac_lean(double H, double C, const ClosureLean &p,
                                              double J[4]) {
  const int reg = lean_regime(H, C, p);
  J[0] = J[1] = J[2] = J[3] = 0.0;
  if (reg == 0) {
    J[0] = p.inv_cp;
  } else if (reg == 2) {
    double por = 1.0, dpH = 0.0, dpC = 0.0;
    if (p.St != 0) {
      const bool clamp = !(C >= -p.CR);
      const double vC = clamp ? -p.CR : C;
      const double b = p.b0 + H * p.omk - vC * p.cpm1;
      const double c = (p.CR + vC) * p.cp + p.k * H;
      const double sD = lean_sqrt(fma(b, b, -p.four_a * c));
      const double isD = lean_rcp(sD);
      por = (-b - sD) * p.inv_2a;
      const double two_a = 2 * p.a;
      const double dbH = p.omk, dbC = clamp ? 0.0 : -p.cpm1;
      const double dcH = p.k, dcC = clamp ? 0.0 : p.cp;
      dpH = (-dbH - (b * dbH - two_a * dcH) * isD) * p.inv_2a;
      dpC = (-dbC - (b * dbC - two_a * dcC) * isD) * p.inv_2a;
    }
    const double num = C + p.CR * (1 - por), den = por + p.k * (1 - por);
    const double iden = lean_rcp(den);
    const double dCl_dpor = (-p.CR * den - num * p.omk) * iden * iden;
    J[2] = dCl_dpor * dpH;
    J[3] = iden + dCl_dpor * dpC;
    J[0] = -J[2];
    J[1] = -J[3];
  } else if (reg == 3) {
    J[0] = 1.0;
    J[3] = 1.0;
  }
}

__device__ __forceinline__ float sqrtT(float x) { return sqrtf(x); }
__device__ __forceinline__ double sqrtT(double x) { return sqrt(x); }

// Regime of (H, C) as t_cl takes it: 0 solid, 1 eutectic, 2 mush, 3 liquid,
// 4 NaN input (no branch)
__device__ __forceinline__ int closure_regime(double H, double C, const ClosureParams &p) {
  double Hs, He, Hl;
  bounding_energy(C, p, Hs, He, Hl);
  if (H <= Hs) return 0;
  if (H > Hs && H <= He) return 1;
  if (H > He && H < Hl) return 2;
  if (H >= Hl) return 3;
  return 4;
}

// FP32 constants of the closure for the FP32 derivative and regime test
// (reciprocals of the constant divisors, so the per-cell work has no FP32
// division by a constant)
struct ClosureF32 {
  float CR, k, cp, St, te, Te, inv_k, inv_CRTe, He_slope, inv_cp, a, two_a, inv_2a, four_a, b0,
      omk, cpm1;
  double inv_k64, inv_CRTe64;  // 1/k, 1/(CR + Te) in FP64
};

__host__ __device__ inline ClosureF32 make_closure_f32(const ClosureParams &p) {
  ClosureF32 f;
  f.CR = (float)p.CR;
  f.k = (float)p.k;
  f.cp = (float)p.cp;
  f.St = (float)p.St;
  f.te = (float)p.te;
  f.Te = (float)p.Te;
  f.inv_k = (float)(1.0 / p.k);
  f.inv_CRTe = (float)(1.0 / (p.CR + p.Te));
  f.He_slope = (float)(p.St + p.te * (1 - p.cp));
  f.inv_cp = (float)(1.0 / p.cp);
  const double a = p.CR * (p.cp - 1) + p.St * (p.k - 1);
  f.a = (float)a;
  f.two_a = (float)(2 * a);
  f.inv_2a = (float)(1.0 / (2 * a));
  f.four_a = (float)(4 * a);
  f.b0 = (float)(p.CR * (1 - 2 * p.cp) - p.k * p.St);
  f.omk = (float)(1 - p.k);
  f.cpm1 = (float)(p.cp - 1);
  f.inv_k64 = 1.0 / p.k;
  f.inv_CRTe64 = 1.0 / (p.CR + p.Te);
  return f;
}

// The regime of a cell near a bound, in FP64 with the constant divisors as
// reciprocals (bounding_energy to an ulp; a cell within an ulp of a bound may
// go either way, which no FP64 iterate resolves anyway): the regime-clipped
// Newton update leaves many cells just past a bound, and FP64 divisions there
// would dominate the kernels that call it.  Out of line: rarely taken, and
// its FP64 registers would lower the callers' occupancy.
static __device__ __noinline__ int closure_regime_near(double H, double C,
                                                       const ClosureParams &p, double inv_k,
                                                       double inv_CRTe) {
  double Hs = (C < -p.CR) ? 0.0 : p.cp * ((-C - p.CR) * inv_k);
  if (Hs < 0.0) Hs = 0.0;
  Hs = Hs + p.te * p.cp;
  const double He = (p.CR + C) * inv_CRTe * (p.St + p.te * (1 - p.cp)) + p.cp * p.te;
  const double Hl = p.St - C + p.te + p.Te;
  if (H <= Hs) return 0;
  if (H > Hs && H <= He) return 1;
  if (H > He && H < Hl) return 2;
  if (H >= Hl) return 3;
  return 4;
}

// The same regime from FP32 bounding energies, with the FP64 test for the
// cells near a bound (within 1e-4 of its scale, far above the FP32 rounding
// of the bounds): every cell gets t_cl's own regime, at FP32 cost for all but
// the few near a phase boundary.
__device__ __forceinline__ int closure_regime_fast(double H, double C, const ClosureParams &p,
                                                   const ClosureF32 &f) {
  const float h = f32_trunc(H), c = f32_trunc(C);
  float Hs = (c < -f.CR) ? 0.f : f.cp * ((-c - f.CR) * f.inv_k);
  if (Hs < 0.f) Hs = 0.f;
  Hs = Hs + f.te * f.cp;
  const float He = (f.CR + c) * f.inv_CRTe * f.He_slope + f.cp * f.te;
  const float Hl = f.St - c + f.te + f.Te;
  const float band = 1e-4f;
  if (fabsf(h - Hs) < band * (1.f + fabsf(Hs)) || fabsf(h - He) < band * (1.f + fabsf(He)) ||
      fabsf(h - Hl) < band * (1.f + fabsf(Hl)))
    return closure_regime_near(H, C, p, f.inv_k64, f.inv_CRTe64);
  if (h <= Hs) return 0;
  if (h <= He) return 1;
  if (h < Hl) return 2;
  if (h >= Hl) return 3;
  return 4;
}

// Derivative of t_cl: J = {dT/dH, dT/dC, dC_l/dH, dC_l/dC} in regime `reg`
// (closure_regime): solid T = H/cp; eutectic constant; mush through the
// porosity root a por^2 + b por + c = 0, differentiated implicitly, with C
// clamped at -CR as CALCULATEPOROSITYMUSH does; liquid T = H - St, C_l = C.
// Used by the linearised cycles of the Newton solve and by the adjoint; it
// has no counterpart in the reference, which only evaluates the closure.
// T = double: the expressions of bounding_energy / porosity_mush in FP64;
// T = float: the same expressions in FP32 at the FP32-rounded state (the
// derivative only steers FP32 linear cycles, whose Newton residual and
// update stay FP64; in FP32 the divisions and the square root cost a few
// instructions instead of the FP64 pipe's tens of cycles per warp).
template <class T>
__device__ __forceinline__ void t_cl_jac_in(int reg, T H, T C, const ClosureParams &p, T J[4]) {
  const T CR = (T)p.CR, k = (T)p.k, cpv = (T)p.cp, St = (T)p.St;
  J[0] = J[1] = J[2] = J[3] = T(0);
  if (reg == 0) {
    J[0] = T(1) / cpv;
  } else if (reg == 2) {
    T por = T(1), dpH = T(0), dpC = T(0);
    if (St != T(0)) {
      const bool clamp = !(C >= -CR);
      const T validC = clamp ? -CR : C;
      const T a = CR * (cpv - T(1)) + St * (k - T(1));
      const T b = CR * (T(1) - T(2) * cpv) + H * (T(1) - k) - validC * (cpv - T(1)) - k * St;
      const T c = (CR + validC) * cpv + k * H;
      const T sD = sqrtT(b * b - T(4) * a * c);
      por = (-b - sD) / (T(2) * a);
      const T dbH = T(1) - k, dbC = clamp ? T(0) : -(cpv - T(1));
      const T dcH = k, dcC = clamp ? T(0) : cpv;
      dpH = (-dbH - (b * dbH - T(2) * a * dcH) / sD) / (T(2) * a);
      dpC = (-dbC - (b * dbC - T(2) * a * dcC) / sD) / (T(2) * a);
    }
    const T num = C + CR * (T(1) - por), den = por + k * (T(1) - por);
    const T dCl_dpor = (-CR * den - num * (T(1) - k)) / (den * den);
    J[2] = dCl_dpor * dpH;
    J[3] = T(1) / den + dCl_dpor * dpC;
    J[0] = -J[2];
    J[1] = -J[3];
  } else if (reg == 3) {
    J[0] = T(1);
    J[3] = T(1);
  }
  // eutectic (1): T and C_l fixed; NaN input (4): zero
}
__device__ __forceinline__ void t_cl_jac(double H, double C, const ClosureParams &p, double J[4]) {
  t_cl_jac_in<double>(closure_regime(H, C, p), H, C, p, J);
}
// FP32 derivative in t_cl's own regime (closure_regime_fast): t_cl_jac_in's
// expressions with the constant divisors as reciprocals and the per-cell
// divisors (sqrt(disc), den) as one correctly rounded reciprocal each
__device__ __forceinline__ void t_cl_jac32(double H, double C, const ClosureParams &p,
                                           const ClosureF32 &f, float J[4]) {
  const int reg = closure_regime_fast(H, C, p, f);
  const float h = f32_trunc(H), c = f32_trunc(C);
  J[0] = J[1] = J[2] = J[3] = 0.f;
  if (reg == 0) {
    J[0] = f.inv_cp;
  } else if (reg == 2) {
    float por = 1.f, dpH = 0.f, dpC = 0.f;
    if (f.St != 0.f) {
      const bool clamp = !(c >= -f.CR);
      const float vC = clamp ? -f.CR : c;
      const float b = f.b0 + h * f.omk - vC * f.cpm1;
      const float cc = (f.CR + vC) * f.cp + f.k * h;
      const float sD = sqrtf(b * b - f.four_a * cc);
      const float isD = __frcp_rn(sD);
      por = (-b - sD) * f.inv_2a;
      const float dbH = f.omk, dbC = clamp ? 0.f : -f.cpm1;
      const float dcH = f.k, dcC = clamp ? 0.f : f.cp;
      dpH = (-dbH - (b * dbH - f.two_a * dcH) * isD) * f.inv_2a;
      dpC = (-dbC - (b * dbC - f.two_a * dcC) * isD) * f.inv_2a;
    }
    const float num = c + f.CR * (1.f - por), den = por + f.k * (1.f - por);
    const float iden = __frcp_rn(den);
    const float dCl_dpor = (-f.CR * den - num * f.omk) * iden * iden;
    J[2] = dCl_dpor * dpH;
    J[3] = iden + dCl_dpor * dpC;
    J[0] = -J[2];
    J[1] = -J[3];
  } else if (reg == 3) {
    J[0] = 1.f;
    J[3] = 1.f;
  }
}

// Derivative of the porosity of the full closure (CALCULATEPOROSITY,
// src/EnthalpyVariablesF.ChF): {d por/dH, d por/dC} -- zero in the solid and
// the liquid, 1/(St + te (1 - cp)) in H on the eutectic, the porosity root
// differentiated implicitly in the mush (C clamped at -CR as
// CALCULATEPOROSITYMUSH does).  No counterpart in the reference.
__device__ __forceinline__ void porosity_jac(double H, double C, const ClosureParams &p,
                                             double dp[2]) {
  double Hs, He, Hl;
  bounding_energy(C, p, Hs, He, Hl);
  dp[0] = dp[1] = 0.0;
  if (H <= Hs) {
  } else if (H > Hs && H <= He) {
    dp[0] = 1.0 / (p.St + p.te * (1 - p.cp));
  } else if (H > He && H < Hl) {
    if (p.St != 0) {
      const bool clamp = !(C >= -p.CR);
      const double validC = clamp ? -p.CR : C;
      const double a = p.CR * (p.cp - 1) + p.St * (p.k - 1);
      const double b = p.CR * (1 - 2 * p.cp) + H * (1 - p.k) - validC * (p.cp - 1) - p.k * p.St;
      const double c = (p.CR + validC) * p.cp + p.k * H;
      const double sD = sqrt(b * b - 4 * a * c);
      const double dbH = 1 - p.k, dbC = clamp ? 0.0 : -(p.cp - 1);
      const double dcH = p.k, dcC = clamp ? 0.0 : p.cp;
      dp[0] = (-dbH - (b * dbH - 2 * a * dcH) / sD) / (2 * a);
      dp[1] = (-dbC - (b * dbC - 2 * a * dcC) / sD) / (2 * a);
    }
  }
}

// ------------------------------------------- nonlinear temperature conditions
// computeTemperature of the scalar phase diagram (src/phaseDiagram.cpp:225-258
// with computeBoundingEnergy :326-341 and computePorosityMushyLayer :298-324),
// the form MushyLayerParams::computeTemperature (src/MushyLayerParams.cpp:
// 1312-1321) hands to the temperature conditions.  It differs from t_cl in
// rounding: H_s is cp (te + max(0, (-C - CR)/k)), the porosity root has no
// clamp on C, and a NaN enthalpy takes the liquid branch.
__device__ __forceinline__ double temperature_pd(double H, double C, const ClosureParams &p) {
  const double zero = 0.0;
  const double x = (-C - p.CR) / p.k;
  const double Hs = p.cp * (p.te + ((zero < x) ? x : zero));  // std::max(zero, x)
  const double chi = (p.CR + C) / (p.Te + p.CR);
  const double He = chi * (p.St + p.te * (1 - p.cp)) + p.cp * p.te;
  const double Hl = p.St - C + p.te + p.Te;
  if (H <= Hs) return H / p.cp;
  if (H > Hs && H <= He) return p.te;
  if (H > He && H < Hl) {
    double por;
    if (p.St == 0) {
      por = 1;
    } else {
      const double a = p.CR * (p.cp - 1) + p.St * (p.k - 1);
      const double b = p.CR * (1 - 2 * p.cp) + H * (1 - p.k) - C * (p.cp - 1) - p.k * p.St;
      const double c = (C + p.CR) * p.cp + p.k * H;
      por = (-b - sqrt(b * b - 4 * a * c)) / (2 * a);
    }
    return -(C + p.CR * (1 - por)) / (por + p.k * (1 - por));
  }
  return H - p.St;
}

// Resolved temperature conditions: per [dir][side] the Robin coefficients
// (FixedTemperature a = 0, b = 1, T_ref = value; TemperatureFlux a = 1,
// F = value; TemperatureFluxRadiation a, b, T_ref given, F = value;
// BCutil/PhysBCUtil.cpp:614-640) and the solver settings.
struct NLBCD {
  double a[3][2], b[3][2], F[3][2], Tref[3][2], lim[3][2];
  double dx, max_resid, relax;
  int method, max_iter;
};

inline bool is_temperature_bc(int type) {
  return type == MLGPU_BC_FIXED_TEMPERATURE || type == MLGPU_BC_TEMPERATURE_FLUX ||
         type == MLGPU_BC_TEMPERATURE_FLUX_RADIATION;
}

inline NLBCD make_nlbcd(const mlgpu_bc &phi_bc, const mlgpu_nlbc &nb, double grid_dx) {
  NLBCD r;
  for (int d = 0; d < 3; d++)
    for (int s = 0; s < 2; s++) {
      const int type = phi_bc.type[d][s][0];
      const double v = phi_bc.value[d][s][0];
      double a = 0.0, b = 0.0, F = 0.0, T = 0.0;
      if (type == MLGPU_BC_FIXED_TEMPERATURE) {
        b = 1.0;
        T = v;
      } else if (type == MLGPU_BC_TEMPERATURE_FLUX) {
        a = 1.0;
        F = v;
      } else if (type == MLGPU_BC_TEMPERATURE_FLUX_RADIATION) {
        a = nb.a[d][s];
        b = nb.b[d][s];
        F = v;
        T = nb.T_ref[d][s];
      }
      r.a[d][s] = a;
      r.b[d][s] = b;
      r.F[d][s] = F;
      r.Tref[d][s] = T;
      r.lim[d][s] = nb.no_flux_limit[d][s];
    }
  r.dx = nb.dx > 0 ? nb.dx : grid_dx;
  r.max_resid = nb.max_residual;
  r.relax = nb.relax_coeff;
  r.method = nb.method;
  r.max_iter = nb.max_iter;
  return r;
}

// NonlinearTemperatureBCRobin::computeResidual (BCutil/NonlinearBC.H:88-116):
// predicted ghost temperature minus T(H_g, C_g), zeroed beyond 10
__device__ __forceinline__ double nlbc_residual(double pred, double Hg, double Cg,
                                                const ClosureParams &p) {
  double r = pred - temperature_pd(Hg, Cg, p);
  if (fabs(r) > 10.0) r = 0.0;
  return r;
}

// Ghost enthalpy on side s of direction d next to interior cell iv (H_i, C_i)
// (BCutil/PhysBCUtil.cpp:690-722): the interior enthalpy below the no-flux
// limit, else the Picard (NonlinearBC.H:194-233) or Newton (:259-301) root of
// the Robin residual started from H_i, with the ghost concentration taken as
// C_i.  Both loops stop after max_iter further steps.
__device__ __forceinline__ double nlbc_ghost_enthalpy(const NLBCD &B, const ClosureParams &p,
                                                      int dim, int d, int s, const int iv[3],
                                                      double Hi, double Ci) {
  const int perp = (d == dim - 1) ? 0 : d + 1;
  const double face_pos = B.dx * (iv[perp] + 0.5);
  if (face_pos < B.lim[d][s]) return Hi;
  const double Ti = temperature_pd(Hi, Ci, p);
  const double a = B.a[d][s], b = B.b[d][s];
  const double pred = (Ti * a / B.dx + B.F[d][s] + b * Ti / 2 - B.Tref[d][s] * b) / (a / B.dx - b / 2);
  double Hg = Hi;
  if (B.method == MLGPU_NLBC_NEWTON) {
    double dH = 0.01;
    double r_old = B.max_resid * 10;
    for (int it = 0; fabs(r_old) > B.max_resid && it < B.max_iter; it++) {
      r_old = nlbc_residual(pred, Hg, Ci, p);
      const double r_new = nlbc_residual(pred, Hg + dH, Ci, p);
      if (fabs(r_new - r_old) < B.max_resid) {
        Hg = Hg + r_old;
        dH = 2 * dH;
      } else {
        Hg = Hg - r_old * dH / (r_new - r_old);
      }
    }
  } else {
    double r = nlbc_residual(pred, Hg, Ci, p);
    Hg = Hg + B.relax * r;
    for (int it = 0; fabs(r) > B.max_resid && it < B.max_iter; it++) {
      r = nlbc_residual(pred, Hg, Ci, p);
      Hg = Hg + B.relax * r;
    }
  }
  return Hg;
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

// Colour-split index of cell (i, j, k) on a level with an even n0: the cells
// of colour (i + j + k) & 1 fill their own half of the array, row by row
// (each row holds n0 / 2 cells of each colour), so a red/black half sweep
// streams the data of its own colour only.
__device__ __forceinline__ long long cs_index(const Geom &G, int i, int j, int k) {
  return ((i + j + k) & 1) * (G.ncell >> 1) + ((long long)k * G.n1 + j) * (G.n0 >> 1) + (i >> 1);
}

// (i, j, k) of colour-split index t (colour c = t >= n/2) on a level with an
// even n0: the inverse of cs_index
__device__ __forceinline__ void cs_cell(const Geom &G, long long t, int &i, int &j, int &k) {
  const unsigned half = (unsigned)(G.ncell >> 1), h0 = (unsigned)(G.n0 >> 1);
  unsigned u = (unsigned)t;
  const unsigned c = u >= half ? 1u : 0u;
  u -= c * half;
  const unsigned row = u / h0;
  const unsigned kk = row / (unsigned)G.n1;
  j = (int)(row - kk * (unsigned)G.n1);
  k = (int)kk;
  i = 2 * (int)(u - row * h0) + (int)(((unsigned)(j + k) + c) & 1u);
}

// cell-array index functors (natural [k][j][i] order, or colour-split):
// index of a cell, and the cell of an index
struct NaturalIdx {
  __device__ __forceinline__ long long operator()(const Geom &G, int i, int j, int k) const {
    return G.cell(i, j, k);
  }
  static __device__ __forceinline__ void ijk(const Geom &G, long long q, int &i, int &j, int &k) {
    cell_ijk(G, q, i, j, k);
  }
};
struct SplitIdx {
  __device__ __forceinline__ long long operator()(const Geom &G, int i, int j, int k) const {
    return cs_index(G, i, j, k);
  }
  static __device__ __forceinline__ void ijk(const Geom &G, long long q, int &i, int &j, int &k) {
    cs_cell(G, q, i, j, k);
  }
};

__host__ __device__ inline long long colour_threads(const Geom &G) {
  return (long long)((G.n0 + 1) / 2) * G.n1 * G.n2;
}

}  // namespace mlgpu
