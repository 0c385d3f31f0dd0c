// vc_lean_kernels.cuh -- lean kernels of the linear variable-coefficient
// cycles (projection / Darcy-Brinkman operator, vc_kernels.cuh) on 3D levels,
// inside the FP64 defect correction: FP32 in the mixed-precision solve, FP64
// in the comparison path built the same way (options.fuse_levels >= 2).  The
// correction equation L e = r with homogeneous boundary conditions is
//   (L e)_j = diag_j e_j - bd sum_(interior faces) b_f e_nb,   bd = beta / dx^2,
//   diag_j = alpha a_j - beta c_j + bd sum_f b_f fac_f,
// fac_f = 1 for an interior or periodic face, 2 for a Dirichlet wall (ghost
// -e_j), 0 for a Neumann wall (ghost e_j): the wall ghosts fold into the
// diagonal, so a red/black update is an exact Gauss-Seidel step,
//   e_j = (r_j + bd sum b_f e_nb) / diag_j,
// reading its own r and 1/diag, the other colour's e and the face
// coefficients.  The per-level arrays e, r, 1/diag, diag are colour-split
// (cs_index), as in lin_lean_kernels.cuh, so a half sweep streams its own
// colour's data only; the face arrays keep their natural layout.  The
// reference-order kernels (vc_gsrb_kernel with resetLambda's 1/diag, which
// ignores the wall rule) are kept for the FP64 path; this form is the mixed
// path's smoother, its FP64 outer residual unchanged.
#pragma once
#include "vc_kernels.cuh"
#include "misc_kernels.cuh"

namespace mlgpu {

template <class T>
struct VCLeanT {
  Geom G;
  T bd;              // beta / dx^2
  const T *b[3];     // face coefficients (natural face layout)
  const T *idg;      // 1 / diag, split
  const T *dg;       // diag, split
  T *e;              // correction, split
  const T *r;        // right-hand side, split
};
using VCLean = VCLeanT<float>;

#ifdef MLGPU_ADJ_F32_UNIT
// diag and 1/diag of every cell into the split layout (once per solver)
template <class T, int DIM>
__global__ void __launch_bounds__(kBlock) vcl_diag_kernel(VCArgs<T> A, T *__restrict__ idg,
                                                          T *__restrict__ dg) {
  const Geom &G = A.G;
  const T bd = A.beta * A.dxinv;
  for (long long q = gtid(); q < G.ncell; q += gstride()) {
    int i, j, k;
    cell_ijk(G, q, i, j, k);
    const int idx[3] = {i, j, k};
    T s = T(0);
#pragma unroll
    for (int d = 0; d < DIM; d++) {
      const int m = G.n(d);
#pragma unroll
      for (int side = 0; side < 2; side++) {
        int fi[3] = {i, j, k};
        if (side) fi[d] += 1;
        const T bf = A.b[d][G.face(d, fi[0], fi[1], fi[2])];
        const int nb = idx[d] + (side ? 1 : -1);
        T fac;
        if (nb >= 0 && nb < m)
          fac = T(1);
        else if (G.per(d))
          fac = m == 1 ? T(0) : T(1);
        else
          fac = A.bc.type[d][side][0] == MLGPU_BC_DIRICHLET ? T(2) : T(0);
        s = fmaT(bf, fac, s);
      }
    }
    T dv = A.alpha * (A.a ? A.a[q] : T(1));
    if (A.c) dv = dv - A.beta * A.c[q];
    dv = fmaT(bd, s, dv);
    const long long o = cs_index(G, i, j, k);
    dg[o] = dv;
    idg[o] = T(1) / dv;
  }
}

// sum over the interior faces (periodic seams wrapped) of b_f e_nb at cell
// (i, j, k) of a split level
template <class T, int DIM>
__device__ __forceinline__ T vcl_nbsum(const VCLeanT<T> &P, int i, int j, int k) {
  const Geom &G = P.G;
  T s = T(0);
  {
    const long long f = ((long long)k * G.n1 + j) * (G.n0 + 1) + i;
    const int il = i > 0 ? i - 1 : (G.per0 && G.n0 > 1 ? G.n0 - 1 : -1);
    const int ih = i < G.n0 - 1 ? i + 1 : (G.per0 && G.n0 > 1 ? 0 : -1);
    if (il >= 0) s = fmaT(P.b[0][f], P.e[cs_index(G, il, j, k)], s);
    if (ih >= 0) s = fmaT(P.b[0][f + 1], P.e[cs_index(G, ih, j, k)], s);
  }
  {
    const long long f = ((long long)k * (G.n1 + 1) + j) * G.n0 + i;
    const int jl = j > 0 ? j - 1 : (G.per1 && G.n1 > 1 ? G.n1 - 1 : -1);
    const int jh = j < G.n1 - 1 ? j + 1 : (G.per1 && G.n1 > 1 ? 0 : -1);
    if (jl >= 0) s = fmaT(P.b[1][f], P.e[cs_index(G, i, jl, k)], s);
    if (jh >= 0) s = fmaT(P.b[1][f + G.n0], P.e[cs_index(G, i, jh, k)], s);
  }
  if (DIM == 3) {
    const long long pl = (long long)G.n0 * G.n1;
    const long long f = ((long long)k * G.n1 + j) * G.n0 + i;
    const int kl = k > 0 ? k - 1 : (G.per2 && G.n2 > 1 ? G.n2 - 1 : -1);
    const int kh = k < G.n2 - 1 ? k + 1 : (G.per2 && G.n2 > 1 ? 0 : -1);
    if (kl >= 0) s = fmaT(P.b[2][f], P.e[cs_index(G, i, j, kl)], s);
    if (kh >= 0) s = fmaT(P.b[2][f + pl], P.e[cs_index(G, i, j, kh)], s);
  }
  return s;
}

// red/black half sweep over the colour `pass` half; zero: the other colour's
// e is zero (the first half sweep of a correction that starts from zero)
template <class T, int DIM>
__global__ void __launch_bounds__(kBlock) vcl_gsrb_kernel(VCLeanT<T> P, int pass, int zero) {
  const Geom &G = P.G;
  const long long half = G.ncell >> 1;
  for (long long t = gtid(); t < half; t += gstride()) {
    const long long q = pass * half + t;
    int i, j, k;
    cs_cell(G, q, i, j, k);
    const T s = zero ? T(0) : vcl_nbsum<T, DIM>(P, i, j, k);
    P.e[q] = P.idg[q] * fmaT(P.bd, s, P.r[q]);
  }
}

// the same half sweep with V = 16 / sizeof(T) consecutive cells of one row of
// the colour's half per thread (lean_gsrb_vec_kernel's scheme: own r and
// 1/diag, the y / z neighbours' e as 16-byte loads, the x neighbours' e as one
// vector and one scalar, e stored as a vector); each cell's arithmetic in
// vcl_gsrb_kernel's order (the same bits).  Needs n0 / 2 a multiple of V.
// The neighbour sums of the V cells hh .. hh + V - 1 of colour `pass` in
// row `row` = (j, k) of a split level (the other colour's e around them,
// vcl_nbsum's order term by term: the same bits)
template <class T, int DIM>
__device__ __forceinline__ void vcl_vsum(const VCLeanT<T> &P, int pass, unsigned row, int hh,
                                         int j, int k, T *s) {
  constexpr int V = Vec16<T>::V;
  const Geom &G = P.G;
  const long long half = G.ncell >> 1;
  const int h0 = G.n0 >> 1;
  const long long obase = half - pass * half;
  const long long pl = (long long)G.n0 * G.n1;
  const T *e = P.e;
  const int par = (j + k + pass) & 1;
#pragma unroll
  for (int v = 0; v < V; v++) s[v] = T(0);
  {  // x: the other colour's e at hh - 1 + par .. hh + V - 1 + par of this row
    const long long ob = obase + (long long)row * h0;
    T wv[V];
    ldv(e + ob + hh, wv);
    int xe = par ? hh + V : hh - 1;
    bool has_e = true;
    if (xe < 0) {
      xe = h0 - 1;
      has_e = G.per0 != 0;
    } else if (xe >= h0) {
      xe = 0;
      has_e = G.per0 != 0;
    }
    const T ev = has_e ? e[ob + xe] : T(0);
    const long long f0 = (long long)row * (G.n0 + 1) + 2 * hh + par;
#pragma unroll
    for (int v = 0; v < V; v++) {
      const long long f = f0 + 2 * v;
      const int vl = v > 0 ? v - 1 : 0, vh = v < V - 1 ? v + 1 : V - 1;
      const bool lo_e = par == 0 && v == 0;
      if (!lo_e || has_e) s[v] = fmaT(P.b[0][f], lo_e ? ev : (par ? wv[v] : wv[vl]), s[v]);
      const bool hi_e = par == 1 && v == V - 1;
      if (!hi_e || has_e) s[v] = fmaT(P.b[0][f + 1], hi_e ? ev : (par ? wv[vh] : wv[v]), s[v]);
    }
  }
#pragma unroll
  for (int d = 1; d < DIM; d++) {
    const int m = d == 1 ? G.n1 : G.n2, c = d == 1 ? j : k;
    const bool per = d == 1 ? G.per1 != 0 : G.per2 != 0;
    const long long step = d == 1 ? G.n0 : pl;
    const long long fb = d == 1 ? ((long long)k * (G.n1 + 1) + j) * G.n0 + 2 * hh + par
                                : (long long)row * G.n0 + 2 * hh + par;
#pragma unroll
    for (int side = 0; side < 2; side++) {
      int cn = c + (side ? 1 : -1);
      if (cn < 0 || cn >= m) {
        if (!per || m == 1) continue;
        cn = cn < 0 ? m - 1 : 0;
      }
      const unsigned nrow = d == 1 ? (unsigned)k * G.n1 + cn : (unsigned)cn * G.n1 + j;
      T nb[V];
      ldv(e + obase + (long long)nrow * h0 + hh, nb);
#pragma unroll
      for (int v = 0; v < V; v++)
        s[v] = fmaT(P.b[d][fb + 2 * v + (side ? step : 0)], nb[v], s[v]);
    }
  }
}

template <class T, int DIM>
__global__ void __launch_bounds__(kBlock) vcl_gsrb_vec_kernel(VCLeanT<T> P, int pass, int zero) {
  constexpr int V = Vec16<T>::V;
  const Geom &G = P.G;
  const long long half = G.ncell >> 1;
  const int h0 = G.n0 >> 1;
  const long long base = pass * half;
  const long long ngroups = half / V;
  for (long long t = gtid(); t < ngroups; t += gstride()) {
    const long long u = t * V;
    const unsigned row = (unsigned)u / (unsigned)h0;
    const int hh = (int)((unsigned)u - row * (unsigned)h0);
    const int k = (int)(row / (unsigned)G.n1), j = (int)(row - (unsigned)k * G.n1);
    const long long q = base + u;
    T s[V];
#pragma unroll
    for (int v = 0; v < V; v++) s[v] = T(0);
    if (!zero) vcl_vsum<T, DIM>(P, pass, row, hh, j, k, s);
    T r[V], id[V], out[V];
    ldv(P.r + q, r);
    ldv(P.idg + q, id);
#pragma unroll
    for (int v = 0; v < V; v++) out[v] = id[v] * fmaT(P.bd, s[v], r[v]);
    stv(P.e + q, out);
  }
}

// r - L e at a cell of a split level
template <class T, int DIM>
__device__ __forceinline__ T vcl_res(const VCLeanT<T> &P, int i, int j, int k, long long q) {
  return fmaT(P.bd, vcl_nbsum<T, DIM>(P, i, j, k), P.r[q]) - P.dg[q] * P.e[q];
}

// coarse r = 2^D average of the fine residual (RED: of the red children, the
// black ones' being zero to rounding after a black half sweep); coarse e = 0
template <class T, int DIM, class CIDX, bool RED>
__global__ void __launch_bounds__(kBlock) vcl_restrict_kernel(VCLeanT<T> P, Geom C,
                                                              T *__restrict__ rc,
                                                              T *__restrict__ ec) {
  const T wgt = DIM == 3 ? T(0.125) : T(0.25);
  for (long long Q = gtid(); Q < C.ncell; Q += gstride()) {
    int I, J, K;
    cell_ijk(C, Q, I, J, K);
    T a = T(0);
#pragma unroll
    for (int kk = 0; kk < (DIM == 3 ? 2 : 1); kk++)
#pragma unroll
      for (int jj = 0; jj < 2; jj++)
#pragma unroll
        for (int ii = 0; ii < 2; ii++) {
          if (RED && ((ii + jj + kk) & 1)) continue;
          const int i = 2 * I + ii, j = 2 * J + jj, k = DIM == 3 ? 2 * K + kk : 0;
          a += vcl_res<T, DIM>(P, i, j, k, cs_index(P.G, i, j, k));
        }
    const long long o = CIDX()(C, I, J, K);
    rc[o] = a * wgt;
    ec[o] = T(0);
  }
}

// vcl_restrict_kernel (RED) with V coarse cells of a coarse row per thread:
// the red children of coarse cells I0 .. I0 + V - 1 in fine row (2J + jj,
// 2K + kk) are that row's red cells I0 .. I0 + V - 1, one vector group per
// child class (vcl_vsum), summed in the scalar kernel's order (the same bits)
template <class T, int DIM, class CIDX>
__global__ void __launch_bounds__(kBlock) vcl_restrict_vec_kernel(VCLeanT<T> P, Geom C,
                                                                  T *__restrict__ rc,
                                                                  T *__restrict__ ec) {
  constexpr int V = Vec16<T>::V;
  const Geom &G = P.G;
  const int h0 = G.n0 >> 1;
  const long long ngroups = C.ncell / V;
  const T wgt = DIM == 3 ? T(0.125) : T(0.25);
  const CIDX at;
  for (long long t = gtid(); t < ngroups; t += gstride()) {
    const long long U = t * V;
    const unsigned crow = (unsigned)U / (unsigned)C.n0;
    const int I0 = (int)((unsigned)U - crow * (unsigned)C.n0);
    const int K = (int)(crow / (unsigned)C.n1), J = (int)(crow - (unsigned)K * C.n1);
    T a[V];
#pragma unroll
    for (int v = 0; v < V; v++) a[v] = T(0);
#pragma unroll
    for (int kk = 0; kk < (DIM == 3 ? 2 : 1); kk++)
#pragma unroll
      for (int jj = 0; jj < 2; jj++)
#pragma unroll
        for (int ii = 0; ii < 2; ii++) {
          if ((ii + jj + kk) & 1) continue;  // black child
          const int j = 2 * J + jj, k = DIM == 3 ? 2 * K + kk : 0;
          const unsigned row = (unsigned)k * G.n1 + j;
          const long long q = (long long)row * h0 + I0;
          T s[V], r[V], dg[V], e[V];
          vcl_vsum<T, DIM>(P, 0, row, I0, j, k, s);
          ldv(P.r + q, r);
          ldv(P.dg + q, dg);
          ldv(P.e + q, e);
#pragma unroll
          for (int v = 0; v < V; v++) a[v] += fmaT(P.bd, s[v], r[v]) - dg[v] * e[v];
        }
#pragma unroll
    for (int v = 0; v < V; v++) {
      const long long o = at(C, I0 + v, J, K);
      rc[o] = a[v] * wgt;
      ec[o] = T(0);
    }
  }
}

// e += prolongation of the coarse correction (BLACK: the black half alone,
// when a red half sweep follows and overwrites the red e unread)
template <class T, int DIM, int KIND, class CIDX, bool BLACK>
__global__ void __launch_bounds__(kBlock) vcl_prolong_kernel(VCLeanT<T> P, Geom C, BCD bc,
                                                             const T *__restrict__ ec) {
  const Geom &G = P.G;
  const long long n = G.ncell, q0 = BLACK ? (n >> 1) : 0;
  for (long long q = q0 + gtid(); q < n; q += gstride()) {
    int i, j, k;
    cs_cell(G, q, i, j, k);
    P.e[q] = prolong_add<T, DIM, KIND, CIDX>(C, bc, 0, i, j, k, P.e[q], ec, nullptr);
  }
}
// The FP64 outer step of a solve whose level 0 is lean: phi_out = phi + e (e
// split, in the cycles' precision E), r = rhs - L(phi_out) with the operator's
// inhomogeneous boundary conditions, its copy into res_inner (E, split) and
// its norm partials.  vc_update_residual_kernel's quantities in a lean FP64 form (FMA
// differences, the FP32 values widened on the integer pipe, the max norm on
// bit patterns): about half its FP64 pipe operations; the same residual to
// rounding.  e null: the residual of phi itself (no update).  `par` as in
// vc_update_residual_kernel (device ping-pong of phi and out_phi).
template <class E>
__device__ __forceinline__ double widen(E v) {
  if constexpr (sizeof(E) == 4)
    return f64_exact(v);
  else
    return v;
}

template <class E, int DIM, int NORM>
__global__ void __launch_bounds__(kBlock) vcl_outer_kernel(
    VCArgs<double> A, const double *phi, const E *__restrict__ e,
    const double *__restrict__ rhs, double *out_phi, E *__restrict__ res_inner,
    double *__restrict__ part, const int *__restrict__ par) {
  const Geom &G = A.G;
  if (par && *par) {
    double *t = out_phi;
    out_phi = (double *)phi;
    phi = t;
  }
  const double bd = A.beta * A.dxinv;
  double acc = 0.0;
  unsigned long long amax = 0ull;
  for (long long q = gtid(); q < G.ncell; q += gstride()) {
    int i, j, k;
    cell_ijk(G, q, i, j, k);
    const double p0 = e ? phi[q] + widen(e[cs_index(G, i, j, k)]) : phi[q];
    double s = 0.0;
#pragma unroll
    for (int d = 0; d < DIM; d++) {
      const int m = G.n(d);
#pragma unroll
      for (int side = 1; side >= 0; side--) {
        int nb[3] = {i, j, k}, fi[3] = {i, j, k};
        nb[d] += side ? 1 : -1;
        if (side) fi[d] += 1;
        double pn;
        if (nb[d] >= 0 && nb[d] < m) {
          const long long qn = G.cell(nb[0], nb[1], nb[2]);
          pn = e ? phi[qn] + widen(e[cs_index(G, nb[0], nb[1], nb[2])]) : phi[qn];
        } else if (G.per(d)) {
          nb[d] = nb[d] < 0 ? m - 1 : 0;
          const long long qn = G.cell(nb[0], nb[1], nb[2]);
          pn = e ? phi[qn] + widen(e[cs_index(G, nb[0], nb[1], nb[2])]) : phi[qn];
        } else {
          pn = ghost_value<double>(A.bc, d, side, 0, p0, A.dx, false);
        }
        s = fma(A.b[d][G.face(d, fi[0], fi[1], fi[2])], pn - p0, s);
      }
    }
    // rhs - (alpha a p0 - beta c p0 - bd s) as FMAs from rhs
    const double aa = A.a ? A.alpha * A.a[q] : A.alpha;
    double t = fma(-aa, p0, rhs[q]);
    if (A.c) t = fma(A.beta * A.c[q], p0, t);
    const double v = fma(bd, s, t);
    if (e) out_phi[q] = p0;
    res_inner[cs_index(G, i, j, k)] = narrow_to<E>(v);
    if (NORM == MLGPU_NORM_MAX) {
      const unsigned long long bits =
          (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
      amax = bits > amax ? bits : amax;
    } else if (NORM == MLGPU_NORM_L1) {
      acc += fabs(v);
    } else {
      acc = fma(v, v, acc);
    }
  }
  if (NORM == MLGPU_NORM_MAX) acc = __longlong_as_double((long long)amax);
  const double r = block_reduce<NORM>(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = r;
}
#endif  // MLGPU_ADJ_F32_UNIT

}  // namespace mlgpu
