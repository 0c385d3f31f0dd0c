// adjoint_kernels.cuh -- discrete adjoint of the nonlinear (H, C) operator.
//
// N(phi) = alpha a phi - beta div(b grad f(phi)), f = (T, C_l) = closure(H, C)
// (nl_kernels.cuh).  Its Jacobian at a state phi is
//   A x = alpha a x - beta dxinv sum_faces b_f (J_nb x_nb - J x),
// J = d(T, C_l)/d(H, C) per cell (t_cl_jac: the porosity root differentiated
// implicitly), with the ghost of J x taken from the boundary rule of N:
// the derived-variable condition (Dirichlet s = -1, Neumann s = +1 on the
// centre's J x) when it is applied, else the (H, C) condition mapped through
// the ghost state's Jacobian J_g.  The transpose, per cell j, is
//   (A^T y)_j = alpha a_j y_j - beta dxinv (J_j^T w_j + e_j),
//   w_j = sum_interior b_f (y_nb - y_j) + sum_derived b_f (s y_j - y_j)
//         - sum_(H,C)-condition b_f y_j,
//   e_j = sum_(H,C)-condition faces S J_g^T (b_f y_j),   S = diag(s_H, s_C),
// which is what these kernels evaluate: the apply / residual (fused norm),
// a red/black block Gauss-Seidel (the 2x2 diagonal block of A^T inverted per
// cell), the single-CTA bottom relaxation, the restriction of g - A^T y by
// 2^D averaging, and the gradient of -y^T N with respect to the boundary
// values.  The reference has no adjoint: the transposition is of its
// discrete operator, term by term, so A^T is the exact transpose of the
// linearisation of the kernels that compute N.  Temperature conditions on H
// (types 2-4) are not differentiated (the entry points refuse them).
#pragma once
#include "nl_kernels.cuh"
#include "reduce.cuh"

namespace mlgpu {

template <class T>
struct AdjArgs {
  Geom G;
  ClosureParams cp;
  BCD phi_bc;
  DBCD dbc;  // the derived (T, C_l) conditions
  int apply_dbc;
  T alpha, beta, dxinv, dx;
  const T *a;           // [2][cells] or null (a == 1)
  const T *b[3];        // [2][faces_d]
  const T *J;           // [4][cells]: dT/dH, dT/dC, dC_l/dH, dC_l/dC
  const double *u;      // [2][cells] state (ghost Jacobians of the (H, C) condition)
  // [4][cells] inverse of each cell's 2x2 diagonal block M of A^T (row-major;
  // A's block is its transpose), precomputed once per state, or null:
  // the smoother then forms and inverts M inline
  const T *Minv = nullptr;
};

// Jacobian of the closure at the (H, C)-condition ghost of cell q across
// face (d, side): the ghost state by the linear rule, then t_cl_jac
template <class T>
__device__ __forceinline__ void adj_ghost_jac(const AdjArgs<T> &A, long long q, int d, int side,
                                              double Jg[4]) {
  const long long n = A.G.ncell;
  const double hg = ghost_value<double>(A.phi_bc, d, side, 0, A.u[q], A.G.dx, false);
  const double cg = ghost_value<double>(A.phi_bc, d, side, 1, A.u[q + n], A.G.dx, false);
  t_cl_jac(hg, cg, A.cp, Jg);
}

// (A^T y) at interior cell (i,j,k); with WANT_M also the 2x2 diagonal block
// M (row-major, M[2c + c'] = d(A^T y)_c / d y_c') of that cell
template <class T, int DIM, bool WANT_M>
__device__ __forceinline__ void adj_cell(const AdjArgs<T> &A, const T *y, int i, int j, int k,
                                         T out[2], T y0[2], T M[4]) {
  const Geom &G = A.G;
  const long long q = G.cell(i, j, k), n = G.ncell;
  y0[0] = y[q];
  y0[1] = y[q + n];
  T w[2], P[2], ex[2] = {T(0), T(0)}, X[4] = {T(0), T(0), T(0), T(0)};
  bool any_phi = false;
#pragma unroll
  for (int c = 0; c < 2; c++) {
    T s = T(0), p = T(0);
#pragma unroll
    for (int d = 0; d < DIM; d++) {
      const int idx[3] = {i, j, k};
      const int m = G.n(d);
      const long long nf = G.nface(d);
#pragma unroll
      for (int side = 1; side >= 0; side--) {  // high face first, as the forward sum
        int nb[3] = {idx[0], idx[1], idx[2]};
        nb[d] += side ? 1 : -1;
        int fi[3] = {idx[0], idx[1], idx[2]};
        if (side) fi[d] += 1;
        const T bf = A.b[d][c * nf + G.face(d, fi[0], fi[1], fi[2])];
        // t: this face's part of w, b_nb y_nb - b y0 (high side) or
        // b y0 - b_nb y_nb (low side, subtracted), b_nb the coefficient the
        // neighbour's own row uses for the face (different only across a
        // periodic seam, where the forward reads face n for cell n-1 and
        // face 0 for cell 0)
        T t;
        T dp;  // contribution of this face to P_c
        if (nb[d] >= 0 && nb[d] < m) {
          const T yn = y[c * n + G.cell(nb[0], nb[1], nb[2])];
          t = side ? bf * (yn - y0[c]) : bf * (y0[c] - yn);
          dp = bf;
        } else if (G.per(d)) {
          nb[d] = nb[d] < 0 ? m - 1 : 0;
          const long long qn = G.cell(nb[0], nb[1], nb[2]);
          int fs[3] = {idx[0], idx[1], idx[2]};
          fs[d] = side ? 0 : m;
          const T bn = A.b[d][c * nf + G.face(d, fs[0], fs[1], fs[2])];
          const T yn = y[c * n + qn];
          if (qn == q)
            t = T(0);
          else
            t = side ? bn * yn - bf * y0[c] : bf * y0[c] - bn * yn;
          dp = qn == q ? T(0) : bf;
        } else if (A.apply_dbc) {
          const T yn = ghost_value<T>(A.dbc, d, side, c, y0[c], A.dx, true);
          t = side ? bf * (yn - y0[c]) : bf * (y0[c] - yn);
          dp = dbc_wall_diag<T>(A.dbc, d, side, c, bf);
        } else {
          t = side ? bf * (T(0) - y0[c]) : bf * (y0[c] - T(0));
          dp = bf;
          any_phi = true;
        }
        // forward order: + b_hi (y_hi - y0), then - b_lo (y0 - y_lo)
        if (side)
          s = (d == 0) ? t : s + t;
        else
          s = s - t;
        if (WANT_M) p = p + dp;
      }
    }
    w[c] = s;
    P[c] = p;
  }
  if (any_phi) {
    // e_c = sum over (H, C)-condition faces of s_c (J_g^T (b_f y0))_c
#pragma unroll
    for (int d = 0; d < DIM; d++) {
      if (G.per(d)) continue;
      const int idx[3] = {i, j, k};
      const int m = G.n(d);
      const long long nf = G.nface(d);
#pragma unroll
      for (int side = 0; side < 2; side++) {
        if (side ? idx[d] != m - 1 : idx[d] != 0) continue;
        int fi[3] = {idx[0], idx[1], idx[2]};
        if (side) fi[d] += 1;
        const long long f = G.face(d, fi[0], fi[1], fi[2]);
        const T b0 = A.b[d][f], b1 = A.b[d][nf + f];
        double Jg[4];
        adj_ghost_jac(A, q, d, side, Jg);
#pragma unroll
        for (int c = 0; c < 2; c++) {
          const T sc = A.phi_bc.type[d][side][c] == MLGPU_BC_DIRICHLET ? T(-1) : T(1);
          const T g0 = (T)Jg[c], g1 = (T)Jg[2 + c];  // J_g(0, c), J_g(1, c)
          ex[c] = ex[c] + sc * (g0 * (b0 * y0[0]) + g1 * (b1 * y0[1]));
          if (WANT_M) {
            X[2 * c + 0] = X[2 * c + 0] + sc * (g0 * b0);
            X[2 * c + 1] = X[2 * c + 1] + sc * (g1 * b1);
          }
        }
      }
    }
  }
#pragma unroll
  for (int c = 0; c < 2; c++) {
    // (J^T w)_c = J(0, c) w_0 + J(1, c) w_1
    const T j0 = A.J[c * n + q], j1 = A.J[(2 + c) * n + q];
    T t = j0 * w[0] + j1 * w[1];
    if (any_phi) t = t + ex[c];
    const T av = A.a ? A.a[q + c * n] : T(1);
    out[c] = A.alpha * av * y0[c] - A.beta * t * A.dxinv;
    if (WANT_M) {
      // d out_c / d y_c' = delta alpha a_c + beta dxinv (J(c', c) P_c' - X(c, c'))
#pragma unroll
      for (int cp = 0; cp < 2; cp++) {
        const T jcc = A.J[(2 * cp + c) * n + q];
        T v = A.beta * A.dxinv * (jcc * P[cp] - X[2 * c + cp]);
        if (cp == c) v = A.alpha * av + v;
        M[2 * c + cp] = v;
      }
    }
  }
}

// (A x) at interior cell (i,j,k), the linearised operator itself, with its
// 2x2 diagonal block D[2c + c'] = d(A x)_c / d x_c' if asked:
//   (A x)_c = alpha a_c x_c - beta dxinv sum_f b_f,c (g_nb,c - g_c),  g = J x,
// ghosts of g: periodic neighbour, derived-rule ghost of the centre's g, or
// J_g S x under the (H, C) condition;
//   D(c, c') = delta alpha a_c + beta dxinv (P_c J(c, c') - Y(c, c')),
//   Y(c, c') = sum over (H, C)-condition faces of b_f,c J_g(c, c') s_c'.
// It is D^T of adj_cell's M, and the row order of the forward operator's sum.
template <class T, int DIM, bool WANT_M>
__device__ __forceinline__ void lin_cell(const AdjArgs<T> &A, const T *x, int i, int j, int k,
                                         T out[2], T x0[2], T M[4]) {
  const Geom &G = A.G;
  const long long q = G.cell(i, j, k), n = G.ncell;
  x0[0] = x[q];
  x0[1] = x[q + n];
  T g0[2];
#pragma unroll
  for (int c = 0; c < 2; c++) g0[c] = A.J[(2 * c) * n + q] * x0[0] + A.J[(2 * c + 1) * n + q] * x0[1];
  T P[2], Y[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
  for (int c = 0; c < 2; c++) {
    T s = T(0), p = T(0);
#pragma unroll
    for (int d = 0; d < DIM; d++) {
      const int idx[3] = {i, j, k};
      const int m = G.n(d);
      const long long nf = G.nface(d);
#pragma unroll
      for (int side = 1; side >= 0; side--) {
        int nb[3] = {idx[0], idx[1], idx[2]};
        nb[d] += side ? 1 : -1;
        int fi[3] = {idx[0], idx[1], idx[2]};
        if (side) fi[d] += 1;
        const T bf = A.b[d][c * nf + G.face(d, fi[0], fi[1], fi[2])];
        T gn, dp;
        bool self = false;
        if (nb[d] >= 0 && nb[d] < m) {
          const long long qn = G.cell(nb[0], nb[1], nb[2]);
          gn = A.J[(2 * c) * n + qn] * x[qn] + A.J[(2 * c + 1) * n + qn] * x[qn + n];
          dp = bf;
        } else if (G.per(d)) {
          nb[d] = nb[d] < 0 ? m - 1 : 0;
          const long long qn = G.cell(nb[0], nb[1], nb[2]);
          gn = A.J[(2 * c) * n + qn] * x[qn] + A.J[(2 * c + 1) * n + qn] * x[qn + n];
          self = qn == q;
          dp = self ? T(0) : bf;
        } else if (A.apply_dbc) {
          gn = ghost_value<T>(A.dbc, d, side, c, g0[c], A.dx, true);
          dp = dbc_wall_diag<T>(A.dbc, d, side, c, bf);
        } else {
          double Jg[4];
          adj_ghost_jac(A, q, d, side, Jg);
          const T s0 = A.phi_bc.type[d][side][0] == MLGPU_BC_DIRICHLET ? T(-1) : T(1);
          const T s1 = A.phi_bc.type[d][side][1] == MLGPU_BC_DIRICHLET ? T(-1) : T(1);
          const T e0 = s0 * x0[0], e1 = s1 * x0[1];
          gn = (T)Jg[2 * c] * e0 + (T)Jg[2 * c + 1] * e1;
          dp = bf;
          if (WANT_M) {
            Y[2 * c + 0] = Y[2 * c + 0] + bf * ((T)Jg[2 * c] * s0);
            Y[2 * c + 1] = Y[2 * c + 1] + bf * ((T)Jg[2 * c + 1] * s1);
          }
        }
        (void)self;
        const T t = side ? bf * (gn - g0[c]) : bf * (g0[c] - gn);
        if (side)
          s = (d == 0) ? t : s + t;
        else
          s = s - t;
        if (WANT_M) p = p + dp;
      }
    }
    P[c] = p;
    const T av = A.a ? A.a[q + c * n] : T(1);
    out[c] = A.alpha * av * x0[c] - A.beta * s * A.dxinv;
    if (WANT_M) {
#pragma unroll
      for (int cp = 0; cp < 2; cp++) {
        T v = A.beta * A.dxinv * (P[c] * A.J[(2 * c + cp) * n + q] - Y[2 * c + cp]);
        if (cp == c) v = A.alpha * av + v;
        M[2 * c + cp] = v;
      }
    }
  }
}

template <class T, int DIM, bool TR, bool WANT_M>
__device__ __forceinline__ void jac_cell(const AdjArgs<T> &A, const T *y, int i, int j, int k,
                                         T out[2], T y0[2], T M[4]) {
  if (TR)
    adj_cell<T, DIM, WANT_M>(A, y, i, j, k, out, y0, M);
  else
    lin_cell<T, DIM, WANT_M>(A, y, i, j, k, out, y0, M);
}

// y_j += M^-1 (g_j - (B y)_j), B = A^T (TR) or A: the exact solve of cell j's
// two rows
template <class T, int DIM, bool TR = true>
__device__ __forceinline__ void adj_gs_cell(const AdjArgs<T> &A, T *y, const T *g, int i, int j,
                                            int k) {
  if (A.Minv) {
    // stored inverse (of M; the transpose serves A): no block assembly and
    // no division in the sweep
    T out[2], y0[2];
    jac_cell<T, DIM, TR, false>(A, y, i, j, k, out, y0, nullptr);
    const long long q = A.G.cell(i, j, k), n = A.G.ncell;
    const T r0 = g[q] - out[0], r1 = g[q + n] - out[1];
    const T m0 = A.Minv[q], m1 = A.Minv[q + n], m2 = A.Minv[q + 2 * n], m3 = A.Minv[q + 3 * n];
    if (TR) {
      y[q] = y0[0] + (m0 * r0 + m1 * r1);
      y[q + n] = y0[1] + (m2 * r0 + m3 * r1);
    } else {
      y[q] = y0[0] + (m0 * r0 + m2 * r1);
      y[q + n] = y0[1] + (m1 * r0 + m3 * r1);
    }
    return;
  }
  T out[2], y0[2], M[4];
  jac_cell<T, DIM, TR, true>(A, y, i, j, k, out, y0, M);
  const long long q = A.G.cell(i, j, k), n = A.G.ncell;
  const T r0 = g[q] - out[0], r1 = g[q + n] - out[1];
  const T det = M[0] * M[3] - M[1] * M[2];
  y[q] = y0[0] + (M[3] * r0 - M[1] * r1) / det;
  y[q + n] = y0[1] + (M[0] * r1 - M[2] * r0) / det;
}

enum { ADJ_APPLY = 0, ADJ_RESIDUAL = 1 };
// bottom levels with at most this many unknowns (2 per cell) are solved
// exactly (adj_bottom_direct_kernel)
constexpr int kAdjDirectMax = 32;

#ifdef MLGPU_ADJ_UNIT  // kernels compiled in launch_f64_adj.cu only
// closure Jacobian of every cell, evaluated in the kernels' precision (FP32:
// t_cl's regime, the derivative at the FP32-rounded state)
template <class T>
__global__ void __launch_bounds__(kBlock) adj_jac_kernel(Geom G, ClosureParams cp,
                                                         const double *__restrict__ u,
                                                         T *__restrict__ J) {
  const long long n = G.ncell;
  const ClosureF32 f = make_closure_f32(cp);
  for (long long q = gtid(); q < n; q += gstride()) {
    T j4[4];
    if constexpr (sizeof(T) == 4)
      t_cl_jac32(u[q], u[q + n], cp, f, j4);
    else
      t_cl_jac(u[q], u[q + n], cp, j4);
#pragma unroll
    for (int m = 0; m < 4; m++) J[q + m * n] = j4[m];
  }
}

#ifndef MLGPU_ADJ_F32_UNIT  // FP64 unit only (launch_f32_adj.cu instantiates the FP32 cycles)
// {d por/dH, d por/dC} of every cell
__global__ void __launch_bounds__(kBlock) porosity_jac_kernel(Geom G, ClosureParams cp,
                                                              const double *__restrict__ u,
                                                              double *__restrict__ dp) {
  const long long n = G.ncell;
  for (long long q = gtid(); q < n; q += gstride()) {
    double d2[2];
    porosity_jac(u[q], u[q + n], cp, d2);
    dp[q] = d2[0];
    dp[q + n] = d2[1];
  }
}
#endif

// the inverse of every cell's diagonal block M of A^T: {M3, -M1, -M2, M0}/det;
// with Dout also A's own block D = M^T (the lean FP32 cycles' residual)
template <class T, int DIM>
__global__ void __launch_bounds__(kBlock) adj_minv_kernel(AdjArgs<T> A, const T *__restrict__ zero,
                                                          T *__restrict__ Minv,
                                                          T *__restrict__ Dout) {
  const Geom &G = A.G;
  const long long n = G.ncell;
  for (long long q = gtid(); q < n; q += gstride()) {
    int i, j, k;
    cell_ijk(G, q, i, j, k);
    T out[2], y0[2], M[4];
    adj_cell<T, DIM, true>(A, zero, i, j, k, out, y0, M);
    const T det = M[0] * M[3] - M[1] * M[2];
    Minv[q] = M[3] / det;
    Minv[q + n] = -M[1] / det;
    Minv[q + 2 * n] = -M[2] / det;
    Minv[q + 3 * n] = M[0] / det;
    if (Dout) {
      Dout[q] = M[0];
      Dout[q + n] = M[2];
      Dout[q + 2 * n] = M[1];
      Dout[q + 3 * n] = M[3];
    }
  }
}

// out = A^T y (ADJ_APPLY) or g - A^T y with a fused norm (ADJ_RESIDUAL)
template <class T, int DIM, int MODE, int NORM, bool TR>
__global__ void __launch_bounds__(kBlock) adj_op_kernel(AdjArgs<T> A, const T *__restrict__ y,
                                                        const T *__restrict__ g,
                                                        T *__restrict__ out,
                                                        double *__restrict__ part) {
  const Geom &G = A.G;
  double acc = 0.0;
  for (long long q = gtid(); q < G.ncell; q += gstride()) {
    int i, j, k;
    cell_ijk(G, q, i, j, k);
    T o[2], y0[2];
    jac_cell<T, DIM, TR, false>(A, y, i, j, k, o, y0, nullptr);
#pragma unroll
    for (int c = 0; c < 2; c++) {
      const long long qc = q + c * G.ncell;
      const T v = MODE == ADJ_RESIDUAL ? g[qc] - o[c] : o[c];
      out[qc] = v;
      if (NORM >= 0) acc = norm_accum<NORM < 0 ? 0 : NORM>(acc, (double)v);
    }
  }
  if (NORM >= 0) {
    double r = block_reduce<NORM < 0 ? 0 : NORM>(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = r;
  }
}

template <class T, int DIM, bool TR>
__global__ void __launch_bounds__(kBlock) adj_gsrb_kernel(AdjArgs<T> A, T *y,
                                                          const T *__restrict__ g, int pass) {
  const long long nt = colour_threads(A.G);
  for (long long t = gtid(); t < nt; t += gstride()) {
    int i, j, k;
    if (colour_cell(A.G, pass, t, i, j, k)) adj_gs_cell<T, DIM, TR>(A, y, g, i, j, k);
  }
}

// bottom: y = 0 (if zero), then `sweeps` red/black sweeps in one block
template <class T, int DIM, bool TR>
__global__ void __launch_bounds__(1024) adj_relax_block_kernel(AdjArgs<T> A, T *y,
                                                               const T *__restrict__ g,
                                                               int sweeps, int zero) {
  const long long n = A.G.ncell;
  if (zero) {
    for (long long q = threadIdx.x; q < 2 * n; q += blockDim.x) y[q] = T(0);
    __syncthreads();
  }
  const long long nt = colour_threads(A.G);
  for (int s = 0; s < sweeps; s++)
    for (int pass = 0; pass < 2; pass++) {
      for (long long t = threadIdx.x; t < nt; t += blockDim.x) {
        int i, j, k;
        if (colour_cell(A.G, pass, t, i, j, k)) adj_gs_cell<T, DIM, TR>(A, y, g, i, j, k);
      }
      __syncthreads();
    }
}

// Exact bottom solve of B y = g (B = A^T or A) when the level has at most
// kAdjDirectMax unknowns: thread k evaluates column k of B as B e_k, cell by
// cell, into the augmented matrix; Gaussian elimination with partial
// pivoting (the first row of largest |pivot|), then back substitution by
// thread 0.  A relaxation bottom of these tiny levels is a chain of ~80
// dependent FP64 phases (0.5 ms for 40 sweeps on 2x2 cells).
template <class T, int DIM, bool TR>
__global__ void __launch_bounds__(kAdjDirectMax) adj_bottom_direct_kernel(
    AdjArgs<T> A, T *__restrict__ y, const T *__restrict__ g) {
  __shared__ T M[kAdjDirectMax][kAdjDirectMax + 1];
  __shared__ T unit[kAdjDirectMax][kAdjDirectMax];
  __shared__ int piv;
  const long long nc = A.G.ncell;
  const int n = (int)(2 * nc);
  const int k = threadIdx.x;
  if (k < n) {
    for (int m = 0; m < n; m++) unit[k][m] = T(0);
    unit[k][k] = T(1);
    for (long long q = 0; q < nc; q++) {
      int i, j, kk;
      cell_ijk(A.G, q, i, j, kk);
      T o[2], y0[2];
      jac_cell<T, DIM, TR, false>(A, unit[k], i, j, kk, o, y0, nullptr);
      M[q][k] = o[0];
      M[q + nc][k] = o[1];
    }
    M[k][n] = g[k];
  }
  __syncthreads();
  for (int p = 0; p < n; p++) {
    if (k == 0) {
      int best = p;
      T bv = fabs(M[p][p]);
      for (int r = p + 1; r < n; r++) {
        const T v = fabs(M[r][p]);
        if (v > bv) {
          bv = v;
          best = r;
        }
      }
      piv = best;
    }
    __syncthreads();
    const int pr = piv;
    if (pr != p)
      for (int col = k; col <= n; col += blockDim.x) {
        const T t = M[p][col];
        M[p][col] = M[pr][col];
        M[pr][col] = t;
      }
    __syncthreads();
    for (int r = p + 1 + k; r < n; r += blockDim.x) {
      const T l = M[r][p] / M[p][p];
      for (int col = p; col <= n; col++) M[r][col] = M[r][col] - l * M[p][col];
    }
    __syncthreads();
  }
  if (k == 0)
    for (int r = n - 1; r >= 0; r--) {
      T s = M[r][n];
      for (int col = r + 1; col < n; col++) s = s - M[r][col] * y[col];
      y[r] = s / M[r][r];
    }
}

// coarse right-hand side: the 2^D average of g - A^T y
template <class T, int DIM, bool TR>
__global__ void __launch_bounds__(kBlock) adj_restrict_kernel(AdjArgs<T> A, Geom C,
                                                              const T *__restrict__ y,
                                                              const T *__restrict__ g,
                                                              T *__restrict__ gc) {
  const Geom &G = A.G;
  const T denom = DIM == 3 ? T(8) : T(4);
  for (long long Q = gtid(); Q < C.ncell; Q += gstride()) {
    int I, J, K;
    cell_ijk(C, Q, I, J, K);
    T acc[2] = {T(0), T(0)};
#pragma unroll
    for (int kk = 0; kk < (DIM == 3 ? 2 : 1); kk++)
#pragma unroll
      for (int jj = 0; jj < 2; jj++)
#pragma unroll
        for (int ii = 0; ii < 2; ii++) {
          const int i = 2 * I + ii, j = 2 * J + jj, k = DIM == 3 ? 2 * K + kk : 0;
          T o[2], y0[2];
          jac_cell<T, DIM, TR, false>(A, y, i, j, k, o, y0, nullptr);
          const long long q = G.cell(i, j, k);
#pragma unroll
          for (int c = 0; c < 2; c++) acc[c] = acc[c] + (g[q + c * G.ncell] - o[c]) / denom;
        }
    gc[Q] = acc[0];
    gc[Q + C.ncell] = acc[1];
  }
}

// Gradient of -y^T N with respect to the boundary values: one block per
// (direction, side), out[(d * 2 + side) * 2 + c].  Derived condition applied:
// d f_g,c / d v_c = 2 (Dirichlet) or s dx (Neumann), so the entry is
// beta dxinv sum y_c b_c df; otherwise the (H, C) condition's value moves
// phi_g,c and f_g through J_g: beta dxinv dphi sum_c' y_c' b_c' J_g(c', c).
template <class T, int DIM>
__global__ void __launch_bounds__(kBlock) adj_bc_grad_kernel(AdjArgs<T> A,
                                                             const T *__restrict__ y,
                                                             double *__restrict__ out) {
  const Geom &G = A.G;
  const int d = blockIdx.x >> 1, side = blockIdx.x & 1;
  double acc[2] = {0.0, 0.0};
  if (d < DIM && !G.per(d)) {
    const int m0 = d == 0 ? G.n1 : G.n0;
    const int m1 = d == 2 ? G.n1 : G.n2;
    const long long nf = G.nface(d), n = G.ncell;
    const long long tot = (long long)m0 * m1;
    for (long long t = threadIdx.x; t < tot; t += blockDim.x) {
      const int a0 = (int)(t % m0), a1 = (int)(t / m0);
      int idx[3];
      idx[d] = side ? G.n(d) - 1 : 0;
      if (d == 0) { idx[1] = a0; idx[2] = a1; }
      if (d == 1) { idx[0] = a0; idx[2] = a1; }
      if (d == 2) { idx[0] = a0; idx[1] = a1; }
      const long long q = G.cell(idx[0], idx[1], idx[2]);
      int fi[3] = {idx[0], idx[1], idx[2]};
      if (side) fi[d] += 1;
      const long long f = G.face(d, fi[0], fi[1], fi[2]);
      const double yb0 = (double)y[q] * (double)A.b[d][f];
      const double yb1 = (double)y[q + n] * (double)A.b[d][nf + f];
      if (A.apply_dbc) {
        acc[0] += yb0;
        acc[1] += yb1;
      } else {
        double Jg[4];
        adj_ghost_jac(A, q, d, side, Jg);
        acc[0] += yb0 * Jg[0] + yb1 * Jg[2];
        acc[1] += yb0 * Jg[1] + yb1 * Jg[3];
      }
    }
  }
  const double s0 = block_reduce<2>(acc[0]);
  __syncthreads();
  const double s1 = block_reduce<2>(acc[1]);
  if (threadIdx.x == 0) {
    const BCD &bc = A.apply_dbc ? A.dbc : A.phi_bc;
    const double isign = side ? 1.0 : -1.0;
    for (int c = 0; c < 2; c++) {
      double v = 0.0;
      if (d < DIM && !G.per(d)) {
        // d(ghost)/d(value): 2 Dirichlet, +-dx Neumann, 1 / p2 mixed
        const double df = bc.type[d][side][c] == MLGPU_BC_DIRICHLET ? 2.0
                          : (A.apply_dbc && bc.type[d][side][c] == MLGPU_BC_MIXED_TEMPERATURE_SALINITY)
                              ? A.dbc.rob[d][side][4]
                              : isign * (double)A.dx;
        v = (double)A.beta * (double)A.dxinv * df * (c == 0 ? s0 : s1);
      }
      out[blockIdx.x * 2 + c] = v;
    }
  }
}
#endif

}  // namespace mlgpu
