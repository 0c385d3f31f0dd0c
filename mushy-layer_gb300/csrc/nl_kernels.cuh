// nl_kernels.cuh -- sm_103a kernels of the nonlinear enthalpy/bulk
// concentration operator (AMRNonLinearMultiCompOp):
//   L(phi) = alpha a phi - beta div(b grad f(phi)),  phi = (H, C), f = (T, C_l).
//
// The diffused variable f(phi) is never stored.  Each stencil evaluates the
// FP64 closure of its centre and of its 2*DIM neighbours in registers; at a
// physical boundary the neighbour value comes from the derived-variable BC
// applied to the centre's (T, C_l) (AMRNonLinearMultiCompOp.cpp:93-97), in a
// periodic direction from the wrapped cell.  Arithmetic follows the Fortran
// evaluation order of NLVCCOMPUTEOP/NLVCCOMPUTERES/NONLINEARSMOOTHING/
// RESTRICTRESNLVC (src/AMRNonLinearMultiCompOpF.ChF) so the FP64 build is
// bitwise equal to a ghost-filled CPU evaluation.
#pragma once
#include "common.cuh"
#include "reduce.cuh"

namespace mlgpu {

template <class T>
struct NLArgs {
  Geom G;
  ClosureParams cp;
  BCD phi_bc;
  DBCD dbc;  // the derived (T, C_l) conditions
  NLBCD nlbc;       // temperature conditions on H (phi_bc comp 0 types 2-4)
  int apply_dbc;
  T alpha, beta, dxinv, dx;
  const T *a;       // [2][cells] or null (a == 1)
  const T *b[3];    // [2][faces_d]
};

// Enthalpy ghost value across face (d, side) of interior cell (i,j,k):
// the temperature condition's root where phi_bc comp 0 has one, else the
// linear rule.
template <class T>
__device__ __forceinline__ double nl_ghost_h(const NLArgs<T> &A, int i, int j, int k, int d,
                                             int side, double h0, double c0) {
  if (A.phi_bc.type[d][side][0] >= MLGPU_BC_FIXED_TEMPERATURE) {
    const int iv[3] = {i, j, k};
    return nlbc_ghost_enthalpy(A.nlbc, A.cp, A.G.dim, d, side, iv, h0, c0);
  }
  return ghost_value<double>(A.phi_bc, d, side, 0, h0, (double)A.dx, false);
}

// Diffused variable (T, C_l) of cell (i,j,k), which must be interior.
template <class T>
__device__ __forceinline__ void nl_dv(const NLArgs<T> &A, const T *phi, int i,
                                      int j, int k, T &t, T &cl) {
  long long q = A.G.cell(i, j, k);
  double Td, Cd;
  t_cl((double)phi[q], (double)phi[q + A.G.ncell], A.cp, Td, Cd);
  t = (T)Td;
  cl = (T)Cd;
}

// Diffused variable at neighbour (i,j,k) + s e_d of an interior cell whose
// own (H, C) and (T, C_l) are h0, c0, t0, l0.
template <class T>
__device__ __forceinline__ void nl_dv_nb(const NLArgs<T> &A, const T *phi, int i,
                                         int j, int k, int d, int side, T h0, T c0, T t0, T l0,
                                         T &t, T &cl) {
  int idx[3] = {i, j, k};
  int m = A.G.n(d);
  idx[d] += side ? 1 : -1;
  if (idx[d] >= 0 && idx[d] < m) {
    nl_dv(A, phi, idx[0], idx[1], idx[2], t, cl);
    return;
  }
  if (A.G.per(d)) {
    idx[d] = idx[d] < 0 ? m - 1 : 0;
    nl_dv(A, phi, idx[0], idx[1], idx[2], t, cl);
    return;
  }
  if (A.apply_dbc) {
    t = ghost_value<T>(A.dbc, d, side, 0, t0, A.dx, false);
    cl = ghost_value<T>(A.dbc, d, side, 1, l0, A.dx, false);
    return;
  }
  T hg = A.phi_bc.type[d][side][0] >= MLGPU_BC_FIXED_TEMPERATURE
             ? (T)nl_ghost_h(A, i, j, k, d, side, (double)h0, (double)c0)
             : ghost_value<T>(A.phi_bc, d, side, 0, h0, A.dx, false);
  T cg = ghost_value<T>(A.phi_bc, d, side, 1, c0, A.dx, false);
  double Td, Cd;
  t_cl((double)hg, (double)cg, A.cp, Td, Cd);
  t = (T)Td;
  cl = (T)Cd;
}

// Face coefficient (comp c) of face (i,j,k) in direction d.
template <class T>
__device__ __forceinline__ T bface(const NLArgs<T> &A, int d, int c, int i, int j, int k) {
  return A.b[d][c * A.G.nface(d) + A.G.face(d, i, j, k)];
}

// L(phi) for both components at interior cell (i,j,k).  Also returns the
// inline relaxation coefficient lambda (resetLambda order) when asked.
template <class T, int DIM, bool WANT_LAMBDA>
__device__ __forceinline__ void nl_lofphi(const NLArgs<T> &A, const T *phi, int i,
                                          int j, int k, T lof[2], T lam[2], T ph[2]) {
  const Geom &G = A.G;
  long long q = G.cell(i, j, k);
  T h0 = phi[q], c0 = phi[q + G.ncell];
  ph[0] = h0;
  ph[1] = c0;
  T pl0[2];
  {
    double Td, Cd;
    t_cl((double)h0, (double)c0, A.cp, Td, Cd);
    pl0[0] = (T)Td;
    pl0[1] = (T)Cd;
  }
  T lo[3][2], hi[3][2];
#pragma unroll
  for (int d = 0; d < DIM; d++) {
    nl_dv_nb(A, phi, i, j, k, d, 0, h0, c0, pl0[0], pl0[1], lo[d][0], lo[d][1]);
    nl_dv_nb(A, phi, i, j, k, d, 1, h0, c0, pl0[0], pl0[1], hi[d][0], hi[d][1]);
  }
#pragma unroll
  for (int c = 0; c < 2; c++) {
    T p0 = pl0[c];
    T bxh = bface(A, 0, c, i + 1, j, k), bxl = bface(A, 0, c, i, j, k);
    T byh = bface(A, 1, c, i, j + 1, k), byl = bface(A, 1, c, i, j, k);
    T s = bxh * (hi[0][c] - p0) - bxl * (p0 - lo[0][c]);
    s = s + byh * (hi[1][c] - p0);
    s = s - byl * (p0 - lo[1][c]);
    T bzh = T(0), bzl = T(0);
    if (DIM == 3) {
      bzh = bface(A, 2, c, i, j, k + 1);
      bzl = bface(A, 2, c, i, j, k);
      s = s + bzh * (hi[2][c] - p0);
      s = s - bzl * (p0 - lo[2][c]);
    }
    T av = A.a ? A.a[q + c * G.ncell] : T(1);
    lof[c] = A.alpha * av * ph[c] - A.beta * s * A.dxinv;
    if (WANT_LAMBDA) {
      T l = av * A.alpha;
      l = l + A.dxinv * A.beta * (bxh + bxl);
      l = l + A.dxinv * A.beta * (byh + byl);
      if (DIM == 3) l = l + A.dxinv * A.beta * (bzh + bzl);
      lam[c] = T(1) / l;
    }
  }
}

enum { NL_RESIDUAL = 0, NL_APPLY = 1, NL_APPLY_PLUS = 2, NL_JACOBI = 3 };

// Pointwise operator kernels:
//   NL_RESIDUAL   out = rhs - L(phi)
//   NL_APPLY      out = L(phi)
//   NL_APPLY_PLUS out = L(phi) + rhs, and copy = phi  (FAS coarse rhs + saved u)
//   NL_JACOBI     out = phi + 0.5 (r lambda)          (levelJacobi)
// NORM >= 0 adds a fused block reduction of `out` (residual mode) into part[].
template <class T, int DIM, int MODE, int NORM>
__global__ void __launch_bounds__(kBlock) nl_op_kernel(NLArgs<T> A, const T *__restrict__ phi,
                                                       const T *__restrict__ rhs,
                                                       T *__restrict__ out,
                                                       T *__restrict__ copy,
                                                       double *__restrict__ part) {
  const Geom &G = A.G;
  double acc = 0.0;
  for (long long q = gtid(); q < G.ncell; q += gstride()) {
    int i, j, k;
    cell_ijk(G, q, i, j, k);
    T lof[2], lam[2], ph[2];
    nl_lofphi<T, DIM, MODE == NL_JACOBI>(A, phi, i, j, k, lof, lam, ph);
#pragma unroll
    for (int c = 0; c < 2; c++) {
      long long qc = q + c * G.ncell;
      T v;
      if (MODE == NL_RESIDUAL) {
        v = rhs[qc] - lof[c];
      } else if (MODE == NL_APPLY) {
        v = lof[c];
      } else if (MODE == NL_APPLY_PLUS) {
        v = lof[c] + rhs[qc];
        copy[qc] = ph[c];
      } else {
        T r = rhs[qc] - lof[c];
        v = ph[c] + T(0.5) * (r * lam[c]);
      }
      out[qc] = v;
      if (NORM >= 0) acc = norm_accum<NORM < 0 ? 0 : NORM>(acc, (double)v);
    }
  }
  if (NORM >= 0) {
    double r = block_reduce<NORM < 0 ? 0 : NORM>(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = r;
  }
}

// One cell of a red/black pass (NONLINEARSMOOTHING).
template <class T, int DIM>
__device__ __forceinline__ void nl_gsrb_cell(const NLArgs<T> &A, T *phi,
                                             const T *__restrict__ rhs, int i, int j, int k) {
  T lof[2], lam[2], ph[2];
  nl_lofphi<T, DIM, true>(A, phi, i, j, k, lof, lam, ph);
  long long q = A.G.cell(i, j, k);
#pragma unroll
  for (int c = 0; c < 2; c++) {
    long long qc = q + c * A.G.ncell;
    phi[qc] = ph[c] - lam[c] * (lof[c] - rhs[qc]);
  }
}

template <class T, int DIM>
__global__ void __launch_bounds__(kBlock) nl_gsrb_kernel(NLArgs<T> A, T *phi,
                                                         const T *__restrict__ rhs, int pass) {
  long long nt = colour_threads(A.G);
  for (long long t = gtid(); t < nt; t += gstride()) {
    int i, j, k;
    if (colour_cell(A.G, pass, t, i, j, k)) nl_gsrb_cell<T, DIM>(A, phi, rhs, i, j, k);
  }
}

// Whole relaxation (n red+black sweeps) inside one thread block: used for the
// bottom solve of tiny coarsest levels, where a launch per half sweep would
// cost more than the arithmetic.
template <class T, int DIM>
__global__ void __launch_bounds__(1024) nl_relax_block_kernel(NLArgs<T> A, T *phi,
                                                              const T *__restrict__ rhs,
                                                              int sweeps) {
  long long nt = colour_threads(A.G);
  for (int s = 0; s < sweeps; s++) {
    for (int pass = 0; pass < 2; pass++) {
      for (long long t = threadIdx.x; t < nt; t += blockDim.x) {
        int i, j, k;
        if (colour_cell(A.G, pass, t, i, j, k)) nl_gsrb_cell<T, DIM>(A, phi, rhs, i, j, k);
      }
      __syncthreads();
    }
  }
}

// FAS restriction (RESTRICTRESNLVC, F.ChF:465-542), optionally fused with
// restrictR (RESTRICT, F.ChF:555-585): one thread per coarse cell, the 2^D
// fine contributions accumulated in the Fortran loop order.
template <class T, int DIM>
__global__ void __launch_bounds__(kBlock) nl_restrict_kernel(NLArgs<T> A, Geom C,
                                                             const T *__restrict__ phi,
                                                             const T *__restrict__ rhs,
                                                             T *__restrict__ res_c,
                                                             T *__restrict__ phi_c) {
  const Geom &G = A.G;
  const T denom = DIM == 3 ? T(8) : T(4);
  for (long long Q = gtid(); Q < C.ncell; Q += gstride()) {
    int I, J, K;
    cell_ijk(C, Q, I, J, K);
    T acc[2] = {T(0), T(0)}, avg[2] = {T(0), T(0)};
#pragma unroll
    for (int kk = 0; kk < (DIM == 3 ? 2 : 1); kk++)
#pragma unroll
      for (int jj = 0; jj < 2; jj++)
#pragma unroll
        for (int ii = 0; ii < 2; ii++) {
          int i = 2 * I + ii, j = 2 * J + jj, k = DIM == 3 ? 2 * K + kk : 0;
          T lof[2], lam[2], ph[2];
          nl_lofphi<T, DIM, false>(A, phi, i, j, k, lof, lam, ph);
          long long q = G.cell(i, j, k);
#pragma unroll
          for (int c = 0; c < 2; c++) {
            acc[c] = acc[c] + (rhs[q + c * G.ncell] - lof[c]) / denom;
            avg[c] = avg[c] + ph[c] / denom;
          }
        }
#pragma unroll
    for (int c = 0; c < 2; c++) {
      res_c[Q + c * C.ncell] = acc[c];
      if (phi_c) phi_c[Q + c * C.ncell] = avg[c];
    }
  }
}

template <class T, int DIM>
__global__ void __launch_bounds__(kBlock) nl_lambda_kernel(NLArgs<T> A, T *__restrict__ lam) {
  const Geom &G = A.G;
  for (long long q = gtid(); q < G.ncell; q += gstride()) {
    int i, j, k;
    cell_ijk(G, q, i, j, k);
#pragma unroll
    for (int c = 0; c < 2; c++) {
      T av = A.a ? A.a[q + c * G.ncell] : T(1);
      T l = av * A.alpha;
      l = l + A.dxinv * A.beta * (bface(A, 0, c, i + 1, j, k) + bface(A, 0, c, i, j, k));
      l = l + A.dxinv * A.beta * (bface(A, 1, c, i, j + 1, k) + bface(A, 1, c, i, j, k));
      if (DIM == 3)
        l = l + A.dxinv * A.beta * (bface(A, 2, c, i, j, k + 1) + bface(A, 2, c, i, j, k));
      lam[q + c * G.ncell] = T(1) / l;
    }
  }
}

}  // namespace mlgpu
