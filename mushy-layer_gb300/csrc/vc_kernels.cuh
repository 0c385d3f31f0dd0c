// vc_kernels.cuh -- sm_103a kernels of the linear variable-coefficient
// operator of one component
//   L(phi) = alpha a phi - beta c phi - beta div(b grad phi)
// c == null: projection operator (AMRProjectionOp / VCAMRPoissonOp2);
// c != null: DarcyBrinkmanOp (src/DarcyBrinkmanOpF.ChF).  Ghost values are
// formed in registers from the adjacent interior cell.  FP64 arithmetic
// follows DBCOMPUTEOP/DBCOMPUTERES/GSRBHELMHOLTZDB/RESTRICTRESDB order.
#pragma once
#include "common.cuh"
#include "reduce.cuh"

namespace mlgpu {

template <class T>
struct VCArgs {
  Geom G;
  BCD bc;
  T alpha, beta, dxinv, dx;
  const T *a;     // [cells] or null (a == 1)
  const T *c;     // [cells] or null (c == 0)
  const T *b[3];  // [faces_d]
  const T *lam;   // stored 1/diag (resetLambda) or null: computed inline
};

// 1/diag(L) at cell q in resetLambda order (DarcyBrinkmanOp.cpp:265-296):
// a*alpha, + (-beta) c, + sum_d scale*beta*(b_hi + b_lo), then 1/x.
template <class T, int DIM>
__device__ __forceinline__ T vc_lambda_at(const VCArgs<T> &A, long long q, T bxh, T bxl, T byh,
                                          T byl, T bzh, T bzl) {
  if (A.lam) return A.lam[q];
  T av = A.a ? A.a[q] : T(1);
  T l = av * A.alpha;
  if (A.c) l = l + (-A.beta) * A.c[q];
  l = l + A.dxinv * A.beta * (bxh + bxl);
  l = l + A.dxinv * A.beta * (byh + byl);
  if (DIM == 3) l = l + A.dxinv * A.beta * (bzh + bzl);
  return T(1) / l;
}

// Reads phi at a cell; the "update" form returns phi + e (FP64 phi, any e)
// so an outer defect-correction step can apply its correction on the fly.
template <class T>
struct PlainRead {
  const T *phi;
  __device__ __forceinline__ T operator()(long long q) const { return phi[q]; }
};
template <class T, class E>
struct UpdateRead {
  const T *phi;
  const E *e;
  __device__ __forceinline__ T operator()(long long q) const { return phi[q] + (T)e[q]; }
};

template <class T, class R>
__device__ __forceinline__ T vc_nb(const VCArgs<T> &A, const R &rd, int i, int j, int k, int d,
                                   int side, T p0, bool homog) {
  int idx[3] = {i, j, k};
  int m = A.G.n(d);
  idx[d] += side ? 1 : -1;
  if (idx[d] >= 0 && idx[d] < m) return rd(A.G.cell(idx[0], idx[1], idx[2]));
  if (A.G.per(d)) {
    idx[d] = idx[d] < 0 ? m - 1 : 0;
    return rd(A.G.cell(idx[0], idx[1], idx[2]));
  }
  return ghost_value<T>(A.bc, d, side, 0, p0, A.dx, homog);
}

template <class T>
__device__ __forceinline__ T vface(const VCArgs<T> &A, int d, int i, int j, int k) {
  return A.b[d][A.G.face(d, i, j, k)];
}

template <class T, int DIM, bool WANT_LAMBDA, class R>
__device__ __forceinline__ T vc_lofphi(const VCArgs<T> &A, const R &rd, int i, int j, int k,
                                       bool homog, T &p0, T &lam) {
  const Geom &G = A.G;
  long long q = G.cell(i, j, k);
  p0 = rd(q);
  T lo[3], hi[3];
#pragma unroll
  for (int d = 0; d < DIM; d++) {
    lo[d] = vc_nb(A, rd, i, j, k, d, 0, p0, homog);
    hi[d] = vc_nb(A, rd, i, j, k, d, 1, p0, homog);
  }
  T bxh = vface(A, 0, i + 1, j, k), bxl = vface(A, 0, i, j, k);
  T byh = vface(A, 1, i, j + 1, k), byl = vface(A, 1, i, j, k);
  T s = bxh * (hi[0] - p0) - bxl * (p0 - lo[0]);
  s = s + byh * (hi[1] - p0);
  s = s - byl * (p0 - lo[1]);
  T bzh = T(0), bzl = T(0);
  if (DIM == 3) {
    bzh = vface(A, 2, i, j, k + 1);
    bzl = vface(A, 2, i, j, k);
    s = s + bzh * (hi[2] - p0);
    s = s - bzl * (p0 - lo[2]);
  }
  T av = A.a ? A.a[q] : T(1);
  T v = A.alpha * av * p0;
  if (A.c) v = v - A.beta * A.c[q] * p0;
  v = v - A.beta * s * A.dxinv;
  if (WANT_LAMBDA) lam = vc_lambda_at<T, DIM>(A, q, bxh, bxl, byh, byl, bzh, bzl);
  return v;
}

enum { VC_RESIDUAL = 0, VC_APPLY = 1, VC_JACOBI = 2 };

template <class T, int DIM, int MODE, int NORM>
__global__ void __launch_bounds__(kBlock) vc_op_kernel(VCArgs<T> A, const T *__restrict__ phi,
                                                       const T *__restrict__ rhs,
                                                       T *__restrict__ out, int homog,
                                                       double *__restrict__ part) {
  const Geom &G = A.G;
  PlainRead<T> rd{phi};
  double acc = 0.0;
  for (long long q = gtid(); q < G.ncell; q += gstride()) {
    int i, j, k;
    cell_ijk(G, q, i, j, k);
    T p0, lam;
    T lof = vc_lofphi<T, DIM, MODE == VC_JACOBI>(A, rd, i, j, k, homog != 0, p0, lam);
    T v;
    if (MODE == VC_RESIDUAL)
      v = rhs[q] - lof;
    else if (MODE == VC_APPLY)
      v = lof;
    else
      v = p0 + T(0.5) * ((rhs[q] - lof) * lam);
    out[q] = v;
    if (NORM >= 0) acc = norm_accum<NORM < 0 ? 0 : NORM>(acc, (double)v);
  }
  if (NORM >= 0) {
    double r = block_reduce<NORM < 0 ? 0 : NORM>(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = r;
  }
}

// Outer defect-correction step: phi <- phi + e, r = rhs - L(phi) with the
// inhomogeneous BC, r written in FP64 and in the inner precision E, plus the
// fused norm.  Neighbours apply their own correction in registers, so the
// update and the residual need one pass over memory.  out_phi must not alias
// phi (other threads still read the old value); it is unused when e is null.
// With `par` non-null the two solution buffers swap roles when *par == 1
// (ping-pong selected on the device by the outer-loop decision kernel).
template <class T, class E, int DIM, int NORM>
__global__ void __launch_bounds__(kBlock) vc_update_residual_kernel(
    VCArgs<T> A, const T *phi, const E *__restrict__ e, const T *__restrict__ rhs,
    T *out_phi, T *__restrict__ res, E *__restrict__ res_inner, double *__restrict__ part,
    const int *__restrict__ par) {
  const Geom &G = A.G;
  if (par && *par) {
    T *t = out_phi;
    out_phi = (T *)phi;
    phi = t;
  }
  double acc = 0.0;
  for (long long q = gtid(); q < G.ncell; q += gstride()) {
    int i, j, k;
    cell_ijk(G, q, i, j, k);
    T p0, lam, lof;
    if (e) {
      UpdateRead<T, E> rd{phi, e};
      lof = vc_lofphi<T, DIM, false>(A, rd, i, j, k, false, p0, lam);
    } else {
      PlainRead<T> rd{phi};
      lof = vc_lofphi<T, DIM, false>(A, rd, i, j, k, false, p0, lam);
    }
    T v = rhs[q] - lof;
    if (res) res[q] = v;
    if (res_inner) res_inner[q] = (E)v;
    acc = norm_accum<NORM>(acc, (double)v);
    if (e) out_phi[q] = p0;
  }
  double r = block_reduce<NORM>(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = r;
}

template <class T, int DIM>
__device__ __forceinline__ void vc_gsrb_cell(const VCArgs<T> &A, T *phi,
                                             const T *__restrict__ rhs, int i, int j, int k) {
  PlainRead<T> rd{phi};
  T p0, lam;
  T lof = vc_lofphi<T, DIM, true>(A, rd, i, j, k, true, p0, lam);
  long long q = A.G.cell(i, j, k);
  phi[q] = p0 - lam * (lof - rhs[q]);
}

// Red/black half sweep with homogeneous BCs (levelGSRB semantics).
template <class T, int DIM>
__global__ void __launch_bounds__(kBlock) vc_gsrb_kernel(VCArgs<T> A, T *phi,
                                                         const T *__restrict__ rhs, int pass) {
  long long nt = colour_threads(A.G);
  for (long long t = gtid(); t < nt; t += gstride()) {
    int i, j, k;
    if (colour_cell(A.G, pass, t, i, j, k)) vc_gsrb_cell<T, DIM>(A, phi, rhs, i, j, k);
  }
}

// First red pass from a zero initial guess: e = 0 everywhere, so the red
// update is lambda * rhs and black cells are written as zero.  Equal to
// "zero the field, then vc_gsrb_kernel(pass 0)" without the extra pass:
// L(0) with homogeneous BCs is exactly 0 in every term, so
// phi = 0 - lambda * (0 - rhs) reproduces the general update bit for bit.
template <class T, int DIM>
__device__ __forceinline__ void vc_gsrb_zero_cell(const VCArgs<T> &A, T *__restrict__ phi,
                                                  const T *__restrict__ rhs, long long q, int i,
                                                  int j, int k) {
  if (((i + j + k) & 1) == 0) {
    T z = T(0);
    T bzh = T(0), bzl = T(0);
    if (DIM == 3) {
      bzh = vface(A, 2, i, j, k + 1);
      bzl = vface(A, 2, i, j, k);
    }
    T lam = vc_lambda_at<T, DIM>(A, q, vface(A, 0, i + 1, j, k), vface(A, 0, i, j, k),
                                 vface(A, 1, i, j + 1, k), vface(A, 1, i, j, k), bzh, bzl);
    T lof = z;
    phi[q] = z - lam * (lof - rhs[q]);
  } else {
    phi[q] = T(0);
  }
}

template <class T, int DIM>
__global__ void __launch_bounds__(kBlock) vc_gsrb_zero_kernel(VCArgs<T> A, T *__restrict__ phi,
                                                              const T *__restrict__ rhs) {
  const Geom &G = A.G;
  for (long long q = gtid(); q < G.ncell; q += gstride()) {
    int i, j, k;
    cell_ijk(G, q, i, j, k);
    vc_gsrb_zero_cell<T, DIM>(A, phi, rhs, q, i, j, k);
  }
}

template <class T, int DIM>
__global__ void __launch_bounds__(1024) vc_relax_block_kernel(VCArgs<T> A, T *phi,
                                                              const T *__restrict__ rhs,
                                                              int sweeps, int zero_first) {
  long long nt = colour_threads(A.G);
  if (zero_first) {
    for (long long q = threadIdx.x; q < A.G.ncell; q += blockDim.x) phi[q] = T(0);
    __syncthreads();
  }
  for (int s = 0; s < sweeps; s++) {
    for (int pass = 0; pass < 2; pass++) {
      for (long long t = threadIdx.x; t < nt; t += blockDim.x) {
        int i, j, k;
        if (colour_cell(A.G, pass, t, i, j, k)) vc_gsrb_cell<T, DIM>(A, phi, rhs, i, j, k);
      }
      __syncthreads();
    }
  }
}

// RESTRICTRESDB (F.ChF:427-505) with homogeneous BCs; optionally zeroes the
// coarse correction (MultiGrid::cycle setToZero) in the same pass.
template <class T, int DIM>
__global__ void __launch_bounds__(kBlock) vc_restrict_kernel(VCArgs<T> A, Geom C,
                                                             const T *__restrict__ phi,
                                                             const T *__restrict__ rhs,
                                                             T *__restrict__ res_c,
                                                             T *__restrict__ zero_c) {
  const Geom &G = A.G;
  const T denom = DIM == 3 ? T(8) : T(4);
  PlainRead<T> rd{phi};
  for (long long Q = gtid(); Q < C.ncell; Q += gstride()) {
    int I, J, K;
    cell_ijk(C, Q, I, J, K);
    T acc = T(0);
#pragma unroll
    for (int kk = 0; kk < (DIM == 3 ? 2 : 1); kk++)
#pragma unroll
      for (int jj = 0; jj < 2; jj++)
#pragma unroll
        for (int ii = 0; ii < 2; ii++) {
          int i = 2 * I + ii, j = 2 * J + jj, k = DIM == 3 ? 2 * K + kk : 0;
          T p0, lam;
          T lof = vc_lofphi<T, DIM, false>(A, rd, i, j, k, true, p0, lam);
          acc = acc + (rhs[G.cell(i, j, k)] - lof) / denom;
        }
    res_c[Q] = acc;
    if (zero_c) zero_c[Q] = T(0);
  }
}

template <class T, int DIM>
__global__ void __launch_bounds__(kBlock) vc_lambda_kernel(VCArgs<T> A, T *__restrict__ lam) {
  const Geom &G = A.G;
  for (long long q = gtid(); q < G.ncell; q += gstride()) {
    int i, j, k;
    cell_ijk(G, q, i, j, k);
    T av = A.a ? A.a[q] : T(1);
    T l = av * A.alpha;
    if (A.c) l = l + (-A.beta) * A.c[q];
    l = l + A.dxinv * A.beta * (vface(A, 0, i + 1, j, k) + vface(A, 0, i, j, k));
    l = l + A.dxinv * A.beta * (vface(A, 1, i, j + 1, k) + vface(A, 1, i, j, k));
    if (DIM == 3) l = l + A.dxinv * A.beta * (vface(A, 2, i, j, k + 1) + vface(A, 2, i, j, k));
    lam[q] = T(1) / l;
  }
}

}  // namespace mlgpu
