// bicgstab_kernels.cuh -- BiCGStab bottom solve of the linear
// variable-coefficient operator (projection / Darcy-Brinkman), the
// reference's default bottom solver of the MAC projection and velocity solves
// (srcSubcycle/Projector.cpp:2976-2986, 3012-3020; AMRLevelMushyLayerInit.cpp:
// 738-739 with s_botSolverUStar).  Chombo's BiCGStabSolver is not in the
// reference tree; this is van der Vorst's right-preconditioned BiCGStab with
// the operator's own preconditioner (DarcyBrinkmanOp::preCond,
// src/DarcyBrinkmanOp.cpp:89-121: x = lambda y, then two red/black sweeps of
// L x = y), relative tolerance 1e-6 of the initial residual in the L2 norm,
// at most `imax` iterations, a restart from the true residual when an
// iteration gains less than 1e-8 (at most 5 restarts) and an exit on
// breakdown.
//
// The coarsest level is a handful of cells, so the whole solve is one thread
// block: element-wise updates over all threads, the operator and the
// red/black sweeps through the same per-cell device functions as the level
// kernels (so every value is bitwise the oracle's), and every dot product in
// a fixed order -- warp 0, lane l summing the cells q = l (mod 32) in
// increasing q, then a halving shuffle tree -- which the oracle reproduces.
// Arithmetic is FP64 whatever the storage type of the correction and the
// right-hand side (the mixed-precision cycles keep their coarsest solve in
// FP64).  Every loop is bounded by imax.
#pragma once
#include "vc_kernels.cuh"

namespace mlgpu {

constexpr int kBiCGThreads = 256;
constexpr double kBiCGEps = 1e-6, kBiCGHang = 1e-8;
constexpr int kBiCGRestarts = 5;
constexpr int kBiCGArrays = 11;  // FP64 work arrays of the bottom level

#ifdef MLGPU_FP64_UNIT
// <a, b> in the fixed lane order; every thread returns the same value
__device__ __forceinline__ double bicg_dot(const double *a, const double *b, long long n,
                                           double *slot) {
  if (threadIdx.x < 32) {
    double acc = 0.0;
    for (long long q = threadIdx.x; q < n; q += 32) acc = acc + a[q] * b[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc = acc + __shfl_down_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) *slot = acc;
  }
  __syncthreads();
  const double v = *slot;
  __syncthreads();
  return v;
}

// out = L(in), homogeneous walls
template <int DIM>
__device__ __forceinline__ void bicg_apply(const VCArgs<double> &A, double *out,
                                           const double *in) {
  PlainRead<double> rd{in};
  for (long long q = threadIdx.x; q < A.G.ncell; q += blockDim.x) {
    int i, j, k;
    cell_ijk(A.G, q, i, j, k);
    double p0, lam;
    out[q] = vc_lofphi<double, DIM, false>(A, rd, i, j, k, true, p0, lam);
  }
  __syncthreads();
}

// x = lambda y, then two red/black sweeps of L x = y
template <int DIM>
__device__ __forceinline__ void bicg_precond(const VCArgs<double> &A, double *x,
                                             const double *y) {
  const Geom &G = A.G;
  for (long long q = threadIdx.x; q < G.ncell; q += blockDim.x) {
    int i, j, k;
    cell_ijk(G, q, i, j, k);
    double bzh = 0.0, bzl = 0.0;
    if (DIM == 3) {
      bzh = vface(A, 2, i, j, k + 1);
      bzl = vface(A, 2, i, j, k);
    }
    const double lam = vc_lambda_at<double, DIM>(A, q, vface(A, 0, i + 1, j, k),
                                                 vface(A, 0, i, j, k), vface(A, 1, i, j + 1, k),
                                                 vface(A, 1, i, j, k), bzh, bzl);
    x[q] = y[q] * lam;
  }
  __syncthreads();
  const long long nt = colour_threads(G);
  for (int s = 0; s < 2; s++)
    for (int pass = 0; pass < 2; pass++) {
      for (long long t = threadIdx.x; t < nt; t += blockDim.x) {
        int i, j, k;
        if (colour_cell(G, pass, t, i, j, k)) vc_gsrb_cell<double, DIM>(A, x, y, i, j, k);
      }
      __syncthreads();
    }
}

// L e = rhs on one (coarsest) level; e in/out, ws: kBiCGArrays * ncell doubles.
// remove_mean: the operator is singular (no alpha, no c, no Dirichlet wall:
// constants are its null space) and the right-hand side came through FP32,
// whose rounding leaves it a small mean that no correction can remove;
// subtract that mean first (the mixed-precision cycles only).
template <class S, int DIM>
__global__ void __launch_bounds__(kBiCGThreads) vc_bicgstab_kernel(VCArgs<double> A, S *e_io,
                                                                   const S *rhs_in,
                                                                   double *ws, int imax,
                                                                   int remove_mean) {
  __shared__ double slot;
  const long long n = A.G.ncell;
  double *e = ws, *f = ws + n, *r = ws + 2 * n, *rt = ws + 3 * n, *x = ws + 4 * n,
         *p = ws + 5 * n, *v = ws + 6 * n, *ph = ws + 7 * n, *s = ws + 8 * n, *sh = ws + 9 * n,
         *t = ws + 10 * n;
  for (long long q = threadIdx.x; q < n; q += blockDim.x) {
    e[q] = (double)e_io[q];
    f[q] = (double)rhs_in[q];
    x[q] = 0.0;
    p[q] = 0.0;
    v[q] = 0.0;
    t[q] = 1.0;
  }
  __syncthreads();
  if (remove_mean) {
    const double mean = bicg_dot(f, t, n, &slot) / (double)n;
    for (long long q = threadIdx.x; q < n; q += blockDim.x) f[q] = f[q] - mean;
    __syncthreads();
  }
  // r = rhs - L(e), r~ = r
  bicg_apply<DIM>(A, t, e);
  for (long long q = threadIdx.x; q < n; q += blockDim.x) {
    r[q] = f[q] - t[q];
    rt[q] = r[q];
  }
  __syncthreads();
  const double norm0 = sqrt(bicg_dot(r, r, n, &slot));
  double norm = norm0, rho0 = 0.0, rho1 = 0.0, alpha = 0.0, omega = 0.0;
  bool init = true;
  int restarts = 0;
  for (int it = 0; it < imax && norm > kBiCGEps * norm0 && restarts <= kBiCGRestarts; it++) {
    rho1 = rho0;
    rho0 = bicg_dot(rt, r, n, &slot);
    if (rho0 == 0.0) break;
    if (init) {
      for (long long q = threadIdx.x; q < n; q += blockDim.x) p[q] = r[q];
      init = false;
    } else {
      const double beta = (rho0 / rho1) * (alpha / omega);
      for (long long q = threadIdx.x; q < n; q += blockDim.x)
        p[q] = r[q] + beta * (p[q] - omega * v[q]);
    }
    __syncthreads();
    bicg_precond<DIM>(A, ph, p);
    bicg_apply<DIM>(A, v, ph);
    const double m = bicg_dot(rt, v, n, &slot);
    if (m == 0.0) break;
    alpha = rho0 / m;
    for (long long q = threadIdx.x; q < n; q += blockDim.x) {
      s[q] = r[q] - alpha * v[q];
      x[q] = x[q] + alpha * ph[q];
    }
    __syncthreads();
    const double snorm = sqrt(bicg_dot(s, s, n, &slot));
    if (snorm <= kBiCGEps * norm0) {
      norm = snorm;
      break;
    }
    bicg_precond<DIM>(A, sh, s);
    bicg_apply<DIM>(A, t, sh);
    const double tt = bicg_dot(t, t, n, &slot);
    const double ts = bicg_dot(t, s, n, &slot);
    omega = tt > 0.0 ? ts / tt : 0.0;
    for (long long q = threadIdx.x; q < n; q += blockDim.x) {
      x[q] = x[q] + omega * sh[q];
      r[q] = s[q] - omega * t[q];
    }
    __syncthreads();
    const double prev = norm;
    norm = sqrt(bicg_dot(r, r, n, &slot));
    if (omega == 0.0 || norm > (1.0 - kBiCGHang) * prev) {
      // restart from the true residual of e + x
      for (long long q = threadIdx.x; q < n; q += blockDim.x) {
        e[q] = e[q] + x[q];
        x[q] = 0.0;
      }
      __syncthreads();
      bicg_apply<DIM>(A, t, e);
      for (long long q = threadIdx.x; q < n; q += blockDim.x) {
        r[q] = f[q] - t[q];
        rt[q] = r[q];
      }
      __syncthreads();
      norm = sqrt(bicg_dot(r, r, n, &slot));
      init = true;
      restarts++;
    }
  }
  for (long long q = threadIdx.x; q < n; q += blockDim.x) e_io[q] = (S)(e[q] + x[q]);
}
#endif  // MLGPU_FP64_UNIT

}  // namespace mlgpu
