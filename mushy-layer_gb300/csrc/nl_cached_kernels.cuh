// nl_cached_kernels.cuh -- FP64 nonlinear (H, C) kernels that read the
// diffused variable (T, C_l) from a per-level cache instead of recomputing the
// closure for a cell and its 2D neighbours at every stencil evaluation.
//
// The reference recomputes (T, C_l) for every cell before each colour pass
// (computeDiffusedVar in levelGSRB, AMRNonLinearMultiCompOp.cpp:834-838) and
// the stencil reads those values; a cell's (T, C_l) only changes when the
// cell itself is updated.  So the cache holds t_cl(H, C) of every cell, a
// red/black pass reads it for the centre and its (opposite-colour)
// neighbours, and every updated cell writes back the closure of its new
// value.  The values are the same calls on the same inputs, so the results
// are bitwise those of the uncached kernels; the closure (five FP64 divisions
// and a square root in the mush, on a GPU whose FP64 pipe runs at 1/64 of the
// FP32 rate) is evaluated once per updated cell instead of 2D+1 times.
// 1/diag comes from the stored resetLambda array, also bitwise the same.
#pragma once
#include "nl_kernels.cuh"

namespace mlgpu {

// 64-thread blocks: small levels spread their FP64 work over more SMs
constexpr int kNLCBlock = 64;
inline int nlc_blocks(long long n) {
  long long b = (n + kNLCBlock - 1) / kNLCBlock;
  if (b < 1) b = 1;
  if (b > kMaxBlocks) b = kMaxBlocks;
  return (int)b;
}

#ifdef MLGPU_NLC_UNIT  // kernels compiled in launch_f64_nlc.cu only
// (T, C_l) at neighbour (i,j,k) + s e_d of an interior cell whose own (H, C)
// and (T, C_l) are h0, c0, t0, l0 (nl_dv_nb with the cache)
__device__ __forceinline__ void nlc_dv_nb(const NLArgs<double> &A, const double *tcl, int i, int j,
                                          int k, int d, int side, double h0, double c0, double t0,
                                          double l0, double &t, double &cl) {
  int idx[3] = {i, j, k};
  const int m = A.G.n(d);
  idx[d] += side ? 1 : -1;
  if (idx[d] < 0 || idx[d] >= m) {
    if (A.G.per(d)) {
      idx[d] = idx[d] < 0 ? m - 1 : 0;
    } else if (A.apply_dbc) {
      t = ghost_value<double>(A.dbc, d, side, 0, t0, A.dx, false);
      cl = ghost_value<double>(A.dbc, d, side, 1, l0, A.dx, false);
      return;
    } else {
      double hg = nl_ghost_h(A, i, j, k, d, side, h0, c0);
      double cg = ghost_value<double>(A.phi_bc, d, side, 1, c0, A.dx, false);
      t_cl(hg, cg, A.cp, t, cl);
      return;
    }
  }
  const long long q = A.G.cell(idx[0], idx[1], idx[2]);
  t = tcl[q];
  cl = tcl[q + A.G.ncell];
}

// L(phi) for both components (nl_lofphi with the cache; same expression order)
template <int DIM>
__device__ __forceinline__ void nlc_lofphi(const NLArgs<double> &A, const double *phi,
                                           const double *tcl, int i, int j, int k, double lof[2],
                                           double ph[2]) {
  const Geom &G = A.G;
  const long long q = G.cell(i, j, k);
  const double h0 = phi[q], c0 = phi[q + G.ncell];
  ph[0] = h0;
  ph[1] = c0;
  const double pl0[2] = {tcl[q], tcl[q + G.ncell]};
  double lo[3][2], hi[3][2];
#pragma unroll
  for (int d = 0; d < DIM; d++) {
    nlc_dv_nb(A, tcl, i, j, k, d, 0, h0, c0, pl0[0], pl0[1], lo[d][0], lo[d][1]);
    nlc_dv_nb(A, tcl, i, j, k, d, 1, h0, c0, pl0[0], pl0[1], hi[d][0], hi[d][1]);
  }
#pragma unroll
  for (int c = 0; c < 2; c++) {
    const double p0 = pl0[c];
    const double bxh = bface(A, 0, c, i + 1, j, k), bxl = bface(A, 0, c, i, j, k);
    const double byh = bface(A, 1, c, i, j + 1, k), byl = bface(A, 1, c, i, j, k);
    double s = bxh * (hi[0][c] - p0) - bxl * (p0 - lo[0][c]);
    s = s + byh * (hi[1][c] - p0);
    s = s - byl * (p0 - lo[1][c]);
    if (DIM == 3) {
      const double bzh = bface(A, 2, c, i, j, k + 1), bzl = bface(A, 2, c, i, j, k);
      s = s + bzh * (hi[2][c] - p0);
      s = s - bzl * (p0 - lo[2][c]);
    }
    const double av = A.a ? A.a[q + c * G.ncell] : 1.0;
    lof[c] = A.alpha * av * ph[c] - A.beta * s * A.dxinv;
  }
}

// the cache of every cell (LEAN: t_cl_lean, for the lean Newton paths)
template <int DIM, bool LEAN>
__global__ void __launch_bounds__(kNLCBlock) nlc_closure_kernel(NLArgs<double> A, ClosureLean P,
                                                                const double *__restrict__ phi,
                                                                double *__restrict__ tcl) {
  const long long n = A.G.ncell;
  for (long long q = gtid(); q < n; q += gstride()) {
    double t, cl;
    if (LEAN)
      t_cl_lean(phi[q], phi[q + n], P, t, cl);
    else
      t_cl(phi[q], phi[q + n], A.cp, t, cl);
    tcl[q] = t;
    tcl[q + n] = cl;
  }
}

// one red/black update (NONLINEARSMOOTHING) and the closure of its result
template <int DIM>
__device__ __forceinline__ void nlc_gsrb_cell(const NLArgs<double> &A, double *phi,
                                              const double *__restrict__ rhs, double *tcl,
                                              const double *__restrict__ lam, int i, int j, int k) {
  double lof[2], ph[2];
  nlc_lofphi<DIM>(A, phi, tcl, i, j, k, lof, ph);
  const long long q = A.G.cell(i, j, k), n = A.G.ncell;
  double nv[2];
#pragma unroll
  for (int c = 0; c < 2; c++) {
    const long long qc = q + c * n;
    nv[c] = ph[c] - lam[qc] * (lof[c] - rhs[qc]);
    phi[qc] = nv[c];
  }
  double t, cl;
  t_cl(nv[0], nv[1], A.cp, t, cl);
  tcl[q] = t;
  tcl[q + n] = cl;
}

template <int DIM>
__global__ void __launch_bounds__(kNLCBlock) nlc_gsrb_kernel(NLArgs<double> A, double *phi,
                                                             const double *__restrict__ rhs,
                                                             double *tcl,
                                                             const double *__restrict__ lam,
                                                             int pass) {
  const long long nt = colour_threads(A.G);
  for (long long t = gtid(); t < nt; t += gstride()) {
    int i, j, k;
    if (colour_cell(A.G, pass, t, i, j, k)) nlc_gsrb_cell<DIM>(A, phi, rhs, tcl, lam, i, j, k);
  }
}

// the whole bottom relaxation in one block; `init` fills the cache first.
// One cell per warp (lane 0): a GB300 FP64 unit takes ~64 cycles per warp
// instruction whatever the number of active lanes, so the few cells of a
// bottom level are spread over the SM's four schedulers instead of sharing
// one warp.
template <int DIM>
__global__ void __launch_bounds__(1024) nlc_relax_block_kernel(NLArgs<double> A, double *phi,
                                                               const double *__restrict__ rhs,
                                                               double *tcl,
                                                               const double *__restrict__ lam,
                                                               int sweeps, int init) {
  const long long n = A.G.ncell;
  if (init) {
    for (long long q = threadIdx.x; q < n; q += blockDim.x) {
      double t, cl;
      t_cl(phi[q], phi[q + n], A.cp, t, cl);
      tcl[q] = t;
      tcl[q + n] = cl;
    }
    __syncthreads();
  }
  const long long nt = colour_threads(A.G);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int s = 0; s < sweeps; s++) {
    for (int pass = 0; pass < 2; pass++) {
      if (lane == 0)
        for (long long t = warp; t < nt; t += nwarps) {
          int i, j, k;
          if (colour_cell(A.G, pass, t, i, j, k)) nlc_gsrb_cell<DIM>(A, phi, rhs, tcl, lam, i, j, k);
        }
      __syncthreads();
    }
  }
}

// NL_RESIDUAL (with a fused norm; MAX2: the max norm too, into part_max)
// and NL_APPLY_PLUS over the cache
template <int DIM, int MODE, int NORM, bool MAX2>
__global__ void __launch_bounds__(kNLCBlock) nlc_op_kernel(NLArgs<double> A,
                                                           const double *__restrict__ phi,
                                                           const double *__restrict__ tcl,
                                                           const double *__restrict__ rhs,
                                                           double *__restrict__ out,
                                                           double *__restrict__ copy,
                                                           double *__restrict__ part,
                                                           double *__restrict__ part_max) {
  const Geom &G = A.G;
  double acc = 0.0, amax = 0.0;
  for (long long q = gtid(); q < G.ncell; q += gstride()) {
    int i, j, k;
    cell_ijk(G, q, i, j, k);
    double lof[2], ph[2];
    nlc_lofphi<DIM>(A, phi, tcl, i, j, k, lof, ph);
#pragma unroll
    for (int c = 0; c < 2; c++) {
      const long long qc = q + c * G.ncell;
      double v;
      if (MODE == NL_RESIDUAL) {
        v = rhs[qc] - lof[c];
      } else {
        v = lof[c] + rhs[qc];
        copy[qc] = ph[c];
      }
      out[qc] = v;
      if (NORM >= 0) acc = norm_accum<NORM < 0 ? 0 : NORM>(acc, v);
      if (MAX2) amax = norm_accum<MLGPU_NORM_MAX>(amax, v);
    }
  }
  if (NORM >= 0) {
    double r = block_reduce<NORM < 0 ? 0 : NORM>(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = r;
  }
  if (MAX2) {
    double r = block_reduce<MLGPU_NORM_MAX>(amax);
    if (threadIdx.x == 0) part_max[blockIdx.x] = r;
  }
}

// the sum of every face coefficient of each cell, per component (the lean
// residual's diagonal term; formed once per solver)
template <int DIM>
__global__ void __launch_bounds__(kNLCBlock) nlc_bsum_kernel(NLArgs<double> A,
                                                             double *__restrict__ sb) {
  const Geom &G = A.G;
  const long long n = G.ncell;
  for (long long q = gtid(); q < n; q += gstride()) {
    int i, j, k;
    cell_ijk(G, q, i, j, k);
#pragma unroll
    for (int c = 0; c < 2; c++) {
      double s = bface(A, 0, c, i + 1, j, k) + bface(A, 0, c, i, j, k);
      s = s + bface(A, 1, c, i, j + 1, k) + bface(A, 1, c, i, j, k);
      if (DIM == 3) s = s + bface(A, 2, c, i, j, k + 1) + bface(A, 2, c, i, j, k);
      sb[q + c * n] = s;
    }
  }
}

// NL_RESIDUAL for the lean Newton paths over the cache:
//   sum_f b_f (f_nb - f_c) = sum_f b_f f_nb - f_c sum_f b_f
// with sum_f b_f per cell precomputed (sb; a wall face's ghost value enters
// as its neighbour value, so the identity holds on every face), by FMA;
// r = rhs - (alpha a) phi + (beta dxinv) s by two FMAs; its L2 norm by FMA and its max norm on
// the bit patterns of |v| (for non-negative doubles the integer order is the
// numeric order, and a NaN's pattern is above every number's, so it stays
// sticky).  Half the reference-order kernel's FP64 pipe operations; the
// cancellation in the product form costs (max |f| / max |f_nb - f_c|) ulps
// of the flux, far below the Newton tolerance's scale for the closure's
// bounded T and C_l.
template <int DIM>
__global__ void __launch_bounds__(kNLCBlock) nlc_res_lean_kernel(NLArgs<double> A,
                                                                 const double *__restrict__ phi,
                                                                 const double *__restrict__ tcl,
                                                                 const double *__restrict__ sb,
                                                                 const double *__restrict__ rhs,
                                                                 double *__restrict__ out,
                                                                 double *__restrict__ part,
                                                                 double *__restrict__ part_max) {
  const Geom &G = A.G;
  const long long n = G.ncell;
  const double bd = A.beta * A.dxinv;
  double acc = 0.0;
  unsigned long long amax = 0ull;
  for (long long q = gtid(); q < n; q += gstride()) {
    int i, j, k;
    cell_ijk(G, q, i, j, k);
    const double h0 = phi[q], c0 = phi[q + n];
    const double pl0[2] = {tcl[q], tcl[q + n]};
    double lo[3][2], hi[3][2];
#pragma unroll
    for (int d = 0; d < DIM; d++) {
      nlc_dv_nb(A, tcl, i, j, k, d, 0, h0, c0, pl0[0], pl0[1], lo[d][0], lo[d][1]);
      nlc_dv_nb(A, tcl, i, j, k, d, 1, h0, c0, pl0[0], pl0[1], hi[d][0], hi[d][1]);
    }
    const double ph[2] = {h0, c0};
#pragma unroll
    for (int c = 0; c < 2; c++) {
      double s = bface(A, 0, c, i + 1, j, k) * hi[0][c];
      s = fma(bface(A, 0, c, i, j, k), lo[0][c], s);
      s = fma(bface(A, 1, c, i, j + 1, k), hi[1][c], s);
      s = fma(bface(A, 1, c, i, j, k), lo[1][c], s);
      if (DIM == 3) {
        s = fma(bface(A, 2, c, i, j, k + 1), hi[2][c], s);
        s = fma(bface(A, 2, c, i, j, k), lo[2][c], s);
      }
      s = fma(-pl0[c], sb[q + c * n], s);
      const double aa = A.a ? A.alpha * A.a[q + c * n] : A.alpha;
      // rhs - (aa phi - bd s) as two FMAs
      const double v = fma(bd, s, fma(-aa, ph[c], rhs[q + c * n]));
      out[q + c * n] = v;
      acc = fma(v, v, acc);
      const unsigned long long bits =
          (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
      amax = bits > amax ? bits : amax;
    }
  }
  // two instantiations of block_reduce: two shared arrays, no reuse race
  const double r = block_reduce<MLGPU_NORM_L2>(acc);
  const double m = block_reduce<MLGPU_NORM_MAX>(__longlong_as_double((long long)amax));
  if (threadIdx.x == 0) {
    part[blockIdx.x] = r;
    part_max[blockIdx.x] = m;
  }
}

// FAS restriction fused with restrictR (nl_restrict_kernel over the cache)
template <int DIM>
__global__ void __launch_bounds__(kNLCBlock) nlc_restrict_kernel(NLArgs<double> A, Geom C,
                                                                 const double *__restrict__ phi,
                                                                 const double *__restrict__ tcl,
                                                                 const double *__restrict__ rhs,
                                                                 double *__restrict__ res_c,
                                                                 double *__restrict__ phi_c) {
  const Geom &G = A.G;
  const double denom = DIM == 3 ? 8.0 : 4.0;
  for (long long Q = gtid(); Q < C.ncell; Q += gstride()) {
    int I, J, K;
    cell_ijk(C, Q, I, J, K);
    double acc[2] = {0.0, 0.0}, avg[2] = {0.0, 0.0};
#pragma unroll
    for (int kk = 0; kk < (DIM == 3 ? 2 : 1); kk++)
#pragma unroll
      for (int jj = 0; jj < 2; jj++)
#pragma unroll
        for (int ii = 0; ii < 2; ii++) {
          const int i = 2 * I + ii, j = 2 * J + jj, k = DIM == 3 ? 2 * K + kk : 0;
          double lof[2], ph[2];
          nlc_lofphi<DIM>(A, phi, tcl, i, j, k, lof, ph);
          const long long q = G.cell(i, j, k);
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
#endif  // MLGPU_NLC_UNIT

}  // namespace mlgpu
