// hcm_kernels.cuh -- inner cycles of the mixed-precision nonlinear (H, C)
// solve.
//
// The FP64 outer loop keeps the nonlinear residual r = f - N(u) (closure and
// stencil in FP64, nl_cached_kernels.cuh).  The correction e solves the
// problem linearised at the current state,
//   M(e) = alpha a e - beta div(b grad(J e)) = r,   J = d(T, C_l)/d(H, C),
// with J evaluated in FP64 from the closure once per outer iteration on every
// level (at the restricted state) and stored in FP32.  The cycles on e run in
// FP32 with no closure evaluation: the same red/black smoother as the
// reference's nonlinear one (e <- e - lambda (M(e) - r), lambda the stored
// resetLambda value), residual restriction by 2^D averaging, the solver's
// prolongation, relaxation at the bottom.  Ghosts of J e follow the
// homogeneous form of the reference's boundary rules: the derived-variable
// condition (Dirichlet -g, Neumann g) when it is applied, else the (H, C)
// condition on e mapped through the cell's J.
#pragma once
#include "nl_kernels.cuh"

namespace mlgpu {

struct HCMArgs {
  Geom G;
  BCD phi_bc;
  DBCD dbc;  // the derived (T, C_l) conditions
  int apply_dbc;
  float alpha, beta, dxinv;
  const float *a;     // [2][cells] or null (a == 1)
  const float *b[3];  // [2][faces_d]
  const float *J;     // [4][cells]: dT/dH, dT/dC, dC_l/dH, dC_l/dC
  const float *lam;   // [2][cells]
};

#ifdef MLGPU_FP32_UNIT  // kernels compiled in launch_f32.cu only
__device__ __forceinline__ float hcm_bsign(const BCD &bc, int d, int s, int c) {
  return bc.type[d][s][c] == MLGPU_BC_DIRICHLET ? -1.0f : 1.0f;
}
// the derived conditions' homogeneous rule: also the mixed temperature
// condition's factor g
__device__ __forceinline__ float hcm_bsign(const DBCD &bc, int d, int s, int c) {
  if (bc.type[d][s][c] == MLGPU_BC_MIXED_TEMPERATURE_SALINITY) return (float)bc.rob[d][s][3];
  return hcm_bsign(static_cast<const BCD &>(bc), d, s, c);
}

// J e at cell q
__device__ __forceinline__ void hcm_g(const HCMArgs &A, const float *e, long long q, float g[2]) {
  const long long n = A.G.ncell;
  const float e0 = e[q], e1 = e[q + n];
  g[0] = fmaf(A.J[q], e0, A.J[q + n] * e1);
  g[1] = fmaf(A.J[q + 2 * n], e0, A.J[q + 3 * n] * e1);
}

// J e across face (d, side) of interior cell (i,j,k) (centre cell q, whose J e
// is g0 and e is e0)
__device__ __forceinline__ void hcm_g_nb(const HCMArgs &A, const float *e, int i, int j, int k,
                                         int d, int side, long long q, const float g0[2],
                                         const float e0[2], float g[2]) {
  int idx[3] = {i, j, k};
  const int m = A.G.n(d);
  idx[d] += side ? 1 : -1;
  if (idx[d] < 0 || idx[d] >= m) {
    if (A.G.per(d)) {
      idx[d] = idx[d] < 0 ? m - 1 : 0;
    } else if (A.apply_dbc) {
      g[0] = hcm_bsign(A.dbc, d, side, 0) * g0[0];
      g[1] = hcm_bsign(A.dbc, d, side, 1) * g0[1];
      return;
    } else {
      const long long n = A.G.ncell;
      const float eg0 = hcm_bsign(A.phi_bc, d, side, 0) * e0[0];
      const float eg1 = hcm_bsign(A.phi_bc, d, side, 1) * e0[1];
      g[0] = fmaf(A.J[q], eg0, A.J[q + n] * eg1);
      g[1] = fmaf(A.J[q + 2 * n], eg0, A.J[q + 3 * n] * eg1);
      return;
    }
  }
  hcm_g(A, e, A.G.cell(idx[0], idx[1], idx[2]), g);
}

// M(e) at interior cell (i,j,k), both components; also returns e there
template <int DIM>
__device__ __forceinline__ void hcm_mop(const HCMArgs &A, const float *e, int i, int j, int k,
                                        float mo[2], float ec[2]) {
  const Geom &G = A.G;
  const long long q = G.cell(i, j, k), n = G.ncell;
  ec[0] = e[q];
  ec[1] = e[q + n];
  float g0[2];
  hcm_g(A, e, q, g0);
  float lo[3][2], hi[3][2];
#pragma unroll
  for (int d = 0; d < DIM; d++) {
    hcm_g_nb(A, e, i, j, k, d, 0, q, g0, ec, lo[d]);
    hcm_g_nb(A, e, i, j, k, d, 1, q, g0, ec, hi[d]);
  }
#pragma unroll
  for (int c = 0; c < 2; c++) {
    float s = 0.f;
#pragma unroll
    for (int d = 0; d < DIM; d++) {
      const long long nf = G.nface(d);
      const int ih = i + (d == 0), jh = j + (d == 1), kh = k + (d == 2);
      const float bh = A.b[d][c * nf + G.face(d, ih, jh, kh)];
      const float bl = A.b[d][c * nf + G.face(d, i, j, k)];
      s = fmaf(bh, hi[d][c] - g0[c], s);
      s = fmaf(-bl, g0[c] - lo[d][c], s);
    }
    const float av = A.a ? A.a[q + c * n] : 1.0f;
    mo[c] = A.alpha * av * ec[c] - A.beta * s * A.dxinv;
  }
}

template <int DIM>
__device__ __forceinline__ void hcm_gsrb_cell(const HCMArgs &A, float *e, const float *r, int i,
                                              int j, int k) {
  float mo[2], ec[2];
  hcm_mop<DIM>(A, e, i, j, k, mo, ec);
  const long long q = A.G.cell(i, j, k), n = A.G.ncell;
#pragma unroll
  for (int c = 0; c < 2; c++) e[q + c * n] = ec[c] - A.lam[q + c * n] * (mo[c] - r[q + c * n]);
}

template <int DIM>
__global__ void __launch_bounds__(kBlock) hcm_gsrb_kernel(HCMArgs A, float *e,
                                                          const float *__restrict__ r, int pass) {
  const long long nt = colour_threads(A.G);
  for (long long t = gtid(); t < nt; t += gstride()) {
    int i, j, k;
    if (colour_cell(A.G, pass, t, i, j, k)) hcm_gsrb_cell<DIM>(A, e, r, i, j, k);
  }
}

// bottom: e = 0, then `sweeps` red/black sweeps in one block
template <int DIM>
__global__ void __launch_bounds__(1024) hcm_relax_block_kernel(HCMArgs A, float *e,
                                                               const float *__restrict__ r,
                                                               int sweeps) {
  const long long n = A.G.ncell;
  for (long long q = threadIdx.x; q < 2 * n; q += blockDim.x) e[q] = 0.f;
  __syncthreads();
  const long long nt = colour_threads(A.G);
  for (int s = 0; s < sweeps; s++)
    for (int pass = 0; pass < 2; pass++) {
      for (long long t = threadIdx.x; t < nt; t += blockDim.x) {
        int i, j, k;
        if (colour_cell(A.G, pass, t, i, j, k)) hcm_gsrb_cell<DIM>(A, e, r, i, j, k);
      }
      __syncthreads();
    }
}

// coarse residual: the 2^D average of r - M(e)
template <int DIM>
__global__ void __launch_bounds__(kBlock) hcm_restrict_kernel(HCMArgs A, Geom C,
                                                              const float *__restrict__ e,
                                                              const float *__restrict__ r,
                                                              float *__restrict__ rc) {
  const Geom &G = A.G;
  const float w = DIM == 3 ? 0.125f : 0.25f;
  for (long long Q = gtid(); Q < C.ncell; Q += gstride()) {
    int I, J, K;
    cell_ijk(C, Q, I, J, K);
    float acc[2] = {0.f, 0.f};
#pragma unroll
    for (int kk = 0; kk < (DIM == 3 ? 2 : 1); kk++)
#pragma unroll
      for (int jj = 0; jj < 2; jj++)
#pragma unroll
        for (int ii = 0; ii < 2; ii++) {
          const int i = 2 * I + ii, j = 2 * J + jj, k = DIM == 3 ? 2 * K + kk : 0;
          float mo[2], ec[2];
          hcm_mop<DIM>(A, e, i, j, k, mo, ec);
          const long long q = G.cell(i, j, k);
#pragma unroll
          for (int c = 0; c < 2; c++) acc[c] = fmaf(r[q + c * G.ncell] - mo[c], w, acc[c]);
        }
    rc[Q] = acc[0];
    rc[Q + C.ncell] = acc[1];
  }
}
#endif  // MLGPU_FP32_UNIT

#ifdef MLGPU_FP64_UNIT  // kernels compiled in launch_f64.cu only
// J of every cell from the FP64 state, stored in FP32
__global__ void __launch_bounds__(kBlock) hcm_jac_kernel(Geom G, ClosureParams cp,
                                                         const double *__restrict__ u,
                                                         float *__restrict__ J) {
  const long long n = G.ncell;
  for (long long q = gtid(); q < n; q += gstride()) {
    double j4[4];
    t_cl_jac(u[q], u[q + n], cp, j4);
#pragma unroll
    for (int m = 0; m < 4; m++) J[q + m * n] = (float)j4[m];
  }
}

// u += e (FP64 state, FP32 correction)
__global__ void __launch_bounds__(kBlock) hcm_update_kernel(long long n, double *__restrict__ u,
                                                            const float *__restrict__ e) {
  for (long long q = gtid(); q < n; q += gstride()) u[q] = u[q] + (double)e[q];
}
#endif  // MLGPU_FP64_UNIT

}  // namespace mlgpu
