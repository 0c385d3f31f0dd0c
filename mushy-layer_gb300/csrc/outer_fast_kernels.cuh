// outer_fast_kernels.cuh -- FP64 outer step of the mixed-precision solver
// (2D): phi <- phi + e (e the FP32 correction of the inner cycle), the FP64
// residual r = rhs - L(phi) with the physical (inhomogeneous) boundary
// conditions, its FP32 copy for the next inner cycle and the residual norm,
// in one launch.
//
// The FP64 pipe of a GB300 runs at 1/64 of the FP32 rate, so this step is
// built around FP64 instruction count: with precomputed FP64 face weights
// c_f = beta b_f / dx^2 and diag = alpha a - beta c + sum_f c_f (the
// reference's resetLambda diagonal), L(phi) = diag phi - sum_f c_f phi_nb(f)
// and the residual is five FP64 FMAs per cell; phi + e is formed once per
// cell in a shared-memory tile (one-cell halo) instead of once per stencil
// read.  The FP64-precision solver keeps the reference's exact expression
// order (vc_update_residual_kernel) for bitwise parity; this form is the
// mixed solver's, whose FP64 residual only has to be FP64-accurate.
//
// The last block to finish combines the per-block partial norms (fixed
// order) and, inside the device-resident outer loop, applies the
// convergence tests and sets the loop's condition.
#pragma once
#include "launch.h"
#include "vc_kernels.cuh"
#include "outer_kernels.cuh"

namespace mlgpu {

struct OuterCoefs {
  const double *cx, *cy, *diag;
};

struct OuterFast {
  Geom G;
  BCD bc;
  OuterCoefs K;
  const double *phi;
  const float *e;        // null: residual of phi itself, no update
  const double *rhs;
  double *out_phi;       // phi + e (unused when e is null)
  float *res_inner;      // FP32 residual for the next inner cycle
  double *part;          // partials; part[kMaxBlocks] receives the norm
  unsigned *count;       // blocks finished; zero between launches
  const int *par;        // ping-pong of phi / out_phi (or null)
  OuterDev *st;          // non-null: apply the outer-loop tests
  OuterCfg cfg;
  cudaGraphConditionalHandle h;
};

constexpr int kOTX = 32, kOTY = 32, kOTThreads = 256;
constexpr int kOTLX = kOTX + 2, kOTLY = kOTY + 2;

#ifdef MLGPU_FP64_UNIT  // kernels compiled in launch_f64.cu only
template <int NORM>
__global__ void __launch_bounds__(kOTThreads) vc_outer_fast_kernel(OuterFast P) {
  __shared__ double sp[kOTLX * kOTLY];
  __shared__ int is_last;
  const Geom &G = P.G;
  const int n0 = G.n0, n1 = G.n1;
  const double *phi = P.phi;
  double *out = P.out_phi;
  if (P.par && *P.par) {
    out = (double *)P.phi;
    phi = P.out_phi;
  }
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
  const int ntx = (n0 + kOTX - 1) / kOTX, nty = (n1 + kOTY - 1) / kOTY;
  double acc = 0.0;
  bool bad = false;
  for (int tile = blockIdx.x; tile < ntx * nty; tile += gridDim.x) {
    const int x0 = (tile % ntx) * kOTX, y0 = (tile / ntx) * kOTY;
    for (int q = tid; q < kOTLX * kOTLY; q += kOTThreads) {
      int gx = x0 - 1 + q % kOTLX, gy = y0 - 1 + q / kOTLX;
      if (gx < 0 || gx >= n0) {
        if (!G.per0 || gx < -1 || gx > n0) continue;
        gx = gx < 0 ? n0 - 1 : 0;
      }
      if (gy < 0 || gy >= n1) {
        if (!G.per1 || gy < -1 || gy > n1) continue;
        gy = gy < 0 ? n1 - 1 : 0;
      }
      const long long g = (long long)gy * n0 + gx;
      double v = phi[g];
      if (P.e) v = v + (double)P.e[g];
      sp[q] = v;
    }
    __syncthreads();
    // tiles away from non-periodic boundaries need no ghost values
    const bool plain = (G.per0 || (x0 > 0 && x0 + kOTX < n0)) &&
                       (G.per1 || (y0 > 0 && y0 + kOTY < n1));
#pragma unroll
    for (int m = 0; m < kOTY / 8; m++) {
      const int gx = x0 + tx, gy = y0 + ty + 8 * m;
      if (gx >= n0 || gy >= n1) continue;
      const int c = (ty + 8 * m + 1) * kOTLX + tx + 1;
      const long long g = (long long)gy * n0 + gx;
      const double p0 = sp[c];
      double ve = sp[c + 1], vw = sp[c - 1], vn = sp[c + kOTLX], vs = sp[c - kOTLX];
      if (!plain) {
        if (gx + 1 >= n0 && !G.per0) ve = ghost_value<double>(P.bc, 0, 1, 0, p0, G.dx, false);
        if (gx == 0 && !G.per0) vw = ghost_value<double>(P.bc, 0, 0, 0, p0, G.dx, false);
        if (gy + 1 >= n1 && !G.per1) vn = ghost_value<double>(P.bc, 1, 1, 0, p0, G.dx, false);
        if (gy == 0 && !G.per1) vs = ghost_value<double>(P.bc, 1, 0, 0, p0, G.dx, false);
      }
      const long long fx = (long long)gy * (n0 + 1) + gx;
      double r = fma(-P.K.diag[g], p0, P.rhs[g]);
      r = fma(P.K.cx[fx + 1], ve, r);
      r = fma(P.K.cx[fx], vw, r);
      r = fma(P.K.cy[g + n0], vn, r);
      r = fma(P.K.cy[g], vs, r);
      const float rf = (float)r;
      P.res_inner[g] = rf;
      if (P.e) out[g] = p0;
      if (NORM == MLGPU_NORM_MAX) {
        // NaN / Inf: all exponent bits set (integer test); the FP64 max is
        // then one operation
        bad |= (__double2hiint(r) & 0x7ff00000) == 0x7ff00000;
        acc = fmax(acc, fabs(r));
      } else {
        acc = norm_accum<NORM>(acc, r);
      }
    }
    __syncthreads();
  }
  if (NORM == MLGPU_NORM_MAX && __syncthreads_or(bad))
    acc = __longlong_as_double(0x7ff8000000000000LL);
  double r = block_reduce<NORM>(acc);
  if (tid == 0) {
    P.part[blockIdx.x] = r;
    __threadfence();
    unsigned t = atomicAdd(P.count, 1u);
    is_last = t == gridDim.x - 1;
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  double a = 0.0;
  for (int q = tid; q < (int)gridDim.x; q += kOTThreads) a = norm_combine<NORM>(a, __ldcg(P.part + q));
  a = block_reduce<NORM>(a);
  if (tid == 0) {
    const double norm = NORM == MLGPU_NORM_L2 ? sqrt(a) : a;
    P.part[kMaxBlocks] = norm;
    *P.count = 0u;
    if (P.st) outer_decide_step(P.st, norm, P.cfg, P.h);
  }
}

// FP64 face weights and diagonal of the outer operator (level 0)
__global__ void __launch_bounds__(kBlock) outer_coefs_kernel(VCArgs<double> A, double *cx,
                                                             double *cy, double *diag) {
  const Geom &G = A.G;
  const double scale = A.dxinv * A.beta;
  for (long long t = gtid(); t < G.nface(0); t += gstride()) cx[t] = scale * A.b[0][t];
  for (long long t = gtid(); t < G.nface(1); t += gstride()) cy[t] = scale * A.b[1][t];
  for (long long q = gtid(); q < G.ncell; q += gstride()) {
    int i, j, k;
    cell_ijk(G, q, i, j, k);
    double av = A.a ? A.a[q] : 1.0;
    double l = av * A.alpha;
    if (A.c) l = l + (-A.beta) * A.c[q];
    l = l + A.dxinv * A.beta * (vface(A, 0, i + 1, j, k) + vface(A, 0, i, j, k));
    l = l + A.dxinv * A.beta * (vface(A, 1, i, j + 1, k) + vface(A, 1, i, j, k));
    diag[q] = l;
  }
}
#endif  // MLGPU_FP64_UNIT

}  // namespace mlgpu
