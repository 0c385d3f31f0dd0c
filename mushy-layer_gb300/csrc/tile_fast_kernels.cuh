// tile_fast_kernels.cuh -- lean FP32 variant of the 2D tile smoother for the
// inner cycles of the mixed-precision solver.
//
// For the operator L e = diag e - sum_f c_f e_nb(f) with c_f = beta b_f / dx^2
// and diag = alpha a - beta c + sum_f c_f (resetLambda's diagonal), the
// Gauss-Seidel update e - lambda (L e - r) with lambda = 1/diag is, in exact
// arithmetic, lambda (r + sum_f c_f e_nb(f)); a homogeneous boundary ghost
// g e (g = -1 Dirichlet, +1 Neumann) contributes c_f g e.  That form needs
// five fused multiply-adds per update instead of the reference expression's
// dozen operations.  It is used only inside FP32 cycles, whose result the
// FP64 defect correction re-checks; FP64 cycles keep the reference's exact
// expression (tile_kernels.cuh) and its bits.
//
// Block layout: a 32 x 32 cell region in shared memory (correction only) =
// a (32 - 2H)^2 interior tile + a halo of H cells, H >= the number of half
// sweeps (+1 when the launch also restricts the residual).  Thread (tx, ty)
// owns the horizontal pair of cells (2tx, 2tx+1) of row ty: exactly one of the
// two has the colour of any given pass, so every thread updates one cell per
// half sweep.  Each cell's right-hand side, 1/diag, face weights and its
// boundary-ghost weight stay in registers for the whole launch; a half sweep
// is five shared-memory loads, five FMAs and one store per thread.
#pragma once
#include "tile_kernels.cuh"

namespace mlgpu {

// per-level FP32 coefficients of the lean form
struct FastCoefs {
  const float *cx;    // (n0+1) x n1 faces: beta b_x / dx^2
  const float *cy;    // n0 x (n1+1)
  const float *lam;   // 1 / diag
  const float *diag;  // diag (residual of the restriction)
};

struct TileFast {
  Geom G;
  BCD bc;
  FastCoefs K;
  const float *e_in;
  float *e_out;
  const float *r;
  int zero_init, n_half, pass0, halo;
  float *rc;
  int prolong;
  const float *ec;
};

constexpr int kTF = 32;                     // shared region edge (cells)
constexpr int kTFThreadsX = kTF / 2, kTFThreadsY = kTF;
constexpr int kTFMaxHalo = 12;              // interior edge >= 8
// interior edge of a tile with halo h
__host__ __device__ inline int tile_fast_edge(int h) { return kTF - 2 * h; }

// homogeneous ghost factor of side s of direction d (comp 0)
__device__ __forceinline__ float ghost_factor(const BCD &bc, int d, int s) {
  return bc.type[d][s][0] == MLGPU_BC_DIRICHLET ? -1.0f : 1.0f;
}

#ifdef MLGPU_FP32_UNIT  // kernels compiled in launch_f32.cu only
struct TFCell {
  int c, lx;        // shared-memory index, local x
  bool valid;       // maps to a domain cell (after periodic wrap)
  float e, r, lam, diag;
  float kself, ke, kw, kn, ks;  // ghost weight on e itself; neighbour weights
};

__device__ __forceinline__ void tf_setup(const TileFast &P, int lx, int ly, int gx0, int gy0,
                                         bool inside, float *se, TFCell &k) {
  const Geom &G = P.G;
  const int n0 = G.n0, n1 = G.n1;
  int gx = gx0 + lx, gy = gy0 + ly;
  k.c = ly * kTF + lx;
  k.lx = lx;
  k.valid = true;
  if (!inside) {
    if (gx < 0 || gx >= n0) {
      if (G.per0)
        gx = ((gx % n0) + n0) % n0;
      else
        k.valid = false;
    }
    if (gy < 0 || gy >= n1) {
      if (G.per1)
        gy = ((gy % n1) + n1) % n1;
      else
        k.valid = false;
    }
  }
  float ev = 0.f;
  k.r = k.lam = k.diag = 0.f;
  k.kself = k.ke = k.kw = k.kn = k.ks = 0.f;
  if (k.valid) {
    const long long q = (long long)gy * n0 + gx;
    if (!P.zero_init) ev = P.e_in[q];
    k.r = P.r[q];
    k.lam = P.K.lam[q];
    if (P.rc) k.diag = P.K.diag[q];
    if (P.prolong == MLGPU_PROLONG_LINEAR)
      ev = prolong_add<float, 2, MLGPU_PROLONG_LINEAR>(coarsen_geom(G), P.bc, 0, gx, gy, 0, ev,
                                                        P.ec, nullptr);
    else if (P.prolong == MLGPU_PROLONG_CONSTANT)
      ev = ev + P.ec[(long long)(gy >> 1) * (n0 >> 1) + (gx >> 1)];
    // the cell's own faces (periodic seams included)
    const long long fx = (long long)gy * (n0 + 1) + gx;
    k.ke = P.K.cx[fx + 1];
    k.kw = P.K.cx[fx];
    k.kn = P.K.cy[q + n0];
    k.ks = P.K.cy[q];
    // a non-periodic boundary face: the ghost is g e of this cell
    if (!inside) {
      if (!G.per0 && gx == n0 - 1) {
        k.kself += ghost_factor(P.bc, 0, 1) * k.ke;
        k.ke = 0.f;
      }
      if (!G.per0 && gx == 0) {
        k.kself += ghost_factor(P.bc, 0, 0) * k.kw;
        k.kw = 0.f;
      }
      if (!G.per1 && gy == n1 - 1) {
        k.kself += ghost_factor(P.bc, 1, 1) * k.kn;
        k.kn = 0.f;
      }
      if (!G.per1 && gy == 0) {
        k.kself += ghost_factor(P.bc, 1, 0) * k.ks;
        k.ks = 0.f;
      }
    }
  }
  k.e = ev;
  se[k.c] = ev;
}

// sum_f c_f e_nb(f), ghosts included
__device__ __forceinline__ float tf_nbsum(const TFCell &k, const float *se) {
  float s = k.kself * k.e;
  s = fmaf(k.ke, se[k.c + 1], s);
  s = fmaf(k.kw, se[k.c - 1], s);
  s = fmaf(k.kn, se[k.c + kTF], s);
  s = fmaf(k.ks, se[k.c - kTF], s);
  return s;
}

// half sweep h updates the cells of [h+1, kTF-2-h]^2 that exist
__device__ __forceinline__ void tf_update(TFCell &k, int ly, int h, float *se) {
  const int lo = h + 1, hi = kTF - 2 - h;
  if (k.valid && k.lx >= lo && k.lx <= hi && ly >= lo && ly <= hi) {
    k.e = k.lam * (k.r + tf_nbsum(k, se));
    se[k.c] = k.e;
  }
}

// three 512-thread blocks per SM (40 registers) so a 512^2 level runs in
// fewer waves
__global__ void __launch_bounds__(kTFThreadsX *kTFThreadsY, 3) vc_tile_fast_kernel(TileFast P) {
  __shared__ float se[kTF * kTF];
  __shared__ float sres[kTF * kTF];
  const Geom &G = P.G;
  const int H = P.halo, TE = tile_fast_edge(H);
  const int x0 = blockIdx.x * TE, y0 = blockIdx.y * TE;
  const int gx0 = x0 - H, gy0 = y0 - H;
  const int n0 = G.n0, n1 = G.n1;
  const bool inside = gx0 >= 0 && gx0 + kTF <= n0 && gy0 >= 0 && gy0 + kTF <= n1;
  const int ly = threadIdx.y;
  // A: the cell of the pair with the colour of pass0, B: the other one
  const int odd = (gx0 + gy0 + ly + P.pass0) & 1;
  TFCell A, B;
  tf_setup(P, 2 * threadIdx.x + odd, ly, gx0, gy0, inside, se, A);
  tf_setup(P, 2 * threadIdx.x + 1 - odd, ly, gx0, gy0, inside, se, B);
  __syncthreads();

  for (int h = 0; h < P.n_half; h += 2) {
    tf_update(A, ly, h, se);
    __syncthreads();
    if (h + 1 < P.n_half) {
      tf_update(B, ly, h + 1, se);
      __syncthreads();
    }
  }

  // interior cells: store; residual r - diag e + sum c e_nb for the restriction
  const bool row_in = ly >= H && ly < H + TE && gy0 + ly < n1;
  const bool a_in = row_in && A.lx >= H && A.lx < H + TE && gx0 + A.lx < n0;
  const bool b_in = row_in && B.lx >= H && B.lx < H + TE && gx0 + B.lx < n0;
  const long long grow = (long long)(gy0 + ly) * n0 + gx0;
  if (a_in) P.e_out[grow + A.lx] = A.e;
  if (b_in) P.e_out[grow + B.lx] = B.e;
  if (P.rc) {
    if (a_in) sres[A.c] = (A.r + tf_nbsum(A, se)) - A.diag * A.e;
    if (b_in) sres[B.c] = (B.r + tf_nbsum(B, se)) - B.diag * B.e;
    __syncthreads();
    const int half = TE / 2;
    const int t = threadIdx.y * kTFThreadsX + threadIdx.x;
    if (t < half * half) {
      const int I = t % half, J = t / half;
      const int CI = (x0 >> 1) + I, CJ = (y0 >> 1) + J;
      const int cn0 = n0 >> 1, cn1 = n1 >> 1;
      if (CI < cn0 && CJ < cn1) {
        float acc = 0.f;
        for (int jj = 0; jj < 2; jj++)
          for (int ii = 0; ii < 2; ii++) {
            float res = sres[(H + 2 * J + jj) * kTF + H + 2 * I + ii];
            acc = acc + res * 0.25f;
          }
        P.rc[(long long)CJ * cn0 + CI] = acc;
      }
    }
  }
}

// FP32 lean coefficients of one level from its FP64 operator
template <int DIM>
__global__ void __launch_bounds__(kBlock) fast_coefs_kernel(VCArgs<double> A, float *cx, float *cy,
                                                            float *lam, float *diag) {
  const Geom &G = A.G;
  double scale = A.dxinv * A.beta;
  for (long long t = gtid(); t < G.nface(0); t += gstride()) cx[t] = (float)(scale * A.b[0][t]);
  for (long long t = gtid(); t < G.nface(1); t += gstride()) cy[t] = (float)(scale * A.b[1][t]);
  for (long long q = gtid(); q < G.ncell; q += gstride()) {
    int i, j, k;
    cell_ijk(G, q, i, j, k);
    double av = A.a ? A.a[q] : 1.0;
    double l = av * A.alpha;
    if (A.c) l = l + (-A.beta) * A.c[q];
    l = l + A.dxinv * A.beta * (vface(A, 0, i + 1, j, k) + vface(A, 0, i, j, k));
    l = l + A.dxinv * A.beta * (vface(A, 1, i, j + 1, k) + vface(A, 1, i, j, k));
    diag[q] = (float)l;
    lam[q] = (float)(1.0 / l);
  }
}
#endif  // MLGPU_FP32_UNIT

}  // namespace mlgpu
