// tile_fast_kernels.cuh -- lean FP32 variant of the 2D tile smoother for the
// inner cycles of the mixed-precision solver.
//
// For the operator L e = diag e - sum_f c_f e_nb(f) with c_f = beta b_f / dx^2
// and diag = alpha a - beta c + sum_f c_f (resetLambda's diagonal), the
// Gauss-Seidel update e - lambda (L e - r) with lambda = 1/diag is, in exact
// arithmetic, lambda (r + sum_f c_f e_nb(f)); a homogeneous boundary ghost
// s e (s = -1 Dirichlet, +1 Neumann) contributes c_f s e.  That form needs
// four fused multiply-adds per update instead of the reference expression's
// dozen operations.  It is used only inside FP32 cycles, whose result the
// FP64 defect correction re-checks; FP64 cycles keep the reference's exact
// expression (tile_kernels.cuh) and its bits.
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

inline size_t tile_fast_smem_bytes(int halo) {
  size_t lx = kTileX + 2 * halo, ly = kTileY + 2 * halo;
  return sizeof(float) * (3 * lx * ly + (lx + 1) * ly + lx * (ly + 1));
}

// homogeneous ghost factor of side s of direction d (comp 0)
__device__ __forceinline__ float ghost_factor(const BCD &bc, int d, int s) {
  return bc.type[d][s][0] == MLGPU_BC_DIRICHLET ? -1.0f : 1.0f;
}

#ifdef MLGPU_FP32_UNIT  // kernels compiled in launch_f32.cu only
__global__ void __launch_bounds__(kTileThreads) vc_tile_fast_kernel(TileFast P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Geom &G = P.G;
  const int H = P.halo;
  const int LX = kTileX + 2 * H, LY = kTileY + 2 * H;
  float *se = (float *)smem_raw;
  float *sr = se + LX * LY;
  float *sl = sr + LX * LY;
  float *scx = sl + LX * LY;         // (LX+1) x LY
  float *scy = scx + (LX + 1) * LY;  // LX x (LY+1)
  const int x0 = blockIdx.x * kTileX, y0 = blockIdx.y * kTileY;
  const int gx0 = x0 - H, gy0 = y0 - H;
  const int n0 = G.n0, n1 = G.n1;
  const bool px = G.per0 != 0, py = G.per1 != 0;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const bool inside = gx0 >= 0 && gx0 + LX <= n0 && gy0 >= 0 && gy0 + LY <= n1;
  const float *cxg = P.K.cx, *cyg = P.K.cy;

  auto gxw = [&](int gx) -> int {
    if (gx >= 0 && gx < n0) return gx;
    if (!px) return -1;
    return ((gx % n0) + n0) % n0;
  };
  auto gyw = [&](int gy) -> int {
    if (gy >= 0 && gy < n1) return gy;
    if (!py) return -1;
    return ((gy % n1) + n1) % n1;
  };

  // ---- load scaled faces, then cells
  for (int ly = ty; ly < LY; ly += kTileTY)
    for (int lx = tx; lx <= LX; lx += kTileTX) {
      float v = 0.f;
      int gy = inside ? gy0 + ly : gyw(gy0 + ly);
      if (gy >= 0) {
        int fx = gx0 + lx;
        if (fx < 0 || fx > n0) fx = px ? ((fx % n0) + n0) % n0 : -1;
        if (fx >= 0) v = cxg[(long long)gy * (n0 + 1) + fx];
      }
      scx[ly * (LX + 1) + lx] = v;
    }
  for (int ly = ty; ly <= LY; ly += kTileTY)
    for (int lx = tx; lx < LX; lx += kTileTX) {
      float v = 0.f;
      int gx = inside ? gx0 + lx : gxw(gx0 + lx);
      if (gx >= 0) {
        int fy = gy0 + ly;
        if (fy < 0 || fy > n1) fy = py ? ((fy % n1) + n1) % n1 : -1;
        if (fy >= 0) v = cyg[(long long)fy * n0 + gx];
      }
      scy[ly * LX + lx] = v;
    }
  const Geom Cg = coarsen_geom(G);
  for (int ly = ty; ly < LY; ly += kTileTY)
    for (int lx = tx; lx < LX; lx += kTileTX) {
      int q = ly * LX + lx;
      int gx = inside ? gx0 + lx : gxw(gx0 + lx), gy = inside ? gy0 + ly : gyw(gy0 + ly);
      float ev = 0.f, rv = 0.f, lv = 0.f;
      if (gx >= 0 && gy >= 0) {
        long long gq = (long long)gy * n0 + gx;
        if (!P.zero_init) ev = P.e_in[gq];
        rv = P.r[gq];
        lv = P.K.lam[gq];
        if (P.prolong == MLGPU_PROLONG_LINEAR)
          ev = prolong_add<float, 2, MLGPU_PROLONG_LINEAR>(Cg, P.bc, 0, gx, gy, 0, ev, P.ec, nullptr);
        else if (P.prolong == MLGPU_PROLONG_CONSTANT)
          ev = prolong_add<float, 2, MLGPU_PROLONG_CONSTANT>(Cg, P.bc, 0, gx, gy, 0, ev, P.ec, nullptr);
      }
      se[q] = ev;
      sr[q] = rv;
      sl[q] = lv;
    }
  __syncthreads();

  // sum_f c_f e_nb(f) at local (lx, ly), global wrapped (gx, gy)
  auto nbsum = [&](int lx, int ly, int gx, int gy) -> float {
    int c = ly * LX + lx, fc = ly * (LX + 1) + lx;
    if (inside) {
      float s = scx[fc + 1] * se[c + 1];
      s = fmaf(scx[fc], se[c - 1], s);
      s = fmaf(scy[c + LX], se[c + LX], s);
      s = fmaf(scy[c], se[c - LX], s);
      return s;
    }
    float p0 = se[c];
    // seam faces of periodic directions come from the cell's own entries
    float cxh = (px && gx == n0 - 1) ? cxg[(long long)gy * (n0 + 1) + n0] : scx[fc + 1];
    float cxl = (px && gx == 0) ? cxg[(long long)gy * (n0 + 1)] : scx[fc];
    float cyh = (py && gy == n1 - 1) ? cyg[(long long)n1 * n0 + gx] : scy[c + LX];
    float cyl = (py && gy == 0) ? cyg[gx] : scy[c];
    float hi0 = (gx0 + lx + 1 >= n0 && !px) ? ghost_factor(P.bc, 0, 1) * p0 : se[c + 1];
    float lo0 = (gx0 + lx - 1 < 0 && !px) ? ghost_factor(P.bc, 0, 0) * p0 : se[c - 1];
    float hi1 = (gy0 + ly + 1 >= n1 && !py) ? ghost_factor(P.bc, 1, 1) * p0 : se[c + LX];
    float lo1 = (gy0 + ly - 1 < 0 && !py) ? ghost_factor(P.bc, 1, 0) * p0 : se[c - LX];
    float s = cxh * hi0;
    s = fmaf(cxl, lo0, s);
    s = fmaf(cyh, hi1, s);
    s = fmaf(cyl, lo1, s);
    return s;
  };

  for (int h = 0; h < P.n_half; h++) {
    const int pass = (P.pass0 + h) & 1;
    const int lo = h + 1, hx = LX - 2 - h, hy = LY - 2 - h;
    for (int ly = lo + ty; ly <= hy; ly += kTileTY) {
      const int gy = gy0 + ly;
      const int xs = lo + ((gx0 + lo + gy + pass) & 1);
      for (int lx = xs + 2 * tx; lx <= hx; lx += 2 * kTileTX) {
        const int c = ly * LX + lx;
        int gxv = gx0 + lx, gyv = gy;
        if (!inside) {
          gxv = gxw(gxv);
          gyv = gyw(gyv);
          if (gxv < 0 || gyv < 0) continue;
        }
        se[c] = sl[c] * (sr[c] + nbsum(lx, ly, gxv, gyv));
      }
    }
    __syncthreads();
  }

  for (int iy = ty; iy < kTileY; iy += kTileTY)
    for (int ix = tx; ix < kTileX; ix += kTileTX) {
      int gx = x0 + ix, gy = y0 + iy;
      if (gx < n0 && gy < n1) P.e_out[(long long)gy * n0 + gx] = se[(iy + H) * LX + ix + H];
    }

  // residual r - diag e + sum c e_nb, averaged onto the coarse cell
  if (P.rc) {
    const int cn0 = n0 >> 1, cn1 = n1 >> 1;
    for (int J = ty; J < kTileY / 2; J += kTileTY)
      for (int I = tx; I < kTileX / 2; I += kTileTX) {
        int CI = (x0 >> 1) + I, CJ = (y0 >> 1) + J;
        if (CI >= cn0 || CJ >= cn1) continue;
        float acc = 0.f;
        for (int jj = 0; jj < 2; jj++)
          for (int ii = 0; ii < 2; ii++) {
            int gx = 2 * CI + ii, gy = 2 * CJ + jj;
            int lx = gx - gx0, ly = gy - gy0;
            int c = ly * LX + lx;
            float res = sr[c] - P.K.diag[(long long)gy * n0 + gx] * se[c] + nbsum(lx, ly, gx, gy);
            acc = acc + res * 0.25f;
          }
        P.rc[(long long)CJ * cn0 + CI] = acc;
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
