// tile_kernels.cuh -- temporal blocking of the red/black smoother on 2D
// levels.  One launch performs, for a TX x TY tile of the level:
//   [zero-init | load e] -> [e += P e_coarse] -> n red/black half sweeps ->
//   [residual restricted to the coarse level]
// with the tile and a halo of H >= n (+1 with the restriction) cells held in
// shared memory.  After half sweep h only cells at least h+1 cells inside the
// loaded halo are valid, so the tile interior ends exact.  Halo cells are
// recomputed by every tile that loads them with the same operands, hence
// with the same bits: results equal the per-level kernels launched one
// after another (relax, restrictResidual, prolongIncrement, relax).
#pragma once
#include "vc_kernels.cuh"
#include "misc_kernels.cuh"

namespace mlgpu {

// The correction is read from `e_in` and written to `e_out`, never the same
// buffer: a block loads its halo from cells other blocks own and write back,
// so an in-place update would race with blocks of a later wave.
template <class T>
struct TileSmooth {
  VCArgs<T> A;        // level operator; A.lam null: 1/diag computed at load
  const T *e_in;      // level correction before (unused with zero_init)
  T *e_out;           // level correction after (interior cells of every tile)
  const T *r;         // level right-hand side
  int zero_init;      // e starts at zero instead of being loaded
  int n_half;         // red/black half sweeps
  int pass0;          // colour of the first half sweep (0 red, 1 black)
  int halo;           // loaded halo width H
  T *rc;              // restricted residual output (coarse level) or null
  int prolong;        // -1: none, else MLGPU_PROLONG_* from ec
  const T *ec;        // coarse correction for the prolongation
};

// Small interior tiles with a wide halo: every level gets many blocks and each
// thread updates about one cell per half sweep; the redundant halo work is
// cheap next to the latency it removes.  Threads are laid out 16 x 32.
constexpr int kTileX = 16, kTileY = 16, kTileThreads = 512;
constexpr int kTileTX = 16, kTileTY = 32;

inline size_t tile_smem_bytes(int halo, size_t elem) {
  size_t lx = kTileX + 2 * halo, ly = kTileY + 2 * halo;
  return elem * (3 * lx * ly + (lx + 1) * ly + lx * (ly + 1));
}

template <class T>
__global__ void __launch_bounds__(kTileThreads) vc_tile_smooth_kernel(TileSmooth<T> P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const VCArgs<T> &A = P.A;
  const Geom &G = A.G;
  const int H = P.halo;
  const int LX = kTileX + 2 * H, LY = kTileY + 2 * H;
  T *se = (T *)smem_raw;
  T *sr = se + LX * LY;
  T *sl = sr + LX * LY;
  T *sbx = sl + LX * LY;           // (LX+1) x LY, face lx between local cells lx-1, lx
  T *sby = sbx + (LX + 1) * LY;    // LX x (LY+1)
  const int x0 = blockIdx.x * kTileX, y0 = blockIdx.y * kTileY;
  const int gx0 = x0 - H, gy0 = y0 - H;
  const int n0 = G.n0, n1 = G.n1;
  const bool px = G.per0 != 0, py = G.per1 != 0;
  const int tx = threadIdx.x, ty = threadIdx.y;
  // whole loaded region inside the box: no wrap, no boundary, no seam faces
  const bool inside = gx0 >= 0 && gx0 + LX <= n0 && gy0 >= 0 && gy0 + LY <= n1;

  // wrapped global coordinate, or -1 when outside a non-periodic domain
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
  // Faces of the cell at local (lx, ly) with wrapped global (gx, gy).  The
  // shared arrays are positional; in a periodic direction the box keeps two
  // entries for the seam face (face 0 for cell 0, face n for cell n-1), so the
  // seam cells read their own entry from global memory, exactly as the
  // per-level kernels index faces by the cell's own coordinates.
  auto fxl = [&](int lx, int ly, int gx, int gy) -> T {
    return (px && gx == 0) ? A.b[0][(long long)gy * (n0 + 1)] : sbx[ly * (LX + 1) + lx];
  };
  auto fxh = [&](int lx, int ly, int gx, int gy) -> T {
    return (px && gx == n0 - 1) ? A.b[0][(long long)gy * (n0 + 1) + n0]
                                : sbx[ly * (LX + 1) + lx + 1];
  };
  auto fyl = [&](int lx, int ly, int gx, int gy) -> T {
    return (py && gy == 0) ? A.b[1][gx] : sby[ly * LX + lx];
  };
  auto fyh = [&](int lx, int ly, int gx, int gy) -> T {
    return (py && gy == n1 - 1) ? A.b[1][(long long)n1 * n0 + gx] : sby[(ly + 1) * LX + lx];
  };

  // ---- load faces, then cells (e, r, 1/diag)
  for (int ly = ty; ly < LY; ly += kTileTY)
    for (int lx = tx; lx <= LX; lx += kTileTX) {
      T v = T(0);
      int gy = inside ? gy0 + ly : gyw(gy0 + ly);
      if (gy >= 0) {
        int fx = gx0 + lx;
        if (fx < 0 || fx > n0) fx = px ? ((fx % n0) + n0) % n0 : -1;
        if (fx >= 0) v = A.b[0][(long long)gy * (n0 + 1) + fx];
      }
      sbx[ly * (LX + 1) + lx] = v;
    }
  for (int ly = ty; ly <= LY; ly += kTileTY)
    for (int lx = tx; lx < LX; lx += kTileTX) {
      T v = T(0);
      int gx = inside ? gx0 + lx : gxw(gx0 + lx);
      if (gx >= 0) {
        int fy = gy0 + ly;
        if (fy < 0 || fy > n1) fy = py ? ((fy % n1) + n1) % n1 : -1;
        if (fy >= 0) v = A.b[1][(long long)fy * n0 + gx];
      }
      sby[ly * LX + lx] = v;
    }
  __syncthreads();
  const Geom Cg = coarsen_geom(G);
  for (int ly = ty; ly < LY; ly += kTileTY)
    for (int lx = tx; lx < LX; lx += kTileTX) {
      int q = ly * LX + lx;
      int gx = inside ? gx0 + lx : gxw(gx0 + lx), gy = inside ? gy0 + ly : gyw(gy0 + ly);
      T ev = T(0), rv = T(0), lv = T(0);
      if (gx >= 0 && gy >= 0) {
        long long gq = (long long)gy * n0 + gx;
        if (!P.zero_init) ev = P.e_in[gq];
        rv = P.r[gq];
        if (A.lam) {
          lv = A.lam[gq];
        } else {
          lv = vc_lambda_at<T, 2>(A, gq, fxh(lx, ly, gx, gy), fxl(lx, ly, gx, gy),
                                  fyh(lx, ly, gx, gy), fyl(lx, ly, gx, gy), T(0), T(0));
        }
        if (P.prolong == MLGPU_PROLONG_LINEAR)
          ev = prolong_add<T, 2, MLGPU_PROLONG_LINEAR>(Cg, A.bc, 0, gx, gy, 0, ev, P.ec, nullptr);
        else if (P.prolong == MLGPU_PROLONG_CONSTANT)
          ev = prolong_add<T, 2, MLGPU_PROLONG_CONSTANT>(Cg, A.bc, 0, gx, gy, 0, ev, P.ec, nullptr);
      }
      se[q] = ev;
      sr[q] = rv;
      sl[q] = lv;
    }
  __syncthreads();

  // L(e) at local (lx, ly), global (gx, gy), homogeneous BCs; same operation
  // order as vc_lofphi.  INSIDE: every neighbour is a loaded interior cell and
  // every face positional.
  auto lofphi_in = [&](int lx, int ly, long long gq, T &p0) -> T {
    int c = ly * LX + lx;
    p0 = se[c];
    T lo0 = se[c - 1], hi0 = se[c + 1], lo1 = se[c - LX], hi1 = se[c + LX];
    int fc = ly * (LX + 1) + lx;
    T bxh = sbx[fc + 1], bxl = sbx[fc];
    T byh = sby[c + LX], byl = sby[c];
    T s = bxh * (hi0 - p0) - bxl * (p0 - lo0);
    s = s + byh * (hi1 - p0);
    s = s - byl * (p0 - lo1);
    T av = A.a ? A.a[gq] : T(1);
    T v = A.alpha * av * p0;
    if (A.c) v = v - A.beta * A.c[gq] * p0;
    v = v - A.beta * s * A.dxinv;
    return v;
  };
  auto lofphi = [&](int lx, int ly, int gx, int gy, T &p0) -> T {
    int c = ly * LX + lx;
    p0 = se[c];
    T lo0 = (gx0 + lx - 1 < 0 && !px) ? ghost_value<T>(A.bc, 0, 0, 0, p0, A.dx, true) : se[c - 1];
    T hi0 = (gx0 + lx + 1 >= n0 && !px) ? ghost_value<T>(A.bc, 0, 1, 0, p0, A.dx, true) : se[c + 1];
    T lo1 = (gy0 + ly - 1 < 0 && !py) ? ghost_value<T>(A.bc, 1, 0, 0, p0, A.dx, true) : se[c - LX];
    T hi1 = (gy0 + ly + 1 >= n1 && !py) ? ghost_value<T>(A.bc, 1, 1, 0, p0, A.dx, true) : se[c + LX];
    T bxh = fxh(lx, ly, gx, gy), bxl = fxl(lx, ly, gx, gy);
    T byh = fyh(lx, ly, gx, gy), byl = fyl(lx, ly, gx, gy);
    T s = bxh * (hi0 - p0) - bxl * (p0 - lo0);
    s = s + byh * (hi1 - p0);
    s = s - byl * (p0 - lo1);
    long long gq = (long long)gy * n0 + gx;
    T av = A.a ? A.a[gq] : T(1);
    T v = A.alpha * av * p0;
    if (A.c) v = v - A.beta * A.c[gq] * p0;
    v = v - A.beta * s * A.dxinv;
    return v;
  };

  // ---- red/black half sweeps over the shrinking valid region
  for (int h = 0; h < P.n_half; h++) {
    const int pass = (P.pass0 + h) & 1;
    const int lo = h + 1, hx = LX - 2 - h, hy = LY - 2 - h;
    for (int ly = lo + ty; ly <= hy; ly += kTileTY) {
      const int gy = gy0 + ly;
      // first local x in [lo, hx] whose global parity matches the pass
      const int xs = lo + ((gx0 + lo + gy + pass) & 1);
      for (int lx = xs + 2 * tx; lx <= hx; lx += 2 * kTileTX) {
        const int c = ly * LX + lx;
        T p0, lof;
        if (inside) {
          lof = lofphi_in(lx, ly, (long long)gy * n0 + gx0 + lx, p0);
        } else {
          int gxv = gxw(gx0 + lx), gyv = gyw(gy);
          if (gxv < 0 || gyv < 0) continue;
          lof = lofphi(lx, ly, gxv, gyv, p0);
        }
        se[c] = p0 - sl[c] * (lof - sr[c]);
      }
    }
    __syncthreads();
  }

  // ---- write the interior back
  for (int iy = ty; iy < kTileY; iy += kTileTY)
    for (int ix = tx; ix < kTileX; ix += kTileTX) {
      int gx = x0 + ix, gy = y0 + iy;
      if (gx < n0 && gy < n1) P.e_out[(long long)gy * n0 + gx] = se[(iy + H) * LX + ix + H];
    }

  // ---- residual of the interior, restricted to the coarse level
  if (P.rc) {
    const T denom = T(4);
    const int cn0 = n0 >> 1, cn1 = n1 >> 1;
    for (int J = ty; J < kTileY / 2; J += kTileTY)
      for (int I = tx; I < kTileX / 2; I += kTileTX) {
        int CI = (x0 >> 1) + I, CJ = (y0 >> 1) + J;
        if (CI >= cn0 || CJ >= cn1) continue;
        T acc = T(0);
        for (int jj = 0; jj < 2; jj++)
          for (int ii = 0; ii < 2; ii++) {
            int gx = 2 * CI + ii, gy = 2 * CJ + jj;
            int lx = gx - gx0, ly = gy - gy0;
            T p0;
            T lof = inside ? lofphi_in(lx, ly, (long long)gy * n0 + gx, p0)
                           : lofphi(lx, ly, gx, gy, p0);
            acc = acc + (sr[ly * LX + lx] - lof) / denom;
          }
        P.rc[(long long)CJ * cn0 + CI] = acc;
      }
  }
}

}  // namespace mlgpu
