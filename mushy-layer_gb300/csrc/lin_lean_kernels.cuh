// lin_lean_kernels.cuh -- lean FP32 kernels of the linear cycles inside the
// mixed-precision Newton solve of the (H, C) system, A x = g with A the
// Jacobian of the nonlinear operator at the current state:
//   (A x)_c = alpha a_c x_c - beta dxinv sum_f b_f,c (w_nb,c - w_c),  w = J x,
// J = d(T, C_l)/d(H, C) per cell.  Every wall ghost of w depends on the cell
// itself (the derived-variable rule on the centre's w, or the (H, C)
// condition mapped through the ghost state's Jacobian), so it lives in the
// cell's 2x2 diagonal block D, which the state set-up stores together with
// K = (D^T)^-1 (adj_minv_kernel, from the same device functions as the FP64
// operator).  What couples cells is then only
//   (A x)_j = D_j x_j - beta dxinv sum_(interior faces) b_f w_nb,
// interior meaning inside the box or across a periodic seam.  The kernels
// keep w = J x of every cell next to x, so a red/black update reads its own
// g, K and J, the neighbours' w and the face coefficients:
//   x_j = K_j^T (g_j + beta dxinv sum b_f w_nb),   w_j = J_j x_j,
// about half the loads and a fraction of the arithmetic of the generic
// linearised kernel (which forms J_nb x_nb for every neighbour), and the same
// update in exact arithmetic.  Residual (with a fused norm), restriction of
// the residual fused with the zeroing of the coarse unknowns, and
// prolongation fused with the refresh of w complete the cycle; the bottom
// solve is the generic one (its w is never read).  FP32 inside the FP64
// Newton loop: its residual, norm and update stay FP64.
#pragma once
#include "adjoint_kernels.cuh"

namespace mlgpu {

// T = float for the mixed-precision Newton cycles, double for the FP64
// comparison path built the same way
template <class T>
struct LinLeanT {
  Geom G;
  BCD ybc;           // wall rule of the prolongation
  T bdx;             // beta / dx^2
  const T *b[3];     // [2][faces_d] face coefficients
  const T *J;        // [4][cells] closure Jacobian (row-major 2x2 per cell)
  const T *K;        // [4][cells] (D^T)^-1
  const T *D;        // [4][cells] diagonal block of A (row-major)
  T *x, *w;          // [2][cells]: unknown and J x
  const T *g;        // [2][cells]: right-hand side
};
using LinLean = LinLeanT<float>;

__device__ __forceinline__ float fmaT(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fmaT(double a, double b, double c) { return fma(a, b, c); }

#ifdef MLGPU_ADJ_F32_UNIT
// s_c = sum over the interior faces of b_f,c w_nb,c (periodic seams wrap;
// a one-cell periodic direction couples the cell to itself and adds nothing)
template <class T, int DIM>
__device__ __forceinline__ void lean_nbsum(const LinLeanT<T> &P, int i, int j, int k,
                                           long long q, T s[2]) {
  const Geom &G = P.G;
  const long long n = G.ncell;
  const T *w = P.w;
  T s0 = T(0), s1 = T(0);
  {
    const long long f = ((long long)k * G.n1 + j) * (G.n0 + 1) + i;
    const long long nf = (long long)(G.n0 + 1) * G.n1 * G.n2;
    const long long ql = i > 0 ? q - 1 : (G.per0 && G.n0 > 1 ? q + (G.n0 - 1) : -1);
    const long long qh = i < G.n0 - 1 ? q + 1 : (G.per0 && G.n0 > 1 ? q - (G.n0 - 1) : -1);
    if (ql >= 0) {
      s0 = fmaT(P.b[0][f], w[ql], s0);
      s1 = fmaT(P.b[0][nf + f], w[n + ql], s1);
    }
    if (qh >= 0) {
      s0 = fmaT(P.b[0][f + 1], w[qh], s0);
      s1 = fmaT(P.b[0][nf + f + 1], w[n + qh], s1);
    }
  }
  {
    const long long s = G.n0;
    const long long f = ((long long)k * (G.n1 + 1) + j) * G.n0 + i;
    const long long nf = (long long)G.n0 * (G.n1 + 1) * G.n2;
    const long long ql = j > 0 ? q - s : (G.per1 && G.n1 > 1 ? q + (G.n1 - 1) * s : -1);
    const long long qh = j < G.n1 - 1 ? q + s : (G.per1 && G.n1 > 1 ? q - (G.n1 - 1) * s : -1);
    if (ql >= 0) {
      s0 = fmaT(P.b[1][f], w[ql], s0);
      s1 = fmaT(P.b[1][nf + f], w[n + ql], s1);
    }
    if (qh >= 0) {
      s0 = fmaT(P.b[1][f + s], w[qh], s0);
      s1 = fmaT(P.b[1][nf + f + s], w[n + qh], s1);
    }
  }
  if (DIM == 3) {
    const long long s = (long long)G.n0 * G.n1;
    const long long f = q;
    const long long nf = s * (G.n2 + 1);
    const long long ql = k > 0 ? q - s : (G.per2 && G.n2 > 1 ? q + (G.n2 - 1) * s : -1);
    const long long qh = k < G.n2 - 1 ? q + s : (G.per2 && G.n2 > 1 ? q - (G.n2 - 1) * s : -1);
    if (ql >= 0) {
      s0 = fmaT(P.b[2][f], w[ql], s0);
      s1 = fmaT(P.b[2][nf + f], w[n + ql], s1);
    }
    if (qh >= 0) {
      s0 = fmaT(P.b[2][f + s], w[qh], s0);
      s1 = fmaT(P.b[2][nf + f + s], w[n + qh], s1);
    }
  }
  s[0] = s0;
  s[1] = s1;
}

// red/black half sweep: x_j = K^T (g + bdx s), w_j = J x_j on the cells of
// colour `pass`
template <class T, int DIM>
__global__ void __launch_bounds__(kBlock) lean_gsrb_kernel(LinLeanT<T> P, int pass) {
  const Geom &G = P.G;
  const long long nt = colour_threads(G), n = G.ncell;
  for (long long t = gtid(); t < nt; t += gstride()) {
    int i, j, k;
    if (!colour_cell(G, pass, t, i, j, k)) continue;
    const long long q = G.cell(i, j, k);
    T s[2];
    lean_nbsum<T, DIM>(P, i, j, k, q, s);
    const T r0 = fmaT(P.bdx, s[0], P.g[q]), r1 = fmaT(P.bdx, s[1], P.g[n + q]);
    const T x0 = fmaT(P.K[q], r0, P.K[2 * n + q] * r1);
    const T x1 = fmaT(P.K[n + q], r0, P.K[3 * n + q] * r1);
    P.x[q] = x0;
    P.x[n + q] = x1;
    P.w[q] = fmaT(P.J[q], x0, P.J[n + q] * x1);
    P.w[n + q] = fmaT(P.J[2 * n + q], x0, P.J[3 * n + q] * x1);
  }
}

// g - A x at cell q (both components)
template <class T, int DIM>
__device__ __forceinline__ void lean_res(const LinLeanT<T> &P, int i, int j, int k, long long q,
                                         T r[2]) {
  const long long n = P.G.ncell;
  T s[2];
  lean_nbsum<T, DIM>(P, i, j, k, q, s);
  const T x0 = P.x[q], x1 = P.x[n + q];
  const T ax0 = fmaT(P.D[q], x0, P.D[n + q] * x1);
  const T ax1 = fmaT(P.D[2 * n + q], x0, P.D[3 * n + q] * x1);
  r[0] = fmaT(P.bdx, s[0], P.g[q]) - ax0;
  r[1] = fmaT(P.bdx, s[1], P.g[n + q]) - ax1;
}

// FP32 norm accumulation of one value (max keeps NaN, as norm_accum)
template <class T, int NORM>
__device__ __forceinline__ T lean_accum(T acc, T v) {
  if (NORM == MLGPU_NORM_MAX) {
    const T a = fabs(v);
    return (a > acc || a != a) ? a : acc;
  }
  if (NORM == MLGPU_NORM_L1) return acc + fabs(v);
  return fmaT(v, v, acc);
}

// out = g - A x with a fused norm of both components (partials per block).
// Each thread accumulates its few cells in T (for FP32: the values are FP32,
// a max is exact, a sum of a few dozen squares loses nothing that matters for
// the linear stopping test, and on GB300 an FP64 operation per cell would
// cost more than the cell's memory traffic); the block combines in FP64.
template <class T, int DIM, int NORM>
__global__ void __launch_bounds__(kBlock) lean_residual_kernel(LinLeanT<T> P, T *out,
                                                               double *part) {
  const Geom &G = P.G;
  const long long n = G.ncell;
  T acc = T(0);
  for (long long q = gtid(); q < n; q += gstride()) {
    int i, j, k;
    cell_ijk(G, q, i, j, k);
    T r[2];
    lean_res<T, DIM>(P, i, j, k, q, r);
    if (out) {
      out[q] = r[0];
      out[n + q] = r[1];
    }
    acc = lean_accum<T, NORM>(acc, r[0]);
    acc = lean_accum<T, NORM>(acc, r[1]);
  }
  const double v = block_reduce<NORM>((double)acc);
  if (threadIdx.x == 0) part[blockIdx.x] = v;
}

// coarse g = 2^D average of the fine residual; the coarse x and w start at 0
template <class T, int DIM>
__global__ void __launch_bounds__(kBlock) lean_restrict_kernel(LinLeanT<T> P, Geom C, T *gc,
                                                               T *xc, T *wc) {
  const long long nc = C.ncell;
  const T wgt = DIM == 3 ? T(0.125) : T(0.25);
  for (long long Q = gtid(); Q < nc; Q += gstride()) {
    int I, J, K;
    cell_ijk(C, Q, I, J, K);
    T a0 = T(0), a1 = T(0);
#pragma unroll
    for (int kk = 0; kk < (DIM == 3 ? 2 : 1); kk++)
#pragma unroll
      for (int jj = 0; jj < 2; jj++)
#pragma unroll
        for (int ii = 0; ii < 2; ii++) {
          const int i = 2 * I + ii, j = 2 * J + jj, k = DIM == 3 ? 2 * K + kk : 0;
          T r[2];
          lean_res<T, DIM>(P, i, j, k, P.G.cell(i, j, k), r);
          a0 += r[0];
          a1 += r[1];
        }
    gc[Q] = a0 * wgt;
    gc[nc + Q] = a1 * wgt;
    xc[Q] = T(0);
    xc[nc + Q] = T(0);
    wc[Q] = T(0);
    wc[nc + Q] = T(0);
  }
}

// x += prolongation of the coarse correction; w = J x
template <class T, int DIM, int KIND>
__global__ void __launch_bounds__(kBlock) lean_prolong_kernel(LinLeanT<T> P, Geom C,
                                                              const T *__restrict__ xc) {
  const Geom &G = P.G;
  const long long n = G.ncell;
  for (long long q = gtid(); q < n; q += gstride()) {
    int i, j, k;
    cell_ijk(G, q, i, j, k);
    const T x0 = prolong_add<T, DIM, KIND>(C, P.ybc, 0, i, j, k, P.x[q], xc, nullptr);
    const T x1 = prolong_add<T, DIM, KIND>(C, P.ybc, 1, i, j, k, P.x[n + q], xc, nullptr);
    P.x[q] = x0;
    P.x[n + q] = x1;
    P.w[q] = fmaT(P.J[q], x0, P.J[n + q] * x1);
    P.w[n + q] = fmaT(P.J[2 * n + q], x0, P.J[3 * n + q] * x1);
  }
}
#endif  // MLGPU_ADJ_F32_UNIT

// ---- one full red + black sweep per launch in 3D (z-march) ----------------
// A half-sweep launch touches every cache line of every array although it
// updates half the cells, so a sweep costs two passes over memory.  Here one
// thread block owns an x-y tile and marches up a chunk of planes; at the step
// that brings plane t in, it updates the red cells of plane t-1 (their black
// neighbours in planes t-2..t are still old) and then the black cells of
// plane t-2 (their red neighbours in planes t-3..t-1 are now new): exactly
// the red-then-black sweep, with the old/new w of four planes staged in
// shared memory and each array read once.  Black cells at the tile edge need
// updated red neighbours of the next tile, so the red pass also runs on a
// one-cell ring around the tile (and one plane below / above the chunk) from
// the same old data: redundant work, identical values, no dependence on
// block order.  The launch reads (x, w) and writes (x_out, w_out), so no block
// sees another's new values; every cell of the box is written once.  The
// arithmetic is that of lean_gsrb_kernel in the same order (a neighbour
// outside the box contributes b * 0), so one launch gives the bits of the
// red and black half sweeps it replaces.  Non-periodic z only (the planes
// beyond the walls are zero).
constexpr int kZMTX = 30, kZMTY = 14;                    // output tile
constexpr int kZMRX = kZMTX + 2, kZMRY = kZMTY + 2;      // red region: one thread per column
constexpr int kZMWX = kZMTX + 4, kZMWY = kZMTY + 4;      // w region (red region + its neighbours)
constexpr int kZMThreads = kZMRX * kZMRY;                // 512
constexpr int kZMChunk = 32;                             // planes per block

template <class T>
struct LeanSweep3T {
  LinLeanT<T> P;         // x, w: input of the sweep
  T *x_out, *w_out;      // output of the sweep
  int ntx, nty, nchunk;
};
using LeanSweep3 = LeanSweep3T<float>;

#ifdef MLGPU_ADJ_F32_UNIT
// FP32: two blocks per SM; FP64 (twice the registers and shared memory): one
template <class T>
__global__ void __launch_bounds__(kZMThreads, sizeof(T) == 4 ? 2 : 1)
    lean_sweep3_kernel(LeanSweep3T<T> S) {
  __shared__ T sw[4][2][kZMWY * kZMWX];
  const LinLeanT<T> &P = S.P;
  const Geom &G = P.G;
  const int n0 = G.n0, n1 = G.n1, n2 = G.n2;
  const long long n = G.ncell, plane = (long long)n0 * n1;
  const long long nfx = G.nface(0), nfy = G.nface(1), nfz = G.nface(2);
  int item = blockIdx.x;
  const int tx = item % S.ntx;
  item /= S.ntx;
  const int ty = item % S.nty, cz = item / S.nty;
  const int x0 = tx * kZMTX, y0 = ty * kZMTY, z0 = cz * kZMChunk;
  const int z1 = min(z0 + kZMChunk, n2);
  const int lx = threadIdx.x % kZMRX, ly = threadIdx.x / kZMRX;
  int gx = x0 - 1 + lx, gy = y0 - 1 + ly;
  const bool interior = lx >= 1 && lx <= kZMTX && ly >= 1 && ly <= kZMTY && gx < n0 && gy < n1;
  bool valid = true;
  if (gx < 0 || gx >= n0) {
    if (G.per0)
      gx = ((gx % n0) + n0) % n0;
    else
      valid = false;
  }
  if (gy < 0 || gy >= n1) {
    if (G.per1)
      gy = ((gy % n1) + n1) % n1;
    else
      valid = false;
  }
  const long long col = valid ? (long long)gy * n0 + gx : 0;
  const int wc = (ly + 1) * kZMWX + (lx + 1);
  const int tb = z0 - 2, te = z1 + 1;
  T Tn[10], R[10], B[10];
#pragma unroll
  for (int m = 0; m < 10; m++) Tn[m] = R[m] = B[m] = T(0);

  // the update of this column's cell at plane p: own data D (g, K, J), w of
  // planes p-1, p, p+1 in shared memory
  auto update = [&](int p, const T *D, T &xo0, T &xo1, T &wo0, T &wo1) {
    const int sm = (p - 1 - tb) & 3, s0 = (p - tb) & 3, sp = (p + 1 - tb) & 3;
    const long long cp = col + (long long)p * plane;
    const long long fx = ((long long)p * n1 + gy) * (n0 + 1) + gx;
    const long long fy = ((long long)p * (n1 + 1) + gy) * n0 + gx;
    T s[2];
#pragma unroll
    for (int c = 0; c < 2; c++) {
      const T *w0 = sw[s0][c];
      T a = P.b[0][c * nfx + fx] * w0[wc - 1];
      a = fmaT(P.b[0][c * nfx + fx + 1], w0[wc + 1], a);
      a = fmaT(P.b[1][c * nfy + fy], w0[wc - kZMWX], a);
      a = fmaT(P.b[1][c * nfy + fy + n0], w0[wc + kZMWX], a);
      a = fmaT(P.b[2][c * nfz + cp], sw[sm][c][wc], a);
      a = fmaT(P.b[2][c * nfz + cp + plane], sw[sp][c][wc], a);
      s[c] = a;
    }
    const T r0 = fmaT(P.bdx, s[0], D[0]), r1 = fmaT(P.bdx, s[1], D[1]);
    xo0 = fmaT(D[2], r0, D[4] * r1);
    xo1 = fmaT(D[3], r0, D[5] * r1);
    wo0 = fmaT(D[6], xo0, D[7] * xo1);
    wo1 = fmaT(D[8], xo0, D[9] * xo1);
  };

  for (int t = tb; t <= te; t++) {
    const int slot = (t - tb) & 3;
    const bool pin = t >= 0 && t < n2;
    // w of plane t over the w region (zero outside the box)
    for (int idx = threadIdx.x; idx < kZMWX * kZMWY; idx += kZMThreads) {
      int ax = x0 - 2 + idx % kZMWX, ay = y0 - 2 + idx / kZMWX;
      bool ok = pin;
      if (ax < 0 || ax >= n0) {
        if (G.per0)
          ax = ((ax % n0) + n0) % n0;
        else
          ok = false;
      }
      if (ay < 0 || ay >= n1) {
        if (G.per1)
          ay = ((ay % n1) + n1) % n1;
        else
          ok = false;
      }
      const long long q = (long long)t * plane + (long long)ay * n0 + ax;
      sw[slot][0][idx] = ok ? P.w[q] : T(0);
      sw[slot][1][idx] = ok ? P.w[n + q] : T(0);
    }
    // this column's own data of plane t: g (2), K (4), J (4)
    const bool own = valid && pin && t >= z0 - 1 && t <= z1;
    if (own) {
      const long long q = col + (long long)t * plane;
      Tn[0] = P.g[q];
      Tn[1] = P.g[n + q];
      Tn[2] = P.K[q];
      Tn[3] = P.K[n + q];
      Tn[4] = P.K[2 * n + q];
      Tn[5] = P.K[3 * n + q];
      Tn[6] = P.J[q];
      Tn[7] = P.J[n + q];
      Tn[8] = P.J[2 * n + q];
      Tn[9] = P.J[3 * n + q];
    }
    __syncthreads();
    // red cells of plane t-1 (on the tile and its ring; the chunk +- a plane)
    const int p = t - 1;
    if (valid && p >= 0 && p < n2 && p >= z0 - 1 && p <= z1 && ((gx + gy + p) & 1) == 0) {
      T xa, xb, wa, wb;
      update(p, R, xa, xb, wa, wb);
      const int s0 = (p - tb) & 3;
      sw[s0][0][wc] = wa;
      sw[s0][1][wc] = wb;
      if (interior && p >= z0 && p < z1) {
        const long long q = col + (long long)p * plane;
        S.x_out[q] = xa;
        S.x_out[n + q] = xb;
        S.w_out[q] = wa;
        S.w_out[n + q] = wb;
      }
    }
    __syncthreads();
    // black cells of plane t-2 (on the tile)
    const int p2 = t - 2;
    if (interior && p2 >= z0 && p2 < z1 && ((gx + gy + p2) & 1) == 1) {
      T xa, xb, wa, wb;
      update(p2, B, xa, xb, wa, wb);
      const long long q = col + (long long)p2 * plane;
      S.x_out[q] = xa;
      S.x_out[n + q] = xb;
      S.w_out[q] = wa;
      S.w_out[n + q] = wb;
    }
    // plane t's data waits for its red step (t+1) or its black step (t+2)
    if (own) {
      if (((gx + gy + t) & 1) == 0) {
#pragma unroll
        for (int m = 0; m < 10; m++) R[m] = Tn[m];
      } else {
#pragma unroll
        for (int m = 0; m < 10; m++) B[m] = Tn[m];
      }
    }
    __syncthreads();
  }
}
#endif  // MLGPU_ADJ_F32_UNIT

}  // namespace mlgpu
