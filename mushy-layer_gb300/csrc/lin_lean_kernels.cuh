// lin_lean_kernels.cuh -- lean kernels of the linear cycles inside the Newton
// solve of the (H, C) system, A x = g with A the Jacobian of the nonlinear
// operator at the current state:
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
// solve is the generic one (its w is never read).
//
// Layout.  The per-cell arrays the smoother updates or reads for its own
// cells -- x, w, g, J, K, D -- are stored colour-split on every smoothed
// level (cs_index: the cells of colour (i + j + k) & 1 in their own half,
// row by row).  A half sweep then streams its own colour's g, K, J and the
// other colour's w, every face coefficient once (the face arrays keep their
// natural layout: each face borders one cell of each colour), and writes its
// own colour's x and w: its DRAM traffic is its compulsory bytes.  In the
// natural layout the two colours share every cache line and a half sweep
// moves 1.7x as much.  The bottom level keeps the natural layout of the
// generic kernels; the restriction into it and the prolongation out of it
// index it so.  J, K, D are computed in the natural layout and permuted once
// per Newton state (lean_pack_kernel); the Newton update reads the split
// correction (lean_step_kernel).  A one-level hierarchy keeps the natural
// layout throughout (its only level is the bottom's).
//
// T = float for the mixed-precision cycles (the FP64 Newton loop keeps its
// residual, norm and update), double for the FP64 comparison path built
// the same way.
#pragma once
#include "adjoint_kernels.cuh"

namespace mlgpu {

// Regime test of the Newton update's clipping.  The common case in FP32
// (bounding energies with the divisions by constants as products with their
// reciprocals); a cell within 1e-4 of a bound, or whose FP32 regime changes,
// is decided again in FP64 by t_cl's own test (closure_regime), and clipped
// at the FP64 bound: a clip at an FP32-rounded bound would pin a cell that
// converges onto a phase boundary 1e-7 away from its solution.
struct StepClip {
  float CR, cp, St, te, Te, inv_k, inv_CRTe, frac;
  ClosureParams p;              // the closure's own parameters (FP64 decisions)
  double inv_k64, inv_CRTe64;   // 1/k, 1/(CR + Te) in FP64
  __host__ __device__ int regime32(float H, float C, float b[3]) const {
    float Hs = (C < -CR) ? 0.f : cp * ((-C - CR) * inv_k);
    if (Hs < 0.f) Hs = 0.f;
    b[0] = Hs + te * cp;
    b[1] = (CR + C) * inv_CRTe * (St + te * (1.f - cp)) + cp * te;
    b[2] = St - C + te + Te;
    return H <= b[0] ? 0 : (H <= b[1] ? 1 : (H < b[2] ? 2 : 3));
  }
  __host__ __device__ static bool near(float H, const float b[3]) {
    const float band = 1e-4f;
    return fabsf(H - b[0]) < band * (1.f + fabsf(b[0])) ||
           fabsf(H - b[1]) < band * (1.f + fabsf(b[1])) ||
           fabsf(H - b[2]) < band * (1.f + fabsf(b[2]));
  }
};

#ifdef MLGPU_ADJ_F32_UNIT
// The FP64 decision of the clipping for a cell near a regime bound: the
// bounds with the constant divisors as reciprocals (to an ulp of the
// closure's own; a cell an ulp from a bound may take either side), h1 clipped
// past the first bound crossed.  Out of line: the regime-clipped update
// leaves many cells near a bound, and inline FP64 code here would lower the
// kernel's occupancy.
static __device__ __noinline__ double step_clip_near(double h0, double c0, double h1, double c1,
                                                     const StepClip &K) {
  const ClosureParams &p = K.p;
  auto bounds = [&](double C, double B[3]) {
    double Hs = (C < -p.CR) ? 0.0 : p.cp * ((-C - p.CR) * K.inv_k64);
    if (Hs < 0.0) Hs = 0.0;
    B[0] = Hs + p.te * p.cp;
    B[1] = (p.CR + C) * K.inv_CRTe64 * (p.St + p.te * (1 - p.cp)) + p.cp * p.te;
    B[2] = p.St - C + p.te + p.Te;
  };
  auto regime = [](double H, const double B[3]) {
    if (H <= B[0]) return 0;
    if (H > B[0] && H <= B[1]) return 1;
    if (H > B[1] && H < B[2]) return 2;
    if (H >= B[2]) return 3;
    return 4;
  };
  double B0[3], B1[3];
  bounds(c0, B0);
  bounds(c1, B1);
  const int r0 = regime(h0, B0), r1 = regime(h1, B1);
  if (r0 != r1 && r0 < 4 && r1 < 4) {
    const double bnd = B1[r1 > r0 ? r0 : r0 - 1];
    return bnd + (double)K.frac * (h1 - bnd);
  }
  return h1;
}
#endif

template <class T>
struct LinLeanT {
  Geom G;
  BCD ybc;           // wall rule of the prolongation
  T bdx;             // beta / dx^2
  const T *b[3];     // [2][faces_d] face coefficients (natural face layout)
  const T *J;        // [4][cells] closure Jacobian (row-major 2x2 per cell), split
  const T *K;        // [4][cells] (D^T)^-1, split
  const T *D;        // [4][cells] diagonal block of A (row-major), split
  T *x, *w;          // [2][cells]: unknown and J x, split
  const T *g;        // [2][cells]: right-hand side, split
};
using LinLean = LinLeanT<float>;

__device__ __forceinline__ float fmaT(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fmaT(double a, double b, double c) { return fma(a, b, c); }

#ifdef MLGPU_ADJ_F32_UNIT
// s_c = sum over the interior faces of b_f,c w_nb,c (periodic seams wrap;
// a one-cell periodic direction couples the cell to itself and adds nothing);
// IDX: the level's cell layout
template <class T, int DIM, class IDX>
__device__ __forceinline__ void lean_nbsum(const LinLeanT<T> &P, int i, int j, int k, T s[2]) {
  const Geom &G = P.G;
  const IDX at;
  const long long n = G.ncell;
  const T *w = P.w;
  T s0 = T(0), s1 = T(0);
  {
    const long long f = ((long long)k * G.n1 + j) * (G.n0 + 1) + i;
    const long long nf = (long long)(G.n0 + 1) * G.n1 * G.n2;
    const int il = i > 0 ? i - 1 : (G.per0 && G.n0 > 1 ? G.n0 - 1 : -1);
    const int ih = i < G.n0 - 1 ? i + 1 : (G.per0 && G.n0 > 1 ? 0 : -1);
    if (il >= 0) {
      const long long q = at(G, il, j, k);
      s0 = fmaT(P.b[0][f], w[q], s0);
      s1 = fmaT(P.b[0][nf + f], w[n + q], s1);
    }
    if (ih >= 0) {
      const long long q = at(G, ih, j, k);
      s0 = fmaT(P.b[0][f + 1], w[q], s0);
      s1 = fmaT(P.b[0][nf + f + 1], w[n + q], s1);
    }
  }
  {
    const long long f = ((long long)k * (G.n1 + 1) + j) * G.n0 + i;
    const long long nf = (long long)G.n0 * (G.n1 + 1) * G.n2;
    const int jl = j > 0 ? j - 1 : (G.per1 && G.n1 > 1 ? G.n1 - 1 : -1);
    const int jh = j < G.n1 - 1 ? j + 1 : (G.per1 && G.n1 > 1 ? 0 : -1);
    if (jl >= 0) {
      const long long q = at(G, i, jl, k);
      s0 = fmaT(P.b[1][f], w[q], s0);
      s1 = fmaT(P.b[1][nf + f], w[n + q], s1);
    }
    if (jh >= 0) {
      const long long q = at(G, i, jh, k);
      s0 = fmaT(P.b[1][f + G.n0], w[q], s0);
      s1 = fmaT(P.b[1][nf + f + G.n0], w[n + q], s1);
    }
  }
  if (DIM == 3) {
    const long long pl = (long long)G.n0 * G.n1;
    const long long f = ((long long)k * G.n1 + j) * G.n0 + i;
    const long long nf = pl * (G.n2 + 1);
    const int kl = k > 0 ? k - 1 : (G.per2 && G.n2 > 1 ? G.n2 - 1 : -1);
    const int kh = k < G.n2 - 1 ? k + 1 : (G.per2 && G.n2 > 1 ? 0 : -1);
    if (kl >= 0) {
      const long long q = at(G, i, j, kl);
      s0 = fmaT(P.b[2][f], w[q], s0);
      s1 = fmaT(P.b[2][nf + f], w[n + q], s1);
    }
    if (kh >= 0) {
      const long long q = at(G, i, j, kh);
      s0 = fmaT(P.b[2][f + pl], w[q], s0);
      s1 = fmaT(P.b[2][nf + f + pl], w[n + q], s1);
    }
  }
  s[0] = s0;
  s[1] = s1;
}

// red/black half sweep over the cells of colour `pass` (the contiguous half
// pass * n/2 .. of the split arrays): x_j = K^T (g + bdx s), w_j = J x_j
template <class T, int DIM>
__global__ void __launch_bounds__(kBlock) lean_gsrb_kernel(LinLeanT<T> P, int pass) {
  const Geom &G = P.G;
  const long long n = G.ncell, half = n >> 1;
  for (long long t = gtid(); t < half; t += gstride()) {
    const long long q = pass * half + t;
    int i, j, k;
    cs_cell(G, q, i, j, k);
    T s[2];
    lean_nbsum<T, DIM, SplitIdx>(P, i, j, k, s);
    const T r0 = fmaT(P.bdx, s[0], P.g[q]), r1 = fmaT(P.bdx, s[1], P.g[n + q]);
    const T x0 = fmaT(P.K[q], r0, P.K[2 * n + q] * r1);
    const T x1 = fmaT(P.K[n + q], r0, P.K[3 * n + q] * r1);
    P.x[q] = x0;
    P.x[n + q] = x1;
    P.w[q] = fmaT(P.J[q], x0, P.J[n + q] * x1);
    P.w[n + q] = fmaT(P.J[2 * n + q], x0, P.J[3 * n + q] * x1);
  }
}

// The same half sweep with V = 16 / sizeof(T) consecutive cells of one row of
// the colour's half per thread (4 in FP32, 2 in FP64): the cells' own g, K,
// J, the y and z neighbours' w (the same positions in the neighbouring rows of
// the other half) as 16-byte vector loads, the x neighbours' w as one vector
// and one scalar, x and w stored as vectors.  Each cell's arithmetic is
// lean_gsrb_kernel's in the same order (the same bits).  Needs n0 / 2 a
// multiple of V (then so are the row starts, the half and the array offsets).
template <class T>
struct Vec16;
template <>
struct Vec16<float> {
  using type = float4;
  static constexpr int V = 4;
};
template <>
struct Vec16<double> {
  using type = double2;
  static constexpr int V = 2;
};

template <class T>
__device__ __forceinline__ void ldv(const T *__restrict__ p, T *out) {
  using VT = typename Vec16<T>::type;
  const VT v = *reinterpret_cast<const VT *>(p);
  if constexpr (Vec16<T>::V == 4) {
    out[0] = v.x;
    out[1] = v.y;
    out[2] = v.z;
    out[3] = v.w;
  } else {
    out[0] = v.x;
    out[1] = v.y;
  }
}

template <class T>
__device__ __forceinline__ void stv(T *__restrict__ p, const T *in) {
  using VT = typename Vec16<T>::type;
  VT v;
  if constexpr (Vec16<T>::V == 4) {
    v.x = in[0];
    v.y = in[1];
    v.z = in[2];
    v.w = in[3];
  } else {
    v.x = in[0];
    v.y = in[1];
  }
  *reinterpret_cast<VT *>(p) = v;
}

// The neighbour sums s_c = sum over interior faces of b_f,c w_nb,c of the V
// cells hh .. hh + V - 1 of colour `pass` in row `row` = (j, k) of a split
// level (the other colour's w around them: one vector load per row and
// component, the row's extra value for x), lean_nbsum's order term by term,
// so the same bits.
template <class T, int DIM>
__device__ __forceinline__ void lean_vsum(const LinLeanT<T> &P, int pass, unsigned row, int hh,
                                          int j, int k, T *s0, T *s1) {
  constexpr int V = Vec16<T>::V;
  const Geom &G = P.G;
  const long long n = G.ncell, half = n >> 1;
  const int h0 = G.n0 >> 1;
  const long long obase = half - pass * half;  // the other colour's half
  const long long nf0 = (long long)(G.n0 + 1) * G.n1 * G.n2;
  const long long nf1 = (long long)G.n0 * (G.n1 + 1) * G.n2;
  const long long pl = (long long)G.n0 * G.n1, nf2 = pl * (G.n2 + 1);
  const T *w = P.w;
  const int par = (j + k + pass) & 1;  // i of the group's first cell = 2 hh + par
#pragma unroll
  for (int v = 0; v < V; v++) s0[v] = s1[v] = T(0);
  // x: the other colour's w at hh - 1 + par .. hh + V - 1 + par of this row
  {
    const long long ob = obase + (long long)row * h0;
    T wv0[V], wv1[V];
    ldv(w + ob + hh, wv0);
    ldv(w + n + ob + hh, wv1);
    // the extra value: hh - 1 (par 0) or hh + V (par 1), wrapped when periodic
    int xe = par ? hh + V : hh - 1;
    bool has_e = true;
    if (xe < 0) {
      xe = h0 - 1;
      has_e = G.per0 != 0;
    } else if (xe >= h0) {
      xe = 0;
      has_e = G.per0 != 0;
    }
    const T e0 = has_e ? w[ob + xe] : T(0), e1 = has_e ? w[n + ob + xe] : T(0);
    const long long f0 = (long long)row * (G.n0 + 1) + 2 * hh + par;  // low face of cell 0
#pragma unroll
    for (int v = 0; v < V; v++) {
      const long long f = f0 + 2 * v;
      // low neighbour: hh + v - 1 + par (register selects: v is a constant
      // of the unrolled loop, only par is not)
      const int vl = v > 0 ? v - 1 : 0, vh = v < V - 1 ? v + 1 : V - 1;
      const bool lo_e = par == 0 && v == 0;
      if (!lo_e || has_e) {
        const T a0 = lo_e ? e0 : (par ? wv0[v] : wv0[vl]);
        const T a1 = lo_e ? e1 : (par ? wv1[v] : wv1[vl]);
        s0[v] = fmaT(P.b[0][f], a0, s0[v]);
        s1[v] = fmaT(P.b[0][nf0 + f], a1, s1[v]);
      }
      // high neighbour: hh + v + par
      const bool hi_e = par == 1 && v == V - 1;
      if (!hi_e || has_e) {
        const T a0 = hi_e ? e0 : (par ? wv0[vh] : wv0[v]);
        const T a1 = hi_e ? e1 : (par ? wv1[vh] : wv1[v]);
        s0[v] = fmaT(P.b[0][f + 1], a0, s0[v]);
        s1[v] = fmaT(P.b[0][nf0 + f + 1], a1, s1[v]);
      }
    }
  }
  // y and z: the same positions hh .. hh + V - 1 in the neighbouring rows
#pragma unroll
  for (int d = 1; d < DIM; d++) {
    const int m = d == 1 ? G.n1 : G.n2, c = d == 1 ? j : k;
    const bool per = d == 1 ? G.per1 != 0 : G.per2 != 0;
    const long long nf = d == 1 ? nf1 : nf2;
    const long long step = d == 1 ? G.n0 : pl;  // face stride of the direction
    // low face of cell v: natural face index of (i_v, j, k) in direction d
    const long long fb = d == 1 ? ((long long)k * (G.n1 + 1) + j) * G.n0 + 2 * hh + par
                                : (long long)row * G.n0 + 2 * hh + par;
#pragma unroll
    for (int side = 0; side < 2; side++) {
      int cn = c + (side ? 1 : -1);
      if (cn < 0 || cn >= m) {
        if (!per || m == 1) continue;
        cn = cn < 0 ? m - 1 : 0;
      }
      const unsigned nrow = d == 1 ? (unsigned)k * G.n1 + cn : (unsigned)cn * G.n1 + j;
      T nb0[V], nb1[V];
      ldv(w + obase + (long long)nrow * h0 + hh, nb0);
      ldv(w + n + obase + (long long)nrow * h0 + hh, nb1);
#pragma unroll
      for (int v = 0; v < V; v++) {
        const long long f = fb + 2 * v + (side ? step : 0);
        s0[v] = fmaT(P.b[d][f], nb0[v], s0[v]);
        s1[v] = fmaT(P.b[d][nf + f], nb1[v], s1[v]);
      }
    }
  }
}

template <class T, int DIM>
__global__ void __launch_bounds__(kBlock) lean_gsrb_vec_kernel(LinLeanT<T> P, int pass) {
  constexpr int V = Vec16<T>::V;
  const Geom &G = P.G;
  const long long n = G.ncell, half = n >> 1;
  const int h0 = G.n0 >> 1;
  const long long base = pass * half;  // own half
  const long long ngroups = half / V;
  for (long long t = gtid(); t < ngroups; t += gstride()) {
    const long long u = t * V;
    const unsigned row = (unsigned)u / (unsigned)h0;
    const int hh = (int)((unsigned)u - row * (unsigned)h0);
    const int k = (int)(row / (unsigned)G.n1), j = (int)(row - (unsigned)k * G.n1);
    const long long q = base + u;
    T s0[V], s1[V];
    lean_vsum<T, DIM>(P, pass, row, hh, j, k, s0, s1);
    T g0[V], g1[V], K0[V], K1[V], K2[V], K3[V], J0[V], J1[V], J2[V], J3[V];
    ldv(P.g + q, g0);
    ldv(P.g + n + q, g1);
    ldv(P.K + q, K0);
    ldv(P.K + n + q, K1);
    ldv(P.K + 2 * n + q, K2);
    ldv(P.K + 3 * n + q, K3);
    ldv(P.J + q, J0);
    ldv(P.J + n + q, J1);
    ldv(P.J + 2 * n + q, J2);
    ldv(P.J + 3 * n + q, J3);
    T x0[V], x1[V], w0[V], w1[V];
#pragma unroll
    for (int v = 0; v < V; v++) {
      const T r0 = fmaT(P.bdx, s0[v], g0[v]), r1 = fmaT(P.bdx, s1[v], g1[v]);
      x0[v] = fmaT(K0[v], r0, K2[v] * r1);
      x1[v] = fmaT(K1[v], r0, K3[v] * r1);
      w0[v] = fmaT(J0[v], x0[v], J1[v] * x1[v]);
      w1[v] = fmaT(J2[v], x0[v], J3[v] * x1[v]);
    }
    stv(P.x + q, x0);
    stv(P.x + n + q, x1);
    stv(P.w + q, w0);
    stv(P.w + n + q, w1);
  }
}

// g - A x at the cell of index q (both components)
template <class T, int DIM, class IDX>
__device__ __forceinline__ void lean_res(const LinLeanT<T> &P, int i, int j, int k, long long q,
                                         T r[2]) {
  const long long n = P.G.ncell;
  T s[2];
  lean_nbsum<T, DIM, IDX>(P, i, j, k, s);
  const T x0 = P.x[q], x1 = P.x[n + q];
  const T ax0 = fmaT(P.D[q], x0, P.D[n + q] * x1);
  const T ax1 = fmaT(P.D[2 * n + q], x0, P.D[3 * n + q] * x1);
  r[0] = fmaT(P.bdx, s[0], P.g[q]) - ax0;
  r[1] = fmaT(P.bdx, s[1], P.g[n + q]) - ax1;
}

// norm accumulation of one value (max keeps NaN, as norm_accum)
template <class T, int NORM>
__device__ __forceinline__ T lean_accum(T acc, T v) {
  if (NORM == MLGPU_NORM_MAX) {
    const T a = fabs(v);
    return (a > acc || a != a) ? a : acc;
  }
  if (NORM == MLGPU_NORM_L1) return acc + fabs(v);
  return fmaT(v, v, acc);
}

// fused norm of g - A x over both components (partials per block).  Each
// thread accumulates its few cells in T (for FP32: the values are FP32, a
// max is exact, a sum of a few dozen squares loses nothing that matters for
// the linear stopping test, and on GB300 an FP64 operation per cell would
// cost more than the cell's memory traffic); the block combines in FP64.
// IDX: split, or natural on a one-level hierarchy (whose only level is the
// bottom's).  RED (split only): the red half alone -- after a black half
// sweep the black cells' residual is zero up to rounding (each black x solves
// its own equations against the current red w), so the norm of a V-cycle that
// ends in post-smoothing is the red cells' norm.
template <class T, int DIM, int NORM, class IDX, bool RED>
__global__ void __launch_bounds__(kBlock) lean_residual_kernel(LinLeanT<T> P, double *part) {
  const Geom &G = P.G;
  const long long n = G.ncell, m = RED ? (n >> 1) : n;
  T acc = T(0);
  for (long long q = gtid(); q < m; q += gstride()) {
    int i, j, k;
    IDX::ijk(G, q, i, j, k);
    T r[2];
    lean_res<T, DIM, IDX>(P, i, j, k, q, r);
    acc = lean_accum<T, NORM>(acc, r[0]);
    acc = lean_accum<T, NORM>(acc, r[1]);
  }
  const double v = block_reduce<NORM>((double)acc);
  if (threadIdx.x == 0) part[blockIdx.x] = v;
}

// coarse g = 2^D average of the fine residual; the coarse x and w start at 0
// (coarse arrays split, or natural on the bottom level).  RED: after
// pre-smoothing that ends in a black half sweep the black children's
// residual is zero up to rounding and only the red children are summed.
template <class T, int DIM, class CIDX, bool RED>
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
          if (RED && ((ii + jj + kk) & 1)) continue;  // the child's colour
          const int i = 2 * I + ii, j = 2 * J + jj, k = DIM == 3 ? 2 * K + kk : 0;
          T r[2];
          lean_res<T, DIM, SplitIdx>(P, i, j, k, cs_index(P.G, i, j, k), r);
          a0 += r[0];
          a1 += r[1];
        }
    const long long oq = CIDX()(C, I, J, K);
    gc[oq] = a0 * wgt;
    gc[nc + oq] = a1 * wgt;
    xc[oq] = T(0);
    xc[nc + oq] = T(0);
    wc[oq] = T(0);
    wc[nc + oq] = T(0);
  }
}

// g - A x of the V cells at q .. q + V - 1 of a split level whose neighbour
// sums are s (lean_res's expression per cell)
template <class T>
__device__ __forceinline__ void lean_vres(const LinLeanT<T> &P, long long q, const T *s0,
                                          const T *s1, T *r0, T *r1) {
  constexpr int V = Vec16<T>::V;
  const long long n = P.G.ncell;
  T g0[V], g1[V], D0[V], D1[V], D2[V], D3[V], x0[V], x1[V];
  ldv(P.g + q, g0);
  ldv(P.g + n + q, g1);
  ldv(P.D + q, D0);
  ldv(P.D + n + q, D1);
  ldv(P.D + 2 * n + q, D2);
  ldv(P.D + 3 * n + q, D3);
  ldv(P.x + q, x0);
  ldv(P.x + n + q, x1);
#pragma unroll
  for (int v = 0; v < V; v++) {
    const T ax0 = fmaT(D0[v], x0[v], D1[v] * x1[v]);
    const T ax1 = fmaT(D2[v], x0[v], D3[v] * x1[v]);
    r0[v] = fmaT(P.bdx, s0[v], g0[v]) - ax0;
    r1[v] = fmaT(P.bdx, s1[v], g1[v]) - ax1;
  }
}

// lean_residual_kernel (split, RED) with V red cells of a row per thread
// (vector loads; the per-cell values bit for bit, the norm's partial sums in
// another order)
template <class T, int DIM, int NORM>
__global__ void __launch_bounds__(kBlock) lean_residual_vec_kernel(LinLeanT<T> P, double *part) {
  constexpr int V = Vec16<T>::V;
  const Geom &G = P.G;
  const int h0 = G.n0 >> 1;
  const long long ngroups = (G.ncell >> 1) / V;
  T acc = T(0);
  for (long long t = gtid(); t < ngroups; t += gstride()) {
    const long long u = t * V;
    const unsigned row = (unsigned)u / (unsigned)h0;
    const int hh = (int)((unsigned)u - row * (unsigned)h0);
    const int k = (int)(row / (unsigned)G.n1), j = (int)(row - (unsigned)k * G.n1);
    T s0[V], s1[V], r0[V], r1[V];
    lean_vsum<T, DIM>(P, 0, row, hh, j, k, s0, s1);
    lean_vres<T>(P, u, s0, s1, r0, r1);
#pragma unroll
    for (int v = 0; v < V; v++) {
      acc = lean_accum<T, NORM>(acc, r0[v]);
      acc = lean_accum<T, NORM>(acc, r1[v]);
    }
  }
  const double v = block_reduce<NORM>((double)acc);
  if (threadIdx.x == 0) part[blockIdx.x] = v;
}

// lean_restrict_kernel (RED) with V coarse cells of a coarse row per thread:
// the red children of coarse cells I0 .. I0 + V - 1 in fine row (2J + jj,
// 2K + kk) are that row's red cells I0 .. I0 + V - 1 (split positions), so each
// child class is one vector group; the children summed in the scalar
// kernel's order (the same bits)
template <class T, int DIM, class CIDX>
__global__ void __launch_bounds__(kBlock) lean_restrict_vec_kernel(LinLeanT<T> P, Geom C, T *gc,
                                                                   T *xc, T *wc) {
  constexpr int V = Vec16<T>::V;
  const Geom &G = P.G;
  const long long nc = C.ncell, ngroups = nc / V;
  const int h0 = G.n0 >> 1;
  const T wgt = DIM == 3 ? T(0.125) : T(0.25);
  const CIDX at;
  for (long long t = gtid(); t < ngroups; t += gstride()) {
    const long long U = t * V;
    const unsigned crow = (unsigned)U / (unsigned)C.n0;
    const int I0 = (int)((unsigned)U - crow * (unsigned)C.n0);
    const int K = (int)(crow / (unsigned)C.n1), J = (int)(crow - (unsigned)K * C.n1);
    T a0[V], a1[V];
#pragma unroll
    for (int v = 0; v < V; v++) a0[v] = a1[v] = T(0);
#pragma unroll
    for (int kk = 0; kk < (DIM == 3 ? 2 : 1); kk++)
#pragma unroll
      for (int jj = 0; jj < 2; jj++)
#pragma unroll
        for (int ii = 0; ii < 2; ii++) {
          if ((ii + jj + kk) & 1) continue;  // black child
          const int j = 2 * J + jj, k = DIM == 3 ? 2 * K + kk : 0;
          const unsigned row = (unsigned)k * G.n1 + j;
          T s0[V], s1[V], r0[V], r1[V];
          lean_vsum<T, DIM>(P, 0, row, I0, j, k, s0, s1);
          lean_vres<T>(P, (long long)row * h0 + I0, s0, s1, r0, r1);
#pragma unroll
          for (int v = 0; v < V; v++) {
            a0[v] += r0[v];
            a1[v] += r1[v];
          }
        }
#pragma unroll
    for (int v = 0; v < V; v++) {
      const long long oq = at(C, I0 + v, J, K);
      gc[oq] = a0[v] * wgt;
      gc[nc + oq] = a1[v] * wgt;
      xc[oq] = T(0);
      xc[nc + oq] = T(0);
      wc[oq] = T(0);
      wc[nc + oq] = T(0);
    }
  }
}

// x += prolongation of the coarse correction (coarse split, or natural on the
// bottom level); w = J x.  BLACK: the black half alone -- when post-smoothing
// follows, its red half sweep overwrites the red x and w without reading
// them (x_red = K^T (g + bdx sum b w_black)), so the result is the same bits.
template <class T, int DIM, int KIND, class CIDX, bool BLACK>
__global__ void __launch_bounds__(kBlock) lean_prolong_kernel(LinLeanT<T> P, Geom C,
                                                              const T *__restrict__ xc) {
  const Geom &G = P.G;
  const long long n = G.ncell, q0 = BLACK ? (n >> 1) : 0;
  for (long long q = q0 + gtid(); q < n; q += gstride()) {
    int i, j, k;
    cs_cell(G, q, i, j, k);
    const T x0 = prolong_add<T, DIM, KIND, CIDX>(C, P.ybc, 0, i, j, k, P.x[q], xc, nullptr);
    const T x1 = prolong_add<T, DIM, KIND, CIDX>(C, P.ybc, 1, i, j, k, P.x[n + q], xc, nullptr);
    P.x[q] = x0;
    P.x[n + q] = x1;
    P.w[q] = fmaT(P.J[q], x0, P.J[n + q] * x1);
    P.w[n + q] = fmaT(P.J[2 * n + q], x0, P.J[3 * n + q] * x1);
  }
}

// P_c of cell (i, j, k): the sum of its face coefficients by face kind
// (interior or periodic: b; derived-rule wall: 2b Dirichlet, 0 Neumann;
// (H, C)-condition wall: b), adj_cell's WANT_M face sum; it reads no state,
// so it is formed once per solver (lean_psum_kernel)
template <class T, int DIM>
__device__ __forceinline__ void lean_face_sums(const AdjArgs<T> &A, int i, int j, int k,
                                               T P[2]) {
  const Geom &G = A.G;
  const int idx[3] = {i, j, k};
#pragma unroll
  for (int c = 0; c < 2; c++) {
    T p = T(0);
#pragma unroll
    for (int d = 0; d < DIM; d++) {
      const int m = G.n(d);
      const long long nf = G.nface(d);
#pragma unroll
      for (int side = 1; side >= 0; side--) {
        int fi[3] = {idx[0], idx[1], idx[2]};
        if (side) fi[d] += 1;
        const T bf = A.b[d][c * nf + G.face(d, fi[0], fi[1], fi[2])];
        const int nb = idx[d] + (side ? 1 : -1);
        T dp;
        if (nb >= 0 && nb < m)
          dp = bf;
        else if (G.per(d))
          dp = m == 1 ? T(0) : bf;
        else if (A.apply_dbc)
          dp = dbc_wall_diag<T>(A.dbc, d, side, c, bf);
        else
          dp = bf;
        p = p + dp;
      }
    }
    P[c] = p;
  }
}

template <class T, int DIM>
__global__ void __launch_bounds__(kBlock) lean_psum_kernel(AdjArgs<T> A, T *__restrict__ Pout) {
  const Geom &G = A.G;
  const long long n = G.ncell;
  for (long long q = gtid(); q < n; q += gstride()) {
    int i, j, k;
    cell_ijk(G, q, i, j, k);
    T P[2];
    lean_face_sums<T, DIM>(A, i, j, k, P);
    Pout[q] = P[0];
    Pout[n + q] = P[1];
  }
}

// 2x2 diagonal block M of A^T at cell (i, j, k) (row-major, M[2c + c'] =
// d(A^T y)_c / d y_c'; A's own block is M^T), given the cell's closure
// Jacobian Jc (row-major {dT/dH, dT/dC, dC_l/dH, dC_l/dC}) and face sums P:
// adj_cell's WANT_M terms alone, which read no neighbour --
//   M(c, c') = delta alpha a_c + beta dxinv (J(c', c) P_c' - X(c, c')),
// X the (H, C)-condition walls' ghost-Jacobian terms (wall cells only).
// X of a cell on an (H, C)-condition wall (out of line: the ghost closure
// Jacobian is FP64 and long, and only wall cells take it)
template <class T, int DIM>
__device__ __noinline__ void lean_wall_terms(const AdjArgs<T> &A, long long q, int i, int j,
                                             int k, T X[4]) {
  const Geom &G = A.G;
  const int idx[3] = {i, j, k};
#pragma unroll
  for (int d = 0; d < DIM; d++) {
    if (G.per(d)) continue;
    const int m = G.n(d);
    const long long nf = G.nface(d);
#pragma unroll
    for (int side = 0; side < 2; side++) {
      if (side ? idx[d] != m - 1 : idx[d] != 0) continue;
      int fi[3] = {idx[0], idx[1], idx[2]};
      if (side) fi[d] += 1;
      const long long f = G.face(d, fi[0], fi[1], fi[2]);
      const T b0 = A.b[d][f], b1 = A.b[d][nf + f];
      double Jg[4];
      adj_ghost_jac(A, q, d, side, Jg);
#pragma unroll
      for (int c = 0; c < 2; c++) {
        const T sc = A.phi_bc.type[d][side][c] == MLGPU_BC_DIRICHLET ? T(-1) : T(1);
        X[2 * c + 0] = X[2 * c + 0] + sc * ((T)Jg[c] * b0);
        X[2 * c + 1] = X[2 * c + 1] + sc * ((T)Jg[2 + c] * b1);
      }
    }
  }
}

template <class T, int DIM>
__device__ __forceinline__ void lean_diag_block(const AdjArgs<T> &A, long long q, int i, int j,
                                                int k, const T Jc[4], const T P[2], T M[4]) {
  const Geom &G = A.G;
  T X[4] = {T(0), T(0), T(0), T(0)};
  const bool wall = (!G.per0 && (i == 0 || i == G.n0 - 1)) ||
                    (!G.per1 && (j == 0 || j == G.n1 - 1)) ||
                    (DIM == 3 && !G.per2 && (k == 0 || k == G.n2 - 1));
  if (!A.apply_dbc && wall) lean_wall_terms<T, DIM>(A, q, i, j, k, X);
  const long long n = G.ncell;
#pragma unroll
  for (int c = 0; c < 2; c++) {
    const T av = A.a ? A.a[q + c * n] : T(1);
#pragma unroll
    for (int cp = 0; cp < 2; cp++) {
      T v = A.beta * A.dxinv * (Jc[2 * cp + c] * P[cp] - X[2 * c + cp]);
      if (cp == c) v = A.alpha * av + v;
      M[2 * c + cp] = v;
    }
  }
}

// Per Newton state, on a smoothed level: the closure Jacobian J (FP32 in t_cl's
// regime for T = float, the lean FP64 Jacobian t_cl_jac_lean for double), A's
// diagonal block D = M^T and K = (D^T)^-1 = M^-1 of every cell (one
// reciprocal of det M: correctly rounded in FP32, refined in FP64), written
// straight to the split layout (the generic route -- adj_jac, adj_minv through
// the full adjoint cell operator, three permutations -- moves four times the
// bytes)
template <class T, int DIM>
__global__ void __launch_bounds__(kBlock) lean_state_kernel(AdjArgs<T> A, ClosureF32 f,
                                                            ClosureLean L,
                                                            const double *__restrict__ u,
                                                            const T *__restrict__ Psum,
                                                            T *__restrict__ Js,
                                                            T *__restrict__ Ks,
                                                            T *__restrict__ Ds) {
  const Geom &G = A.G;
  const long long n = G.ncell;
  // the next cell's state and face sums are loaded while this one is formed
  long long q = gtid();
  double hn = 0.0, cn = 0.0;
  T pn0 = T(0), pn1 = T(0);
  if (q < n) {
    hn = u[q];
    cn = u[q + n];
    pn0 = Psum[q];
    pn1 = Psum[n + q];
  }
  for (; q < n; q += gstride()) {
    const double h0 = hn, c0 = cn;
    const T P[2] = {pn0, pn1};
    const long long qn = q + gstride();
    if (qn < n) {
      hn = u[qn];
      cn = u[qn + n];
      pn0 = Psum[qn];
      pn1 = Psum[n + qn];
    }
    int i, j, k;
    cell_ijk(G, q, i, j, k);
    T Jc[4], M[4];
    if constexpr (sizeof(T) == 4)
      t_cl_jac32(h0, c0, A.cp, f, Jc);
    else
      t_cl_jac_lean(h0, c0, L, Jc);
    lean_diag_block<T, DIM>(A, q, i, j, k, Jc, P, M);
    const T det = M[0] * M[3] - M[1] * M[2];
    const long long o = cs_index(G, i, j, k);
#pragma unroll
    for (int m = 0; m < 4; m++) Js[o + m * n] = Jc[m];
    if constexpr (sizeof(T) == 4) {  // one correctly rounded reciprocal
      const float id = __frcp_rn(det);
      Ks[o] = M[3] * id;
      Ks[o + n] = -M[1] * id;
      Ks[o + 2 * n] = -M[2] * id;
      Ks[o + 3 * n] = M[0] * id;
    } else {
      const double id = lean_rcp(det);
      Ks[o] = M[3] * id;
      Ks[o + n] = -M[1] * id;
      Ks[o + 2 * n] = -M[2] * id;
      Ks[o + 3 * n] = M[0] * id;
    }
    Ds[o] = M[0];
    Ds[o + n] = M[2];
    Ds[o + 2 * n] = M[1];
    Ds[o + 3 * n] = M[3];
  }
}

// The linear prolongation onto the black half (BLACK of lean_prolong_kernel
// with KIND linear) by coarse tiles: a block stages the coarse values of its
// tile of kBlock coarse cells and their one-cell halo in shared memory -- each
// value as coarse_at forms it (periodic wrap; a wall clamps to the edge cell
// and negates it for a Dirichlet rule of that component, the product of +-1
// signs being exact) -- and each thread forms its coarse cell's black children
// (the fine cells of odd (ii + jj + kk)) from the tile with prolong_add's
// expression: the same bits as one thread per fine cell, with each coarse
// value loaded about 1.6 times per tile instead of 8 times per child.
template <int DIM>
struct ProlongTile {
  static constexpr int TX = 32, TY = DIM == 3 ? 4 : 8, TZ = DIM == 3 ? 2 : 1;
  static constexpr int HX = TX + 2, HY = TY + 2, HZ = DIM == 3 ? TZ + 2 : 1;
  static_assert(TX * TY * TZ == kBlock, "one thread per coarse cell of the tile");
};

template <class T, int DIM, class CIDX>
__global__ void __launch_bounds__(kBlock) lean_prolong_lin_black_kernel(LinLeanT<T> P, Geom C,
                                                                        const T *__restrict__ xc) {
  using PT = ProlongTile<DIM>;
  constexpr int TX = PT::TX, TY = PT::TY, TZ = PT::TZ, HX = PT::HX, HY = PT::HY, HZ = PT::HZ;
  constexpr int HN = HX * HY * HZ;
  __shared__ T tile[2 * HN];
  const Geom &G = P.G;
  const long long n = G.ncell;
  const T den = T(1) / (DIM == 3 ? T(64) : T(16));
  const T fx1 = T(3) * den, fx2 = T(9) * den, fx3 = T(27) * den, f0 = T(1) * den;
  const CIDX at;
  const int ntx = (C.n0 + TX - 1) / TX, nty = (C.n1 + TY - 1) / TY;
  const int ntz = DIM == 3 ? (C.n2 + TZ - 1) / TZ : 1;
  const long long ntiles = (long long)ntx * nty * ntz;
  const int lx = threadIdx.x % TX, ly = (threadIdx.x / TX) % TY, lz = threadIdx.x / (TX * TY);
  for (long long tb = blockIdx.x; tb < ntiles; tb += gridDim.x) {
    const int tx = (int)(tb % ntx), ty = (int)((tb / ntx) % nty), tz = (int)(tb / ((long long)ntx * nty));
    const int org[3] = {tx * TX - 1, ty * TY - 1, DIM == 3 ? tz * TZ - 1 : 0};
    __syncthreads();  // the previous tile's readers are done
    for (int e = threadIdx.x; e < 2 * HN; e += kBlock) {
      const int c = e / HN;
      int r = e - c * HN;
      const int z = r / (HX * HY);
      r -= z * (HX * HY);
      const int y = r / HX, xx = r - y * HX;
      int cc[3] = {org[0] + xx, org[1] + y, org[2] + z};
      unsigned fl = 0u;
#pragma unroll
      for (int d = 0; d < DIM; d++) {
        const int m = C.n(d);
        int v = cc[d];
        if (v < 0 || v >= m) {
          const int side = v < 0 ? 0 : 1;
          if (v == -1 || v == m) {  // the halo of an edge tile: coarse_at's rule
            if (C.per(d)) {
              v = v < 0 ? m - 1 : 0;
            } else {
              v = v < 0 ? 0 : m - 1;
              fl ^= P.ybc.type[d][side][c] == MLGPU_BC_DIRICHLET ? 1u : 0u;
            }
          } else {  // past a partial tile: read by no coarse cell of the box
            v = m - 1;
          }
        }
        cc[d] = v;
      }
      const T v = xc[(long long)c * C.ncell + at(C, cc[0], cc[1], cc[2])];
      tile[e] = fl ? -v : v;
    }
    __syncthreads();
    const int I = org[0] + 1 + lx, J = org[1] + 1 + ly, K = DIM == 3 ? org[2] + 1 + lz : 0;
    if (I >= C.n0 || J >= C.n1 || (DIM == 3 && K >= C.n2)) continue;
    auto cv = [&](int c, int ox, int oy, int oz) -> T {
      return tile[c * HN + ((DIM == 3 ? lz + 1 + oz : 0) * HY + ly + 1 + oy) * HX + lx + 1 + ox];
    };
#pragma unroll
    for (int kk = 0; kk < (DIM == 3 ? 2 : 1); kk++)
#pragma unroll
      for (int jj = 0; jj < 2; jj++)
#pragma unroll
        for (int ii = 0; ii < 2; ii++) {
          if (((ii + jj + kk) & 1) == 0) continue;  // red child: not prolonged
          const int i = 2 * I + ii, j = 2 * J + jj, k = DIM == 3 ? 2 * K + kk : 0;
          const long long qf = cs_index(G, i, j, k);
          const int o1 = 2 * ii - 1, o2 = 2 * jj - 1, o3 = DIM == 3 ? 2 * kk - 1 : 0;
          T xv[2];
#pragma unroll
          for (int c = 0; c < 2; c++) {
            T p = P.x[c * n + qf];
            if (DIM == 2) {
              p = p + fx2 * cv(c, 0, 0, 0) + f0 * cv(c, o1, o2, 0);
              p = p + fx1 * (cv(c, o1, 0, 0) + cv(c, 0, o2, 0));
            } else {
              p = p + fx3 * cv(c, 0, 0, 0) + f0 * cv(c, o1, o2, o3);
              p = p + fx2 * (cv(c, o1, 0, 0) + cv(c, 0, o2, 0) + cv(c, 0, 0, o3));
              p = p + fx1 * (cv(c, o1, o2, 0) + cv(c, 0, o2, o3) + cv(c, o1, 0, o3));
            }
            xv[c] = p;
          }
          P.x[qf] = xv[0];
          P.x[n + qf] = xv[1];
          P.w[qf] = fmaT(P.J[qf], xv[0], P.J[n + qf] * xv[1]);
          P.w[n + qf] = fmaT(P.J[2 * n + qf], xv[0], P.J[3 * n + qf] * xv[1]);
        }
  }
}

// dst (T, layout IDX) = src (natural) for `ncomp` components of n cells each
template <class T, class S, class IDX>
__global__ void __launch_bounds__(kBlock) lean_pack_kernel(Geom G, int ncomp,
                                                           const S *__restrict__ src,
                                                           T *__restrict__ dst) {
  const long long n = G.ncell;
  const IDX at;
  for (long long q = gtid(); q < n; q += gstride()) {
    int i, j, k;
    cell_ijk(G, q, i, j, k);
    const long long o = at(G, i, j, k);
    for (int c = 0; c < ncomp; c++) {
      if constexpr (sizeof(T) == 4 && sizeof(S) == 8)
        dst[c * n + o] = f32_round(src[c * n + q]);  // integer pipe
      else
        dst[c * n + o] = (T)src[c * n + q];
    }
  }
}

// Newton update u = u_old + scale e, e the correction in layout IDX (both
// components).  CLIP: a cell whose H would leave its closure regime (solid /
// eutectic / mush / liquid, bounded by H_s, H_e, H_l at the new C) stops at
// the first regime boundary it crosses plus `frac` of its overshoot, so its
// next linearisation is the new regime's.
template <class T, class IDX, bool CLIP>
__global__ void __launch_bounds__(kBlock) lean_step_kernel(Geom G, StepClip K,
                                                           double *__restrict__ u,
                                                           const double *__restrict__ u_old,
                                                           double scale,
                                                           const T *__restrict__ e) {
  const long long n = G.ncell;
  const IDX at;
  // the next cell's old state and correction are loaded while this one is
  // updated
  auto load = [&](long long q, double &h, double &c, T &eh, T &ec) {
    int i, j, k;
    cell_ijk(G, q, i, j, k);
    const long long o = at(G, i, j, k);
    h = u_old[q];
    c = u_old[n + q];
    eh = e[o];
    ec = e[n + o];
  };
  long long q = gtid();
  double hn = 0.0, cn = 0.0;
  T ehn = T(0), ecn = T(0);
  if (q < n) load(q, hn, cn, ehn, ecn);
  for (; q < n; q += gstride()) {
    const double h0 = hn, c0 = cn;
    const T eh = ehn, ec = ecn;
    if (q + gstride() < n) load(q + gstride(), hn, cn, ehn, ecn);
    double h1, c1;
    if constexpr (sizeof(T) == 4) {
      h1 = h0 + scale * f64_exact(eh);
      c1 = c0 + scale * f64_exact(ec);
    } else {
      h1 = h0 + scale * (double)eh;
      c1 = c0 + scale * (double)ec;
    }
    if (CLIP) {
      // FP32 regime test (truncated conversions: the near-bound band is 1e-4)
      float b0[3], b1[3];
      const float h0f = f32_trunc(h0), h1f = f32_trunc(h1);
      const int f0 = K.regime32(h0f, f32_trunc(c0), b0);
      const int f1 = K.regime32(h1f, f32_trunc(c1), b1);
      if (f0 != f1 || StepClip::near(h0f, b0) || StepClip::near(h1f, b1))
        h1 = step_clip_near(h0, c0, h1, c1, K);
    }
    u[q] = h1;
    u[n + q] = c1;
  }
}
#endif  // MLGPU_ADJ_F32_UNIT

}  // namespace mlgpu
