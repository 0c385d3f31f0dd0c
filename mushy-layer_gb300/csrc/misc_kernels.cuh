// misc_kernels.cuh -- multigrid transfers, coefficient coarsening, the full
// closure, MAC divergence/gradient correction and elementwise helpers.
#pragma once
#include "common.cuh"
#include "reduce.cuh"

namespace mlgpu {

// ---------------------------------------------------------------- restrict
// phi_c = avg_{2^D} phi_f, accumulated as in RESTRICT (F.ChF:555-585).
template <class T, int DIM>
__global__ void __launch_bounds__(kBlock) restrict_avg_kernel(Geom F, Geom C, int ncomp,
                                                              const T *__restrict__ fine,
                                                              T *__restrict__ coarse) {
  // acc + f / 2^D as one FMA with 1 / 2^D: the scaling by a power of two is
  // exact (for results above the subnormal range), so the sum is the same
  // bits with half the FP64 pipe operations
  const T inv = DIM == 3 ? T(0.125) : T(0.25);
  constexpr int NCH = DIM == 3 ? 8 : 4;
  long long total = C.ncell * ncomp;
  // the children of the next coarse cell are loaded while this one is summed
  auto load = [&](long long t, T v[NCH]) {
    const int c = (int)(t / C.ncell);
    const long long Q = t % C.ncell;
    int I, J, K;
    cell_ijk(C, Q, I, J, K);
#pragma unroll
    for (int kk = 0; kk < (DIM == 3 ? 2 : 1); kk++)
#pragma unroll
      for (int jj = 0; jj < 2; jj++)
#pragma unroll
        for (int ii = 0; ii < 2; ii++) {
          const int k = DIM == 3 ? 2 * K + kk : 0;
          v[(kk * 2 + jj) * 2 + ii] = fine[c * F.ncell + F.cell(2 * I + ii, 2 * J + jj, k)];
        }
  };
  long long t = gtid();
  T nxt[NCH];
  if (t < total) load(t, nxt);
  for (; t < total; t += gstride()) {
    T cur[NCH];
#pragma unroll
    for (int m = 0; m < NCH; m++) cur[m] = nxt[m];
    if (t + gstride() < total) load(t + gstride(), nxt);
    T acc = T(0);
#pragma unroll
    for (int m = 0; m < NCH; m++) {  // Fortran loop order: k, j outer, i fastest
      if constexpr (sizeof(T) == 4)
        acc = fmaf(cur[m], inv, acc);
      else
        acc = fma(cur[m], inv, acc);
    }
    coarse[t] = acc;
  }
}

// ---------------------------------------------------------------- prolong
// Coarse value with the homogeneous ghost rule applied per direction:
// periodic wrap, else clamp to the boundary cell and negate for Dirichlet.
template <class T, class IDX = NaturalIdx>
__device__ __forceinline__ T coarse_at(const Geom &C, const BCD &bc, int comp,
                                       const T *__restrict__ a, const T *__restrict__ b,
                                       int I, int J, int K) {
  int idx[3] = {I, J, K};
  T sign = T(1);
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (d >= C.dim) break;
    int m = C.n(d);
    if (idx[d] < 0 || idx[d] >= m) {
      int side = idx[d] < 0 ? 0 : 1;
      if (C.per(d)) {
        idx[d] = idx[d] < 0 ? m - 1 : 0;
      } else {
        idx[d] = idx[d] < 0 ? 0 : m - 1;
        if (bc.type[d][side][comp] == MLGPU_BC_DIRICHLET) sign = -sign;
      }
    }
  }
  long long q = comp * C.ncell + IDX()(C, idx[0], idx[1], idx[2]);
  T v = b ? (a[q] - b[q]) : a[q];
  return sign * v;
}

// phi_f += P (a - b) (b may be null): KIND 0 piecewise constant (Chombo
// FORT_PROLONG), KIND 1 the linear stencil of PROLONG_JP
// (src/AMRProjectionOpF.ChF:15-78).  The FAS correction u_c - u_c,old is
// formed on the fly from its two operands.
// p + (P (a - b))(i, j, k) for component c: the prolongation increment of one
// fine cell, arithmetic identical to prolong_one below.
template <class T, int DIM, int KIND, class IDX = NaturalIdx>
__device__ __forceinline__ T prolong_add(const Geom &C, const BCD &bc, int c, int i, int j, int k,
                                         T p, const T *__restrict__ a, const T *__restrict__ b) {
  const T den = T(1) / (DIM == 3 ? T(64) : T(16));
  const T fx1 = T(3) * den, fx2 = T(9) * den, fx3 = T(27) * den, f0 = T(1) * den;
  int ic = i >> 1, jc = j >> 1, kc = DIM == 3 ? k >> 1 : 0;
  if (KIND == MLGPU_PROLONG_CONSTANT) return p + coarse_at<T, IDX>(C, bc, c, a, b, ic, jc, kc);
  int o1 = 2 * (i & 1) - 1, o2 = 2 * (j & 1) - 1, o3 = DIM == 3 ? 2 * (k & 1) - 1 : 0;
  if (DIM == 2) {
    p = p + fx2 * coarse_at<T, IDX>(C, bc, c, a, b, ic, jc, kc) +
        f0 * coarse_at<T, IDX>(C, bc, c, a, b, ic + o1, jc + o2, kc);
    p = p + fx1 * (coarse_at<T, IDX>(C, bc, c, a, b, ic + o1, jc, kc) +
                   coarse_at<T, IDX>(C, bc, c, a, b, ic, jc + o2, kc));
  } else {
    p = p + fx3 * coarse_at<T, IDX>(C, bc, c, a, b, ic, jc, kc) +
        f0 * coarse_at<T, IDX>(C, bc, c, a, b, ic + o1, jc + o2, kc + o3);
    p = p + fx2 * (coarse_at<T, IDX>(C, bc, c, a, b, ic + o1, jc, kc) +
                   coarse_at<T, IDX>(C, bc, c, a, b, ic, jc + o2, kc) +
                   coarse_at<T, IDX>(C, bc, c, a, b, ic, jc, kc + o3));
    p = p + fx1 * (coarse_at<T, IDX>(C, bc, c, a, b, ic + o1, jc + o2, kc) +
                   coarse_at<T, IDX>(C, bc, c, a, b, ic, jc + o2, kc + o3) +
                   coarse_at<T, IDX>(C, bc, c, a, b, ic + o1, jc, kc + o3));
  }
  return p;
}

// One fine value t (component-major index) of the prolongation.
template <class T, int DIM, int KIND>
__device__ __forceinline__ void prolong_one(const Geom &F, const Geom &C, const BCD &bc,
                                            long long t, T *__restrict__ fine,
                                            const T *__restrict__ a, const T *__restrict__ b) {
  unsigned nc = (unsigned)F.ncell;
  int c = (int)((unsigned)t / nc);
  long long q = (unsigned)t - (unsigned)c * nc;
  int i, j, k;
  cell_ijk(F, q, i, j, k);
  fine[t] = prolong_add<T, DIM, KIND>(C, bc, c, i, j, k, fine[t], a, b);
}

template <class T, int DIM, int KIND>
__global__ void __launch_bounds__(kBlock) prolong_kernel(Geom F, Geom C, BCD bc, int ncomp,
                                                         T *__restrict__ fine,
                                                         const T *__restrict__ a,
                                                         const T *__restrict__ b) {
  long long total = F.ncell * ncomp;
  for (long long t = gtid(); t < total; t += gstride())
    prolong_one<T, DIM, KIND>(F, C, bc, t, fine, a, b);
}

// ------------------------------------------------------- face coarsening
// CoarseAverageFace (arithmetic): mean of the 2^(D-1) covered fine faces.
template <class T, int DIM>
__global__ void __launch_bounds__(kBlock) coarsen_faces_kernel(Geom F, Geom C, int ncomp, int d,
                                                               const T *__restrict__ ff,
                                                               T *__restrict__ cf) {
  long long nfc = C.nface(d), nff = F.nface(d);
  long long total = nfc * ncomp;
  const T refScale = DIM == 3 ? T(0.25) : T(0.5);
  int m0 = C.n0 + (d == 0), m1 = C.n1 + (d == 1);
  for (long long t = gtid(); t < total; t += gstride()) {
    int c = (int)(t / nfc);
    long long r = t % nfc;
    int I = (int)(r % m0);
    long long rr = r / m0;
    int J = (int)(rr % m1);
    int K = (int)(rr / m1);
    int rk = (DIM == 3 && d != 2) ? 2 : 1, rj = d != 1 ? 2 : 1, ri = d != 0 ? 2 : 1;
    T sum = T(0);
    for (int kk = 0; kk < rk; kk++)
      for (int jj = 0; jj < rj; jj++)
        for (int ii = 0; ii < ri; ii++) {
          int fi = 2 * I + ii, fj = 2 * J + jj, fk = DIM == 3 ? 2 * K + kk : 0;
          sum = sum + ff[c * nff + F.face(d, fi, fj, fk)];
        }
    cf[t] = sum * refScale;
  }
}

#ifdef MLGPU_FP64_UNIT  // FP64-only kernels: compiled in launch_f64.cu alone
// ------------------------------------------------------------ full closure
// updateEnthalpyVariables (src/phaseDiagram.cpp:92-177) for one cell:
// CALCULATEPOROSITY/CL/CS/T with the bounding energies.
__global__ void __launch_bounds__(kBlock) closure_full_kernel(long long n, ClosureParams p,
                                                              const double *__restrict__ HC,
                                                              double *T, double *por, double *Cl,
                                                              double *Cs, double *Hs,
                                                              double *He, double *Hl) {
  for (long long q = gtid(); q < n; q += gstride()) {
    double H = HC[q], C = HC[q + n];
    double hs, he, hl;
    bounding_energy(C, p, hs, he, hl);
    double t, po, cl, cs;
    if (H <= hs) {
      po = 0;
      cl = p.Te;
      cs = C;
      t = H / p.cp;
    } else if (H > hs && H <= he) {
      po = (H - p.te * p.cp) / (p.St + p.te * (1 - p.cp));
      cl = p.Te;
      double pm = porosity_mush(C, H, p);  // CALCULATECS uses the mush root here
      cs = C / (1 - pm);
      t = p.te;
    } else if (H > he && H < hl) {
      double pm = porosity_mush(C, H, p);
      po = pm;
      cl = (C + p.CR * (1 - pm)) / (pm + p.k * (1 - pm));
      cs = (C * p.k - p.CR * pm) / (pm + p.k * (1 - pm));
      t = -(C + p.CR * (1 - pm)) / (pm + p.k * (1 - pm));
    } else if (H >= hl) {
      po = 1;
      cl = C;
      cs = 0;
      t = H - p.St;
    } else {
      po = H; cl = H; cs = H; t = H;
    }
    if (T) T[q] = t;
    if (por) por[q] = po;
    if (Cl) Cl[q] = cl;
    if (Cs) Cs[q] = cs;
    if (Hs) Hs[q] = hs;
    if (He) He[q] = he;
    if (Hl) Hl[q] = hl;
  }
}

__global__ void __launch_bounds__(kBlock) closure_tcl_kernel(long long n, ClosureParams p,
                                                             const double *__restrict__ HC,
                                                             double *__restrict__ TCl) {
  for (long long q = gtid(); q < n; q += gstride()) t_cl(HC[q], HC[q + n], p, TCl[q], TCl[q + n]);
}

// the lean Newton paths' closure (t_cl_lean)
__global__ void __launch_bounds__(kBlock) closure_tcl_lean_kernel(long long n, ClosureLean p,
                                                                  const double *__restrict__ HC,
                                                                  double *__restrict__ TCl) {
  for (long long q = gtid(); q < n; q += gstride())
    t_cl_lean(HC[q], HC[q + n], p, TCl[q], TCl[q + n]);
}

// ---------------------------------------------------- face geometric mean
// CELLTOEDGEGEOMETRIC: sqrt(|c_lo c_hi|); non-periodic boundary faces see a
// zero-gradient ghost (face = |c|).
__global__ void __launch_bounds__(kBlock) face_geomean_kernel(Geom G, int d,
                                                              const double *__restrict__ cell,
                                                              double *__restrict__ face) {
  long long nf = G.nface(d);
  int m0 = G.n0 + (d == 0), m1 = G.n1 + (d == 1);
  for (long long t = gtid(); t < nf; t += gstride()) {
    int i = (int)(t % m0);
    long long r = t / m0;
    int j = (int)(r % m1);
    int k = (int)(r / m1);
    int hi[3] = {i, j, k}, lo[3] = {i, j, k};
    lo[d] -= 1;
    int m = G.n(d);
    if (hi[d] >= m) hi[d] = G.per(d) ? 0 : m - 1;
    if (lo[d] < 0) lo[d] = G.per(d) ? m - 1 : 0;
    double a = cell[G.cell(lo[0], lo[1], lo[2])], b = cell[G.cell(hi[0], hi[1], hi[2])];
    face[t] = sqrt(fabs(a * b));
  }
}

// ----------------------------------------------------- MAC div / correct
__global__ void __launch_bounds__(kBlock) mac_div_kernel(Geom G, const double *__restrict__ u0,
                                                         const double *__restrict__ u1,
                                                         const double *__restrict__ u2,
                                                         double *__restrict__ div) {
  double one_on_dx = 1.0 / G.dx;
  for (long long q = gtid(); q < G.ncell; q += gstride()) {
    int i, j, k;
    cell_ijk(G, q, i, j, k);
    double v = 0.0;
    v = v + one_on_dx * (u0[G.face(0, i + 1, j, k)] - u0[G.face(0, i, j, k)]);
    v = v + one_on_dx * (u1[G.face(1, i, j + 1, k)] - u1[G.face(1, i, j, k)]);
    if (G.dim == 3) v = v + one_on_dx * (u2[G.face(2, i, j, k + 1)] - u2[G.face(2, i, j, k)]);
    div[q] = v;
  }
}

__global__ void __launch_bounds__(kBlock) mac_correct_kernel(Geom G, BCD bc, int d,
                                                             const double *__restrict__ phi,
                                                             const double *__restrict__ scale,
                                                             double *__restrict__ u) {
  long long nf = G.nface(d);
  int m0 = G.n0 + (d == 0), m1 = G.n1 + (d == 1);
  int m = G.n(d);
  for (long long t = gtid(); t < nf; t += gstride()) {
    int i = (int)(t % m0);
    long long r = t / m0;
    int j = (int)(r % m1);
    int k = (int)(r / m1);
    int hi[3] = {i, j, k}, lo[3] = {i, j, k};
    lo[d] -= 1;
    double ph, pl;
    if (hi[d] < m && lo[d] >= 0) {
      ph = phi[G.cell(hi[0], hi[1], hi[2])];
      pl = phi[G.cell(lo[0], lo[1], lo[2])];
    } else if (G.per(d)) {
      if (hi[d] >= m) hi[d] = 0;
      if (lo[d] < 0) lo[d] = m - 1;
      ph = phi[G.cell(hi[0], hi[1], hi[2])];
      pl = phi[G.cell(lo[0], lo[1], lo[2])];
    } else if (lo[d] < 0) {
      ph = phi[G.cell(hi[0], hi[1], hi[2])];
      pl = ghost_value<double>(bc, d, 0, 0, ph, G.dx, false);
    } else {
      pl = phi[G.cell(lo[0], lo[1], lo[2])];
      ph = ghost_value<double>(bc, d, 1, 0, pl, G.dx, false);
    }
    double grad = (ph - pl) / G.dx;
    if (scale) grad = grad * scale[t];
    u[t] = u[t] - grad;
  }
}
// --------------------------------------------- MAC projection adjoint
// The projection u = u* - Pi G p, D Pi G p = D u* (mac_div_kernel,
// mac_correct_kernel, the projection operator) transposes to
//   q: D Pi G q = G^T (Pi ubar),  ustar_bar = ubar - D^T q,
//   pi_bar = -ustar_bar * (G p)   (G p the corrected gradient, all faces),
// with G^T and D^T the exact transposes of the face arrays as the forward
// kernels index them: on a periodic seam faces 0 and n both carry the
// gradient (p_0 - p_(n-1))/dx; at a wall the ghost rule's derivative
// (Dirichlet -1, Neumann +1) enters.

// r = G^T (scale * y) at every cell (scale == null: 1)
__global__ void __launch_bounds__(kBlock) mac_grad_t_kernel(Geom G, BCD bc,
                                                            const double *__restrict__ y0,
                                                            const double *__restrict__ y1,
                                                            const double *__restrict__ y2,
                                                            const double *__restrict__ s0,
                                                            const double *__restrict__ s1,
                                                            const double *__restrict__ s2,
                                                            double *__restrict__ r) {
  for (long long q = gtid(); q < G.ncell; q += gstride()) {
    int idx[3];
    cell_ijk(G, q, idx[0], idx[1], idx[2]);
    double v = 0.0;
    for (int d = 0; d < G.dim; d++) {
      const double *y = d == 0 ? y0 : (d == 1 ? y1 : y2);
      const double *sc = d == 0 ? s0 : (d == 1 ? s1 : s2);
      const int m = G.n(d), a = idx[d];
      int f[3] = {idx[0], idx[1], idx[2]};
      const long long flo = G.face(d, f[0], f[1], f[2]);
      f[d] += 1;
      const long long fhi = G.face(d, f[0], f[1], f[2]);
      const double ylo = sc ? y[flo] * sc[flo] : y[flo];
      const double yhi = sc ? y[fhi] * sc[fhi] : y[fhi];
      // d(grad at the low face)/d p_a, d(grad at the high face)/d p_a
      double clo = 1.0, chi = -1.0;
      if (!G.per(d)) {
        if (a == 0) clo = bc.type[d][0][0] == MLGPU_BC_DIRICHLET ? 2.0 : 0.0;
        if (a == m - 1) chi = bc.type[d][1][0] == MLGPU_BC_DIRICHLET ? -2.0 : 0.0;
      }
      double t = clo * ylo + chi * yhi;
      if (G.per(d)) {
        // the seam's other face: face n holds the gradient of cell 0 as its
        // high neighbour, face 0 that of cell n-1 as its low neighbour
        if (a == 0) {
          f[d] = m;
          const long long fs = G.face(d, f[0], f[1], f[2]);
          t = t + (sc ? y[fs] * sc[fs] : y[fs]);
        }
        if (a == m - 1) {
          f[d] = 0;
          const long long fs = G.face(d, f[0], f[1], f[2]);
          t = t - (sc ? y[fs] * sc[fs] : y[fs]);
        }
      }
      v = v + t / G.dx;
    }
    r[q] = v;
  }
}

// out = ubar - D^T q on every face of direction d
__global__ void __launch_bounds__(kBlock) mac_div_t_kernel(Geom G, int d,
                                                           const double *__restrict__ q,
                                                           const double *__restrict__ ubar,
                                                           double *__restrict__ out) {
  const double one_on_dx = 1.0 / G.dx;
  const long long nf = G.nface(d);
  const int m0 = G.n0 + (d == 0), m1 = G.n1 + (d == 1);
  const int m = G.n(d);
  for (long long t = gtid(); t < nf; t += gstride()) {
    int f[3];
    f[0] = (int)(t % m0);
    long long rr = t / m0;
    f[1] = (int)(rr % m1);
    f[2] = (int)(rr / m1);
    const int b = f[d];
    double dt = 0.0;
    if (b >= 1) {
      int c[3] = {f[0], f[1], f[2]};
      c[d] = b - 1;
      dt = dt + one_on_dx * q[G.cell(c[0], c[1], c[2])];
    }
    if (b <= m - 1) dt = dt - one_on_dx * q[G.cell(f[0], f[1], f[2])];
    out[t] = ubar[t] - dt;
  }
}

// pi_bar = -ustar_bar * (corrected gradient of p) on every face of direction d
__global__ void __launch_bounds__(kBlock) mac_pi_bar_kernel(Geom G, BCD bc, int d,
                                                            const double *__restrict__ phi,
                                                            const double *__restrict__ usb,
                                                            double *__restrict__ pib) {
  long long nf = G.nface(d);
  int m0 = G.n0 + (d == 0), m1 = G.n1 + (d == 1);
  int m = G.n(d);
  for (long long t = gtid(); t < nf; t += gstride()) {
    int i = (int)(t % m0);
    long long r = t / m0;
    int j = (int)(r % m1);
    int k = (int)(r / m1);
    int hi[3] = {i, j, k}, lo[3] = {i, j, k};
    lo[d] -= 1;
    double ph, pl;
    if (hi[d] < m && lo[d] >= 0) {
      ph = phi[G.cell(hi[0], hi[1], hi[2])];
      pl = phi[G.cell(lo[0], lo[1], lo[2])];
    } else if (G.per(d)) {
      if (hi[d] >= m) hi[d] = 0;
      if (lo[d] < 0) lo[d] = m - 1;
      ph = phi[G.cell(hi[0], hi[1], hi[2])];
      pl = phi[G.cell(lo[0], lo[1], lo[2])];
    } else if (lo[d] < 0) {
      ph = phi[G.cell(hi[0], hi[1], hi[2])];
      pl = ghost_value<double>(bc, d, 0, 0, ph, G.dx, false);
    } else {
      pl = phi[G.cell(lo[0], lo[1], lo[2])];
      ph = ghost_value<double>(bc, d, 1, 0, pl, G.dx, false);
    }
    const double grad = (ph - pl) / G.dx;
    pib[t] = -(usb[t] * grad);
  }
}

// Backward-Euler step adjoint: phi_old_bar = a mu (a == null: mu),
// src_bar = dt mu (either output may be null)
__global__ void __launch_bounds__(kBlock) be_adj_kernel(long long n, const double *__restrict__ mu,
                                                        const double *__restrict__ a, double dt,
                                                        double *__restrict__ old_bar,
                                                        double *__restrict__ src_bar) {
  for (long long q = gtid(); q < n; q += gstride()) {
    const double m = mu[q];
    if (old_bar) old_bar[q] = a ? a[q] * m : m;
    if (src_bar) src_bar[q] = dt * m;
  }
}

// Backward-Euler right-hand side (LevelBackwardEuler::updateSoln):
// rhs = phi_old * a + dt * src; a == null means a == 1, src == null no source.
__global__ void __launch_bounds__(kBlock) be_rhs_kernel(long long n, const double *__restrict__ phi_old,
                                                        const double *__restrict__ a,
                                                        const double *__restrict__ src, double dt,
                                                        double *__restrict__ rhs) {
  for (long long q = gtid(); q < n; q += gstride()) {
    double v = a ? phi_old[q] * a[q] : phi_old[q];
    if (src) v = v + dt * src[q];
    rhs[q] = v;
  }
}
// TGA right-hand side pieces: out = base + dt src (src may be null), and
// out = a x (a null: a == 1)
__global__ void __launch_bounds__(kBlock) add_dt_src_kernel(long long n, double *__restrict__ out,
                                                            const double *__restrict__ src,
                                                            double dt) {
  for (long long q = gtid(); q < n; q += gstride()) out[q] = out[q] + dt * src[q];
}
__global__ void __launch_bounds__(kBlock) scale_by_a_kernel(long long n,
                                                            const double *__restrict__ x,
                                                            const double *__restrict__ a,
                                                            double *__restrict__ out) {
  for (long long q = gtid(); q < n; q += gstride()) out[q] = a ? x[q] * a[q] : x[q];
}
#endif  // MLGPU_FP64_UNIT

// ------------------------------------------------------------ elementwise
template <class T>
__global__ void __launch_bounds__(kBlock) axpby_kernel(long long n, T a, const T *__restrict__ x,
                                                       T b, T *__restrict__ y) {
  for (long long q = gtid(); q < n; q += gstride()) y[q] = a * x[q] + b * y[q];
}

template <class D, class S>
__global__ void __launch_bounds__(kBlock) convert_kernel(long long n, D *__restrict__ dst,
                                                         const S *__restrict__ src) {
  for (long long q = gtid(); q < n; q += gstride()) dst[q] = (D)src[q];
}

template <class T, int NORM>
__global__ void __launch_bounds__(kBlock) norm_partial_kernel(long long n,
                                                              const T *__restrict__ x,
                                                              double *__restrict__ part) {
  double acc = 0.0;
  for (long long q = gtid(); q < n; q += gstride()) acc = norm_accum<NORM>(acc, (double)x[q]);
  double r = block_reduce<NORM>(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = r;
}

}  // namespace mlgpu
