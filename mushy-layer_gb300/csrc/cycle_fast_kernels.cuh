// cycle_fast_kernels.cuh -- lean FP32 coarse end of the mixed-precision
// V-cycle (2D): every level from a top of at most 1024 cells down to the
// bottom inside one CTA (one thread per quad of the top level); levels of at
// most 32 quads and a bottom of at most 32 cells run on warp 0 alone.
//
// Same V-cycle as the per-level path (pre-smoothing + residual restriction on
// the way down, bottom relaxation, prolongation + post-smoothing on the way
// up), in the lean FP32 form of the tile smoother: with c_f = beta b_f / dx^2
// and diag = resetLambda's diagonal, a red/black update is
//   e <- (1/diag) (r + sum_f c_f e_nb(f)),
// where a homogeneous boundary ghost contributes c_f (-e) (Dirichlet) or
// c_f e (Neumann).  Thread t owns the 2x2 fine quad under coarse cell t, so
// the restriction of its residual needs no exchange; on each level visit it
// keeps its cells' neighbour indices, ghost-folded weights, 1/diag and
// right-hand side in registers, and a half sweep is four shared-memory loads
// and five FP32 operations per cell.  Everything lives in shared memory; only
// the top level's correction goes back to global memory.
#pragma once
#include "tile_fast_kernels.cuh"

namespace mlgpu {

constexpr int kFastCycLevels = 12;
constexpr int kFastCycThreads = 256;  // quads of a 1024-cell top level
constexpr long long kFastCycCells = 4 * kFastCycThreads;

struct CycFast {
  int nlev, pre, post, bottom, prolong, zero_init;
  BCD bc;
  Geom G[kFastCycLevels];
  FastCoefs K[kFastCycLevels];
  float *e0;        // top level correction (written; read first unless zero_init)
  const float *r0;  // top level right-hand side
};

// shared-memory floats of level m: e, r, lam, diag (cells), cx, cy (faces)
__host__ __device__ inline int cyc_fast_level_floats(const Geom &G) {
  return 4 * G.n0 * G.n1 + (G.n0 + 1) * G.n1 + G.n0 * (G.n1 + 1);
}
inline size_t cyc_fast_smem_bytes(const CycFast &P) {
  size_t n = 0;
  for (int m = 0; m < P.nlev; m++) n += cyc_fast_level_floats(P.G[m]);
  return n * sizeof(float);
}

#ifdef MLGPU_FP32_UNIT  // kernels compiled in launch_f32.cu only
struct CycLevel {
  int n0, n1, per0, per1;
  float *e, *r, *lam, *diag, *cx, *cy;
};

// one cell's update data on the current level visit
struct CycCell {
  int c, w, e, s, n;
  float kw, ke, ks, kn, lam, r;
};

__device__ __forceinline__ void cyc_cell_setup(const CycLevel &V, const BCD &bc, int i, int j,
                                               CycCell &k) {
  const int n0 = V.n0, n1 = V.n1;
  const int c = j * n0 + i, fc = j * (n0 + 1) + i;
  k.c = c;
  float cxh = V.cx[fc + 1], cxl = V.cx[fc], cyh = V.cy[c + n0], cyl = V.cy[c];
  if (i + 1 < n0) {
    k.e = c + 1;
    k.ke = cxh;
  } else if (V.per0) {
    k.e = j * n0;
    k.ke = cxh;
  } else {
    k.e = c;
    k.ke = ghost_factor(bc, 0, 1) * cxh;
  }
  if (i > 0) {
    k.w = c - 1;
    k.kw = cxl;
  } else if (V.per0) {
    k.w = j * n0 + n0 - 1;
    k.kw = cxl;
  } else {
    k.w = c;
    k.kw = ghost_factor(bc, 0, 0) * cxl;
  }
  if (j + 1 < n1) {
    k.n = c + n0;
    k.kn = cyh;
  } else if (V.per1) {
    k.n = i;
    k.kn = cyh;
  } else {
    k.n = c;
    k.kn = ghost_factor(bc, 1, 1) * cyh;
  }
  if (j > 0) {
    k.s = c - n0;
    k.ks = cyl;
  } else if (V.per1) {
    k.s = (n1 - 1) * n0 + i;
    k.ks = cyl;
  } else {
    k.s = c;
    k.ks = ghost_factor(bc, 1, 0) * cyl;
  }
  k.lam = V.lam[c];
  k.r = V.r[c];
}

__device__ __forceinline__ float cyc_nbsum(const float *e, const CycCell &k) {
  float s = k.ke * e[k.e];
  s = fmaf(k.kw, e[k.w], s);
  s = fmaf(k.kn, e[k.n], s);
  s = fmaf(k.ks, e[k.s], s);
  return s;
}

__device__ __forceinline__ void cyc_update(float *e, const CycCell &k) {
  e[k.c] = k.lam * (k.r + cyc_nbsum(e, k));
}

template <bool WARP>
__device__ __forceinline__ void cycf_sync() {
  if (WARP)
    __syncwarp();
  else
    __syncthreads();
}

// two same-colour cells of a quad: all eight neighbour values are read
// before either cell is written (same-colour cells are never neighbours)
__device__ __forceinline__ void cyc_update2(float *e, const CycCell &a, const CycCell &b) {
  float a0 = e[a.e], a1 = e[a.w], a2 = e[a.n], a3 = e[a.s];
  float b0 = e[b.e], b1 = e[b.w], b2 = e[b.n], b3 = e[b.s];
  float sa = a.ke * a0, sb = b.ke * b0;
  sa = fmaf(a.kw, a1, sa);
  sb = fmaf(b.kw, b1, sb);
  sa = fmaf(a.kn, a2, sa);
  sb = fmaf(b.kn, b2, sb);
  sa = fmaf(a.ks, a3, sa);
  sb = fmaf(b.ks, b3, sb);
  e[a.c] = a.lam * (a.r + sa);
  e[b.c] = b.lam * (b.r + sb);
}

// n red/black sweeps of the quad's four cells: pass 0 updates (0,0), (1,1),
// pass 1 updates (1,0), (0,1) of the quad (its origin has even i + j)
template <bool WARP>
__device__ __forceinline__ void cyc_quad_relax(float *e, const CycCell *q, bool own, int n) {
  for (int s = 0; s < n; s++) {
    if (own) cyc_update2(e, q[0], q[3]);
    cycf_sync<WARP>();
    if (own) cyc_update2(e, q[1], q[2]);
    cycf_sync<WARP>();
  }
}

__device__ __forceinline__ CycLevel cyc_level(const CycFast &P, const int *off, float *pool,
                                              int m) {
  CycLevel V;
  const Geom &G = P.G[m];
  V.n0 = G.n0;
  V.n1 = G.n1;
  V.per0 = G.per0;
  V.per1 = G.per1;
  const int n = G.n0 * G.n1;
  V.e = pool + off[m];
  V.r = V.e + n;
  V.lam = V.r + n;
  V.diag = V.lam + n;
  V.cx = V.diag + n;
  V.cy = V.cx + (G.n0 + 1) * G.n1;
  return V;
}

__device__ __forceinline__ void cyc_quad_setup(const CycLevel &V, const BCD &bc, int I, int J,
                                               CycCell *q) {
  cyc_cell_setup(V, bc, 2 * I, 2 * J, q[0]);
  cyc_cell_setup(V, bc, 2 * I + 1, 2 * J, q[1]);
  cyc_cell_setup(V, bc, 2 * I, 2 * J + 1, q[2]);
  cyc_cell_setup(V, bc, 2 * I + 1, 2 * J + 1, q[3]);
}

// level m on the way down: pre-smoothing, residual restricted to level m+1
template <bool WARP>
__device__ __forceinline__ void cyc_down(const CycFast &P, const int *off, float *pool, int m) {
  const int tid = threadIdx.x;
  CycLevel V = cyc_level(P, off, pool, m);
  const int cn0 = V.n0 >> 1, cn1 = V.n1 >> 1;
  const bool own = tid < cn0 * cn1;
  CycCell q[4];
  int I = 0, J = 0;
  if (own) {
    I = tid % cn0;
    J = tid / cn0;
    cyc_quad_setup(V, P.bc, I, J, q);
  }
  cyc_quad_relax<WARP>(V.e, q, own, P.pre);
  if (own) {
    // residual r - diag e + sum c e_nb of the four cells, averaged
    float acc = 0.f;
#pragma unroll
    for (int t = 0; t < 4; t++) {
      float res = q[t].r - V.diag[q[t].c] * V.e[q[t].c] + cyc_nbsum(V.e, q[t]);
      acc = acc + res * 0.25f;
    }
    CycLevel W = cyc_level(P, off, pool, m + 1);
    W.r[J * cn0 + I] = acc;
  }
  cycf_sync<WARP>();
}

// level m on the way up: prolong level m+1's correction, post-smoothing
template <bool WARP>
__device__ __forceinline__ void cyc_up(const CycFast &P, const int *off, float *pool, int m) {
  const int tid = threadIdx.x;
  CycLevel V = cyc_level(P, off, pool, m);
  CycLevel W = cyc_level(P, off, pool, m + 1);
  const int cn0 = V.n0 >> 1, cn1 = V.n1 >> 1;
  const bool own = tid < cn0 * cn1;
  CycCell q[4];
  if (own) {
    const int I = tid % cn0, J = tid / cn0;
    cyc_quad_setup(V, P.bc, I, J, q);
    if (P.prolong == MLGPU_PROLONG_LINEAR) {
      const Geom &C = P.G[m + 1];
#pragma unroll
      for (int t = 0; t < 4; t++) {
        int i = 2 * I + (t & 1), j = 2 * J + (t >> 1);
        V.e[q[t].c] = prolong_add<float, 2, MLGPU_PROLONG_LINEAR>(C, P.bc, 0, i, j, 0,
                                                                  V.e[q[t].c], W.e, nullptr);
      }
    } else {
      float ec = W.e[J * cn0 + I];
#pragma unroll
      for (int t = 0; t < 4; t++) V.e[q[t].c] = V.e[q[t].c] + ec;
    }
  }
  cycf_sync<WARP>();
  cyc_quad_relax<WARP>(V.e, q, own, P.post);
}

// bottom level: relaxation from zero, one cell per thread.  With an odd
// periodic extent two same-colour cells meet across the seam; the values
// are then all read before any is written (the reference reads that
// neighbour from a ghost filled before the pass).
template <bool WARP>
__device__ __forceinline__ void cyc_bottom(const CycFast &P, const int *off, float *pool) {
  const int tid = threadIdx.x;
  CycLevel V = cyc_level(P, off, pool, P.nlev - 1);
  const int n = V.n0 * V.n1;
  const bool own = tid < n;
  const bool seam = (V.per0 && (V.n0 & 1)) || (V.per1 && (V.n1 & 1));
  CycCell b;
  int colour = 0;
  if (own) {
    int i = tid % V.n0, j = tid / V.n0;
    colour = (i + j) & 1;
    cyc_cell_setup(V, P.bc, i, j, b);
  }
  for (int s = 0; s < 2 * P.bottom; s++) {
    const bool mine = own && colour == (s & 1);
    if (seam) {
      float v = mine ? b.lam * (b.r + cyc_nbsum(V.e, b)) : 0.f;
      cycf_sync<WARP>();
      if (mine) V.e[b.c] = v;
    } else if (mine) {
      cyc_update(V.e, b);
    }
    cycf_sync<WARP>();
  }
}

__device__ __forceinline__ void cyc_copy_async(float *dst, const float *src) {
  unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}

__global__ void __launch_bounds__(kFastCycThreads) vc_cycle_fast_kernel(CycFast P) {
  extern __shared__ __align__(16) float cyc_pool[];
  __shared__ int off[kFastCycLevels + 1];
  const int tid = threadIdx.x, nth = blockDim.x;
  if (tid == 0) {
    int o = 0;
    for (int m = 0; m < P.nlev; m++) {
      off[m] = o;
      o += cyc_fast_level_floats(P.G[m]);
    }
    off[P.nlev] = o;
  }
  __syncthreads();
  // stage coefficients of every level and the top level's r (and e): all
  // copies in flight at once
  for (int m = 0; m < P.nlev; m++) {
    CycLevel V = cyc_level(P, off, cyc_pool, m);
    const int n = V.n0 * V.n1, nfx = (V.n0 + 1) * V.n1, nfy = V.n0 * (V.n1 + 1);
    for (int q = tid; q < n; q += nth) {
      cyc_copy_async(V.lam + q, P.K[m].lam + q);
      cyc_copy_async(V.diag + q, P.K[m].diag + q);
      if (m == 0) {
        cyc_copy_async(V.r + q, P.r0 + q);
        if (!P.zero_init)
          cyc_copy_async(V.e + q, P.e0 + q);
        else
          V.e[q] = 0.f;
      } else {
        V.e[q] = 0.f;
      }
    }
    for (int q = tid; q < nfx; q += nth) cyc_copy_async(V.cx + q, P.K[m].cx + q);
    for (int q = tid; q < nfy; q += nth) cyc_copy_async(V.cy + q, P.K[m].cy + q);
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  __syncthreads();

  const int last = P.nlev - 1;
  // first level whose quads fit in one warp (the rest run on warp 0 alone)
  int mw = last;
  for (int m = 0; m < last; m++)
    if ((P.G[m].n0 >> 1) * (P.G[m].n1 >> 1) <= 32) {
      mw = m;
      break;
    }
  for (int m = 0; m < mw; m++) cyc_down<false>(P, off, cyc_pool, m);
  if (mw < last) {
    if (tid < 32) {
      for (int m = mw; m < last; m++) cyc_down<true>(P, off, cyc_pool, m);
      cyc_bottom<true>(P, off, cyc_pool);
      for (int m = last - 1; m >= mw; m--) cyc_up<true>(P, off, cyc_pool, m);
    }
    __syncthreads();
  } else {
    cyc_bottom<false>(P, off, cyc_pool);
  }
  for (int m = mw - 1; m >= 0; m--) cyc_up<false>(P, off, cyc_pool, m);
  // the top level's correction back to global memory
  {
    CycLevel V = cyc_level(P, off, cyc_pool, 0);
    const int n = V.n0 * V.n1;
    for (int c = tid; c < n; c += nth) P.e0[c] = V.e[c];
  }
}
#endif  // MLGPU_FP32_UNIT

}  // namespace mlgpu
