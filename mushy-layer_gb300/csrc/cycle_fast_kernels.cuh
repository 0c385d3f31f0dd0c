// cycle_fast_kernels.cuh -- lean FP32 coarse end of the mixed-precision
// V-cycle (2D): every level from a top of at most 1024 cells down to the
// bottom inside one CTA (one thread per quad of the top level); levels of at
// most 32 quads and the bottom run on warp 0 alone.
//
// Same V-cycle as the per-level path (pre-smoothing + residual restriction on
// the way down, bottom relaxation, prolongation + post-smoothing on the way
// up), in the lean FP32 form of the tile smoother: with c_f = beta b_f / dx^2
// and diag = resetLambda's diagonal, a red/black update is
//   e <- (1/diag) (r + sum_f w_f e[nb_f]),
// where w_f = c_f and nb_f the neighbour across face f, or, across a
// non-periodic boundary face, w_f = g c_f (g = -1 Dirichlet, +1 Neumann: the
// homogeneous ghost g e) and nb_f the cell itself.
//
// The per-cell constants of every level (1/diag, diag, the four weights and
// the four neighbour indices packed two per word) are built once per operator
// into one "level pack" laid out exactly like the kernel's shared-memory
// image, so staging is one bulk (TMA) copy and a level visit reads each
// cell's constants with a few vector shared-memory loads.  Thread t owns the
// 2x2 fine quad under coarse cell t, so the restriction of its residual needs
// no exchange.  Only the top level's correction goes back to global memory.
#pragma once
#include "tile_fast_kernels.cuh"

namespace mlgpu {

constexpr int kFastCycLevels = 12;
constexpr int kFastCycThreads = 256;  // quads of a 1024-cell top level
constexpr long long kFastCycCells = 4 * kFastCycThreads;

// cells of a level rounded up to a multiple of 4 (16-byte segments)
__host__ __device__ inline int cyc_pad(int n) { return (n + 3) & ~3; }
// floats of one level in the pack: lam, diag (np each), weights (4 np),
// neighbour words (2 np)
__host__ __device__ inline int cyc_pack_level_floats(int ncell) { return 8 * cyc_pad(ncell); }

struct CycFast {
  int nlev, pre, post, bottom, prolong, zero_init;
  BCD bc;
  Geom G[kFastCycLevels];
  int off[kFastCycLevels + 1];  // level offsets in the pack (floats); off[nlev] = pack size
  const float4 *pack;           // 16-byte aligned
  float *e0;                    // top level correction (written; read first unless zero_init)
  const float *r0;              // top level right-hand side (16-byte aligned)
  int *fault;                   // set to 1 when the staging wait runs past its bound
};

// shared-memory bytes: the pack + e and r of every level
inline size_t cyc_fast_smem_bytes(const CycFast &P) {
  size_t n = (size_t)P.off[P.nlev];
  for (int m = 0; m < P.nlev; m++) n += 2 * (size_t)cyc_pad((int)P.G[m].ncell);
  return n * sizeof(float);
}

#ifdef MLGPU_FP32_UNIT  // kernels compiled in launch_f32.cu only
// pack entries of one level (FP32 lean coefficients and boundary conditions)
__global__ void __launch_bounds__(kBlock) cyc_pack_kernel(Geom G, BCD bc, FastCoefs K, float *lv) {
  const int n0 = G.n0, n1 = G.n1, n = n0 * n1, np = cyc_pad(n);
  float *lam = lv, *diag = lv + np;
  float4 *w = reinterpret_cast<float4 *>(lv + 2 * np);
  uint2 *nb = reinterpret_cast<uint2 *>(lv + 6 * np);
  for (int c = (int)gtid(); c < np; c += (int)gstride()) {
    if (c >= n) {
      lam[c] = diag[c] = 0.f;
      w[c] = make_float4(0.f, 0.f, 0.f, 0.f);
      nb[c] = make_uint2((unsigned)c | ((unsigned)c << 16), (unsigned)c | ((unsigned)c << 16));
      continue;
    }
    const int i = c % n0, j = c / n0, fc = j * (n0 + 1) + i;
    float ke = K.cx[fc + 1], kw = K.cx[fc], kn = K.cy[c + n0], ks = K.cy[c];
    int ie, iw, in, is;
    if (i + 1 < n0) {
      ie = c + 1;
    } else if (G.per0) {
      ie = j * n0;
    } else {
      ie = c;
      ke = ghost_factor(bc, 0, 1) * ke;
    }
    if (i > 0) {
      iw = c - 1;
    } else if (G.per0) {
      iw = j * n0 + n0 - 1;
    } else {
      iw = c;
      kw = ghost_factor(bc, 0, 0) * kw;
    }
    if (j + 1 < n1) {
      in = c + n0;
    } else if (G.per1) {
      in = i;
    } else {
      in = c;
      kn = ghost_factor(bc, 1, 1) * kn;
    }
    if (j > 0) {
      is = c - n0;
    } else if (G.per1) {
      is = (n1 - 1) * n0 + i;
    } else {
      is = c;
      ks = ghost_factor(bc, 1, 0) * ks;
    }
    lam[c] = K.lam[c];
    diag[c] = K.diag[c];
    w[c] = make_float4(ke, kw, kn, ks);
    nb[c] = make_uint2((unsigned)ie | ((unsigned)iw << 16), (unsigned)in | ((unsigned)is << 16));
  }
}

struct CycLevel {
  int n0, n1, np;
  const float *lam, *diag;
  const float4 *w;
  const uint2 *nb;
  float *e, *r;
};

// one cell's update data on the current level visit
struct CycCell {
  int c, ie, iw, in, is;
  float ke, kw, kn, ks, lam, r;
};

__device__ __forceinline__ void cyc_cell_setup(const CycLevel &V, int c, CycCell &k) {
  const float4 w = V.w[c];
  const uint2 nb = V.nb[c];
  k.c = c;
  k.ke = w.x;
  k.kw = w.y;
  k.kn = w.z;
  k.ks = w.w;
  k.ie = (int)(nb.x & 0xffffu);
  k.iw = (int)(nb.x >> 16);
  k.in = (int)(nb.y & 0xffffu);
  k.is = (int)(nb.y >> 16);
  k.lam = V.lam[c];
  k.r = V.r[c];
}

__device__ __forceinline__ float cyc_nbsum(const float *e, const CycCell &k) {
  float s = k.ke * e[k.ie];
  s = fmaf(k.kw, e[k.iw], s);
  s = fmaf(k.kn, e[k.in], s);
  s = fmaf(k.ks, e[k.is], s);
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
  float a0 = e[a.ie], a1 = e[a.iw], a2 = e[a.in], a3 = e[a.is];
  float b0 = e[b.ie], b1 = e[b.iw], b2 = e[b.in], b3 = e[b.is];
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

// per-level geometry, built once per launch in shared memory (reading the
// launch parameters with a run-time level index goes through the constant
// cache, which costs hundreds of cycles per level visit)
struct CycTab {
  int n0, n1, np, pack, dyn, cshift;  // cshift: log2(n0 / 2), or -1
  int per0, per1;
};

// shared-memory view of level m: constants in the staged pack, then e, r
__device__ __forceinline__ CycLevel cyc_level(const CycTab *tab, float *pool, int m) {
  CycLevel V;
  const CycTab &t = tab[m];
  V.n0 = t.n0;
  V.n1 = t.n1;
  V.np = t.np;
  const float *lv = pool + t.pack;
  V.lam = lv;
  V.diag = lv + t.np;
  V.w = reinterpret_cast<const float4 *>(lv + 2 * t.np);
  V.nb = reinterpret_cast<const uint2 *>(lv + 6 * t.np);
  V.e = pool + t.dyn;
  V.r = V.e + t.np;
  return V;
}

// quad coordinates of thread tid on a level (shift when n0 / 2 is a power of 2)
__device__ __forceinline__ void cyc_quad_of(const CycTab &t, int tid, int &I, int &J) {
  if (t.cshift >= 0) {
    I = tid & ((1 << t.cshift) - 1);
    J = tid >> t.cshift;
  } else {
    I = tid % (t.n0 >> 1);
    J = tid / (t.n0 >> 1);
  }
}

__device__ __forceinline__ void cyc_quad_setup(const CycLevel &V, int I, int J, CycCell *q) {
  const int c = 2 * J * V.n0 + 2 * I;
  cyc_cell_setup(V, c, q[0]);
  cyc_cell_setup(V, c + 1, q[1]);
  cyc_cell_setup(V, c + V.n0, q[2]);
  cyc_cell_setup(V, c + V.n0 + 1, q[3]);
}

// level m on the way down: pre-smoothing, residual restricted to level m+1
template <bool WARP>
__device__ __forceinline__ void cyc_down(const CycFast &P, const CycTab *tab, float *pool, int m) {
  const int tid = threadIdx.x;
  CycLevel V = cyc_level(tab, pool, m);
  const int cn0 = V.n0 >> 1, cn1 = V.n1 >> 1;
  const bool own = tid < cn0 * cn1;
  CycCell q[4];
  int I = 0, J = 0;
  if (own) {
    cyc_quad_of(tab[m], tid, I, J);
    cyc_quad_setup(V, I, J, q);
  }
  cyc_quad_relax<WARP>(V.e, q, own, P.pre);
  if (own) {
    // residual r - diag e + sum w e_nb of the four cells, averaged
    float acc = 0.f;
#pragma unroll
    for (int t = 0; t < 4; t++) {
      float res = q[t].r - V.diag[q[t].c] * V.e[q[t].c] + cyc_nbsum(V.e, q[t]);
      acc = acc + res * 0.25f;
    }
    CycLevel W = cyc_level(tab, pool, m + 1);
    W.r[J * cn0 + I] = acc;
  }
  cycf_sync<WARP>();
}

// level m on the way up: prolong level m+1's correction, post-smoothing
template <bool WARP>
__device__ __forceinline__ void cyc_up(const CycFast &P, const CycTab *tab, float *pool, int m) {
  const int tid = threadIdx.x;
  CycLevel V = cyc_level(tab, pool, m);
  CycLevel W = cyc_level(tab, pool, m + 1);
  const int cn0 = V.n0 >> 1, cn1 = V.n1 >> 1;
  const bool own = tid < cn0 * cn1;
  CycCell q[4];
  if (own) {
    int I, J;
    cyc_quad_of(tab[m], tid, I, J);
    cyc_quad_setup(V, I, J, q);
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
__device__ __forceinline__ void cyc_bottom(const CycFast &P, const CycTab *tab, float *pool) {
  const int tid = threadIdx.x;
  const CycTab &t = tab[P.nlev - 1];
  CycLevel V = cyc_level(tab, pool, P.nlev - 1);
  const int n = V.n0 * V.n1;
  const bool own = tid < n;
  const bool seam = (t.per0 && (V.n0 & 1)) || (t.per1 && (V.n1 & 1));
  CycCell b;
  int colour = 0;
  if (own) {
    colour = ((tid % V.n0) + (tid / V.n0)) & 1;
    cyc_cell_setup(V, tid, b);
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

__device__ __forceinline__ unsigned cyc_smem_addr(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

// bound of the staging wait (polls of mbarrier.try_wait, each of which may
// itself suspend the thread for a while); far beyond any real copy time
constexpr int kCycWaitPolls = 1 << 22;

__device__ __forceinline__ bool cyc_try_wait(unsigned long long *bar) {
  unsigned ok;
  asm volatile(
      "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0; selp.u32 %0, 1, 0, p; }"
      : "=r"(ok)
      : "r"(cyc_smem_addr(bar))
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ void cyc_bulk_copy(void *dst, const void *src, unsigned bytes,
                                              unsigned long long *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          cyc_smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(cyc_smem_addr(bar))
      : "memory");
}

__global__ void __launch_bounds__(kFastCycThreads) vc_cycle_fast_kernel(CycFast P) {
  extern __shared__ __align__(16) float cyc_pool[];
  __shared__ CycTab tab[kFastCycLevels];
  __shared__ __align__(8) unsigned long long bar;
  const int tid = threadIdx.x, nth = blockDim.x;
  const int n_top = P.G[0].n0 * P.G[0].n1, np_top = cyc_pad(n_top);
  const int dyn0 = P.off[P.nlev];
  // per-level table (one thread per level)
  if (tid < P.nlev) {
    const Geom &G = P.G[tid];
    CycTab t;
    t.n0 = G.n0;
    t.n1 = G.n1;
    t.np = cyc_pad(G.n0 * G.n1);
    t.pack = P.off[tid];
    int dyn = dyn0;
    for (int k = 0; k < tid; k++) dyn += 2 * cyc_pad(P.G[k].n0 * P.G[k].n1);
    t.dyn = dyn;
    const int c0 = G.n0 >> 1;
    t.cshift = (c0 > 0 && (c0 & (c0 - 1)) == 0) ? __ffs(c0) - 1 : -1;
    t.per0 = G.per0;
    t.per1 = G.per1;
    tab[tid] = t;
  }
  // bulk copies (TMA): the whole pack, the top level's r (and e), whole
  // 16-byte segments; the few trailing values with plain loads
  const unsigned pack_bytes = 4u * (unsigned)P.off[P.nlev];
  const unsigned top_bytes = 16u * (unsigned)(n_top >> 2);
  float *top_e = cyc_pool + dyn0, *top_r = top_e + np_top;
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(cyc_smem_addr(&bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    const unsigned total = pack_bytes + top_bytes + (P.zero_init ? 0u : top_bytes);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(cyc_smem_addr(&bar)),
                 "r"(total)
                 : "memory");
    cyc_bulk_copy(cyc_pool, P.pack, pack_bytes, &bar);
    if (top_bytes) {
      cyc_bulk_copy(top_r, P.r0, top_bytes, &bar);
      if (!P.zero_init) cyc_bulk_copy(top_e, P.e0, top_bytes, &bar);
    }
  }
  // meanwhile: the trailing top values and the zero corrections (other bytes)
  for (int q = (n_top & ~3) + tid; q < n_top; q += nth) {
    top_r[q] = P.r0[q];
    if (!P.zero_init) top_e[q] = P.e0[q];
  }
  {
    float *e_end = cyc_pool + dyn0;
    for (int m = 0; m < P.nlev; m++) e_end += 2 * cyc_pad(P.G[m].n0 * P.G[m].n1);
    // top e when starting from zero, every coarser e and r
    for (float *p = (P.zero_init ? top_e : top_e + 2 * np_top) + tid; p < e_end; p += nth)
      if (p < top_r || p >= top_r + np_top) *p = 0.f;
  }
  __syncthreads();  // the barrier is initialised before anyone polls it
  bool ready = false;
  for (int it = 0; it < kCycWaitPolls && !ready; it++) ready = cyc_try_wait(&bar);
  if (__syncthreads_or(!ready)) {
    // report and leave; the copies get a second bounded wait first
    if (tid == 0) {
      if (P.fault) *P.fault = 1;
      for (int it = 0; it < kCycWaitPolls; it++)
        if (cyc_try_wait(&bar)) break;
    }
    __syncthreads();
    return;
  }

  const int last = P.nlev - 1;
  // first level whose quads fit in one warp (the rest run on warp 0 alone)
  int mw = last;
  for (int m = 0; m < last; m++)
    if ((tab[m].n0 >> 1) * (tab[m].n1 >> 1) <= 32) {
      mw = m;
      break;
    }
  for (int m = 0; m < mw; m++) cyc_down<false>(P, tab, cyc_pool, m);
  if (mw < last) {
    if (tid < 32) {
      for (int m = mw; m < last; m++) cyc_down<true>(P, tab, cyc_pool, m);
      cyc_bottom<true>(P, tab, cyc_pool);
      for (int m = last - 1; m >= mw; m--) cyc_up<true>(P, tab, cyc_pool, m);
    }
    __syncthreads();
  } else {
    cyc_bottom<false>(P, tab, cyc_pool);
  }
  for (int m = mw - 1; m >= 0; m--) cyc_up<false>(P, tab, cyc_pool, m);
  // the top level's correction back to global memory
  for (int c = tid; c < n_top; c += nth) P.e0[c] = top_e[c];
}
#endif  // MLGPU_FP32_UNIT

}  // namespace mlgpu
