// cycle_kernels.cuh -- the coarse end of a multigrid V-cycle in ONE thread
// block.  Below a few hundred cells a level's work is far smaller than a
// kernel launch, so every level from `A[0]` down to the bottom runs inside a
// single CTA: relax, restrict, bottom relaxation, prolong, relax.  Levels of
// at most 64 cells (and the bottom) are finished by warp 0 alone with warp
// barriers, the larger ones by the whole block with block barriers.  Each
// cell update calls the same device functions as the per-level kernels, so
// results are bit-identical to launching the per-level kernels in sequence.
#pragma once
#include "vc_kernels.cuh"
#include "misc_kernels.cuh"

namespace mlgpu {

constexpr int kMaxBlockLevels = 12;
constexpr long long kWarpLevelCells = 64;

template <class T>
struct VCBlockCycle {
  int nlev;                       // levels A[0..nlev-1]; A[nlev-1] is the bottom
  int pre, post, bottom, prolong;
  int zero_init;                  // the top level starts from e = 0
  BCD bc;
  VCArgs<T> A[kMaxBlockLevels];
  T *e[kMaxBlockLevels];
  T *r[kMaxBlockLevels];
};

// WARP: the phase is run by warp 0 only (32 lanes, __syncwarp); otherwise by
// the whole block (__syncthreads).
template <bool WARP>
__device__ __forceinline__ void cyc_sync() {
  if (WARP)
    __syncwarp();
  else
    __syncthreads();
}
template <bool WARP>
__device__ __forceinline__ int cyc_nthreads() {
  return WARP ? 32 : (int)blockDim.x;
}

template <class T, int DIM, bool WARP>
__device__ __noinline__ void blk_half_sweep(const VCArgs<T> &A, T *e, const T *r, int pass) {
  long long nt = colour_threads(A.G);
  for (long long t = threadIdx.x; t < nt; t += cyc_nthreads<WARP>()) {
    int i, j, k;
    if (colour_cell(A.G, pass, t, i, j, k)) vc_gsrb_cell<T, DIM>(A, e, r, i, j, k);
  }
  cyc_sync<WARP>();
}

// VCSolver::relax for GSRB, inside the block (or warp)
template <class T, int DIM, bool WARP>
__device__ __noinline__ void blk_relax(const VCArgs<T> &A, T *e, const T *r, int n, bool zero_init) {
  const int nth = cyc_nthreads<WARP>();
  if (zero_init) {
    if (n == 0) {
      for (long long q = threadIdx.x; q < A.G.ncell; q += nth) e[q] = T(0);
      cyc_sync<WARP>();
      return;
    }
    for (long long q = threadIdx.x; q < A.G.ncell; q += nth) {
      int i, j, k;
      cell_ijk(A.G, q, i, j, k);
      vc_gsrb_zero_cell<T, DIM>(A, e, r, q, i, j, k);
    }
    cyc_sync<WARP>();
    blk_half_sweep<T, DIM, WARP>(A, e, r, 1);
    n--;
  }
  for (int s = 0; s < n; s++) {
    blk_half_sweep<T, DIM, WARP>(A, e, r, 0);
    blk_half_sweep<T, DIM, WARP>(A, e, r, 1);
  }
}

template <class T, int DIM, bool WARP>
__device__ __noinline__ void blk_restrict(const VCBlockCycle<T> &P, int l) {
  const VCArgs<T> &A = P.A[l];
  const T denom = DIM == 3 ? T(8) : T(4);
  const Geom &C = P.A[l + 1].G;
  PlainRead<T> rd{P.e[l]};
  for (long long Q = threadIdx.x; Q < C.ncell; Q += cyc_nthreads<WARP>()) {
    int I, J, K;
    cell_ijk(C, Q, I, J, K);
    T acc = T(0);
    for (int kk = 0; kk < (DIM == 3 ? 2 : 1); kk++)
      for (int jj = 0; jj < 2; jj++)
        for (int ii = 0; ii < 2; ii++) {
          int i = 2 * I + ii, j = 2 * J + jj, k = DIM == 3 ? 2 * K + kk : 0;
          T p0, lam;
          T lof = vc_lofphi<T, DIM, false>(A, rd, i, j, k, true, p0, lam);
          acc = acc + (P.r[l][A.G.cell(i, j, k)] - lof) / denom;
        }
    P.r[l + 1][Q] = acc;
  }
  cyc_sync<WARP>();
}

template <class T, int DIM, bool WARP>
__device__ __noinline__ void blk_prolong(const VCBlockCycle<T> &P, int l) {
  const Geom &F = P.A[l].G, &C = P.A[l + 1].G;
  for (long long t = threadIdx.x; t < F.ncell; t += cyc_nthreads<WARP>()) {
    if (P.prolong == MLGPU_PROLONG_LINEAR)
      prolong_one<T, DIM, MLGPU_PROLONG_LINEAR>(F, C, P.bc, t, P.e[l], P.e[l + 1], nullptr);
    else
      prolong_one<T, DIM, MLGPU_PROLONG_CONSTANT>(F, C, P.bc, t, P.e[l], P.e[l + 1], nullptr);
  }
  cyc_sync<WARP>();
}

// levels [l0, last] with the bottom, by the block (WARP false) or warp 0
template <class T, int DIM, bool WARP>
__device__ void blk_cycle_range(const VCBlockCycle<T> &P, int l0, int l1, bool zero_top) {
  // down over [l0, l1): pre-smooth and restrict; l1 is handled by the caller
  for (int l = l0; l < l1; l++) {
    blk_relax<T, DIM, WARP>(P.A[l], P.e[l], P.r[l], P.pre, l > l0 || zero_top);
    blk_restrict<T, DIM, WARP>(P, l);
  }
}
template <class T, int DIM, bool WARP>
__device__ void blk_cycle_up(const VCBlockCycle<T> &P, int l0, int l1) {
  // up over (l0 .. l1] reversed: prolong into l, post-smooth l
  for (int l = l1 - 1; l >= l0; l--) {
    blk_prolong<T, DIM, WARP>(P, l);
    blk_relax<T, DIM, WARP>(P.A[l], P.e[l], P.r[l], P.post, false);
  }
}

// Shared-memory image of every level of the cycle: the descriptor itself and,
// per level, e, r, 1/diag and the faces.  The cell-update code reads them
// through the descriptor's pointers, so the arithmetic is unchanged; only the
// latency of each of the ~80 barrier-separated phases drops from L2 round
// trips to shared-memory accesses.
template <class T>
__host__ __device__ inline size_t block_cycle_smem_elems(const VCBlockCycle<T> &P) {
  size_t n = 0;
  for (int m = 0; m < P.nlev; m++) {
    const Geom &G = P.A[m].G;
    n += 3 * (size_t)G.ncell;
    for (int d = 0; d < G.dim; d++) n += (size_t)G.nface(d);
  }
  return n;
}
template <class T>
inline size_t block_cycle_smem_bytes(const VCBlockCycle<T> &P) {
  return ((sizeof(VCBlockCycle<T>) + 15) & ~(size_t)15) + sizeof(T) * block_cycle_smem_elems(P);
}

template <class T, int DIM>
__global__ void __launch_bounds__(256) vc_block_cycle_kernel(VCBlockCycle<T> Pg) {
  extern __shared__ __align__(16) unsigned char cyc_smem[];
  VCBlockCycle<T> &P = *reinterpret_cast<VCBlockCycle<T> *>(cyc_smem);
  T *pool = reinterpret_cast<T *>(cyc_smem + ((sizeof(VCBlockCycle<T>) + 15) & ~(size_t)15));
  T *top_e = Pg.e[0];
  if (threadIdx.x == 0) {
    P = Pg;
    size_t off = 0;
    for (int m = 0; m < Pg.nlev; m++) {
      const Geom &G = Pg.A[m].G;
      P.e[m] = pool + off;
      off += G.ncell;
      P.r[m] = pool + off;
      off += G.ncell;
      P.A[m].lam = pool + off;
      off += G.ncell;
      for (int d = 0; d < G.dim; d++) {
        P.A[m].b[d] = pool + off;
        off += G.nface(d);
      }
    }
  }
  __syncthreads();
  // stage faces, the top level's right-hand side and correction
  for (int m = 0; m < Pg.nlev; m++) {
    const Geom &G = Pg.A[m].G;
    for (int d = 0; d < G.dim; d++)
      for (long long q = threadIdx.x; q < G.nface(d); q += blockDim.x)
        const_cast<T *>(P.A[m].b[d])[q] = Pg.A[m].b[d][q];
  }
  for (long long q = threadIdx.x; q < Pg.A[0].G.ncell; q += blockDim.x) {
    P.r[0][q] = Pg.r[0][q];
    if (!Pg.zero_init) P.e[0][q] = top_e[q];
  }
  __syncthreads();
  // 1/diag per level, from the stored array or in resetLambda order
  for (int m = 0; m < Pg.nlev; m++) {
    const VCArgs<T> &A = P.A[m];
    for (long long q = threadIdx.x; q < A.G.ncell; q += blockDim.x) {
      T lv;
      if (Pg.A[m].lam) {
        lv = Pg.A[m].lam[q];
      } else {
        int i, j, k;
        cell_ijk(A.G, q, i, j, k);
        T bzh = T(0), bzl = T(0);
        if (DIM == 3) {
          bzh = vface(A, 2, i, j, k + 1);
          bzl = vface(A, 2, i, j, k);
        }
        VCArgs<T> Ai = A;
        Ai.lam = nullptr;
        lv = vc_lambda_at<T, DIM>(Ai, q, vface(A, 0, i + 1, j, k), vface(A, 0, i, j, k),
                                  vface(A, 1, i, j + 1, k), vface(A, 1, i, j, k), bzh, bzl);
      }
      const_cast<T *>(A.lam)[q] = lv;
    }
  }
  __syncthreads();
  const int last = P.nlev - 1;
  // first level small enough for warp 0 alone (the bottom at the latest)
  int lw = last;
  for (int l = 0; l < last; l++)
    if (P.A[l].G.ncell <= kWarpLevelCells) {
      lw = l;
      break;
    }
  const bool warp_bottom = P.A[last].G.ncell <= kWarpLevelCells;
  // block part, down
  blk_cycle_range<T, DIM, false>(P, 0, lw, P.zero_init != 0);
  if (warp_bottom) {
    if (threadIdx.x < 32) {
      blk_cycle_range<T, DIM, true>(P, lw, last, lw > 0 || P.zero_init != 0);
      blk_relax<T, DIM, true>(P.A[last], P.e[last], P.r[last], P.bottom, true);
      blk_cycle_up<T, DIM, true>(P, lw, last);
    }
    __syncthreads();
  } else {
    blk_relax<T, DIM, false>(P.A[last], P.e[last], P.r[last], P.bottom, true);
  }
  // block part, up
  blk_cycle_up<T, DIM, false>(P, 0, lw);
  // the top level's correction is what the caller prolongs from
  for (long long q = threadIdx.x; q < Pg.A[0].G.ncell; q += blockDim.x) top_e[q] = P.e[0][q];
}

}  // namespace mlgpu
