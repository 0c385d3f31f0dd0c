// cycle_kernels.cuh -- the coarse end of a multigrid V-cycle in ONE thread
// block.  Below a few thousand cells a level's work is far smaller than a
// kernel launch, so every level from `A[0]` down to the bottom runs inside a
// single CTA: relax, restrict, bottom relaxation, prolong, relax, separated
// by __syncthreads().  Each cell update calls the same device functions as
// the per-level kernels, so the results are bit-identical to launching the
// per-level kernels one after another.
#pragma once
#include "vc_kernels.cuh"
#include "misc_kernels.cuh"

namespace mlgpu {

constexpr int kMaxBlockLevels = 12;

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

template <class T, int DIM>
__device__ __forceinline__ void blk_half_sweep(const VCArgs<T> &A, T *e, const T *r, int pass) {
  long long nt = colour_threads(A.G);
  for (long long t = threadIdx.x; t < nt; t += blockDim.x) {
    int i, j, k;
    if (colour_cell(A.G, pass, t, i, j, k)) vc_gsrb_cell<T, DIM>(A, e, r, i, j, k);
  }
  __syncthreads();
}

// VCSolver::relax for GSRB, inside the block
template <class T, int DIM>
__device__ void blk_relax(const VCArgs<T> &A, T *e, const T *r, int n, bool zero_init) {
  if (zero_init) {
    if (n == 0) {
      for (long long q = threadIdx.x; q < A.G.ncell; q += blockDim.x) e[q] = T(0);
      __syncthreads();
      return;
    }
    for (long long q = threadIdx.x; q < A.G.ncell; q += blockDim.x) {
      int i, j, k;
      cell_ijk(A.G, q, i, j, k);
      vc_gsrb_zero_cell<T, DIM>(A, e, r, q, i, j, k);
    }
    __syncthreads();
    blk_half_sweep<T, DIM>(A, e, r, 1);
    n--;
  }
  for (int s = 0; s < n; s++) {
    blk_half_sweep<T, DIM>(A, e, r, 0);
    blk_half_sweep<T, DIM>(A, e, r, 1);
  }
}

template <class T, int DIM>
__global__ void __launch_bounds__(1024) vc_block_cycle_kernel(VCBlockCycle<T> P) {
  const int last = P.nlev - 1;
  const T denom = DIM == 3 ? T(8) : T(4);
  // down: pre-smooth, restrict the residual
  for (int l = 0; l < last; l++) {
    const VCArgs<T> &A = P.A[l];
    blk_relax<T, DIM>(A, P.e[l], P.r[l], P.pre, l > 0 || P.zero_init);
    const Geom &C = P.A[l + 1].G;
    PlainRead<T> rd{P.e[l]};
    for (long long Q = threadIdx.x; Q < C.ncell; Q += blockDim.x) {
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
    __syncthreads();
  }
  // bottom: zero, then relaxation sweeps (RelaxSolver role)
  blk_relax<T, DIM>(P.A[last], P.e[last], P.r[last], P.bottom, true);
  // up: prolong the correction, post-smooth
  for (int l = last - 1; l >= 0; l--) {
    const Geom &F = P.A[l].G, &C = P.A[l + 1].G;
    for (long long t = threadIdx.x; t < F.ncell; t += blockDim.x) {
      if (P.prolong == MLGPU_PROLONG_LINEAR)
        prolong_one<T, DIM, MLGPU_PROLONG_LINEAR>(F, C, P.bc, t, P.e[l], P.e[l + 1], nullptr);
      else
        prolong_one<T, DIM, MLGPU_PROLONG_CONSTANT>(F, C, P.bc, t, P.e[l], P.e[l + 1], nullptr);
    }
    __syncthreads();
    blk_relax<T, DIM>(P.A[l], P.e[l], P.r[l], P.post, false);
  }
}

}  // namespace mlgpu
