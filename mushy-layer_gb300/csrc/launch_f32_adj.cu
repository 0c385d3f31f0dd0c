// launch_f32_adj.cu -- launchers of the lean cycles: the FP32 Jacobian
// kernels (adjoint_kernels.cuh) and the lean colour-split kernels
// (lin_lean_kernels.cuh, FP32 and FP64) of the Newton step's linear cycles,
// and the lean FP32 3D cycles of the linear operator (vc_lean_kernels.cuh).
// FMA contraction is left on, as in launch_f32.cu.
#define MLGPU_ADJ_UNIT 1
#define MLGPU_ADJ_F32_UNIT 1
#include "launch_impl.cuh"
#include "adjoint_kernels.cuh"
#include "lin_lean_kernels.cuh"
#include "vc_lean_kernels.cuh"

namespace mlgpu {

#define MLGPU_TR_SWITCH32(tr, ...) \
  do {                             \
    if (tr) {                      \
      constexpr bool TR = true;    \
      __VA_ARGS__;                 \
    } else {                       \
      constexpr bool TR = false;   \
      __VA_ARGS__;                 \
    }                              \
  } while (0)

cudaError_t launch_adj_jac(const Geom &G, const ClosureParams &cp, const double *u, float *J,
                           cudaStream_t s) {
  adj_jac_kernel<float><<<blocks_for(G.ncell), kBlock, 0, s>>>(G, cp, u, J);
  return cudaGetLastError();
}

cudaError_t launch_adj_op(const AdjArgs<float> &A, int mode, int norm, const float *y,
                          const float *g, float *out, double *part, int *nparts, cudaStream_t s,
                          bool tr) {
  const int nb = blocks_for(A.G.ncell);
  if (nparts) *nparts = (part && mode == ADJ_RESIDUAL && norm >= 0) ? nb : 0;
  if (mode == ADJ_RESIDUAL && norm >= 0) {
    if (!part) return cudaErrorInvalidValue;
    MLGPU_TR_SWITCH32(tr, MLGPU_DIM_SWITCH(A.G.dim, MLGPU_NORM_SWITCH(norm, (adj_op_kernel<float, DIM, ADJ_RESIDUAL, NORM, TR><<<nb, kBlock, 0, s>>>(A, y, g, out, part)))));
  } else if (mode == ADJ_RESIDUAL) {
    MLGPU_TR_SWITCH32(tr, MLGPU_DIM_SWITCH(A.G.dim, (adj_op_kernel<float, DIM, ADJ_RESIDUAL, -1, TR><<<nb, kBlock, 0, s>>>(A, y, g, out, part))));
  } else {
    MLGPU_TR_SWITCH32(tr, MLGPU_DIM_SWITCH(A.G.dim, (adj_op_kernel<float, DIM, ADJ_APPLY, -1, TR><<<nb, kBlock, 0, s>>>(A, y, g, out, part))));
  }
  return cudaGetLastError();
}

cudaError_t launch_adj_gsrb(const AdjArgs<float> &A, float *y, const float *g, int pass,
                            cudaStream_t s, bool tr) {
  MLGPU_TR_SWITCH32(tr, MLGPU_DIM_SWITCH(A.G.dim, (adj_gsrb_kernel<float, DIM, TR><<<blocks_for(colour_threads(A.G)), kBlock, 0, s>>>(A, y, g, pass))));
  return cudaGetLastError();
}

cudaError_t launch_adj_relax_block(const AdjArgs<float> &A, float *y, const float *g, int sweeps,
                                   int zero, cudaStream_t s, bool tr) {
  MLGPU_TR_SWITCH32(tr, MLGPU_DIM_SWITCH(A.G.dim, (adj_relax_block_kernel<float, DIM, TR><<<1, 1024, 0, s>>>(A, y, g, sweeps, zero))));
  return cudaGetLastError();
}

cudaError_t launch_adj_minv(const AdjArgs<float> &A, const float *zero, float *Minv, float *D,
                            cudaStream_t s) {
  MLGPU_DIM_SWITCH(A.G.dim, (adj_minv_kernel<float, DIM><<<blocks_for(A.G.ncell), kBlock, 0, s>>>(A, zero, Minv, D)));
  return cudaGetLastError();
}

cudaError_t launch_adj_bottom_direct(const AdjArgs<float> &A, float *y, const float *g,
                                     cudaStream_t s, bool tr) {
  if (2 * A.G.ncell > kAdjDirectMax) return cudaErrorInvalidValue;
  MLGPU_TR_SWITCH32(tr, MLGPU_DIM_SWITCH(A.G.dim, (adj_bottom_direct_kernel<float, DIM, TR><<<1, kAdjDirectMax, 0, s>>>(A, y, g))));
  return cudaGetLastError();
}

cudaError_t launch_adj_restrict(const AdjArgs<float> &A, const Geom &C, const float *y,
                                const float *g, float *gc, cudaStream_t s, bool tr) {
  MLGPU_TR_SWITCH32(tr, MLGPU_DIM_SWITCH(A.G.dim, (adj_restrict_kernel<float, DIM, TR><<<blocks_for(C.ncell), kBlock, 0, s>>>(A, C, y, g, gc))));
  return cudaGetLastError();
}

// ---- lean cycles of the Newton step (lin_lean_kernels.cuh), FP32 for the
// mixed-precision solve and FP64 for the comparison path built the same way
template <class T>
cudaError_t launch_lean_gsrb(const LinLeanT<T> &P, int pass, cudaStream_t s, int vec) {
  constexpr int V = Vec16<T>::V;
  if (vec && ((P.G.n0 >> 1) % V) == 0) {
    const long long groups = (P.G.ncell >> 1) / V;
    MLGPU_DIM_SWITCH(P.G.dim, (lean_gsrb_vec_kernel<T, DIM><<<blocks_for(groups), kBlock, 0, s>>>(P, pass)));
  } else {
    MLGPU_DIM_SWITCH(P.G.dim, (lean_gsrb_kernel<T, DIM><<<blocks_for(P.G.ncell >> 1), kBlock, 0, s>>>(P, pass)));
  }
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_lean_residual(const LinLeanT<T> &P, int split, int red, int norm,
                                 double *part, int *nparts, cudaStream_t s, int vec) {
  red = split && red;
  if (norm < 0) norm = MLGPU_NORM_MAX;
  constexpr int V = Vec16<T>::V;
  if (vec && red && ((P.G.n0 >> 1) % V) == 0) {
    const int nb = blocks_for((P.G.ncell >> 1) / V);
    if (nparts) *nparts = nb;
    MLGPU_DIM_SWITCH(P.G.dim, MLGPU_NORM_SWITCH(norm, {
      if (NORM >= 0)
        lean_residual_vec_kernel<T, DIM, (NORM < 0 ? 0 : NORM)><<<nb, kBlock, 0, s>>>(P, part);
    }));
    return cudaGetLastError();
  }
  const int nb = blocks_for(red ? P.G.ncell >> 1 : P.G.ncell);
  if (nparts) *nparts = nb;
#define MLGPU_LEAN_RES(IDX, RED)                                                          \
  MLGPU_DIM_SWITCH(P.G.dim, MLGPU_NORM_SWITCH(norm, {                                     \
    if (NORM >= 0)                                                                        \
      lean_residual_kernel<T, DIM, (NORM < 0 ? 0 : NORM), IDX, RED>                       \
          <<<nb, kBlock, 0, s>>>(P, part);                                                \
  }))
  if (red)
    MLGPU_LEAN_RES(SplitIdx, true);
  else if (split)
    MLGPU_LEAN_RES(SplitIdx, false);
  else
    MLGPU_LEAN_RES(NaturalIdx, false);
#undef MLGPU_LEAN_RES
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_lean_restrict(const LinLeanT<T> &P, const Geom &C, int csplit, int red, T *gc,
                                 T *xc, T *wc, cudaStream_t s, int vec) {
  constexpr int V = Vec16<T>::V;
  if (vec && red && ((P.G.n0 >> 1) % V) == 0 && C.n0 == (P.G.n0 >> 1)) {
    const int nbv = blocks_for(C.ncell / V);
    if (csplit)
      MLGPU_DIM_SWITCH(P.G.dim, (lean_restrict_vec_kernel<T, DIM, SplitIdx><<<nbv, kBlock, 0, s>>>(P, C, gc, xc, wc)));
    else
      MLGPU_DIM_SWITCH(P.G.dim, (lean_restrict_vec_kernel<T, DIM, NaturalIdx><<<nbv, kBlock, 0, s>>>(P, C, gc, xc, wc)));
    return cudaGetLastError();
  }
  const int nb = blocks_for(C.ncell);
#define MLGPU_LEAN_RST(IDX, RED) \
  MLGPU_DIM_SWITCH(P.G.dim, (lean_restrict_kernel<T, DIM, IDX, RED><<<nb, kBlock, 0, s>>>(P, C, gc, xc, wc)))
  if (csplit) {
    if (red)
      MLGPU_LEAN_RST(SplitIdx, true);
    else
      MLGPU_LEAN_RST(SplitIdx, false);
  } else {
    if (red)
      MLGPU_LEAN_RST(NaturalIdx, true);
    else
      MLGPU_LEAN_RST(NaturalIdx, false);
  }
#undef MLGPU_LEAN_RST
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_lean_prolong(const LinLeanT<T> &P, const Geom &C, int csplit, int black,
                                int kind, const T *xc, cudaStream_t s) {
  if (black && kind == MLGPU_PROLONG_LINEAR) {  // coarse tiles, one thread per coarse cell
    long long ntiles;
    if (P.G.dim == 3)
      ntiles = (long long)((C.n0 + ProlongTile<3>::TX - 1) / ProlongTile<3>::TX) *
               ((C.n1 + ProlongTile<3>::TY - 1) / ProlongTile<3>::TY) *
               ((C.n2 + ProlongTile<3>::TZ - 1) / ProlongTile<3>::TZ);
    else
      ntiles = (long long)((C.n0 + ProlongTile<2>::TX - 1) / ProlongTile<2>::TX) *
               ((C.n1 + ProlongTile<2>::TY - 1) / ProlongTile<2>::TY);
    const int nbc = (int)std::min<long long>(ntiles, 1LL << 20);
    if (csplit) {
      MLGPU_DIM_SWITCH(P.G.dim, (lean_prolong_lin_black_kernel<T, DIM, SplitIdx><<<nbc, kBlock, 0, s>>>(P, C, xc)));
    } else {
      MLGPU_DIM_SWITCH(P.G.dim, (lean_prolong_lin_black_kernel<T, DIM, NaturalIdx><<<nbc, kBlock, 0, s>>>(P, C, xc)));
    }
    return cudaGetLastError();
  }
  const int nb = blocks_for(black ? P.G.ncell >> 1 : P.G.ncell);
#define MLGPU_LEAN_PRO(KIND, IDX, BL) \
  MLGPU_DIM_SWITCH(P.G.dim, (lean_prolong_kernel<T, DIM, KIND, IDX, BL><<<nb, kBlock, 0, s>>>(P, C, xc)))
#define MLGPU_LEAN_PRO2(KIND, IDX)      \
  if (black)                            \
    MLGPU_LEAN_PRO(KIND, IDX, true);    \
  else                                  \
    MLGPU_LEAN_PRO(KIND, IDX, false);
  if (kind == MLGPU_PROLONG_LINEAR) {
    if (csplit) {
      MLGPU_LEAN_PRO2(MLGPU_PROLONG_LINEAR, SplitIdx)
    } else {
      MLGPU_LEAN_PRO2(MLGPU_PROLONG_LINEAR, NaturalIdx)
    }
  } else {
    if (csplit) {
      MLGPU_LEAN_PRO2(MLGPU_PROLONG_CONSTANT, SplitIdx)
    } else {
      MLGPU_LEAN_PRO2(MLGPU_PROLONG_CONSTANT, NaturalIdx)
    }
  }
#undef MLGPU_LEAN_PRO2
#undef MLGPU_LEAN_PRO
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_lean_psum(const AdjArgs<T> &A, T *P, cudaStream_t s) {
  MLGPU_DIM_SWITCH(A.G.dim, (lean_psum_kernel<T, DIM><<<blocks_for(A.G.ncell), kBlock, 0, s>>>(A, P)));
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_lean_state(const AdjArgs<T> &A, const double *u, const T *P, T *Js, T *Ks,
                              T *Ds, cudaStream_t s) {
  const ClosureF32 f = make_closure_f32(A.cp);
  const ClosureLean L = make_closure_lean(A.cp);
  MLGPU_DIM_SWITCH(A.G.dim, (lean_state_kernel<T, DIM><<<blocks_for(A.G.ncell), kBlock, 0, s>>>(A, f, L, u, P, Js, Ks, Ds)));
  return cudaGetLastError();
}

template <class T, class S>
cudaError_t launch_lean_pack(const Geom &G, int split, int ncomp, const S *src, T *dst,
                             cudaStream_t s) {
  if (split)
    lean_pack_kernel<T, S, SplitIdx><<<blocks_for(G.ncell), kBlock, 0, s>>>(G, ncomp, src, dst);
  else
    lean_pack_kernel<T, S, NaturalIdx><<<blocks_for(G.ncell), kBlock, 0, s>>>(G, ncomp, src, dst);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_lean_step(const Geom &G, int split, const StepClip *clip, double *u,
                             const double *u_old, double scale, const T *e, cudaStream_t s) {
  const int nb = blocks_for(G.ncell);
  StepClip K{};
  if (clip) K = *clip;
#define MLGPU_LEAN_STEP(IDX)                                                           \
  if (clip)                                                                            \
    lean_step_kernel<T, IDX, true><<<nb, kBlock, 0, s>>>(G, K, u, u_old, scale, e);    \
  else                                                                                 \
    lean_step_kernel<T, IDX, false><<<nb, kBlock, 0, s>>>(G, K, u, u_old, scale, e);
  if (split) {
    MLGPU_LEAN_STEP(SplitIdx)
  } else {
    MLGPU_LEAN_STEP(NaturalIdx)
  }
#undef MLGPU_LEAN_STEP
  return cudaGetLastError();
}

// ---- lean cycles of the linear operator on 3D levels (vc_lean_kernels.cuh),
// FP32 for the mixed solve and FP64 for the comparison path
template <class T>
cudaError_t launch_vcl_diag(const VCArgs<T> &A, T *idg, T *dg, cudaStream_t s) {
  MLGPU_DIM_SWITCH(A.G.dim, (vcl_diag_kernel<T, DIM><<<blocks_for(A.G.ncell), kBlock, 0, s>>>(A, idg, dg)));
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_vcl_gsrb(const VCLeanT<T> &P, int pass, int zero, cudaStream_t s, int vec) {
  constexpr int V = Vec16<T>::V;
  if (vec && ((P.G.n0 >> 1) % V) == 0) {
    MLGPU_DIM_SWITCH(P.G.dim, (vcl_gsrb_vec_kernel<T, DIM><<<blocks_for((P.G.ncell >> 1) / V), kBlock, 0, s>>>(P, pass, zero)));
  } else {
    MLGPU_DIM_SWITCH(P.G.dim, (vcl_gsrb_kernel<T, DIM><<<blocks_for(P.G.ncell >> 1), kBlock, 0, s>>>(P, pass, zero)));
  }
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_vcl_restrict(const VCLeanT<T> &P, const Geom &C, int csplit, int red, T *rc,
                                T *ec, cudaStream_t s) {
  constexpr int V = Vec16<T>::V;
  if (red && ((P.G.n0 >> 1) % V) == 0 && C.n0 == (P.G.n0 >> 1)) {  // vector groups
    const int nbv = blocks_for(C.ncell / V);
    if (csplit)
      MLGPU_DIM_SWITCH(P.G.dim, (vcl_restrict_vec_kernel<T, DIM, SplitIdx><<<nbv, kBlock, 0, s>>>(P, C, rc, ec)));
    else
      MLGPU_DIM_SWITCH(P.G.dim, (vcl_restrict_vec_kernel<T, DIM, NaturalIdx><<<nbv, kBlock, 0, s>>>(P, C, rc, ec)));
    return cudaGetLastError();
  }
  const int nb = blocks_for(C.ncell);
#define MLGPU_VCL_RST(IDX, RED) \
  MLGPU_DIM_SWITCH(P.G.dim, (vcl_restrict_kernel<T, DIM, IDX, RED><<<nb, kBlock, 0, s>>>(P, C, rc, ec)))
  if (csplit) {
    if (red)
      MLGPU_VCL_RST(SplitIdx, true);
    else
      MLGPU_VCL_RST(SplitIdx, false);
  } else {
    if (red)
      MLGPU_VCL_RST(NaturalIdx, true);
    else
      MLGPU_VCL_RST(NaturalIdx, false);
  }
#undef MLGPU_VCL_RST
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_vcl_prolong(const VCLeanT<T> &P, const Geom &C, const BCD &bc, int csplit,
                               int black, int kind, const T *ec, cudaStream_t s) {
  const int nb = blocks_for(black ? P.G.ncell >> 1 : P.G.ncell);
#define MLGPU_VCL_PRO(KIND, IDX, BL) \
  MLGPU_DIM_SWITCH(P.G.dim, (vcl_prolong_kernel<T, DIM, KIND, IDX, BL><<<nb, kBlock, 0, s>>>(P, C, bc, ec)))
#define MLGPU_VCL_PRO2(KIND, IDX)    \
  if (black)                         \
    MLGPU_VCL_PRO(KIND, IDX, true);  \
  else                               \
    MLGPU_VCL_PRO(KIND, IDX, false);
  if (kind == MLGPU_PROLONG_LINEAR) {
    if (csplit) {
      MLGPU_VCL_PRO2(MLGPU_PROLONG_LINEAR, SplitIdx)
    } else {
      MLGPU_VCL_PRO2(MLGPU_PROLONG_LINEAR, NaturalIdx)
    }
  } else {
    if (csplit) {
      MLGPU_VCL_PRO2(MLGPU_PROLONG_CONSTANT, SplitIdx)
    } else {
      MLGPU_VCL_PRO2(MLGPU_PROLONG_CONSTANT, NaturalIdx)
    }
  }
#undef MLGPU_VCL_PRO2
#undef MLGPU_VCL_PRO
  return cudaGetLastError();
}

template <class E>
cudaError_t launch_vcl_outer(const VCArgs<double> &A, int norm, const double *phi, const E *e,
                             const double *rhs, double *out_phi, E *res_inner, double *part,
                             int *nparts, cudaStream_t s, const int *par) {
  const int nb = blocks_for(A.G.ncell);
  if (nparts) *nparts = nb;
  if (norm < 0) norm = MLGPU_NORM_MAX;
  MLGPU_DIM_SWITCH(A.G.dim, MLGPU_NORM_SWITCH(norm, {
    if (NORM >= 0)
      vcl_outer_kernel<E, DIM, (NORM < 0 ? 0 : NORM)>
          <<<nb, kBlock, 0, s>>>(A, phi, e, rhs, out_phi, res_inner, part, par);
  }));
  return cudaGetLastError();
}

#define MLGPU_VCL_INST(T)                                                                       \
  template cudaError_t launch_vcl_diag<T>(const VCArgs<T> &, T *, T *, cudaStream_t);           \
  template cudaError_t launch_vcl_gsrb<T>(const VCLeanT<T> &, int, int, cudaStream_t, int);     \
  template cudaError_t launch_vcl_restrict<T>(const VCLeanT<T> &, const Geom &, int, int, T *,  \
                                             T *, cudaStream_t);                               \
  template cudaError_t launch_vcl_prolong<T>(const VCLeanT<T> &, const Geom &, const BCD &, int, \
                                            int, int, const T *, cudaStream_t);                \
  template cudaError_t launch_vcl_outer<T>(const VCArgs<double> &, int, const double *,         \
                                          const T *, const double *, double *, T *, double *,  \
                                          int *, cudaStream_t, const int *);
MLGPU_VCL_INST(float)
MLGPU_VCL_INST(double)
#undef MLGPU_VCL_INST

#define MLGPU_LEAN_INST(T)                                                                     \
  template cudaError_t launch_lean_gsrb<T>(const LinLeanT<T> &, int, cudaStream_t, int);      \
  template cudaError_t launch_lean_residual<T>(const LinLeanT<T> &, int, int, int, double *,   \
                                              int *, cudaStream_t, int);                      \
  template cudaError_t launch_lean_restrict<T>(const LinLeanT<T> &, const Geom &, int, int,    \
                                              T *, T *, T *, cudaStream_t, int);              \
  template cudaError_t launch_lean_prolong<T>(const LinLeanT<T> &, const Geom &, int, int,     \
                                             int, const T *, cudaStream_t);                   \
  template cudaError_t launch_lean_pack<T, double>(const Geom &, int, int, const double *, T *, \
                                                  cudaStream_t);                              \
  template cudaError_t launch_lean_step<T>(const Geom &, int, const StepClip *, double *,        \
                                          const double *, double, const T *, cudaStream_t);     \
  template cudaError_t launch_lean_state<T>(const AdjArgs<T> &, const double *, const T *, T *,  \
                                           T *, T *, cudaStream_t);                              \
  template cudaError_t launch_lean_psum<T>(const AdjArgs<T> &, T *, cudaStream_t);
MLGPU_LEAN_INST(float)
MLGPU_LEAN_INST(double)
template cudaError_t launch_lean_pack<float, float>(const Geom &, int, int, const float *,
                                                    float *, cudaStream_t);
#undef MLGPU_LEAN_INST

}  // namespace mlgpu
