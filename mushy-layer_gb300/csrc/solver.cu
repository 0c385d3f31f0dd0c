// solver.cu -- host-side multigrid drivers over the sm_103a kernels.
//
//  * VCSolver: correction-scheme multigrid for the projection and
//    Darcy-Brinkman operators, restating Chombo's AMRMultiGrid::solveNoInit
//    on one level + MultiGrid::cycle (relax, restrictResidual, coarse cycle,
//    prolongIncrement, relax) with the bottom solve done by relaxation.
//    MLGPU_PREC_MIXED runs the inner cycles in FP32 inside an FP64
//    defect-correction loop (FP64 residual, FP64 update, FP64 norm).
//  * HCSolver: FAS multigrid for AMRNonLinearMultiCompOp (the role of
//    Chombo's AMRFASMultiGrid): relax, restrictR + restrictResidual, coarse
//    rhs = N_c(R u) + R r, coarse cycle, prolong (u_c - R u), relax.
//
// All device memory comes from the caller's workspace.  One outer iteration
// (cycle + residual + norm + norm read-back) is captured once in a CUDA graph
// and replayed, so a solve costs one graph launch and one host wait per outer
// iteration.
#include <cstring>
#include <cmath>
#include <vector>
#include "capi_internal.h"

using namespace mlgpu;

// A solver runs on its own non-blocking stream (graph capture is not allowed
// on the legacy default stream a caller may pass); it is ordered after the
// caller's stream on entry and the caller's stream waits for it on exit.
struct mlgpu_solver {
  cudaStream_t user = nullptr, s = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  virtual ~mlgpu_solver() {
    if (ev_in) cudaEventDestroy(ev_in);
    if (ev_out) cudaEventDestroy(ev_out);
    if (s) cudaStreamDestroy(s);
  }
  int init_streams(cudaStream_t caller) {
    user = caller;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return MLGPU_ERR_CUDA;
    if (cudaEventCreateWithFlags(&ev_in, cudaEventDisableTiming) != cudaSuccess) return MLGPU_ERR_CUDA;
    if (cudaEventCreateWithFlags(&ev_out, cudaEventDisableTiming) != cudaSuccess) return MLGPU_ERR_CUDA;
    return MLGPU_OK;
  }
  int enter() {
    if (cudaEventRecord(ev_in, user) != cudaSuccess) return MLGPU_ERR_CUDA;
    if (cudaStreamWaitEvent(s, ev_in, 0) != cudaSuccess) return MLGPU_ERR_CUDA;
    return MLGPU_OK;
  }
  int leave() {
    if (cudaEventRecord(ev_out, s) != cudaSuccess) return MLGPU_ERR_CUDA;
    if (cudaStreamWaitEvent(user, ev_out, 0) != cudaSuccess) return MLGPU_ERR_CUDA;
    return MLGPU_OK;
  }
  virtual int solve(double *phi, const double *rhs, mlgpu_solve_stats *st) = 0;
  virtual int set_alpha_beta(double a, double b) = 0;

  // kernels a piece of host code launches: captured once into a graph that
  // is never run, and its kernel nodes counted (-1 if the capture failed)
  template <class F>
  int count_kernels(F &&f) {
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return -1;
    int rc = f();
    cudaError_t e = cudaStreamEndCapture(s, &g);
    cudaGetLastError();
    if (rc || e != cudaSuccess || !g) {
      if (g) cudaGraphDestroy(g);
      return -1;
    }
    int n = kernel_nodes(g);
    cudaGraphDestroy(g);
    return n;
  }
  static int kernel_nodes(cudaGraph_t g) {
    size_t n = 0;
    if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess) return -1;
    std::vector<cudaGraphNode_t> nodes(n);
    if (n && cudaGraphGetNodes(g, nodes.data(), &n) != cudaSuccess) return -1;
    int k = 0;
    for (auto nd : nodes) {
      cudaGraphNodeType t;
      if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) k++;
    }
    return k;
  }
};

namespace {

struct Arena {
  char *base = nullptr;
  size_t off = 0;
  template <class T>
  T *get(size_t n) {
    off = (off + 255) & ~(size_t)255;
    T *p = base ? (T *)(base + off) : nullptr;
    off += n * sizeof(T);
    return p;
  }
};

int mg_depth(const mlgpu_grid &g, int max_coarse) {
  if (max_coarse < 1) max_coarse = 1;
  int depth = 0;
  while (true) {
    long long c = (1LL << (depth + 1)) * max_coarse;
    bool ok = true;
    for (int d = 0; d < g.dim; d++)
      if (g.n[d] % c != 0) ok = false;
    if (!ok || depth > 40) break;
    depth++;
  }
  return depth;
}

mlgpu_grid coarsen_grid(const mlgpu_grid &f) {
  mlgpu_grid c = f;
  for (int d = 0; d < f.dim; d++) c.n[d] = f.n[d] / 2;
  c.dx = f.dx * 2;
  return c;
}

size_t nfaces(const mlgpu_grid &g, int d) {
  size_t m = 1;
  for (int e = 0; e < 3; e++) m *= (size_t)(g.n[e] + (e == d ? 1 : 0));
  return m;
}
size_t ncells(const mlgpu_grid &g) { return (size_t)g.n[0] * g.n[1] * g.n[2]; }

#define CK(...)                                   \
  do {                                            \
    cudaError_t e_ = (__VA_ARGS__);               \
    if (e_ != cudaSuccess) return MLGPU_ERR_CUDA; \
  } while (0)

// Per-level coefficient storage in one precision.
template <class T>
struct Coefs {
  T *a = nullptr, *c = nullptr, *b[3] = {nullptr, nullptr, nullptr};
};

// outer convergence bookkeeping (AMRMultiGrid::solveNoInit semantics)
struct Outer {
  double norm0 = 0, norm = 0, prev = 0;
  int iter = 0, status = 0;
};

void stats_begin(mlgpu_solve_stats *st, int levels, double norm0) {
  memset(st, 0, sizeof(*st));
  st->levels = levels;
  st->initial_norm = norm0;
  st->norm_history[0] = norm0;
}

// returns true when iterating should continue
bool outer_continue(const mlgpu_mg_options &o, Outer &S) {
  return S.norm > o.tolerance * S.norm0 && S.norm0 > o.norm_thresh && S.iter < o.max_iter &&
         S.status == 0;
}

void outer_after(const mlgpu_mg_options &o, Outer &S, mlgpu_solve_stats *st) {
  S.iter++;
  if (S.iter < 64) st->norm_history[S.iter] = S.norm;
  if (!std::isfinite(S.norm)) {
    S.status = 8;
    return;
  }
  if (S.norm > (1.0 - o.hang) * S.prev && S.norm > o.tolerance * S.norm0) {
    S.status = 2;
    return;
  }
  S.prev = S.norm;
}

int outer_finish(const mlgpu_mg_options &o, Outer &S, mlgpu_solve_stats *st) {
  st->iterations = S.iter;
  st->final_norm = S.norm;
  if (S.status == 0 && S.norm > o.tolerance * S.norm0 && S.norm0 > o.norm_thresh) S.status = 4;
  st->exit_status = S.status;
  if (S.status == kStatusDeviceFault) return MLGPU_ERR_CUDA;
  if (S.status == 8) return MLGPU_ERR_NAN;
  if (S.status == 2) return MLGPU_ERR_HANG;
  if (S.status == 4) return MLGPU_ERR_NOT_CONVERGED;
  return MLGPU_OK;
}

// ====================================================================== VC
struct VCLevel {
  mlgpu_grid grid;
  Geom G;
  Coefs<double> c64;
  Coefs<float> c32;
  void *e = nullptr, *r = nullptr, *t = nullptr;  // inner precision
  void *ecur = nullptr;  // which of e / t holds the correction after the last pass
  double *lam64 = nullptr;  // stored 1/diag for FP64 inner cycles
  float *fcx = nullptr, *fcy = nullptr, *flam = nullptr, *fdiag = nullptr;  // lean FP32 tiles
  double *ocx = nullptr, *ocy = nullptr, *odiag = nullptr;  // FP64 outer step (level 0, mixed)
  // 3D levels above the single-CTA block cycle, in mixed precision or with
  // options.fuse_levels >= 2 in FP64: the lean cycles (vc_lean_kernels.cuh,
  // inner precision) with e, r colour-split and the diagonal folded
  bool lean = false;
  void *idg = nullptr, *dg = nullptr;
};

class VCSolver : public mlgpu_solver {
 public:
  // V-cycles per outer iteration: the option, or by default 3 in mixed
  // precision (amortises the FP64 outer step over more FP32 cycles; the
  // convergence test stays on the FP64 residual) and 1 in FP64 (the
  // reference's one cycle per AMRMultiGrid iteration)
  int inner_cycles() const { return o.inner_cycles > 0 ? o.inner_cycles : (mixed ? 3 : 1); }
  mlgpu_vcop op;
  mlgpu_mg_options o;
  std::vector<VCLevel> L;
  double *phi[2] = {nullptr, nullptr};
  double *rhs = nullptr, *part = nullptr;
  double *host_norm = nullptr;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  cudaGraphExec_t loop_exec = nullptr;
  bool loop_failed = false;
  OuterDev *dev_state = nullptr, *host_state = nullptr;
  bool mixed = false;
  bool use_block_cycle = true;
  bool use_tiles = true;
  double updates_per_iter = 0;
  int kern_init = -1, kern_iter = -1, kern_loop = -1;  // kernels per piece (counted)
  // level pack of the lean FP32 coarse cycle (mixed 2D): levels cyc_top..last
  float *cyc_pack = nullptr;
  int cyc_top = -1;
  // BiCGStab bottom solve: FP64 work arrays of the coarsest level
  double *bicg_ws = nullptr;
  std::vector<int> cyc_off;

  ~VCSolver() override {
    for (auto &g : graph)
      if (g) cudaGraphExecDestroy(g);
    if (loop_exec) cudaGraphExecDestroy(loop_exec);
    if (host_norm) cudaFreeHost(host_norm);
    if (host_state) cudaFreeHost(host_state);
  }

  void drop_graphs() {
    for (auto &g : graph)
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
    if (loop_exec) {
      cudaGraphExecDestroy(loop_exec);
      loop_exec = nullptr;
    }
  }

  // constants are in the operator's null space: no alpha a term, no c, and
  // no Dirichlet wall
  bool singular() const {
    if (op.alpha != 0.0 || op.cCoef) return false;
    for (int d = 0; d < op.grid.dim; d++)
      if (!op.grid.periodic[d])
        for (int s2 = 0; s2 < 2; s2++)
          if (op.bc.type[d][s2][0] == MLGPU_BC_DIRICHLET) return false;
    return true;
  }

  // lay out (or size, when base is null) the workspace
  size_t layout(char *base) {
    Arena A;
    A.base = base;
    int depth = mg_depth(op.grid, o.max_coarse);
    L.assign(depth + 1, VCLevel());
    mlgpu_grid g = op.grid;
    for (int l = 0; l <= depth; l++) {
      L[l].grid = g;
      L[l].G = make_geom(g);
      size_t n = ncells(g);
      if (l == 0) {
        L[l].c64.a = (double *)op.aCoef;
        L[l].c64.c = (double *)op.cCoef;
        for (int d = 0; d < 3; d++) L[l].c64.b[d] = (double *)op.bCoef[d];
      } else {
        if (op.aCoef) L[l].c64.a = A.get<double>(n);
        if (op.cCoef) L[l].c64.c = A.get<double>(n);
        for (int d = 0; d < g.dim; d++) L[l].c64.b[d] = A.get<double>(nfaces(g, d));
      }
      if (mixed) {
        if (op.aCoef) L[l].c32.a = A.get<float>(n);
        if (op.cCoef) L[l].c32.c = A.get<float>(n);
        for (int d = 0; d < g.dim; d++) L[l].c32.b[d] = A.get<float>(nfaces(g, d));
        L[l].e = A.get<float>(n);
        L[l].r = A.get<float>(n);
        L[l].t = A.get<float>(n);
        if (g.dim == 2 && l == 0) {
          L[l].ocx = A.get<double>(nfaces(g, 0));
          L[l].ocy = A.get<double>(nfaces(g, 1));
          L[l].odiag = A.get<double>(n);
        }
        if (g.dim == 2) {
          L[l].fcx = A.get<float>(nfaces(g, 0));
          L[l].fcy = A.get<float>(nfaces(g, 1));
          L[l].flam = A.get<float>(n);
          L[l].fdiag = A.get<float>(n);
        }
      } else {
        L[l].e = A.get<double>(n);
        L[l].r = A.get<double>(n);
        L[l].t = A.get<double>(n);
        // FP64 has 1/57 of the FP32 rate on GB300: store 1/diag instead of a
        // division per cell per half sweep (the reference stores it too)
        L[l].lam64 = A.get<double>(n);
      }
      g = coarsen_grid(g);
    }
    // the fused single-block coarse cycles end in relaxation: a BiCGStab
    // bottom takes the per-level path
    use_block_cycle = o.relax_mode == MLGPU_RELAX_GSRB && o.num_mg == 1 && o.fuse_levels &&
                      o.bottom_solver == MLGPU_BOTTOM_RELAX;
    if (o.bottom_solver == MLGPU_BOTTOM_BICGSTAB)
      bicg_ws = A.get<double>(kBiCGArrays * ncells(L[depth].grid));
    // the lean coarse cycle starts at the first level of at most kFastCycCells
    cyc_top = -1;
    cyc_off.clear();
    if (mixed && op.grid.dim == 2) {
      for (int l = 0; l < depth; l++)
        if (L[l].G.ncell <= kFastCycCells && depth - l + 1 <= kFastCycLevels) {
          cyc_top = l;
          break;
        }
      if (cyc_top >= 0) {
        int o2 = 0;
        for (int l = cyc_top; l <= depth; l++) {
          cyc_off.push_back(o2);
          o2 += cyc_pack_level_floats((int)L[l].G.ncell);
        }
        cyc_off.push_back(o2);
        cyc_pack = A.get<float>(o2);
      }
    }
    // FP32 tiles pay for their halo recomputation; FP64 tiles (4 extra half
    // sweeps of redundant FP64 work per tile) only when asked for explicitly
    use_tiles = use_block_cycle && (mixed || o.fuse_levels >= 2);
    // 3D, mixed or FP64 with fuse_levels >= 2: every level above the block
    // cycle (and above the bottom) runs the lean split cycles; such a level
    // has even extents
    if ((mixed || o.fuse_levels >= 2) && op.grid.dim == 3 && o.relax_mode == MLGPU_RELAX_GSRB)
      for (int l = 0; l < depth; l++) {
        if (use_block_cycle && L[l].G.ncell <= kBlockCycleCells && depth - l + 1 <= kMaxBlockLevels)
          break;
        L[l].lean = true;
        const size_t nb = (mixed ? sizeof(float) : sizeof(double)) * ncells(L[l].grid);
        L[l].idg = A.get<char>(nb);
        L[l].dg = A.get<char>(nb);
      }
    size_t n0 = ncells(op.grid);
    phi[0] = A.get<double>(n0);
    phi[1] = A.get<double>(n0);
    rhs = A.get<double>(n0);
    part = A.get<double>(kNormScratchDoubles);
    dev_state = A.get<OuterDev>(1);
    return A.off + 256;
  }

  int build_coefs() {
    for (size_t l = 1; l < L.size(); l++) {
      Geom F = L[l - 1].G;
      if (op.aCoef) CK(launch_restrict_avg<double>(F, 1, L[l - 1].c64.a, L[l].c64.a, s));
      if (op.cCoef) CK(launch_restrict_avg<double>(F, 1, L[l - 1].c64.c, L[l].c64.c, s));
      for (int d = 0; d < F.dim; d++)
        CK(launch_coarsen_faces<double>(F, 1, d, L[l - 1].c64.b[d], L[l].c64.b[d], s));
    }
    if (mixed) {
      for (auto &lv : L) {
        long long n = lv.G.ncell;
        if (op.aCoef) CK(launch_convert<float, double>(n, lv.c32.a, lv.c64.a, s));
        if (op.cCoef) CK(launch_convert<float, double>(n, lv.c32.c, lv.c64.c, s));
        for (int d = 0; d < lv.G.dim; d++)
          CK(launch_convert<float, double>(lv.G.nface(d), lv.c32.b[d], lv.c64.b[d], s));
      }
      int rc = build_fast();
      if (rc) return rc;
    } else {
      int rc = build_lambda();
      if (rc) return rc;
    }
    // cell updates per outer iteration (same accounting as the CPU oracle)
    double u = 0;
    int last = (int)L.size() - 1;
    std::vector<double> visits(L.size(), 0);
    visits[0] = inner_cycles();
    for (int l = 1; l <= last; l++) visits[l] = visits[l - 1] * o.num_mg;
    for (int l = 0; l <= last; l++) {
      double n = (double)L[l].G.ncell;
      if (l == last)
        u += visits[l] * o.bottom_max_iter * n;
      else
        u += visits[l] * ((o.num_smooth_down + o.num_smooth_up) * n + n);
    }
    updates_per_iter = u + (double)L[0].G.ncell;  // + outer residual
    return MLGPU_OK;
  }

  // FP32 coefficients of the lean tile smoother and FP64 ones of the outer
  // step (2D mixed precision)
  int build_fast() {
    if (L[0].ocx) CK(launch_outer_coefs(outer_args(), L[0].ocx, L[0].ocy, L[0].odiag, s));
    for (size_t l = 0; l < L.size(); l++)
      if (L[l].lean)
        CK(launch_vcl_diag<float>(args<float>((int)l), (float *)L[l].idg, (float *)L[l].dg, s));
    for (size_t l = 0; l < L.size(); l++) {
      if (!L[l].fcx) continue;
      VCArgs<double> A = args<double>((int)l);
      A.lam = nullptr;
      CK(launch_fast_coefs(A, L[l].fcx, L[l].fcy, L[l].flam, L[l].fdiag, s));
    }
    if (cyc_top >= 0)
      for (int l = cyc_top; l < (int)L.size(); l++)
        CK(launch_cyc_pack(L[l].G, make_bcd(op.bc),
                           FastCoefs{L[l].fcx, L[l].fcy, L[l].flam, L[l].fdiag},
                           cyc_pack + cyc_off[l - cyc_top], s));
    return MLGPU_OK;
  }

  int build_lambda() {
    for (size_t l = 0; l < L.size(); l++) {
      VCArgs<double> A = args<double>((int)l);
      A.lam = nullptr;
      CK(launch_vc_lambda<double>(A, L[l].lam64, s));
      if (L[l].lean) CK(launch_vcl_diag<double>(A, (double *)L[l].idg, (double *)L[l].dg, s));
    }
    return MLGPU_OK;
  }

  // level-0 FP64 operator on the caller's coefficient arrays
  VCArgs<double> outer_args() {
    VCArgs<double> A = args<double>(0);
    A.a = (const double *)op.aCoef;
    A.c = (const double *)op.cCoef;
    for (int d = 0; d < 3; d++) A.b[d] = (const double *)op.bCoef[d];
    A.lam = nullptr;
    return A;
  }

  // mixed 2D: phi_out = phi_in + e, FP64 residual, FP32 copy, norm (and, with
  // `st`, the outer-loop decision) in one launch; the norm lands in
  // part[kMaxBlocks]
  int outer_fast(const double *phi_in, const float *e, double *phi_out, const int *par,
                 OuterDev *st, cudaGraphConditionalHandle h) {
    OuterFast P;
    P.G = L[0].G;
    P.bc = make_bcd(op.bc);
    P.K = OuterCoefs{L[0].ocx, L[0].ocy, L[0].odiag};
    P.phi = phi_in;
    P.e = e;
    P.rhs = rhs;
    P.out_phi = phi_out;
    P.res_inner = (float *)L[0].r;
    P.part = part;
    P.count = (unsigned *)(part + kMaxBlocks + 1);
    P.par = par;
    P.st = st;
    P.cfg = OuterCfg{o.tolerance, o.hang, o.norm_thresh, o.max_iter};
    P.h = h;
    CK(launch_vc_outer_fast(P, o.norm_type, s));
    return MLGPU_OK;
  }

  template <class T>
  VCArgs<T> args(int l) {
    mlgpu_vcop lop = op;
    lop.grid = L[l].grid;
    VCArgs<T> A = make_vc_args<T>(lop);
    if (sizeof(T) == 8) {
      A.a = (const T *)L[l].c64.a;
      A.c = (const T *)L[l].c64.c;
      for (int d = 0; d < 3; d++) A.b[d] = (const T *)L[l].c64.b[d];
      A.lam = (const T *)L[l].lam64;
    } else {
      A.a = (const T *)L[l].c32.a;
      A.c = (const T *)L[l].c32.c;
      for (int d = 0; d < 3; d++) A.b[d] = (const T *)L[l].c32.b[d];
    }
    return A;
  }

  template <class T>
  int relax(int l, int n, bool zero_init) {
    VCArgs<T> A = args<T>(l);
    T *e = (T *)L[l].e;
    const T *r = (const T *)L[l].r;
    if (o.relax_mode == MLGPU_RELAX_JACOBI) {
      if (zero_init) CK(cudaMemsetAsync(e, 0, sizeof(T) * L[l].G.ncell, s));
      for (int i = 0; i < n; i++) {
        CK(launch_vc_op<T>(A, VC_JACOBI, -1, e, r, (T *)L[l].t, 1, nullptr, nullptr, s));
        CK(cudaMemcpyAsync(e, L[l].t, sizeof(T) * L[l].G.ncell, cudaMemcpyDeviceToDevice, s));
      }
      return MLGPU_OK;
    }
    if (zero_init) {
      if (n == 0) {
        CK(cudaMemsetAsync(e, 0, sizeof(T) * L[l].G.ncell, s));
        return MLGPU_OK;
      }
      CK(launch_vc_gsrb_zero<T>(A, e, r, s));
      CK(launch_vc_gsrb<T>(A, e, r, 1, s));
      n--;
    }
    for (int i = 0; i < n; i++) {
      CK(launch_vc_gsrb<T>(A, e, r, 0, s));
      CK(launch_vc_gsrb<T>(A, e, r, 1, s));
    }
    return MLGPU_OK;
  }

  // nh red/black half sweeps on level l in shared-memory tiles (2D), with an
  // optional zero start, prolongation before and residual restriction after;
  // split into several launches when the halo would not fit in shared memory
  template <class T>
  int tile_sweeps(int l, int nh, bool zero, bool with_restrict, bool with_prolong) {
    const int hmax = (sizeof(T) == 4 && L[l].fcx) ? kTFMaxHalo : tile_max_halo(sizeof(T));
    int done = 0;
    bool first = true;
    do {
      int chunk = std::min(nh - done, hmax - 1);
      bool is_last = done + chunk == nh;
      TileSmooth<T> P;
      P.A = args<T>(l);
      // ping-pong: read the current buffer, write the other one
      if (first && zero) {
        P.e_in = nullptr;
        P.e_out = (T *)L[l].e;
      } else {
        P.e_in = (const T *)L[l].ecur;
        P.e_out = (T *)(L[l].ecur == L[l].e ? L[l].t : L[l].e);
      }
      L[l].ecur = P.e_out;
      P.r = (const T *)L[l].r;
      P.zero_init = (first && zero) ? 1 : 0;
      P.n_half = chunk;
      P.pass0 = done & 1;
      P.rc = (is_last && with_restrict) ? (T *)L[l + 1].r : nullptr;
      P.halo = chunk + (P.rc ? 1 : 0);
      P.prolong = (first && with_prolong) ? o.prolong : -1;
      P.ec = with_prolong ? (const T *)L[l + 1].ecur : nullptr;
      if constexpr (sizeof(T) == 4) {
        if (L[l].fcx) {
          // lean FP32 form with precomputed face weights and 1/diag
          TileFast F;
          F.G = P.A.G;
          F.bc = P.A.bc;
          F.K = FastCoefs{L[l].fcx, L[l].fcy, L[l].flam, L[l].fdiag};
          F.e_in = P.e_in;
          F.e_out = P.e_out;
          F.r = P.r;
          F.zero_init = P.zero_init;
          F.n_half = P.n_half;
          F.pass0 = P.pass0;
          F.halo = P.halo;
          F.rc = P.rc;
          F.prolong = P.prolong;
          F.ec = P.ec;
          CK(launch_vc_tile_fast(F, s));
          first = false;
          done += chunk;
          continue;
        }
      }
      CK(launch_vc_tile_smooth<T>(P, s));
      first = false;
      done += chunk;
    } while (done < nh);
    return MLGPU_OK;
  }

  // lean operator of a lean 3D level, in the inner precision T
  template <class T>
  VCLeanT<T> vclean(int l) {
    const VCArgs<T> A = args<T>(l);
    VCLeanT<T> P;
    P.G = A.G;
    P.bd = A.beta * A.dxinv;
    for (int d = 0; d < 3; d++) P.b[d] = A.b[d];
    P.idg = (const T *)L[l].idg;
    P.dg = (const T *)L[l].dg;
    P.e = (T *)L[l].e;
    P.r = (const T *)L[l].r;
    return P;
  }

  // n red/black sweeps of a lean level; a zero start skips the first half
  // sweep's neighbour reads
  template <class T>
  int relax_lean(int l, int n, bool zero_init) {
    const VCLeanT<T> P = vclean<T>(l);
    if (n == 0) {
      if (zero_init) CK(cudaMemsetAsync(P.e, 0, sizeof(T) * L[l].G.ncell, s));
      return MLGPU_OK;
    }
    for (int i = 0; i < n; i++) {
      CK(launch_vcl_gsrb<T>(P, 0, (zero_init && i == 0) ? 1 : 0, s));
      CK(launch_vcl_gsrb<T>(P, 1, 0, s));
    }
    return MLGPU_OK;
  }

  // V-cycle from a lean level: pre-smoothing, red-children restriction (the
  // black residual vanishes after the black half sweep), the coarser levels,
  // black-only prolongation (the red half sweep that follows overwrites the
  // red e unread), post-smoothing
  template <class T>
  int cycle_lean(int l, bool zero_init) {
    const VCLeanT<T> P = vclean<T>(l);
    const int csplit = L[l + 1].lean ? 1 : 0;
    int rc = relax_lean<T>(l, o.num_smooth_down, zero_init);
    if (rc) return rc;
    CK(launch_vcl_restrict<T>(P, L[l + 1].G, csplit, o.num_smooth_down >= 1 ? 1 : 0,
                              (T *)L[l + 1].r, (T *)L[l + 1].e, s));
    for (int m = 0; m < o.num_mg; m++) {
      rc = cycle<T>(l + 1, m == 0);
      if (rc) return rc;
    }
    CK(launch_vcl_prolong<T>(P, L[l + 1].G, make_bcd(op.bc), csplit,
                             o.num_smooth_up >= 1 ? 1 : 0, o.prolong, (const T *)L[l + 1].ecur,
                             s));
    return relax_lean<T>(l, o.num_smooth_up, false);
  }

  template <class T>
  int cycle(int l, bool zero_init) {
    int last = (int)L.size() - 1;
    VCArgs<T> A = args<T>(l);
    // a fresh correction starts in e; a continued one stays where the last
    // pass left it (the tile path alternates e / t, the other paths work in e)
    if (zero_init || !L[l].ecur) L[l].ecur = L[l].e;
    if (L[l].lean) return cycle_lean<T>(l, zero_init);
    // the lean FP32 single-CTA cycle takes levels up to 1024 cells
    const long long block_cells = (sizeof(T) == 4 && L[l].fcx) ? kFastCycCells : kBlockCycleCells;
    if (use_tiles && l < last && L[l].G.dim == 2 && L[l].G.ncell > block_cells) {
      int rc = tile_sweeps<T>(l, 2 * o.num_smooth_down, zero_init, true, false);
      if (rc) return rc;
      rc = cycle<T>(l + 1, true);
      if (rc) return rc;
      return tile_sweeps<T>(l, 2 * o.num_smooth_up, false, false, true);
    }
    if (use_block_cycle && L[l].G.ncell <= block_cells && last - l + 1 <= kMaxBlockLevels &&
        last > l) {
      // this level and every coarser one inside one thread block
      if constexpr (sizeof(T) == 4) {
        const Geom &G0 = L[l].G;
        if (L[l].fcx && l == cyc_top && last - l + 1 <= kFastCycLevels &&
            (G0.n0 / 2) * (G0.n1 / 2) <= kFastCycThreads) {
          // lean FP32 form with the precomputed face weights and 1/diag
          CycFast F;
          F.nlev = last - l + 1;
          F.pre = o.num_smooth_down;
          F.post = o.num_smooth_up;
          F.bottom = o.bottom_max_iter;
          F.prolong = o.prolong;
          F.zero_init = zero_init ? 1 : 0;
          F.bc = make_bcd(op.bc);
          for (int m = 0; m < F.nlev; m++) F.G[m] = L[l + m].G;
          for (int m = 0; m <= F.nlev; m++) F.off[m] = cyc_off[m];
          F.pack = reinterpret_cast<const float4 *>(cyc_pack);
          F.e0 = (float *)L[l].e;
          F.r0 = (const float *)L[l].r;
          F.fault = &dev_state->fault;
          CK(launch_vc_cycle_fast(F, s));
          return MLGPU_OK;
        }
      }
      VCBlockCycle<T> P;
      P.nlev = last - l + 1;
      P.pre = o.num_smooth_down;
      P.post = o.num_smooth_up;
      P.bottom = o.bottom_max_iter;
      P.prolong = o.prolong;
      P.zero_init = zero_init ? 1 : 0;
      P.bc = make_bcd(op.bc);
      for (int m = 0; m < P.nlev; m++) {
        P.A[m] = args<T>(l + m);
        P.e[m] = (T *)L[l + m].e;
        P.r[m] = (T *)L[l + m].r;
      }
      CK(launch_vc_block_cycle<T>(P, s));
      return MLGPU_OK;
    }
    if (l == last) {
      if (o.bottom_solver == MLGPU_BOTTOM_BICGSTAB) {
        if (zero_init) CK(cudaMemsetAsync(L[l].e, 0, sizeof(T) * L[l].G.ncell, s));
        VCArgs<double> A64 = args<double>(l);
        CK(launch_vc_bicgstab<T>(A64, (T *)L[l].e, (const T *)L[l].r, bicg_ws,
                                 o.bottom_max_iter, (sizeof(T) == 4 && singular()) ? 1 : 0, s));
        return MLGPU_OK;
      }
      if (o.relax_mode == MLGPU_RELAX_JACOBI) return relax<T>(l, o.bottom_max_iter, zero_init);
      CK(launch_vc_relax_block<T>(A, (T *)L[l].e, (const T *)L[l].r, o.bottom_max_iter,
                                  zero_init ? 1 : 0, s));
      return MLGPU_OK;
    }
    int rc = relax<T>(l, o.num_smooth_down, zero_init);
    if (rc) return rc;
    CK(launch_vc_restrict<T>(A, L[l + 1].G, (const T *)L[l].e, (const T *)L[l].r,
                             (T *)L[l + 1].r, nullptr, s));
    for (int m = 0; m < o.num_mg; m++) {
      rc = cycle<T>(l + 1, m == 0);
      if (rc) return rc;
    }
    CK(launch_prolong<T>(L[l].G, make_bcd(op.bc), 1, o.prolong, (T *)L[l].e,
                         (const T *)L[l + 1].ecur, nullptr, s));
    return relax<T>(l, o.num_smooth_up, false);
  }

  // one outer iteration: inner cycles on (e0, r0), then phi_out = phi_in + e0
  // and the new residual (r0 in inner precision) with its norm
  // one outer iteration; `par` (device) selects the ping-pong direction when
  // the loop runs on the device, and then the decision kernel ends the body
  int iteration(int from, const int *par = nullptr, cudaGraphConditionalHandle h = 0) {
    int rc;
    int cycles = inner_cycles();
    for (int c = 0; c < cycles; c++) {
      rc = mixed ? cycle<float>(0, c == 0) : cycle<double>(0, c == 0);
      if (rc) return rc;
    }
    if (L[0].ocx) {
      int rc2 = outer_fast(phi[from], (const float *)L[0].ecur, phi[1 - from], par,
                           par ? dev_state : nullptr, h);
      if (rc2) return rc2;
      if (!par)
        CK(cudaMemcpyAsync(host_norm, part + kMaxBlocks, sizeof(double), cudaMemcpyDeviceToHost, s));
      return MLGPU_OK;
    }
    VCArgs<double> A = args<double>(0);
    A.a = (const double *)op.aCoef;
    A.c = (const double *)op.cCoef;
    for (int d = 0; d < 3; d++) A.b[d] = (const double *)op.bCoef[d];
    int nparts = 0;
    if (mixed && L[0].lean)
      CK(launch_vcl_outer<float>(A, o.norm_type, phi[from], (const float *)L[0].ecur, rhs,
                                 phi[1 - from], (float *)L[0].r, part, &nparts, s, par));
    else if (L[0].lean)
      CK(launch_vcl_outer<double>(A, o.norm_type, phi[from], (const double *)L[0].ecur, rhs,
                                  phi[1 - from], (double *)L[0].r, part, &nparts, s, par));
    else if (mixed)
      CK((launch_vc_update_residual<double, float>(A, o.norm_type, phi[from],
                                                   (const float *)L[0].ecur, rhs, phi[1 - from],
                                                   nullptr, (float *)L[0].r, part, &nparts, s,
                                                   par)));
    else
      CK((launch_vc_update_residual<double, double>(A, o.norm_type, phi[from],
                                                    (const double *)L[0].ecur, rhs, phi[1 - from],
                                                    nullptr, (double *)L[0].r, part, &nparts, s,
                                                    par)));
    CK(launch_finalize_norm(o.norm_type, part, nparts, part + kMaxBlocks, s));
    if (par) {
      OuterCfg cfg{o.tolerance, o.hang, o.norm_thresh, o.max_iter};
      CK(launch_outer_decide(dev_state, part + kMaxBlocks, cfg, h, s));
    } else {
      CK(cudaMemcpyAsync(host_norm, part + kMaxBlocks, sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    return MLGPU_OK;
  }

  // whole outer loop as a graph WHILE node (one launch per solve)
  int build_loop() {
    cudaGraph_t g;
    CK(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
    cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    if (e == cudaSuccess) e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np);
    if (e == cudaSuccess)
      e = cudaStreamBeginCaptureToGraph(s, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                        cudaStreamCaptureModeThreadLocal);
    int rc = MLGPU_OK;
    if (e == cudaSuccess) {
      rc = iteration(0, &dev_state->parity, h);
      cudaGraph_t body;
      e = cudaStreamEndCapture(s, &body);
      if (e == cudaSuccess) kern_loop = kernel_nodes(body);
    }
    if (e == cudaSuccess && rc == MLGPU_OK) e = cudaGraphInstantiate(&loop_exec, g, 0);
    cudaGraphDestroy(g);
    cudaGetLastError();
    if (rc) return rc;
    return e == cudaSuccess ? MLGPU_OK : MLGPU_ERR_CUDA;
  }

  int run_iteration(int from) {
    if (!o.use_graph) return iteration(from);
    if (!graph[from]) {
      cudaGraph_t g;
      CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      int rc = iteration(from);
      cudaError_t e = cudaStreamEndCapture(s, &g);
      if (rc) return rc;
      CK(e);
      e = cudaGraphInstantiate(&graph[from], g, 0);
      cudaGraphDestroy(g);
      CK(e);
    }
    CK(cudaGraphLaunch(graph[from], s));
    return MLGPU_OK;
  }

  // residual and norm of the starting field (no update); norm in part[kMaxBlocks]
  int initial_residual() {
    VCArgs<double> A = args<double>(0);
    A.a = (const double *)op.aCoef;
    A.c = (const double *)op.cCoef;
    for (int d = 0; d < 3; d++) A.b[d] = (const double *)op.bCoef[d];
    if (L[0].ocx) {
      int rc0 = outer_fast(phi[0], nullptr, nullptr, nullptr, nullptr, 0);
      if (rc0) return rc0;
    } else {
      int nparts = 0;
      if (mixed && L[0].lean)
        CK(launch_vcl_outer<float>(A, o.norm_type, phi[0], nullptr, rhs, nullptr,
                                   (float *)L[0].r, part, &nparts, s));
      else if (L[0].lean)
        CK(launch_vcl_outer<double>(A, o.norm_type, phi[0], nullptr, rhs, nullptr,
                                    (double *)L[0].r, part, &nparts, s));
      else if (mixed)
        CK((launch_vc_update_residual<double, float>(A, o.norm_type, phi[0], nullptr, rhs, nullptr,
                                                     nullptr, (float *)L[0].r, part, &nparts, s)));
      else
        CK((launch_vc_update_residual<double, double>(A, o.norm_type, phi[0], nullptr, rhs, nullptr,
                                                      nullptr, (double *)L[0].r, part, &nparts,
                                                      s)));
      CK(launch_finalize_norm(o.norm_type, part, nparts, part + kMaxBlocks, s));
    }
    return MLGPU_OK;
  }

  int solve(double *user_phi, const double *user_rhs, mlgpu_solve_stats *st) override {
    if (!user_phi || !user_rhs || !st) return MLGPU_ERR_ARG;
    size_t bytes = sizeof(double) * L[0].G.ncell;
    cudaGetLastError();  // clear any stale error of an earlier call
    if (enter()) return MLGPU_ERR_CUDA;
    CK(cudaMemcpyAsync(phi[0], user_phi, bytes, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(rhs, user_rhs, bytes, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemsetAsync(&dev_state->fault, 0, sizeof(int), s));
    // initial residual (no update)
    if (kern_init < 0) {
      kern_init = count_kernels([&] { return initial_residual(); });
      kern_iter = count_kernels([&] { return iteration(0); });
    }
    int rc_init = initial_residual();
    if (rc_init) return rc_init;
    CK(cudaMemcpyAsync(host_norm, part + kMaxBlocks, sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    Outer S;
    S.norm0 = S.norm = S.prev = *host_norm;
    stats_begin(st, (int)L.size(), S.norm0);
    st->cell_updates = (double)L[0].G.ncell;
    st->kernel_launches = kern_init;
    if (!std::isfinite(S.norm0)) S.status = 8;
    int cur = 0;
    if (o.use_graph >= 2 && !loop_failed && outer_continue(o, S)) {
      if (!loop_exec && build_loop() != MLGPU_OK) loop_failed = true;
      if (!loop_failed) {
        memset(host_state, 0, sizeof(OuterDev));
        host_state->norm0 = host_state->norm = host_state->prev = S.norm0;
        CK(cudaMemcpyAsync(dev_state, host_state, sizeof(OuterDev), cudaMemcpyHostToDevice, s));
        CK(cudaGraphLaunch(loop_exec, s));
        CK(cudaMemcpyAsync(host_state, dev_state, sizeof(OuterDev), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        S.iter = host_state->iter;
        S.norm = host_state->norm;
        S.prev = host_state->prev;
        S.status = host_state->status;
        for (int i = 1; i <= S.iter && i < 64; i++) st->norm_history[i] = host_state->hist[i];
        cur = host_state->parity;
        st->cycles = S.iter * inner_cycles();
        st->cell_updates += S.iter * updates_per_iter;
        st->kernel_launches += (double)S.iter * kern_loop;
      }
    }
    while (outer_continue(o, S)) {
      int rc = run_iteration(cur);
      if (rc) return rc;
      CK(cudaStreamSynchronize(s));
      cur = 1 - cur;
      S.norm = *host_norm;
      st->cycles += inner_cycles();
      st->cell_updates += updates_per_iter;
      st->kernel_launches += kern_iter;
      outer_after(o, S, st);
    }
    CK(cudaMemcpyAsync(user_phi, phi[cur], bytes, cudaMemcpyDeviceToDevice, s));
    // a kernel whose bounded wait ran out leaves its mark in the device state
    CK(cudaMemcpyAsync(&host_state->fault, &dev_state->fault, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (host_state->fault) S.status = kStatusDeviceFault;
    if (leave()) return MLGPU_ERR_CUDA;
    return outer_finish(o, S, st);
  }

  int set_alpha_beta(double a, double b) override {
    op.alpha = a;
    op.beta = b;
    drop_graphs();
    if (enter()) return MLGPU_ERR_CUDA;
    int rc = mixed ? build_fast() : build_lambda();
    if (!rc) rc = leave();
    return rc;
  }
};

// ====================================================================== HC
struct HCLevel {
  mlgpu_grid grid;
  Geom G;
  Coefs<double> c64;
  double *u = nullptr, *f = nullptr, *r = nullptr, *uold = nullptr, *t = nullptr;
  double *tcl = nullptr;  // (T, C_l) of u, valid while tcl_ok says so
  double *lam = nullptr;  // stored 1/diag (resetLambda)
  // mixed precision: FP32 correction, residual, closure Jacobian, 1/diag, coefficients
  float *e32 = nullptr, *r32 = nullptr, *J32 = nullptr, *lam32 = nullptr;
  float *a32 = nullptr, *b32[3] = {nullptr, nullptr, nullptr};
};

class HCSolver : public mlgpu_solver {
 public:
  mlgpu_nlop op;
  mlgpu_mg_options o;
  std::vector<HCLevel> L;
  double *part = nullptr, *host_norm = nullptr;
  int kern_init = -1, kern_iter = -1;  // kernels per piece (counted)
  bool mixed = false;  // FP32 linearised inner cycles in FP64 defect correction
  // within a mixed solve: take linearised steps now?  The solve starts with
  // FP64 FAS cycles (a linearisation at a state far from the solution
  // overshoots across closure regime boundaries) and switches to the FP32
  // linearised cycles once a FAS iteration has at least halved the residual;
  // a linearised step that fails to reduce the residual goes back to FAS, and
  // after two such failures the solve stays with FAS
  bool lin = false;
  int lin_fail = 0;
  cudaGraphExec_t graph_m = nullptr;
  int kern_iter_fas = -1;
  double upd_fas = 0, upd_lin = 0;
  // per level: does tcl hold the closure of the current u?  Tracked on the
  // host along the launch sequence (the same sequence every iteration)
  std::vector<char> tcl_ok;
  cudaGraphExec_t graph = nullptr;
  double updates_per_iter = 0;

  ~HCSolver() override {
    if (graph) cudaGraphExecDestroy(graph);
    if (graph_m) cudaGraphExecDestroy(graph_m);
    if (host_norm) cudaFreeHost(host_norm);
  }

  size_t layout(char *base) {
    Arena A;
    A.base = base;
    int depth = mg_depth(op.grid, o.max_coarse);
    L.assign(depth + 1, HCLevel());
    mlgpu_grid g = op.grid;
    for (int l = 0; l <= depth; l++) {
      L[l].grid = g;
      L[l].G = make_geom(g);
      size_t n = 2 * ncells(g);
      if (l == 0) {
        L[l].c64.a = (double *)op.aCoef;
        for (int d = 0; d < 3; d++) L[l].c64.b[d] = (double *)op.bCoef[d];
      } else {
        if (op.aCoef) L[l].c64.a = A.get<double>(n);
        for (int d = 0; d < g.dim; d++) L[l].c64.b[d] = A.get<double>(2 * nfaces(g, d));
      }
      L[l].u = A.get<double>(n);
      L[l].f = A.get<double>(n);
      L[l].r = A.get<double>(n);
      L[l].uold = A.get<double>(n);
      L[l].t = A.get<double>(n);
      L[l].tcl = A.get<double>(n);
      L[l].lam = A.get<double>(n);
      if (mixed) {
        L[l].e32 = A.get<float>(n);
        L[l].r32 = A.get<float>(n);
        L[l].J32 = A.get<float>(2 * n);
        L[l].lam32 = A.get<float>(n);
        if (op.aCoef) L[l].a32 = A.get<float>(n);
        for (int d = 0; d < g.dim; d++) L[l].b32[d] = A.get<float>(2 * nfaces(g, d));
      }
      g = coarsen_grid(g);
    }
    tcl_ok.assign(L.size(), 0);
    part = A.get<double>(kNormScratchDoubles);
    return A.off + 256;
  }

  int build_coefs() {
    for (size_t l = 1; l < L.size(); l++) {
      Geom F = L[l - 1].G;
      if (op.aCoef) CK(launch_restrict_avg<double>(F, 2, L[l - 1].c64.a, L[l].c64.a, s));
      for (int d = 0; d < F.dim; d++)
        CK(launch_coarsen_faces<double>(F, 2, d, L[l - 1].c64.b[d], L[l].c64.b[d], s));
    }
    int rc = build_lambda();
    if (rc) return rc;
    if (mixed) {
      for (auto &lv : L) {
        long long n = 2 * lv.G.ncell;
        if (lv.a32) CK(launch_convert<float, double>(n, lv.a32, lv.c64.a, s));
        for (int d = 0; d < lv.G.dim; d++)
          CK(launch_convert<float, double>(2 * lv.G.nface(d), lv.b32[d], lv.c64.b[d], s));
      }
    }
    int last = (int)L.size() - 1;
    std::vector<double> visits(L.size(), 0);
    visits[0] = 1;
    for (int l = 1; l <= last; l++) visits[l] = visits[l - 1] * o.num_mg;
    for (int lin_cycle = 0; lin_cycle < 2; lin_cycle++) {
      double u = 0;
      for (int l = 0; l <= last; l++) {
        double n = (double)L[l].G.ncell;
        if (l == last)
          u += visits[l] * o.bottom_max_iter * n;
        else  // the FAS cycle also applies the coarse operator once per visit
          u += visits[l] * ((o.num_smooth_down + o.num_smooth_up) * n + n +
                            (lin_cycle ? 0.0 : (double)L[l + 1].G.ncell));
      }
      (lin_cycle ? upd_lin : upd_fas) = u + (double)L[0].G.ncell;
    }
    updates_per_iter = mixed ? upd_lin : upd_fas;
    return MLGPU_OK;
  }

  // stored 1/diag of every level (bitwise the inline resetLambda value)
  int build_lambda() {
    for (size_t l = 0; l < L.size(); l++) {
      CK(launch_nl_lambda<double>(args((int)l), L[l].lam, s));
      if (L[l].lam32)
        CK(launch_convert<float, double>(2 * L[l].G.ncell, L[l].lam32, L[l].lam, s));
    }
    return MLGPU_OK;
  }

  // ---- mixed precision: FP32 cycles on the problem linearised at u
  HCMArgs margs(int l) {
    NLArgs<double> D = args(l);
    HCMArgs M;
    M.G = D.G;
    M.phi_bc = D.phi_bc;
    M.dbc = D.dbc;
    M.apply_dbc = D.apply_dbc;
    M.alpha = (float)D.alpha;
    M.beta = (float)D.beta;
    M.dxinv = (float)D.dxinv;
    M.a = L[l].a32;
    for (int d = 0; d < 3; d++) M.b[d] = L[l].b32[d];
    M.J = L[l].J32;
    M.lam = L[l].lam32;
    return M;
  }

  // correction-scheme V-cycle on level l (e starts at zero)
  int mcycle(int l) {
    const int last = (int)L.size() - 1;
    HCMArgs M = margs(l);
    if (l == last) {
      CK(launch_hcm_relax_block(M, L[l].e32, L[l].r32, o.bottom_max_iter, s));
      return MLGPU_OK;
    }
    CK(cudaMemsetAsync(L[l].e32, 0, sizeof(float) * 2 * L[l].G.ncell, s));
    for (int i = 0; i < o.num_smooth_down; i++)
      for (int pass = 0; pass < 2; pass++) CK(launch_hcm_gsrb(M, L[l].e32, L[l].r32, pass, s));
    CK(launch_hcm_restrict(M, L[l + 1].G, L[l].e32, L[l].r32, L[l + 1].r32, s));
    for (int m = 0; m < o.num_mg; m++) {
      int rc = mcycle(l + 1);
      if (rc) return rc;
    }
    CK(launch_prolong<float>(L[l].G, make_bcd(op.phi_bc), 2, o.prolong, L[l].e32, L[l + 1].e32,
                             nullptr, s));
    for (int i = 0; i < o.num_smooth_up; i++)
      for (int pass = 0; pass < 2; pass++) CK(launch_hcm_gsrb(M, L[l].e32, L[l].r32, pass, s));
    return MLGPU_OK;
  }

  // one defect-correction step: J at the current state on every level (the
  // state restricted by averaging), FP32 cycle on r = f - N(u) (left in
  // L[0].r by the previous residual), u += e, FP64 residual and norm
  int iteration_mixed() {
    for (size_t l = 1; l < L.size(); l++)
      CK(launch_restrict_avg<double>(L[l - 1].G, 2, L[l - 1].u, L[l].u, s));
    for (size_t l = 0; l < L.size(); l++)
      CK(launch_hcm_jac(L[l].G, args((int)l).cp, L[l].u, L[l].J32, s));
    CK(launch_convert<float, double>(2 * L[0].G.ncell, L[0].r32, L[0].r, s));
    int rc = mcycle(0);
    if (rc) return rc;
    CK(launch_hcm_update(2 * L[0].G.ncell, L[0].u, L[0].e32, s));
    tcl_ok[0] = 0;
    return residual_norm();
  }

  // make tcl of level l the closure of its u
  int ensure_tcl(int l) {
    if (!tcl_ok[l]) CK(launch_nlc_closure(args(l), L[l].u, L[l].tcl, s));
    tcl_ok[l] = 1;
    return MLGPU_OK;
  }

  NLArgs<double> args(int l) {
    mlgpu_nlop lop = op;
    lop.grid = L[l].grid;
    NLArgs<double> A = make_nl_args<double>(lop);
    A.a = L[l].c64.a;
    for (int d = 0; d < 3; d++) A.b[d] = L[l].c64.b[d];
    return A;
  }

  int relax(int l, int n) {
    NLArgs<double> A = args(l);
    for (int i = 0; i < n; i++) {
      if (o.relax_mode == MLGPU_RELAX_JACOBI) {
        CK(launch_nl_op<double>(A, NL_JACOBI, -1, L[l].u, L[l].f, L[l].t, nullptr, nullptr, nullptr,
                                s));
        CK(cudaMemcpyAsync(L[l].u, L[l].t, sizeof(double) * 2 * L[l].G.ncell,
                           cudaMemcpyDeviceToDevice, s));
        tcl_ok[l] = 0;
      } else {
        int rc = ensure_tcl(l);
        if (rc) return rc;
        CK(launch_nlc_gsrb(A, L[l].u, L[l].f, L[l].tcl, L[l].lam, 0, s));
        CK(launch_nlc_gsrb(A, L[l].u, L[l].f, L[l].tcl, L[l].lam, 1, s));
      }
    }
    return MLGPU_OK;
  }

  int cycle(int l) {
    int last = (int)L.size() - 1;
    NLArgs<double> A = args(l);
    if (l == last) {
      if (o.relax_mode == MLGPU_RELAX_JACOBI) return relax(l, o.bottom_max_iter);
      CK(launch_nlc_relax_block(A, L[l].u, L[l].f, L[l].tcl, L[l].lam, o.bottom_max_iter,
                                tcl_ok[l] ? 0 : 1, s));
      tcl_ok[l] = 1;
      return MLGPU_OK;
    }
    int rc = relax(l, o.num_smooth_down);
    if (rc) return rc;
    HCLevel &C = L[l + 1];
    rc = ensure_tcl(l);
    if (rc) return rc;
    CK(launch_nlc_restrict(A, C.G, L[l].u, L[l].tcl, L[l].f, C.r, C.u, s));
    tcl_ok[l + 1] = 0;
    rc = ensure_tcl(l + 1);
    if (rc) return rc;
    CK(launch_nlc_op(args(l + 1), NL_APPLY_PLUS, -1, C.u, C.tcl, C.r, C.f, C.uold, nullptr, nullptr,
                     s));
    for (int m = 0; m < o.num_mg; m++) {
      rc = cycle(l + 1);
      if (rc) return rc;
    }
    CK(launch_prolong<double>(L[l].G, make_bcd(op.phi_bc), 2, o.prolong, L[l].u, C.u, C.uold, s));
    tcl_ok[l] = 0;
    return relax(l, o.num_smooth_up);
  }

  int residual_norm() {
    int rc = ensure_tcl(0);
    if (rc) return rc;
    int nparts = 0;
    CK(launch_nlc_op(args(0), NL_RESIDUAL, o.norm_type, L[0].u, L[0].tcl, L[0].f, L[0].r, nullptr,
                     part, &nparts, s));
    CK(launch_finalize_norm(o.norm_type, part, nparts, part + kMaxBlocks, s));
    CK(cudaMemcpyAsync(host_norm, part + kMaxBlocks, sizeof(double), cudaMemcpyDeviceToHost, s));
    return MLGPU_OK;
  }

  // one FAS iteration; on entry tcl of level 0 is valid (the residual norm
  // that ended the previous iteration, or the initial one, left it so)
  int iteration() {
    tcl_ok[0] = 1;
    if (mixed && lin) return iteration_mixed();
    int rc = cycle(0);
    if (rc) return rc;
    return residual_norm();
  }

  int run_iteration() {
    if (!o.use_graph) return iteration();
    cudaGraphExec_t &gx = (mixed && lin) ? graph_m : graph;
    if (!gx) {
      cudaGraph_t g;
      CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      int rc = iteration();
      cudaError_t e = cudaStreamEndCapture(s, &g);
      if (rc) return rc;
      CK(e);
      e = cudaGraphInstantiate(&gx, g, 0);
      cudaGraphDestroy(g);
      CK(e);
    }
    CK(cudaGraphLaunch(gx, s));
    return MLGPU_OK;
  }

  int solve(double *user_phi, const double *user_rhs, mlgpu_solve_stats *st) override {
    if (!user_phi || !user_rhs || !st) return MLGPU_ERR_ARG;
    size_t bytes = sizeof(double) * 2 * L[0].G.ncell;
    cudaGetLastError();  // clear any stale error of an earlier call
    if (enter()) return MLGPU_ERR_CUDA;
    CK(cudaMemcpyAsync(L[0].u, user_phi, bytes, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(L[0].f, user_rhs, bytes, cudaMemcpyDeviceToDevice, s));
    tcl_ok.assign(L.size(), 0);  // u of level 0 was just replaced
    if (kern_init < 0) {
      kern_init = count_kernels([&] { return residual_norm(); });
      lin = mixed;
      kern_iter = count_kernels([&] { return iteration(); });
      lin = false;
      kern_iter_fas = count_kernels([&] { return iteration(); });
      tcl_ok.assign(L.size(), 0);  // the counting captures launched nothing
    }
    lin = false;
    lin_fail = 0;
    int rc = residual_norm();
    if (rc) return rc;
    CK(cudaStreamSynchronize(s));
    Outer S;
    S.norm0 = S.norm = S.prev = *host_norm;
    stats_begin(st, (int)L.size(), S.norm0);
    st->cell_updates = (double)L[0].G.ncell;
    st->kernel_launches = kern_init;
    if (!std::isfinite(S.norm0)) S.status = 8;
    while (outer_continue(o, S)) {
      const bool was_lin = mixed && lin;
      rc = run_iteration();
      if (rc) return rc;
      CK(cudaStreamSynchronize(s));
      S.norm = *host_norm;
      st->cycles += 1;
      st->cell_updates += was_lin ? upd_lin : upd_fas;
      st->kernel_launches += was_lin ? kern_iter : kern_iter_fas;
      if (was_lin && std::isfinite(S.norm) && S.norm > (1.0 - o.hang) * S.prev &&
          S.norm > o.tolerance * S.norm0) {
        // the linearised step did not reduce the FP64 residual: back to FP64
        // FAS cycles (the state and its FP64 residual stay valid)
        lin = false;
        lin_fail++;
        S.iter++;
        if (S.iter < 64) st->norm_history[S.iter] = S.norm;
        S.prev = S.norm;
        continue;
      }
      if (mixed && !was_lin && lin_fail < 2 && std::isfinite(S.norm) && S.norm < 0.5 * S.prev)
        lin = true;
      outer_after(o, S, st);
    }
    CK(cudaMemcpyAsync(user_phi, L[0].u, bytes, cudaMemcpyDeviceToDevice, s));
    CK(cudaStreamSynchronize(s));
    if (leave()) return MLGPU_ERR_CUDA;
    return outer_finish(o, S, st);
  }

  // new wall conditions: kernel arguments only (1/diag does not see them)
  int set_bcs(const mlgpu_bc *phi_bc, const mlgpu_bc *derived_bc) {
    mlgpu_nlop t = op;
    if (phi_bc) t.phi_bc = *phi_bc;
    if (derived_bc) t.derived_bc = *derived_bc;
    if (!valid_nl_bcs(t)) return MLGPU_ERR_ARG;
    op = t;
    for (auto *gp : {&graph, &graph_m})
      if (*gp) {
        cudaGraphExecDestroy(*gp);
        *gp = nullptr;
      }
    return MLGPU_OK;
  }

  int set_alpha_beta(double a, double b) override {
    op.alpha = a;
    op.beta = b;
    for (auto *gp : {&graph, &graph_m})
      if (*gp) {
        cudaGraphExecDestroy(*gp);
        *gp = nullptr;
      }
    // 1/diag depends on alpha and beta
    if (enter()) return MLGPU_ERR_CUDA;
    int rc = build_lambda();
    if (!rc) rc = leave();
    return rc;
  }
};

// ================================================================ adjoint
// Multigrid for A^T y = g, A = dN/dphi at a given state (adjoint_kernels.cuh).
// The hierarchy is the FAS solver's: coefficients coarsened the same way,
// the state averaged down, J per level from its state; correction-scheme
// V-cycles (block red/black smoothing, 2^D residual averaging, the solver's
// prolongation with the adjoint variable's wall rule; at the bottom an exact
// dense solve when it has at most kAdjDirectMax unknowns, else single-CTA
// relaxation) inside an FP64 residual loop.
struct AdjLevel {
  mlgpu_grid grid;
  Geom G;
  Coefs<double> c64;
  double *u = nullptr, *J = nullptr, *y = nullptr, *g = nullptr, *r = nullptr;
  double *Minv = nullptr;  // inverse diagonal blocks of A^T, per state
  // mixed-precision Newton: FP32 copies of the coefficients, J (from the FP64
  // closure derivative), the inverse diagonal blocks and the cycle's fields
  Coefs<float> c32;
  float *J32 = nullptr, *Minv32 = nullptr, *y32 = nullptr, *g32 = nullptr, *r32 = nullptr;
  float *D32 = nullptr, *w32 = nullptr;  // diagonal blocks of A, and w = J y (lean cycles)
  // FP64 lean cycles (the comparison path): w = J y, A's diagonal blocks, and
  // on level 0 the right-hand side in the lean layout
  double *w64 = nullptr, *D64 = nullptr, *g64s = nullptr;
  // lean cycles on a smoothed level (every level above the bottom): J,
  // K = (D^T)^-1 and D permuted to the colour-split layout, in the cycles'
  // precision (the natural ones above feed the bottom solve and the packing)
  float *J32s = nullptr, *K32s = nullptr, *D32s = nullptr;
  double *J64s = nullptr, *K64s = nullptr, *D64s = nullptr;
  // their face sums P (lean_face_sums, natural layout), formed once
  float *P32 = nullptr;
  double *P64 = nullptr;
};

class HCAdjSolver : public mlgpu_solver {
 public:
  mlgpu_nlop op;
  mlgpu_mg_options o;
  std::vector<AdjLevel> L;
  double *part = nullptr, *host_norm = nullptr, *bcg = nullptr;
  double *part2 = nullptr;  // max-norm partials of the Newton residual
  double updates_per_iter = 0;
  int kern_iter = -1, kern_init = -1;
  // tr: cycles on A^T (adjoint) or on A (the linear solve of a Newton step);
  // one captured iteration graph per mode
  bool tr = true;
  // MLGPU_PREC_MIXED: the linear cycles of a Newton step run in FP32 (the
  // Newton residual, its norm, the update and the closure stay FP64); the
  // adjoint solve stays FP64
  bool mixed = false;
  // FP64 with options.fuse_levels >= 2: Newton's linear cycles run the lean
  // kernels in FP64 -- the same design and layout as the mixed cycles, the
  // reference's expression order given up -- the comparison path for the
  // mixed-precision speed-up
  bool fast64 = false;
  cudaGraphExec_t graph = nullptr, graph_lin = nullptr, graph_lin32 = nullptr;
  double *nf = nullptr, *nuold = nullptr;  // Newton: rhs of N(u) = f, previous u
  double *ntcl = nullptr;  // Newton: (T, C_l) of level 0, the residual's closure cache
  double *nsb = nullptr;   // lean Newton: level 0's face sums per cell and component
  // Newton's kernels per piece (counted once): state and Jacobians of every
  // level, one linear cycle + residual
  int nk_state = -1, nk_iter = -1;
  // kernels of nl_residual (closure, stencil + norms, combine, combine; a
  // stopping norm other than max adds its own pass) and of one step update
  static constexpr int kStepKernels = 1;
  int nl_residual_kernels() const { return o.norm_type == MLGPU_NORM_MAX ? 4 : 5; }

  ~HCAdjSolver() override {
    if (graph) cudaGraphExecDestroy(graph);
    if (graph_lin) cudaGraphExecDestroy(graph_lin);
    if (graph_lin32) cudaGraphExecDestroy(graph_lin32);
    if (host_norm) cudaFreeHost(host_norm);
  }

  bool lin32() const { return mixed && !tr; }
  // the lean cycles' arrays of level l are colour-split on every smoothed
  // level (all but the bottom, whose dimensions are then all even)
  bool split(int l) const { return l < (int)L.size() - 1; }

  size_t layout(char *base) {
    Arena A;
    A.base = base;
    mixed = o.precision == MLGPU_PREC_MIXED;
    fast64 = !mixed && o.fuse_levels >= 2;
    int depth = mg_depth(op.grid, o.max_coarse);
    L.assign(depth + 1, AdjLevel());
    mlgpu_grid g = op.grid;
    for (int l = 0; l <= depth; l++) {
      L[l].grid = g;
      L[l].G = make_geom(g);
      size_t n = 2 * ncells(g);
      if (l == 0) {
        L[l].c64.a = (double *)op.aCoef;
        for (int d = 0; d < 3; d++) L[l].c64.b[d] = (double *)op.bCoef[d];
      } else {
        if (op.aCoef) L[l].c64.a = A.get<double>(n);
        for (int d = 0; d < g.dim; d++) L[l].c64.b[d] = A.get<double>(2 * nfaces(g, d));
      }
      L[l].u = A.get<double>(n);
      L[l].J = A.get<double>(2 * n);
      L[l].Minv = A.get<double>(2 * n);
      L[l].y = A.get<double>(n);
      L[l].g = A.get<double>(n);
      L[l].r = A.get<double>(n);
      if (mixed) {
        if (op.aCoef) L[l].c32.a = A.get<float>(n);
        for (int d = 0; d < g.dim; d++) L[l].c32.b[d] = A.get<float>(2 * nfaces(g, d));
        L[l].J32 = A.get<float>(2 * n);
        L[l].Minv32 = A.get<float>(2 * n);
        L[l].D32 = A.get<float>(2 * n);
        L[l].y32 = A.get<float>(n);
        L[l].w32 = A.get<float>(n);
        L[l].g32 = A.get<float>(n);
        L[l].r32 = A.get<float>(n);
        if (l < depth) {
          L[l].J32s = A.get<float>(2 * n);
          L[l].K32s = A.get<float>(2 * n);
          L[l].D32s = A.get<float>(2 * n);
          L[l].P32 = A.get<float>(n);
        }
      }
      if (fast64) {
        L[l].w64 = A.get<double>(n);
        L[l].D64 = A.get<double>(2 * n);
        if (l == 0) L[l].g64s = A.get<double>(n);
        if (l < depth) {
          L[l].J64s = A.get<double>(2 * n);
          L[l].K64s = A.get<double>(2 * n);
          L[l].D64s = A.get<double>(2 * n);
          L[l].P64 = A.get<double>(n);
        }
      }
      g = coarsen_grid(g);
    }
    part = A.get<double>(kNormScratchDoubles);
    part2 = A.get<double>(kMaxBlocks);
    bcg = A.get<double>(16);
    nf = A.get<double>(2 * ncells(op.grid));
    nuold = A.get<double>(2 * ncells(op.grid));
    ntcl = A.get<double>(2 * ncells(op.grid));
    if (mixed || fast64) nsb = A.get<double>(2 * ncells(op.grid));
    return A.off + 256;
  }

  int build_coefs() {
    for (size_t l = 1; l < L.size(); l++) {
      Geom F = L[l - 1].G;
      if (op.aCoef) CK(launch_restrict_avg<double>(F, 2, L[l - 1].c64.a, L[l].c64.a, s));
      for (int d = 0; d < F.dim; d++)
        CK(launch_coarsen_faces<double>(F, 2, d, L[l - 1].c64.b[d], L[l].c64.b[d], s));
    }
    if (mixed)
      for (auto &lv : L) {
        const long long n = 2 * lv.G.ncell;
        if (op.aCoef) CK(launch_convert<float, double>(n, lv.c32.a, lv.c64.a, s));
        for (int d = 0; d < lv.G.dim; d++)
          CK(launch_convert<float, double>(2 * lv.G.nface(d), lv.c32.b[d], lv.c64.b[d], s));
      }
    if (nsb) CK(launch_nlc_bsum(make_nl_args<double>(op), nsb, s));
    // the lean cycles' face sums of every smoothed level
    for (size_t l = 0; l < L.size(); l++) {
      if (L[l].P32) CK(launch_lean_psum<float>(args32((int)l), L[l].P32, s));
      if (L[l].P64) CK(launch_lean_psum<double>(args((int)l), L[l].P64, s));
    }
    const int last = (int)L.size() - 1;
    double u = 0;
    for (int l = 0; l <= last; l++) {
      double n = (double)L[l].G.ncell;
      u += l == last ? o.bottom_max_iter * n : (o.num_smooth_down + o.num_smooth_up + 1) * n;
    }
    updates_per_iter = u + (double)L[0].G.ncell;
    return MLGPU_OK;
  }

  AdjArgs<double> args(int l) {
    mlgpu_nlop lop = op;
    lop.grid = L[l].grid;
    lop.aCoef = L[l].c64.a;
    for (int d = 0; d < 3; d++) lop.bCoef[d] = L[l].c64.b[d];
    AdjArgs<double> A = make_adj_args(lop, L[l].u, L[l].J);
    A.Minv = L[l].Minv;
    return A;
  }

  // FP32 operator of level l (mixed-precision Newton cycles)
  AdjArgs<float> args32(int l) {
    const AdjArgs<double> D = args(l);
    AdjArgs<float> A;
    A.G = D.G;
    A.cp = D.cp;
    A.phi_bc = D.phi_bc;
    A.dbc = D.dbc;
    A.apply_dbc = D.apply_dbc;
    A.alpha = (float)D.alpha;
    A.beta = (float)D.beta;
    A.dxinv = (float)D.dxinv;
    A.dx = (float)D.dx;
    A.a = L[l].c32.a;
    for (int d = 0; d < 3; d++) A.b[d] = L[l].c32.b[d];
    A.J = L[l].J32;
    A.u = L[l].u;
    A.Minv = L[l].Minv32;
    return A;
  }

  // lean operator of level l (lin_lean_kernels.cuh): FP32 arrays for the
  // mixed-precision cycles, FP64 ones for the FP64 comparison path; the
  // split copies of J, K, D on a smoothed level, the natural ones on the
  // bottom (x and g hold whichever layout the level's kernels use)
  template <class T>
  LinLeanT<T> leanT(int l) {
    const AdjArgs<double> D = args(l);
    LinLeanT<T> P;
    P.G = D.G;
    P.ybc = ybc();
    P.bdx = (T)(D.beta * D.dxinv);
    const bool sp = split(l);
    if constexpr (sizeof(T) == 4) {
      for (int d = 0; d < 3; d++) P.b[d] = L[l].c32.b[d];
      P.J = sp ? L[l].J32s : L[l].J32;
      P.K = sp ? L[l].K32s : L[l].Minv32;
      P.D = sp ? L[l].D32s : L[l].D32;
      P.x = L[l].y32;
      P.w = L[l].w32;
      P.g = L[l].g32;
    } else {
      for (int d = 0; d < 3; d++) P.b[d] = L[l].c64.b[d];
      P.J = sp ? L[l].J64s : L[l].J;
      P.K = sp ? L[l].K64s : L[l].Minv;
      P.D = sp ? L[l].D64s : L[l].D64;
      P.x = L[l].y;
      P.w = L[l].w64;
      P.g = l == 0 ? L[l].g64s : L[l].g;
    }
    return P;
  }
  LinLean lean(int l) { return leanT<float>(l); }

  // the wall rule of the adjoint variable in the prolongation
  BCD ybc() const { return make_bcd(op.apply_derived_bc ? op.derived_bc : op.phi_bc); }

  // state on every level and its Jacobians
  int set_state(const double *phi) {
    CK(cudaMemcpyAsync(L[0].u, phi, sizeof(double) * 2 * L[0].G.ncell, cudaMemcpyDeviceToDevice,
                       s));
    return state_levels();
  }
  // the coarse states averaged from level 0's, J everywhere
  int state_levels() {
    for (size_t l = 1; l < L.size(); l++)
      CK(launch_restrict_avg<double>(L[l - 1].G, 2, L[l - 1].u, L[l].u, s));
    const ClosureParams cp = make_cp(op.params);
    if (lin32()) {
      // smoothed levels: J (FP32, t_cl's regime), D and K straight to the
      // split layout; the bottom: J, the inverse blocks and D natural, for the
      // generic bottom solve
      for (size_t l = 0; l < L.size(); l++) {
        AdjLevel &lv = L[l];
        if (split((int)l)) {
          CK(launch_lean_state<float>(args32((int)l), lv.u, lv.P32, lv.J32s, lv.K32s, lv.D32s,
                                      s));
          continue;
        }
        CK(launch_adj_jac(lv.G, cp, lv.u, lv.J32, s));
        CK(cudaMemsetAsync(lv.r32, 0, sizeof(float) * 2 * lv.G.ncell, s));
        CK(launch_adj_minv(args32((int)l), lv.r32, lv.Minv32, lv.D32, s));
      }
      return MLGPU_OK;
    }
    const bool lean64 = fast64 && !tr;
    for (size_t l = 0; l < L.size(); l++) {
      AdjLevel &lv = L[l];
      if (lean64 && split((int)l)) {
        CK(launch_lean_state<double>(args((int)l), lv.u, lv.P64, lv.J64s, lv.K64s, lv.D64s, s));
        continue;
      }
      CK(launch_adj_jac(lv.G, cp, lv.u, lv.J, s));
      // the smoother's inverse diagonal blocks (r is free here: a zero field)
      CK(cudaMemsetAsync(lv.r, 0, sizeof(double) * 2 * lv.G.ncell, s));
      CK(launch_adj_minv(args((int)l), lv.r, lv.Minv, lean64 ? lv.D64 : nullptr, s));
    }
    return MLGPU_OK;
  }

  int smooth(int l, int n) {
    AdjArgs<double> A = args(l);
    for (int i = 0; i < n; i++)
      for (int pass = 0; pass < 2; pass++) CK(launch_adj_gsrb(A, L[l].y, L[l].g, pass, s, tr));
    return MLGPU_OK;
  }

  // V-cycle on level l; coarse levels start from zero
  int cycle(int l) {
    const int last = (int)L.size() - 1;
    AdjArgs<double> A = args(l);
    if (l == last) {
      if (2 * L[l].G.ncell <= kAdjDirectMax)
        CK(launch_adj_bottom_direct(A, L[l].y, L[l].g, s, tr));
      else
        CK(launch_adj_relax_block(A, L[l].y, L[l].g, o.bottom_max_iter, l > 0 ? 1 : 0, s, tr));
      return MLGPU_OK;
    }
    if (l > 0) CK(cudaMemsetAsync(L[l].y, 0, sizeof(double) * 2 * L[l].G.ncell, s));
    int rc = smooth(l, o.num_smooth_down);
    if (rc) return rc;
    CK(launch_adj_restrict(A, L[l + 1].G, L[l].y, L[l].g, L[l + 1].g, s, tr));
    for (int m = 0; m < o.num_mg; m++) {
      rc = cycle(l + 1);
      if (rc) return rc;
    }
    CK(launch_prolong<double>(L[l].G, ybc(), 2, o.prolong, L[l].y, L[l + 1].y, nullptr, s));
    return smooth(l, o.num_smooth_up);
  }

  int residual_norm() {
    int nparts = 0;
    CK(launch_adj_op(args(0), ADJ_RESIDUAL, o.norm_type, L[0].y, L[0].g, L[0].r, part, &nparts, s,
                     tr));
    CK(launch_finalize_norm(o.norm_type, part, nparts, part + kMaxBlocks, s));
    CK(cudaMemcpyAsync(host_norm, part + kMaxBlocks, sizeof(double), cudaMemcpyDeviceToHost, s));
    return MLGPU_OK;
  }

  // ---- lean cycles on A (Newton's linear solve): FP32 in mixed precision,
  // FP64 on the comparison path built the same way; same structure as the
  // generic cycles above.  They keep w = J y next to y on every level: zero
  // together, refreshed by every update and by the prolongation.  Smoothed
  // levels hold their arrays colour-split; each red/black half sweep is one
  // launch over its colour's contiguous half.
  template <class T>
  int lin_smooth(int l, int n) {
    const LinLeanT<T> P = leanT<T>(l);
    for (int i = 0; i < n; i++)
      for (int pass = 0; pass < 2; pass++) CK(launch_lean_gsrb<T>(P, pass, s, lean_vec));
    return MLGPU_OK;
  }

  template <class T>
  int lin_cycle(int l) {
    const int last = (int)L.size() - 1;
    const LinLeanT<T> P = leanT<T>(l);
    if (l == last) {
      // the bottom solve updates y alone: its w is never read
      if constexpr (sizeof(T) == 4) {
        AdjArgs<float> A = args32(l);
        if (2 * L[l].G.ncell <= kAdjDirectMax)
          CK(launch_adj_bottom_direct(A, P.x, P.g, s, false));
        else
          CK(launch_adj_relax_block(A, P.x, P.g, o.bottom_max_iter, l > 0 ? 1 : 0, s, false));
      } else {
        AdjArgs<double> A = args(l);
        if (2 * L[l].G.ncell <= kAdjDirectMax)
          CK(launch_adj_bottom_direct(A, P.x, P.g, s, false));
        else
          CK(launch_adj_relax_block(A, P.x, P.g, o.bottom_max_iter, l > 0 ? 1 : 0, s, false));
      }
      return MLGPU_OK;
    }
    // a coarse level's y and w were zeroed by the restriction that fed it
    int rc = lin_smooth<T>(l, o.num_smooth_down);
    if (rc) return rc;
    const LinLeanT<T> C = leanT<T>(l + 1);
    CK(launch_lean_restrict<T>(P, C.G, split(l + 1), o.num_smooth_down >= 1, (T *)C.g, C.x, C.w,
                               s, lean_vec));
    for (int m = 0; m < o.num_mg; m++) {
      if (m > 0) {  // every coarse visit starts from zero
        CK(cudaMemsetAsync(C.x, 0, sizeof(T) * 2 * C.G.ncell, s));
        CK(cudaMemsetAsync(C.w, 0, sizeof(T) * 2 * C.G.ncell, s));
      }
      rc = lin_cycle<T>(l + 1);
      if (rc) return rc;
    }
    CK(launch_lean_prolong<T>(P, C.G, split(l + 1), o.num_smooth_up >= 1, o.prolong, C.x, s));
    return lin_smooth<T>(l, o.num_smooth_up);
  }

  // linear residual g - A y of level 0 with its norm (combined in FP64);
  // after_cycle: at the end of a V-cycle whose post-smoothing ended in a
  // black half sweep (the red cells' residual alone)
  template <class T>
  int lin_residual_norm(bool after_cycle = false) {
    int nparts = 0;
    const bool red = after_cycle && o.num_smooth_up >= 1 && (int)L.size() > 1;
    CK(launch_lean_residual<T>(leanT<T>(0), split(0), red, o.norm_type, part, &nparts, s,
                               lean_vec));
    CK(launch_finalize_norm(o.norm_type, part, nparts, part + kMaxBlocks, s));
    CK(cudaMemcpyAsync(host_norm, part + kMaxBlocks, sizeof(double), cudaMemcpyDeviceToHost, s));
    return MLGPU_OK;
  }

  int iteration() {
    if (lin32()) {
      int rc = lin_cycle<float>(0);
      if (rc) return rc;
      return lin_residual_norm<float>(true);
    }
    if (fast64 && !tr) {
      int rc = lin_cycle<double>(0);
      if (rc) return rc;
      return lin_residual_norm<double>(true);
    }
    int rc = cycle(0);
    if (rc) return rc;
    return residual_norm();
  }

  int run_iteration() {
    if (!o.use_graph) return iteration();
    cudaGraphExec_t &gx = tr ? graph : (mixed ? graph_lin32 : graph_lin);
    if (!gx) {
      cudaGraph_t g;
      CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      int rc = iteration();
      cudaError_t e = cudaStreamEndCapture(s, &g);
      if (rc) return rc;
      CK(e);
      e = cudaGraphInstantiate(&gx, g, 0);
      cudaGraphDestroy(g);
      CK(e);
    }
    CK(cudaGraphLaunch(gx, s));
    return MLGPU_OK;
  }

  // ---- Newton for N(u) = f: u += d, A(u) d = f - N(u) solved by these
  // cycles on A to eta relative (at most `lin_max` cycles), halving d while
  // the FP64 residual grows (at most 4 times).  eta: `lin_tol`, or with
  // `forcing` the Eisenstat-Walker forcing term (their choice 2, gamma 0.9,
  // alpha 2, with their safeguard; capped at lin_tol, and never below what
  // the nonlinear tolerance needs), loose while the linearisation is poor,
  // tight in the quadratic phase (defaults: forcing on, cap 0.3; the 256^3
  // step then takes 9 Newton steps and 13 cycles, against 8 and 19 with a
  // fixed 1e-3).  With clip >= 0 a cell
  // whose H would leave its closure regime stops at the first regime
  // boundary it crosses plus `clip` of its overshoot (lean_step_kernel), so
  // that the next step linearises the new regime instead of extrapolating
  // the old one across the kink (halves the Newton steps of the 256^3
  // backward-Euler step)
  double lin_tol = 0.3;
  int lin_max = 12;
  double clip = 0.1;
  int forcing = 1;
  int lean_vec = 1;  // vector-load half sweeps where a level's rows allow them

  StepClip step_clip() const {
    const ClosureParams cp = make_cp(op.params);
    StepClip K;
    K.CR = (float)cp.CR;
    K.cp = (float)cp.cp;
    K.St = (float)cp.St;
    K.te = (float)cp.te;
    K.Te = (float)cp.Te;
    K.inv_k = (float)(1.0 / cp.k);
    K.inv_CRTe = (float)(1.0 / (cp.CR + cp.Te));
    K.frac = (float)clip;
    K.p = cp;
    K.inv_k64 = 1.0 / cp.k;
    K.inv_CRTe64 = 1.0 / (cp.CR + cp.Te);
    return K;
  }

  // f - N(u) into L[0].g; host_norm[0] = its norm of the options' kind (the
  // stopping test), host_norm[1] = its L2 norm (the merit of the step
  // halving: a max norm would halve every cell's step for the one cell that
  // crosses a closure regime boundary)
  int nl_residual() {
    const long long n2 = 2 * L[0].G.ncell;
    int nparts = 0;
    // the closure once per cell into the cache (t_cl, or t_cl_lean on the
    // lean paths), then the stencil over it (with t_cl bitwise the residual
    // that evaluates the closure at every stencil point) with its L2 norm and,
    // for a max-norm stopping test, its max norm in the same pass
    const NLArgs<double> N = make_nl_args<double>(op);
    const bool both = o.norm_type == MLGPU_NORM_MAX;
    const bool lean = mixed || fast64;
    CK(launch_nlc_closure(N, L[0].u, ntcl, s, lean));
    if (lean && both)
      CK(launch_nlc_res_lean(N, L[0].u, ntcl, nsb, nf, L[0].g, part, part2, &nparts, s));
    else
      CK(launch_nlc_op(N, NL_RESIDUAL, MLGPU_NORM_L2, L[0].u, ntcl, nf, L[0].g, nullptr, part,
                       &nparts, s, both ? part2 : nullptr));
    CK(launch_finalize_norm(MLGPU_NORM_L2, part, nparts, part + kMaxBlocks, s));
    if (both) {
      CK(launch_finalize_norm(MLGPU_NORM_MAX, part2, nparts, part + kMaxBlocks + 1, s));
    } else {
      CK(launch_norm_partial<double>(n2, L[0].g, o.norm_type, part, &nparts, s));
      CK(launch_finalize_norm(o.norm_type, part, nparts, part + kMaxBlocks + 1, s));
    }
    CK(cudaMemcpyAsync(host_norm, part + kMaxBlocks, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                       s));
    CK(cudaStreamSynchronize(s));
    std::swap(host_norm[0], host_norm[1]);
    return MLGPU_OK;
  }

  // the cycles run on A for the duration of a Newton solve, on A^T otherwise
  // (also after an error return)
  struct ForwardMode {
    bool &tr;
    explicit ForwardMode(bool &t) : tr(t) { tr = false; }
    ~ForwardMode() { tr = true; }
  };

  int newton(double *user_u, const double *user_f, mlgpu_solve_stats *st) {
    ForwardMode mode(tr);
    const long long n2 = 2 * L[0].G.ncell;
    const size_t bytes = sizeof(double) * n2;
    cudaGetLastError();
    if (enter()) return MLGPU_ERR_CUDA;
    CK(cudaMemcpyAsync(L[0].u, user_u, bytes, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(nf, user_f, bytes, cudaMemcpyDeviceToDevice, s));
    if (nk_state < 0) {
      nk_state = count_kernels([&] { return state_levels(); });
      nk_iter = count_kernels([&] { return iteration(); });
    }
    int rc = nl_residual();
    if (rc) return rc;
    Outer S;
    S.norm0 = S.norm = S.prev = *host_norm;
    stats_begin(st, (int)L.size(), S.norm0);
    st->cell_updates = (double)L[0].G.ncell;
    st->kernel_launches = nl_residual_kernels();
    if (!std::isfinite(S.norm0)) S.status = 8;
    int stall = 0;  // consecutive steps that cut the residual by under 5%
    double merit = host_norm[1];
    double eta = lin_tol;
    while (outer_continue(o, S)) {
      rc = state_levels();
      if (rc) return rc;
      // linear solve A d = r, d in L[0].y (FP64) or L[0].y32 (mixed) from
      // zero: its starting residual is r itself, whose norm the nonlinear
      // residual just gave (the options' norm kind: the linear test's)
      if (mixed) {
        CK(launch_lean_pack<float, double>(L[0].G, split(0), 2, L[0].g, L[0].g32, s));
        CK(cudaMemsetAsync(L[0].y32, 0, sizeof(float) * n2, s));
        CK(cudaMemsetAsync(L[0].w32, 0, sizeof(float) * n2, s));
      } else if (fast64) {
        CK(launch_lean_pack<double, double>(L[0].G, split(0), 2, L[0].g, L[0].g64s, s));
        CK(cudaMemsetAsync(L[0].y, 0, bytes, s));
        CK(cudaMemsetAsync(L[0].w64, 0, bytes, s));
      } else {
        CK(cudaMemsetAsync(L[0].y, 0, bytes, s));
      }
      st->kernel_launches += nk_state + (mixed || fast64 ? 1 : 0);
      const double l0 = S.norm;
      *host_norm = l0;
      for (int c = 0; c < lin_max && *host_norm > eta * l0; c++) {
        rc = run_iteration();
        if (rc) return rc;
        CK(cudaStreamSynchronize(s));
        st->cycles += 1;
        st->cell_updates += updates_per_iter;
        st->kernel_launches += nk_iter;
      }
      CK(cudaMemcpyAsync(nuold, L[0].u, bytes, cudaMemcpyDeviceToDevice, s));
      double scale = 1.0;
      const StepClip K = step_clip();
      const StepClip *kp = clip >= 0 ? &K : nullptr;
      for (int h = 0; h <= 4; h++) {
        // u = u_old + scale d (d split on the lean paths' smoothed level 0)
        if (mixed)
          CK(launch_lean_step<float>(L[0].G, split(0), kp, L[0].u, nuold, scale, L[0].y32, s));
        else
          CK(launch_lean_step<double>(L[0].G, fast64 ? split(0) : 0, kp, L[0].u, nuold, scale,
                                      L[0].y, s));
        rc = nl_residual();
        if (rc) return rc;
        st->cell_updates += (double)L[0].G.ncell;
        st->kernel_launches += kStepKernels + nl_residual_kernels();
        if (std::isfinite(host_norm[1]) && host_norm[1] <= merit) break;
        scale *= 0.5;
      }
      const double merit_prev = merit;
      merit = host_norm[1];
      S.norm = host_norm[0];
      stall = S.norm >= 0.95 * S.prev ? stall + 1 : 0;
      // as outer_after, with the stagnation test on the L2 merit (the max
      // norm may rise while the step is accepted)
      S.iter++;
      if (S.iter < 64) st->norm_history[S.iter] = S.norm;
      if (!std::isfinite(S.norm) || !std::isfinite(merit))
        S.status = 8;
      else if (merit > (1.0 - o.hang) * merit_prev && S.norm > o.tolerance * S.norm0)
        S.status = 2;
      if (forcing && S.prev > 0 && std::isfinite(S.norm)) {
        const double ratio = S.norm / S.prev;
        double e = 0.9 * ratio * ratio;
        const double guard = 0.9 * eta * eta;
        if (guard > 0.1) e = std::max(e, guard);
        e = std::min(e, lin_tol);
        const double fin = 0.5 * o.tolerance * S.norm0 / S.norm;
        eta = std::min(lin_tol, std::max(e, fin));
        // a converging step whose forcing would stop just short of the
        // tolerance: force down to the one that ends the solve when that
        // costs at most a tenth more reduction (about one more cycle) --
        // a whole Newton iteration less
        if (ratio < 0.1 && fin < eta && fin >= 0.1 * eta) eta = fin;
      }
      S.prev = S.norm;
      // three stalled steps far below the start: the FP64 residual has
      // reached its round-off floor (stalls of the damped early steps, where
      // the closure's regime switches cut the step, do not count)
      if (stall >= 3 && S.norm < 1e-8 * S.norm0 && S.status == 0) S.status = 2;
    }
    CK(cudaMemcpyAsync(user_u, L[0].u, bytes, cudaMemcpyDeviceToDevice, s));
    CK(cudaStreamSynchronize(s));
    if (leave()) return MLGPU_ERR_CUDA;
    return outer_finish(o, S, st);
  }

  // Device time of the lean red/black half sweep on the finest level, at the
  // state and right-hand side of the last mixed-precision Newton step: `reps`
  // launches, passes alternating, between two events on the solver's stream
  // (y and w of the finest level are scratch between Newton steps).  `kind`
  // 0 is the only kind; the finest level must be a smoothed one.
  int time_lean_sweep(int kind, int reps, double *ms_per_launch) {
    if (!mixed || reps < 1 || !ms_per_launch || kind != 0 || !split(0)) return MLGPU_ERR_ARG;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaGetLastError();
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
      if (e0) cudaEventDestroy(e0);
      return MLGPU_ERR_CUDA;
    }
    int rc = enter();
    const LinLean P = lean(0);
    auto one = [&](int i) { return launch_lean_gsrb(P, i & 1, s, lean_vec); };
    if (!rc && one(0) != cudaSuccess) rc = MLGPU_ERR_CUDA;  // warm
    if (!rc && cudaEventRecord(e0, s) != cudaSuccess) rc = MLGPU_ERR_CUDA;
    for (int i = 0; i < reps && !rc; i++)
      if (one(i + 1) != cudaSuccess) rc = MLGPU_ERR_CUDA;
    if (!rc && cudaEventRecord(e1, s) != cudaSuccess) rc = MLGPU_ERR_CUDA;
    float ms = 0.f;
    if (!rc && (cudaEventSynchronize(e1) != cudaSuccess ||
                cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
      rc = MLGPU_ERR_CUDA;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (leave()) rc = MLGPU_ERR_CUDA;
    if (!rc) *ms_per_launch = (double)ms / reps;
    return rc;
  }

  // A^T y = g at the state already set; y, g device arrays of the caller
  int solve_at_state(double *user_y, const double *user_g, mlgpu_solve_stats *st) {
    size_t bytes = sizeof(double) * 2 * L[0].G.ncell;
    CK(cudaMemcpyAsync(L[0].y, user_y, bytes, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(L[0].g, user_g, bytes, cudaMemcpyDeviceToDevice, s));
    if (kern_iter < 0) {
      kern_init = count_kernels([&] { return residual_norm(); });
      kern_iter = count_kernels([&] { return iteration(); });
    }
    int rc = residual_norm();
    if (rc) return rc;
    CK(cudaStreamSynchronize(s));
    Outer S;
    S.norm0 = S.norm = S.prev = *host_norm;
    stats_begin(st, (int)L.size(), S.norm0);
    st->cell_updates = (double)L[0].G.ncell;
    st->kernel_launches = kern_init;
    if (!std::isfinite(S.norm0)) S.status = 8;
    while (outer_continue(o, S)) {
      rc = run_iteration();
      if (rc) return rc;
      CK(cudaStreamSynchronize(s));
      S.norm = *host_norm;
      st->cycles += 1;
      st->cell_updates += updates_per_iter;
      st->kernel_launches += kern_iter;
      outer_after(o, S, st);
    }
    CK(cudaMemcpyAsync(user_y, L[0].y, bytes, cudaMemcpyDeviceToDevice, s));
    CK(cudaStreamSynchronize(s));
    return outer_finish(o, S, st);
  }

  int adjoint_solve(const double *phi, const double *g, double *y, mlgpu_solve_stats *st) {
    cudaGetLastError();
    if (enter()) return MLGPU_ERR_CUDA;
    int rc = set_state(phi);
    if (rc) return rc;
    rc = solve_at_state(y, g, st);
    if (leave()) return MLGPU_ERR_CUDA;
    return rc;
  }

  // gradient of -y^T N with respect to the wall values at the current state
  int bc_gradient(const double *y, double grad[12]) {
    cudaGetLastError();
    if (enter()) return MLGPU_ERR_CUDA;
    CK(launch_adj_bc_grad(args(0), y, bcg, s));
    CK(cudaMemcpyAsync(grad, bcg, 12 * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (leave()) return MLGPU_ERR_CUDA;
    return MLGPU_OK;
  }

  // the base-class solve: A^T y = g at the state of the last adjoint solve
  int solve(double *y, const double *g, mlgpu_solve_stats *st) override {
    if (!y || !g || !st) return MLGPU_ERR_ARG;
    cudaGetLastError();
    if (enter()) return MLGPU_ERR_CUDA;
    int rc = solve_at_state(y, g, st);
    if (leave()) return MLGPU_ERR_CUDA;
    return rc;
  }

  int set_alpha_beta(double a, double b) override {
    op.alpha = a;
    op.beta = b;
    for (auto *gp : {&graph, &graph_lin, &graph_lin32})
      if (*gp) {
        cudaGraphExecDestroy(*gp);
        *gp = nullptr;
      }
    return MLGPU_OK;
  }

  int set_bcs(const mlgpu_bc *phi_bc, const mlgpu_bc *derived_bc) {
    mlgpu_nlop t = op;
    if (phi_bc) t.phi_bc = *phi_bc;
    if (derived_bc) t.derived_bc = *derived_bc;
    if (!valid_adjoint_op(&t)) return MLGPU_ERR_ARG;
    op = t;
    return set_alpha_beta(op.alpha, op.beta);
  }
};

bool valid_options(const mlgpu_mg_options *o) {
  if (!o) return false;
  if (o->num_smooth_down < 0 || o->num_smooth_up < 0 || o->num_mg < 1 || o->max_iter < 0)
    return false;
  if (o->relax_mode != MLGPU_RELAX_GSRB && o->relax_mode != MLGPU_RELAX_JACOBI) return false;
  if (o->bottom_max_iter < 0 || o->max_coarse < 1) return false;
  if (o->bottom_solver != MLGPU_BOTTOM_RELAX && o->bottom_solver != MLGPU_BOTTOM_BICGSTAB)
    return false;
  if (o->prolong != MLGPU_PROLONG_CONSTANT && o->prolong != MLGPU_PROLONG_LINEAR) return false;
  if (o->precision != MLGPU_PREC_F64 && o->precision != MLGPU_PREC_MIXED) return false;
  if (o->norm_type < MLGPU_NORM_MAX || o->norm_type > MLGPU_NORM_L2) return false;
  return true;
}

}  // namespace

extern "C" {

void mlgpu_mg_default_options(mlgpu_mg_options *o, int hc) {
  if (!o) return;
  memset(o, 0, sizeof(*o));
  // HCMultigrid defaults (srcSubcycle/MushyLayerSubcycleUtils.cpp:668-678)
  // or projection defaults (srcSubcycle/Projector.cpp:44-64)
  o->num_smooth_down = hc ? 1 : 2;
  o->num_smooth_up = 4;
  o->num_mg = 1;
  o->max_iter = hc ? 10 : 20;
  o->tolerance = hc ? 1e-10 : 1e-15;
  o->hang = hc ? 1e-10 : 1e-15;
  o->norm_thresh = hc ? 1e-10 : 1e-30;
  o->relax_mode = MLGPU_RELAX_GSRB;
  o->bottom_solver = MLGPU_BOTTOM_RELAX;
  o->bottom_max_iter = hc ? 40 : 20;
  o->max_coarse = 2;
  o->prolong = hc ? MLGPU_PROLONG_LINEAR : MLGPU_PROLONG_CONSTANT;
  o->precision = MLGPU_PREC_F64;
  o->inner_cycles = 0;
  o->norm_type = MLGPU_NORM_MAX;
  o->use_graph = 2;
  o->fuse_levels = 1;
}

int mlgpu_vc_solver_workspace(const mlgpu_vcop *op, const mlgpu_mg_options *o, size_t *bytes) {
  if (!op || !valid_grid(&op->grid) || !valid_options(o) || !bytes) return MLGPU_ERR_ARG;
  if (!valid_bc(op->bc, op->grid.dim, false)) return MLGPU_ERR_ARG;
  VCSolver S;
  S.op = *op;
  S.o = *o;
  S.mixed = o->precision == MLGPU_PREC_MIXED;
  *bytes = S.layout(nullptr);
  return MLGPU_OK;
}

int mlgpu_vc_solver_create(const mlgpu_vcop *op, const mlgpu_mg_options *o, void *ws,
                           size_t bytes, void *stream, mlgpu_solver **out) {
  if (!op || !valid_grid(&op->grid) || !valid_options(o) || !ws || !out) return MLGPU_ERR_ARG;
  if (op->dtype != MLGPU_F64 || !valid_bc(op->bc, op->grid.dim, false)) return MLGPU_ERR_ARG;
  for (int d = 0; d < op->grid.dim; d++)
    if (!op->bCoef[d]) return MLGPU_ERR_ARG;
  if (((uintptr_t)ws) & 255) return MLGPU_ERR_WORKSPACE;
  VCSolver *S = new VCSolver;
  S->op = *op;
  S->o = *o;
  S->mixed = o->precision == MLGPU_PREC_MIXED;
  cudaGetLastError();
  if (S->init_streams((cudaStream_t)stream)) {
    delete S;
    return MLGPU_ERR_CUDA;
  }
  size_t need = S->layout(nullptr);
  if (bytes < need) {
    delete S;
    return MLGPU_ERR_WORKSPACE;
  }
  S->layout((char *)ws);
  if (cudaHostAlloc((void **)&S->host_norm, sizeof(double), cudaHostAllocDefault) != cudaSuccess ||
      cudaHostAlloc((void **)&S->host_state, sizeof(OuterDev), cudaHostAllocDefault) != cudaSuccess) {
    delete S;
    return MLGPU_ERR_CUDA;
  }
  int rc = S->enter();
  // norm partials and the finished-block counter of the fused outer step
  if (!rc && cudaMemsetAsync(S->part, 0, kNormScratchDoubles * sizeof(double), S->s) != cudaSuccess)
    rc = MLGPU_ERR_CUDA;
  if (!rc) rc = S->build_coefs();
  if (!rc) rc = S->leave();
  if (rc) {
    delete S;
    return rc;
  }
  *out = S;
  return MLGPU_OK;
}

int mlgpu_hc_solver_workspace(const mlgpu_nlop *op, const mlgpu_mg_options *o, size_t *bytes) {
  if (!op || !valid_grid(&op->grid) || !valid_options(o) || !bytes) return MLGPU_ERR_ARG;
  // the FAS bottom solve is relaxation (the reference's HC default)
  if (!valid_nl_bcs(*op) || o->bottom_solver != MLGPU_BOTTOM_RELAX) return MLGPU_ERR_ARG;
  HCSolver S;
  S.op = *op;
  S.o = *o;
  S.mixed = o->precision == MLGPU_PREC_MIXED;
  *bytes = S.layout(nullptr);
  return MLGPU_OK;
}

int mlgpu_hc_solver_create(const mlgpu_nlop *op, const mlgpu_mg_options *o, void *ws,
                           size_t bytes, void *stream, mlgpu_solver **out) {
  if (!op || !valid_grid(&op->grid) || !valid_options(o) || !ws || !out) return MLGPU_ERR_ARG;
  if (o->bottom_solver != MLGPU_BOTTOM_RELAX) return MLGPU_ERR_ARG;
  if (op->dtype != MLGPU_F64 || !valid_nl_bcs(*op)) return MLGPU_ERR_ARG;
  // mixed precision needs red/black smoothing (the linearised cycles)
  if (o->precision == MLGPU_PREC_MIXED && o->relax_mode != MLGPU_RELAX_GSRB) return MLGPU_ERR_ARG;
  for (int d = 0; d < op->grid.dim; d++)
    if (!op->bCoef[d]) return MLGPU_ERR_ARG;
  if (((uintptr_t)ws) & 255) return MLGPU_ERR_WORKSPACE;
  HCSolver *S = new HCSolver;
  S->op = *op;
  // the temperature conditions keep the finest spacing on every level
  if (!(S->op.nlbc.dx > 0)) S->op.nlbc.dx = op->grid.dx;
  S->o = *o;
  S->mixed = o->precision == MLGPU_PREC_MIXED;
  cudaGetLastError();
  if (S->init_streams((cudaStream_t)stream)) {
    delete S;
    return MLGPU_ERR_CUDA;
  }
  size_t need = S->layout(nullptr);
  if (bytes < need) {
    delete S;
    return MLGPU_ERR_WORKSPACE;
  }
  S->layout((char *)ws);
  if (cudaHostAlloc((void **)&S->host_norm, sizeof(double), cudaHostAllocDefault) != cudaSuccess) {
    delete S;
    return MLGPU_ERR_CUDA;
  }
  int rc = S->enter();
  if (!rc) rc = S->build_coefs();
  if (!rc) rc = S->leave();
  if (rc) {
    delete S;
    return rc;
  }
  *out = S;
  return MLGPU_OK;
}

int mlgpu_solver_solve(mlgpu_solver *s, double *phi, const double *rhs, mlgpu_solve_stats *st) {
  if (!s) return MLGPU_ERR_ARG;
  return s->solve(phi, rhs, st);
}

int mlgpu_solver_set_alpha_beta(mlgpu_solver *s, double a, double b) {
  if (!s) return MLGPU_ERR_ARG;
  return s->set_alpha_beta(a, b);
}

int mlgpu_hc_solver_set_bcs(mlgpu_solver *S, const mlgpu_bc *phi_bc, const mlgpu_bc *derived_bc) {
  if (HCSolver *H = dynamic_cast<HCSolver *>(S)) return H->set_bcs(phi_bc, derived_bc);
  if (HCAdjSolver *A = dynamic_cast<HCAdjSolver *>(S)) return A->set_bcs(phi_bc, derived_bc);
  return MLGPU_ERR_ARG;
}

int mlgpu_mac_project(mlgpu_solver *S, const mlgpu_grid *grid, const mlgpu_bc *phi_bc,
                      double *u[3], const double *pi_face[3], double *phi, double *scratch,
                      mlgpu_solve_stats *stats) {
  if (!S || !valid_grid(grid) || !phi_bc || !u || !phi || !scratch || !stats)
    return MLGPU_ERR_ARG;
  if (!valid_bc(*phi_bc, grid->dim, false)) return MLGPU_ERR_ARG;
  VCSolver *V = dynamic_cast<VCSolver *>(S);
  if (!V) return MLGPU_ERR_ARG;
  for (int d = 0; d < 3; d++)
    if (grid->n[d] != V->op.grid.n[d]) return MLGPU_ERR_ARG;
  for (int d = 0; d < grid->dim; d++)
    if (!u[d]) return MLGPU_ERR_ARG;
  Geom G = make_geom(*grid);
  cudaGetLastError();
  if (S->enter()) return MLGPU_ERR_CUDA;
  CK(launch_mac_div(G, u[0], u[1], grid->dim == 3 ? u[2] : nullptr, scratch, S->s));
  int rc = S->solve(phi, scratch, stats);
  if (rc != MLGPU_OK && rc != MLGPU_ERR_NOT_CONVERGED && rc != MLGPU_ERR_HANG) return rc;
  BCD b = make_bcd(*phi_bc);
  for (int d = 0; d < grid->dim; d++)
    CK(launch_mac_correct(G, b, d, phi, pi_face ? pi_face[d] : nullptr, u[d], S->s));
  if (S->leave()) return MLGPU_ERR_CUDA;
  return rc;
}

int mlgpu_hc_backward_euler(mlgpu_solver *S, double *phi_new, const double *phi_old,
                            const double *src, const double *aCoef, double dt,
                            double *rhs_scratch, mlgpu_solve_stats *stats) {
  if (!S || !phi_new || !phi_old || !rhs_scratch || !stats || !(dt > 0)) return MLGPU_ERR_ARG;
  HCSolver *H = dynamic_cast<HCSolver *>(S);
  if (!H) return MLGPU_ERR_ARG;
  long long n = 2 * H->L[0].G.ncell;
  if (H->op.alpha != 1.0 || H->op.beta != -dt) {
    int rc = S->set_alpha_beta(1.0, -dt);
    if (rc) return rc;
  }
  cudaGetLastError();
  if (S->enter()) return MLGPU_ERR_CUDA;
  CK(launch_be_rhs(n, phi_old, aCoef, src, dt, rhs_scratch, S->s));
  return S->solve(phi_new, rhs_scratch, stats);
}

// The TGA scheme's constants (Twizell, Gumel & Arigu, "Second-order,
// L0-stable methods for the heat equation with time-dependent boundary
// conditions", 1996, in the form Chombo's LevelTGA drives): a = 2 - sqrt(2)
// - eps, mu1,2 = (a -+ sqrt(a^2 - 4a + 2)) / 2, mu3 = 1 - a (the source
// weight mu4 = 1/2 - a is not used: the source enters as dt src)
void tga_constants(double mu[3]) {
  const double a = 2.0 - std::sqrt(2.0) - 1e-12;
  const double d = std::sqrt(a * a - 4.0 * a + 2.0);
  mu[0] = 0.5 * (a - d);
  mu[1] = 0.5 * (a + d);
  mu[2] = 1.0 - a;
}

}  // extern "C"

// The TGA step on solver X (HCSolver: FAS solves; HCAdjSolver: Newton solves)
template <class X, class Solve>
static int tga_step(X *H, Solve solve, double *phi_new, const double *phi_old, const double *src,
                    const double *aCoef, double dt, double *scratch, mlgpu_solve_stats *stats) {
  const long long n = 2 * H->L[0].G.ncell;
  double mu[3];
  tga_constants(mu);
  double *R = scratch, *psi = scratch + n;
  cudaGetLastError();
  if (H->enter()) return MLGPU_ERR_CUDA;
  // R = (a + mu3 dt L) phi_old + dt src: the operator with alpha 1, beta
  // mu3 dt applied to phi_old (alpha a phi + beta L, L = -div(b grad f(phi));
  // the solves below take beta -mu dt, as the backward-Euler step takes -dt)
  mlgpu_nlop opR = H->op;
  opR.alpha = 1.0;
  opR.beta = mu[2] * dt;
  CK(launch_nl_op<double>(make_nl_args<double>(opR), NL_APPLY, -1, phi_old, nullptr, R, nullptr,
                          nullptr, nullptr, H->s));
  if (src) CK(launch_add_dt_src(n, R, src, dt, H->s));
  CK(cudaMemcpyAsync(psi, phi_old, sizeof(double) * n, cudaMemcpyDeviceToDevice, H->s));
  if (H->leave()) return MLGPU_ERR_CUDA;
  // (a - mu1 dt L) psi = R, then (a - mu2 dt L) phi_new = a psi
  mlgpu_solve_stats st1;
  int rc = H->set_alpha_beta(1.0, -mu[0] * dt);
  if (rc) return rc;
  rc = solve(psi, R, &st1);
  if (rc != MLGPU_OK && rc != MLGPU_ERR_NOT_CONVERGED && rc != MLGPU_ERR_HANG) return rc;
  if (H->enter()) return MLGPU_ERR_CUDA;
  CK(launch_scale_by_a(n, psi, aCoef, R, H->s));
  CK(cudaMemcpyAsync(phi_new, psi, sizeof(double) * n, cudaMemcpyDeviceToDevice, H->s));
  if (H->leave()) return MLGPU_ERR_CUDA;
  rc = H->set_alpha_beta(1.0, -mu[1] * dt);
  if (rc) return rc;
  const int rc2 = solve(phi_new, R, stats);
  stats->iterations += st1.iterations;
  stats->cycles += st1.cycles;
  stats->cell_updates += st1.cell_updates;
  stats->kernel_launches += st1.kernel_launches;
  if (rc2 == MLGPU_OK) return rc;  // the first solve's status when the second converged
  return rc2;
}

extern "C" {

int mlgpu_hc_tga_step(mlgpu_solver *S, double *phi_new, const double *phi_old,
                      const double *src, const double *aCoef, double dt, double *scratch,
                      mlgpu_solve_stats *stats) {
  if (!S || !phi_new || !phi_old || !scratch || !stats || !(dt > 0)) return MLGPU_ERR_ARG;
  if (HCSolver *H = dynamic_cast<HCSolver *>(S))
    return tga_step(
        H, [H](double *x, const double *r, mlgpu_solve_stats *st) { return H->solve(x, r, st); },
        phi_new, phi_old, src, aCoef, dt, scratch, stats);
  if (HCAdjSolver *A = dynamic_cast<HCAdjSolver *>(S))
    return tga_step(
        A, [A](double *x, const double *r, mlgpu_solve_stats *st) { return A->newton(x, r, st); },
        phi_new, phi_old, src, aCoef, dt, scratch, stats);
  return MLGPU_ERR_ARG;
}

int mlgpu_hc_adjoint_workspace(const mlgpu_nlop *op, const mlgpu_mg_options *o,
                               size_t *bytes) {
  if (!valid_adjoint_op(op) || !valid_options(o) || !bytes) return MLGPU_ERR_ARG;
  if (o->bottom_solver != MLGPU_BOTTOM_RELAX) return MLGPU_ERR_ARG;
  HCAdjSolver S;
  S.op = *op;
  S.o = *o;
  *bytes = S.layout(nullptr);
  return MLGPU_OK;
}

int mlgpu_hc_adjoint_create(const mlgpu_nlop *op, const mlgpu_mg_options *o, void *ws,
                            size_t bytes, void *stream, mlgpu_solver **out) {
  if (!valid_adjoint_op(op) || !valid_options(o) || !ws || !out) return MLGPU_ERR_ARG;
  if (o->bottom_solver != MLGPU_BOTTOM_RELAX) return MLGPU_ERR_ARG;
  if (((uintptr_t)ws) & 255) return MLGPU_ERR_WORKSPACE;
  HCAdjSolver *S = new HCAdjSolver;
  S->op = *op;
  // the mixed temperature condition keeps the finest spacing on every level
  if (!(S->op.nlbc.dx > 0)) S->op.nlbc.dx = op->grid.dx;
  S->o = *o;
  cudaGetLastError();
  if (S->init_streams((cudaStream_t)stream)) {
    delete S;
    return MLGPU_ERR_CUDA;
  }
  size_t need = S->layout(nullptr);
  if (bytes < need) {
    delete S;
    return MLGPU_ERR_WORKSPACE;
  }
  S->layout((char *)ws);
  if (cudaHostAlloc((void **)&S->host_norm, 2 * sizeof(double), cudaHostAllocDefault) != cudaSuccess) {
    delete S;
    return MLGPU_ERR_CUDA;
  }
  int rc = S->enter();
  if (!rc) rc = S->build_coefs();
  if (!rc) rc = S->leave();
  if (rc) {
    delete S;
    return rc;
  }
  *out = S;
  return MLGPU_OK;
}

int mlgpu_hc_adjoint_solve(mlgpu_solver *S, const double *phi, const double *g, double *y,
                           mlgpu_solve_stats *stats) {
  HCAdjSolver *A = dynamic_cast<HCAdjSolver *>(S);
  if (!A || !phi || !g || !y || !stats) return MLGPU_ERR_ARG;
  return A->adjoint_solve(phi, g, y, stats);
}

int mlgpu_hc_newton_solve(mlgpu_solver *S, double *phi, const double *rhs,
                          mlgpu_solve_stats *stats) {
  HCAdjSolver *A = dynamic_cast<HCAdjSolver *>(S);
  if (!A || !phi || !rhs || !stats) return MLGPU_ERR_ARG;
  return A->newton(phi, rhs, stats);
}

int mlgpu_hc_backward_euler_newton(mlgpu_solver *S, double *phi_new, const double *phi_old,
                                   const double *src, const double *aCoef, double dt,
                                   double *rhs_scratch, mlgpu_solve_stats *stats) {
  HCAdjSolver *A = dynamic_cast<HCAdjSolver *>(S);
  if (!A || !phi_new || !phi_old || !rhs_scratch || !stats || !(dt > 0)) return MLGPU_ERR_ARG;
  if (A->op.alpha != 1.0 || A->op.beta != -dt) A->set_alpha_beta(1.0, -dt);
  cudaGetLastError();
  if (A->enter()) return MLGPU_ERR_CUDA;
  CK(launch_be_rhs(2 * A->L[0].G.ncell, phi_old, aCoef, src, dt, rhs_scratch, A->s));
  if (A->leave()) return MLGPU_ERR_CUDA;
  return A->newton(phi_new, rhs_scratch, stats);
}

int mlgpu_hc_newton_params(mlgpu_solver *S, double lin_tol, int lin_max, double clip,
                           int forcing, int vector_sweeps) {
  HCAdjSolver *A = dynamic_cast<HCAdjSolver *>(S);
  if (!A || !(lin_tol > 0.0 && lin_tol < 1.0) || lin_max < 1 || !(clip < 0.0 || clip <= 1.0) ||
      (forcing != 0 && forcing != 1) || (vector_sweeps != 0 && vector_sweeps != 1))
    return MLGPU_ERR_ARG;
  if (A->lean_vec != vector_sweeps) {  // the captured cycles name the kernel
    for (auto *gp : {&A->graph, &A->graph_lin, &A->graph_lin32})
      if (*gp) {
        cudaGraphExecDestroy(*gp);
        *gp = nullptr;
      }
    A->nk_iter = -1;
    A->nk_state = -1;
  }
  A->lin_tol = lin_tol;
  A->lin_max = lin_max;
  A->forcing = forcing;
  A->lean_vec = vector_sweeps;
  A->clip = clip < 0.0 ? -1.0 : clip;
  return MLGPU_OK;
}

int mlgpu_hc_newton_sweep_time(mlgpu_solver *S, int kind, int reps, double *ms_per_launch) {
  HCAdjSolver *A = dynamic_cast<HCAdjSolver *>(S);
  if (!A) return MLGPU_ERR_ARG;
  return A->time_lean_sweep(kind, reps, ms_per_launch);
}

int mlgpu_hc_adjoint_bc_gradient(mlgpu_solver *S, const double *y, double grad[12]) {
  HCAdjSolver *A = dynamic_cast<HCAdjSolver *>(S);
  if (!A || !y || !grad) return MLGPU_ERR_ARG;
  return A->bc_gradient(y, grad);
}

int mlgpu_hc_backward_euler_adjoint(mlgpu_solver *S, const double *phi_new,
                                    const double *phi_new_bar, const double *aCoef, double dt,
                                    double *mu, double *phi_old_bar, double *src_bar,
                                    double bc_grad[12], mlgpu_solve_stats *stats) {
  HCAdjSolver *A = dynamic_cast<HCAdjSolver *>(S);
  if (!A || !phi_new || !phi_new_bar || !mu || !stats || !(dt > 0)) return MLGPU_ERR_ARG;
  if (A->op.alpha != 1.0 || A->op.beta != -dt) A->set_alpha_beta(1.0, -dt);
  int rc = A->adjoint_solve(phi_new, phi_new_bar, mu, stats);
  if (rc != MLGPU_OK && rc != MLGPU_ERR_NOT_CONVERGED && rc != MLGPU_ERR_HANG) return rc;
  cudaGetLastError();
  if (A->enter()) return MLGPU_ERR_CUDA;
  if (phi_old_bar || src_bar)
    CK(launch_be_adj(2 * A->L[0].G.ncell, mu, aCoef, dt, phi_old_bar, src_bar, A->s));
  if (A->leave()) return MLGPU_ERR_CUDA;
  if (bc_grad) {
    int rc2 = A->bc_gradient(mu, bc_grad);
    if (rc2) return rc2;
  }
  return rc;
}

int mlgpu_mac_project_adjoint(mlgpu_solver *S, const mlgpu_grid *grid, const mlgpu_bc *phi_bc,
                              const double *ubar[3], const double *pi_face[3],
                              const double *p, double *ustar_bar[3], double *pi_bar[3],
                              double *q, double *scratch, mlgpu_solve_stats *stats) {
  if (!S || !valid_grid(grid) || !phi_bc || !ubar || !ustar_bar || !q || !scratch || !stats)
    return MLGPU_ERR_ARG;
  if (!valid_bc(*phi_bc, grid->dim, false)) return MLGPU_ERR_ARG;
  if (pi_bar && !p) return MLGPU_ERR_ARG;
  VCSolver *V = dynamic_cast<VCSolver *>(S);
  if (!V) return MLGPU_ERR_ARG;
  for (int d = 0; d < 3; d++)
    if (grid->n[d] != V->op.grid.n[d]) return MLGPU_ERR_ARG;
  for (int d = 0; d < grid->dim; d++)
    if (!ubar[d] || !ustar_bar[d]) return MLGPU_ERR_ARG;
  Geom G = make_geom(*grid);
  BCD b = make_bcd(*phi_bc);
  const double *y[3] = {ubar[0], ubar[1], grid->dim == 3 ? ubar[2] : nullptr};
  const double *sc[3] = {nullptr, nullptr, nullptr};
  if (pi_face)
    for (int d = 0; d < grid->dim; d++) sc[d] = pi_face[d];
  cudaGetLastError();
  if (S->enter()) return MLGPU_ERR_CUDA;
  CK(launch_mac_grad_t(G, b, y, sc, scratch, S->s));
  int rc = S->solve(q, scratch, stats);
  if (rc != MLGPU_OK && rc != MLGPU_ERR_NOT_CONVERGED && rc != MLGPU_ERR_HANG) return rc;
  for (int d = 0; d < grid->dim; d++) {
    CK(launch_mac_div_t(G, d, q, ubar[d], ustar_bar[d], S->s));
    if (pi_bar && pi_bar[d]) CK(launch_mac_pi_bar(G, b, d, p, ustar_bar[d], pi_bar[d], S->s));
  }
  if (S->leave()) return MLGPU_ERR_CUDA;
  return rc;
}

int mlgpu_solver_destroy(mlgpu_solver *s) {
  delete s;
  return MLGPU_OK;
}

}  // extern "C"
