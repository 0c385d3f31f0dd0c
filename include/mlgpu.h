/*
 * mlgpu.h -- C ABI of the GB300 (sm_103a) elliptic/closure hot path of the
 * mushy-layer solidification code.
 *
 * Everything here is plain C: device pointers, extents, POD parameter structs
 * and a cudaStream_t passed as `void*`.  No allocation happens inside any
 * entry point except where a function says so; multigrid hierarchies live in
 * a caller-provided workspace.
 *
 * Data layout (one uniform box per level, no ghost cells stored):
 *   cell field  [comp][k][j][i]            i fastest, n[0] x n[1] x n[2] cells
 *   face field  b_d[comp][k][j][i]         direction d has n[d]+1 faces,
 *                                          the other directions n cells
 * Ghost values required by the 5/7-point stencils are produced in registers
 * from the adjacent interior cell according to `mlgpu_bc` (first-order
 * Dirichlet: ghost = 2v - interior; Neumann: ghost = interior + s*dx*g) or by
 * periodic wrap.  That is exactly what a one-ghost-cell fill followed by the
 * stencil computes in the reference, without the fill pass.
 *
 * Return codes: every entry point returns MLGPU_OK (0) or one of the codes
 * below; nothing aborts the process and no kernel traps.
 */
#ifndef MLGPU_H_
#define MLGPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define MLGPU_OK 0
#define MLGPU_ERR_ARG 1           /* bad extents, null pointer, unsupported option */
#define MLGPU_ERR_CUDA 2          /* a CUDA runtime call failed */
#define MLGPU_ERR_NAN 3           /* NaN or Inf found by a fused norm */
#define MLGPU_ERR_NOT_CONVERGED 4 /* iteration limit reached above tolerance */
#define MLGPU_ERR_WORKSPACE 5     /* workspace too small or misaligned */
#define MLGPU_ERR_HANG 6          /* solver stopped reducing the residual */
#define MLGPU_ERR_SCRATCH 7       /* request exceeds a fixed-size scratch area */

/* ---------------------------------------------------------------- types */
enum { MLGPU_F64 = 0, MLGPU_F32 = 1 };
enum { MLGPU_BC_NEUMANN = 0, MLGPU_BC_DIRICHLET = 1 };
/* Temperature conditions applied to the enthalpy ghost cells of the (H, C)
 * operator (PhysBCUtil::FixedTemperature, TemperatureFlux,
 * TemperatureFluxRadiation; BCutil/PhysBCUtil.cpp:590-722): the ghost
 * enthalpy is solved so that the ghost temperature meets the Robin condition
 * a (T_g - T_i)/dx = F + b (T_b - T_ref), T_b = (T_g + T_i)/2, on each side
 * (NonlinearTemperatureBCRobin's predicted ghost temperature; see mlgpu_nlbc).  Only phi_bc comp 0 (H) of a
 * nonlinear operator may use them (the reference stops with "Can't apply
 * temperature bcs to bulk concentration"); elsewhere they are MLGPU_ERR_ARG. */
enum {
  MLGPU_BC_FIXED_TEMPERATURE = 2,         /* value = T on the boundary */
  MLGPU_BC_TEMPERATURE_FLUX = 3,          /* value = F (a = 1, b = 0) */
  MLGPU_BC_TEMPERATURE_FLUX_RADIATION = 4 /* value = F, a, b, T_ref from mlgpu_nlbc */
};
/* PhysBCUtil::MixedBCTemperatureSalinity (BCutil/PhysBCUtil.cpp:764-800) on
 * the derived (T, C_l) state: a linear Robin ghost temperature
 *   T_g = (T_i (a/dx + b/2) + F - b T_ref) / (a/dx - b/2),
 * value = F, a, b, T_ref from mlgpu_nlbc's [dir][side] entries and dx its
 * spacing (0: the grid's), the same constants as the radiation condition.
 * Only derived_bc comp 0 (T) may use it; C_l's ghost follows comp 1's own
 * type (the reference writes a zero-gradient C_l ghost, which comp 1's
 * condition then overwrites).  a/dx - b/2 must be nonzero.  In linearised
 * (Newton, adjoint) use the ghost's derivative (a/dx + b/2) / (a/dx - b/2)
 * multiplies the interior value, and the boundary-value gradient is taken
 * with respect to F. */
enum { MLGPU_BC_MIXED_TEMPERATURE_SALINITY = 5 };
enum { MLGPU_NLBC_PICARD = 0, MLGPU_NLBC_NEWTON = 1 };
enum { MLGPU_RELAX_GSRB = 1, MLGPU_RELAX_JACOBI = 4 };     /* reference s_relaxMode */
enum { MLGPU_PROLONG_CONSTANT = 0, MLGPU_PROLONG_LINEAR = 1 };
enum { MLGPU_BOTTOM_RELAX = 0, MLGPU_BOTTOM_BICGSTAB = 1 };
enum { MLGPU_PREC_F64 = 0, MLGPU_PREC_MIXED = 1 };
enum { MLGPU_NORM_MAX = 0, MLGPU_NORM_L1 = 1, MLGPU_NORM_L2 = 2 };

/* One uniform box: the reference's ProblemDomain + single-box layout. */
typedef struct mlgpu_grid {
  int dim;          /* 2 or 3 */
  int n[3];         /* cells per direction; n[2] == 1 when dim == 2 */
  double dx;        /* isotropic cell size */
  int periodic[3];  /* ProblemDomain::isPeriodic(dir) */
} mlgpu_grid;

/* Physical boundary conditions per [dir][side][comp] for up to 2 components.
 * side 0 = low, 1 = high.  Ignored in periodic directions. */
typedef struct mlgpu_bc {
  int type[3][2][2];
  double value[3][2][2];
} mlgpu_bc;

/* MushyLayerParams fields used by the path (src/MushyLayerParams.h). */
typedef struct mlgpu_params {
  double compositionRatio;       /* CR */
  double waterDistributionCoeff; /* k (partition coefficient) */
  double specificHeatRatio;      /* cp */
  double stefan;                 /* St */
  double thetaEutectic;          /* theta_e */
  double ThetaEutectic;          /* Theta_e */
  double heatConductivityRatio;  /* k_T */
  double heatDiffusionCoeff;     /* D_H */
  double saltDiffusionCoeff;     /* D_C */
  double darcyCoeff;
  double viscosityCoeff;
} mlgpu_params;

/* Parameters of the nonlinear temperature conditions (BCutil/NonlinearBC.H:
 * NonlinearTemperatureBCRobin residual, Picard / Newton ghost solvers;
 * MushyLayerParams max_bc_iter 2, max_bc_residual 1e-5, bc_relax_coeff 0.5). */
typedef struct mlgpu_nlbc {
  double a[3][2], b[3][2], T_ref[3][2];  /* radiation coefficients per [dir][side] */
  double no_flux_limit[3][2];  /* below this position (cell centre along the next
                                  direction) the ghost enthalpy is the interior one */
  int method;                  /* MLGPU_NLBC_PICARD or MLGPU_NLBC_NEWTON */
  int max_iter;                /* max_bc_iter */
  double max_residual;         /* max_bc_residual */
  double relax_coeff;          /* bc_relax_coeff (Picard) */
  double dx;                   /* spacing the condition is built with (PhysBCUtil
                                  m_dx: the AMR level's spacing, also on the
                                  coarser multigrid levels); 0 = the grid's dx */
} mlgpu_nlbc;

/* Nonlinear enthalpy/bulk-concentration operator
 *   L(phi) = alpha a phi - beta div(b grad f(phi)),  phi = (H, C), f = (T, C_l)
 * (AMRNonLinearMultiCompOp).  Coefficient pointers are device pointers in the
 * precision named by `dtype`; aCoef may be NULL meaning aCoef == 1. */
typedef struct mlgpu_nlop {
  mlgpu_grid grid;
  mlgpu_params params;
  mlgpu_bc phi_bc;       /* BC on (H, C): noFluxBC in the reference */
  mlgpu_bc derived_bc;   /* BC on (T, C_l): temperatureLiquidSalinityBC */
  int apply_derived_bc;  /* m_apply_bcs_to_diagnostic_var (default 1) */
  double alpha, beta;
  const void *aCoef;     /* [2][cells] or NULL */
  const void *bCoef[3];  /* [2][faces_d] per direction */
  int dtype;
  mlgpu_nlbc nlbc;       /* used where phi_bc comp 0 has a temperature type or
                            derived_bc comp 0 the mixed temperature condition */
} mlgpu_nlop;

/* Linear variable-coefficient operator for one component
 *   L(phi) = alpha a phi - beta c phi - beta div(b grad phi)
 * with c == NULL giving the VCAMRPoissonOp2/AMRProjectionOp operator and
 * c != NULL the DarcyBrinkmanOp operator. */
typedef struct mlgpu_vcop {
  mlgpu_grid grid;
  mlgpu_bc bc;           /* comp 0 only */
  double alpha, beta;
  const void *aCoef;     /* [cells] or NULL (== 1) */
  const void *cCoef;     /* [cells] or NULL (== 0) */
  const void *bCoef[3];  /* [faces_d] */
  int dtype;
} mlgpu_vcop;

/* Multigrid / FAS solver settings (AMRMultiGrid::setSolverParameters). */
typedef struct mlgpu_mg_options {
  int num_smooth_down;   /* pre-smoothing sweeps */
  int num_smooth_up;     /* post-smoothing sweeps */
  int num_mg;            /* coarse-grid visits per level: 1 = V, 2 = W */
  int max_iter;          /* outer iterations */
  double tolerance;      /* stop when |r| <= tolerance * |r0| */
  double hang;           /* stop when |r| > (1 - hang) * |r_prev| */
  double norm_thresh;    /* stop when |r0| <= norm_thresh */
  int relax_mode;        /* MLGPU_RELAX_GSRB or MLGPU_RELAX_JACOBI */
  int bottom_solver;     /* MLGPU_BOTTOM_RELAX; MLGPU_BOTTOM_BICGSTAB (the role
                            of Chombo's BiCGStabSolver, the projection's and
                            velocity solves' default bottom in the reference,
                            srcSubcycle/Projector.cpp:2976-2986,3012-3020):
                            linear solvers only, one thread block in FP64,
                            bottom_max_iter iterations at most; the FAS and
                            Jacobian solvers refuse it (MLGPU_ERR_ARG) */
  int bottom_max_iter;   /* m_imax of the bottom solver */
  int max_coarse;        /* s_maxCoarse: coarsen while coarsenable(2^d * max_coarse) */
  int prolong;           /* MLGPU_PROLONG_* */
  int precision;         /* MLGPU_PREC_F64 or MLGPU_PREC_MIXED */
  int inner_cycles;      /* V-cycles per outer iteration (FP32 cycles per FP64
                            defect-correction step in mixed precision); 0
                            (default): 3 in mixed precision, 1 in FP64 */
  int norm_type;         /* MLGPU_NORM_MAX (reference default) or L2 */
  int use_graph;         /* 0: plain launches; 1: one outer iteration captured in a
                            CUDA graph and replayed; 2 (default): the whole outer
                            loop as a graph WHILE node, decided on the device
                            (linear solvers; the FAS solver treats 2 as 1) */
  int fuse_levels;       /* 1 (default): the coarse levels run one single-CTA cycle
                            (levels of at most 256 cells; in 2D mixed precision
                            1024) and, in mixed precision, 2D levels above that run
                            FP32 shared-memory tiles (smoothing fused with
                            restriction / prolongation), 3D levels the lean
                            colour-split cycles; 2: FP64 cycles use the tiles (2D)
                            and the lean cycles (3D; the Jacobian solver's Newton
                            cycles too) as well; 0: one launch per smoothing pass /
                            transfer.  FP64 results are the same bits for 0, 1 and
                            for 2 in 2D (the 3D lean FP64 cycles keep the FP64
                            residual and tolerance, not the reference's bits) */
} mlgpu_mg_options;

typedef struct mlgpu_solve_stats {
  int exit_status;       /* 0 converged, 2 hang, 4 max_iter, 8 NaN, 16 a device-side
                            wait ran past its bound (solve returns MLGPU_ERR_CUDA) */
  int iterations;        /* outer iterations done */
  int cycles;            /* V-cycles done (all precisions) */
  int levels;            /* multigrid depth used */
  double initial_norm;
  double final_norm;
  double cell_updates;   /* smoothing sweeps + residual/operator evaluations, in cells */
  double norm_history[64];
  double kernel_launches; /* sm_103a kernels this solve launched (counted from the
                             captured iteration graph; -1 per piece not counted) */
} mlgpu_solve_stats;

typedef struct mlgpu_solver mlgpu_solver;  /* opaque */

/* ------------------------------------------------------------ utilities */
const char *mlgpu_status_string(int status);
int mlgpu_version(void);

/* ------------------------------------------------------------ closure -------
 * Full enthalpy closure H, C -> T, porosity, C_l, C_s and the bounding
 * energies, FP64 on every cell.  Replaces updateEnthalpyVariables
 * (src/phaseDiagram.cpp:92-177) and the Fortran CALCULATE_BOUNDING_ENERGY /
 * CALCULATEPOROSITY / CALCULATECL / CALCULATECS / CALCULATET
 * (src/EnthalpyVariablesF.ChF:13-284, :657-698).
 * HC = [2][cells]; any output pointer may be NULL. */
int mlgpu_closure(const mlgpu_grid *grid, const mlgpu_params *p,
                  const double *HC, double *T, double *porosity, double *Cl,
                  double *Cs, double *Hs, double *He, double *Hl, void *stream);

/* (T, C_l) = f(H, C) on every cell: CALCULATE_T_CL
 * (src/EnthalpyVariablesF.ChF:419-467) preceded by CALCULATE_BOUNDING_ENERGY,
 * i.e. AMRNonLinearMultiCompOp::computeDiffusedVar on valid cells
 * (src/AMRNonLinearMultiCompOp.cpp:57-98). */
int mlgpu_closure_tcl(const mlgpu_grid *grid, const mlgpu_params *p,
                      const double *HC, double *TCl, void *stream);
/* mlgpu_closure_tcl as the lean Newton paths evaluate it (mixed precision and
 * the FP64 comparison path): the divisions by constants as products with
 * their reciprocals, the porosity root's square root and the C_l quotient from
 * FP32 seeds refined in FP64 (Markstein / Karp-Markstein iterations).  Within a
 * few ulps of mlgpu_closure_tcl, not its bit pattern.  No counterpart in the
 * reference. */
int mlgpu_closure_tcl_lean(const mlgpu_grid *grid, const mlgpu_params *p,
                           const double *HC, double *TCl, void *stream);

/* ------------------------------------------------- nonlinear operator --- */
/* Bytes of device scratch the fused norms need (norm_type >= 0 below). */
size_t mlgpu_norm_workspace_bytes(void);

/* res = rhs - L(phi); with norm_type >= 0 also the norm of res (MLGPU_NORM_*)
 * into *norm (host, the call then synchronises `stream`), using `ws` of at
 * least mlgpu_norm_workspace_bytes() bytes.  norm_type < 0: no norm, ws may
 * be NULL.
 * AMRNonLinearMultiCompOp::residualI (src/AMRNonLinearMultiCompOp.cpp:100-166)
 * -> NLVCCOMPUTERES (src/AMRNonLinearMultiCompOpF.ChF:350-434). */
int mlgpu_nl_residual(const mlgpu_nlop *op, void *res, const void *phi,
                      const void *rhs, int norm_type, double *norm, void *ws,
                      size_t ws_bytes, void *stream);

/* lhs = L(phi): applyOpI / applyOpNoBoundary2 (:208-352) -> NLVCCOMPUTEOP
 * (src/AMRNonLinearMultiCompOpF.ChF:233-313). */
int mlgpu_nl_apply(const mlgpu_nlop *op, void *lhs, const void *phi,
                   void *stream);

/* One red (pass 0) or black (pass 1) nonlinear Gauss-Seidel half sweep:
 * levelGSRB (:815-949) -> NONLINEARSMOOTHING (F.ChF:50-198), lambda from
 * resetLambda/SUMFACESNLVC (:540-573, F.ChF:598-625) recomputed inline. */
int mlgpu_nl_gsrb_pass(const mlgpu_nlop *op, void *phi, const void *rhs,
                       int pass, void *stream);

/* n full red+black sweeps (levelGSRB called n times, AMRPoissonOp::relax). */
int mlgpu_nl_relax(const mlgpu_nlop *op, void *phi, const void *rhs,
                   int n_sweeps, void *stream);

/* Weighted Jacobi: phi += 0.5 lambda (rhs - L phi): levelJacobi (:1077-1101).
 * `tmp` is caller scratch of the size of phi. */
int mlgpu_nl_jacobi(const mlgpu_nlop *op, void *phi, const void *rhs,
                    void *tmp, void *stream);

/* lambda = 1 / diag(L): resetLambda (:540-573) as an explicit field. */
int mlgpu_nl_lambda(const mlgpu_nlop *op, void *lambda, void *stream);

/* FAS residual restriction: res_c = avg_{2^D}(rhs - L phi), with res_c fully
 * overwritten.  restrictResidual (:373-451) -> RESTRICTRESNLVC (F.ChF:465-542). */
int mlgpu_nl_restrict_residual(const mlgpu_nlop *op, void *res_coarse,
                               const void *phi, const void *rhs, void *stream);

/* ----------------------------------------------------------- transfers -- */
/* phi_c = avg_{2^D} phi_f for ncomp components (restrictR :492-514 ->
 * RESTRICT F.ChF:555-585; also CoarseAverage for cell coefficients). */
int mlgpu_restrict_average(const mlgpu_grid *fine, int ncomp, int dtype,
                           void *coarse, const void *fine_data, void *stream);

/* phi_f += P e_c.  MLGPU_PROLONG_LINEAR follows the stencil of PROLONG_JP
 * (src/AMRProjectionOpF.ChF:15-78), MLGPU_PROLONG_CONSTANT is piecewise
 * constant injection.  Coarse ghosts use the homogeneous form of `bc`. */
int mlgpu_prolong_increment(const mlgpu_grid *fine, const mlgpu_bc *bc,
                            int ncomp, int dtype, int kind, void *fine_data,
                            const void *coarse, void *stream);

/* Face coefficient coarsening (CoarseAverageFace, arithmetic): each coarse
 * face is the mean of the 2^(D-1) fine faces it covers. */
int mlgpu_coarsen_faces(const mlgpu_grid *fine, int ncomp, int dtype, int dir,
                        void *coarse_faces, const void *fine_faces,
                        void *stream);

/* Geometric-mean face average sqrt(|c_lo c_hi|) (CELLTOEDGEGEOMETRIC,
 * src/CellToEdge2F.ChF) of a cell field; boundary faces of non-periodic
 * directions use a zero-gradient ghost (face = |c|). FP64. */
int mlgpu_face_geomean(const mlgpu_grid *grid, const double *cell,
                       double *faces[3], void *stream);

/* ---------------------------------------------------- linear operators -- */
/* res = rhs - L(phi) for the projection (c == NULL) or Darcy-Brinkman op:
 * VCCOMPUTERES / DBCOMPUTERES (src/DarcyBrinkmanOpF.ChF:299-396). */
int mlgpu_vc_residual(const mlgpu_vcop *op, void *res, const void *phi,
                      const void *rhs, int homogeneous, int norm_type,
                      double *norm, void *ws, size_t ws_bytes, void *stream);
int mlgpu_vc_apply(const mlgpu_vcop *op, void *lhs, const void *phi,
                   int homogeneous, void *stream);
/* GSRB half sweep (GSRBHELMHOLTZDB, F.ChF:46-159; homogeneous BCs as in
 * DarcyBrinkmanOp::levelGSRB :503-576). */
int mlgpu_vc_gsrb_pass(const mlgpu_vcop *op, void *phi, const void *rhs,
                       int pass, void *stream);
int mlgpu_vc_relax(const mlgpu_vcop *op, void *phi, const void *rhs,
                   int n_sweeps, void *stream);
int mlgpu_vc_jacobi(const mlgpu_vcop *op, void *phi, const void *rhs,
                    void *tmp, void *stream);
/* mlgpu_vc_jacobi without the caller's `tmp`: the temporary field lives in a
   fixed 8 MiB device array of the library, so the call allocates nothing.  No
   counterpart in the reference (its levelJacobi builds a temporary LevelData
   per call); it serves hosts that cannot allocate device memory.  At most
   1,048,576 FP64 / 2,097,152 FP32 cells (else MLGPU_ERR_SCRATCH, nothing
   launched).  One scratch per device: calls that may overlap in time on one
   device race.  The first call on a device looks the scratch up and should
   come before any stream capture; the address is kept until exit, so after a
   reset of that device's context the library must be reloaded before this
   entry point is called there again. */
int mlgpu_vc_jacobi_noalloc(const mlgpu_vcop *op, void *phi, const void *rhs,
                            void *stream);
int mlgpu_vc_lambda(const mlgpu_vcop *op, void *lambda, void *stream);
/* RESTRICTRESDB (F.ChF:427-505), homogeneous BCs. */
int mlgpu_vc_restrict_residual(const mlgpu_vcop *op, void *res_coarse,
                               const void *phi, const void *rhs, void *stream);

/* ----------------------------------------------- MAC projection pieces -- */
/* div = sum_d (u_d[i+e_d] - u_d[i]) / dx  (DIVERGENCE, util/DivergenceF.ChF) */
int mlgpu_mac_divergence(const mlgpu_grid *grid, double *div,
                         const double *u[3], void *stream);
/* u_d -= scale_d * (phi[i] - phi[i-e_d]) / dx on every face, ghosts of phi
 * from `bc` (inhomogeneous): levelGradientMAC + the correction loop of
 * Projector::levelMacProject (srcSubcycle/Projector.cpp:942-968).
 * scale may be NULL (scale == 1). */
int mlgpu_mac_correct(const mlgpu_grid *grid, const mlgpu_bc *bc,
                      const double *phi, const double *scale[3], double *u[3],
                      void *stream);

/* ---------------------------------------------- elementwise utilities -- */
/* y = a x + b y on n elements (LinearOp::axby / incr). */
int mlgpu_axpby(size_t n, int dtype, double a, const void *x, double b,
                void *y, void *stream);
/* norm of n elements into *out (host), MLGPU_NORM_*; FP64 accumulation;
 * `ws` as for mlgpu_nl_residual. */
int mlgpu_norm(size_t n, int dtype, const void *x, int norm_type, double *out,
               void *ws, size_t ws_bytes, void *stream);
/* dst (dtype_dst) = src (dtype_src) elementwise conversion. */
int mlgpu_convert(size_t n, int dtype_dst, void *dst, int dtype_src,
                  const void *src, void *stream);

/* ---------------------------------------------------- solvers (E1-E4) -- */
void mlgpu_mg_default_options(mlgpu_mg_options *opt, int hc_defaults);

/* Bytes of device workspace a solver needs (coarse levels, coefficients,
 * reduction scratch).  The caller allocates it (256-byte aligned). */
int mlgpu_hc_solver_workspace(const mlgpu_nlop *op, const mlgpu_mg_options *o,
                              size_t *bytes);
int mlgpu_vc_solver_workspace(const mlgpu_vcop *op, const mlgpu_mg_options *o,
                              size_t *bytes);

/* FAS multigrid for the nonlinear H-C operator (AMRFASMultiGrid driving
 * AMRNonLinearMultiCompOp; MGnewOp coarsening :1285-1501).  `op` must be FP64.
 * MLGPU_PREC_MIXED (GSRB smoothing only) keeps the FP64 nonlinear residual and
 * takes FP32 cycles on the problem linearised with the closure Jacobian once a
 * FAS iteration has at least halved the residual, going back to FAS cycles
 * when a linearised step does not reduce it (no counterpart in the
 * reference); the FP32 copies live inside the workspace. */
int mlgpu_hc_solver_create(const mlgpu_nlop *op, const mlgpu_mg_options *o,
                           void *workspace, size_t bytes, void *stream,
                           mlgpu_solver **out);
/* Linear multigrid for the projection / Darcy-Brinkman operator
 * (AMRMultiGrid + VCAMRPoissonOp2 / DarcyBrinkmanOp). FP64 `op`. */
int mlgpu_vc_solver_create(const mlgpu_vcop *op, const mlgpu_mg_options *o,
                           void *workspace, size_t bytes, void *stream,
                           mlgpu_solver **out);
/* Solve L(phi) = rhs in place (phi holds the initial guess), FP64 arrays. */
int mlgpu_solver_solve(mlgpu_solver *s, double *phi, const double *rhs,
                       mlgpu_solve_stats *stats);
/* Re-read alpha/beta (setAlphaAndBeta) and rebuild what depends on them:
 * the stored 1/diag of every level and, in mixed precision, the FP32 face
 * weights.  The coefficient arrays themselves are coarsened once, when the
 * solver is created: new coefficients need a new solver. */
int mlgpu_solver_set_alpha_beta(mlgpu_solver *s, double alpha, double beta);
int mlgpu_solver_destroy(mlgpu_solver *s);
/* Replace the wall conditions of an (H, C) solver or adjoint solver
 * (either pointer may be NULL to keep that one); MLGPU_ERR_ARG if the new
 * set is not allowed for the solver. */
int mlgpu_hc_solver_set_bcs(mlgpu_solver *s, const mlgpu_bc *phi_bc, const mlgpu_bc *derived_bc);

/* MAC projection of a face velocity, the sequence of
 * Projector::levelMacProject (srcSubcycle/Projector.cpp:858-982):
 * rhs = div u (DIVERGENCE, util/DivergenceF.ChF), solve div(Pi grad phi) = rhs
 * with `S` (a projection solver built with bCoef = -Pi_face, alpha = 0,
 * beta = 1), then u_d -= Pi_d (phi[i] - phi[i-e_d]) / dx on every face
 * (levelGradientMAC + the correction loop), ghosts of phi from `phi_bc`.
 * phi: initial guess in, pressure correction out.  `scratch`: one cell field.
 * pi_face may be NULL (unit scaling).  Runs on the solver's stream. */
int mlgpu_mac_project(mlgpu_solver *S, const mlgpu_grid *grid, const mlgpu_bc *phi_bc,
                      double *u[3], const double *pi_face[3], double *phi, double *scratch,
                      mlgpu_solve_stats *stats);

/* One backward-Euler step of the enthalpy/bulk-concentration equations, as
 * LevelBackwardEuler::updateSoln drives the FAS solve
 * (srcSubcycle/AMRLevelMushyLayer.cpp:1766-1779): rhs = phi_old * a + dt src
 * (aCoef NULL: a == 1; src NULL: no source), alpha = 1, beta = -dt, then the
 * solve of `S` (an HC solver) for phi_new, whose content is the initial guess.
 * `rhs_scratch` has the size of phi. */
int mlgpu_hc_backward_euler(mlgpu_solver *S, double *phi_new, const double *phi_old,
                            const double *src, const double *aCoef, double dt,
                            double *rhs_scratch, mlgpu_solve_stats *stats);
/* One TGA step of the same equations (time_integration_order = 2, the
 * reference's LevelTGA::updateSoln at srcSubcycle/AMRLevelMushyLayer.cpp:1766-
 * 1772; Chombo's LevelTGA is not in the reference tree, so the scheme is
 * restated from Twizell, Gumel & Arigu 1996: a = 2 - sqrt(2) - 1e-12,
 * mu1,2 = (a -+ sqrt(a^2 - 4a + 2)) / 2, mu3 = 1 - a):
 *   R = a phi_old + mu3 dt L(phi_old) + dt src,
 *   (a - mu1 dt L) psi = R,   (a - mu2 dt L) phi_new = a psi,
 * L(phi) = -div(b grad f(phi)) the nonlinear operator as the backward-Euler
 * step takes it (the operator with alpha = 1, beta = mu3 dt gives R's first
 * two terms); each solve by `S` with alpha = 1, beta = -mu dt (psi starts
 * from phi_old, phi_new from psi): FAS solves on an HC solver
 * (mlgpu_hc_solver_create), Newton solves (mlgpu_hc_newton_solve) on a
 * Jacobian solver (mlgpu_hc_adjoint_create).  The source enters as dt src: the
 * scheme's second-order source weight dt (a + mu4 dt L) src is not formed for
 * the nonlinear operator, so the step is second order in time without a
 * source and first order in the source's contribution.  `scratch`: two fields
 * of phi's size.  stats: the second solve's,
 * iterations, cycles, cell updates and launches summed over both; the status
 * is the second solve's, or the first's when the second converged. */
int mlgpu_hc_tga_step(mlgpu_solver *S, double *phi_new, const double *phi_old,
                      const double *src, const double *aCoef, double dt, double *scratch,
                      mlgpu_solve_stats *stats);

/* ----------------------------------------------- device memory helpers
 * For hosts that link only libmlgpu.so (no CUDA runtime of their own, e.g.
 * the C++ classes of mlgpu.hpp or a Fortran stepper): these are the only
 * entry points that allocate or free device memory.  kind: 0 host to
 * device, 1 device to host, 2 device to device; copies are asynchronous on
 * `stream` (NULL: the legacy default stream). */
int mlgpu_device_alloc(size_t bytes, void **ptr);
int mlgpu_device_free(void *ptr);
int mlgpu_memcpy(void *dst, const void *src, size_t bytes, int kind, void *stream);
int mlgpu_memset_zero(void *ptr, size_t bytes, void *stream);
int mlgpu_stream_synchronize(void *stream);

/* ------------------------------------------------------------ adjoint
 * Discrete adjoint of the path (no counterpart in the reference, which has
 * no derivatives): the transpose of the Jacobian of the nonlinear operator
 * N(phi) = alpha a phi - beta div(b grad f(phi)),
 *   A = dN/dphi = alpha a - beta div(b grad (J .)),  J = d(T, C_l)/d(H, C)
 * (the closure's derivative, including the porosity root's), with the
 * ghost rule of N differentiated at the walls.  FP64 throughout.  The
 * temperature conditions (phi_bc comp 0 types 2-4) are refused
 * (MLGPU_ERR_ARG). */

/* J of every cell: [4][cells] = dT/dH, dT/dC, dC_l/dH, dC_l/dC. */
int mlgpu_closure_jacobian(const mlgpu_grid *g, const mlgpu_params *p, const double *HC,
                           double *J, void *stream);
/* d porosity / d(H, C) of every cell: [2][cells] (porosity of mlgpu_closure). */
int mlgpu_porosity_jacobian(const mlgpu_grid *g, const mlgpu_params *p, const double *HC,
                            double *dpor, void *stream);
/* out = A^T y (g NULL) or g - A^T y, A at state phi whose Jacobian is J
 * (mlgpu_closure_jacobian of phi); op FP64. */
int mlgpu_hc_adjoint_apply(const mlgpu_nlop *op, const double *phi, const double *J,
                           const double *y, const double *g, double *out, void *stream);
/* One red/black pass (0 red, 1 black) of block Gauss-Seidel on A^T y = g:
 * each cell of the colour solves its own two rows exactly. */
int mlgpu_hc_adjoint_gsrb_pass(const mlgpu_nlop *op, const double *phi, const double *J,
                               double *y, const double *g, int pass, void *stream);
/* The untransposed operator: out = A x (r NULL) or r - A x, and one
 * red/black block Gauss-Seidel pass on A x = r (Newton's linear solve). */
int mlgpu_hc_linearized_apply(const mlgpu_nlop *op, const double *phi, const double *J,
                              const double *x, const double *r, double *out, void *stream);
int mlgpu_hc_linearized_gsrb_pass(const mlgpu_nlop *op, const double *phi, const double *J,
                                  double *x, const double *r, int pass, void *stream);
/* gc = 2^D average of g - A^T y on the grid coarsened by 2. */
int mlgpu_hc_adjoint_restrict(const mlgpu_nlop *op, const double *phi, const double *J,
                              const double *y, const double *g, double *gc, void *stream);

/* Multigrid solver of A^T y = g (correction-scheme V-cycles of the block
 * smoother on the operator rediscretised per level at the averaged state,
 * coefficients coarsened as the FAS hierarchy does; options as for the FAS
 * solver: smoothing counts, bottom sweeps, tolerance, max_iter, norm).
 * Workspace/creation as mlgpu_hc_solver_*; alpha/beta via
 * mlgpu_solver_set_alpha_beta. */
int mlgpu_hc_adjoint_workspace(const mlgpu_nlop *op, const mlgpu_mg_options *o,
                               size_t *bytes);
int mlgpu_hc_adjoint_create(const mlgpu_nlop *op, const mlgpu_mg_options *o, void *workspace,
                            size_t bytes, void *stream, mlgpu_solver **out);
/* Solve A^T y = g with A the Jacobian at state phi; y: initial guess in,
 * solution out. */
int mlgpu_hc_adjoint_solve(mlgpu_solver *S, const double *phi, const double *g, double *y,
                           mlgpu_solve_stats *stats);
/* The same object also solves N(phi) = rhs by Newton's method: each step
 * solves A(phi) d = rhs - N(phi) with V-cycles on A (the untransposed
 * operator, same hierarchy and block smoother) to the forcing term's
 * relative tolerance (mlgpu_hc_newton_params: by default Eisenstat-Walker,
 * at most 0.3), then phi = phi_old + s d with the cells that would leave
 * their closure regime clipped past the first regime bound, s halved (at
 * most 4 times) while the L2 norm of the FP64 residual grows; the options'
 * tolerance / max_iter / hang apply to the FP64 residual, and three
 * consecutive steps that cut it by under 5% once it is below 1e-8 of its
 * start end the solve with the hang status (its round-off floor).  phi:
 * initial guess in, solution out.  No counterpart in the reference (whose
 * FAS smoother ignores dT/dH and converges slowly through phase change).
 * With options.precision == MLGPU_PREC_MIXED the V-cycles of each step run
 * in FP32 (J in FP32 in the closure's own regime; w = J d kept per cell, wall
 * ghosts folded into the stored diagonal blocks, colour-split arrays); the
 * residual, its norms, the step and the closure stay FP64 (the lean closure,
 * within a few ulps of mlgpu_closure_tcl).  options.fuse_levels >= 2 in FP64
 * runs the same lean design in FP64. */
int mlgpu_hc_newton_solve(mlgpu_solver *S, double *phi, const double *rhs,
                          mlgpu_solve_stats *stats);
/* Newton settings of an adjoint solver's mlgpu_hc_newton_solve.  Each step's
 * linear solve runs V-cycles on A until its residual is below eta of its start,
 * at most lin_max (>= 1) cycles: eta = lin_tol (0 < .. < 1) with forcing 0; with
 * forcing 1 the Eisenstat-Walker forcing term (choice 2: 0.9 (|r_k| / |r_k-1|)^2,
 * their safeguard, at most lin_tol, at least 0.5 tolerance |r_0| / |r_k|).  The
 * step is u_old + s d, s halved while the L2 residual grows; with clip in [0, 1]
 * a cell whose H would leave its closure regime (solid, eutectic, mush, liquid)
 * stops at the first regime boundary it crosses plus clip times its overshoot;
 * clip < 0: no clipping.  vector_sweeps 1: the lean cycles' red/black half
 * sweeps take 16-byte vector loads (4 FP32 / 2 FP64 cells of a row per thread)
 * on the levels whose rows allow it, 0: one cell per thread; the same bits.
 * Defaults: lin_tol 0.3, lin_max 12, clip 0.1, forcing 1, vector_sweeps 1.
 * MLGPU_ERR_ARG for other values.  No counterpart in the reference. */
int mlgpu_hc_newton_params(mlgpu_solver *S, double lin_tol, int lin_max, double clip,
                           int forcing, int vector_sweeps);
/* Measurement: device time (ms per launch, host double) of `reps` FP32
 * smoothing launches on the finest level of a mixed-precision Newton solver,
 * at the state of its last step, timed with CUDA events on the solver's
 * stream: kind 0 = red/black half sweep (colours alternating), the only kind;
 * MLGPU_ERR_ARG for another kind or a finest level that is also the bottom.
 * No counterpart in the reference. */
int mlgpu_hc_newton_sweep_time(mlgpu_solver *S, int kind, int reps, double *ms_per_launch);
/* mlgpu_hc_backward_euler with the Newton solve of `S` (an adjoint solver). */
int mlgpu_hc_backward_euler_newton(mlgpu_solver *S, double *phi_new, const double *phi_old,
                                   const double *src, const double *aCoef, double dt,
                                   double *rhs_scratch, mlgpu_solve_stats *stats);
/* grad[(d * 2 + side) * 2 + comp] = -y^T dN/dv for every boundary value v of
 * the condition N applies at the walls (derived_bc when apply_derived_bc,
 * else phi_bc), at the state of the last mlgpu_hc_adjoint_solve; 0 on
 * periodic or absent sides.  grad: 12 host doubles. */
int mlgpu_hc_adjoint_bc_gradient(mlgpu_solver *S, const double *y, double grad[12]);
/* Adjoint of mlgpu_hc_backward_euler: given phi_new (the converged step)
 * and phi_new_bar = dJ/dphi_new, solve A^T mu = phi_new_bar (alpha 1,
 * beta -dt; mu: initial guess in, solution out), then phi_old_bar = a mu,
 * src_bar = dt mu and bc_grad (12 host doubles) as
 * mlgpu_hc_adjoint_bc_gradient; each output may be NULL. */
int mlgpu_hc_backward_euler_adjoint(mlgpu_solver *S, const double *phi_new,
                                    const double *phi_new_bar, const double *aCoef, double dt,
                                    double *mu, double *phi_old_bar, double *src_bar,
                                    double bc_grad[12], mlgpu_solve_stats *stats);
/* Adjoint of mlgpu_mac_project.  Forward: u = u* - Pi G p, D Pi G p = D u*.
 * Given ubar = dJ/du: solve D Pi G q = G^T (Pi ubar) with `S` (q: initial
 * guess in, solution out), ustar_bar = ubar - D^T q and, if pi_bar is not
 * NULL, pi_bar = -ustar_bar * (G p) with p the forward pressure (so that
 * dJ/dPi_face = pi_bar).  G^T, D^T are the exact transposes of the face
 * arrays as mlgpu_mac_project indexes them.  Across a periodic seam the
 * forward needs equal coefficients on faces 0 and n, so only the sum of the
 * two pi_bar entries there is a derivative.  `scratch`: one cell field. */
int mlgpu_mac_project_adjoint(mlgpu_solver *S, const mlgpu_grid *grid, const mlgpu_bc *phi_bc,
                              const double *ubar[3], const double *pi_face[3],
                              const double *p, double *ustar_bar[3], double *pi_bar[3],
                              double *q, double *scratch, mlgpu_solve_stats *stats);

#ifdef __cplusplus
}
#endif

#endif /* MLGPU_H_ */
