"""ctypes mirror of include/mlgpu.h and the loader of the sm_103a library.

The structures below are byte-for-byte the C structs of mlgpu.h.  `load()`
returns the in-tree `libmlgpu.so`; it raises if the library has not been
built, so nothing silently falls back to another implementation.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG_ROOT, "_build", "libmlgpu.so")

OK = 0
ERR_ARG = 1
ERR_CUDA = 2
ERR_NAN = 3
ERR_NOT_CONVERGED = 4
ERR_WORKSPACE = 5
ERR_HANG = 6
ERR_SCRATCH = 7

F64, F32 = 0, 1
BC_NEUMANN, BC_DIRICHLET = 0, 1
BC_FIXED_TEMPERATURE, BC_TEMPERATURE_FLUX, BC_TEMPERATURE_FLUX_RADIATION = 2, 3, 4
BC_MIXED_TEMPERATURE_SALINITY = 5  # derived_bc comp 0 only
NLBC_PICARD, NLBC_NEWTON = 0, 1
RELAX_GSRB, RELAX_JACOBI = 1, 4
PROLONG_CONSTANT, PROLONG_LINEAR = 0, 1
BOTTOM_RELAX, BOTTOM_BICGSTAB = 0, 1
PREC_F64, PREC_MIXED = 0, 1
NORM_MAX, NORM_L1, NORM_L2 = 0, 1, 2


class Grid(C.Structure):
    _fields_ = [("dim", C.c_int), ("n", C.c_int * 3), ("dx", C.c_double),
                ("periodic", C.c_int * 3)]


class BC(C.Structure):
    _fields_ = [("type", ((C.c_int * 2) * 2) * 3),
                ("value", ((C.c_double * 2) * 2) * 3)]


class Params(C.Structure):
    _fields_ = [(name, C.c_double) for name in (
        "compositionRatio", "waterDistributionCoeff", "specificHeatRatio",
        "stefan", "thetaEutectic", "ThetaEutectic", "heatConductivityRatio",
        "heatDiffusionCoeff", "saltDiffusionCoeff", "darcyCoeff",
        "viscosityCoeff")]


class NLBC(C.Structure):
    _fields_ = [("a", (C.c_double * 2) * 3), ("b", (C.c_double * 2) * 3),
                ("T_ref", (C.c_double * 2) * 3), ("no_flux_limit", (C.c_double * 2) * 3),
                ("method", C.c_int), ("max_iter", C.c_int),
                ("max_residual", C.c_double), ("relax_coeff", C.c_double),
                ("dx", C.c_double)]


class NLOp(C.Structure):
    _fields_ = [("grid", Grid), ("params", Params), ("phi_bc", BC),
                ("derived_bc", BC), ("apply_derived_bc", C.c_int),
                ("alpha", C.c_double), ("beta", C.c_double),
                ("aCoef", C.c_void_p), ("bCoef", C.c_void_p * 3),
                ("dtype", C.c_int), ("nlbc", NLBC)]


class VCOp(C.Structure):
    _fields_ = [("grid", Grid), ("bc", BC), ("alpha", C.c_double),
                ("beta", C.c_double), ("aCoef", C.c_void_p),
                ("cCoef", C.c_void_p), ("bCoef", C.c_void_p * 3),
                ("dtype", C.c_int)]


class MGOptions(C.Structure):
    _fields_ = [("num_smooth_down", C.c_int), ("num_smooth_up", C.c_int),
                ("num_mg", C.c_int), ("max_iter", C.c_int),
                ("tolerance", C.c_double), ("hang", C.c_double),
                ("norm_thresh", C.c_double), ("relax_mode", C.c_int),
                ("bottom_solver", C.c_int), ("bottom_max_iter", C.c_int),
                ("max_coarse", C.c_int), ("prolong", C.c_int),
                ("precision", C.c_int), ("inner_cycles", C.c_int),
                ("norm_type", C.c_int), ("use_graph", C.c_int), ("fuse_levels", C.c_int)]


class SolveStats(C.Structure):
    _fields_ = [("exit_status", C.c_int), ("iterations", C.c_int),
                ("cycles", C.c_int), ("levels", C.c_int),
                ("initial_norm", C.c_double), ("final_norm", C.c_double),
                ("cell_updates", C.c_double),
                ("norm_history", C.c_double * 64),
                ("kernel_launches", C.c_double)]


def make_grid(n, dx=None, periodic=(0, 0, 0)):
    n = list(n)
    dim = len(n)
    g = Grid()
    g.dim = dim
    for d in range(3):
        g.n[d] = n[d] if d < dim else 1
        g.periodic[d] = int(periodic[d]) if d < dim else 0
    g.dx = float(dx if dx is not None else 1.0 / n[0])
    return g


def make_bc(spec=None):
    """spec: dict {(dir, side, comp): (type, value)}; default Neumann 0."""
    b = BC()
    for (d, s, c), (t, v) in (spec or {}).items():
        b.type[d][s][c] = int(t)
        b.value[d][s][c] = float(v)
    return b


def make_nlbc(radiation=None, no_flux_limit=None, method=0, max_iter=2,
              max_residual=1e-5, relax_coeff=0.5, dx=0.0):
    """Nonlinear temperature-BC parameters (reference defaults: Picard, 2
    iterations, residual 1e-5, relaxation 0.5).  radiation: {(dir, side):
    (a, b, T_ref)}; no_flux_limit: {(dir, side): position}."""
    n = NLBC()
    for (d, s), (a, b, t) in (radiation or {}).items():
        n.a[d][s], n.b[d][s], n.T_ref[d][s] = float(a), float(b), float(t)
    for (d, s), v in (no_flux_limit or {}).items():
        n.no_flux_limit[d][s] = float(v)
    n.method, n.max_iter = int(method), int(max_iter)
    n.max_residual, n.relax_coeff = float(max_residual), float(relax_coeff)
    n.dx = float(dx)
    return n


def make_params(**kw):
    p = Params()
    defaults = dict(compositionRatio=5.0, waterDistributionCoeff=1e-3,
                    specificHeatRatio=1.0, stefan=5.0, thetaEutectic=0.0,
                    ThetaEutectic=0.0, heatConductivityRatio=1.0,
                    heatDiffusionCoeff=1.0, saltDiffusionCoeff=0.0,
                    darcyCoeff=0.0, viscosityCoeff=0.0)
    defaults.update(kw)
    for k, v in defaults.items():
        setattr(p, k, float(v))
    return p


def ncells(g):
    return g.n[0] * g.n[1] * g.n[2]


def face_shape(g, d):
    """(nz, ny, nx) shape of the face array of direction d."""
    n = [g.n[0], g.n[1], g.n[2]]
    n[d] += 1
    return (n[2], n[1], n[0])


def cell_shape(g):
    return (g.n[2], g.n[1], g.n[0])


_lib = None


def _declare(lib):
    vp, i, d, sz = C.c_void_p, C.c_int, C.c_double, C.c_size_t
    P = C.POINTER
    sig = {
        "mlgpu_status_string": (C.c_char_p, [i]),
        "mlgpu_version": (i, []),
        "mlgpu_closure": (i, [P(Grid), P(Params)] + [vp] * 8 + [vp]),
        "mlgpu_closure_tcl": (i, [P(Grid), P(Params), vp, vp, vp]),
        "mlgpu_closure_tcl_lean": (i, [P(Grid), P(Params), vp, vp, vp]),
        "mlgpu_norm_workspace_bytes": (sz, []),
        "mlgpu_nl_residual": (i, [P(NLOp), vp, vp, vp, i, P(d), vp, sz, vp]),
        "mlgpu_nl_apply": (i, [P(NLOp), vp, vp, vp]),
        "mlgpu_nl_gsrb_pass": (i, [P(NLOp), vp, vp, i, vp]),
        "mlgpu_nl_relax": (i, [P(NLOp), vp, vp, i, vp]),
        "mlgpu_nl_jacobi": (i, [P(NLOp), vp, vp, vp, vp]),
        "mlgpu_nl_lambda": (i, [P(NLOp), vp, vp]),
        "mlgpu_nl_restrict_residual": (i, [P(NLOp), vp, vp, vp, vp]),
        "mlgpu_restrict_average": (i, [P(Grid), i, i, vp, vp, vp]),
        "mlgpu_prolong_increment": (i, [P(Grid), P(BC), i, i, i, vp, vp, vp]),
        "mlgpu_coarsen_faces": (i, [P(Grid), i, i, i, vp, vp, vp]),
        "mlgpu_face_geomean": (i, [P(Grid), vp, vp * 3, vp]),
        "mlgpu_vc_residual": (i, [P(VCOp), vp, vp, vp, i, i, P(d), vp, sz, vp]),
        "mlgpu_vc_apply": (i, [P(VCOp), vp, vp, i, vp]),
        "mlgpu_vc_gsrb_pass": (i, [P(VCOp), vp, vp, i, vp]),
        "mlgpu_vc_relax": (i, [P(VCOp), vp, vp, i, vp]),
        "mlgpu_vc_jacobi": (i, [P(VCOp), vp, vp, vp, vp]),
        "mlgpu_vc_jacobi_noalloc": (i, [P(VCOp), vp, vp, vp]),
        "mlgpu_vc_lambda": (i, [P(VCOp), vp, vp]),
        "mlgpu_vc_restrict_residual": (i, [P(VCOp), vp, vp, vp, vp]),
        "mlgpu_mac_divergence": (i, [P(Grid), vp, vp * 3, vp]),
        "mlgpu_mac_correct": (i, [P(Grid), P(BC), vp, vp * 3, vp * 3, vp]),
        "mlgpu_axpby": (i, [sz, i, d, vp, d, vp, vp]),
        "mlgpu_norm": (i, [sz, i, vp, i, P(d), vp, sz, vp]),
        "mlgpu_convert": (i, [sz, i, vp, i, vp, vp]),
        "mlgpu_mg_default_options": (None, [P(MGOptions), i]),
        "mlgpu_hc_solver_workspace": (i, [P(NLOp), P(MGOptions), P(sz)]),
        "mlgpu_vc_solver_workspace": (i, [P(VCOp), P(MGOptions), P(sz)]),
        "mlgpu_hc_solver_create": (i, [P(NLOp), P(MGOptions), vp, sz, vp, P(vp)]),
        "mlgpu_vc_solver_create": (i, [P(VCOp), P(MGOptions), vp, sz, vp, P(vp)]),
        "mlgpu_solver_solve": (i, [vp, vp, vp, P(SolveStats)]),
        "mlgpu_solver_set_alpha_beta": (i, [vp, d, d]),
        "mlgpu_solver_destroy": (i, [vp]),
        "mlgpu_mac_project": (i, [vp, P(Grid), P(BC), vp * 3, vp * 3, vp, vp, P(SolveStats)]),
        "mlgpu_hc_backward_euler": (i, [vp, vp, vp, vp, vp, d, vp, P(SolveStats)]),
        "mlgpu_hc_tga_step": (i, [vp, vp, vp, vp, vp, d, vp, P(SolveStats)]),
        "mlgpu_closure_jacobian": (i, [P(Grid), P(Params), vp, vp, vp]),
        "mlgpu_device_alloc": (i, [sz, P(vp)]),
        "mlgpu_device_free": (i, [vp]),
        "mlgpu_memcpy": (i, [vp, vp, sz, i, vp]),
        "mlgpu_memset_zero": (i, [vp, sz, vp]),
        "mlgpu_stream_synchronize": (i, [vp]),
        "mlgpu_hc_solver_set_bcs": (i, [vp, P(BC), P(BC)]),
        "mlgpu_porosity_jacobian": (i, [P(Grid), P(Params), vp, vp, vp]),
        "mlgpu_hc_adjoint_apply": (i, [P(NLOp), vp, vp, vp, vp, vp, vp]),
        "mlgpu_hc_adjoint_gsrb_pass": (i, [P(NLOp), vp, vp, vp, vp, i, vp]),
        "mlgpu_hc_adjoint_restrict": (i, [P(NLOp), vp, vp, vp, vp, vp, vp]),
        "mlgpu_hc_linearized_apply": (i, [P(NLOp), vp, vp, vp, vp, vp, vp]),
        "mlgpu_hc_linearized_gsrb_pass": (i, [P(NLOp), vp, vp, vp, vp, i, vp]),
        "mlgpu_hc_adjoint_workspace": (i, [P(NLOp), P(MGOptions), P(sz)]),
        "mlgpu_hc_adjoint_create": (i, [P(NLOp), P(MGOptions), vp, sz, vp, P(vp)]),
        "mlgpu_hc_adjoint_solve": (i, [vp, vp, vp, vp, P(SolveStats)]),
        "mlgpu_hc_adjoint_bc_gradient": (i, [vp, vp, P(d)]),
        "mlgpu_hc_newton_solve": (i, [vp, vp, vp, P(SolveStats)]),
        "mlgpu_hc_newton_sweep_time": (i, [vp, i, i, P(d)]),
        "mlgpu_hc_newton_params": (i, [vp, d, i, d, i, i]),
        "mlgpu_hc_backward_euler_newton": (i, [vp, vp, vp, vp, vp, d, vp, P(SolveStats)]),
        "mlgpu_hc_backward_euler_adjoint": (i, [vp, vp, vp, vp, d, vp, vp, vp, P(d),
                                                P(SolveStats)]),
        "mlgpu_mac_project_adjoint": (i, [vp, P(Grid), P(BC), vp * 3, vp * 3, vp, vp * 3,
                                          vp * 3, vp, vp, P(SolveStats)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return sig


def declared_symbols():
    """Names the Python binding declares (must equal those in mlgpu.h)."""
    class _Fake:
        def __getattr__(self, name):
            class F:
                pass
            return F()
    return sorted(_declare(_Fake()).keys())


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                "libmlgpu.so is not built (%s); run __graft_entry__.build()" % LIB_PATH)
        lib = C.CDLL(LIB_PATH)
        _declare(lib)
        _lib = lib
    return _lib


def check(rc, what="mlgpu call"):
    if rc != OK:
        msg = load().mlgpu_status_string(rc).decode()
        raise RuntimeError("%s failed: %s (%d)" % (what, msg, rc))
