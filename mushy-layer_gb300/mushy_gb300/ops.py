"""Python mirror of the reference's level-operator surface over the C ABI.

Class and method names follow Chombo's LinearOp / MGLevelOp / AMRLevelOp as
overridden by the reference (src/AMRNonLinearMultiCompOp.H:51-352,
src/DarcyBrinkmanOp.H:49-256, src/AMRProjectionOp.h:32-36): residual,
applyOp, relax, levelGSRB, levelJacobi, restrictResidual, restrictR,
prolongIncrement, createCoarser, resetLambda/computeLambda, norm.  Fields are
torch CUDA tensors ([comp][k][j][i], no ghosts); every call goes through
libmlgpu.so on the current torch stream.  Errors raise RuntimeError with the
library's status string (the reference aborts through MayDay instead).

Beyond the reference's surface: the Jacobian pieces of the discrete adjoint
(closureJacobian, porosityJacobian, adjointApply, adjointGSRBPass,
adjointRestrict, linearizedApply, linearizedGSRBPass), AdjointMultiGrid
(transposed-Jacobian solves, Newton steps, wall-value gradients) and
macProjectAdjoint.

setSolveLog(log) installs a mushy_gb300.solvelog.SolveLog: every solver call
then appends one JSON line (status, residual history, work, wall time).
"""
import ctypes as C
import time

import torch

from . import abi

_SOLVE_LOG = None


def setSolveLog(log):
    """Install a SolveLog (None: no logging) for every solver call."""
    global _SOLVE_LOG
    _SOLVE_LOG = log


def _log(what, solver, st, rc, t0):
    """One log line for `solver`'s call started at perf_counter() == t0 (the
    C calls return after their stream is synchronised)."""
    if _SOLVE_LOG is None:
        return
    d = solver.desc
    _SOLVE_LOG.record(what, solver.kind, d.grid, solver.opts, st, rc,
                      time.perf_counter() - t0, has_a=bool(d.aCoef),
                      has_c=bool(getattr(d, "cCoef", None)))


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    if t is None:
        return None
    if not t.is_cuda or not t.is_contiguous():
        raise RuntimeError("fields must be contiguous CUDA tensors")
    return C.c_void_p(t.data_ptr())


def _dtype_code(t):
    if t.dtype == torch.float64:
        return abi.F64
    if t.dtype == torch.float32:
        return abi.F32
    raise RuntimeError("unsupported dtype %s" % t.dtype)


def coarse_grid(g):
    return abi.make_grid([g.n[d] // 2 for d in range(g.dim)], g.dx * 2,
                         [g.periodic[d] for d in range(3)])


def cell_tensor(g, ncomp, dtype=torch.float64, device="cuda"):
    return torch.zeros((ncomp,) + abi.cell_shape(g), dtype=dtype, device=device)


def face_tensor(g, d, ncomp, dtype=torch.float64, device="cuda"):
    return torch.zeros((ncomp,) + abi.face_shape(g, d), dtype=dtype, device=device)


class _NormScratch:
    _t = None

    @classmethod
    def get(cls):
        if cls._t is None:
            n = abi.load().mlgpu_norm_workspace_bytes()
            cls._t = torch.empty(n // 8 + 1, dtype=torch.float64, device="cuda")
        return cls._t


def norm(x, kind=abi.NORM_MAX):
    ws = _NormScratch.get()
    out = C.c_double()
    abi.check(abi.load().mlgpu_norm(x.numel(), _dtype_code(x), _ptr(x), kind, C.byref(out),
                                    _ptr(ws), ws.numel() * 8, _stream()), "mlgpu_norm")
    return out.value


class NLMultiCompOp:
    """AMRNonLinearMultiCompOp on one uniform box (H, C) -> (T, C_l)."""

    ncomp = 2

    def __init__(self, grid, params, phi_bc, derived_bc, alpha, beta, aCoef, bCoef,
                 apply_derived_bc=True, nlbc=None):
        self.grid, self.params = grid, params
        self.phi_bc, self.derived_bc = phi_bc, derived_bc
        # temperature-condition settings (reference defaults when not given)
        self.nlbc = nlbc if nlbc is not None else abi.make_nlbc()
        self.alpha, self.beta = float(alpha), float(beta)
        self.aCoef, self.bCoef = aCoef, list(bCoef)
        self.apply_derived_bc = int(apply_derived_bc)
        self.dtype = bCoef[0].dtype

    def desc(self):
        op = abi.NLOp()
        op.grid, op.params = self.grid, self.params
        op.phi_bc, op.derived_bc = self.phi_bc, self.derived_bc
        op.nlbc = self.nlbc
        op.apply_derived_bc = self.apply_derived_bc
        op.alpha, op.beta = self.alpha, self.beta
        op.aCoef = _ptr(self.aCoef)
        for d in range(3):
            op.bCoef[d] = _ptr(self.bCoef[d]) if d < self.grid.dim else None
        op.dtype = _dtype_code(self.bCoef[0])
        return op

    def setAlphaAndBeta(self, alpha, beta):
        self.alpha, self.beta = float(alpha), float(beta)

    def create(self, like=None):
        return cell_tensor(self.grid, 2, self.dtype)

    def residual(self, lhs, phi, rhs, homogeneous=False, norm_type=-1):
        ws = _NormScratch.get()
        out = C.c_double()
        abi.check(abi.load().mlgpu_nl_residual(C.byref(self.desc()), _ptr(lhs), _ptr(phi),
                                               _ptr(rhs), norm_type, C.byref(out), _ptr(ws),
                                               ws.numel() * 8, _stream()), "residual")
        return out.value if norm_type >= 0 else lhs

    def applyOp(self, lhs, phi, homogeneous=False):
        abi.check(abi.load().mlgpu_nl_apply(C.byref(self.desc()), _ptr(lhs), _ptr(phi),
                                            _stream()), "applyOp")
        return lhs

    def levelGSRBPass(self, phi, rhs, pass_):
        abi.check(abi.load().mlgpu_nl_gsrb_pass(C.byref(self.desc()), _ptr(phi), _ptr(rhs),
                                                pass_, _stream()), "levelGSRB")

    def levelGSRB(self, phi, rhs):
        self.levelGSRBPass(phi, rhs, 0)
        self.levelGSRBPass(phi, rhs, 1)

    def relax(self, phi, rhs, n):
        abi.check(abi.load().mlgpu_nl_relax(C.byref(self.desc()), _ptr(phi), _ptr(rhs), n,
                                            _stream()), "relax")

    def levelJacobi(self, phi, rhs):
        tmp = torch.empty_like(phi)
        abi.check(abi.load().mlgpu_nl_jacobi(C.byref(self.desc()), _ptr(phi), _ptr(rhs),
                                             _ptr(tmp), _stream()), "levelJacobi")

    def computeLambda(self):
        lam = cell_tensor(self.grid, 2, self.dtype)
        abi.check(abi.load().mlgpu_nl_lambda(C.byref(self.desc()), _ptr(lam), _stream()),
                  "computeLambda")
        return lam

    def restrictResidual(self, resCoarse, phiFine, rhsFine):
        abi.check(abi.load().mlgpu_nl_restrict_residual(C.byref(self.desc()), _ptr(resCoarse),
                                                        _ptr(phiFine), _ptr(rhsFine), _stream()),
                  "restrictResidual")
        return resCoarse

    def restrictR(self, phiCoarse, phiFine):
        abi.check(abi.load().mlgpu_restrict_average(C.byref(self.grid), 2, _dtype_code(phiFine),
                                                    _ptr(phiCoarse), _ptr(phiFine), _stream()),
                  "restrictR")
        return phiCoarse

    def prolongIncrement(self, phiThisLevel, correctCoarse, kind=abi.PROLONG_LINEAR):
        abi.check(abi.load().mlgpu_prolong_increment(C.byref(self.grid), C.byref(self.phi_bc), 2,
                                                     _dtype_code(phiThisLevel), kind,
                                                     _ptr(phiThisLevel), _ptr(correctCoarse),
                                                     _stream()), "prolongIncrement")
        return phiThisLevel

    def createCoarser(self):
        return cell_tensor(coarse_grid(self.grid), 2, self.dtype)


class VCOp:
    """alpha a phi - beta c phi - beta div(b grad phi) on one component."""

    prolong_kind = abi.PROLONG_CONSTANT

    def __init__(self, grid, bc, alpha, beta, aCoef, bCoef, cCoef=None):
        self.grid, self.bc = grid, bc
        self.alpha, self.beta = float(alpha), float(beta)
        self.aCoef, self.cCoef, self.bCoef = aCoef, cCoef, list(bCoef)
        self.dtype = bCoef[0].dtype

    def desc(self):
        op = abi.VCOp()
        op.grid, op.bc = self.grid, self.bc
        op.alpha, op.beta = self.alpha, self.beta
        op.aCoef, op.cCoef = _ptr(self.aCoef), _ptr(self.cCoef)
        for d in range(3):
            op.bCoef[d] = _ptr(self.bCoef[d]) if d < self.grid.dim else None
        op.dtype = _dtype_code(self.bCoef[0])
        return op

    def setAlphaAndBeta(self, alpha, beta):
        self.alpha, self.beta = float(alpha), float(beta)

    def create(self):
        return cell_tensor(self.grid, 1, self.dtype)

    def residual(self, lhs, phi, rhs, homogeneous=False, norm_type=-1):
        ws = _NormScratch.get()
        out = C.c_double()
        abi.check(abi.load().mlgpu_vc_residual(C.byref(self.desc()), _ptr(lhs), _ptr(phi),
                                               _ptr(rhs), int(homogeneous), norm_type,
                                               C.byref(out), _ptr(ws), ws.numel() * 8,
                                               _stream()), "residual")
        return out.value if norm_type >= 0 else lhs

    def applyOp(self, lhs, phi, homogeneous=False):
        abi.check(abi.load().mlgpu_vc_apply(C.byref(self.desc()), _ptr(lhs), _ptr(phi),
                                            int(homogeneous), _stream()), "applyOp")
        return lhs

    def levelGSRBPass(self, phi, rhs, pass_):
        abi.check(abi.load().mlgpu_vc_gsrb_pass(C.byref(self.desc()), _ptr(phi), _ptr(rhs),
                                                pass_, _stream()), "levelGSRB")

    def levelGSRB(self, phi, rhs):
        self.levelGSRBPass(phi, rhs, 0)
        self.levelGSRBPass(phi, rhs, 1)

    def relax(self, phi, rhs, n):
        abi.check(abi.load().mlgpu_vc_relax(C.byref(self.desc()), _ptr(phi), _ptr(rhs), n,
                                            _stream()), "relax")

    def levelJacobi(self, phi, rhs):
        tmp = torch.empty_like(phi)
        abi.check(abi.load().mlgpu_vc_jacobi(C.byref(self.desc()), _ptr(phi), _ptr(rhs),
                                             _ptr(tmp), _stream()), "levelJacobi")

    def computeLambda(self):
        lam = cell_tensor(self.grid, 1, self.dtype)
        abi.check(abi.load().mlgpu_vc_lambda(C.byref(self.desc()), _ptr(lam), _stream()),
                  "computeLambda")
        return lam

    def restrictResidual(self, resCoarse, phiFine, rhsFine):
        abi.check(abi.load().mlgpu_vc_restrict_residual(C.byref(self.desc()), _ptr(resCoarse),
                                                        _ptr(phiFine), _ptr(rhsFine), _stream()),
                  "restrictResidual")
        return resCoarse

    def prolongIncrement(self, phiThisLevel, correctCoarse, kind=None):
        kind = self.prolong_kind if kind is None else kind
        abi.check(abi.load().mlgpu_prolong_increment(C.byref(self.grid), C.byref(self.bc), 1,
                                                     _dtype_code(phiThisLevel), kind,
                                                     _ptr(phiThisLevel), _ptr(correctCoarse),
                                                     _stream()), "prolongIncrement")
        return phiThisLevel

    def createCoarser(self):
        return cell_tensor(coarse_grid(self.grid), 1, self.dtype)


class ProjectionOp(VCOp):
    """AMRProjectionOp: alpha = 0, bCoef = -Pi_face, beta = 1
    (srcSubcycle/Projector.cpp:2942-2973); piecewise-constant prolongation
    (src/AMRProjectionOp.cpp:67-98)."""


class DarcyBrinkmanOp(VCOp):
    """DarcyBrinkmanOp: (alpha a - beta c - beta div b grad) u = rho."""


def default_options(hc):
    o = abi.MGOptions()
    abi.load().mlgpu_mg_default_options(C.byref(o), int(hc))
    return o


class _Solver:
    def __init__(self, op, opts, kind):
        self.op, self.opts, self.kind = op, opts, kind
        lib = abi.load()
        self.desc = op.desc()
        nbytes = C.c_size_t()
        fn_ws, fn_cr = {"hc": (lib.mlgpu_hc_solver_workspace, lib.mlgpu_hc_solver_create),
                        "vc": (lib.mlgpu_vc_solver_workspace, lib.mlgpu_vc_solver_create),
                        "adj": (lib.mlgpu_hc_adjoint_workspace, lib.mlgpu_hc_adjoint_create)}[kind]
        abi.check(fn_ws(C.byref(self.desc), C.byref(opts), C.byref(nbytes)), "workspace")
        self.ws = torch.empty(nbytes.value // 8 + 64, dtype=torch.float64, device="cuda")
        base = self.ws.data_ptr()
        aligned = (base + 255) & ~255
        self.h = C.c_void_p()
        abi.check(fn_cr(C.byref(self.desc), C.byref(opts), C.c_void_p(aligned),
                        self.ws.numel() * 8 - (aligned - base), _stream(), C.byref(self.h)),
                  "solver create")

    def solve(self, phi, rhs, check=False):
        st = abi.SolveStats()
        t0 = time.perf_counter()
        rc = abi.load().mlgpu_solver_solve(self.h, _ptr(phi), _ptr(rhs), C.byref(st))
        _log("solve", self, st, rc, t0)
        if check:
            abi.check(rc, "solve")
        elif rc not in (abi.OK, abi.ERR_NOT_CONVERGED, abi.ERR_HANG):
            abi.check(rc, "solve")
        return st, rc

    def setAlphaAndBeta(self, a, b):
        abi.check(abi.load().mlgpu_solver_set_alpha_beta(self.h, a, b), "setAlphaAndBeta")

    def setBCs(self, phi_bc=None, derived_bc=None):
        """New wall conditions for an (H, C) or adjoint solver."""
        abi.check(abi.load().mlgpu_hc_solver_set_bcs(
            self.h, C.byref(phi_bc) if phi_bc is not None else None,
            C.byref(derived_bc) if derived_bc is not None else None), "setBCs")

    def __del__(self):
        if getattr(self, "h", None):
            try:
                abi.load().mlgpu_solver_destroy(self.h)
            except Exception:
                pass
            self.h = None


def _faces3(ts):
    arr = (C.c_void_p * 3)()
    for d, t in enumerate(ts):
        arr[d] = t.data_ptr() if t is not None else None
    return arr


class AMRFASMultiGrid(_Solver):
    """FAS multigrid driving NLMultiCompOp (AMRFASMultiGrid's role)."""

    def __init__(self, op, opts=None):
        super().__init__(op, opts or default_options(True), "hc")

    def backwardEuler(self, phi_new, phi_old, dt, src=None, aCoef=None):
        """LevelBackwardEuler::updateSoln: solve (a - dt L) phi_new = a phi_old + dt src."""
        scratch = torch.empty_like(phi_old)
        st = abi.SolveStats()
        t0 = time.perf_counter()
        rc = abi.load().mlgpu_hc_backward_euler(self.h, _ptr(phi_new), _ptr(phi_old), _ptr(src),
                                                _ptr(aCoef), float(dt), _ptr(scratch),
                                                C.byref(st))
        _log("backwardEuler", self, st, rc, t0)
        if rc not in (abi.OK, abi.ERR_NOT_CONVERGED, abi.ERR_HANG):
            abi.check(rc, "backwardEuler")
        return st, rc

    def tgaStep(self, phi_new, phi_old, dt, src=None, aCoef=None):
        """LevelTGA::updateSoln (time_integration_order = 2): two solves,
        (a - mu1 dt L) psi = (a + mu3 dt L) phi_old + dt src and
        (a - mu2 dt L) phi_new = a psi."""
        scratch = torch.empty((2,) + tuple(phi_old.shape), dtype=phi_old.dtype,
                              device=phi_old.device)
        st = abi.SolveStats()
        t0 = time.perf_counter()
        rc = abi.load().mlgpu_hc_tga_step(self.h, _ptr(phi_new), _ptr(phi_old), _ptr(src),
                                          _ptr(aCoef), float(dt), _ptr(scratch), C.byref(st))
        _log("tgaStep", self, st, rc, t0)
        if rc not in (abi.OK, abi.ERR_NOT_CONVERGED, abi.ERR_HANG):
            abi.check(rc, "tgaStep")
        return st, rc


class AMRMultiGrid(_Solver):
    """Linear multigrid driving ProjectionOp / DarcyBrinkmanOp."""

    def __init__(self, op, opts=None):
        super().__init__(op, opts or default_options(False), "vc")

    def levelMacProject(self, u, pi_face, phi, phi_bc=None):
        """Projector::levelMacProject: u <- u - Pi grad(phi), div(Pi grad phi) = div u."""
        g = self.op.grid
        scratch = cell_tensor(g, 1, torch.float64)
        st = abi.SolveStats()
        bc = phi_bc if phi_bc is not None else self.op.bc
        t0 = time.perf_counter()
        rc = abi.load().mlgpu_mac_project(self.h, C.byref(g), C.byref(bc),
                                          _faces3(list(u) + [None] * (3 - len(u))),
                                          _faces3(list(pi_face) + [None] * (3 - len(pi_face)))
                                          if pi_face is not None else None,
                                          _ptr(phi), _ptr(scratch), C.byref(st))
        _log("levelMacProject", self, st, rc, t0)
        if rc not in (abi.OK, abi.ERR_NOT_CONVERGED, abi.ERR_HANG):
            abi.check(rc, "levelMacProject")
        return st, rc


def _ok(rc, what):
    if rc not in (abi.OK, abi.ERR_NOT_CONVERGED, abi.ERR_HANG):
        abi.check(rc, what)


def closureJacobian(grid, params, HC):
    """d(T, C_l)/d(H, C) of every cell: tensor [4][cells...]."""
    J = torch.empty((4,) + tuple(HC.shape[1:]), dtype=torch.float64, device=HC.device)
    abi.check(abi.load().mlgpu_closure_jacobian(C.byref(grid), C.byref(params), _ptr(HC),
                                                _ptr(J), _stream()), "closureJacobian")
    return J


def porosityJacobian(grid, params, HC):
    """d porosity/d(H, C) of every cell: tensor [2][cells...]."""
    dp = torch.empty_like(HC)
    abi.check(abi.load().mlgpu_porosity_jacobian(C.byref(grid), C.byref(params), _ptr(HC),
                                                 _ptr(dp), _stream()), "porosityJacobian")
    return dp


def closureFull(grid, params, HC):
    """updateEnthalpyVariables: dict of T, porosity, Cl, Cs, Hs, He, Hl tensors."""
    keys = ("T", "porosity", "Cl", "Cs", "Hs", "He", "Hl")
    out = {k: torch.empty(tuple(HC.shape[1:]), dtype=torch.float64, device=HC.device)
           for k in keys}
    abi.check(abi.load().mlgpu_closure(C.byref(grid), C.byref(params), _ptr(HC),
                                       *[_ptr(out[k]) for k in keys], _stream()), "closure")
    return out


def adjointApply(op, phi, J, y, g=None):
    """A^T y (g None) or g - A^T y, A = dN/dphi of `op` at phi (J of phi)."""
    out = torch.empty_like(y)
    abi.check(abi.load().mlgpu_hc_adjoint_apply(C.byref(op.desc()), _ptr(phi), _ptr(J), _ptr(y),
                                                _ptr(g), _ptr(out), _stream()), "adjointApply")
    return out


def adjointGSRBPass(op, phi, J, y, g, pass_):
    abi.check(abi.load().mlgpu_hc_adjoint_gsrb_pass(C.byref(op.desc()), _ptr(phi), _ptr(J),
                                                    _ptr(y), _ptr(g), int(pass_), _stream()),
              "adjointGSRBPass")


def linearizedApply(op, phi, J, x, r=None):
    """A x (r None) or r - A x, A = dN/dphi of `op` at phi."""
    out = torch.empty_like(x)
    abi.check(abi.load().mlgpu_hc_linearized_apply(C.byref(op.desc()), _ptr(phi), _ptr(J),
                                                   _ptr(x), _ptr(r), _ptr(out), _stream()),
              "linearizedApply")
    return out


def linearizedGSRBPass(op, phi, J, x, r, pass_):
    abi.check(abi.load().mlgpu_hc_linearized_gsrb_pass(C.byref(op.desc()), _ptr(phi), _ptr(J),
                                                       _ptr(x), _ptr(r), int(pass_), _stream()),
              "linearizedGSRBPass")


def adjointRestrict(op, phi, J, y, g):
    gc = cell_tensor(coarse_grid(op.grid), 2, torch.float64)
    abi.check(abi.load().mlgpu_hc_adjoint_restrict(C.byref(op.desc()), _ptr(phi), _ptr(J),
                                                   _ptr(y), _ptr(g), _ptr(gc), _stream()),
              "adjointRestrict")
    return gc


class AdjointMultiGrid(_Solver):
    """Multigrid for A^T y = g, A the Jacobian of NLMultiCompOp at a state
    (the discrete adjoint of the converged nonlinear solve)."""

    def __init__(self, op, opts=None):
        super().__init__(op, opts or default_options(True), "adj")

    def adjointSolve(self, phi, g, y):
        st = abi.SolveStats()
        t0 = time.perf_counter()
        rc = abi.load().mlgpu_hc_adjoint_solve(self.h, _ptr(phi), _ptr(g), _ptr(y), C.byref(st))
        _log("adjointSolve", self, st, rc, t0)
        _ok(rc, "adjointSolve")
        return st, rc

    def setNewtonParams(self, lin_tol=0.3, lin_max=12, clip=0.1, forcing=1, vector_sweeps=1):
        """Linear tolerance (the cap of the Eisenstat-Walker forcing term when
        forcing=1) and cycle cap of each Newton step, the regime clipping of
        its update (clip < 0: off), vector-load half sweeps (same bits)."""
        abi.check(abi.load().mlgpu_hc_newton_params(self.h, float(lin_tol), int(lin_max),
                                                    float(clip), int(forcing),
                                                    int(vector_sweeps)),
                  "setNewtonParams")

    def newtonSolve(self, phi, rhs):
        """N(phi) = rhs by Newton steps on the Jacobian hierarchy (phi in/out)."""
        st = abi.SolveStats()
        t0 = time.perf_counter()
        rc = abi.load().mlgpu_hc_newton_solve(self.h, _ptr(phi), _ptr(rhs), C.byref(st))
        _log("newtonSolve", self, st, rc, t0)
        _ok(rc, "newtonSolve")
        return st, rc

    def backwardEulerNewton(self, phi_new, phi_old, dt, src=None, aCoef=None):
        scratch = torch.empty_like(phi_old)
        st = abi.SolveStats()
        t0 = time.perf_counter()
        rc = abi.load().mlgpu_hc_backward_euler_newton(self.h, _ptr(phi_new), _ptr(phi_old),
                                                       _ptr(src), _ptr(aCoef), float(dt),
                                                       _ptr(scratch), C.byref(st))
        _log("backwardEulerNewton", self, st, rc, t0)
        _ok(rc, "backwardEulerNewton")
        return st, rc

    def tgaStep(self, phi_new, phi_old, dt, src=None, aCoef=None):
        """The TGA step (time_integration_order = 2) with Newton's solves:
        (a - mu1 dt L) psi = (a + mu3 dt L) phi_old + dt src and
        (a - mu2 dt L) phi_new = a psi."""
        scratch = torch.empty((2,) + tuple(phi_old.shape), dtype=phi_old.dtype,
                              device=phi_old.device)
        st = abi.SolveStats()
        t0 = time.perf_counter()
        rc = abi.load().mlgpu_hc_tga_step(self.h, _ptr(phi_new), _ptr(phi_old), _ptr(src),
                                          _ptr(aCoef), float(dt), _ptr(scratch), C.byref(st))
        _log("tgaStepNewton", self, st, rc, t0)
        _ok(rc, "tgaStep")
        return st, rc

    def bcGradient(self, y):
        """-y^T dN/dv for the 12 wall values [dir][side][comp] at the last state."""
        out = (C.c_double * 12)()
        torch.cuda.current_stream().synchronize()
        abi.check(abi.load().mlgpu_hc_adjoint_bc_gradient(self.h, _ptr(y), out), "bcGradient")
        return [out[q] for q in range(12)]

    def backwardEulerAdjoint(self, phi_new, phi_new_bar, dt, mu, aCoef=None, want_src=True):
        """Adjoint of backwardEuler: returns (phi_old_bar, src_bar, bc_grad, stats, rc)."""
        old_bar = torch.empty_like(phi_new)
        src_bar = torch.empty_like(phi_new) if want_src else None
        bcg = (C.c_double * 12)()
        st = abi.SolveStats()
        t0 = time.perf_counter()
        rc = abi.load().mlgpu_hc_backward_euler_adjoint(
            self.h, _ptr(phi_new), _ptr(phi_new_bar), _ptr(aCoef), float(dt), _ptr(mu),
            _ptr(old_bar), _ptr(src_bar), bcg, C.byref(st))
        _log("backwardEulerAdjoint", self, st, rc, t0)
        _ok(rc, "backwardEulerAdjoint")
        return old_bar, src_bar, [bcg[q] for q in range(12)], st, rc


def macProjectAdjoint(solver, ubar, pi_face, p, q=None, phi_bc=None, want_pi=True):
    """Adjoint of AMRMultiGrid.levelMacProject: returns (ustar_bar, pi_bar, q, stats, rc)."""
    g = solver.op.grid
    dim = g.dim
    scratch = cell_tensor(g, 1, torch.float64)
    if q is None:
        q = cell_tensor(g, 1, torch.float64)
        q.zero_()
    usb = [torch.empty_like(ubar[d]) for d in range(dim)]
    pib = [torch.empty_like(ubar[d]) for d in range(dim)] if want_pi else None
    st = abi.SolveStats()
    bc = phi_bc if phi_bc is not None else solver.op.bc
    pad = lambda L: list(L) + [None] * (3 - len(L))
    t0 = time.perf_counter()
    rc = abi.load().mlgpu_mac_project_adjoint(
        solver.h, C.byref(g), C.byref(bc), _faces3(pad(ubar[:dim])),
        _faces3(pad(pi_face[:dim])) if pi_face is not None else None, _ptr(p),
        _faces3(pad(usb)), _faces3(pad(pib)) if want_pi else None, _ptr(q), _ptr(scratch),
        C.byref(st))
    _log("macProjectAdjoint", solver, st, rc, t0)
    _ok(rc, "macProjectAdjoint")
    return usb, pib, q, st, rc
