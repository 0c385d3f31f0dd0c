"""numpy front end of the CPU oracle (oracle.cpp).

TEST INFRASTRUCTURE ONLY.  The product never imports this module; tests,
__graft_entry__.smoke() and the CPU-baseline leg of bench.py use it as the
checker.  Arrays are C-contiguous float64 numpy arrays in the mlgpu.h layout
([comp][k][j][i] cells, [comp][k][j][i] faces with n[d]+1 in direction d).
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "mushy-layer_gb300"))
from mushy_gb300 import abi  # noqa: E402  (struct layouts only)
from . import build as _build  # noqa: E402

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        vp, i, d, sz = C.c_void_p, C.c_int, C.c_double, C.c_size_t
        P = C.POINTER
        sig = {
            "orc_closure": (i, [P(abi.Grid), P(abi.Params)] + [vp] * 8),
            "orc_closure_tcl": (i, [P(abi.Grid), P(abi.Params), vp, vp]),
            "orc_closure_jac": (i, [P(abi.Grid), P(abi.Params), vp, vp]),
            "orc_porosity_jac": (i, [P(abi.Grid), P(abi.Params), vp, vp]),
            "orc_nl_residual": (i, [P(abi.NLOp), vp, vp, vp]),
            "orc_nl_apply": (i, [P(abi.NLOp), vp, vp]),
            "orc_nl_gsrb_pass": (i, [P(abi.NLOp), vp, vp, i]),
            "orc_nl_relax": (i, [P(abi.NLOp), vp, vp, i]),
            "orc_nl_jacobi": (i, [P(abi.NLOp), vp, vp]),
            "orc_nl_lambda": (i, [P(abi.NLOp), vp]),
            "orc_nl_restrict_residual": (i, [P(abi.NLOp), vp, vp, vp]),
            "orc_restrict_average": (i, [P(abi.Grid), i, vp, vp]),
            "orc_prolong_increment": (i, [P(abi.Grid), P(abi.BC), i, i, vp, vp]),
            "orc_coarsen_faces": (i, [P(abi.Grid), i, i, vp, vp]),
            "orc_face_geomean": (i, [P(abi.Grid), vp, vp * 3]),
            "orc_vc_residual": (i, [P(abi.VCOp), vp, vp, vp, i]),
            "orc_vc_apply": (i, [P(abi.VCOp), vp, vp, i]),
            "orc_vc_gsrb_pass": (i, [P(abi.VCOp), vp, vp, i]),
            "orc_vc_relax": (i, [P(abi.VCOp), vp, vp, i]),
            "orc_vc_jacobi": (i, [P(abi.VCOp), vp, vp]),
            "orc_vc_lambda": (i, [P(abi.VCOp), vp]),
            "orc_vc_restrict_residual": (i, [P(abi.VCOp), vp, vp, vp]),
            "orc_mac_divergence": (i, [P(abi.Grid), vp, vp * 3]),
            "orc_mac_correct": (i, [P(abi.Grid), P(abi.BC), vp, vp * 3, vp * 3]),
            "orc_norm": (d, [sz, vp, i]),
            "orc_set_threads": (i, [i]),
            "orc_mg_default_options": (None, [P(abi.MGOptions), i]),
            "orc_mg_depth": (i, [P(abi.Grid), i]),
            "orc_pd_temperature": (d, [d, d, P(abi.Params)]),
            "orc_hc_adjoint_apply": (i, [P(abi.NLOp), vp, vp, vp, vp, vp]),
            "orc_hc_adjoint_gsrb_pass": (i, [P(abi.NLOp), vp, vp, vp, vp, i]),
            "orc_hc_adjoint_restrict": (i, [P(abi.NLOp), vp, vp, vp, vp, vp]),
            "orc_hc_linearized_apply": (i, [P(abi.NLOp), vp, vp, vp, vp]),
            "orc_hc_lin_gsrb_pass": (i, [P(abi.NLOp), vp, vp, vp, vp, i]),
            "orc_hc_newton_solve": (i, [P(abi.NLOp), P(abi.MGOptions), vp, vp,
                                        P(abi.SolveStats)]),
            "orc_hc_adjoint_solve": (i, [P(abi.NLOp), P(abi.MGOptions), vp, vp, vp,
                                         P(abi.SolveStats)]),
            "orc_hc_adjoint_bc_gradient": (i, [P(abi.NLOp), vp, vp, vp, vp]),
            "orc_hc_backward_euler_adjoint": (i, [P(abi.NLOp), P(abi.MGOptions), vp, vp, vp, d,
                                                  vp, vp, vp, vp, P(abi.SolveStats)]),
            "orc_mac_project_adjoint": (i, [P(abi.VCOp), P(abi.MGOptions), P(abi.BC), vp * 3,
                                            vp * 3, vp, vp * 3, vp * 3, vp, P(abi.SolveStats)]),
            "orc_hc_solve": (i, [P(abi.NLOp), P(abi.MGOptions), vp, vp, P(abi.SolveStats)]),
            "orc_vc_solve": (i, [P(abi.VCOp), P(abi.MGOptions), vp, vp, P(abi.SolveStats)]),
            "orc_mac_project": (i, [P(abi.VCOp), P(abi.MGOptions), P(abi.BC), vp * 3, vp * 3,
                                    vp, P(abi.SolveStats)]),
            "orc_hc_backward_euler": (i, [P(abi.NLOp), P(abi.MGOptions), vp, vp, vp, vp, d,
                                          P(abi.SolveStats)]),
            "orc_hc_tga_step": (i, [P(abi.NLOp), P(abi.MGOptions), vp, vp, vp, vp, d,
                                          P(abi.SolveStats)]),
            "orc_hc_tga_step_newton": (i, [P(abi.NLOp), P(abi.MGOptions), vp, vp, vp, vp, d,
                                           P(abi.SolveStats)]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data


def _faces3(arrs):
    t = (C.c_void_p * 3)()
    for d, a in enumerate(arrs):
        t[d] = _p(a) if a is not None else None
    return t


# ------------------------------------------------------------------ closure
def closure(g, p, HC):
    n = abi.ncells(g)
    out = {k: np.zeros(n) for k in ("T", "porosity", "Cl", "Cs", "Hs", "He", "Hl")}
    lib().orc_closure(C.byref(g), C.byref(p), _p(HC), *[_p(out[k]) for k in
                      ("T", "porosity", "Cl", "Cs", "Hs", "He", "Hl")])
    return out


def closure_tcl(g, p, HC):
    out = np.zeros_like(HC)
    lib().orc_closure_tcl(C.byref(g), C.byref(p), _p(HC), _p(out))
    return out


def porosity_jac(g, p, HC):
    """d porosity/d(H, C) per cell: [2][cells]."""
    out = np.zeros_like(HC)
    lib().orc_porosity_jac(C.byref(g), C.byref(p), _p(HC), _p(out))
    return out


def pd_temperature(p, H, C_):
    """Scalar phase-diagram temperature (computeTemperature) of one (H, C)."""
    return lib().orc_pd_temperature(float(H), float(C_), C.byref(p))


def closure_jac(g, p, HC):
    """d(T, C_l)/d(H, C) per cell: array [4][cells] = dT/dH, dT/dC, dCl/dH, dCl/dC."""
    n = HC.size // 2
    out = np.zeros((4,) + HC.shape[1:])
    lib().orc_closure_jac(C.byref(g), C.byref(p), _p(HC), _p(out))
    return out


# -------------------------------------------------- operator descriptors
class NLOpHost:
    """Holds numpy coefficient arrays alive and exposes an NLOp struct."""

    def __init__(self, g, p, phi_bc, derived_bc, alpha, beta, aCoef, bCoef,
                 apply_derived_bc=1, nlbc=None):
        self.g, self.keep = g, [aCoef] + list(bCoef)
        op = abi.NLOp()
        op.grid, op.params, op.phi_bc, op.derived_bc = g, p, phi_bc, derived_bc
        op.nlbc = nlbc if nlbc is not None else abi.make_nlbc()
        op.apply_derived_bc = apply_derived_bc
        op.alpha, op.beta = alpha, beta
        op.aCoef = _p(aCoef)
        for d in range(3):
            op.bCoef[d] = _p(bCoef[d]) if d < g.dim else None
        op.dtype = abi.F64
        self.op = op


class VCOpHost:
    def __init__(self, g, bc, alpha, beta, aCoef, bCoef, cCoef=None):
        self.g, self.keep = g, [aCoef, cCoef] + list(bCoef)
        op = abi.VCOp()
        op.grid, op.bc, op.alpha, op.beta = g, bc, alpha, beta
        op.aCoef, op.cCoef = _p(aCoef), _p(cCoef)
        for d in range(3):
            op.bCoef[d] = _p(bCoef[d]) if d < g.dim else None
        op.dtype = abi.F64
        self.op = op


def nl_residual(o, phi, rhs):
    res = np.zeros_like(phi)
    lib().orc_nl_residual(C.byref(o.op), _p(res), _p(phi), _p(rhs))
    return res


def nl_apply(o, phi):
    out = np.zeros_like(phi)
    lib().orc_nl_apply(C.byref(o.op), _p(out), _p(phi))
    return out


def nl_gsrb_pass(o, phi, rhs, pass_):
    phi = phi.copy()
    lib().orc_nl_gsrb_pass(C.byref(o.op), _p(phi), _p(rhs), pass_)
    return phi


def nl_relax(o, phi, rhs, n):
    phi = phi.copy()
    lib().orc_nl_relax(C.byref(o.op), _p(phi), _p(rhs), n)
    return phi


def nl_jacobi(o, phi, rhs):
    phi = phi.copy()
    lib().orc_nl_jacobi(C.byref(o.op), _p(phi), _p(rhs))
    return phi


def nl_lambda(o):
    out = np.zeros((2,) + abi.cell_shape(o.g))
    lib().orc_nl_lambda(C.byref(o.op), _p(out))
    return out


def coarse_shape(g, ncomp):
    dim = g.dim
    n = [g.n[0] // 2, g.n[1] // 2, g.n[2] // 2 if dim == 3 else 1]
    return (ncomp, n[2], n[1], n[0])


def nl_restrict_residual(o, phi, rhs):
    out = np.zeros(coarse_shape(o.g, 2))
    lib().orc_nl_restrict_residual(C.byref(o.op), _p(out), _p(phi), _p(rhs))
    return out


def restrict_average(g, ncomp, fine):
    out = np.zeros(coarse_shape(g, ncomp))
    lib().orc_restrict_average(C.byref(g), ncomp, _p(out), _p(fine))
    return out


def prolong_increment(g, bc, ncomp, kind, fine, coarse):
    fine = fine.copy()
    lib().orc_prolong_increment(C.byref(g), C.byref(bc), ncomp, kind, _p(fine), _p(coarse))
    return fine


def coarsen_faces(g, ncomp, d, ff):
    cg = abi.make_grid([g.n[e] // 2 for e in range(g.dim)], g.dx * 2,
                       [g.periodic[e] for e in range(3)])
    out = np.zeros((ncomp,) + abi.face_shape(cg, d))
    lib().orc_coarsen_faces(C.byref(g), ncomp, d, _p(out), _p(ff))
    return out


def face_geomean(g, cell):
    faces = [np.zeros(abi.face_shape(g, d)) if d < g.dim else None for d in range(3)]
    lib().orc_face_geomean(C.byref(g), _p(cell), _faces3(faces))
    return faces[:g.dim]


def vc_residual(o, phi, rhs, homogeneous=0):
    res = np.zeros_like(phi)
    lib().orc_vc_residual(C.byref(o.op), _p(res), _p(phi), _p(rhs), homogeneous)
    return res


def vc_apply(o, phi, homogeneous=0):
    out = np.zeros_like(phi)
    lib().orc_vc_apply(C.byref(o.op), _p(out), _p(phi), homogeneous)
    return out


def vc_gsrb_pass(o, phi, rhs, pass_):
    phi = phi.copy()
    lib().orc_vc_gsrb_pass(C.byref(o.op), _p(phi), _p(rhs), pass_)
    return phi


def vc_relax(o, phi, rhs, n):
    phi = phi.copy()
    lib().orc_vc_relax(C.byref(o.op), _p(phi), _p(rhs), n)
    return phi


def vc_jacobi(o, phi, rhs):
    phi = phi.copy()
    lib().orc_vc_jacobi(C.byref(o.op), _p(phi), _p(rhs))
    return phi


def vc_lambda(o):
    out = np.zeros(abi.cell_shape(o.g))
    lib().orc_vc_lambda(C.byref(o.op), _p(out))
    return out


def vc_restrict_residual(o, phi, rhs):
    out = np.zeros(coarse_shape(o.g, 1))
    lib().orc_vc_restrict_residual(C.byref(o.op), _p(out), _p(phi), _p(rhs))
    return out


def mac_divergence(g, u):
    out = np.zeros(abi.cell_shape(g))
    lib().orc_mac_divergence(C.byref(g), _p(out), _faces3(list(u) + [None] * (3 - len(u))))
    return out


def mac_correct(g, bc, phi, u, scale=None):
    u = [x.copy() for x in u]
    sc = None if scale is None else _faces3(list(scale) + [None] * (3 - len(scale)))
    lib().orc_mac_correct(C.byref(g), C.byref(bc), _p(phi), sc,
                          _faces3(u + [None] * (3 - len(u))))
    return u


def set_threads(n=0):
    """Host threads of the oracle's OpenMP loops (n <= 0: leave as is);
    returns the count in effect."""
    return lib().orc_set_threads(int(n))


def norm(x, kind=abi.NORM_MAX):
    x = np.ascontiguousarray(x, dtype=np.float64)
    return lib().orc_norm(x.size, _p(x), kind)


def default_options(hc):
    o = abi.MGOptions()
    lib().orc_mg_default_options(C.byref(o), int(hc))
    return o


def mg_depth(g, max_coarse=2):
    return lib().orc_mg_depth(C.byref(g), max_coarse)


def hc_solve(o, opts, phi, rhs):
    phi = phi.copy()
    st = abi.SolveStats()
    rc = lib().orc_hc_solve(C.byref(o.op), C.byref(opts), _p(phi), _p(rhs), C.byref(st))
    return phi, st, rc


def vc_solve(o, opts, phi, rhs):
    phi = phi.copy()
    st = abi.SolveStats()
    rc = lib().orc_vc_solve(C.byref(o.op), C.byref(opts), _p(phi), _p(rhs), C.byref(st))
    return phi, st, rc


def mac_project(o, opts, phi_bc, u, pi, phi):
    u = [x.copy() for x in u]
    phi = phi.copy()
    st = abi.SolveStats()
    rc = lib().orc_mac_project(C.byref(o.op), C.byref(opts), C.byref(phi_bc),
                               _faces3(u + [None] * (3 - len(u))),
                               _faces3(list(pi) + [None] * (3 - len(pi))), _p(phi), C.byref(st))
    return u, phi, st, rc


def hc_tga_step(o, opts, phi_new, phi_old, dt, src=None, a=None, newton=False):
    """mlgpu_hc_tga_step restated: the TGA step by two FAS solves (newton:
    two Newton solves, as on a Jacobian solver)."""
    phi_new = phi_new.copy()
    st = abi.SolveStats()
    f = lib().orc_hc_tga_step_newton if newton else lib().orc_hc_tga_step
    rc = f(C.byref(o.op), C.byref(opts), _p(phi_new), _p(phi_old), _p(src), _p(a), float(dt),
           C.byref(st))
    return phi_new, st, rc


def hc_backward_euler(o, opts, phi_new, phi_old, dt, src=None, a=None):
    phi_new = phi_new.copy()
    st = abi.SolveStats()
    rc = lib().orc_hc_backward_euler(C.byref(o.op), C.byref(opts), _p(phi_new), _p(phi_old),
                                     _p(src), _p(a), float(dt), C.byref(st))
    return phi_new, st, rc


# ------------------------------------------------------------------ adjoint
def adjoint_apply(o, phi, J, y, g=None):
    """A^T y (g None) or g - A^T y, A = dN/dphi at phi (J = closure_jac(phi))."""
    out = np.empty_like(y)
    lib().orc_hc_adjoint_apply(C.byref(o.op), _p(phi), _p(J), _p(y), _p(g), _p(out))
    return out


def adjoint_gsrb_pass(o, phi, J, y, g, pass_):
    y = y.copy()
    lib().orc_hc_adjoint_gsrb_pass(C.byref(o.op), _p(phi), _p(J), _p(y), _p(g), int(pass_))
    return y


def adjoint_restrict(o, phi, J, y, g):
    gc = np.zeros(coarse_shape(o.g, 2))
    lib().orc_hc_adjoint_restrict(C.byref(o.op), _p(phi), _p(J), _p(y), _p(g), _p(gc))
    return gc


def linearized_apply(o, phi, J, x):
    """A x, the Jacobian of the nonlinear operator at phi applied to x."""
    out = np.empty_like(x)
    lib().orc_hc_linearized_apply(C.byref(o.op), _p(phi), _p(J), _p(x), _p(out))
    return out


def lin_gsrb_pass(o, phi, J, x, r, pass_):
    x = x.copy()
    lib().orc_hc_lin_gsrb_pass(C.byref(o.op), _p(phi), _p(J), _p(x), _p(r), int(pass_))
    return x


def adjoint_solve(o, opts, phi, g, y=None):
    y = np.zeros_like(g) if y is None else y.copy()
    st = abi.SolveStats()
    rc = lib().orc_hc_adjoint_solve(C.byref(o.op), C.byref(opts), _p(phi), _p(g), _p(y),
                                    C.byref(st))
    return y, st, rc


def adjoint_bc_gradient(o, phi, J, y):
    out = np.zeros(12)
    lib().orc_hc_adjoint_bc_gradient(C.byref(o.op), _p(phi), _p(J), _p(y), _p(out))
    return out


def backward_euler_adjoint(o, opts, phi_new, phi_new_bar, dt, a=None, mu=None):
    mu = np.zeros_like(phi_new) if mu is None else mu.copy()
    old_bar, src_bar, bcg = np.empty_like(phi_new), np.empty_like(phi_new), np.zeros(12)
    st = abi.SolveStats()
    rc = lib().orc_hc_backward_euler_adjoint(C.byref(o.op), C.byref(opts), _p(phi_new),
                                             _p(phi_new_bar), _p(a), float(dt), _p(mu),
                                             _p(old_bar), _p(src_bar), _p(bcg), C.byref(st))
    return old_bar, src_bar, bcg, mu, st, rc


def mac_project_adjoint(o, opts, phi_bc, ubar, pi, p, q=None):
    g = o.g
    q = np.zeros(abi.cell_shape(g)) if q is None else q.copy()
    usb = [np.empty_like(ubar[d]) for d in range(g.dim)]
    pib = [np.empty_like(ubar[d]) for d in range(g.dim)]
    st = abi.SolveStats()
    rc = lib().orc_mac_project_adjoint(C.byref(o.op), C.byref(opts), C.byref(phi_bc),
                                       _faces3(ubar), _faces3(pi) if pi is not None else None,
                                       _p(p), _faces3(usb), _faces3(pib), _p(q), C.byref(st))
    return usb, pib, q, st, rc


def newton_solve(o, opts, phi, rhs):
    """N(phi) = rhs by the Newton driver on the Jacobian hierarchy."""
    phi = phi.copy()
    st = abi.SolveStats()
    rc = lib().orc_hc_newton_solve(C.byref(o.op), C.byref(opts), _p(phi), _p(rhs), C.byref(st))
    return phi, st, rc
