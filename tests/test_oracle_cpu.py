"""CPU tests of the oracle (the checker) and of the host-side library surface.

* closure identities and known answers from the reference's phase diagram
  (src/EnthalpyVariablesF.ChF, src/phaseDiagram.cpp);
* an independent pure-numpy restatement of the nonlinear residual and one
  GSRB pass with explicit ghost cells, compared with the C++ oracle;
* manufactured-solution checks of the linear operator and multigrid solver;
* the C-ABI library exports every entry point declared in include/mlgpu.h.
"""
import ctypes as C
import os
import re

import numpy as np
import pytest

import problems as P
from mushy_gb300 import abi
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


# ------------------------------------------------------------ closure
def test_closure_regimes_known_answers():
    g = P.grid((4, 1))
    p = P.mushy_params()  # St=5, CR=5, k=1e-3, cp=1, theta_e=Theta_e=0
    HC = np.zeros((2, 1, 1, 4))
    HC[0, 0, 0] = [6.0, 5.0, 0.5, -0.5]   # liquid, mush, eutectic, solid
    HC[1, 0, 0] = [-1.0, -1.0, -4.0, -4.0]
    out = O.closure(g, p, HC)
    T, chi, Cl = out["T"], out["porosity"], out["Cl"]
    # liquid: T = H - St, C_l = C, chi = 1
    assert T[0] == 1.0 and Cl[0] == -1.0 and chi[0] == 1.0
    # mush: T = -C_l, chi in (0,1), H = chi*St + T (cp = 1), C = chi*C_l + (1-chi)*C_s
    assert T[1] == -Cl[1] and 0 < chi[1] < 1
    assert abs(chi[1] * 5.0 + T[1] - 5.0) < 1e-12
    assert abs(chi[1] * Cl[1] + (1 - chi[1]) * out["Cs"][1] - (-1.0)) < 1e-12
    # eutectic (H_s < H <= H_e): T = theta_e = 0, C_l = Theta_e = 0
    assert T[2] == 0.0 and Cl[2] == 0.0 and abs(chi[2] - 0.5 / 5.0) < 1e-15
    # solid: T = H / cp, porosity 0
    assert T[3] == -0.5 and chi[3] == 0.0
    # bounding energies: H_l = St - C, H_e = chi_e St with chi_e = (CR + C)/CR
    assert out["Hl"][0] == 6.0 and abs(out["He"][0] - 4.0) < 1e-15 and out["Hs"][0] == 0.0


def test_closure_continuous_at_liquidus():
    g = P.grid((2, 1))
    p = P.mushy_params()
    C = -1.3
    Hl = 5.0 - C
    HC = np.array([[[[Hl - 1e-9, Hl + 1e-9]]], [[[C, C]]]])
    out = O.closure(g, p, HC)
    assert abs(out["porosity"][0] - 1.0) < 1e-6
    assert abs(out["T"][0] - out["T"][1]) < 1e-6


def test_closure_tcl_matches_full_closure():
    rng = np.random.default_rng(0)
    g = P.grid((16, 8))
    p = P.mushy_params(specificHeatRatio=1.2, waterDistributionCoeff=0.02)
    HC = P.hc_state(g, rng)
    full = O.closure(g, p, HC)
    tcl = O.closure_tcl(g, p, HC).reshape(2, -1)
    assert np.array_equal(tcl[0], full["T"]) and np.array_equal(tcl[1], full["Cl"])


def test_closure_jacobian_matches_finite_differences():
    """d(T, C_l)/d(H, C) of the closure (linearised inner cycles of the mixed
    nonlinear solve) against central differences, away from regime edges."""
    rng = np.random.default_rng(3)
    g = P.grid((64, 32))
    p = P.mushy_params(specificHeatRatio=1.2, waterDistributionCoeff=0.02)
    HC = P.hc_state(g, rng)
    J = O.closure_jac(g, p, HC).reshape(4, -1)
    h = 1e-6
    fd = np.empty_like(J)
    for col in range(2):
        dp, dm = HC.copy(), HC.copy()
        dp[col] += h
        dm[col] -= h
        tp = O.closure_tcl(g, p, dp).reshape(2, -1)
        tm = O.closure_tcl(g, p, dm).reshape(2, -1)
        fd[0 + col] = (tp[0] - tm[0]) / (2 * h)
        fd[2 + col] = (tp[1] - tm[1]) / (2 * h)
    # cells whose regime is the same at +-h (the closure is piecewise smooth)
    reg = lambda x: O.closure(g, p, x)["porosity"].reshape(-1)
    same = np.ones(J.shape[1], bool)
    for col in range(2):
        for sgn in (1, -1):
            d = HC.copy()
            d[col] += sgn * 2 * h
            pr, p0 = reg(d), reg(HC)
            same &= ((pr < 1) == (p0 < 1)) & ((pr > 0) == (p0 > 0))
    assert same.sum() > 0.9 * same.size
    err = np.abs(J[:, same] - fd[:, same])
    assert np.all(err <= 1e-6 * (1 + np.abs(fd[:, same]))), err.max()


def test_porosity_clamps_c_below_minus_cr():
    # CALCULATEPOROSITYMUSH uses max(C, -CR); the scalar C++ version does not
    g = P.grid((1, 1))
    p = P.mushy_params()
    HC = np.array([[[[4.0]]], [[[-5.5]]]])
    out = O.closure(g, p, HC)
    assert np.isfinite(out["porosity"]).all()


# --------------------------------------- independent numpy restatement
def _np_closure_tcl(H, C, p):
    CR, k, cp, St = (p.compositionRatio, p.waterDistributionCoeff, p.specificHeatRatio,
                     p.stefan)
    Hs = np.where(C < -CR, 0.0, cp * ((-C - CR) / k))
    Hs = np.where(Hs < 0, 0.0, Hs)
    He = (CR + C) / CR * St
    Hl = St - C
    T = np.empty_like(H)
    Cl = np.empty_like(H)
    vC = np.where(C >= -CR, C, -CR)
    a = CR * (cp - 1) + St * (k - 1)
    b = CR * (1 - 2 * cp) + H * (1 - k) - vC * (cp - 1) - k * St
    c = (CR + vC) * cp + k * H
    with np.errstate(invalid="ignore"):
        chi = (-b - np.sqrt(b * b - 4 * a * c)) / (2 * a)
    solid, eut = H <= Hs, (H > Hs) & (H <= He)
    mush, liq = (H > He) & (H < Hl), H >= Hl
    T[solid], Cl[solid] = H[solid] / cp, 0.0
    T[eut], Cl[eut] = 0.0, 0.0
    cl = (C + CR * (1 - chi)) / (chi + k * (1 - chi))
    T[mush], Cl[mush] = -cl[mush], cl[mush]
    T[liq], Cl[liq] = H[liq] - St, C[liq]
    return T, Cl


def test_oracle_nl_residual_against_numpy_ghost_fill():
    rng = np.random.default_rng(5)
    nx, ny = 10, 6
    g = P.grid((nx, ny), (1, 0, 0))
    p = P.mushy_params()
    phi_bc, der = P.hc_bcs("mixed")
    phi = P.hc_state(g, rng)
    rhs = rng.standard_normal(phi.shape)
    bx, by = P.faces(g, rng, 2)
    alpha, beta, dx = 1.0, -3e-3, g.dx
    ref = O.NLOpHost(g, p, phi_bc, der, alpha, beta, None, [bx, by])
    res = O.nl_residual(ref, phi, rhs)
    # numpy: closure on interior, periodic x ghosts, derived BC rows in y
    T, Cl = _np_closure_tcl(phi[0, 0], phi[1, 0], p)
    pl = np.zeros((2, ny + 2, nx + 2))
    pl[0, 1:-1, 1:-1], pl[1, 1:-1, 1:-1] = T, Cl
    pl[:, 1:-1, 0], pl[:, 1:-1, -1] = pl[:, 1:-1, -2], pl[:, 1:-1, 1]
    for c, (vlo, vhi) in enumerate([(-1.0, 0.5), (-1.0, -1.0)]):
        pl[c, 0, 1:-1] = 2 * vlo - pl[c, 1, 1:-1]
        pl[c, -1, 1:-1] = 2 * vhi - pl[c, -2, 1:-1]
    mine = np.empty_like(phi)
    for c in range(2):
        q = pl[c]
        p0 = q[1:-1, 1:-1]
        s = (bx[c, 0, :, 1:] * (q[1:-1, 2:] - p0) - bx[c, 0, :, :-1] * (p0 - q[1:-1, :-2]))
        s = s + by[c, 0, 1:, :] * (q[2:, 1:-1] - p0)
        s = s - by[c, 0, :-1, :] * (p0 - q[:-2, 1:-1])
        mine[c, 0] = rhs[c, 0] - (alpha * phi[c, 0] - beta * s * (1.0 / (dx * dx)))
    assert np.allclose(mine, res, rtol=1e-13, atol=1e-13)


def test_oracle_gsrb_colours_and_fixed_point():
    rng = np.random.default_rng(6)
    g = P.grid((8, 6))
    p = P.mushy_params()
    phi_bc, der = P.hc_bcs("mixed")
    phi = P.hc_state(g, rng)
    rhs = phi.copy()
    b = P.faces(g, rng, 2)
    ref = O.NLOpHost(g, p, phi_bc, der, 1.0, -1e-3, None, b)
    red = O.nl_gsrb_pass(ref, phi, rhs, 0)
    changed = red != phi
    ii, jj = np.meshgrid(np.arange(8), np.arange(6))
    black = ((ii + jj) % 2 == 1)[None, None]
    assert not changed[:, :, black[0, 0]].any()  # black cells untouched by red pass
    # at a converged solution a sweep is a fixed point
    sol, st, rc = O.hc_solve(ref, _opts(hc=True, tol=1e-13, iters=60), phi, rhs)
    again = O.nl_relax(ref, sol, rhs, 1)
    assert np.abs(again - sol).max() < 1e-9


def _opts(hc, tol, iters):
    o = O.default_options(hc)
    o.tolerance, o.max_iter, o.hang = tol, iters, 0.0
    return o


# ------------------------------------------------ linear operator / solver
def test_vc_operator_exact_on_quadratic():
    # div(grad x^2) = 2 with b = -1, alpha=0, beta=1: L = div grad
    n = 16
    g = abi.make_grid([n, n], 1.0 / n, (0, 0, 0))
    x = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, x)
    phi = (X ** 2 + 2 * Y ** 2)[None]
    b = [np.ones(abi.face_shape(g, d)) for d in range(2)]
    ref = O.VCOpHost(g, abi.make_bc(), 0.0, -1.0, None, b)
    lhs = O.vc_apply(ref, phi, 0)
    # interior cells only (ghosts from Neumann 0 spoil the boundary rows)
    assert np.allclose(lhs[0, 1:-1, 1:-1], 6.0, atol=1e-9)


def test_vc_multigrid_solves_manufactured_problem():
    n = 64
    g = abi.make_grid([n, n], 1.0 / n, (1, 0, 0))
    rng = np.random.default_rng(7)
    sol = rng.standard_normal((1, n, n))
    b = [-rng.uniform(0.5, 2.0, abi.face_shape(g, d)) for d in range(2)]
    bc = abi.make_bc({(1, 0, 0): (abi.BC_DIRICHLET, 0.3), (1, 1, 0): (abi.BC_NEUMANN, 0.7)})
    ref = O.VCOpHost(g, bc, 0.0, 1.0, None, b)
    f = O.vc_apply(ref, sol, 0)
    out, st, rc = O.vc_solve(ref, _opts(False, 1e-12, 60), np.zeros_like(sol), f)
    assert rc == 0
    assert np.abs(out - sol).max() < 1e-8


def test_mg_depth_follows_max_coarse():
    assert O.mg_depth(P.grid((64, 64)), 2) == 5        # 64 -> 2
    assert O.mg_depth(P.grid((512, 512)), 2) == 8      # 512 -> 2
    assert O.mg_depth(P.grid((96, 64)), 2) == 4        # limited by 96 = 3 * 32
    assert O.mg_depth(P.grid((256, 256, 256)), 2) == 7


def test_restriction_prolongation_adjoint_scaling():
    # constant prolongation of a restricted constant field reproduces it
    g = P.grid((8, 8))
    fine = np.full((1, 1, 8, 8), 3.25)
    c = O.restrict_average(g, 1, fine)
    assert np.all(c == 3.25)
    back = O.prolong_increment(g, abi.make_bc(), 1, abi.PROLONG_CONSTANT, np.zeros_like(fine), c)
    assert np.all(back == 3.25)
    lin = O.prolong_increment(g, abi.make_bc(), 1, abi.PROLONG_LINEAR, np.zeros_like(fine), c)
    assert np.allclose(lin, 3.25, rtol=0, atol=1e-15)


# ------------------------------------------------------ ABI surface
def _header_symbols():
    txt = open(os.path.join(ROOT, "include", "mlgpu.h")).read()
    return sorted(set(re.findall(r"\b(mlgpu_[a-z0-9_]+)\s*\(", txt)))


def test_python_binding_declares_every_header_symbol():
    assert abi.declared_symbols() == _header_symbols()


def test_library_exports_every_symbol():
    import __graft_entry__
    __graft_entry__.build()
    lib = C.CDLL(abi.LIB_PATH)
    for name in _header_symbols():
        assert hasattr(lib, name), name
    lib2 = abi.load()
    assert lib2.mlgpu_version() >= 1
    assert lib2.mlgpu_status_string(abi.ERR_ARG) == b"invalid argument"


def test_argument_validation_without_gpu():
    lib = abi.load()
    bad = abi.make_grid([8, 8])
    bad.dim = 4
    p = abi.make_params()
    assert lib.mlgpu_closure(C.byref(bad), C.byref(p), None, None, None, None, None, None,
                             None, None, None) == abi.ERR_ARG
    nbytes = C.c_size_t()
    op = abi.VCOp()
    op.grid = abi.make_grid([64, 64])
    opts = abi.MGOptions()
    lib.mlgpu_mg_default_options(C.byref(opts), 0)
    assert lib.mlgpu_vc_solver_workspace(C.byref(op), C.byref(opts), C.byref(nbytes)) == 0
    assert nbytes.value > 64 * 64 * 8 * 3
    opts.relax_mode = 7
    assert lib.mlgpu_vc_solver_workspace(C.byref(op), C.byref(opts), C.byref(nbytes)) == abi.ERR_ARG
    # BiCGStab bottom: the linear solver takes it (and its FP64 work arrays),
    # the FAS solver refuses it (its bottom is relaxation); unknown ones refused
    lib.mlgpu_mg_default_options(C.byref(opts), 0)
    opts.bottom_solver = abi.BOTTOM_BICGSTAB
    nb2 = C.c_size_t()
    assert lib.mlgpu_vc_solver_workspace(C.byref(op), C.byref(opts), C.byref(nb2)) == 0
    assert nb2.value > nbytes.value
    hop = abi.NLOp()
    hop.grid = abi.make_grid([64, 64])
    assert lib.mlgpu_hc_solver_workspace(C.byref(hop), C.byref(opts), C.byref(nb2)) == abi.ERR_ARG
    opts.bottom_solver = 2
    assert lib.mlgpu_vc_solver_workspace(C.byref(op), C.byref(opts), C.byref(nb2)) == abi.ERR_ARG


# ------------------------------------------- nonlinear temperature conditions
def test_pd_temperature_matches_closure():
    """The scalar phase diagram used by the temperature conditions agrees with
    the Fortran closure (exactly outside the mush, to rounding inside it)."""
    rng = np.random.default_rng(21)
    g = P.grid((40, 10))
    p = P.mushy_params()
    HC = P.hc_state(g, rng)
    tcl = O.closure_tcl(g, p, HC)
    H, Cc = HC[0].ravel(), HC[1].ravel()
    T = np.array([O.pd_temperature(p, h, c) for h, c in zip(H, Cc)])
    ref = tcl[0].ravel()
    assert np.allclose(T, ref, rtol=1e-12, atol=1e-12)
    liquid = H >= 5.0 - Cc
    assert np.array_equal(T[liquid], H[liquid] - 5.0)


def _ghost_temperature(nlbc, spec, state, cell, face):
    """Ghost temperature across `face` = (dir, side) of `cell` in a uniform
    (H, C) field: with alpha = 0, beta = -1 and unit face coefficients the
    operator there is (T_g - T_0)/dx^2 (the other faces see T_0)."""
    g = P.grid((8, 6))
    p = P.mushy_params()
    phi = np.empty((2,) + abi.cell_shape(g))
    phi[0], phi[1] = state
    b = [np.ones((2,) + abi.face_shape(g, d)) for d in range(2)]
    ref = O.NLOpHost(g, p, abi.make_bc(spec), abi.make_bc(), 0.0, -1.0, None, b,
                     apply_derived_bc=0, nlbc=nlbc)
    L = O.nl_apply(ref, phi)
    i, j = cell
    T0 = O.pd_temperature(p, *state)
    return T0 + L[0, 0, j, i] * g.dx * g.dx, T0, g.dx


LIQUID = (6.5, -1.0)  # T = H - St = 1.5, ghost stays liquid


def test_fixed_temperature_known_answers():
    spec = {(0, 0, 0): (abi.BC_FIXED_TEMPERATURE, 1.4)}
    # Newton: residual linear in the liquid, exact after one step
    Tg, T0, _ = _ghost_temperature(abi.make_nlbc(method=abi.NLBC_NEWTON), spec, LIQUID,
                                   (0, 3), (0, 0))
    assert abs(Tg - (2 * 1.4 - T0)) < 1e-12
    # Picard, max_bc_iter 2, relaxation 0.5: three relaxed steps, r halving
    Tg, T0, _ = _ghost_temperature(abi.make_nlbc(), spec, LIQUID, (0, 3), (0, 0))
    r0 = (2 * 1.4 - T0) - T0
    assert abs(Tg - (T0 + 0.875 * r0)) < 1e-12
    # Picard run to convergence
    Tg, T0, _ = _ghost_temperature(abi.make_nlbc(max_iter=80, max_residual=1e-15), spec,
                                   LIQUID, (0, 3), (0, 0))
    assert abs(Tg - (2 * 1.4 - T0)) < 1e-12


def test_temperature_flux_and_radiation_known_answers():
    F = 0.8
    spec = {(0, 1, 0): (abi.BC_TEMPERATURE_FLUX, F)}
    Tg, T0, dx = _ghost_temperature(abi.make_nlbc(method=abi.NLBC_NEWTON), spec, LIQUID,
                                    (7, 2), (0, 1))
    assert abs((Tg - T0) / dx - F) < 1e-9
    a, bb, Tref, F = 0.7, 1.3, 1.2, -0.3
    spec = {(1, 0, 0): (abi.BC_TEMPERATURE_FLUX_RADIATION, F)}
    nl = abi.make_nlbc(radiation={(1, 0): (a, bb, Tref)}, method=abi.NLBC_NEWTON)
    Tg, T0, dx = _ghost_temperature(nl, spec, LIQUID, (3, 0), (1, 0))
    assert abs(a * (Tg - T0) / dx - (F + bb * ((Tg + T0) / 2 - Tref))) < 1e-9
    # below the no-flux limit (cell centres along x) the ghost is the interior
    nl = abi.make_nlbc(radiation={(1, 0): (a, bb, Tref)}, no_flux_limit={(1, 0): 0.5},
                       method=abi.NLBC_NEWTON)
    Tg, T0, _ = _ghost_temperature(nl, spec, LIQUID, (3, 0), (1, 0))  # x = 0.4375 < 0.5
    assert Tg == T0
    Tg, T0, dx = _ghost_temperature(nl, spec, LIQUID, (4, 0), (1, 0))  # x = 0.5625
    assert abs(a * (Tg - T0) / dx - (F + bb * ((Tg + T0) / 2 - Tref))) < 1e-9


def test_temperature_condition_in_the_mush_converges():
    """Newton in the mush (nonlinear T(H)) reaches the condition with enough
    iterations; the converged ghost stays in the mush."""
    p = P.mushy_params()
    state = (5.0, -1.0)  # mush: T = 0.528
    T0 = O.pd_temperature(p, *state)
    spec = {(0, 0, 0): (abi.BC_FIXED_TEMPERATURE, T0 - 0.05)}
    nl = abi.make_nlbc(method=abi.NLBC_NEWTON, max_iter=30, max_residual=1e-13)
    Tg, T0b, _ = _ghost_temperature(nl, spec, state, (0, 3), (0, 0))
    assert T0b == T0 and abs(Tg - (2 * (T0 - 0.05) - T0)) < 1e-10


def test_temperature_conditions_rejected_off_enthalpy():
    """Temperature conditions only apply to H of the nonlinear operator; on C
    (the reference stops there) or on a linear operator the call is refused
    before any device work."""
    lib = abi.load()
    g = P.grid((8, 8))
    nl = abi.NLOp()
    nl.grid, nl.params, nl.dtype = g, P.mushy_params(), abi.F64
    nl.nlbc = abi.make_nlbc()
    opts = abi.MGOptions()
    lib.mlgpu_mg_default_options(C.byref(opts), 1)
    nbytes = C.c_size_t()

    def ws():  # host-only sizing call: validates the operator, no device work
        return lib.mlgpu_hc_solver_workspace(C.byref(nl), C.byref(opts), C.byref(nbytes))

    nl.phi_bc, _, nl.nlbc = P.temperature_bcs()
    assert ws() == 0
    nl.phi_bc = abi.make_bc({(0, 0, 1): (abi.BC_FIXED_TEMPERATURE, 0.0)})
    assert ws() == abi.ERR_ARG
    nl.phi_bc = abi.make_bc({(0, 0, 0): (7, 0.0)})
    assert ws() == abi.ERR_ARG
    nl.phi_bc = abi.make_bc({(0, 0, 0): (abi.BC_TEMPERATURE_FLUX_RADIATION, 0.0)})
    nl.nlbc = abi.make_nlbc(radiation={(0, 0): (0.0, 0.0, 0.0)})  # a/dx - b/2 == 0
    assert ws() == abi.ERR_ARG
    nl.nlbc = abi.make_nlbc(radiation={(0, 0): (0.0, 1.0, 0.0)})
    assert ws() == 0
    vc = abi.VCOp()
    vc.grid = g
    vc.bc = abi.make_bc({(1, 1, 0): (abi.BC_FIXED_TEMPERATURE, 0.0)})
    lib.mlgpu_mg_default_options(C.byref(opts), 0)
    assert lib.mlgpu_vc_solver_workspace(C.byref(vc), C.byref(opts), C.byref(nbytes)) == abi.ERR_ARG


def test_mixed_temperature_condition_validation():
    """The mixed temperature condition (MLGPU_BC_MIXED_TEMPERATURE_SALINITY)
    is accepted on the derived T only, with a nonzero Robin denominator, and
    refused on C_l, on the (H, C) condition and on a linear operator; the
    TGA step refuses a missing solver, null fields and dt <= 0 -- all before
    any device work."""
    lib = abi.load()
    g = P.grid((8, 8))
    nl = abi.NLOp()
    nl.grid, nl.params, nl.dtype = g, P.mushy_params(), abi.F64
    nl.apply_derived_bc = 1
    opts = abi.MGOptions()
    lib.mlgpu_mg_default_options(C.byref(opts), 1)
    nbytes = C.c_size_t()

    def ws():
        return lib.mlgpu_hc_solver_workspace(C.byref(nl), C.byref(opts), C.byref(nbytes))

    mixed = abi.BC_MIXED_TEMPERATURE_SALINITY
    nl.nlbc = abi.make_nlbc(radiation={(1, 1): (0.5, -1.0, 4.0)})
    nl.derived_bc = abi.make_bc({(1, 1, 0): (mixed, -0.5)})
    assert ws() == 0
    nl.derived_bc = abi.make_bc({(1, 1, 1): (mixed, -0.5)})  # on C_l
    assert ws() == abi.ERR_ARG
    nl.derived_bc = abi.make_bc({(1, 1, 0): (mixed, -0.5)})
    nl.nlbc = abi.make_nlbc(radiation={(1, 1): (0.0, 0.0, 4.0)})  # a/dx - b/2 == 0
    assert ws() == abi.ERR_ARG
    nl.apply_derived_bc = 0  # the condition is not applied: nothing to check
    assert ws() == 0
    nl.apply_derived_bc = 1
    nl.nlbc = abi.make_nlbc(radiation={(1, 1): (0.5, -1.0, 4.0)})
    nl.derived_bc = abi.make_bc()
    nl.phi_bc = abi.make_bc({(1, 1, 0): (mixed, -0.5)})  # on the (H, C) condition
    assert ws() == abi.ERR_ARG
    vc = abi.VCOp()
    vc.grid = g
    vc.bc = abi.make_bc({(1, 1, 0): (mixed, 0.0)})
    lib.mlgpu_mg_default_options(C.byref(opts), 0)
    assert lib.mlgpu_vc_solver_workspace(C.byref(vc), C.byref(opts), C.byref(nbytes)) == abi.ERR_ARG
    st = abi.SolveStats()
    buf = (C.c_double * 4)()
    assert lib.mlgpu_hc_tga_step(None, buf, buf, None, None, 1e-3, buf, C.byref(st)) == abi.ERR_ARG


def test_temperature_condition_large_residual_is_zeroed():
    """NonlinearTemperatureBCRobin zeroes a residual above 10 (the reference
    warns and leaves the ghost enthalpy at its guess): a fixed temperature 20
    above the interior gives the interior enthalpy as ghost, i.e. no flux."""
    spec = {(0, 0, 0): (abi.BC_FIXED_TEMPERATURE, 25.0)}
    for method in (abi.NLBC_PICARD, abi.NLBC_NEWTON):
        Tg, T0, _ = _ghost_temperature(abi.make_nlbc(method=method), spec, LIQUID, (0, 3),
                                       (0, 0))
        assert Tg == T0



@pytest.mark.parametrize("a,b,F,Tref", [(0.5, -1.0, -1.0, 2.0), (1.0, 0.0, -0.7, 0.0),
                                        (0.5, -1.0, -0.5, 4.0)])
def test_steady_robin_conduction_matches_the_analytic_profile(a, b, F, Tref):
    """The reference's diffusive-growth check (test/diffusiveGrowth/
    testDiffusionAndBCs.py, V = 0): steady conduction between a fixed
    temperature T_max at the bottom and the mixed condition
    a dT/dz = F + b (T - T_ref) at the top has the linear solution
    T = T_max + s z, s = (F + b (T_max - T_ref)) / (a - b).  Liquid
    throughout, both walls as nonlinear temperature conditions on H (Newton
    ghost solves run to convergence), backward-Euler steps with a long time
    step to the steady state; the discrete profile is exact for a linear T."""
    n = 32
    g = abi.make_grid([4, n], 1.0 / n, [1, 0, 0])
    p = P.mushy_params()  # St = 5, CR = 5: liquid for C = -1 above T = 1
    T_max = 3.0
    s = (F + b * (T_max - Tref)) / (a - b)
    phi_bc = abi.make_bc({(1, 0, 0): (abi.BC_FIXED_TEMPERATURE, T_max),
                          (1, 1, 0): (abi.BC_TEMPERATURE_FLUX_RADIATION, F)})
    nl = abi.make_nlbc(radiation={(1, 1): (a, b, Tref)}, method=abi.NLBC_NEWTON, max_iter=50,
                       max_residual=1e-14)
    phi = np.empty((2, 1, n, 4))
    phi[0] = 5.0 + 2.5
    phi[1] = -1.0
    bcoef = [np.stack([-np.ones(abi.face_shape(g, d)), np.zeros(abi.face_shape(g, d))])
             for d in range(2)]
    ref = O.NLOpHost(g, p, phi_bc, abi.make_bc(), 1.0, -1.0, None, bcoef, apply_derived_bc=0,
                     nlbc=nl)
    opts = O.default_options(1)
    opts.tolerance, opts.hang, opts.max_iter = 1e-13, 0.0, 200
    for _ in range(6):
        phi, st, rc = O.hc_backward_euler(ref, opts, phi, phi, 1e4)
    T = phi[0, 0, :, 0] - 5.0  # liquid: T = H - St
    z = (np.arange(n) + 0.5) / n
    assert np.abs(T - (T_max + s * z)).max() < 1e-8 * max(1.0, abs(s))
    assert np.abs(phi[1] + 1.0).max() == 0.0  # no solute diffusion: C unchanged


@pytest.mark.parametrize("a,b,F,Tref", [(0.5, -1.0, -0.5, 4.0), (1.0, 0.0, -0.7, 0.0),
                                        (2.0, -0.5, 0.3, -1.0)])
def test_steady_mixed_condition_on_the_derived_temperature(a, b, F, Tref):
    """The same steady profile with the walls as the reference's inputs
    give them (test/diffusiveGrowth/inputs: bc.temperatureHi = 1 9): the
    derived-variable conditions, T Dirichlet at the bottom and the
    MixedBCTemperatureSalinity Robin ghost on T at the top
    (BCutil/PhysBCUtil.cpp:764-800), which is linear in T, so the
    discrete profile T = T_max + s z is exact."""
    n = 32
    g = abi.make_grid([4, n], 1.0 / n, [1, 0, 0])
    p = P.mushy_params()
    T_max = 3.0
    s = (F + b * (T_max - Tref)) / (a - b)
    der = abi.make_bc({(1, 0, 0): (abi.BC_DIRICHLET, T_max),
                       (1, 1, 0): (abi.BC_MIXED_TEMPERATURE_SALINITY, F)})
    nl = abi.make_nlbc(radiation={(1, 1): (a, b, Tref)})
    phi = np.empty((2, 1, n, 4))
    phi[0] = 5.0 + 2.5
    phi[1] = -1.0
    bcoef = [np.stack([-np.ones(abi.face_shape(g, d)), np.zeros(abi.face_shape(g, d))])
             for d in range(2)]
    ref = O.NLOpHost(g, p, abi.make_bc(), der, 1.0, -1.0, None, bcoef, apply_derived_bc=1,
                     nlbc=nl)
    opts = O.default_options(1)
    opts.tolerance, opts.hang, opts.max_iter = 1e-13, 0.0, 200
    for _ in range(4):
        phi, st, rc = O.hc_backward_euler(ref, opts, phi, phi, 1e4)
    T = phi[0, 0, :, 0] - 5.0
    z = (np.arange(n) + 0.5) / n
    assert np.abs(T - (T_max + s * z)).max() < 1e-8 * max(1.0, abs(s))
    # the ghost the operator uses: a (T_g - T_i)/dx = F + b ((T_g + T_i)/2 - T_ref)
    Ti = T[-1]
    Tg = (Ti * (a * n + b / 2) + F - b * Tref) / (a * n - b / 2)
    assert abs(a * (Tg - Ti) * n - (F + b * ((Tg + Ti) / 2 - Tref))) < 1e-10


def test_darcy_brinkman_poiseuille_matches_the_analytic_profile():
    """The reference's Poiseuille check (test/poiseuilleFlow/
    testPoiseuilleFlow.py): v'' = (chi / Pi) v / Da - chi F between no-slip
    walls.  With chi = Pi = 1, Da = 0.01 the solution is
    v = F Da (1 - cosh((x - 1/2) / sqrt(Da)) / cosh(1 / (2 sqrt(Da)))).
    DarcyBrinkmanOp with c = chi / (Pi Da), b = -1, beta = -1 (so
    L v = c v - v'') solved by the linear multigrid: second-order
    convergence to the profile."""
    Da, F = 0.01, 2.0
    errs = []
    for n in (32, 64, 128):
        g = abi.make_grid([n, n], 1.0 / n, [0, 1, 0])  # square: a deep hierarchy
        bc = abi.make_bc({(0, 0, 0): (abi.BC_DIRICHLET, 0.0), (0, 1, 0): (abi.BC_DIRICHLET, 0.0)})
        b = [-np.ones(abi.face_shape(g, d)) for d in range(2)]
        c = np.full(abi.cell_shape(g), 1.0 / Da)
        ref = O.VCOpHost(g, bc, 0.0, -1.0, None, b, cCoef=c)
        rho = np.full(abi.cell_shape(g), F)
        opts = O.default_options(0)
        opts.tolerance, opts.hang, opts.max_iter = 1e-13, 0.0, 200
        v, st, rc = O.vc_solve(ref, opts, np.zeros(abi.cell_shape(g)), rho)
        x = (np.arange(n) + 0.5) / n
        exact = F * Da * (1 - np.cosh((x - 0.5) / np.sqrt(Da)) / np.cosh(0.5 / np.sqrt(Da)))
        errs.append(np.abs(v[0, 0, :] - exact).max() / exact.max())
        # uniform along the periodic direction (to the red/black rounding)
        assert np.abs(v - v[:, :1, :]).max() <= 1e-14 * np.abs(v).max()
    # the Brinkman layer (width sqrt(Da) = 0.1) on 32, 64, 128 cells:
    # relative errors 9.9e-3, 2.8e-3, 7.3e-4
    assert errs[-1] < 1e-3, errs
    assert 3.4 < errs[0] / errs[1] < 4.6 and 3.4 < errs[1] / errs[2] < 4.6, errs


# ------------------------------------------------------------- MAC projection
def _projected(n=(64, 32), seed=23):
    g, chi, perm, u = P.projection_problem(n, seed, sigma=6.0)
    u[0][..., -1] = u[0][..., 0]          # one periodic seam value
    u[1][:, 0, :] = 0.0                   # no flux through the walls
    u[1][:, -1, :] = 0.0
    pi = O.face_geomean(g, perm)
    bc = abi.make_bc()
    ref = O.VCOpHost(g, bc, 0.0, 1.0, None, [-x for x in pi])
    opts = O.default_options(0)
    opts.tolerance, opts.hang, opts.max_iter = 1e-13, 0.0, 400
    return g, bc, ref, opts, pi, u


def test_mac_projection_properties():
    """levelMacProject's size-independent properties on the oracle:
    divergence-free output, idempotence, exact removal of a pi-weighted
    gradient, and the output orthogonal to the removed gradient."""
    g, bc, ref, opts, pi, u = _projected()
    zero = np.zeros(abi.cell_shape(g))
    u1, p1, st, rc = O.mac_project(ref, opts, bc, u, pi, zero)
    d0 = np.abs(O.mac_divergence(g, u)).max()
    assert np.abs(O.mac_divergence(g, u1)).max() <= 1e-10 * d0
    scale = max(np.abs(x).max() for x in u1)
    # idempotent
    u2, p2, _, _ = O.mac_project(ref, opts, bc, u1, pi, zero)
    assert max(np.abs(a - b).max() for a, b in zip(u2, u1)) <= 1e-10 * scale
    # u1 + Pi G q projects back onto u1
    q = np.random.default_rng(5).standard_normal(abi.cell_shape(g))
    ug = O.mac_correct(g, bc, -q, u1, pi)
    u3, p3, _, _ = O.mac_project(ref, opts, bc, ug, pi, zero)
    added = max(np.abs(a - b).max() for a, b in zip(ug, u1))     # |Pi G q|, ~1e5
    assert max(np.abs(a - b).max() for a, b in zip(u3, u1)) <= 1e-11 * added
    # the pressure is q up to its constant (Neumann walls, periodic x)
    assert np.abs((p3 - p3.mean()) - (q - q.mean())).max() <= 5e-8 * np.abs(q).max()
    # discrete orthogonality: sum over faces of u1 . G p1 = -sum D u1 p1 = 0
    gp = [a - b for a, b in zip(u, u1)]            # Pi G p1, face by face
    inner = sum((a[..., :-1] * b[..., :-1]).sum() if d == 0 else (a * b).sum()
                for d, (a, b) in enumerate(zip(u1, [x / y for x, y in zip(gp, pi)])))
    norm = np.sqrt(sum((a * a).sum() for a in u1) * sum((b * b).sum() for b in gp))
    assert abs(inner) <= 1e-9 * norm


@pytest.mark.parametrize("dim", [2, 3])
def test_linear_prolongation_exact_on_linear_fields(dim):
    """Linear prolongation (weights 3/4, 1/4 per direction) reproduces a
    linear field exactly at every fine cell whose stencil stays inside the
    box; piecewise-constant prolongation copies the coarse value to its
    2^D children everywhere."""
    n = [16, 12, 8][:dim]
    g = abi.make_grid(n, 1.0 / n[0])
    cs = O.coarse_shape(g, 1)
    H = g.dx * 2
    k, j, i = np.meshgrid(*[np.arange(m) for m in cs[1:]], indexing="ij")
    slope = (0.7, -1.3, 0.4)
    lin = lambda x, y, z: 2.0 + slope[0] * x + slope[1] * y + (slope[2] * z if dim == 3 else 0)
    coarse = lin((i + 0.5) * H, (j + 0.5) * H, (k + 0.5) * H)[None]
    zero = np.zeros((1,) + abi.cell_shape(g))
    fine = O.prolong_increment(g, abi.make_bc(), 1, abi.PROLONG_LINEAR, zero, coarse)
    kf, jf, if_ = np.meshgrid(*[np.arange(m) for m in abi.cell_shape(g)], indexing="ij")
    want = lin((if_ + 0.5) * g.dx, (jf + 0.5) * g.dx, (kf + 0.5) * g.dx)
    inner = (slice(1, -1) if dim == 3 else slice(None), slice(1, -1), slice(1, -1))
    assert np.abs(fine[0][inner] - want[inner]).max() <= 1e-13
    const = O.prolong_increment(g, abi.make_bc(), 1, abi.PROLONG_CONSTANT, zero, coarse)
    rep = coarse[0]
    for ax in range(3):
        if const[0].shape[ax] == 2 * rep.shape[ax]:
            rep = np.repeat(rep, 2, axis=ax)
    assert np.array_equal(const[0], rep)
