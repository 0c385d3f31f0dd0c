"""CPU tests of the discrete adjoint restated in the oracle.

* the linearised operator A x matches central differences of the nonlinear
  operator N (so J, including the porosity root's derivative, and the
  differentiated wall rules are right);
* A^T is the transpose of A (dot-product identity, 2D/3D, periodic, with and
  without the derived-variable condition);
* the adjoint multigrid solve agrees with a dense solve of A^T y = g;
* boundary-value gradients, the backward-Euler step adjoint and the MAC
  projection adjoint agree with finite differences of the forward oracle.
"""
import numpy as np
import pytest

import problems as P
from mushy_gb300 import abi
from oracle import oracle as O


# the mixed temperature condition on the derived T (a, b, T_ref per side)
ROBIN = {(1, 1): (0.5, -1.0, 4.0), (0, 0): (1.0, 2.0, -0.5)}


def _op(n, per, seed, dbc=True, mush=False, alpha=1.0, beta=-2e-3, robin=False):
    rng = np.random.default_rng(seed)
    g = P.grid(n, per)
    p = P.mushy_params()
    phi_bc, der = P.hc_bcs("mixed")
    nl = None
    if robin:
        nl = abi.make_nlbc(radiation=ROBIN)
        for (d, s) in ROBIN:
            der.type[d][s][0] = abi.BC_MIXED_TEMPERATURE_SALINITY
    if not dbc:
        phi_bc = abi.make_bc({(0, 0, 0): (abi.BC_DIRICHLET, 6.2), (0, 1, 1): (abi.BC_NEUMANN, 0.3),
                              (1, 0, 0): (abi.BC_NEUMANN, -0.4), (1, 1, 1): (abi.BC_DIRICHLET, -1.1),
                              (2, 0, 1): (abi.BC_DIRICHLET, -0.9)})
    phi = P.hc_state(g, rng, regimes=False)
    if mush:
        phi[0] = rng.uniform(4.4, 5.6, phi[0].shape)
    b = P.faces(g, rng, 2)
    aC = rng.uniform(0.5, 1.5, phi.shape)
    o = O.NLOpHost(g, p, phi_bc, der, alpha, beta, aC, b, apply_derived_bc=int(dbc), nlbc=nl)
    J = O.closure_jac(g, p, phi)
    return g, o, phi, J, rng


CASES = [((10, 8), (0, 0, 0), True), ((10, 8), (0, 0, 0), False), ((12, 6), (1, 0, 0), True),
         ((6, 4, 4), (0, 0, 0), True), ((6, 4, 4), (0, 1, 0), False)]


ROBIN_CASES = [((10, 8), (0, 0, 0)), ((12, 6), (0, 0, 0)), ((6, 4, 4), (0, 0, 1))]


@pytest.mark.parametrize("n,per", ROBIN_CASES)
def test_mixed_temperature_condition_linearization_and_transpose(n, per):
    """The derived mixed temperature condition (linear Robin ghost on T):
    A x against central differences of N, and A^T the transpose of A."""
    g, o, phi, J, rng = _op(n, per, 13, True, True, robin=True)
    x = rng.standard_normal(phi.shape)
    Ax = O.linearized_apply(o, phi, J, x)
    h = 1e-6
    fd = (O.nl_apply(o, phi + h * x) - O.nl_apply(o, phi - h * x)) / (2 * h)
    assert np.abs(Ax - fd).max() <= 1e-6 * np.abs(fd).max()
    y = rng.standard_normal(phi.shape)
    lhs = float((Ax * y).sum())
    rhs = float((x * O.adjoint_apply(o, phi, J, y)).sum())
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0)


@pytest.mark.parametrize("n,per,dbc", CASES)
@pytest.mark.parametrize("mush", [False, True])
def test_linearization_matches_finite_differences(n, per, dbc, mush):
    g, o, phi, J, rng = _op(n, per, 3, dbc, mush)
    x = rng.standard_normal(phi.shape)
    Ax = O.linearized_apply(o, phi, J, x)
    h = 1e-6
    fd = (O.nl_apply(o, phi + h * x) - O.nl_apply(o, phi - h * x)) / (2 * h)
    assert np.abs(Ax - fd).max() <= 1e-6 * np.abs(fd).max()


@pytest.mark.parametrize("n,per,dbc", CASES)
@pytest.mark.parametrize("mush", [False, True])
def test_adjoint_is_the_transpose(n, per, dbc, mush):
    g, o, phi, J, rng = _op(n, per, 4, dbc, mush)
    x = rng.standard_normal(phi.shape)
    y = rng.standard_normal(phi.shape)
    lhs = float((O.linearized_apply(o, phi, J, x) * y).sum())
    rhs = float((x * O.adjoint_apply(o, phi, J, y)).sum())
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0)
    # g - A^T y form and the smoother's exact per-cell solve
    gg = rng.standard_normal(phi.shape)
    assert np.allclose(O.adjoint_apply(o, phi, J, y, gg), gg - O.adjoint_apply(o, phi, J, y),
                       rtol=0, atol=1e-12 * np.abs(gg).max())


def _dense_adjoint(o, phi, J):
    m = phi.size
    A_T = np.empty((m, m))
    e = np.zeros(phi.shape)
    for q in range(m):
        e.flat[q] = 1.0
        A_T[:, q] = O.adjoint_apply(o, phi, J, e).ravel()
        e.flat[q] = 0.0
    return A_T


@pytest.mark.parametrize("n,per,dbc,robin", [((8, 8), (0, 0, 0), True, False),
                                             ((8, 8), (0, 0, 0), False, False),
                                             ((8, 4), (1, 0, 0), True, False),
                                             ((4, 4, 4), (0, 0, 1), True, False),
                                             ((8, 8), (0, 0, 0), True, True)])
def test_adjoint_solve_matches_dense_solve(n, per, dbc, robin):
    g, o, phi, J, rng = _op(n, per, 5, dbc, alpha=1.0, beta=-1e-2, robin=robin)
    A_T = _dense_adjoint(o, phi, J)
    gg = rng.standard_normal(phi.shape)
    ref = np.linalg.solve(A_T, gg.ravel()).reshape(phi.shape)
    opts = O.default_options(1)
    opts.tolerance, opts.max_iter, opts.hang = 1e-13, 60, 1e-15
    y, st, rc = O.adjoint_solve(o, opts, phi, gg)
    assert rc == 0, (rc, st.iterations, st.final_norm / st.initial_norm)
    assert np.abs(y - ref).max() <= 1e-10 * np.abs(ref).max()
    # a converged solution is a fixed point of a smoothing pass
    y2 = O.adjoint_gsrb_pass(o, phi, J, y, gg, 0)
    assert np.abs(y2 - y).max() <= 1e-9 * np.abs(y).max()


@pytest.mark.parametrize("dbc,robin", [(True, False), (False, False), (True, True)])
def test_bc_gradient_matches_finite_differences(dbc, robin):
    g, o, phi, J, rng = _op((10, 8), (0, 0, 0), 6, dbc, robin=robin)
    y = rng.standard_normal(phi.shape)
    grad = O.adjoint_bc_gradient(o, phi, J, y)
    bc_name = "derived_bc" if dbc else "phi_bc"
    h = 1e-6
    for d in range(2):
        for s in range(2):
            for c in range(2):
                bc = getattr(o.op, bc_name)
                v0 = bc.value[d][s][c]
                bc.value[d][s][c] = v0 + h
                Np = O.nl_apply(o, phi)
                bc.value[d][s][c] = v0 - h
                Nm = O.nl_apply(o, phi)
                bc.value[d][s][c] = v0
                fd = -float((y * (Np - Nm)).sum()) / (2 * h)
                k = (d * 2 + s) * 2 + c
                assert abs(grad[k] - fd) <= 1e-6 * max(abs(fd), 1e-3), (d, s, c, grad[k], fd)


def _tight(hc):
    opts = O.default_options(hc)
    opts.tolerance, opts.hang, opts.max_iter = 1e-14, 0.0, 200
    return opts


def test_backward_euler_adjoint_matches_finite_differences():
    """Objective J = <w, phi_new>, phi_new = BE step of phi_old with source
    and derived wall values: the adjoint's phi_old, source and wall-value
    gradients against central differences of tightly converged steps."""
    g, o, phi, J, rng = _op((16, 16), (0, 0, 0), 7, True, mush=True, beta=-1.0)
    dt = 2e-3
    src = 0.3 * rng.standard_normal(phi.shape)
    w = rng.standard_normal(phi.shape)
    opts = _tight(1)

    def step(phi_old, src_, bcv=None):
        if bcv is not None:
            o.op.derived_bc.value[1][0][0] = bcv
        out, st, rc = O.hc_backward_euler(o, opts, phi_old.copy(), phi_old, dt, src=src_)
        assert rc in (0, abi.ERR_HANG), rc
        return out

    v0 = o.op.derived_bc.value[1][0][0]
    phi_new = step(phi, src)
    old_bar, src_bar, bcg, mu, st, rc = O.backward_euler_adjoint(o, _tight(1), phi_new, w, dt)
    assert rc in (0, abi.ERR_HANG)
    h = 1e-6
    for what in ("old", "src"):
        dirn = rng.standard_normal(phi.shape)
        if what == "old":
            jp = (w * step(phi + h * dirn, src)).sum()
            jm = (w * step(phi - h * dirn, src)).sum()
            ad = (old_bar * dirn).sum()
        else:
            jp = (w * step(phi, src + h * dirn)).sum()
            jm = (w * step(phi, src - h * dirn)).sum()
            ad = (src_bar * dirn).sum()
        fd = (jp - jm) / (2 * h)
        assert abs(ad - fd) <= 1e-6 * abs(fd), (what, ad, fd)
    jp = (w * step(phi, src, v0 + h)).sum()
    jm = (w * step(phi, src, v0 - h)).sum()
    step(phi, src, v0)
    fd = (jp - jm) / (2 * h)
    assert abs(bcg[(1 * 2 + 0) * 2 + 0] - fd) <= 1e-6 * abs(fd)


def test_mac_project_adjoint_dot_product_and_permeability_gradient():
    g, chi, perm, u = P.projection_problem((16, 16), 9, sigma=3.0)
    u[0][..., -1] = u[0][..., 0]
    u[1][:, 0, :] = 0.0
    u[1][:, -1, :] = 0.0
    pi = O.face_geomean(g, perm)
    bc = abi.make_bc()
    rng = np.random.default_rng(9)
    v = [rng.standard_normal(x.shape) for x in u]

    def project(pi_):
        o = O.VCOpHost(g, bc, 0.0, 1.0, None, [-x for x in pi_])
        out, p, st, rc = O.mac_project(o, _tight(0), bc, u, pi_, np.zeros(abi.cell_shape(g)))
        return out, p, o

    out, p, o = project(pi)
    usb, pib, q, st, rc = O.mac_project_adjoint(o, _tight(0), bc, v, pi, p)
    # <P u*, v> = <u*, P^T v>: the map is linear in u* with homogeneous walls
    lhs = sum(float((out[d] * v[d]).sum()) for d in range(2))
    rhs = sum(float((u[d] * usb[d]).sum()) for d in range(2))
    assert abs(lhs - rhs) <= 1e-9 * abs(lhs)
    # d<v, P_Pi u*>/dPi along a random direction
    dpi = [rng.standard_normal(x.shape) * x for x in pi]
    # the forward problem needs equal coefficients on the two entries of a
    # periodic seam face (else D Pi G is not symmetric and the singular
    # system loses its compatibility), so perturb them together
    dpi[0][..., -1] = dpi[0][..., 0]
    h = 1e-6
    jp = sum(float((project([pi[d] + h * dpi[d] for d in range(2)])[0][d] * v[d]).sum())
             for d in range(2))
    jm = sum(float((project([pi[d] - h * dpi[d] for d in range(2)])[0][d] * v[d]).sum())
             for d in range(2))
    fd = (jp - jm) / (2 * h)
    ad = sum(float((pib[d] * dpi[d]).sum()) for d in range(2))
    assert abs(ad - fd) <= 1e-6 * abs(fd), (ad, fd)


@pytest.mark.parametrize("dbc", [True, False])
def test_newton_driver_matches_fas_solution(dbc):
    """The Newton driver on the Jacobian hierarchy (oracle restatement of
    mlgpu_hc_newton_solve) reaches the FP64 tolerance in fewer iterations
    than FAS cycles and lands on the FAS solution of the same step."""
    # the GPU Newton test's problem: mush and liquid, heat and weak solute
    # diffusion
    rng = np.random.default_rng(8)
    g = P.grid((32, 32))
    p = P.mushy_params()
    phi_bc, der = P.hc_bcs("mixed")
    if not dbc:
        phi_bc = abi.make_bc({(1, 0, 0): (abi.BC_DIRICHLET, 5.5), (1, 1, 1): (abi.BC_NEUMANN, 0.0)})
    phi = P.hc_state(g, rng, regimes=False)
    phi[0] = rng.uniform(4.6, 6.4, phi[0].shape)
    b = [np.stack([-np.ones(abi.face_shape(g, d)), -0.01 * np.ones(abi.face_shape(g, d))])
         for d in range(2)]
    o = O.NLOpHost(g, p, phi_bc, der, 1.0, -2e-3, None, b, apply_derived_bc=int(dbc))
    opts = O.default_options(1)
    opts.tolerance, opts.hang, opts.max_iter = 1e-12, -1.0, 300
    rhs = phi.copy()
    u_fas, st_f, rc_f = O.hc_solve(o, opts, phi, rhs)
    u_n, st_n, rc_n = O.newton_solve(o, opts, phi, rhs)
    assert rc_n in (0, abi.ERR_HANG) and st_n.final_norm <= 1e-10 * st_n.initial_norm
    assert st_n.iterations < st_f.iterations, (st_n.iterations, st_f.iterations)
    assert np.abs(O.nl_residual(o, u_n, rhs)).max() <= 1.01 * st_n.final_norm
    assert np.abs(u_n - u_fas).max() <= 1e-9 * np.abs(u_fas).max()
