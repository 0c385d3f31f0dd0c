"""GPU parity of the discrete adjoint: every adjoint kernel and driver
against the oracle's restatement (bitwise in FP64, except the wall-value
gradient whose sums run in a different order: 1e-12 relative)."""
import numpy as np
import pytest

import problems as P
from mushy_gb300 import abi
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from test_gpu_parity import dev, host, exact  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import __graft_entry__
    __graft_entry__.build()
    yield


def setup(n, per, seed, dbc=True, mush=False, beta=-2e-3):
    from mushy_gb300 import ops
    rng = np.random.default_rng(seed)
    g = P.grid(n, per)
    p = P.mushy_params()
    phi_bc, der = P.hc_bcs("mixed")
    if not dbc:
        phi_bc = abi.make_bc({(0, 0, 0): (abi.BC_DIRICHLET, 6.2), (0, 1, 1): (abi.BC_NEUMANN, 0.3),
                              (1, 0, 0): (abi.BC_NEUMANN, -0.4), (1, 1, 1): (abi.BC_DIRICHLET, -1.1),
                              (2, 0, 1): (abi.BC_DIRICHLET, -0.9)})
    phi = P.hc_state(g, rng, regimes=False)
    if mush:
        phi[0] = rng.uniform(4.4, 5.6, phi[0].shape)
    b = P.faces(g, rng, 2)
    aC = rng.uniform(0.5, 1.5, phi.shape)
    ref = O.NLOpHost(g, p, phi_bc, der, 1.0, beta, aC, b, apply_derived_bc=int(dbc))
    op = ops.NLMultiCompOp(g, p, phi_bc, der, 1.0, beta, dev(aC), [dev(x) for x in b],
                           apply_derived_bc=dbc)
    return g, p, ref, op, phi, rng


CASES = [((16, 12), (0, 0, 0), True), ((16, 12), (0, 0, 0), False), ((18, 10), (1, 0, 0), True),
         ((8, 6, 4), (0, 0, 0), True), ((6, 4, 8), (0, 1, 1), False)]


@pytest.mark.parametrize("n,per,dbc", CASES)
def test_adjoint_kernels_bitwise(n, per, dbc):
    from mushy_gb300 import ops
    g, p, ref, op, phi, rng = setup(n, per, 20, dbc, mush=True)
    d_phi = dev(phi)
    J = ops.closureJacobian(g, p, d_phi)
    Jr = O.closure_jac(g, p, phi)
    exact(host(J), Jr)
    y = rng.standard_normal(phi.shape)
    gg = rng.standard_normal(phi.shape)
    d_y, d_g = dev(y), dev(gg)
    exact(host(ops.adjointApply(op, d_phi, J, d_y)), O.adjoint_apply(ref, phi, Jr, y))
    exact(host(ops.adjointApply(op, d_phi, J, d_y, d_g)), O.adjoint_apply(ref, phi, Jr, y, gg))
    exact(host(ops.adjointRestrict(op, d_phi, J, d_y, d_g)),
          O.adjoint_restrict(ref, phi, Jr, y, gg))
    ops.adjointGSRBPass(op, d_phi, J, d_y, d_g, 0)
    r = O.adjoint_gsrb_pass(ref, phi, Jr, y, gg, 0)
    exact(host(d_y), r)
    ops.adjointGSRBPass(op, d_phi, J, d_y, d_g, 1)
    exact(host(d_y), O.adjoint_gsrb_pass(ref, phi, Jr, r, gg, 1))


@pytest.mark.parametrize("n,per,dbc", [((32, 32), (0, 0, 0), True), ((32, 16), (1, 0, 0), False),
                                       ((16, 16, 16), (0, 0, 0), True)])
def test_adjoint_solve_and_bc_gradient_match_oracle(n, per, dbc):
    from mushy_gb300 import ops
    g, p, ref, op, phi, rng = setup(n, per, 21, dbc, mush=True, beta=-1e-2)
    gg = rng.standard_normal(phi.shape)
    opts = O.default_options(1)
    opts.tolerance, opts.max_iter = 1e-12, 40
    y_ref, st_ref, rc_ref = O.adjoint_solve(ref, opts, phi, gg)
    Jr = O.closure_jac(g, p, phi)
    bcg_ref = O.adjoint_bc_gradient(ref, phi, Jr, y_ref)
    for graph in (0, 1):
        o = ops.default_options(True)
        o.tolerance, o.max_iter, o.use_graph = 1e-12, 40, graph
        S = ops.AdjointMultiGrid(op, o)
        d_y = dev(np.zeros_like(phi))
        st, rc = S.adjointSolve(dev(phi), dev(gg), d_y)
        assert rc == rc_ref and st.iterations == st_ref.iterations
        assert st.cell_updates == st_ref.cell_updates
        exact(host(d_y), y_ref)
        bcg = np.array(S.bcGradient(d_y))
        assert np.abs(bcg - bcg_ref).max() <= 1e-12 * max(np.abs(bcg_ref).max(), 1e-300)


def test_backward_euler_adjoint_matches_oracle():
    from mushy_gb300 import ops
    g, p, ref, op, phi, rng = setup((32, 32), (0, 0, 0), 22, True, mush=True, beta=-1.0)
    dt = 2e-3
    w = rng.standard_normal(phi.shape)
    opts = O.default_options(1)
    opts.tolerance, opts.max_iter = 1e-12, 40
    old_r, src_r, bcg_r, mu_r, st_r, rc_r = O.backward_euler_adjoint(ref, opts, phi, w, dt,
                                                                      a=None)
    o = ops.default_options(True)
    o.tolerance, o.max_iter = 1e-12, 40
    S = ops.AdjointMultiGrid(op, o)
    mu = dev(np.zeros_like(phi))
    old, src, bcg, st, rc = S.backwardEulerAdjoint(dev(phi), dev(w), dt, mu)
    assert rc == rc_r and st.iterations == st_r.iterations
    exact(host(mu), mu_r)
    exact(host(old), old_r)
    exact(host(src), src_r)
    assert np.abs(np.array(bcg) - bcg_r).max() <= 1e-12 * np.abs(bcg_r).max()


def test_mac_project_adjoint_matches_oracle():
    from mushy_gb300 import ops
    g, chi, perm, u = P.projection_problem((64, 32), 23, sigma=6.0)
    u[0][..., -1] = u[0][..., 0]
    u[1][:, 0, :] = 0.0
    u[1][:, -1, :] = 0.0
    pi = O.face_geomean(g, perm)
    bc = abi.make_bc()
    rng = np.random.default_rng(23)
    v = [rng.standard_normal(x.shape) for x in u]
    ref = O.VCOpHost(g, bc, 0.0, 1.0, None, [-x for x in pi])
    opts = O.default_options(0)
    opts.tolerance, opts.hang, opts.max_iter = 1e-12, 0.0, 400
    _, p_ref, _, _ = O.mac_project(ref, opts, bc, u, pi, np.zeros(abi.cell_shape(g)))
    usb_r, pib_r, q_r, st_r, rc_r = O.mac_project_adjoint(ref, opts, bc, v, pi, p_ref)
    op = ops.ProjectionOp(g, bc, 0.0, 1.0, None, [dev(-x) for x in pi])
    o = ops.default_options(False)
    o.tolerance, o.hang, o.max_iter = 1e-12, 0.0, 400
    S = ops.AMRMultiGrid(op, o)
    usb, pib, q, st, rc = ops.macProjectAdjoint(S, [dev(x) for x in v], [dev(x) for x in pi],
                                                dev(p_ref))
    assert rc == rc_r and st.iterations == st_r.iterations
    exact(host(q), q_r)
    for d in range(2):
        exact(host(usb[d]), usb_r[d])
        exact(host(pib[d]), pib_r[d])


@pytest.mark.parametrize("n,per,dbc", CASES)
def test_linearized_kernels_bitwise(n, per, dbc):
    """The untransposed Jacobian A (Newton's linear operator): apply and one
    block red/black pass against the oracle."""
    from mushy_gb300 import ops
    g, p, ref, op, phi, rng = setup(n, per, 24, dbc, mush=True)
    d_phi = dev(phi)
    J = ops.closureJacobian(g, p, d_phi)
    Jr = O.closure_jac(g, p, phi)
    x = rng.standard_normal(phi.shape)
    r = rng.standard_normal(phi.shape)
    d_x, d_r = dev(x), dev(r)
    exact(host(ops.linearizedApply(op, d_phi, J, d_x)), O.linearized_apply(ref, phi, Jr, x))
    ops.linearizedGSRBPass(op, d_phi, J, d_x, d_r, 0)
    x1 = O.lin_gsrb_pass(ref, phi, Jr, x, r, 0)
    exact(host(d_x), x1)
    ops.linearizedGSRBPass(op, d_phi, J, d_x, d_r, 1)
    exact(host(d_x), O.lin_gsrb_pass(ref, phi, Jr, x1, r, 1))


@pytest.mark.parametrize("n", [(64, 64), (32, 32, 32)])
def test_newton_backward_euler_matches_fas(n):
    """Newton on the Jacobian hierarchy reaches the FP64 residual tolerance
    in fewer iterations than the FAS solve and lands on the same solution."""
    from mushy_gb300 import ops
    g = P.grid(n)
    p = P.mushy_params()
    phi_bc, der = P.hc_bcs("mixed")
    rng = np.random.default_rng(25)
    phi = P.hc_state(g, rng, regimes=False)
    phi[0] = rng.uniform(4.6, 6.4, phi[0].shape)
    b = [np.stack([-np.ones(abi.face_shape(g, d)), -0.01 * np.ones(abi.face_shape(g, d))])
         for d in range(len(n))]
    op = ops.NLMultiCompOp(g, p, phi_bc, der, 1.0, -1e-3, None, [dev(x) for x in b])
    dt = 2e-3
    o = ops.default_options(True)
    o.tolerance, o.hang, o.max_iter = 1e-12, -1.0, 300
    fas = dev(phi)
    st_f, rc_f = ops.AMRFASMultiGrid(op, o).backwardEuler(fas, dev(phi), dt)
    A = ops.AdjointMultiGrid(op, o)
    nt = dev(phi)
    st_n, rc_n = A.backwardEulerNewton(nt, dev(phi), dt)
    # semi-smooth Newton: the closure's regime switches (liquidus) slow the
    # steps that move cells across them; still far fewer than FAS iterations
    assert rc_n == 0 and st_n.iterations <= 30, (rc_n, st_n.iterations, st_n.cycles)
    assert st_n.iterations < st_f.iterations, (st_n.iterations, st_f.iterations)
    assert st_n.final_norm <= 1e-12 * st_n.initial_norm
    ref = O.NLOpHost(g, p, phi_bc, der, 1.0, -dt, None, b)
    r = O.nl_residual(ref, host(nt), phi)
    assert np.abs(r).max() <= 1.01e-12 * st_n.initial_norm
    scale = np.abs(host(fas)).max()
    assert np.abs(host(nt) - host(fas)).max() <= 1e-9 * scale


def test_newton_driver_agrees_with_oracle():
    """The device Newton driver against its oracle restatement on the same
    step (same linear cycles, stored inverse blocks, step halving); the L2
    merit is summed in another order on the device, so the comparison is to
    1e-10 rather than bitwise."""
    from mushy_gb300 import ops
    rng = np.random.default_rng(26)
    g = P.grid((32, 32))
    p = P.mushy_params()
    phi_bc, der = P.hc_bcs("mixed")
    phi = P.hc_state(g, rng, regimes=False)
    phi[0] = rng.uniform(4.6, 6.4, phi[0].shape)
    b = [np.stack([-np.ones(abi.face_shape(g, d)), -0.01 * np.ones(abi.face_shape(g, d))])
         for d in range(2)]
    ref = O.NLOpHost(g, p, phi_bc, der, 1.0, -2e-3, None, b)
    opts = O.default_options(1)
    opts.tolerance, opts.hang, opts.max_iter = 1e-12, -1.0, 100
    u_ref, st_ref, rc_ref = O.newton_solve(ref, opts, phi, phi.copy())
    op = ops.NLMultiCompOp(g, p, phi_bc, der, 1.0, -2e-3, None, [dev(x) for x in b])
    o = ops.default_options(True)
    o.tolerance, o.hang, o.max_iter = 1e-12, -1.0, 100
    A = ops.AdjointMultiGrid(op, o)
    d_u = dev(phi)
    st, rc = A.newtonSolve(d_u, dev(phi))
    assert rc == rc_ref and abs(st.iterations - st_ref.iterations) <= 1
    assert np.abs(host(d_u) - u_ref).max() <= 1e-10 * np.abs(u_ref).max()


def test_adjoint_workload_step_gradient_matches_oracle_256():
    """The adjoint workload at its own size (256^2, the solidification model's
    operator and first step): Newton's backward-Euler step forward on the
    GPU, then the step's adjoint on the GPU and in the oracle from the same
    converged state -- the multiplier, the old-state and source gradients
    bit for bit, the wall-value gradient to 1e-12 (a sum in another order)."""
    from mushy_gb300 import darcy_model as M, ops
    model = M.DarcySolidification(256)
    phi0 = M.initial_state(256, seed=5)
    g, p, dt = model.grid, model.params, model.dt
    o = ops.default_options(True)
    o.tolerance, o.hang, o.max_iter = 1e-12, -1.0, 200
    A = ops.AdjointMultiGrid(model.hop, o)
    new = phi0.clone()
    st_n, rc_n = A.backwardEulerNewton(new, phi0, dt)
    assert rc_n in (0, abi.ERR_HANG) and st_n.final_norm <= 1e-10 * st_n.initial_norm
    phi = host(new)
    b = [host(x) for x in model.bcoef]
    der = abi.make_bc({(1, 0, 0): (abi.BC_DIRICHLET, 0.5),
                       (1, 1, 0): (abi.BC_DIRICHLET, model.T_top)})
    ref = O.NLOpHost(g, p, abi.make_bc(), der, 1.0, -dt, None, b)
    w = np.random.default_rng(55).standard_normal(phi.shape)
    opts = O.default_options(1)
    opts.tolerance, opts.hang, opts.max_iter = 1e-12, -1.0, 200
    old_r, src_r, bcg_r, mu_r, st_r, rc_r = O.backward_euler_adjoint(ref, opts, phi, w, dt)
    d_phi, d_w, mu = dev(phi), dev(w), dev(np.zeros_like(phi))
    old, src, bcg, st, rc = A.backwardEulerAdjoint(d_phi, d_w, dt, mu)
    assert rc == rc_r and st.iterations == st_r.iterations
    exact(host(mu), mu_r)
    exact(host(old), old_r)
    exact(host(src), src_r)
    assert np.abs(np.array(bcg) - bcg_r).max() <= 1e-12 * np.abs(bcg_r).max()
