"""The mixed temperature condition on the derived (T, C_l) state
(MLGPU_BC_MIXED_TEMPERATURE_SALINITY; the reference's
MixedBCTemperatureSalinity, BCutil/PhysBCUtil.cpp:764-800): a linear Robin
ghost T_g = (T_i (a/dx + b/2) + F - b T_ref) / (a/dx - b/2) on T, C_l's
ghost by its own condition.

Checked against the oracle: the nonlinear operator's residual, apply, GSRB
and FAS restriction bitwise (2D, 3D, periodic directions); the FAS solve
bitwise; the adjoint kernels and solve bitwise and the wall-value gradient
(whose sums run in another order) to 1e-12; the FP64 Newton step to 1e-10
and the mixed-precision and lean FP64 Newton steps (natural 2D layout and
the 3D colour-split layout) converged to 1e-10 within 1e-8 of it.
"""
import numpy as np
import pytest

import problems as P
from mushy_gb300 import abi
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from test_gpu_parity import ALL, dev, exact, host  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import __graft_entry__
    __graft_entry__.build()
    yield


# (a, b, T_ref) per [dir][side] of the mixed walls: the reference's
# diffusive-growth top wall and a second, heat-gaining wall
ROBIN = {(1, 1): (0.5, -1.0, 4.0), (0, 0): (1.0, 2.0, -0.5)}


def _bcs(g):
    phi_bc, der = P.hc_bcs("mixed")
    for (d, s) in ROBIN:
        if not g.periodic[d]:
            der.type[d][s][0] = abi.BC_MIXED_TEMPERATURE_SALINITY
    return phi_bc, der, abi.make_nlbc(radiation=ROBIN)


def setup(n, per, seed, state="regimes", beta=-2e-3):
    from mushy_gb300 import ops
    rng = np.random.default_rng(seed)
    g = P.grid(n, per)
    p = P.mushy_params()
    phi_bc, der, nl = _bcs(g)
    phi = P.hc_state(g, rng, regimes=state == "regimes")
    if state == "mush":
        phi[0] = rng.uniform(4.4, 5.6, phi[0].shape)
    b = P.faces(g, rng, 2)
    aC = rng.uniform(0.5, 1.5, phi.shape)
    ref = O.NLOpHost(g, p, phi_bc, der, 1.0, beta, aC, b, nlbc=nl)
    op = ops.NLMultiCompOp(g, p, phi_bc, der, 1.0, beta, dev(aC), [dev(x) for x in b],
                           nlbc=nl)
    return g, p, ref, op, phi, rng


@pytest.mark.parametrize("n,per", ALL)
def test_mixed_condition_operator_kernels_bitwise(n, per):
    g, p, ref, op, phi, rng = setup(n, per, 31)
    rhs = phi + 0.1 * rng.standard_normal(phi.shape)
    d_phi, d_rhs = dev(phi), dev(rhs)
    res = torch.empty_like(d_phi)
    op.residual(res, d_phi, d_rhs, norm_type=abi.NORM_MAX)
    exact(host(res), O.nl_residual(ref, phi, rhs))
    lhs = torch.empty_like(d_phi)
    op.applyOp(lhs, d_phi)
    exact(host(lhs), O.nl_apply(ref, phi))
    rc = op.createCoarser()
    op.restrictResidual(rc, d_phi, d_rhs)
    exact(host(rc), O.nl_restrict_residual(ref, phi, rhs))
    op.relax(d_phi, d_rhs, 2)
    exact(host(d_phi), O.nl_relax(ref, phi, rhs, 2))


def test_mixed_condition_changes_the_operator():
    """The condition is applied: the wall cells' residual differs from the
    Neumann condition's, and only there."""
    g, p, ref, op, phi, rng = setup((16, 12), (0, 0, 0), 32)
    r_mixed = O.nl_apply(ref, phi)
    ref.op.derived_bc.type[1][1][0] = abi.BC_NEUMANN
    ref.op.derived_bc.type[0][0][0] = abi.BC_NEUMANN
    r_neu = O.nl_apply(ref, phi)
    diff = r_mixed != r_neu
    assert diff[0, 0, -1, :].all() and diff[0, 0, :, 0].all()
    assert not diff[0, 0, 1:-1, 1:].any() and not diff[1].any()


@pytest.mark.parametrize("n", [(32, 32), (16, 16, 16)])
def test_mixed_condition_fas_solve_bitwise(n):
    from mushy_gb300 import ops
    g, p, ref, op, phi, rng = setup(n, (0, 0, 0), 33, state="near", beta=-1e-2)
    rhs = phi + 0.05 * rng.standard_normal(phi.shape)
    opts = O.default_options(1)
    opts.tolerance, opts.max_iter = 1e-10, 30
    u_ref, st_ref, rc_ref = O.hc_solve(ref, opts, phi, rhs)
    o = ops.default_options(True)
    o.tolerance, o.max_iter = 1e-10, 30
    d_phi = dev(phi)
    st, rc = ops.AMRFASMultiGrid(op, o).solve(d_phi, dev(rhs))
    assert rc == rc_ref and st.iterations == st_ref.iterations
    assert st.final_norm == st_ref.final_norm
    exact(host(d_phi), u_ref)


@pytest.mark.parametrize("n,per", [((16, 12), (0, 0, 0)), ((18, 10), (1, 0, 0)),
                                   ((8, 6, 4), (0, 0, 0))])
def test_mixed_condition_adjoint_kernels_bitwise(n, per):
    from mushy_gb300 import ops
    g, p, ref, op, phi, rng = setup(n, per, 34, state="mush")
    d_phi = dev(phi)
    J = ops.closureJacobian(g, p, d_phi)
    Jr = O.closure_jac(g, p, phi)
    y = rng.standard_normal(phi.shape)
    gg = rng.standard_normal(phi.shape)
    d_y, d_g = dev(y), dev(gg)
    exact(host(ops.adjointApply(op, d_phi, J, d_y)), O.adjoint_apply(ref, phi, Jr, y))
    exact(host(ops.adjointApply(op, d_phi, J, d_y, d_g)), O.adjoint_apply(ref, phi, Jr, y, gg))
    exact(host(ops.adjointRestrict(op, d_phi, J, d_y, d_g)),
          O.adjoint_restrict(ref, phi, Jr, y, gg))
    ops.adjointGSRBPass(op, d_phi, J, d_y, d_g, 0)
    exact(host(d_y), O.adjoint_gsrb_pass(ref, phi, Jr, y, gg, 0))


def test_mixed_condition_adjoint_solve_and_gradient():
    from mushy_gb300 import ops
    g, p, ref, op, phi, rng = setup((32, 32), (0, 0, 0), 35, state="mush", beta=-1e-2)
    gg = rng.standard_normal(phi.shape)
    opts = O.default_options(1)
    opts.tolerance, opts.max_iter = 1e-12, 40
    y_ref, st_ref, rc_ref = O.adjoint_solve(ref, opts, phi, gg)
    bcg_ref = O.adjoint_bc_gradient(ref, phi, O.closure_jac(g, p, phi), y_ref)
    o = ops.default_options(True)
    o.tolerance, o.max_iter = 1e-12, 40
    S = ops.AdjointMultiGrid(op, o)
    d_y = dev(np.zeros_like(phi))
    st, rc = S.adjointSolve(dev(phi), dev(gg), d_y)
    assert rc == rc_ref and st.iterations == st_ref.iterations
    exact(host(d_y), y_ref)
    bcg = np.array(S.bcGradient(d_y))
    assert np.abs(bcg - bcg_ref).max() <= 1e-12 * np.abs(bcg_ref).max()


def _newton(op, phi0, dt, prec, fuse=1):
    from mushy_gb300 import ops
    o = ops.default_options(True)
    o.tolerance, o.hang, o.max_iter, o.precision, o.fuse_levels = 1e-10, -1.0, 60, prec, fuse
    new = dev(phi0)
    st, rc = ops.AdjointMultiGrid(op, o).backwardEulerNewton(new, dev(phi0), dt)
    assert rc == 0 and st.final_norm <= 1e-10 * st.initial_norm, (prec, fuse, rc)
    return host(new)


@pytest.mark.parametrize("n", [(64, 64), (32, 32, 32)])
def test_mixed_condition_newton_steps(n):
    """A backward-Euler step through the mush with the mixed walls (slow
    solute diffusion, b_C = -0.01): FP64 Newton against the oracle's Newton,
    mixed precision and the lean FP64 cycles against FP64 (the 3D box runs
    the colour-split lean levels)."""
    from mushy_gb300 import ops
    dt = 2e-3
    rng = np.random.default_rng(36)
    g = P.grid(n)
    p = P.mushy_params()
    phi_bc, der, nl = _bcs(g)
    phi = P.hc_state(g, rng, regimes=False)
    phi[0] = rng.uniform(4.6, 6.4, phi[0].shape)
    b = [np.stack([-np.ones(abi.face_shape(g, d)), -0.01 * np.ones(abi.face_shape(g, d))])
         for d in range(len(n))]
    ref = O.NLOpHost(g, p, phi_bc, der, 1.0, -dt, None, b, nlbc=nl)
    op = ops.NLMultiCompOp(g, p, phi_bc, der, 1.0, -dt, None, [dev(x) for x in b], nlbc=nl)
    u64 = _newton(op, phi, dt, abi.PREC_F64)
    um = _newton(op, phi, dt, abi.PREC_MIXED)
    ul = _newton(op, phi, dt, abi.PREC_F64, fuse=2)
    scale = np.abs(u64).max()
    assert np.abs(um - u64).max() <= 1e-8 * scale
    assert np.abs(ul - u64).max() <= 1e-8 * scale
    # the oracle's residual of the mixed state (backward-Euler right-hand
    # side phi^n) and its Newton step
    r0 = O.norm(O.nl_residual(ref, phi, phi))
    assert O.norm(O.nl_residual(ref, um, phi)) <= 1e-10 * r0 * 1.0001
    oo = O.default_options(1)
    oo.tolerance, oo.hang, oo.max_iter = 1e-10, -1.0, 60
    h, st_r, rc_r = O.newton_solve(ref, oo, phi, phi.copy())
    assert rc_r == 0
    assert np.abs(u64 - h).max() <= 1e-10 * scale


def test_mixed_condition_fas_mixed_precision():
    """The FAS solve in mixed precision (FP32 linearised cycles, whose
    homogeneous wall rule for the mixed condition is its derivative g, inside
    the FP64 defect correction): 1e-10 under the oracle's FP64 residual and
    within 1e-8 of the FP64 FAS solution when that one converges."""
    from mushy_gb300 import ops
    dt = 1e-3
    g = P.grid((48, 32))
    p = P.mushy_params()
    phi_bc, der, nl = _bcs(g)
    rng = np.random.default_rng(37)
    phi = P.hc_state(g, rng, regimes=False)
    b = [np.stack([-np.ones(abi.face_shape(g, d)), -0.01 * np.ones(abi.face_shape(g, d))])
         for d in range(2)]
    rhs = phi.copy()
    ref = O.NLOpHost(g, p, phi_bc, der, 1.0, -dt, None, b, nlbc=nl)
    op = ops.NLMultiCompOp(g, p, phi_bc, der, 1.0, -dt, None, [dev(x) for x in b], nlbc=nl)
    sols = {}
    for prec in (abi.PREC_F64, abi.PREC_MIXED):
        o = ops.default_options(True)
        o.max_iter, o.tolerance, o.hang, o.precision = 60, 1e-10, 1e-15, prec
        d_phi = dev(phi)
        st, rc = ops.AMRFASMultiGrid(op, o).solve(d_phi, dev(rhs))
        sols[prec] = (host(d_phi), st, rc)
    um, stm, rcm = sols[abi.PREC_MIXED]
    assert rcm == 0 and stm.final_norm <= 1e-10 * stm.initial_norm
    r0 = np.abs(O.nl_residual(ref, phi, rhs)).max()
    assert np.abs(O.nl_residual(ref, um, rhs)).max() <= 1.05e-10 * r0
    u64, st64, rc64 = sols[abi.PREC_F64]
    if rc64 == 0:
        assert np.abs(um - u64).max() <= 1e-8 * np.abs(u64).max()
