"""Failure detection on the host: faults injected into the inputs of the
oracle's solvers (a NaN or Inf in the right-hand side, the initial guess or
a face coefficient, zeroed permeability faces, an iteration cap, a stalled
solve) come back as the status codes of include/mlgpu.h and the exit codes
of the reference's solvers (0 converged, 2 hang, 4 iteration limit, 8
non-finite norm), never as a converged solve of a poisoned field.

The device solvers follow the same rules (NaN-sticky fused norms,
`outer_finish` in csrc/solver.cu); these tests pin the oracle they are
compared against.  No fault reaches a GPU here.
"""
import numpy as np
import pytest

import problems as P
from mushy_gb300 import abi
from oracle import oracle as O


def _hc(seed=41, newton=False):
    g = P.grid((32, 32))
    p = P.mushy_params()
    phi_bc, der = P.hc_bcs("mixed")
    rng = np.random.default_rng(seed)
    phi = P.hc_state(g, rng, regimes=False)
    if newton:
        phi[0] = rng.uniform(4.6, 6.4, phi[0].shape)
    b = [np.stack([-np.ones(abi.face_shape(g, d)), -0.01 * np.ones(abi.face_shape(g, d))])
         for d in range(2)]
    return g, p, phi_bc, der, phi, b, rng


def _hc_solve(g, p, phi_bc, der, b, phi0, rhs, **opts):
    o = O.default_options(1)
    for k, v in opts.items():
        setattr(o, k, v)
    ref = O.NLOpHost(g, p, phi_bc, der, 1.0, -1e-3, None, b)
    sol, st, rc = O.hc_solve(ref, o, phi0, rhs)
    return sol, st, rc


@pytest.mark.parametrize("where", ["rhs", "phi", "face"])
@pytest.mark.parametrize("bad", [np.nan, np.inf])
def test_hc_solve_reports_non_finite_input(where, bad):
    g, p, phi_bc, der, phi, b, _ = _hc()
    rhs = phi.copy()
    phi0 = phi.copy()
    if where == "rhs":
        rhs[0, 0, 5, 7] = bad
    elif where == "phi":
        phi0[1, 0, 3, 3] = bad
    else:
        b = [x.copy() for x in b]
        b[0][0, 0, 4, 4] = bad
    _, st, rc = _hc_solve(g, p, phi_bc, der, b, phi0, rhs)
    assert rc == abi.ERR_NAN and st.exit_status == 8 and st.iterations == 0
    assert not np.isfinite(st.initial_norm)


def test_hc_solve_iteration_cap_and_hang():
    g, p, phi_bc, der, phi, b, _ = _hc()
    _, st, rc = _hc_solve(g, p, phi_bc, der, b, phi, phi + 0.01)
    assert rc == abi.OK and st.exit_status == 0
    assert st.final_norm <= 1e-10 * st.initial_norm
    _, st, rc = _hc_solve(g, p, phi_bc, der, b, phi, phi + 0.01, max_iter=1, tolerance=1e-14)
    assert rc == abi.ERR_NOT_CONVERGED and st.exit_status == 4 and st.iterations == 1
    # demanding a 95% reduction per iteration: the FAS cycle stalls
    _, st, rc = _hc_solve(g, p, phi_bc, der, b, phi, phi + 0.01, hang=0.95, tolerance=1e-14,
                          max_iter=50)
    assert rc == abi.ERR_HANG and st.exit_status == 2
    assert st.final_norm > 0.05 * st.norm_history[st.iterations - 1]


def _vc(bb_edit=None, f_edit=None):
    g, chi, perm, u = P.projection_problem((64, 64), 5, sigma=8.0)
    b = [-f for f in O.face_geomean(g, perm)]
    f = O.mac_divergence(g, u)
    f -= f.mean()
    if bb_edit:
        b = bb_edit(b)
    if f_edit:
        f = f_edit(f)
    o = O.default_options(0)
    o.tolerance, o.max_iter = 1e-10, 40
    ref = O.VCOpHost(g, abi.make_bc(), 0.0, 1.0, None, b)
    sol, st, rc = O.vc_solve(ref, o, np.zeros_like(f), f)
    return sol, st, rc


def test_vc_solve_statuses_under_faults():
    sol, st, rc = _vc()
    assert rc == abi.OK and st.exit_status == 0 and np.isfinite(sol).all()

    def nan_rhs(f):
        f = f.copy()
        f[..., 3, 3] = np.nan
        return f

    def nan_face(b):
        b = [x.copy() for x in b]
        b[1][..., 10, 20] = np.nan
        return b

    for kw in ({"f_edit": nan_rhs}, {"bb_edit": nan_face}):
        _, st, rc = _vc(**kw)
        assert rc == abi.ERR_NAN and st.exit_status == 8 and st.iterations == 0, kw
    # zero permeability everywhere: the diagonal vanishes, the first sweep
    # divides by it and the next norm is non-finite
    _, st, rc = _vc(bb_edit=lambda b: [0.0 * x for x in b])
    assert rc == abi.ERR_NAN and st.exit_status == 8 and st.iterations == 1
    assert np.isfinite(st.initial_norm)


def test_newton_and_adjoint_statuses_under_faults():
    g, p, phi_bc, der, phi, b, rng = _hc(seed=41, newton=True)
    ref = O.NLOpHost(g, p, phi_bc, der, 1.0, -2e-3, None, b)
    o = O.default_options(1)
    o.tolerance, o.hang, o.max_iter = 1e-12, -1.0, 100
    rhs = phi.copy()
    rhs[0, 0, 5, 7] = np.nan
    _, st, rc = O.newton_solve(ref, o, phi, rhs)
    assert rc == abi.ERR_NAN and st.exit_status == 8 and st.iterations == 0
    _, st, rc = O.newton_solve(ref, o, phi, phi.copy())
    assert rc == abi.OK and st.exit_status == 0
    o.max_iter = 1
    _, st, rc = O.newton_solve(ref, o, phi, phi.copy())
    assert rc == abi.ERR_NOT_CONVERGED and st.exit_status == 4 and st.iterations == 1

    gg = rng.standard_normal(phi.shape)
    o = O.default_options(1)
    o.tolerance, o.max_iter = 1e-12, 40
    y, st, rc = O.adjoint_solve(ref, o, phi, gg)
    assert rc == abi.OK and np.isfinite(y).all()
    o.max_iter = 2
    _, st, rc = O.adjoint_solve(ref, o, phi, gg)
    assert rc == abi.ERR_NOT_CONVERGED and st.exit_status == 4 and st.iterations == 2
    gg[1, 0, 2, 2] = np.nan
    o.max_iter = 40
    _, st, rc = O.adjoint_solve(ref, o, phi, gg)
    assert rc == abi.ERR_NAN and st.exit_status == 8 and st.iterations == 0
