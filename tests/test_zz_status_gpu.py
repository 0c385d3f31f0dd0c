"""Failure detection on the device, faults injected on the host: the sm_103a
solvers return the oracle's status code, exit status and iteration count
for a NaN / Inf in the right-hand side, the initial guess or a face
coefficient, zeroed permeability faces, an iteration cap and a stalled solve
(every kernel computes through the non-finite values; no wait, index or
trap depends on them).  The finite cases also match the oracle bit for bit.
The statuses are read through the C ABI on the solver handle; the Python
mirror turns MLGPU_ERR_NAN into a RuntimeError, checked once.
"""
import ctypes as C

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


def _hc_case(seed=41, newton=False):
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


def _raw(fn, h, *arrays):
    from mushy_gb300 import ops
    st = abi.SolveStats()
    rc = fn(h, *[ops._ptr(a) for a in arrays], C.byref(st))
    return st, rc


def _same(st, rc, st_r, rc_r):
    assert rc == rc_r and st.exit_status == st_r.exit_status, (rc, rc_r, st.exit_status)
    assert st.iterations == st_r.iterations, (st.iterations, st_r.iterations)


@pytest.mark.parametrize("case", ["nan_rhs", "inf_rhs", "nan_phi", "nan_face", "cap", "hang"])
def test_hc_solve_status_matches_oracle(case):
    from mushy_gb300 import ops
    g, p, phi_bc, der, phi, b, _ = _hc_case()
    phi0, rhs = phi.copy(), phi + 0.01
    kw = {}
    if case == "nan_rhs":
        rhs[0, 0, 5, 7] = np.nan
    elif case == "inf_rhs":
        rhs[1, 0, 9, 2] = np.inf
    elif case == "nan_phi":
        phi0[1, 0, 3, 3] = np.nan
    elif case == "nan_face":
        b = [x.copy() for x in b]
        b[0][0, 0, 4, 4] = np.nan
    elif case == "cap":
        kw = dict(max_iter=1, tolerance=1e-14)
    else:
        kw = dict(hang=0.95, tolerance=1e-14, max_iter=50)
    opts = O.default_options(1)
    for k, v in kw.items():
        setattr(opts, k, v)
    ref = O.NLOpHost(g, p, phi_bc, der, 1.0, -1e-3, None, b)
    sol_r, st_r, rc_r = O.hc_solve(ref, opts, phi0, rhs)
    op = ops.NLMultiCompOp(g, p, phi_bc, der, 1.0, -1e-3, None, [dev(x) for x in b])
    for graph in (0, 1):
        o = ops.default_options(True)
        o.use_graph = graph
        for k, v in kw.items():
            setattr(o, k, v)
        d_phi = dev(phi0)
        S = ops.AMRFASMultiGrid(op, o)
        st, rc = _raw(abi.load().mlgpu_solver_solve, S.h, d_phi, dev(rhs))
        _same(st, rc, st_r, rc_r)
        if rc != abi.ERR_NAN:
            exact(host(d_phi), sol_r)
    if case.startswith(("nan", "inf")):
        assert rc_r == abi.ERR_NAN and st_r.exit_status == 8
        with pytest.raises(RuntimeError, match="NaN"):
            S.solve(dev(phi0), dev(rhs))


@pytest.mark.parametrize("case", ["nan_rhs", "nan_face", "zero_faces"])
def test_vc_solve_status_matches_oracle(case):
    from mushy_gb300 import ops
    g, chi, perm, u = P.projection_problem((64, 64), 5, sigma=8.0)
    b = [-f for f in O.face_geomean(g, perm)]
    f = O.mac_divergence(g, u)
    f -= f.mean()
    if case == "nan_rhs":
        f[..., 3, 3] = np.nan
    elif case == "nan_face":
        b[1][..., 10, 20] = np.nan
    else:
        b = [0.0 * x for x in b]
    bc = abi.make_bc()
    opts = O.default_options(0)
    opts.tolerance, opts.max_iter = 1e-10, 40
    ref = O.VCOpHost(g, bc, 0.0, 1.0, None, b)
    _, st_r, rc_r = O.vc_solve(ref, opts, np.zeros_like(f), f)
    assert rc_r == abi.ERR_NAN and st_r.exit_status == 8
    op = ops.ProjectionOp(g, bc, 0.0, 1.0, None, [dev(x) for x in b])
    for graph in (0, 1, 2):
        o = ops.default_options(False)
        o.tolerance, o.max_iter, o.use_graph = 1e-10, 40, graph
        d_phi = torch.zeros_like(dev(f))
        S = ops.AMRMultiGrid(op, o)
        st, rc = _raw(abi.load().mlgpu_solver_solve, S.h, d_phi, dev(f))
        _same(st, rc, st_r, rc_r)


def test_newton_and_adjoint_status_match_oracle():
    from mushy_gb300 import ops
    g, p, phi_bc, der, phi, b, rng = _hc_case(newton=True)
    ref = O.NLOpHost(g, p, phi_bc, der, 1.0, -2e-3, None, b)
    op = ops.NLMultiCompOp(g, p, phi_bc, der, 1.0, -2e-3, None, [dev(x) for x in b])
    rhs = phi.copy()
    rhs[0, 0, 5, 7] = np.nan
    for max_iter, f in ((100, rhs), (1, phi)):
        opts = O.default_options(1)
        opts.tolerance, opts.hang, opts.max_iter = 1e-12, -1.0, max_iter
        _, st_r, rc_r = O.newton_solve(ref, opts, phi, f)
        o = ops.default_options(True)
        o.tolerance, o.hang, o.max_iter = 1e-12, -1.0, max_iter
        A = ops.AdjointMultiGrid(op, o)
        st, rc = _raw(abi.load().mlgpu_hc_newton_solve, A.h, dev(phi), dev(f))
        _same(st, rc, st_r, rc_r)
    assert rc == abi.ERR_NOT_CONVERGED
    gg = rng.standard_normal(phi.shape)
    gg[1, 0, 2, 2] = np.nan
    opts = O.default_options(1)
    opts.tolerance, opts.max_iter = 1e-12, 40
    _, st_r, rc_r = O.adjoint_solve(ref, opts, phi, gg)
    o = ops.default_options(True)
    o.tolerance, o.max_iter = 1e-12, 40
    A = ops.AdjointMultiGrid(op, o)
    st, rc = _raw(abi.load().mlgpu_hc_adjoint_solve, A.h, dev(phi), dev(gg),
                  dev(np.zeros_like(phi)))
    _same(st, rc, st_r, rc_r)
    assert rc == abi.ERR_NAN


def test_solve_log_records_device_solves():
    """With a SolveLog installed, each solver call appends one line that
    carries the call's own stats."""
    import io
    import json
    from mushy_gb300 import ops, solvelog
    g, chi, perm, u = P.projection_problem((64, 64), 5, sigma=8.0)
    b = [-f for f in O.face_geomean(g, perm)]
    f = O.mac_divergence(g, u)
    f -= f.mean()
    buf = io.StringIO()
    ops.setSolveLog(solvelog.SolveLog(buf))
    try:
        op = ops.ProjectionOp(g, abi.make_bc(), 0.0, 1.0, None, [dev(x) for x in b])
        o = ops.default_options(False)
        o.tolerance, o.max_iter = 1e-10, 40
        st, rc = ops.AMRMultiGrid(op, o).solve(torch.zeros_like(dev(f)), dev(f))
        gh, p, phi_bc, der, phi, bh, _ = _hc_case()
        hop = ops.NLMultiCompOp(gh, p, phi_bc, der, 1.0, -1e-3, None, [dev(x) for x in bh])
        st2, rc2 = ops.AMRFASMultiGrid(hop).backwardEuler(dev(phi), dev(phi), 1e-3)
    finally:
        ops.setSolveLog(None)
    recs = [json.loads(x) for x in buf.getvalue().splitlines()]
    assert [r["what"] for r in recs] == ["solve", "backwardEuler"]
    for r, s, c in zip(recs, (st, st2), (rc, rc2)):
        assert r["rc"] == c and r["iterations"] == s.iterations
        assert r["cell_updates"] == s.cell_updates and r["seconds"] > 0
        assert r["residual_history"][0] == s.initial_norm
