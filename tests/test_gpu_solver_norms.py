"""Residual norms of the device solvers against the oracle's.

Every solver decides convergence on a fused FP64 residual norm: one partial
per thread block, combined by a finalize kernel.  These tests put the
largest residual in the last rows of the grid (a cold wall on top, so it
lies outside the first quarter of the cells) and check, with no iteration
cap in the way, that the norms the solvers report are the oracle's:

* FP64 FAS (H, C), FP64 linear multigrid, adjoint multigrid: initial norm,
  final norm and the whole norm history bit for bit (max norm: the result
  does not depend on the order in which the partials are combined), with the
  same iteration count and the same solution;
* mixed-precision (H, C) and Newton: the initial norm bit for bit, and the
  final norm equal to the oracle's max norm of the residual of the solution
  the device returned;
* mixed-precision linear multigrid: the initial norm bit for bit, the final
  norm within 1e-4 of the oracle's (its FP64 outer residual is the lean
  fused-multiply-add form, not the reference's expression order).
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


def _history(st):
    return [st.norm_history[i] for i in range(min(st.iterations, 63) + 1)]


def _same_norms(st, st_r):
    assert st.iterations == st_r.iterations, (st.iterations, st_r.iterations)
    assert st.initial_norm == st_r.initial_norm, (st.initial_norm, st_r.initial_norm)
    assert st.final_norm == st_r.final_norm, (st.final_norm, st_r.final_norm)
    assert _history(st) == _history(st_r), (_history(st), _history(st_r))


def _cold_top(n, dt, seed=7):
    """Liquid (H, C) near the liquidus under a cold top wall (T = C_l = -1),
    no-flux bottom and sides: the largest residual is in the top row."""
    g = P.grid((n, n))
    p = P.mushy_params()
    phi_bc = abi.make_bc()
    der = abi.make_bc({(1, 1, 0): (abi.BC_DIRICHLET, -1.0), (1, 1, 1): (abi.BC_DIRICHLET, -1.0)})
    rng = np.random.default_rng(seed)
    phi = P.hc_state(g, rng, regimes=False)
    b = [np.stack([-np.ones(abi.face_shape(g, d)), -0.01 * np.ones(abi.face_shape(g, d))])
         for d in range(2)]
    ref = O.NLOpHost(g, p, phi_bc, der, 1.0, -dt, None, b)
    r0 = O.nl_residual(ref, phi, phi)
    q = int(np.abs(r0).reshape(2, -1).max(axis=0).argmax())
    assert q >= 3 * g.n[0] * g.n[1] // 4, "largest residual must be in the last quarter"
    return g, p, phi_bc, der, phi, b, ref


# hang = -1 keeps the reference's stall test from ending the 256^2 solve at
# its early bump (27 -> 3.3 -> 5.4 -> 2.7 -> ... -> 1.6e-9)
@pytest.mark.parametrize("n,dt", [(64, 1e-3), (256, 1e-4)])
def test_fas_norms_bitwise(n, dt):
    from mushy_gb300 import ops
    g, p, phi_bc, der, phi, b, ref = _cold_top(n, dt)
    opts = O.default_options(1)
    opts.tolerance, opts.max_iter, opts.hang = 1e-10, 100, -1.0
    sol_r, st_r, rc_r = O.hc_solve(ref, opts, phi, phi.copy())
    assert rc_r == 0 and st_r.iterations > 10
    op = ops.NLMultiCompOp(g, p, phi_bc, der, 1.0, -dt, None, [dev(x) for x in b])
    for graph in (0, 1):
        o = ops.default_options(True)
        o.tolerance, o.max_iter, o.hang, o.use_graph = 1e-10, 100, -1.0, graph
        d_phi = dev(phi)
        st, rc = ops.AMRFASMultiGrid(op, o).solve(d_phi, dev(phi))
        assert rc == rc_r
        _same_norms(st, st_r)
        exact(host(d_phi), sol_r)


@pytest.mark.parametrize("n,dt", [(64, 1e-3), (256, 1e-4)])
def test_mixed_hc_norms_match_oracle_residual(n, dt):
    from mushy_gb300 import ops
    g, p, phi_bc, der, phi, b, ref = _cold_top(n, dt)
    opts = O.default_options(1)
    opts.tolerance, opts.max_iter, opts.hang = 1e-10, 100, -1.0
    sol_r, st_r, rc_r = O.hc_solve(ref, opts, phi, phi.copy())
    op = ops.NLMultiCompOp(g, p, phi_bc, der, 1.0, -dt, None, [dev(x) for x in b])
    o = ops.default_options(True)
    o.tolerance, o.max_iter, o.hang, o.precision = 1e-10, 100, -1.0, abi.PREC_MIXED
    d_phi = dev(phi)
    st, rc = ops.AMRFASMultiGrid(op, o).solve(d_phi, dev(phi))
    assert rc == 0, (rc, st.iterations, _history(st))
    assert st.initial_norm == st_r.initial_norm
    u = host(d_phi)
    assert st.final_norm == O.norm(O.nl_residual(ref, u, phi))
    assert st.final_norm <= 1e-10 * st.initial_norm
    assert np.abs(u - sol_r).max() <= 1e-8 * np.abs(sol_r).max()


@pytest.mark.parametrize("n,seed", [((64, 64), 5), ((256, 128), 9)])
def test_linear_mg_norms(n, seed):
    from mushy_gb300 import ops
    g, chi, perm, u = P.projection_problem(n, seed, sigma=8.0)
    b = [-f for f in O.face_geomean(g, perm)]
    f = O.mac_divergence(g, u)
    f -= f.mean()
    ny, nx = f.shape[-2:]
    f[..., ny - 3, nx // 2] += 50.0 * np.abs(f).max()  # largest residual in the top rows
    f -= f.mean()
    assert int(np.abs(f).argmax()) >= 3 * f.size // 4
    bc = abi.make_bc()
    ref = O.VCOpHost(g, bc, 0.0, 1.0, None, b)
    opts = O.default_options(0)
    opts.tolerance, opts.hang, opts.max_iter = 1e-10, 1e-15, 300
    sol_r, st_r, rc_r = O.vc_solve(ref, opts, np.zeros_like(f), f)
    assert rc_r == 0
    op = ops.ProjectionOp(g, bc, 0.0, 1.0, None, [dev(x) for x in b])
    for graph in (0, 1, 2):
        o = ops.default_options(False)
        o.tolerance, o.hang, o.max_iter, o.use_graph = 1e-10, 1e-15, 300, graph
        d_phi = torch.zeros_like(dev(f))
        st, rc = ops.AMRMultiGrid(op, o).solve(d_phi, dev(f))
        assert rc == rc_r
        _same_norms(st, st_r)
        exact(host(d_phi), sol_r)
    o = ops.default_options(False)
    o.tolerance, o.hang, o.max_iter, o.precision = 1e-10, 1e-15, 300, abi.PREC_MIXED
    d_phi = torch.zeros_like(dev(f))
    st, rc = ops.AMRMultiGrid(op, o).solve(d_phi, dev(f))
    assert rc == 0
    assert st.initial_norm == st_r.initial_norm
    r1 = O.norm(O.vc_residual(ref, host(d_phi), f))
    assert abs(st.final_norm - r1) <= 1e-4 * r1 + 1e-15 * st.initial_norm
    assert r1 <= 1.01e-10 * st.initial_norm


def test_newton_norms_match_oracle_residual():
    from mushy_gb300 import ops
    g, p, phi_bc, der, phi, b, ref = _cold_top(64, 2e-3, seed=11)
    opts = O.default_options(1)
    opts.tolerance, opts.hang, opts.max_iter = 1e-12, -1.0, 100
    u_r, st_r, rc_r = O.newton_solve(ref, opts, phi, phi.copy())
    op = ops.NLMultiCompOp(g, p, phi_bc, der, 1.0, -2e-3, None, [dev(x) for x in b])
    o = ops.default_options(True)
    o.tolerance, o.hang, o.max_iter = 1e-12, -1.0, 100
    d_u = dev(phi)
    st, rc = ops.AdjointMultiGrid(op, o).newtonSolve(d_u, dev(phi))
    assert rc == rc_r == 0
    assert st.initial_norm == st_r.initial_norm
    u = host(d_u)
    assert st.final_norm == O.norm(O.nl_residual(ref, u, phi))
    assert np.abs(u - u_r).max() <= 1e-10 * np.abs(u_r).max()


def test_adjoint_norms_bitwise():
    from mushy_gb300 import ops
    g, p, phi_bc, der, phi, b, ref = _cold_top(64, 1e-3, seed=12)
    rng = np.random.default_rng(12)
    gg = rng.standard_normal(phi.shape)
    gg[:, :, -2, 5] += 40.0  # largest right-hand side in the top rows
    opts = O.default_options(1)
    opts.tolerance, opts.max_iter = 1e-12, 60
    y_r, st_r, rc_r = O.adjoint_solve(ref, opts, phi, gg)
    assert rc_r == 0
    op = ops.NLMultiCompOp(g, p, phi_bc, der, 1.0, -1e-3, None, [dev(x) for x in b])
    o = ops.default_options(True)
    o.tolerance, o.max_iter = 1e-12, 60
    A = ops.AdjointMultiGrid(op, o)
    st = abi.SolveStats()
    # the device arrays are held for the whole call (a temporary passed
    # straight to ops._ptr would be freed, and its block handed to the next
    # tensor, before the library reads it)
    d_phi, d_g, d_y = dev(phi), dev(gg), dev(np.zeros_like(phi))
    rc = abi.load().mlgpu_hc_adjoint_solve(A.h, ops._ptr(d_phi), ops._ptr(d_g), ops._ptr(d_y),
                                           C.byref(st))
    assert rc == rc_r
    _same_norms(st, st_r)
    exact(host(d_y), y_r)
