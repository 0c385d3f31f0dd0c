"""BiCGStab bottom solver of the linear multigrid (projection and
Darcy-Brinkman operators) against its oracle restatement.

The bottom solve is one thread block in FP64 with every dot product in a
fixed lane order the oracle reproduces, so the FP64 solves are bitwise
equal: iteration counts, status, residual-norm histories and solutions.
Boxes whose whole hierarchy is one level make every outer iteration a
BiCGStab solve; the others put it at the coarsest of several levels.  The
mixed-precision solver keeps its coarsest solve in FP64 through the same
kernel and must reach the FP64 solution to 1e-8.
"""
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


def _hist(st):
    return [st.norm_history[i] for i in range(min(st.iterations, 63) + 1)]


CASES = [((16, 16), 16, False), ((12, 8), 4, True), ((8, 8, 8), 8, False), ((48, 32), 2, False),
         ((64, 64), 2, True), ((16, 8, 8), 2, False)]


@pytest.mark.parametrize("n,max_coarse,with_c", CASES)
def test_bicgstab_bottom_bitwise(n, max_coarse, with_c):
    from mushy_gb300 import ops
    g, chi, perm, u = P.projection_problem(n, 5, sigma=4.0)
    b = [-f for f in O.face_geomean(g, perm)]
    f = O.mac_divergence(g, u)
    f -= f.mean()
    rng = np.random.default_rng(7)
    if with_c:
        # Darcy-Brinkman: (Da^-1 chi / Pi) u - lap u, walls no-slip
        cC = chi / (1e-2 * np.minimum(perm, 1e4))
        bc = abi.make_bc({(d, s, 0): (abi.BC_DIRICHLET, 0.0) for d in range(g.dim)
                          for s in range(2) if not g.periodic[d]})
        ref = O.VCOpHost(g, bc, 0.0, -1.0, None, [-np.ones_like(x) for x in b], cC)
        op = ops.DarcyBrinkmanOp(g, bc, 0.0, -1.0, None, [dev(-np.ones_like(x)) for x in b],
                                 dev(cC))
        f = rng.standard_normal(f.shape)
    else:
        bc = abi.make_bc()
        ref = O.VCOpHost(g, bc, 0.0, 1.0, None, b)
        op = ops.ProjectionOp(g, bc, 0.0, 1.0, None, [dev(x) for x in b])
    opts = O.default_options(0)
    opts.tolerance, opts.hang, opts.max_iter = 1e-10, 1e-15, 60
    opts.max_coarse, opts.bottom_solver = max_coarse, abi.BOTTOM_BICGSTAB
    sol_r, st_r, rc_r = O.vc_solve(ref, opts, np.zeros_like(f), f)
    assert rc_r == 0, (rc_r, st_r.iterations)
    for graph in (0, 1, 2):
        o = ops.default_options(False)
        o.tolerance, o.hang, o.max_iter, o.use_graph = 1e-10, 1e-15, 60, graph
        o.max_coarse, o.bottom_solver = max_coarse, abi.BOTTOM_BICGSTAB
        d_phi = torch.zeros_like(dev(f))
        st, rc = ops.AMRMultiGrid(op, o).solve(d_phi, dev(f))
        assert rc == rc_r and st.iterations == st_r.iterations, (graph, rc, st.iterations)
        assert _hist(st) == _hist(st_r), graph
        assert st.cell_updates == st_r.cell_updates
        exact(host(d_phi), sol_r)
    o = ops.default_options(False)
    o.tolerance, o.hang, o.max_iter, o.precision = 1e-10, 1e-15, 60, abi.PREC_MIXED
    o.max_coarse, o.bottom_solver = max_coarse, abi.BOTTOM_BICGSTAB
    d_m = torch.zeros_like(dev(f))
    st_m, rc_m = ops.AMRMultiGrid(op, o).solve(d_m, dev(f))
    assert rc_m == 0
    m = host(d_m)
    a = sol_r
    if not with_c:
        a, m = a - a.mean(), m - m.mean()
    assert np.abs(a - m).max() <= 1e-8 * np.abs(a).max()


def test_bicgstab_refused_by_fas_and_jacobian_solvers():
    from mushy_gb300 import ops
    g = P.grid((16, 16))
    p = P.mushy_params()
    phi_bc, der = P.hc_bcs("mixed")
    b = [dev(-np.ones((2,) + abi.face_shape(g, d))) for d in range(2)]
    op = ops.NLMultiCompOp(g, p, phi_bc, der, 1.0, -1e-3, None, b)
    o = ops.default_options(True)
    o.bottom_solver = abi.BOTTOM_BICGSTAB
    for cls in (ops.AMRFASMultiGrid, ops.AdjointMultiGrid):
        with pytest.raises(RuntimeError):
            cls(op, o)
