"""Converged nonlinear (H, C) solves in mixed precision.

The reference's FAS smoother divides by the diagonal of the diffusion
operator alone and ignores dT/dH, so with its 10-iteration cap the (H, C)
backward-Euler steps of the 64x64 and 1024x1024 configurations stop short of
1e-10.  Newton's method on the Jacobian multigrid (block red/black smoother
with each cell's exact 2x2 diagonal block, closure derivative included)
reaches it.  The mixed-precision Newton runs those linear cycles in FP32;
the Newton residual, its norm, the closure and the update stay FP64, so its
fixed point is the FP64 one.  Checked here:

* every step ends with status 0 at 1e-10 of its initial residual, in FP64
  and in mixed precision;
* the oracle's FP64 residual of the mixed solution is below 1e-10 of the
  initial one;
* mixed and FP64 states agree to 1e-8 of the field scale;
* the FP64 Newton step agrees with the oracle's Newton driver to 1e-10.
"""
import numpy as np
import pytest

import problems as P
from mushy_gb300 import abi
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from test_gpu_parity import dev, host  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import __graft_entry__
    __graft_entry__.build()
    yield


def _opts(prec):
    from mushy_gb300 import ops
    o = ops.default_options(True)
    o.tolerance, o.hang, o.max_iter, o.precision = 1e-10, -1.0, 60, prec
    return o


def _c1():
    g = P.grid((64, 64))
    prm = abi.make_params(stefan=5.0, compositionRatio=5.0, waterDistributionCoeff=1e-3,
                          specificHeatRatio=1.0, heatConductivityRatio=1.0)
    phi_bc = abi.make_bc()
    der = abi.make_bc({(1, 0, 0): (abi.BC_DIRICHLET, -1.0), (1, 1, 0): (abi.BC_DIRICHLET, 0.5),
                       (1, 0, 1): (abi.BC_DIRICHLET, -1.0), (1, 1, 1): (abi.BC_DIRICHLET, -1.0)})
    phi0 = np.empty((2,) + abi.cell_shape(g))
    phi0[0], phi0[1] = 6.0, -1.0
    b = [np.stack([-np.ones(abi.face_shape(g, d)), np.zeros(abi.face_shape(g, d))])
         for d in range(2)]
    return g, prm, phi_bc, der, phi0, b


def test_c1_newton_steps_converge_mixed_matches_fp64():
    from mushy_gb300 import ops
    g, prm, phi_bc, der, phi0, b = _c1()
    dt = 1e-3
    op = ops.NLMultiCompOp(g, prm, phi_bc, der, 1.0, -dt, None, [dev(x) for x in b])
    ref = O.NLOpHost(g, prm, phi_bc, der, 1.0, -dt, None, b)
    S64 = ops.AdjointMultiGrid(op, _opts(abi.PREC_F64))
    SM = ops.AdjointMultiGrid(op, _opts(abi.PREC_MIXED))
    oo = O.default_options(1)
    oo.tolerance, oo.hang, oo.max_iter = 1e-10, -1.0, 60
    c64, cm, h = dev(phi0), dev(phi0), phi0.copy()
    for step in range(10):
        n64, nm = c64.clone(), cm.clone()
        st64, rc64 = S64.backwardEulerNewton(n64, c64, dt)
        stm, rcm = SM.backwardEulerNewton(nm, cm, dt)
        assert rc64 == 0 and rcm == 0, (step, rc64, rcm)
        assert st64.final_norm <= 1e-10 * st64.initial_norm
        assert stm.final_norm <= 1e-10 * stm.initial_norm
        u64, um = host(n64), host(nm)
        # the oracle's residual of the mixed state, and its Newton step
        r0 = O.norm(O.nl_residual(ref, host(cm), host(cm)))
        assert O.norm(O.nl_residual(ref, um, host(cm))) <= 1e-10 * r0 * 1.0001
        h, st_r, rc_r = O.newton_solve(ref, oo, h, h)
        assert rc_r == 0
        assert np.abs(u64 - h).max() <= 1e-10 * np.abs(h).max(), step
        assert np.abs(um - u64).max() <= 1e-8 * np.abs(u64).max(), step
        c64, cm = n64, nm


def test_fp64_lean_cycles_2d_match_reference_order():
    """The FP64 Newton on the lean kernels (options.fuse_levels = 2) against
    the FP64 Newton in the reference's expression order, 2D 64^2 config:
    both converge, same FP64 fixed point to 1e-11."""
    from mushy_gb300 import ops
    g, prm, phi_bc, der, phi0, b = _c1()
    dt = 1e-3
    op = ops.NLMultiCompOp(g, prm, phi_bc, der, 1.0, -dt, None, [dev(x) for x in b])
    out = []
    for fuse in (1, 2):
        o = _opts(abi.PREC_F64)
        o.fuse_levels = fuse
        new = dev(phi0)
        st, rc = ops.AdjointMultiGrid(op, o).backwardEulerNewton(new, dev(phi0), dt)
        assert rc == 0 and st.final_norm <= 1e-10 * st.initial_norm
        out.append(host(new))
    assert np.abs(out[1] - out[0]).max() <= 1e-11 * np.abs(out[0]).max()


def test_c3_size_newton_step_mixed_matches_fp64():
    """One backward-Euler (H, C) step of the 1024x1024 mushy-layer
    configuration (CR=25, Le=200, liquid + 1e-3 noise, cold bottom,
    dt=1e-5) to 1e-10, FP64 and mixed."""
    from mushy_gb300 import ops
    n, dt = 1024, 1e-5
    g = P.grid((n, n))
    rng = np.random.default_rng(3)
    prm = abi.make_params(stefan=5.0, compositionRatio=25.0, waterDistributionCoeff=1e-3,
                          specificHeatRatio=1.0, heatConductivityRatio=1.0)
    phi_bc = abi.make_bc()
    der = abi.make_bc({(1, 0, 0): (abi.BC_DIRICHLET, -1.0), (1, 0, 1): (abi.BC_DIRICHLET, -1.0)})
    phi0 = np.empty((2,) + abi.cell_shape(g))
    phi0[0] = 6.0 + 1e-3 * rng.standard_normal(abi.cell_shape(g))
    phi0[1] = -1.0 + 1e-3 * rng.standard_normal(abi.cell_shape(g))
    b = [np.stack([-np.ones(abi.face_shape(g, d)), -np.full(abi.face_shape(g, d), 1.0 / 200)])
         for d in range(2)]
    op = ops.NLMultiCompOp(g, prm, phi_bc, der, 1.0, -dt, None, [dev(x) for x in b])
    out = {}
    for prec in (abi.PREC_F64, abi.PREC_MIXED):
        new = dev(phi0)
        st, rc = ops.AdjointMultiGrid(op, _opts(prec)).backwardEulerNewton(new, dev(phi0), dt)
        assert rc == 0, (prec, rc, st.iterations)
        assert st.final_norm <= 1e-10 * st.initial_norm
        out[prec] = host(new)
    ref = O.NLOpHost(g, prm, phi_bc, der, 1.0, -dt, None, b)
    r0 = O.norm(O.nl_residual(ref, phi0, phi0))
    assert O.norm(O.nl_residual(ref, out[abi.PREC_MIXED], phi0)) <= 1e-10 * r0 * 1.0001
    u64 = out[abi.PREC_F64]
    assert np.abs(out[abi.PREC_MIXED] - u64).max() <= 1e-8 * np.abs(u64).max()


def _c4_like(n):
    """A 3D box like the 256^3 benchmark step (periodic x / y, cold bottom
    wall, H falling from 6 at the top to 2 at the bottom with 1e-2 noise)."""
    from mushy_gb300 import ops
    rng = np.random.default_rng(4)
    g = abi.make_grid([n, n, n], 1.0 / n, (1, 1, 0))
    z = (np.arange(n) + 0.5) / n
    phi0 = np.empty((2, n, n, n))
    phi0[0] = 6.0 - 4.0 * (1.0 - z)[:, None, None] * (1.0 + 1e-2 * rng.standard_normal((n, n, n)))
    phi0[1] = -1.0
    prm = abi.make_params(stefan=5.0, compositionRatio=5.0, waterDistributionCoeff=1e-3,
                          specificHeatRatio=1.0, heatConductivityRatio=1.0)
    der = abi.make_bc({(2, 0, 0): (abi.BC_DIRICHLET, -1.0), (2, 0, 1): (abi.BC_DIRICHLET, -1.0)})
    b = [np.stack([-np.ones(abi.face_shape(g, d)), np.full(abi.face_shape(g, d), -1e-2)])
         for d in range(3)]
    dt = 1e-4
    op = ops.NLMultiCompOp(g, prm, abi.make_bc(), der, 1.0, -dt, None, [dev(x) for x in b])
    ref = O.NLOpHost(g, prm, abi.make_bc(), der, 1.0, -dt, None, b)
    return g, phi0, op, ref, dt


def test_3d_newton_step_split_layout_converged():
    """64^3 (the lean cycles' arrays colour-split on every smoothed level):
    the mixed step reaches 1e-10 under the oracle's residual, within 1e-8 of
    FP64 Newton; the FP64 path on the lean kernels takes the same Newton
    steps and cycles as the FP64 path in the reference's expression order
    and reaches the same FP64 solution to 1e-11."""
    from mushy_gb300 import ops
    g, phi0, op, ref, dt = _c4_like(64)
    out = {}
    for key, prec, fuse in (("mixed", abi.PREC_MIXED, 1), ("fp64", abi.PREC_F64, 1),
                            ("fp64_fast", abi.PREC_F64, 2)):
        o = _opts(prec)
        o.fuse_levels = fuse
        new = dev(phi0)
        st, rc = ops.AdjointMultiGrid(op, o).backwardEulerNewton(new, dev(phi0), dt)
        assert rc == 0, (key, rc, st.iterations)
        assert st.final_norm <= 1e-10 * st.initial_norm
        out[key] = (host(new), st)
    um = out["mixed"][0]
    r0 = O.norm(O.nl_residual(ref, phi0, phi0))
    assert O.norm(O.nl_residual(ref, um, phi0)) <= 1e-10 * r0 * 1.0001
    u64, s64 = out["fp64"]
    assert np.abs(um - u64).max() <= 1e-8 * np.abs(u64).max()
    uf, sf = out["fp64_fast"]
    assert sf.iterations == s64.iterations and sf.cycles == s64.cycles
    assert np.abs(uf - u64).max() <= 1e-11 * np.abs(u64).max()


@pytest.mark.parametrize("shape", [(5, 3), (9, 7)])
def test_one_level_hierarchy_natural_layout(shape):
    """Grids that do not coarsen (one level, the bottom's: natural layout,
    direct solve at 15 cells, relaxation at 63): the mixed and the lean FP64
    Newton steps converge to the FP64 solution."""
    from mushy_gb300 import ops
    g = P.grid(shape)
    rng = np.random.default_rng(7)
    prm = abi.make_params(stefan=5.0, compositionRatio=5.0, waterDistributionCoeff=1e-3,
                          specificHeatRatio=1.0, heatConductivityRatio=1.0)
    der = abi.make_bc({(1, 0, 0): (abi.BC_DIRICHLET, -1.0), (1, 0, 1): (abi.BC_DIRICHLET, -1.0)})
    phi0 = np.empty((2,) + abi.cell_shape(g))
    phi0[0] = 5.0 + 0.5 * rng.standard_normal(abi.cell_shape(g))
    phi0[1] = -1.0
    b = [np.stack([-np.ones(abi.face_shape(g, d)), np.full(abi.face_shape(g, d), -1e-2)])
         for d in range(2)]
    dt = 1e-2
    op = ops.NLMultiCompOp(g, prm, abi.make_bc(), der, 1.0, -dt, None, [dev(x) for x in b])
    out = {}
    for key, prec, fuse in (("mixed", abi.PREC_MIXED, 1), ("fp64", abi.PREC_F64, 1),
                            ("fp64_fast", abi.PREC_F64, 2)):
        o = _opts(prec)
        o.fuse_levels = fuse
        new = dev(phi0)
        st, rc = ops.AdjointMultiGrid(op, o).backwardEulerNewton(new, dev(phi0), dt)
        assert rc == 0, (key, rc, st.iterations)
        assert st.levels == 1
        assert st.final_norm <= 1e-10 * st.initial_norm
        out[key] = host(new)
    u64 = out["fp64"]
    assert np.abs(out["mixed"] - u64).max() <= 1e-8 * np.abs(u64).max()
    assert np.abs(out["fp64_fast"] - u64).max() <= 1e-11 * np.abs(u64).max()


@pytest.mark.parametrize("prec,fuse", [(abi.PREC_MIXED, 1), (abi.PREC_F64, 2)])
@pytest.mark.parametrize("case", ["3d_periodic_xy", "2d_walls"])
def test_vector_half_sweeps_same_bits(prec, fuse, case):
    """The lean cycles' vector-load half sweeps (4 FP32 / 2 FP64 cells per
    thread) against one cell per thread: the same Newton steps, cycles and
    solution bits (3D periodic x / y with walls in z; 2D walls all round)."""
    from mushy_gb300 import ops
    if case == "3d_periodic_xy":
        g, phi0, op, ref, dt = _c4_like(32)
    else:
        g, prm, phi_bc, der, phi0, b = _c1()
        dt = 1e-3
        op = ops.NLMultiCompOp(g, prm, phi_bc, der, 1.0, -dt, None, [dev(x) for x in b])
    out = []
    for vec in (0, 1):
        o = _opts(prec)
        o.fuse_levels = fuse
        S = ops.AdjointMultiGrid(op, o)
        S.setNewtonParams(vector_sweeps=vec)
        new = dev(phi0)
        st, rc = S.backwardEulerNewton(new, dev(phi0), dt)
        assert rc == 0 and st.final_norm <= 1e-10 * st.initial_norm
        out.append((host(new), st.iterations, st.cycles))
    assert out[0][1:] == out[1][1:]
    assert np.array_equal(out[0][0], out[1][0])


@pytest.mark.parametrize("shape,per", [((32, 24, 40), (0, 0, 1)), ((36, 32, 32), (1, 0, 0)),
                                       ((48, 40, 1), (1, 0, 0))])
def test_lean_layouts_walls_and_rows(shape, per):
    """The lean cycles on other box shapes: walls in x with a periodic z
    (the vector sweep's wall ends), a level-0 row of 18 cells per colour (the
    one-cell-per-thread sweep), a 2D box periodic in x; mixed and lean FP64
    Newton steps converge to the FP64 solution."""
    from mushy_gb300 import ops
    dim = 3 if shape[2] > 1 else 2
    n = list(shape[:dim])
    g = abi.make_grid(n, 1.0 / n[0], per)
    rng = np.random.default_rng(31)
    cs = abi.cell_shape(g)
    prm = abi.make_params(stefan=5.0, compositionRatio=5.0, waterDistributionCoeff=1e-3,
                          specificHeatRatio=1.0)
    wall = dim - 1 if not per[dim - 1] else 0
    der = abi.make_bc({(wall, 0, 0): (abi.BC_DIRICHLET, -1.0), (wall, 0, 1): (abi.BC_DIRICHLET, -1.0)})
    phi0 = np.empty((2,) + cs)
    phi0[0] = 5.0 + 0.8 * rng.standard_normal(cs)
    phi0[1] = -1.0
    b = [np.stack([-np.ones(abi.face_shape(g, d)), np.full(abi.face_shape(g, d), -1e-2)])
         for d in range(dim)]
    dt = 2e-3
    op = ops.NLMultiCompOp(g, prm, abi.make_bc(), der, 1.0, -dt, None, [dev(x) for x in b])
    ref = O.NLOpHost(g, prm, abi.make_bc(), der, 1.0, -dt, None, b)
    out = {}
    for key, prec, fuse in (("mixed", abi.PREC_MIXED, 1), ("fp64", abi.PREC_F64, 1),
                            ("fp64_fast", abi.PREC_F64, 2)):
        o = _opts(prec)
        o.fuse_levels = fuse
        new = dev(phi0)
        st, rc = ops.AdjointMultiGrid(op, o).backwardEulerNewton(new, dev(phi0), dt)
        assert rc == 0, (key, rc, st.iterations)
        assert st.levels >= 2
        out[key] = host(new)
    u64 = out["fp64"]
    r0 = O.norm(O.nl_residual(ref, phi0, phi0))
    assert O.norm(O.nl_residual(ref, out["mixed"], phi0)) <= 1e-10 * r0 * 1.0001
    assert np.abs(out["mixed"] - u64).max() <= 1e-8 * np.abs(u64).max()
    assert np.abs(out["fp64_fast"] - u64).max() <= 1e-11 * np.abs(u64).max()
