"""Mixed-precision linear solves on 3D boxes: the lean FP32 cycles
(vc_lean_kernels.cuh: colour-split e and r, the wall ghosts folded into the
diagonal, red-children restriction, black-only prolongation) inside the FP64
defect correction.

Checked against the oracle's FP64 residual of the returned solution (1e-10 of
the initial one), and against the FP64 solve's solution (1e-8 of its scale,
the null-space constant removed where the operator has one), for the
projection operator (periodic x / y, Neumann z; Kozeny-Carman coefficients),
the Darcy-Brinkman operator (a, c coefficients, inhomogeneous Dirichlet /
Neumann walls), the BiCGStab bottom (every level above the bottom lean), a
W-cycle, and no pre- or no post-smoothing.
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


def _projection(n, seed):
    g, chi, perm, u = P.projection_problem((n, n, n), seed, sigma=6.0)
    g = abi.make_grid([n, n, n], 1.0 / n, (1, 1, 0))
    faces = O.face_geomean(g, perm)
    b = [-x for x in faces]
    u = [np.random.default_rng(seed).standard_normal(abi.face_shape(g, d)) for d in range(3)]
    f = O.mac_divergence(g, u)
    f -= f.mean()
    return g, abi.make_bc(), 0.0, 1.0, None, b, None, f


def _darcy(shape, seed):
    rng = np.random.default_rng(seed)
    g = P.grid(shape)
    bc = P.vc_bc("mixed")
    b = [-rng.uniform(0.2, 3.0, abi.face_shape(g, d)) for d in range(3)]
    aC = rng.uniform(0.5, 1.5, abi.cell_shape(g))
    cC = rng.uniform(0.1, 2.0, abi.cell_shape(g))
    f = rng.standard_normal(abi.cell_shape(g))
    return g, bc, 1.0, -0.5, aC, b, cC, f


def _solve(case, prec, **opt):
    from mushy_gb300 import ops
    g, bc, alpha, beta, aC, b, cC, f = case
    if cC is None:
        op = ops.ProjectionOp(g, bc, alpha, beta, None, [dev(x) for x in b])
    else:
        op = ops.DarcyBrinkmanOp(g, bc, alpha, beta, dev(aC), [dev(x) for x in b], dev(cC))
    o = ops.default_options(False)
    o.tolerance, o.hang, o.max_iter, o.precision = 1e-10, 1e-15, 300, prec
    for k, v in opt.items():
        setattr(o, k, v)
    d_phi = torch.zeros_like(dev(f))
    st, rc = ops.AMRMultiGrid(op, o).solve(d_phi, dev(f))
    return host(d_phi), st, rc


def _check(case, singular, fp64_converges=True, **opt):
    g, bc, alpha, beta, aC, b, cC, f = case
    um, stm, rcm = _solve(case, abi.PREC_MIXED, **opt)
    u64, st64, rc64 = _solve(case, abi.PREC_F64, **opt)
    assert rcm == 0, (rcm, stm.iterations)
    ref = O.VCOpHost(g, bc, alpha, beta, aC, b, cC)
    r0 = O.norm(O.vc_residual(ref, np.zeros_like(f), f))
    r1 = O.norm(O.vc_residual(ref, um, f))
    assert r1 <= 1.01e-10 * r0, (r1, r0)
    if not fp64_converges:
        return stm, st64
    assert rc64 == 0, (rc64, st64.iterations)
    if singular:
        um, u64 = um - um.mean(), u64 - u64.mean()
    assert np.abs(um - u64).max() <= 1e-8 * np.abs(u64).max()
    return stm, st64


def test_projection_3d_periodic_xy():
    stm, st64 = _check(_projection(64, 21), True)
    # the FP32 cycles cost no extra outer iterations in kind: three of them
    # per FP64 step against one FP64 cycle per iteration
    assert stm.iterations <= st64.iterations


def test_darcy_brinkman_3d_walls():
    _check(_darcy((48, 32, 40), 22), False)


@pytest.mark.parametrize("opt", [dict(bottom_solver=abi.BOTTOM_BICGSTAB, bottom_max_iter=80),
                                 dict(num_mg=2), dict(num_smooth_down=0), dict(fuse_levels=0)])
def test_lean3d_cycle_variants(opt):
    _check(_darcy((32, 32, 32), 23), False, **opt)


def test_lean3d_no_post_smoothing():
    """V(2, 0): the full prolongation; the mixed solve converges (the FP64
    path in the reference's form stops on its hang test after one iteration
    on this operator, so only the oracle's residual is checked)."""
    _check(_darcy((32, 32, 32), 23), False, fp64_converges=False, num_smooth_up=0)


@pytest.mark.parametrize("shape,per", [((40, 24, 32), (0, 0, 1)), ((36, 32, 16), (1, 1, 1))])
def test_lean3d_other_boxes(shape, per):
    """Walls in x with a periodic z (the vector sweep's wall ends), and a
    fully periodic projection with 18 cells per colour row on level 0 (the
    one-cell-per-thread sweep)."""
    rng = np.random.default_rng(24)
    g = abi.make_grid(list(shape), 1.0 / shape[0], per)
    if all(per):
        b = [-rng.uniform(0.2, 3.0, abi.face_shape(g, d)) for d in range(3)]
        # a periodic seam is one face: its two entries (0 and n) equal, or
        # the operator is not symmetric and the singular system inconsistent
        for d in range(3):
            ax = 2 - d  # face arrays are [k][j][i]
            lo = [slice(None)] * 3
            hi = [slice(None)] * 3
            lo[ax], hi[ax] = 0, -1
            b[d][tuple(lo)] = b[d][tuple(hi)]
        f = rng.standard_normal(abi.cell_shape(g))
        f -= f.mean()
        _check((g, abi.make_bc(), 0.0, 1.0, None, b, None, f), True)
    else:
        bc = P.vc_bc("mixed")
        b = [-rng.uniform(0.2, 3.0, abi.face_shape(g, d)) for d in range(3)]
        aC = rng.uniform(0.5, 1.5, abi.cell_shape(g))
        cC = rng.uniform(0.1, 2.0, abi.cell_shape(g))
        f = rng.standard_normal(abi.cell_shape(g))
        _check((g, bc, 1.0, -0.5, aC, b, cC, f), False)


@pytest.mark.parametrize("case", ["projection", "darcy"])
def test_fp64_lean3d_matches_reference_order(case):
    """The FP64 comparison path (options.fuse_levels = 2: the mixed path's
    lean split cycles and outer step in FP64) reaches the same FP64 solution
    as the reference-order FP64 cycles: both stop at 1e-10 of the initial
    residual, so they agree to that times the operator's conditioning (1e-8
    of the solution's scale, as the mixed solves are held to)."""
    c = _projection(32, 25) if case == "projection" else _darcy((32, 24, 16), 26)
    g, bc, alpha, beta, aC, b, cC, f = c
    ul, stl, rcl = _solve(c, abi.PREC_F64, fuse_levels=2)
    ur, str_, rcr = _solve(c, abi.PREC_F64)
    assert rcl == 0 and rcr == 0
    ref = O.VCOpHost(g, bc, alpha, beta, aC, b, cC)
    r0 = O.norm(O.vc_residual(ref, np.zeros_like(f), f))
    assert O.norm(O.vc_residual(ref, ul, f)) <= 1.01e-10 * r0
    if case == "projection":
        ul, ur = ul - ul.mean(), ur - ur.mean()
    assert np.abs(ul - ur).max() <= 1e-8 * np.abs(ur).max()
