"""GPU parity at the sizes of the benchmark configurations.

* 64x64 diffusive solidification, ten backward-Euler steps with the
  reference's solver settings (FAS to 1e-10, at most 10 iterations a step):
  FP64 bitwise against the oracle step by step, with the iteration count,
  status and residual norms of every step.
* 512x512 projection Poisson: the FP64 solve bitwise against the oracle's
  (iterations, norms, solution); the mixed-precision solution within 1e-8 of
  it (null space removed).
* 1024x1024: one application of every kernel family of the mushy-layer step
  (closure, nonlinear residual, red/black pass and FAS restriction; the
  Darcy-Brinkman and projection residual, red/black pass and restriction;
  prolongation) bitwise against the oracle.
* 256^3: one nonlinear residual and one red/black pass of the (H, C)
  operator, one projection residual and red/black pass, bitwise.
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


def test_c1_ten_backward_euler_steps_bitwise():
    """64x64, St=5, CR=5, k=1e-3, liquid H=6, C=-1; T=-1 bottom, 0.5 top,
    C_l=-1 on both; sides Neumann; dt=1e-3; the reference's FAS settings."""
    from mushy_gb300 import ops
    n, dt = 64, 1e-3
    g = P.grid((n, n))
    prm = abi.make_params(stefan=5.0, compositionRatio=5.0, waterDistributionCoeff=1e-3,
                          specificHeatRatio=1.0, heatConductivityRatio=1.0)
    phi_bc = abi.make_bc()
    der = abi.make_bc({(1, 0, 0): (abi.BC_DIRICHLET, -1.0), (1, 1, 0): (abi.BC_DIRICHLET, 0.5),
                       (1, 0, 1): (abi.BC_DIRICHLET, -1.0), (1, 1, 1): (abi.BC_DIRICHLET, -1.0)})
    phi0 = np.empty((2,) + abi.cell_shape(g))
    phi0[0], phi0[1] = 6.0, -1.0
    b = [np.stack([-np.ones(abi.face_shape(g, d)), np.zeros(abi.face_shape(g, d))])
         for d in range(2)]
    ref = O.NLOpHost(g, prm, phi_bc, der, 1.0, 1.0, None, b)
    op = ops.NLMultiCompOp(g, prm, phi_bc, der, 1.0, 1.0, None, [dev(x) for x in b])
    S = ops.AMRFASMultiGrid(op, ops.default_options(True))
    oo = O.default_options(1)
    h, cur = phi0.copy(), dev(phi0)
    for step in range(10):
        h, st_r, rc_r = O.hc_backward_euler(ref, oo, h, h, dt)
        new = cur.clone()
        st, rc = S.backwardEuler(new, cur, dt)
        cur = new
        assert rc == rc_r and st.iterations == st_r.iterations, (step, rc, rc_r)
        assert st.initial_norm == st_r.initial_norm and st.final_norm == st_r.final_norm, step
        assert _hist(st) == _hist(st_r), step
        exact(host(cur), h)


def test_c2_projection_512_fp64_bitwise_and_mixed():
    from mushy_gb300 import ops
    g, chi, perm, u = P.projection_problem((512, 512), 1, sigma=32.0)
    b = [-f for f in O.face_geomean(g, perm)]
    f = O.mac_divergence(g, u)
    f -= f.mean()
    bc = abi.make_bc()
    ref = O.VCOpHost(g, bc, 0.0, 1.0, None, b)
    opts = O.default_options(0)
    opts.tolerance, opts.hang, opts.max_iter = 1e-10, 1e-15, 300
    sol_r, st_r, rc_r = O.vc_solve(ref, opts, np.zeros_like(f), f)
    assert rc_r == 0
    op = ops.ProjectionOp(g, bc, 0.0, 1.0, None, [dev(x) for x in b])
    o = ops.default_options(False)
    o.tolerance, o.hang, o.max_iter = 1e-10, 1e-15, 300
    d_phi = torch.zeros_like(dev(f))
    st, rc = ops.AMRMultiGrid(op, o).solve(d_phi, dev(f))
    assert rc == 0 and st.iterations == st_r.iterations
    assert st.initial_norm == st_r.initial_norm and st.final_norm == st_r.final_norm
    assert _hist(st) == _hist(st_r)
    exact(host(d_phi), sol_r)
    o.precision = abi.PREC_MIXED
    d_m = torch.zeros_like(dev(f))
    st_m, rc_m = ops.AMRMultiGrid(op, o).solve(d_m, dev(f))
    assert rc_m == 0
    m = host(d_m)
    assert np.abs(O.vc_residual(ref, m, f)).max() <= 1.01e-10 * st_r.initial_norm
    a = sol_r - sol_r.mean()
    assert np.abs(a - (m - m.mean())).max() <= 1e-8 * np.abs(a).max()


def _nl_big(n, seed):
    from mushy_gb300 import ops
    rng = np.random.default_rng(seed)
    g = P.grid(n)
    p = P.mushy_params()
    phi_bc, der = P.hc_bcs("mixed")
    phi = P.hc_state(g, rng)
    rhs = phi + 0.1 * rng.standard_normal(phi.shape)
    b = P.faces(g, rng, 2)
    ref = O.NLOpHost(g, p, phi_bc, der, 1.0, -2e-3, None, b)
    op = ops.NLMultiCompOp(g, p, phi_bc, der, 1.0, -2e-3, None, [dev(x) for x in b])
    return g, p, ref, op, phi, rhs


def _vc_big(n, seed, with_c):
    from mushy_gb300 import ops
    rng = np.random.default_rng(seed)
    g = P.grid(n)
    bc = P.vc_bc("mixed")
    b = [x[0] for x in P.faces(g, rng, 1)]
    cC = rng.uniform(0.1, 3.0, abi.cell_shape(g)) if with_c else None
    alpha, beta = (0.0, -0.9) if with_c else (0.0, 1.0)
    ref = O.VCOpHost(g, bc, alpha, beta, None, b, cC)
    cls = ops.DarcyBrinkmanOp if with_c else ops.ProjectionOp
    op = cls(g, bc, alpha, beta, None, [dev(x) for x in b], None if cC is None else dev(cC))
    phi = rng.standard_normal(abi.cell_shape(g))
    rhs = rng.standard_normal(abi.cell_shape(g))
    return g, ref, op, phi, rhs


def test_c3_kernel_families_1024_bitwise():
    import ctypes as C
    from mushy_gb300 import ops
    g, p, ref, op, phi, rhs = _nl_big((1024, 1024), 31)
    # closure
    out = torch.empty_like(dev(phi))
    abi.check(abi.load().mlgpu_closure_tcl(C.byref(g), C.byref(p), ops._ptr(dev(phi)),
                                           ops._ptr(out), ops._stream()))
    exact(host(out), O.closure_tcl(g, p, phi))
    d_phi, d_rhs = dev(phi), dev(rhs)
    res = torch.empty_like(d_phi)
    nrm = op.residual(res, d_phi, d_rhs, norm_type=abi.NORM_MAX)
    r_ref = O.nl_residual(ref, phi, rhs)
    exact(host(res), r_ref)
    assert nrm == np.abs(r_ref).max()
    rc = op.createCoarser()
    op.restrictResidual(rc, d_phi, d_rhs)
    exact(host(rc), O.nl_restrict_residual(ref, phi, rhs))
    op.levelGSRB(d_phi, d_rhs)
    exact(host(d_phi), O.nl_relax(ref, phi, rhs, 1))
    del d_phi, d_rhs, res, rc, out
    for with_c in (True, False):
        g, vref, vop, x, f = _vc_big((1024, 1024), 32, with_c)
        d_x, d_f = dev(x), dev(f)
        res = torch.empty_like(d_x)
        vop.residual(res, d_x, d_f)
        exact(host(res), O.vc_residual(vref, x, f))
        rc = vop.createCoarser()
        vop.restrictResidual(rc, d_x, d_f)
        exact(host(rc), O.vc_restrict_residual(vref, x, f))
        vop.levelGSRB(d_x, d_f)
        exact(host(d_x), O.vc_relax(vref, x, f, 1))
    # linear prolongation of a coarse correction
    rng = np.random.default_rng(33)
    bc = P.vc_bc("mixed")
    fine = rng.standard_normal((2,) + abi.cell_shape(g))
    coarse = rng.standard_normal(O.coarse_shape(g, 2))
    df = dev(fine)
    abi.check(abi.load().mlgpu_prolong_increment(C.byref(g), C.byref(bc), 2, abi.F64,
                                                 abi.PROLONG_LINEAR, ops._ptr(df),
                                                 ops._ptr(dev(coarse)), ops._stream()))
    exact(host(df), O.prolong_increment(g, bc, 2, abi.PROLONG_LINEAR, fine, coarse))


def test_c4_256cubed_residual_and_gsrb_bitwise():
    g, p, ref, op, phi, rhs = _nl_big((256, 256, 256), 41)
    d_phi, d_rhs = dev(phi), dev(rhs)
    res = torch.empty_like(d_phi)
    nrm = op.residual(res, d_phi, d_rhs, norm_type=abi.NORM_MAX)
    r_ref = O.nl_residual(ref, phi, rhs)
    exact(host(res), r_ref)
    assert nrm == np.abs(r_ref).max()
    del res, r_ref
    op.levelGSRBPass(d_phi, d_rhs, 0)
    op.levelGSRBPass(d_phi, d_rhs, 1)
    exact(host(d_phi), O.nl_relax(ref, phi, rhs, 1))
    del d_phi, d_rhs, op, ref, phi, rhs
    g, vref, vop, x, f = _vc_big((256, 256, 256), 42, False)
    d_x, d_f = dev(x), dev(f)
    res = torch.empty_like(d_x)
    vop.residual(res, d_x, d_f)
    exact(host(res), O.vc_residual(vref, x, f))
    vop.levelGSRB(d_x, d_f)
    exact(host(d_x), O.vc_relax(vref, x, f, 1))
