"""GPU parity: every sm_103a kernel against the CPU oracle on seeded inputs.

FP64 kernels are required to be bitwise equal to the oracle (both evaluate
the reference's Fortran expressions in the same order without contraction).
FP32 kernels (inner cycles of the mixed solver) are checked against the
FP64 oracle with a relative tolerance of 1e-5 of the field scale.
"""
import numpy as np
import pytest

import problems as P
from mushy_gb300 import abi
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import __graft_entry__
    __graft_entry__.build()
    from mushy_gb300 import ops  # noqa: F401
    yield


def dev(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    return t.to(dtype) if dtype is not None else t


def host(t):
    torch.cuda.synchronize()
    return t.double().cpu().numpy()


def exact(a, b):
    assert a.size == b.size, (a.shape, b.shape)
    a = a.reshape(b.shape)
    if not np.array_equal(a, b):
        d = np.abs(a - b)
        raise AssertionError("not bitwise equal: max diff %g at %s (%r vs %r)"
                             % (d.max(), np.unravel_index(d.argmax(), d.shape),
                                a.flat[d.argmax()], b.flat[d.argmax()]))


def close32(gpu, ref, rtol=1e-5):
    scale = max(np.abs(ref).max(), 1e-30)
    err = np.abs(gpu - ref).max() / scale
    assert err < rtol, "FP32 relative error %g >= %g" % (err, rtol)


CASES_2D = [((16, 12), (0, 0, 0)), ((18, 10), (1, 0, 0)), ((8, 8), (1, 1, 0))]
CASES_3D = [((8, 6, 4), (0, 0, 0)), ((6, 4, 8), (0, 1, 1))]
ALL = CASES_2D + CASES_3D


def nl_setup(n, per, seed, a=True, dbc=True, kind="mixed"):
    from mushy_gb300 import ops
    rng = np.random.default_rng(seed)
    g = P.grid(n, per)
    p = P.mushy_params()
    phi_bc, der = P.hc_bcs(kind)
    phi = P.hc_state(g, rng)
    rhs = phi + 0.1 * rng.standard_normal(phi.shape)
    b = P.faces(g, rng, 2)
    aC = rng.uniform(0.5, 1.5, phi.shape) if a else None
    alpha, beta = 1.0, -2e-3
    ref = O.NLOpHost(g, p, phi_bc, der, alpha, beta, aC, b, apply_derived_bc=int(dbc))
    op = ops.NLMultiCompOp(g, p, phi_bc, der, alpha, beta, None if aC is None else dev(aC),
                           [dev(x) for x in b], apply_derived_bc=dbc)
    return g, p, ref, op, phi, rhs


# ------------------------------------------------------------------ closure
@pytest.mark.parametrize("seed", [0, 1])
def test_closure_full_bitwise(seed):
    from mushy_gb300 import ops
    import ctypes as C
    rng = np.random.default_rng(seed)
    g = P.grid((33, 17))
    for params in (P.mushy_params(), P.mushy_params(specificHeatRatio=1.3, thetaEutectic=0.2,
                                                    ThetaEutectic=0.1, waterDistributionCoeff=0.05)):
        HC = P.hc_state(g, rng)
        ref = O.closure(g, params, HC)
        d = dev(HC)
        outs = {k: torch.empty(abi.ncells(g), dtype=torch.float64, device="cuda")
                for k in ("T", "porosity", "Cl", "Cs", "Hs", "He", "Hl")}
        abi.check(abi.load().mlgpu_closure(C.byref(g), C.byref(params), ops._ptr(d),
                                           *[ops._ptr(outs[k]) for k in
                                             ("T", "porosity", "Cl", "Cs", "Hs", "He", "Hl")],
                                           ops._stream()))
        for k in outs:
            exact(host(outs[k]), ref[k])


def test_closure_tcl_bitwise():
    from mushy_gb300 import ops
    import ctypes as C
    rng = np.random.default_rng(3)
    g = P.grid((40, 9))
    p = P.mushy_params()
    HC = P.hc_state(g, rng)
    ref = O.closure_tcl(g, p, HC)
    d = dev(HC)
    out = torch.empty_like(d)
    abi.check(abi.load().mlgpu_closure_tcl(C.byref(g), C.byref(p), ops._ptr(d), ops._ptr(out),
                                           ops._stream()))
    exact(host(out), ref)


# ------------------------------------------------------ nonlinear operator
@pytest.mark.parametrize("n,per", ALL)
@pytest.mark.parametrize("dbc", [True, False])
def test_nl_residual_apply_bitwise(n, per, dbc):
    g, p, ref, op, phi, rhs = nl_setup(n, per, 11, dbc=dbc)
    d_phi, d_rhs = dev(phi), dev(rhs)
    res = torch.empty_like(d_phi)
    nrm = op.residual(res, d_phi, d_rhs, norm_type=abi.NORM_MAX)
    r_ref = O.nl_residual(ref, phi, rhs)
    exact(host(res), r_ref)
    assert nrm == np.abs(r_ref).max()
    lhs = torch.empty_like(d_phi)
    op.applyOp(lhs, d_phi)
    exact(host(lhs), O.nl_apply(ref, phi))
    nrm2 = op.residual(res, d_phi, d_rhs, norm_type=abi.NORM_L2)
    assert abs(nrm2 - np.sqrt((r_ref ** 2).sum())) <= 1e-12 * nrm2


@pytest.mark.parametrize("n,per", ALL)
def test_nl_gsrb_bitwise(n, per):
    g, p, ref, op, phi, rhs = nl_setup(n, per, 12)
    d_phi, d_rhs = dev(phi), dev(rhs)
    op.levelGSRBPass(d_phi, d_rhs, 0)
    exact(host(d_phi), O.nl_gsrb_pass(ref, phi, rhs, 0))
    op.relax(d_phi, d_rhs, 3)
    r = O.nl_gsrb_pass(ref, phi, rhs, 0)
    r = O.nl_relax(ref, r, rhs, 3)
    exact(host(d_phi), r)


@pytest.mark.parametrize("n,per", CASES_2D[:2] + CASES_3D[:1])
def test_nl_jacobi_lambda_bitwise(n, per):
    g, p, ref, op, phi, rhs = nl_setup(n, per, 13)
    d_phi, d_rhs = dev(phi), dev(rhs)
    exact(host(op.computeLambda()), O.nl_lambda(ref))
    op.levelJacobi(d_phi, d_rhs)
    exact(host(d_phi), O.nl_jacobi(ref, phi, rhs))


@pytest.mark.parametrize("n,per", ALL)
def test_nl_restrict_residual_bitwise(n, per):
    g, p, ref, op, phi, rhs = nl_setup(n, per, 14)
    d_phi, d_rhs = dev(phi), dev(rhs)
    rc = op.createCoarser()
    op.restrictResidual(rc, d_phi, d_rhs)
    exact(host(rc), O.nl_restrict_residual(ref, phi, rhs))
    pc = op.createCoarser()
    op.restrictR(pc, d_phi)
    exact(host(pc), O.restrict_average(g, 2, phi))


def test_nl_fp32_kernels_close():
    from mushy_gb300 import ops
    g, p, ref, op64, phi, rhs = nl_setup((20, 16), (1, 0, 0), 15, kind="mixed")
    rng = np.random.default_rng(15)
    op = ops.NLMultiCompOp(g, p, op64.phi_bc, op64.derived_bc, op64.alpha, op64.beta,
                           op64.aCoef.float(), [b.float() for b in op64.bCoef])
    d_phi, d_rhs = dev(phi, torch.float32), dev(rhs, torch.float32)
    res = torch.empty_like(d_phi)
    op.residual(res, d_phi, d_rhs)
    close32(host(res), O.nl_residual(ref, host(d_phi), host(d_rhs)), 1e-4)
    op.levelGSRB(d_phi, d_rhs)
    close32(host(d_phi), O.nl_relax(ref, phi, rhs, 1), 1e-5)


# ---------------------------------------------------------------- transfers
@pytest.mark.parametrize("n,per", ALL)
@pytest.mark.parametrize("kind", [abi.PROLONG_CONSTANT, abi.PROLONG_LINEAR])
def test_prolong_bitwise(n, per, kind):
    import ctypes as C
    from mushy_gb300 import ops
    rng = np.random.default_rng(20)
    g = P.grid(n, per)
    bc = P.vc_bc("mixed")
    for ncomp in (1, 2):
        fine = rng.standard_normal((ncomp,) + abi.cell_shape(g))
        coarse = rng.standard_normal(O.coarse_shape(g, ncomp))
        ref = O.prolong_increment(g, bc, ncomp, kind, fine, coarse)
        df, dc = dev(fine), dev(coarse)
        abi.check(abi.load().mlgpu_prolong_increment(C.byref(g), C.byref(bc), ncomp, abi.F64,
                                                     kind, ops._ptr(df), ops._ptr(dc),
                                                     ops._stream()))
        exact(host(df), ref)


@pytest.mark.parametrize("n,per", ALL)
def test_coarsen_coefficients_bitwise(n, per):
    import ctypes as C
    from mushy_gb300 import ops
    rng = np.random.default_rng(21)
    g = P.grid(n, per)
    for d in range(g.dim):
        ff = rng.uniform(0.1, 2.0, (2,) + abi.face_shape(g, d))
        ref = O.coarsen_faces(g, 2, d, ff)
        out = torch.empty(ref.shape, dtype=torch.float64, device="cuda")
        abi.check(abi.load().mlgpu_coarsen_faces(C.byref(g), 2, abi.F64, d, ops._ptr(out),
                                                 ops._ptr(dev(ff)), ops._stream()))
        exact(host(out), ref)


@pytest.mark.parametrize("n,per", CASES_2D + CASES_3D[:1])
def test_face_geomean_and_mac_bitwise(n, per):
    import ctypes as C
    from mushy_gb300 import ops
    rng = np.random.default_rng(22)
    g = P.grid(n, per)
    cell = rng.uniform(0.05, 1.0, abi.cell_shape(g))
    ref = O.face_geomean(g, cell)
    outs = [torch.empty(abi.face_shape(g, d), dtype=torch.float64, device="cuda")
            for d in range(g.dim)]
    arr = (C.c_void_p * 3)(*([o.data_ptr() for o in outs] + [None] * (3 - g.dim)))
    abi.check(abi.load().mlgpu_face_geomean(C.byref(g), ops._ptr(dev(cell)), arr, ops._stream()))
    for d in range(g.dim):
        exact(host(outs[d]), ref[d])
    # MAC divergence and gradient correction
    u = [rng.standard_normal(abi.face_shape(g, d)) for d in range(g.dim)]
    du = [dev(x) for x in u]
    div = torch.empty(abi.cell_shape(g), dtype=torch.float64, device="cuda")
    uarr = (C.c_void_p * 3)(*([x.data_ptr() for x in du] + [None] * (3 - g.dim)))
    abi.check(abi.load().mlgpu_mac_divergence(C.byref(g), ops._ptr(div), uarr, ops._stream()))
    exact(host(div), O.mac_divergence(g, u))
    bc = P.vc_bc("mixed")
    phi = rng.standard_normal(abi.cell_shape(g))
    scale = [rng.uniform(0.1, 1, abi.face_shape(g, d)) for d in range(g.dim)]
    dsc = [dev(x) for x in scale]
    sarr = (C.c_void_p * 3)(*([x.data_ptr() for x in dsc] + [None] * (3 - g.dim)))
    abi.check(abi.load().mlgpu_mac_correct(C.byref(g), C.byref(bc), ops._ptr(dev(phi)), sarr,
                                           uarr, ops._stream()))
    ref_u = O.mac_correct(g, bc, phi, u, scale)
    for d in range(g.dim):
        exact(host(du[d]), ref_u[d])


# ------------------------------------------------------- linear operators
def vc_setup(n, per, seed, with_c, with_a, dtype=torch.float64):
    from mushy_gb300 import ops
    rng = np.random.default_rng(seed)
    g = P.grid(n, per)
    bc = P.vc_bc("mixed")
    b = P.faces(g, rng, 1)
    b = [x[0] for x in b]
    aC = rng.uniform(0.5, 1.5, abi.cell_shape(g)) if with_a else None
    cC = rng.uniform(0.1, 3.0, abi.cell_shape(g)) if with_c else None
    alpha, beta = (0.7, -0.9) if with_c else (0.0, 1.0)
    ref = O.VCOpHost(g, bc, alpha, beta, aC, b, cC)
    cls = ops.DarcyBrinkmanOp if with_c else ops.ProjectionOp
    op = cls(g, bc, alpha, beta, None if aC is None else dev(aC, dtype),
             [dev(x, dtype) for x in b], None if cC is None else dev(cC, dtype))
    phi = rng.standard_normal(abi.cell_shape(g))
    rhs = rng.standard_normal(abi.cell_shape(g))
    return g, ref, op, phi, rhs


@pytest.mark.parametrize("n,per", ALL)
@pytest.mark.parametrize("with_c", [False, True])
def test_vc_ops_bitwise(n, per, with_c):
    g, ref, op, phi, rhs = vc_setup(n, per, 30, with_c, with_c)
    d_phi, d_rhs = dev(phi), dev(rhs)
    res = torch.empty_like(d_phi)
    for hom in (0, 1):
        nrm = op.residual(res, d_phi, d_rhs, homogeneous=hom, norm_type=abi.NORM_MAX)
        r = O.vc_residual(ref, phi, rhs, hom)
        exact(host(res), r)
        assert nrm == np.abs(r).max()
        op.applyOp(res, d_phi, homogeneous=hom)
        exact(host(res), O.vc_apply(ref, phi, hom))
    exact(host(op.computeLambda()), O.vc_lambda(ref))
    rc = op.createCoarser()
    op.restrictResidual(rc, d_phi, d_rhs)
    exact(host(rc), O.vc_restrict_residual(ref, phi, rhs))
    op.levelGSRBPass(d_phi, d_rhs, 0)
    r1 = O.vc_gsrb_pass(ref, phi, rhs, 0)
    exact(host(d_phi), r1)
    op.relax(d_phi, d_rhs, 2)
    exact(host(d_phi), O.vc_relax(ref, r1, rhs, 2))
    op.levelJacobi(d_phi, d_rhs)
    exact(host(d_phi), O.vc_jacobi(ref, O.vc_relax(ref, r1, rhs, 2), rhs))


def test_vc_fp32_close():
    g, ref, op, phi, rhs = vc_setup((24, 16), (1, 0, 0), 31, True, True, torch.float32)
    d_phi, d_rhs = dev(phi, torch.float32), dev(rhs, torch.float32)
    res = torch.empty_like(d_phi)
    op.residual(res, d_phi, d_rhs)
    close32(host(res), O.vc_residual(ref, host(d_phi), host(d_rhs)), 1e-5)
    op.relax(d_phi, d_rhs, 2)
    close32(host(d_phi), O.vc_relax(ref, phi, rhs, 2), 1e-5)


# -------------------------------------------------------------------- solvers
def test_vc_solver_fp64_matches_oracle():
    from mushy_gb300 import ops
    g, chi, perm, u = P.projection_problem((64, 64), 5, sigma=8.0)
    faces = O.face_geomean(g, perm)
    b = [-f for f in faces]
    f = O.mac_divergence(g, u)
    f -= f.mean()
    bc = abi.make_bc()
    ref = O.VCOpHost(g, bc, 0.0, 1.0, None, b)
    opts = O.default_options(0)
    opts.tolerance, opts.hang, opts.max_iter = 1e-30, 0.0, 12   # fixed 12 iterations
    sol_ref, st_ref, rc_ref = O.vc_solve(ref, opts, np.zeros_like(f), f)
    assert st_ref.iterations == 12
    op = ops.ProjectionOp(g, bc, 0.0, 1.0, None, [dev(x) for x in b])
    for graph in (0, 1, 2):
        o = ops.default_options(False)
        o.tolerance, o.hang, o.max_iter, o.use_graph = 1e-30, 0.0, 12, graph
        S = ops.AMRMultiGrid(op, o)
        d_phi = torch.zeros_like(dev(f))
        st, rc = S.solve(d_phi, dev(f))
        assert rc == rc_ref and st.iterations == st_ref.iterations
        assert [st.norm_history[i] for i in range(13)] == [st_ref.norm_history[i] for i in range(13)]
        exact(host(d_phi), sol_ref)
        assert st.cell_updates == st_ref.cell_updates


@pytest.mark.parametrize("n,per,with_c,bckind,pre,post", [
    ((256, 128), (1, 0, 0), False, "neumann", 2, 4),
    ((192, 128), (0, 0, 0), True, "mixed", 1, 3),
    ((128, 256), (0, 1, 0), False, "mixed", 2, 8),
    ((256, 96), (1, 1, 0), True, "neumann", 3, 2),
])
def test_vc_solver_tiled_levels_bitwise(n, per, with_c, bckind, pre, post):
    """Levels above 4096 cells run the shared-memory tile smoother (temporal
    blocking of pre-smoothing + restriction and prolongation +
    post-smoothing); the result must equal the per-level oracle bit for bit."""
    from mushy_gb300 import ops
    rng = np.random.default_rng(50)
    g = P.grid(n, per)
    bc = P.vc_bc(bckind)
    b = [-rng.uniform(0.2, 3.0, abi.face_shape(g, d)) for d in range(2)]
    aC = rng.uniform(0.5, 1.5, abi.cell_shape(g)) if with_c else None
    cC = rng.uniform(0.1, 2.0, abi.cell_shape(g)) if with_c else None
    alpha, beta = (1.0, -0.5) if with_c else (0.0, 1.0)
    f = rng.standard_normal(abi.cell_shape(g))
    if not with_c and bckind == "neumann":
        f -= f.mean()
    ref = O.VCOpHost(g, bc, alpha, beta, aC, b, cC)
    opts = O.default_options(0)
    opts.tolerance, opts.hang, opts.max_iter = 1e-30, 0.0, 5
    opts.num_smooth_down, opts.num_smooth_up = pre, post
    sol_ref, st_ref, rc_ref = O.vc_solve(ref, opts, np.zeros_like(f), f)
    cls = ops.DarcyBrinkmanOp if with_c else ops.ProjectionOp
    op = cls(g, bc, alpha, beta, None if aC is None else dev(aC), [dev(x) for x in b],
             None if cC is None else dev(cC))
    o = ops.default_options(False)
    o.tolerance, o.hang, o.max_iter, o.fuse_levels = 1e-30, 0.0, 5, 2
    o.num_smooth_down, o.num_smooth_up = pre, post
    S = ops.AMRMultiGrid(op, o)
    d_phi = torch.zeros_like(dev(f))
    st, rc = S.solve(d_phi, dev(f))
    assert st.iterations == st_ref.iterations == 5
    exact(host(d_phi), sol_ref)
    assert [st.norm_history[i] for i in range(6)] == [st_ref.norm_history[i] for i in range(6)]
    # mixed precision on the same tiled path converges like the FP64 one
    om = ops.default_options(False)
    om.tolerance, om.hang, om.max_iter, om.precision = 1e-30, 0.0, 5, abi.PREC_MIXED
    om.num_smooth_down, om.num_smooth_up = pre, post
    pm = torch.zeros_like(dev(f))
    stm, rcm = ops.AMRMultiGrid(op, om).solve(pm, dev(f))
    assert stm.final_norm <= 1.5 * st.final_norm + 1e-12 * st.initial_norm
    one_cycle_agrees(op, f)


@pytest.mark.parametrize("pre,post", [(0, 3), (2, 0)])
def test_vc_solver_zero_sweeps(pre, post):
    """No pre- or no post-smoothing: the fused paths still restrict,
    prolong and cycle exactly like the per-level oracle (FP64 bits) and like
    the per-level FP32 path (mixed)."""
    from mushy_gb300 import ops
    rng = np.random.default_rng(60 + pre)
    g = P.grid((256, 128), (1, 0, 0))
    bc = P.vc_bc("mixed")
    b = [-rng.uniform(0.2, 3.0, abi.face_shape(g, d)) for d in range(2)]
    f = rng.standard_normal(abi.cell_shape(g))
    ref = O.VCOpHost(g, bc, 0.0, 1.0, None, b)
    opts = O.default_options(0)
    opts.tolerance, opts.hang, opts.max_iter = 1e-30, 0.0, 4
    opts.num_smooth_down, opts.num_smooth_up = pre, post
    sol_ref, st_ref, rc_ref = O.vc_solve(ref, opts, np.zeros_like(f), f)
    op = ops.ProjectionOp(g, bc, 0.0, 1.0, None, [dev(x) for x in b])
    o = ops.default_options(False)
    o.tolerance, o.hang, o.max_iter, o.fuse_levels = 1e-30, 0.0, 4, 2
    o.num_smooth_down, o.num_smooth_up = pre, post
    d_phi = torch.zeros_like(dev(f))
    st, rc = ops.AMRMultiGrid(op, o).solve(d_phi, dev(f))
    exact(host(d_phi), sol_ref)
    one_cycle_agrees(op, f, pre=pre, post=post)


@pytest.mark.parametrize("mixed", [False, True])
def test_vc_fused_levels_match_unfused_multiwave(mixed):
    """1024x768 puts thousands of tiles in flight (several waves), where a
    tile reading halo cells that another tile already rewrote would show up.
    FP64: fused == per-level launches bit for bit; mixed: same convergence."""
    from mushy_gb300 import ops
    g, chi, perm, u = P.projection_problem((1024, 768), 9, sigma=24.0)
    faces = O.face_geomean(g, perm)
    b = [-x for x in faces]
    f = O.mac_divergence(g, u)
    f -= f.mean()
    op = ops.ProjectionOp(g, abi.make_bc(), 0.0, 1.0, None, [dev(x) for x in b])
    out = {}
    for fuse in (0, 2):
        o = ops.default_options(False)
        o.tolerance, o.hang, o.max_iter, o.fuse_levels = 1e-30, 0.0, 6, fuse
        o.precision = abi.PREC_MIXED if mixed else abi.PREC_F64
        # one FP32 cycle per outer step: several cycles on one FP32
        # correction reach the FP32 floor of this ill-conditioned operator,
        # where the lean and the per-level forms stall at different levels
        o.inner_cycles = 1
        d_phi = torch.zeros_like(dev(f))
        st, rc = ops.AMRMultiGrid(op, o).solve(d_phi, dev(f))
        out[fuse] = (host(d_phi), [st.norm_history[i] for i in range(7)])
    if not mixed:
        exact(out[2][0], out[0][0])
        assert out[2][1] == out[0][1]
    else:
        # FP32 rounding reaches the FP64 residual amplified by the operator's
        # conditioning (Kozeny-Carman contrast 1e4): histories agree loosely,
        # the single-cycle corrections tightly
        h0, h1 = np.array(out[0][1]), np.array(out[2][1])
        assert np.all(np.abs(h1 - h0) <= 0.1 * h0), (h0, h1)
        one_cycle_agrees(op, f)


def one_cycle_agrees(op, f, rel=2e-5, pre=None, post=None):
    """One FP32 V-cycle from zero (one outer iteration) is the same linear
    map of the right-hand side whether it runs per level or fused in tiles
    (lean FP32 form); its results must agree to FP32 rounding."""
    from mushy_gb300 import ops
    sol = {}
    for fuse in (0, 1):
        o = ops.default_options(False)
        o.tolerance, o.hang, o.max_iter, o.fuse_levels = 1e-30, 0.0, 1, fuse
        o.precision = abi.PREC_MIXED
        o.inner_cycles = 1
        if pre is not None:
            o.num_smooth_down, o.num_smooth_up = pre, post
        d_phi = torch.zeros_like(dev(f))
        ops.AMRMultiGrid(op, o).solve(d_phi, dev(f))
        sol[fuse] = host(d_phi)
    scale = np.abs(sol[0]).max()
    err = np.abs(sol[1] - sol[0]).max()
    assert err <= rel * scale, (err, scale)


@pytest.mark.parametrize("norm", [abi.NORM_MAX, abi.NORM_L2])
def test_vc_solver_mixed_inhomogeneous_bc(norm):
    """Mixed solver on a Darcy-Brinkman operator (a, c coefficients) with
    inhomogeneous Dirichlet / Neumann values: the FP64 outer residual it
    reports agrees with the oracle's residual of the same field, and the
    returned solution meets the tolerance under the oracle's residual."""
    from mushy_gb300 import ops
    rng = np.random.default_rng(77)
    g = P.grid((96, 64), (0, 0, 0))
    bc = P.vc_bc("mixed")
    b = [-rng.uniform(0.2, 3.0, abi.face_shape(g, d)) for d in range(2)]
    aC = rng.uniform(0.5, 1.5, abi.cell_shape(g))
    cC = rng.uniform(0.1, 2.0, abi.cell_shape(g))
    f = rng.standard_normal(abi.cell_shape(g))
    phi0 = 0.1 * rng.standard_normal(abi.cell_shape(g))
    ref = O.VCOpHost(g, bc, 1.0, -0.5, aC, b, cC)
    op = ops.DarcyBrinkmanOp(g, bc, 1.0, -0.5, dev(aC), [dev(x) for x in b], dev(cC))
    o = ops.default_options(False)
    o.tolerance, o.hang, o.max_iter, o.precision = 1e-10, 1e-15, 100, abi.PREC_MIXED
    o.norm_type = norm
    d_phi = dev(phi0)
    st, rc = ops.AMRMultiGrid(op, o).solve(d_phi, dev(f))
    assert rc == 0
    r0 = O.norm(O.vc_residual(ref, phi0, f), norm)
    assert abs(st.initial_norm - r0) <= 1e-12 * r0
    r1 = O.norm(O.vc_residual(ref, host(d_phi), f), norm)
    assert abs(st.final_norm - r1) <= 1e-4 * r1 + 1e-14 * r0
    assert r1 <= 1.01e-10 * r0


def test_vc_solver_mixed_converges():
    from mushy_gb300 import ops
    g, chi, perm, u = P.projection_problem((128, 128), 6, sigma=16.0)
    faces = O.face_geomean(g, perm)
    b = [-f for f in faces]
    f = O.mac_divergence(g, u)
    f -= f.mean()
    bc = abi.make_bc()
    op = ops.ProjectionOp(g, bc, 0.0, 1.0, None, [dev(x) for x in b])
    o64 = ops.default_options(False)
    o64.tolerance, o64.hang, o64.max_iter = 1e-10, 1e-15, 300
    om = ops.default_options(False)
    om.tolerance, om.hang, om.max_iter, om.precision = 1e-10, 1e-15, 300, abi.PREC_MIXED
    p64 = torch.zeros_like(dev(f))
    st64, rc64 = ops.AMRMultiGrid(op, o64).solve(p64, dev(f))
    pm = torch.zeros_like(dev(f))
    stm, rcm = ops.AMRMultiGrid(op, om).solve(pm, dev(f))
    assert rc64 == 0 and rcm == 0
    assert stm.final_norm <= 1e-10 * stm.initial_norm
    # FP64-checked residual of the mixed solution
    ref = O.VCOpHost(g, bc, 0.0, 1.0, None, b)
    r = O.vc_residual(ref, host(pm), f)
    assert np.abs(r).max() <= 1e-10 * np.abs(f).max() * 1.0001
    # solutions agree up to the null-space constant
    a, m = host(p64), host(pm)
    diff = (a - a.mean()) - (m - m.mean())
    assert np.abs(diff).max() <= 1e-8 * np.abs(a - a.mean()).max()


def test_hc_solver_fp64_matches_oracle():
    from mushy_gb300 import ops
    n = 32
    g = P.grid((n, n))
    p = P.mushy_params()
    phi_bc, der = P.hc_bcs("mixed")
    rng = np.random.default_rng(40)
    phi = P.hc_state(g, rng, regimes=False)
    dt = 1e-3
    b = [np.stack([-np.ones(abi.face_shape(g, d)), -0.01 * np.ones(abi.face_shape(g, d))])
         for d in range(2)]
    ref = O.NLOpHost(g, p, phi_bc, der, 1.0, -dt, None, b)
    opts = O.default_options(1)
    opts.max_iter = 6
    sol_ref, st_ref, rc_ref = O.hc_solve(ref, opts, phi, phi.copy())
    op = ops.NLMultiCompOp(g, p, phi_bc, der, 1.0, -dt, None, [dev(x) for x in b])
    for graph in (0, 1, 2):
        o = ops.default_options(True)
        o.max_iter, o.use_graph = 6, graph
        S = ops.AMRFASMultiGrid(op, o)
        d_phi = dev(phi)
        st, rc = S.solve(d_phi, dev(phi))
        assert rc == rc_ref and st.iterations == st_ref.iterations
        exact(host(d_phi), sol_ref)
        assert st.cell_updates == st_ref.cell_updates


@pytest.mark.parametrize("n,dt", [((48, 32), 1e-3), ((64, 64), 1e-3)])
def test_hc_solver_mixed_converges_to_fp64_solution(n, dt):
    """Mixed precision for the nonlinear (H, C) solve: FP32 cycles on the
    problem linearised with the FP64 closure Jacobian, inside an FP64
    defect-correction loop (switching to FP64 FAS cycles if a linearised step
    fails to reduce the residual: the 64x64 case needs it).  It reaches 1e-10
    under the oracle's own FP64 residual and agrees with the FP64 FAS
    solution to 1e-8."""
    from mushy_gb300 import ops
    g = P.grid(n)
    p = P.mushy_params()
    phi_bc, der = P.hc_bcs("mixed")
    rng = np.random.default_rng(44)
    phi = P.hc_state(g, rng, regimes=False)  # straddles the liquidus (mush + liquid)
    b = [np.stack([-np.ones(abi.face_shape(g, d)), -0.01 * np.ones(abi.face_shape(g, d))])
         for d in range(2)]
    rhs = phi.copy()
    ref = O.NLOpHost(g, p, phi_bc, der, 1.0, -dt, None, b)
    op = ops.NLMultiCompOp(g, p, phi_bc, der, 1.0, -dt, None, [dev(x) for x in b])
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


def test_hc_backward_euler_mixed_matches_fp64():
    """Three backward-Euler steps with the mixed nonlinear solve against the
    FP64 FAS, both iterated to 1e-10."""
    from mushy_gb300 import ops
    n, dt = 32, 1e-3
    g = P.grid((n, n))
    p = P.mushy_params()
    phi_bc, der = P.hc_bcs("mixed")
    rng = np.random.default_rng(45)
    phi = P.hc_state(g, rng, regimes=False)
    b = [np.stack([-np.ones(abi.face_shape(g, d)), -0.02 * np.ones(abi.face_shape(g, d))])
         for d in range(2)]
    src = dev(0.1 * rng.standard_normal(phi.shape))
    op = ops.NLMultiCompOp(g, p, phi_bc, der, 1.0, 1.0, None, [dev(x) for x in b])
    out = {}
    for prec in (abi.PREC_F64, abi.PREC_MIXED):
        o = ops.default_options(True)
        o.max_iter, o.tolerance, o.hang, o.precision = 60, 1e-10, 1e-15, prec
        S = ops.AMRFASMultiGrid(op, o)
        cur = dev(phi)
        for _ in range(3):
            new = cur.clone()
            st, rc = S.backwardEuler(new, cur, dt, src=src)
            assert rc == 0, (prec, rc, st.iterations)
            cur = new
        out[prec] = host(cur)
    scale = np.abs(out[abi.PREC_F64]).max()
    assert np.abs(out[abi.PREC_MIXED] - out[abi.PREC_F64]).max() <= 1e-8 * scale


# ------------------------------------------------- composed "next" rows
def test_mac_project_bitwise_and_divergence_free():
    from mushy_gb300 import ops
    g, chi, perm, u = P.projection_problem((64, 32), 8, sigma=6.0)
    # a compatible u*: periodic in x (seam faces equal), solid walls in y
    u[0][..., -1] = u[0][..., 0]
    u[1][:, 0, :] = 0.0
    u[1][:, -1, :] = 0.0
    pi = O.face_geomean(g, perm)
    b = [-x for x in pi]
    bc = abi.make_bc()
    ref = O.VCOpHost(g, bc, 0.0, 1.0, None, b)
    opts = O.default_options(0)
    opts.tolerance, opts.hang, opts.max_iter = 1e-12, 0.0, 400
    u_ref, phi_ref, st_ref, rc_ref = O.mac_project(ref, opts, bc, u, pi, np.zeros(abi.cell_shape(g)))
    div0 = np.abs(O.mac_divergence(g, u)).max()
    assert np.abs(O.mac_divergence(g, u_ref)).max() <= 1e-10 * div0
    op = ops.ProjectionOp(g, bc, 0.0, 1.0, None, [dev(x) for x in b])
    o = ops.default_options(False)
    o.tolerance, o.hang, o.max_iter = 1e-12, 0.0, 400
    S = ops.AMRMultiGrid(op, o)
    du = [dev(x) for x in u]
    d_phi = torch.zeros(abi.cell_shape(g), dtype=torch.float64, device="cuda")
    st, rc = S.levelMacProject(du, [dev(x) for x in pi], d_phi)
    assert rc == rc_ref and st.iterations == st_ref.iterations
    exact(host(d_phi), phi_ref)
    for d in range(2):
        exact(host(du[d]), u_ref[d])


def test_backward_euler_steps_bitwise():
    from mushy_gb300 import ops
    n, dt = 32, 1e-3
    g = P.grid((n, n))
    p = P.mushy_params()
    phi_bc, der = P.hc_bcs("mixed")
    rng = np.random.default_rng(41)
    phi = P.hc_state(g, rng, regimes=False)
    b = [np.stack([-np.ones(abi.face_shape(g, d)), -0.02 * np.ones(abi.face_shape(g, d))])
         for d in range(2)]
    src = 0.1 * rng.standard_normal(phi.shape)
    ref = O.NLOpHost(g, p, phi_bc, der, 1.0, 1.0, None, b)
    opts = O.default_options(1)
    op = ops.NLMultiCompOp(g, p, phi_bc, der, 1.0, 1.0, None, [dev(x) for x in b])
    S = ops.AMRFASMultiGrid(op, ops.default_options(True))
    h_phi, d_phi = phi.copy(), dev(phi)
    d_src = dev(src)
    for step in range(3):
        new_ref, st_ref, rc_ref = O.hc_backward_euler(ref, opts, h_phi, h_phi, dt, src)
        d_new = d_phi.clone()
        st, rc = S.backwardEuler(d_new, d_phi, dt, src=d_src)
        assert rc == rc_ref and st.iterations == st_ref.iterations
        exact(host(d_new), new_ref)
        h_phi, d_phi = new_ref, d_new


@pytest.mark.parametrize("n", [(32, 32), (16, 16, 8)])
def test_tga_steps_bitwise(n):
    """mlgpu_hc_tga_step against the oracle's TGA step: the right-hand side
    (a + mu3 dt L) phi_old + dt src and both FAS solves, with a source, an a
    coefficient and mixed walls, three steps through phase change."""
    from mushy_gb300 import ops
    dt = 1e-3
    g = P.grid(n)
    p = P.mushy_params()
    phi_bc, der = P.hc_bcs("mixed")
    rng = np.random.default_rng(42)
    phi = P.hc_state(g, rng, regimes=False)
    phi[0] = rng.uniform(4.4, 5.6, phi[0].shape)
    b = [np.stack([-np.ones(abi.face_shape(g, d)), -0.02 * np.ones(abi.face_shape(g, d))])
         for d in range(g.dim)]
    aC = rng.uniform(0.8, 1.2, phi.shape)
    src = 0.1 * rng.standard_normal(phi.shape)
    ref = O.NLOpHost(g, p, phi_bc, der, 1.0, 1.0, aC, b)
    opts = O.default_options(1)
    op = ops.NLMultiCompOp(g, p, phi_bc, der, 1.0, 1.0, dev(aC), [dev(x) for x in b])
    S = ops.AMRFASMultiGrid(op, ops.default_options(True))
    h_phi, d_phi = phi.copy(), dev(phi)
    d_src, d_a = dev(src), dev(aC)
    for step in range(3):
        new_ref, st_ref, rc_ref = O.hc_tga_step(ref, opts, h_phi, h_phi, dt, src, aC)
        d_new = d_phi.clone()
        st, rc = S.tgaStep(d_new, d_phi, dt, src=d_src, aCoef=d_a)
        assert rc == rc_ref and st.iterations == st_ref.iterations
        exact(host(d_new), new_ref)
        h_phi, d_phi = new_ref, d_new


@pytest.mark.parametrize("n", [(64, 64), (32, 32, 32)])
def test_tga_steps_newton(n):
    """The TGA step on a Jacobian solver (Newton's solves, to 1e-10): FP64
    against the oracle's Newton TGA step to 1e-10 (the L2 merit is summed in
    another order), mixed precision within 1e-8 of FP64, three steps with a
    source through the mush, slow solute diffusion."""
    from mushy_gb300 import ops
    dt = 2e-3
    g = P.grid(n)
    p = P.mushy_params()
    phi_bc, der = P.hc_bcs("mixed")
    rng = np.random.default_rng(43)
    phi = P.hc_state(g, rng, regimes=False)
    phi[0] = rng.uniform(4.6, 6.4, phi[0].shape)
    b = [np.stack([-np.ones(abi.face_shape(g, d)), -0.01 * np.ones(abi.face_shape(g, d))])
         for d in range(g.dim)]
    src = 0.1 * rng.standard_normal(phi.shape)
    ref = O.NLOpHost(g, p, phi_bc, der, 1.0, -dt, None, b)
    oo = O.default_options(1)
    oo.tolerance, oo.hang, oo.max_iter = 1e-10, -1.0, 60
    op = ops.NLMultiCompOp(g, p, phi_bc, der, 1.0, -dt, None, [dev(x) for x in b])
    solvers = {}
    for prec in (abi.PREC_F64, abi.PREC_MIXED):
        o = ops.default_options(True)
        o.tolerance, o.hang, o.max_iter, o.precision = 1e-10, -1.0, 60, prec
        solvers[prec] = ops.AdjointMultiGrid(op, o)
    h = phi.copy()
    cur = {k: dev(phi) for k in solvers}
    d_src = dev(src)
    for step in range(3):
        h, st_r, rc_r = O.hc_tga_step(ref, oo, h, h, dt, src, newton=True)
        assert rc_r == 0
        out = {}
        for k, S in solvers.items():
            new = cur[k].clone()
            st, rc = S.tgaStep(new, cur[k], dt, src=d_src)
            assert rc == 0 and st.final_norm <= 1e-10 * st.initial_norm, (k, step, rc)
            out[k] = host(new)
            cur[k] = new
        scale = np.abs(h).max()
        assert np.abs(out[abi.PREC_F64] - h).max() <= 1e-10 * scale, step
        assert np.abs(out[abi.PREC_MIXED] - out[abi.PREC_F64]).max() <= 1e-8 * scale, step


# ----------------------------------- nonlinear temperature conditions on H
def nl_setup_temperature(n, per, seed, method, limit):
    from mushy_gb300 import ops
    rng = np.random.default_rng(seed)
    g = P.grid(n, per)
    p = P.mushy_params()
    phi_bc, der, nlbc = P.temperature_bcs(method, limit=limit, dim=len(n))
    phi = P.hc_state(g, rng)
    rhs = phi + 0.1 * rng.standard_normal(phi.shape)
    b = P.faces(g, rng, 2)
    aC = rng.uniform(0.5, 1.5, phi.shape)
    alpha, beta = 1.0, -2e-3
    ref = O.NLOpHost(g, p, phi_bc, der, alpha, beta, aC, b, apply_derived_bc=0, nlbc=nlbc)
    op = ops.NLMultiCompOp(g, p, phi_bc, der, alpha, beta, dev(aC), [dev(x) for x in b],
                           apply_derived_bc=False, nlbc=nlbc)
    return g, ref, op, phi, rhs


@pytest.mark.parametrize("n,per", [CASES_2D[0], CASES_2D[1], CASES_3D[0], CASES_3D[1]])
@pytest.mark.parametrize("method", [abi.NLBC_PICARD, abi.NLBC_NEWTON])
@pytest.mark.parametrize("limit", [0.0, 0.3])
def test_nl_temperature_bc_bitwise(n, per, method, limit):
    """Fixed-temperature, temperature-flux and radiation conditions on H
    (ghost enthalpy solved per boundary cell, every closure regime next to
    the walls, no-flux limit on part of one wall): residual, apply, red/black
    passes and FAS restriction bitwise equal to the oracle."""
    g, ref, op, phi, rhs = nl_setup_temperature(n, per, 60, method, limit)
    d_phi, d_rhs = dev(phi), dev(rhs)
    res = torch.empty_like(d_phi)
    op.residual(res, d_phi, d_rhs)
    exact(host(res), O.nl_residual(ref, phi, rhs))
    lhs = torch.empty_like(d_phi)
    op.applyOp(lhs, d_phi)
    exact(host(lhs), O.nl_apply(ref, phi))
    rc = op.createCoarser()
    op.restrictResidual(rc, d_phi, d_rhs)
    exact(host(rc), O.nl_restrict_residual(ref, phi, rhs))
    op.levelGSRBPass(d_phi, d_rhs, 1)
    r = O.nl_gsrb_pass(ref, phi, rhs, 1)
    exact(host(d_phi), r)
    op.relax(d_phi, d_rhs, 2)
    exact(host(d_phi), O.nl_relax(ref, r, rhs, 2))


def _temperature_solve_problem(n, seed, method=abi.NLBC_PICARD):
    from mushy_gb300 import ops
    g = P.grid(n)
    p = P.mushy_params()
    phi_bc, der, nlbc = P.temperature_bcs(method, limit=0.3)
    rng = np.random.default_rng(seed)
    phi = P.hc_state(g, rng, regimes=False)
    b = [np.stack([-np.ones(abi.face_shape(g, d)), -0.01 * np.ones(abi.face_shape(g, d))])
         for d in range(2)]
    dt = 1e-3
    ref = O.NLOpHost(g, p, phi_bc, der, 1.0, -dt, None, b, apply_derived_bc=0, nlbc=nlbc)
    op = ops.NLMultiCompOp(g, p, phi_bc, der, 1.0, -dt, None, [dev(x) for x in b],
                           apply_derived_bc=False, nlbc=nlbc)
    return g, ref, op, phi


@pytest.mark.parametrize("method", [abi.NLBC_PICARD, abi.NLBC_NEWTON])
def test_hc_solver_temperature_bc_matches_oracle(method):
    """FAS solve with temperature conditions on H: the coarse levels keep the
    condition built at the finest spacing; iterations, statistics and the
    solution bitwise equal to the oracle's driver."""
    from mushy_gb300 import ops
    g, ref, op, phi = _temperature_solve_problem((32, 32), 61, method)
    opts = O.default_options(1)
    opts.max_iter = 6
    sol_ref, st_ref, rc_ref = O.hc_solve(ref, opts, phi, phi.copy())
    assert st_ref.final_norm < st_ref.initial_norm
    for graph in (0, 2):
        o = ops.default_options(True)
        o.max_iter, o.use_graph = 6, graph
        d_phi = dev(phi)
        st, rc = ops.AMRFASMultiGrid(op, o).solve(d_phi, dev(phi))
        assert rc == rc_ref and st.iterations == st_ref.iterations
        exact(host(d_phi), sol_ref)


def test_hc_solver_mixed_with_temperature_bc():
    """The mixed nonlinear solve (FP32 linearised cycles, whose ghosts use the
    homogeneous form of the condition: e_H ghost = interior) still reaches
    1e-10 under the FP64 residual that carries the temperature conditions."""
    from mushy_gb300 import ops
    g, ref, op, phi = _temperature_solve_problem((48, 32), 62)
    rhs = phi.copy()
    sols = {}
    for prec in (abi.PREC_F64, abi.PREC_MIXED):
        o = ops.default_options(True)
        o.max_iter, o.tolerance, o.hang, o.precision = 80, 1e-10, 1e-15, prec
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
