"""The oracle's TGA step of the (H, C) equations (orc_hc_tga_step).

On a periodic box in the liquid (T = H - St, C_l = C, so the operator is the
discrete Laplacian), a Fourier mode sampled at cell centres is an eigenvector
of the discrete operator: the exact solution of the semi-discrete equations
is the mode times exp(lambda t).  The TGA step is second order in time (the
error falls by ~4 when dt halves, against ~2 for backward Euler on the same
problem), and keeps the mean of a periodic field.
"""
import numpy as np
import pytest

import problems as P
from mushy_gb300 import abi
from oracle import oracle as O


def _liquid(n=32, k=1, amp=0.1):
    g = P.grid((n, n), (1, 1, 0))
    p = P.mushy_params()
    x = (np.arange(n) + 0.5) / n
    phi = np.empty((2, n, n))
    phi[0] = 5.0 + 4.0 + amp * np.sin(2 * np.pi * k * x)[None, :]
    phi[1] = -1.0 + amp * np.cos(2 * np.pi * k * x)[None, :]
    ones = np.ones((2, n, n))
    b = [-np.ones((2,) + abi.face_shape(g, d)) for d in range(2)]
    o = O.NLOpHost(g, p, abi.make_bc(), abi.make_bc(), 1.0, -1.0, ones, b)
    cl = O.closure(g, p, phi)
    assert np.all(phi[0].ravel() > cl["Hl"])  # every cell liquid
    lam = -4.0 * n * n * np.sin(np.pi * k / n) ** 2
    return g, o, phi, lam


def _opts():
    opts = O.default_options(1)
    opts.tolerance, opts.hang, opts.max_iter = 1e-11, 0.0, 100
    return opts


def _run(step, o, phi, dt, nsteps):
    cur = phi.copy()
    for _ in range(nsteps):
        cur, st, rc = step(o, _opts(), cur.copy(), cur, dt)
        assert rc in (0, abi.ERR_HANG), rc
    return cur


def _tga_newton(o, opts, phi_new, phi_old, dt):
    return O.hc_tga_step(o, opts, phi_new, phi_old, dt, newton=True)


@pytest.mark.parametrize("scheme,order", [("tga", 2), ("tga_newton", 2), ("be", 1)])
def test_tga_second_order_in_time(scheme, order):
    g, o, phi, lam = _liquid()
    step = {"tga": O.hc_tga_step, "tga_newton": _tga_newton,
            "be": O.hc_backward_euler}[scheme]
    t_end = 0.04
    exact = phi.copy()
    exact[0] = 9.0 + (phi[0] - 9.0) * np.exp(lam * t_end)
    exact[1] = -1.0 + (phi[1] + 1.0) * np.exp(lam * t_end)
    errs = []
    for nsteps in (4, 8, 16):
        out = _run(step, o, phi, t_end / nsteps, nsteps)
        errs.append(np.abs(out - exact).max())
    rates = [np.log2(errs[i] / errs[i + 1]) for i in range(2)]
    assert all(abs(r - order) < 0.25 for r in rates), (errs, rates)
    if scheme != "be":
        # the TGA error at 16 steps is well below backward Euler's at 16
        be = _run(O.hc_backward_euler, o, phi, t_end / 16, 16)
        assert errs[-1] < 0.05 * np.abs(be - exact).max()


def test_tga_keeps_the_mean_and_the_steady_state():
    g, o, phi, lam = _liquid(k=2)
    out, st, rc = O.hc_tga_step(o, _opts(), phi.copy(), phi, 0.01)
    assert rc in (0, abi.ERR_HANG)
    assert abs(out[0].mean() - phi[0].mean()) < 1e-12
    assert abs(out[1].mean() - phi[1].mean()) < 1e-12
    flat = np.stack([np.full_like(phi[0], 9.0), np.full_like(phi[1], -1.0)])
    out, st, rc = O.hc_tga_step(o, _opts(), flat.copy(), flat, 0.01)
    assert rc in (0, abi.ERR_HANG)
    assert np.abs(out - flat).max() < 1e-12


def test_tga_source_and_a_coefficient():
    """With a source s and a coefficient a on the time derivative, the step
    still solves both stages: (a - mu1 dt L) psi = R, (a - mu2 dt L) phi_new
    = a psi, checked by applying the operators to the returned fields."""
    g, o, phi, lam = _liquid(n=16)
    rng = np.random.default_rng(5)
    aC = rng.uniform(0.8, 1.2, phi.shape)
    o.op.aCoef = O._p(aC)
    o.keep.append(aC)
    src = 0.1 * rng.standard_normal(phi.shape)
    dt = 0.01
    out, st, rc = O.hc_tga_step(o, _opts(), phi.copy(), phi, dt, src=src, a=aC)
    assert rc in (0, abi.ERR_HANG)
    a = 2.0 - np.sqrt(2.0) - 1e-12
    d = np.sqrt(a * a - 4 * a + 2)
    mu1, mu2, mu3 = 0.5 * (a - d), 0.5 * (a + d), 1.0 - a

    def apply(beta, x):
        o.op.alpha, o.op.beta = 1.0, beta
        return O.nl_apply(o, x)

    R = apply(mu3 * dt, phi) + dt * src
    # psi from the second stage's equation: a psi = (a - mu2 dt L) phi_new
    psi = apply(-mu2 * dt, out) / aC
    res = apply(-mu1 * dt, psi) - R
    assert np.abs(res).max() <= 1e-9 * np.abs(R).max()
