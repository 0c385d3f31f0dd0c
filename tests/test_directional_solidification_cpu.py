"""The nonlinear (H, C) operator, its closure and Dirichlet diagnostic walls
pinned in the mushy regime by the reference's own analytic solution:
steady directional solidification without flow (Worster's mushy layer),
which the reference's convergence test test/testDiffusiveSolidification.py
compares its runs against (analyticSolnSolidificationNoFlow,
src/analyticSolns.cpp:39-260; z(theta) of the mush,
MushyLayerParams::directionalSolidificationMushyZ,
src/MushyLayerParams.cpp:1092-1115).

Parameters of that test (params/convergenceTest/noFlowConvTest.parameters):
St = 5, CR = 5, cp = 1, k = 1e-3, frame velocity V = 1 (the file's later
definition wins), Lewis number infinite (no salt diffusion), bottom liquid
H = 6.1 (T = 1.1), C = -1, top at the eutectic (T = 0), periodic in x.

Backward-Euler steps of the oracle's Newton driver on the path's operator,
with the frame advection -V dH/dz as the explicit step source (central
differences; test glue, not on the path), run to the steady state; the
cell temperatures and porosities converge to the analytic profile at second
order.  The device solvers equal the oracle bit for bit (GPU tests), so the
pin carries over to them.
"""
import os

import numpy as np
import pytest
from scipy.optimize import brentq

import refpaths
from mushy_gb300 import abi
from oracle import oracle as O

ST, CR, K, V = 5.0, 5.0, 1e-3, 1.0
H_BOTTOM, T_TOP = 6.1, 0.0
T_BOTTOM = H_BOTTOM - ST   # the liquid closure of the bottom wall, as the reference forms it
Z_EUTECTIC = 1.0   # the top wall: the top temperature is the eutectic's


def _z_mush(theta, theta_inf):
    """Height of temperature theta in the mush (directionalSolidificationMushyZ)."""
    A = 0.5 * (CR + theta_inf + ST)
    B = np.sqrt(A * A - CR * theta_inf - ST)
    al, be = A + B, A - B
    return Z_EUTECTIC - (1 / V) * (((al - CR) / (al - be)) * np.log(al / (al - theta))
                                   + ((CR - be) / (al - be)) * np.log(be / (be - theta)))


def analytic(z):
    """(theta, porosity, interface height h, far-field theta) at heights z:
    liquid below h (exponential approach to theta_inf, which is found so that
    the bottom temperature is met), mush above with porosity from the
    liquidus and C = -1."""
    theta_i = 1.0   # liquidus temperature of C = -1 (infinite Lewis number)
    f = lambda ti: ti + (theta_i - ti) * np.exp(V * (0 - _z_mush(theta_i, ti))) - T_BOTTOM
    theta_inf = brentq(f, T_BOTTOM, 100 * T_BOTTOM, xtol=1e-15)
    h = _z_mush(theta_i, theta_inf)
    theta = np.empty_like(z)
    for i, zz in enumerate(z):
        if zz < h:
            theta[i] = theta_inf + (theta_i - theta_inf) * np.exp(V * (zz - h))
        else:
            theta[i] = brentq(lambda t: _z_mush(t, theta_inf) - zz, 1e-14, theta_i, xtol=1e-15)
    chi = np.where(z < h, 1.0, 1 - (1 - theta) / (CR - theta))
    return theta, chi, h, theta_inf


def steady_state(nz, nx=4, t_end=6.0):
    g = abi.make_grid([nx, nz], 1.0 / nz, (1, 0, 0))
    p = abi.make_params(stefan=ST, compositionRatio=CR, waterDistributionCoeff=K,
                        specificHeatRatio=1.0)
    der = abi.make_bc({(1, 0, 0): (abi.BC_DIRICHLET, T_BOTTOM), (1, 1, 0): (abi.BC_DIRICHLET, T_TOP),
                       (1, 0, 1): (abi.BC_DIRICHLET, -1.0), (1, 1, 1): (abi.BC_DIRICHLET, 0.0)})
    dz = 1.0 / nz
    dt = dz / V
    # heat: -D_H (chi + k_T (1 - chi)) = -1 with k_T = 1; salt: no diffusion
    b = [np.stack([-np.ones(abi.face_shape(g, d)), np.zeros(abi.face_shape(g, d))])
         for d in range(2)]
    ref = O.NLOpHost(g, p, abi.make_bc(), der, 1.0, -dt, None, b)
    z = (np.arange(nz) + 0.5) * dz
    phi = np.empty((2, 1, nz, nx))
    phi[0] = (H_BOTTOM * (1 - z))[None, :, None]
    phi[1] = -1.0
    o = O.default_options(1)
    o.tolerance, o.hang, o.max_iter = 1e-12, -1.0, 100
    t, change = 0.0, None
    while t < t_end:
        H = phi[0, 0]
        below = np.vstack([2 * H_BOTTOM - H[:1], H[:-1]])       # Dirichlet H at the bottom
        above = np.vstack([H[1:], 2 * H[-1:] - H[-2:-1]])       # outflow at the top
        rhs = phi.copy()
        rhs[0, 0] += dt * (-V * (above - below) / (2 * dz))
        new, st, rc = O.newton_solve(ref, o, phi, rhs)
        # steps near the steady state stop at the round-off floor
        assert rc in (abi.OK, abi.ERR_HANG) or st.final_norm < 1e-11, (t, rc, st.final_norm)
        change = np.abs(new - phi).max() / dt
        phi, t = new, t + dt
    cl = O.closure(g, p, np.ascontiguousarray(phi))
    T = cl["T"].reshape(nz, nx)
    chi = cl["porosity"].reshape(nz, nx)
    # uniform in x (to round-off: the red/black smoother of an inexact
    # linear solve is not invariant under a one-cell shift in x)
    assert np.abs(T - T[:, :1]).max() <= 1e-12 * np.abs(T).max()
    return z, T[:, 0], chi[:, 0], change


def test_analytic_solution_properties():
    z = (np.arange(64) + 0.5) / 64
    theta, chi, h, theta_inf = analytic(z)
    assert 0.2 < h < 0.25 and theta_inf > T_BOTTOM
    # continuous at the interface, eutectic at the top, monotone cooling upwards
    assert abs(_z_mush(1.0, theta_inf) - h) < 1e-14 and abs(_z_mush(0.0, theta_inf) - 1) < 1e-14
    assert np.all(np.diff(theta) < 0) and chi.min() > 0.8 - 1e-12


def test_steady_mushy_layer_converges_to_the_analytic_profile():
    errs = {}
    for nz in (16, 32):
        z, T, chi, change = steady_state(nz)
        assert change < 1e-9, change                      # steady
        theta, chi_a, h, _ = analytic(z)
        assert (chi < 1).sum() > 0.7 * nz                  # mostly mush
        errs[nz] = (np.abs(T - theta).max(), np.abs(chi - chi_a).max())
    (eT16, ec16), (eT32, ec32) = errs[16], errs[32]
    assert eT16 < 2.5e-3 and eT32 < 7e-4, errs
    assert ec16 < 4e-4 and ec32 < 1.2e-4, errs
    # second order in dz
    assert eT16 / eT32 > 3.2 and ec16 / ec32 > 3.0, errs


PARAMS = refpaths.ref("params", "convergenceTest", "noFlowConvTest.parameters")


@pytest.mark.skipif(not os.path.exists(PARAMS), reason="reference tree not mounted")
def test_setup_is_the_reference_parameter_file():
    """The constants above are what the inputs reader derives from the
    reference's own parameter file of that test."""
    from mushy_gb300.inputs import Inputs
    inp = Inputs.read(PARAMS)
    p, q = inp.params()
    assert (p.stefan, p.compositionRatio, p.waterDistributionCoeff) == (ST, CR, K)
    assert (p.specificHeatRatio, p.heatConductivityRatio) == (1.0, 1.0)
    assert (p.thetaEutectic, p.ThetaEutectic, q["ThetaInitial"]) == (0.0, 0.0, -1.0)
    assert inp.get("parameters.nonDimVel") == V        # the later definition wins
    assert p.saltDiffusionCoeff == 1e-300             # Lewis number 1e300
    g = inp.grid(2)
    assert g.periodic[0] == 1 and g.periodic[1] == 0
    phi_bc, der, adb, nl = inp.hc_bcs(g)
    assert adb == 1
    assert (der.type[1][0][0], der.value[1][0][0]) == (abi.BC_DIRICHLET, T_BOTTOM)
    assert (der.type[1][1][0], der.value[1][1][0]) == (abi.BC_DIRICHLET, T_TOP)
    assert (der.value[1][0][1], der.value[1][1][1]) == (-1.0, 0.0)
