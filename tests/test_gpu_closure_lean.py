"""The lean closure of the Newton paths (t_cl_lean: reciprocal constants,
square root and quotient from FP32 seeds refined in FP64) against the
closure evaluated in 40-digit decimal arithmetic and against the oracle's
t_cl (the reference's CALCULATE_T_CL in FP64).

The porosity root cancels (-b - sqrt(b^2 - 4ac)), so rounding in its inputs
is amplified: t_cl itself lies up to ~13 ulp (of max(|value|, 1)) from the
decimal closure on random mush states.  Bound tested: the lean closure
within max(32, 2 e_ref + 8) ulp of the decimal closure, e_ref being t_cl's own
largest error there, in every regime (solid, eutectic, mush, liquid, C
clamped at -CR), on random states, on states within a few ulps of every
regime bound (where the regime may flip and the closure's continuity bounds
the difference) and on the 256^3 workload's mushy range, with a median at
most 1 ulp.
"""
from decimal import Decimal, getcontext

import ctypes as C

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


def _lean(g, p, HC):
    from mushy_gb300 import ops
    d = dev(HC)
    out = torch.empty_like(d)
    abi.check(abi.load().mlgpu_closure_tcl_lean(C.byref(g), C.byref(p), ops._ptr(d),
                                                ops._ptr(out), ops._stream()))
    return host(out)


def _truth(H, C_, p):
    """t_cl in 40-digit decimal arithmetic (regime by the decimal bounds)."""
    getcontext().prec = 40
    D = lambda x: Decimal(float(x))
    CR, k, cp, St = D(p.compositionRatio), D(p.waterDistributionCoeff), D(p.specificHeatRatio), D(p.stefan)
    te, Te = D(p.thetaEutectic), D(p.ThetaEutectic)
    H, C_ = D(H), D(C_)
    Hs = Decimal(0) if C_ < -CR else cp * ((-C_ - CR) / k)
    Hs = max(Hs, Decimal(0)) + te * cp
    He = (CR + C_) / (CR + Te) * (St + te * (1 - cp)) + cp * te
    Hl = St - C_ + te + Te
    if H <= Hs:
        return float(H / cp), float(Te)
    if H <= He:
        return float(te), float(Te)
    if H < Hl:
        vC = C_ if C_ >= -CR else -CR
        a = CR * (cp - 1) + St * (k - 1)
        b = CR * (1 - 2 * cp) + H * (1 - k) - vC * (cp - 1) - k * St
        c = (CR + vC) * cp + k * H
        por = (-b - (b * b - 4 * a * c).sqrt()) / (2 * a) if St != 0 else Decimal(1)
        cl = (C_ + CR * (1 - por)) / (por + k * (1 - por))
        return float(-cl), float(cl)
    return float(H - St), float(C_)


def _check(g, p, HC, ulps=32):
    ref = O.closure_tcl(g, p, HC)
    got = _lean(g, p, HC)
    assert np.all(np.isfinite(got))
    eps = np.finfo(np.float64).eps
    H, C_ = HC[0].ravel(), HC[1].ravel()
    tru = np.array([_truth(h, c, p) for h, c in zip(H, C_)]).T.reshape(HC.shape)
    scale = np.maximum(np.abs(tru), 1.0) * eps
    e_lean = np.abs(got - tru) / scale
    e_ref = np.abs(ref - tru) / scale
    e_pair = np.abs(got - ref) / scale
    # as accurate as t_cl: the cancellation in the porosity root amplifies
    # the inputs' rounding alike in both (t_cl reaches ~50 ulp at CR = 25)
    assert e_lean.max() <= max(ulps, 2 * e_ref.max() + 8), (e_lean.max(), e_ref.max())
    assert e_pair.max() <= max(ulps, 3 * e_ref.max() + 8), (e_pair.max(), e_ref.max())
    assert np.median(e_lean) <= 1.0
    return e_lean, e_ref


@pytest.mark.parametrize("params", [dict(), dict(compositionRatio=25.0),
                                    dict(specificHeatRatio=0.7, thetaEutectic=-0.2,
                                         ThetaEutectic=0.3),
                                    dict(waterDistributionCoeff=0.1, stefan=2.0)])
def test_lean_closure_random_states(params):
    rng = np.random.default_rng(11)
    g = P.grid((64, 48))
    p = P.mushy_params(**params)
    HC = np.ascontiguousarray(P.hc_state(g, rng))
    _check(g, p, HC)
    # the mush is exercised
    cl = O.closure(g, p, HC)
    H = HC[0].ravel()
    assert np.count_nonzero((H > cl["He"]) & (H < cl["Hl"])) > 100


def test_lean_closure_near_regime_bounds():
    """States a few ulps either side of H_s, H_e and H_l: the lean bounds may
    put such a cell in the neighbouring regime, where the closure takes the
    same value to within the bound's rounding (the default phase diagram,
    continuous at every bound)."""
    g = P.grid((96, 32))
    p = P.mushy_params()
    rng = np.random.default_rng(12)
    C_ = rng.uniform(-4.0, -0.5, abi.cell_shape(g))
    B = O.closure(g, p, np.ascontiguousarray(np.stack([np.zeros_like(C_), C_])))
    bounds = [B[k].reshape(C_.shape) for k in ("Hs", "He", "Hl")]
    which = np.arange(C_.size).reshape(C_.shape) % 3
    off = rng.integers(-4, 5, C_.shape)
    H = np.choose(which, bounds)
    H = H + off * np.spacing(H)
    _check(g, p, np.ascontiguousarray(np.stack([H, C_])))


def test_lean_closure_workload_range():
    """The mushy states of the 256^3 step: H in (2, 6), C near -1."""
    rng = np.random.default_rng(13)
    g = P.grid((128, 128))
    p = P.mushy_params()
    H = rng.uniform(2.0, 6.0, abi.cell_shape(g))
    C_ = -1.0 + 1e-3 * rng.standard_normal(abi.cell_shape(g))
    _check(g, p, np.stack([H, C_]))
