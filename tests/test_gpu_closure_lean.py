"""The lean closure of the Newton paths (t_cl_lean: reciprocal constants,
square root and quotient from FP32 seeds refined in FP64) against the
oracle's t_cl (the reference's CALCULATE_T_CL in FP64).

Error bound tested: |lean - exact| <= 8 ulp of the closure's scale in every
regime (solid, eutectic, mush, liquid, C clamped at -CR), on random states and
on states within a few ulps of every regime bound; 4 ulp on the mushy states
of the 256^3 workload's range.
"""
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


def _check(g, p, HC, ulps=8):
    ref = O.closure_tcl(g, p, HC)
    got = _lean(g, p, HC)
    scale = np.maximum(np.abs(ref), 1.0)
    err = np.abs(got - ref) / (scale * np.finfo(np.float64).eps)
    assert np.all(np.isfinite(got))
    assert err.max() <= ulps, (err.max(), np.unravel_index(err.argmax(), err.shape))
    return err


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
    same value to within the bound's rounding."""
    g = P.grid((96, 32))
    p = P.mushy_params(thetaEutectic=-0.2)
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
    err = _check(g, p, np.stack([H, C_]), ulps=4)
    assert np.median(err) <= 1.0
