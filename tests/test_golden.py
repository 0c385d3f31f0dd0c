"""Closure parity pinned to the reference's own output.

tests/golden/closure_plt000100.npz holds every cell of the reference's
test/unit/data/plt000100.2d.hdf5 (3 AMR levels, 3200 cells, liquid and mushy
regimes): (H, C) in, (T, porosity, C_l) as written by the reference's
updateEnthalpyVariables.  The oracle and the sm_103a closure must reproduce
them bit for bit.
"""
import ctypes as C
import os

import numpy as np
import pytest

from mushy_gb300 import abi
from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "closure_plt000100.npz")
REF_PLT = "/root/reference/test/unit/data/plt000100.2d.hdf5"


def _load():
    z = np.load(GOLD)
    p = abi.make_params(compositionRatio=float(z["compositionRatio"]),
                        stefan=float(z["stefan"]),
                        specificHeatRatio=float(z["specificHeatRatio"]),
                        waterDistributionCoeff=float(z["waterDistributionCoeff"]),
                        thetaEutectic=0.0, ThetaEutectic=0.0)
    n = z["H"].size
    g = abi.make_grid([n, 1])
    HC = np.ascontiguousarray(np.stack([z["H"], z["C"]]).reshape(2, 1, 1, n))
    return z, p, g, HC


def test_golden_fixture_known_answers():
    z = np.load(GOLD)
    # the reference's own unit test pins these (test/unit/test_MushyPltFile.py:29-32)
    assert abs(float(z["max_enthalpy_level0"]) - 6.302214) < 1e-6
    assert abs(float(z["max_enthalpy_level2"]) - 6.307355035152367) < 1e-9
    mush = (z["porosity"] > 0) & (z["porosity"] < 1)
    assert mush.sum() > 400 and (z["porosity"] == 1).sum() > 2000


def test_oracle_closure_bitwise_vs_reference_output():
    z, p, g, HC = _load()
    out = O.closure(g, p, HC)
    for k in ("T", "porosity", "Cl"):
        assert np.array_equal(out[k], z[k]), k


@pytest.mark.skipif(not os.path.exists(REF_PLT), reason="reference tree not mounted")
def test_hdf5_reader_matches_fixture():
    from mushy_gb300 import chombo_hdf5
    pf = chombo_hdf5.read_plotfile(REF_PLT)
    assert pf["attrs"]["num_levels"] == 3
    h0 = np.concatenate([b["data"][0].ravel() for b in pf["levels"][0]["boxes"]])
    z = np.load(GOLD)
    assert np.array_equal(h0, z["H"][z["level"] == 0])


@pytest.mark.gpu
def test_gpu_closure_bitwise_vs_reference_output():
    torch = pytest.importorskip("torch")
    import __graft_entry__
    __graft_entry__.build()
    from mushy_gb300 import ops
    z, p, g, HC = _load()
    d = torch.from_numpy(HC).cuda()
    n = HC.shape[-1]
    outs = {k: torch.empty(n, dtype=torch.float64, device="cuda") for k in ("T", "porosity", "Cl")}
    abi.check(abi.load().mlgpu_closure(C.byref(g), C.byref(p), ops._ptr(d), ops._ptr(outs["T"]),
                                       ops._ptr(outs["porosity"]), ops._ptr(outs["Cl"]),
                                       None, None, None, None, ops._stream()))
    torch.cuda.synchronize()
    for k in outs:
        assert np.array_equal(outs[k].cpu().numpy(), z[k]), k
