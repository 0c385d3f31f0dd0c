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

import refpaths
from mushy_gb300 import abi
from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "closure_plt000100.npz")
REF_PLT = refpaths.ref("test", "unit", "data", "plt000100.2d.hdf5")


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


CHK_GOLD = os.path.join(HERE, "golden", "checkpoint_chk000100.npz")
REF_CHK = refpaths.ref("test", "unit", "data", "chk000100.2d.hdf5")


def test_checkpoint_state_closure_matches_plotfile():
    """The reference's checkpoint of step 100 as a restart state: its one-box
    levels' (H, C), in the operators' layout, closed by the oracle, give the
    temperature, porosity and liquid concentration the plotfile of the same
    step holds, bit for bit."""
    z, p, _, _ = _load()
    c = np.load(CHK_GOLD)
    for lev in (0, 1):
        st = c["state%d" % lev]
        ny, nx = st.shape[-2:]
        g = abi.make_grid([nx, ny], float(c["dx%d" % lev]))
        out = O.closure(g, p, np.ascontiguousarray(st))
        sel = z["level"] == lev
        assert np.array_equal(st[0].ravel(), z["H"][sel])
        assert np.array_equal(st[1].ravel(), z["C"][sel])
        for k in ("T", "porosity", "Cl"):
            assert np.array_equal(out[k].ravel(), z[k][sel]), (lev, k)


@pytest.mark.skipif(not (os.path.exists(REF_CHK) and os.path.exists(REF_PLT)),
                    reason="reference tree not mounted")
def test_checkpoint_reader_against_plotfile():
    """Checkpoint and plotfile of the same step: same boxes, the same (H, C)
    bit for bit on every level, and the face-centred advection velocity
    (FluxBox advVel) averaged to cells equals the plotfile's cell-centred
    advection velocity bit for bit -- the face layout (x faces, then y faces,
    i fastest) is read as written."""
    from mushy_gb300 import chombo_hdf5
    chk = chombo_hdf5.read_checkpoint(REF_CHK)
    pf = chombo_hdf5.read_plotfile(REF_PLT)
    ci = {n: i for i, n in enumerate(pf["components"])}
    assert chk["space_dim"] == 2 and chk["attrs"]["iteration"] == 100
    assert chk["components"][:2] == ["Enthalpy", "Bulk concentration"]
    assert len(chk["levels"]) == len(pf["levels"]) == 3
    for lev, (L, P) in enumerate(zip(chk["levels"], pf["levels"])):
        assert len(L["boxes"]) == len(P["boxes"])
        for b, ((lo, hi), pb) in enumerate(zip(L["boxes"], P["boxes"])):
            assert np.array_equal(lo, pb["lo"]) and np.array_equal(hi, pb["hi"])
            for name in ("Enthalpy", "Bulk concentration"):
                assert np.array_equal(L["fields"][name][b][0], pb["data"][ci[name]]), (lev, b, name)
            ux, uy = L["fields"]["advVel"][b]
            assert np.array_equal(0.5 * (ux[0][:, :-1] + ux[0][:, 1:]),
                                  pb["data"][ci["xAdvection velocity"]]), (lev, b)
            assert np.array_equal(0.5 * (uy[0][:-1, :] + uy[0][1:, :]),
                                  pb["data"][ci["yAdvection velocity"]]), (lev, b)
            dv = L["fields"]["Darcy velocity"][b]
            assert np.array_equal(dv[0], pb["data"][ci["xDarcy velocity"]])
    c = np.load(CHK_GOLD)
    for lev in (0, 1):
        st, (lo, hi), dx = chombo_hdf5.level_state(chk, lev)
        assert np.array_equal(st, c["state%d" % lev]) and dx == float(c["dx%d" % lev])
        for d in range(2):
            assert np.array_equal(chk["levels"][lev]["fields"]["advVel"][0][d],
                                  c["advVel%d_%d" % (lev, d)])
    with pytest.raises(ValueError):
        chombo_hdf5.level_state(chk, 2)   # seven boxes
