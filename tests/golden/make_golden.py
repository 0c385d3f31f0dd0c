"""Generates tests/golden/closure_plt000100.npz and
tests/golden/checkpoint_chk000100.npz from the reference's own data.

Source: test/unit/data/plt000100.2d.hdf5 of the mushy-layer project, a
3-level AMR plotfile written by the reference (AMRLevelMushyLayer plot
output; components 0-4 are Enthalpy, Bulk concentration, Temperature,
Porosity, Liquid concentration, the last three produced by
updateEnthalpyVariables, src/phaseDiagram.cpp:92-177).  The phase-diagram
parameters are the file's root attributes (C = compositionRatio,
S = stefan, cp = specificHeatRatio, pc = waterDistributionCoeff).

The second fixture comes from test/unit/data/chk000100.2d.hdf5, the
checkpoint the same run wrote at the same step: the (H, C) state and the
face-centred advection velocity (advVel) of its one-box levels 0 and 1.
The third, inputs_unit_data.json, keeps the keys of the run's
test/unit/data/inputs that mushy_gb300.inputs reads, beside the parameters
and base spacing the run wrote into its plotfile.

The reference tree is only present where the fixture is generated; the GPU
box and the tests read the committed .npz.  Run:
    python tests/golden/make_golden.py /path/to/mushy-layer
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "mushy-layer_gb300"))
from mushy_gb300 import chombo_hdf5  # noqa: E402


def main(ref_root):
    path = os.path.join(ref_root, "test", "unit", "data", "plt000100.2d.hdf5")
    pf = chombo_hdf5.read_plotfile(path)
    a = pf["attrs"]
    assert pf["components"][:5] == ["Enthalpy", "Bulk concentration", "Temperature",
                                    "Porosity", "Liquid concentration"]
    cols = [[] for _ in range(5)]
    level = []
    for lev_i, lev in enumerate(pf["levels"]):
        for b in lev["boxes"]:
            for c in range(5):
                cols[c].append(b["data"][c].ravel())
            level.append(np.full(b["data"][0].size, lev_i, dtype=np.int8))
    H, C, T, chi, Cl = [np.concatenate(x) for x in cols]
    out = os.path.join(HERE, "closure_plt000100.npz")
    np.savez_compressed(
        out, H=H, C=C, T=T, porosity=chi, Cl=Cl, level=np.concatenate(level),
        compositionRatio=float(a["C"]), stefan=float(a["S"]),
        specificHeatRatio=float(a["cp"]), waterDistributionCoeff=float(a["pc"]),
        max_enthalpy_level0=max(b["data"][0].max() for b in pf["levels"][0]["boxes"]),
        max_enthalpy_level2=max(b["data"][0].max() for b in pf["levels"][2]["boxes"]))
    print("wrote", out, H.size, "cells")

    chk = chombo_hdf5.read_checkpoint(
        os.path.join(ref_root, "test", "unit", "data", "chk000100.2d.hdf5"))
    fx = {}
    for lev in (0, 1):
        state, (lo, hi), dx = chombo_hdf5.level_state(chk, lev)
        fx["state%d" % lev] = state
        fx["lo%d" % lev], fx["hi%d" % lev], fx["dx%d" % lev] = lo, hi, dx
        for d, f in enumerate(chk["levels"][lev]["fields"]["advVel"][0]):
            fx["advVel%d_%d" % (lev, d)] = f
    out = os.path.join(HERE, "checkpoint_chk000100.npz")
    np.savez_compressed(out, **fx)
    print("wrote", out)

    # the run's inputs, reduced to the keys the inputs reader takes, with
    # the parameters and spacing the run wrote into its plotfile
    from mushy_gb300 import inputs as mi
    inp = mi.Inputs.read(os.path.join(ref_root, "test", "unit", "data", "inputs"))
    keep = ("parameters.", "bc.", "main.num_cells", "main.domain_", "main.periodic_bc",
            "main.nondimensionalisation", "main.max_bc", "main.bc_", "main.nonlinear_bc",
            "main.apply_diagnostic_bcs", "HCMultigrid.", "projection.", "VelocityMultigrid.")
    table = {k: v for k, v in sorted(inp.table.items()) if k.startswith(keep)}
    written = {k: float(a[k]) for k in ("C", "D", "L", "S", "cp", "k", "pc")}
    written.update(timescale=a["timescale"], velocity_scale=a["velocity_scale"],
                   dx0=float(pf["levels"][0]["attrs"]["dx"]),
                   prob_domain=[int(x) for x in pf["levels"][0]["attrs"]["prob_domain"].tolist()])
    out = os.path.join(HERE, "inputs_unit_data.json")
    with open(out, "w") as f:
        json.dump({"inputs": table, "plotfile": written}, f, indent=1, sort_keys=True)
        f.write("\n")
    print("wrote", out)


if __name__ == "__main__":
    # default: MUSHY_LAYER_REFERENCE, else the directory `reference` beside
    # this repository's root (tests/refpaths.py)
    sys.path.insert(0, os.path.dirname(HERE))
    import refpaths
    main(sys.argv[1] if len(sys.argv) > 1 else refpaths.reference_root())
