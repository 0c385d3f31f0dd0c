"""The inputs-file reader (mushy_gb300/inputs.py) against the reference's
own run: tests/golden/inputs_unit_data.json holds the keys of the inputs of
test/unit/data (the run that wrote plt000100.2d.hdf5) and the parameters and
base spacing that run wrote into its plotfile.  The reader must derive
exactly those values, and the wall values of the (H, C) operator from the
same phase diagram the oracle restates."""
import json
import os

import numpy as np
import pytest

import problems as P
import refpaths
from mushy_gb300 import abi
from mushy_gb300 import inputs as mi
from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "inputs_unit_data.json")
REF_INPUTS = refpaths.ref("test", "unit", "data", "inputs")


def _run_inputs():
    z = json.load(open(FIX))
    text = "\n".join("%s = %s" % (k, " ".join(v)) for k, v in z["inputs"].items())
    return mi.Inputs.parse(text), z["plotfile"]


def test_parameters_equal_the_values_the_run_wrote():
    inp, w = _run_inputs()
    p, q = inp.params()
    assert p.compositionRatio == w["C"] and p.stefan == w["S"]
    assert p.specificHeatRatio == w["cp"] and p.heatConductivityRatio == w["k"]
    assert p.waterDistributionCoeff == w["pc"]
    assert q["lewis"] == w["L"] and q["darcy"] == w["D"]
    assert (w["timescale"], w["velocity_scale"]) == ("Diffusive", "Advective")
    assert q["nondimensionalisation"] == 0
    # diffusive timescale, advective velocity (src/MushyLayerParams.cpp:734-751)
    assert p.heatDiffusionCoeff == 1.0 and p.saltDiffusionCoeff == 1 / w["L"]
    assert p.viscosityCoeff == q["prandtl"] and p.darcyCoeff == q["prandtl"] / w["D"]
    # reference point at the eutectic: theta_e = Theta_e = 0
    assert p.thetaEutectic == 0.0 and p.ThetaEutectic == 0.0
    assert q["ThetaInitial"] == -1.0 and q["heleShawPermeability"] == 1e4
    g = inp.grid(2)
    lo_i, lo_j, hi_i, hi_j = w["prob_domain"]
    assert (g.n[0], g.n[1]) == (hi_i - lo_i + 1, hi_j - lo_j + 1)
    assert g.dx == w["dx0"] and list(g.periodic) == [0, 0, 0]


def test_wall_values_of_the_run():
    """The run's walls: x no flux; y bottom H 6.3 with no-flux C (closed with
    the initial bulk concentration: liquid, T = 1.3, C_l = -1); y top H 2.5,
    C -1 (eutectic point: T = C_l = 0)."""
    inp, _ = _run_inputs()
    p, q = inp.params()
    g = inp.grid(2)
    T, V = inp.scalar_bcs(2, q)
    assert T["temperatureLo"] == [1, 1] and T["temperatureHi"] == [1, 0]
    assert V["temperatureLo"][1] == O.pd_temperature(p, 6.3, -1.0) == 6.3 - 5.0
    assert V["liquidConcentrationLo"][1] == -1.0
    assert V["temperatureHi"][1] == O.pd_temperature(p, 2.5, -1.0) == 0.0
    assert V["liquidConcentrationHi"][1] == 0.0 and V["porosityHi"][1] == 0.5
    phi_bc, der, adb, nl = inp.hc_bcs(g)
    assert adb == 1
    for d in range(2):
        for s in range(2):
            for c in range(2):
                assert phi_bc.type[d][s][c] == abi.BC_NEUMANN and phi_bc.value[d][s][c] == 0.0
                want = (abi.BC_DIRICHLET, 0.0) if (d, s) == (1, 1) else (abi.BC_NEUMANN, 0.0)
                assert (der.type[d][s][c], der.value[d][s][c]) == want, (d, s, c)
    assert (nl.method, nl.max_iter, nl.max_residual, nl.relax_coeff, nl.dx) == \
        (abi.NLBC_PICARD, 2, 1e-5, 0.5, g.dx)
    o = inp.hc_options()
    assert (o.num_smooth_down, o.num_smooth_up, o.max_iter, o.bottom_max_iter) == (1, 4, 10, 40)
    assert (o.tolerance, o.hang, o.norm_thresh) == (1e-10, 1e-10, 1e-10)
    o = inp.projection_options()
    assert (o.num_smooth_down, o.num_smooth_up, o.max_iter) == (2, 8, 20)   # numSmoothUp=8
    assert o.tolerance == 1e-15


@pytest.mark.skipif(not os.path.exists(REF_INPUTS), reason="reference tree not mounted")
def test_fixture_is_the_runs_inputs():
    inp = mi.Inputs.read(REF_INPUTS)
    z = json.load(open(FIX))
    for k, v in z["inputs"].items():
        assert inp.table[k] == v, k


def test_phase_diagram_point_against_the_oracle():
    """The wall-value phase diagram equals the oracle's scalar restatement
    (temperature, bitwise) and the closure (porosity, C_l) over every
    regime."""
    rng = np.random.default_rng(80)
    p = P.mushy_params()
    q = {k: getattr(p, k) for k in ("compositionRatio", "waterDistributionCoeff",
                                    "specificHeatRatio", "stefan", "thetaEutectic",
                                    "ThetaEutectic")}
    H = rng.uniform(-0.5, 7.0, 400)
    Cc = rng.uniform(-4.0, -0.5, 400)
    g = abi.make_grid([400, 1])
    cl = O.closure(g, p, np.ascontiguousarray(np.stack([H, Cc]).reshape(2, 1, 1, 400)))
    regimes = set()
    for i in range(400):
        por, theta, c_l, _ = mi.phase_diagram_point(H[i], Cc[i], q)
        assert theta == O.pd_temperature(p, H[i], Cc[i])
        assert abs(por - cl["porosity"][i]) <= 1e-13 and abs(c_l - cl["Cl"][i]) <= 1e-12
        regimes.add(0 if por == 0 else 1 if por == 1 else 2)
    assert regimes == {0, 1, 2}


def test_parser_rules():
    inp = mi.Inputs.parse("""
# comment line
parameters.stefan = 4.0   # trailing comment
parameters.stefan = 6.0
bc.scalarLo = noflux fixed open
bc.scalarHi = -1 1
bc.temperatureHi = 1 -1
bc.aLo = 0.1 0.2
bc.bHi = 0.3 0.7
bc.TRefLo = -1.1 0
bc.enthalpyLoVal = 6.0 6.0
bc.enthalpyHiVal = 6.0 1.0
bc.bulkConcentrationLoVal = -1 -1
bc.bulkConcentrationHiVal = -1 -1
main.title = "two words"
main.apply_diagnostic_bcs = false
main.num_cells = 64 32
main.domain_width = 2.0
main.periodic_bc = 1 0
HCMultigrid.relaxMode = 4
HCMultigrid.useRelaxBottomSolver = false
VelocityMultigrid.num_smooth = 3
parameters.compositionRatio = 2
parameters.waterDistributionCoeff = 1e-3
parameters.specificHeatRatio = 1
parameters.heatConductivityRatio = 1
parameters.lewis = 100
parameters.darcy = 0
parameters.eutecticTemp = -23
parameters.eutecticComposition = 230
parameters.initialComposition = 30
parameters.liquidusSlope = -0.1
""")
    assert inp.get("parameters.stefan") == 6.0                 # last definition wins
    assert inp.table["main.title"] == ["two words"]
    T, V = inp.scalar_bcs(2)
    assert T["enthalpyLo"] == [1, 0]                           # names, first match
    assert T["enthalpyHi"] == [0, 0]    # "-1" is not all digits: every token read as a name
    assert T["temperatureHi"] == [1, 0]    # -1 keeps the default (scalarHi, read as names)
    g = inp.grid(2)
    assert list(g.n)[:2] == [64, 32] and g.dx == 2.0 / 64 and g.periodic[0] == 1
    phi_bc, der, adb, nl = inp.hc_bcs(g)
    assert adb == 0 and all(der.type[d][s][c] == abi.BC_NEUMANN for d in range(2)
                            for s in range(2) for c in range(2))
    f32 = lambda v: float(np.float32(v))
    assert nl.a[0][0] == f32(0.1) != 0.1 and nl.a[1][0] == f32(0.2)
    assert nl.b[1][1] == f32(0.7) and nl.T_ref[0][0] == f32(-1.1)
    assert nl.a[0][1] == 0.0                                   # absent: 0
    o = inp.hc_options()
    assert o.relax_mode == abi.RELAX_JACOBI and o.bottom_solver == abi.BOTTOM_RELAX
    o = inp.velocity_options()
    assert (o.num_smooth_down, o.num_smooth_up, o.max_iter, o.tolerance) == (3, 3, 10, 1e-10)
    with pytest.raises(ValueError):
        mi.Inputs.parse("parameters.darcy = 0\nmain.nondimensionalisation = 1\n"
                        "parameters.lewis = 1\nparameters.prandtl = 1").params()


def test_temperature_condition_on_enthalpy_from_inputs():
    """A fixed-temperature enthalpy wall (type 6) becomes the temperature
    condition on H with its wall value; a diagnostic condition the path does
    not have is refused."""
    base = """
bc.scalarLo = 1 1
bc.enthalpyHi = 1 6
bc.enthalpyLoVal = 0 6.3
bc.enthalpyHiVal = 0 -0.4
bc.bulkConcentrationLoVal = -1 -1
bc.bulkConcentrationHiVal = -1 -1
main.num_cells = 16 16
main.domain_width = 1
parameters.stefan = 5
parameters.compositionRatio = 2
parameters.waterDistributionCoeff = 1e-5
parameters.specificHeatRatio = 1
parameters.heatConductivityRatio = 1
parameters.lewis = 200
parameters.darcy = 0
parameters.prandtl = 0
parameters.eutecticTemp = -23
parameters.eutecticComposition = 230
parameters.initialComposition = 30
parameters.liquidusSlope = -0.1
"""
    for adb_key in ("false", "true"):
        inp = mi.Inputs.parse(base + "bc.scalarHi = 1 0\nmain.apply_diagnostic_bcs = %s\n"
                              % adb_key)
        phi_bc, der, adb, nl = inp.hc_bcs(inp.grid(2))
        assert phi_bc.type[1][1][0] == abi.BC_FIXED_TEMPERATURE
        assert phi_bc.value[1][1][0] == -0.4 and phi_bc.type[1][0][0] == abi.BC_NEUMANN
        assert adb == (adb_key == "true")
    # the scalar type reaches the diagnostic temperature too: refused
    inp = mi.Inputs.parse(base + "bc.scalarHi = 1 6\n")
    with pytest.raises(ValueError, match="not on this path"):
        inp.hc_bcs(inp.grid(2))


def test_hc_face_coefficients_order():
    chi = [np.array([[0.0, 0.25, 1.0]]), np.array([[0.5, 0.75]])]
    q = {"heatConductivityRatio": 2.0, "heatDiffusionCoeff": 1.0, "saltDiffusionCoeff": 0.005}
    b = mi.hc_face_coefficients(chi, q)
    assert b[0].shape == (2, 1, 3)
    assert np.array_equal(b[0][0], ((1.0 - chi[0]) * 2.0 + chi[0]) * -1.0)
    assert np.array_equal(b[0][1], chi[0] * -0.005)
    assert b[0][0][0, 2] == -1.0 and b[0][0][0, 0] == -2.0


REG = refpaths.ref("test", "regression")


@pytest.mark.skipif(not os.path.exists(REG), reason="reference tree not mounted")
def test_regression_restart_cases():
    """The reference's two restart regression cases read end to end: inputs
    -> grid, parameters and walls; checkpoint -> restart state.  The grid
    the inputs describe is the checkpoint's base level; later definitions
    win; a wall the path does not have is refused."""
    from mushy_gb300 import chombo_hdf5
    # Darcy-Brinkman restart: the unit-test run, with the Hele-Shaw cell
    # given as nonDimReluctance instead of heleShawPermeability
    inp = mi.Inputs.read(os.path.join(REG, "AMRRestartDarcyBrinkman", "inputs"))
    chk = chombo_hdf5.read_checkpoint(os.path.join(REG, "AMRRestartDarcyBrinkman",
                                                   "restart.2d.hdf5"))
    g = inp.grid(2)
    state, (lo, hi), dx = chombo_hdf5.level_state(chk, 0)
    assert dx == g.dx and list(hi - lo + 1) == [g.n[0], g.n[1]]
    assert int(chk["levels"][0]["attrs"]["is_periodic_0"]) == g.periodic[0] == 0
    p, q = inp.params()
    ref_inp, _ = _run_inputs()
    p_ref, q_ref = ref_inp.params()
    for k in ("compositionRatio", "stefan", "specificHeatRatio", "waterDistributionCoeff",
              "heatConductivityRatio", "saltDiffusionCoeff", "darcyCoeff"):
        assert getattr(p, k) == getattr(p_ref, k), k
    assert q["heleShawPermeability"] == q_ref["heleShawPermeability"] == 1e4
    phi_bc, der, adb, nl = inp.hc_bcs(g)
    cl = O.closure(abi.make_grid([g.n[0], g.n[1]], g.dx), p, state)
    z = np.load(os.path.join(HERE, "golden", "closure_plt000100.npz"))
    sel = z["level"] == 0
    for key in ("T", "porosity", "Cl"):
        assert np.array_equal(cl[key].ravel(), z[key][sel]), key
    # Darcy restart: periodic in x, later definitions of a key win, the
    # partition coefficient is never given (the reference keeps its -999
    # default), and the bottom's inflow/outflow wall is not on the path
    inp = mi.Inputs.read(os.path.join(REG, "AMRRestartDarcy", "inputs"))
    chk = chombo_hdf5.read_checkpoint(os.path.join(REG, "AMRRestartDarcy", "restart.2d.hdf5"))
    g = inp.grid(2)
    state, (lo, hi), dx = chombo_hdf5.level_state(chk, 0)
    assert dx == g.dx and list(hi - lo + 1) == [g.n[0], g.n[1]]
    assert int(chk["levels"][0]["attrs"]["is_periodic_0"]) == g.periodic[0] == 1
    p, q = inp.params()
    assert q["rayleighComposition"] == 400 and q["heleShawPermeability"] == 2.0
    assert p.waterDistributionCoeff == -999.0 and p.specificHeatRatio == 0.529
    T, _ = inp.scalar_bcs(2, q)
    assert T["temperatureLo"][1] == mi.INFLOW_OUTFLOW
    with pytest.raises(ValueError, match="not on this path"):
        inp.hc_bcs(g)


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(REG), "diffusiveGrowth")),
                    reason="reference tree not mounted")
def test_diffusive_growth_inputs():
    """The reference's diffusive-growth case: its Robin coefficients read
    (through single precision, exact here), and its top wall, a mixed
    temperature/salinity condition on the diagnostic temperature, given as
    the derived condition MLGPU_BC_MIXED_TEMPERATURE_SALINITY on T with the
    wall's flux value and the radiation constants of that side."""
    inp = mi.Inputs.read(os.path.join(os.path.dirname(REG), "diffusiveGrowth", "inputs"))
    g = inp.grid(2)
    T, V = inp.scalar_bcs(2)
    assert T["temperatureHi"][1] == mi.MIXED_T_S
    phi_bc, der, apply_dbc, nl = inp.hc_bcs(g)
    assert apply_dbc == 1
    assert der.type[1][1][0] == abi.BC_MIXED_TEMPERATURE_SALINITY
    assert der.value[1][1][0] == -0.5
    assert der.type[1][1][1] in (abi.BC_NEUMANN, abi.BC_DIRICHLET)
    assert (nl.a[1][1], nl.b[1][1], nl.T_ref[1][1]) == (0.5, -1.0, 4.0)
    a, b = inp._bc_info("a", 2), inp._bc_info("b", 2)
    tref = inp._bc_info("TRef", 2)
    assert (a[1][1], b[1][1], tref[1][1]) == (0.5, -1.0, 4.0)
    assert (a[0][1], b[0][1], tref[0][1]) == (1.0, 1.0, 0.0)


POISEUILLE = os.path.join(os.path.dirname(REG), "poiseuilleFlow", "inputs")


@pytest.mark.skipif(not os.path.exists(POISEUILLE), reason="reference tree not mounted")
def test_poiseuille_inputs_give_the_pinned_coefficients():
    """The reference's Poiseuille case (Da 0.01, Pr 1, diffusive timescale):
    the Darcy-Brinkman coefficients the reader derives are the ones the
    Poiseuille-Brinkman pin of the oracle uses, c = chi / (Pi Da) = 100 for
    chi = Pi = 1 and viscosity 1 (b = -1)."""
    inp = mi.Inputs.read(POISEUILLE)
    p, q = inp.params()
    assert q["nondimensionalisation"] == 0 and q["darcy"] == 0.01 and q["prandtl"] == 1.0
    assert p.darcyCoeff == 1 / 0.01 == 100.0 and p.viscosityCoeff == 1.0
    g = inp.grid(2)
    assert list(g.n)[:2] == [64, 64] and g.dx == 1.0 / 64


def test_time_integration_order():
    """main.time_integration_order picks the (H, C) step: the reference's
    unit-test and restart-regression inputs ask for TGA (2), its
    diffusive-growth inputs for backward Euler (1); absent, 1."""
    assert mi.Inputs.parse("main.num_cells = 8 8\n").time_integration_order() == 1
    assert mi.Inputs.parse("main.time_integration_order = 2\n").time_integration_order() == 2
    with pytest.raises(ValueError, match="time_integration_order"):
        mi.Inputs.parse("main.time_integration_order = 3\n").time_integration_order()
    cases = [(REF_INPUTS, 2),
             (os.path.join(os.path.dirname(REG), "diffusiveGrowth", "inputs"), 1),
             (os.path.join(REG, "AMRRestartDarcyBrinkman", "inputs"), 2)]
    for path, order in cases:
        if os.path.exists(path):
            assert mi.Inputs.read(path).time_integration_order() == order, path
