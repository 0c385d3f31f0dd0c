"""Reader of the reference's `inputs` files (Chombo ParmParse, `key = value
value ...`) for the quantities this path takes: the phase-diagram and
transport parameters (mlgpu_params), the boundary conditions of the
(H, C) operator, the temperature-condition parameters (mlgpu_nlbc), the
multigrid settings of the enthalpy, projection and velocity solves, and the
base grid.

Each step restates the reference's own parsing, with the results-relevant
quirks kept:
* parameters: MushyLayerParams::getParameters (src/MushyLayerParams.cpp:
  215-500, derived groups when a key is absent; :705-828, the transport
  coefficients of each nondimensionalisation and their main.* overrides);
* BC types and values: parseBCs / parseBCVals (:864-1013; a type that is
  not all digits is read as a name, unknown names become Dirichlet),
  the defaults and override order of :535-693, and computeDerivedBCs
  (:130-180), which closes the (H, C) wall values with the scalar phase
  diagram (src/phaseDiagram.cpp:178-341) for the T and C_l wall values;
* BCInfo (BCutil/BCInfo.h), which reads bc.aLo / bc.bHi / bc.TRefLo /
  bc.NoFluxLimitHi ... through a std::vector<float>: those values are
  rounded to single precision;
* the (H, C) operator's walls: no flux on (H, C) (`noFluxBC`,
  srcSubcycle/AMRLevelMushyLayerInit.cpp:956-966) except enthalpy
  temperature conditions, and the diagnostic (T, C_l) conditions of
  temperatureLiquidSalinityBC (BCutil/PhysBCUtil.cpp:3741-3788) where
  Neumann is always a zero gradient (PhysBCUtil.cpp:975-981);
* solver settings: HCMultigrid.* and VelocityMultigrid.*
  (srcSubcycle/MushyLayerSubcycleUtils.cpp:654-692), projection.*
  (srcSubcycle/Projector.cpp:44-64,388-443); the projection and velocity
  solves take the BiCGStab bottom as the reference does (relaxation when
  projection.relax_bottom_solver is set), the (H, C) solve relaxation;
* the grid: main.num_cells, main.domain_width / domain_length /
  domain_height (srcSubcycle/MushyLayerSubcycleUtils.cpp:115-140),
  main.periodic_bc.

Host-side setup code: nothing here runs on the GPU.
"""
import ctypes
import struct

import numpy as np

from . import abi

# scalar BC types (BCutil/PhysBCUtil.H:57-137)
DIRICHLET, NEUMANN, INFLOW_OUTFLOW, ONLY_INFLOW, ROBIN, VARIABLE_FLUX = 0, 1, 2, 3, 4, 5
FIXED_TEMPERATURE, TEMPERATURE_FLUX, TEMPERATURE_FLUX_RADIATION = 6, 7, 8
MIXED_T_S, MULTI_DIRI, LIN_DIRI = 9, 10, 11

# names parseBCs accepts, in its order (the first match wins: "open" is 2)
_BC_NAMES = [("noflux", 1), ("fixed", 0), ("open", 2), ("inflow", 3), ("mixed", 9),
             ("solidwall", 0), ("noflow", 0), ("inflowVelocity", 1), ("outflow", 2),
             ("outflownormal", 3), ("inflowoutflow", 4), ("noshear", 5), ("symmetry", 6),
             ("inflowPlume", 7), ("outflowPressureGrad", 8), ("pressureHead", 9)]

_UNSET = -999.0  # MushyLayerParams constructor default (src/MushyLayerParams.cpp:60-100)


def _tokens(line):
    out, cur, quoted = [], "", False
    for ch in line:
        if ch == '"':
            quoted = not quoted
            continue
        if ch.isspace() and not quoted:
            if cur:
                out.append(cur)
                cur = ""
            continue
        cur += ch
    if cur:
        out.append(cur)
    return out


class Inputs:
    """Parsed `key = values` table; a key defined twice keeps its last
    definition, as ParmParse::get returns it."""

    def __init__(self, table):
        self.table = dict(table)

    @classmethod
    def parse(cls, text):
        table = {}
        for raw in text.splitlines():
            line = raw.split("#", 1)[0].strip()
            if "=" not in line:
                continue
            key, val = line.split("=", 1)
            key = key.strip()
            if key:
                table[key] = _tokens(val)
        return cls(table)

    @classmethod
    def read(cls, path):
        with open(path) as f:
            return cls.parse(f.read())

    def has(self, key):
        return key in self.table

    def get(self, key, default=None, kind=float):
        if key not in self.table or not self.table[key]:
            return default
        return _convert(self.table[key][0], kind)

    def getarr(self, key, n, kind=float, default=None):
        if key not in self.table:
            return default
        v = self.table[key]
        if len(v) < n:
            raise ValueError("%s needs %d values, has %d" % (key, n, len(v)))
        return [_convert(x, kind) for x in v[:n]]

    # ------------------------------------------------------------- grid
    def grid(self, dim=2):
        """Base-level box of main.num_cells with the reference's spacing
        (domain width / cells in x); periodicity from main.periodic_bc."""
        n = self.getarr("main.num_cells", dim, int)
        if n is None:
            raise ValueError("main.num_cells missing")
        width = -1.0
        width = self.get("main.domain_length", width)
        width = self.get("main.domain_width", width)
        if self.has("main.domain_height"):
            height = self.get("main.domain_height")
            width = height * n[0] / n[dim - 1]
        if width <= 0:
            raise ValueError("no domain width specified, or domain width is invalid")
        per = self.getarr("main.periodic_bc", dim, int, [0] * dim)
        return abi.make_grid(n, width / n[0], list(per) + [0] * (3 - dim))

    # ------------------------------------------------------- parameters
    def physical_parameters(self):
        """Every named MushyLayerParams quantity the path needs, derived as
        getParameters derives it when the key is absent (IEEE arithmetic: a
        missing key leaves its -999 default in the formulas, as there)."""
        with np.errstate(all="ignore"):
            return self._physical_parameters()

    def _physical_parameters(self):
        P = lambda k, d=_UNSET: np.float64(self.get("parameters." + k, d))
        q = {k: P(k) for k in (
            "viscosity", "heatConductivityLiquid", "heatConductivitySolid",
            "specificHeatLiquid", "specificHeatSolid", "liquidDensity",
            "latentHeatDissolution", "thermalExpansivity", "solutalExpansivity",
            "liquidSoluteDiffusivity", "d", "height", "referencePermeability",
            "gravitationalAcceleration", "eutecticTemp", "eutecticComposition",
            "initialComposition", "liquidusSlope", "waterDistributionCoeff")}
        q["permeabilityFunction"] = self.get("parameters.permeabilityFunction", 2, int)
        q["heleShaw"] = self.get("parameters.heleShaw", False, bool)
        q["problem_type"] = self.get("parameters.problem_type", 0, int)

        def derive(name, fn):
            q[name] = P(name) if self.has("parameters." + name) else fn()

        derive("deltaSalt", lambda: q["eutecticComposition"] - q["initialComposition"])
        derive("deltaTemp", lambda: -q["liquidusSlope"] * q["deltaSalt"])
        derive("stefan", lambda: q["latentHeatDissolution"] / (q["specificHeatLiquid"]
                                                                * q["deltaTemp"]))
        derive("compositionRatio", lambda: (1 - q["waterDistributionCoeff"])
               * q["eutecticComposition"] / q["deltaSalt"])
        derive("liquidHeatDiffusivity", lambda: q["heatConductivityLiquid"]
               / (q["liquidDensity"] * q["specificHeatLiquid"]))
        derive("heatConductivityRatio", lambda: q["heatConductivitySolid"]
               / q["heatConductivityLiquid"])
        derive("specificHeatRatio", lambda: q["specificHeatSolid"] / q["specificHeatLiquid"])
        derive("lewis", lambda: q["liquidHeatDiffusivity"] / q["liquidSoluteDiffusivity"])
        # as written at src/MushyLayerParams.cpp:382
        derive("prandtl", lambda: q["viscosity"] / q["liquidDensity"]
               * q["liquidHeatDiffusivity"])
        derive("darcy", lambda: q["referencePermeability"] / (q["height"] * q["height"]))
        if self.has("parameters.heleShawPermeability"):
            q["heleShawPermeability"] = P("heleShawPermeability")
        elif self.has("parameters.nonDimReluctance"):
            q["heleShawPermeability"] = 1.0 / P("nonDimReluctance")
        else:
            q["heleShawPermeability"] = q["d"] * q["d"] / (12 * q["referencePermeability"])
        derive("rayleighTemp", lambda: q["thermalExpansivity"] * q["liquidDensity"]
               * q["gravitationalAcceleration"] * q["height"] * q["deltaTemp"]
               * q["referencePermeability"] / (q["liquidHeatDiffusivity"] * q["viscosity"]))
        q["rayleighComposition"] = P("rayleighComp") if self.has("parameters.rayleighComp") \
            else (q["solutalExpansivity"] * q["liquidDensity"] * q["gravitationalAcceleration"]
                  * q["height"] * q["deltaSalt"] * q["referencePermeability"]
                  / (q["liquidHeatDiffusivity"] * q["viscosity"]))
        q["referenceTemperature"] = P("referenceTemperature", q["eutecticTemp"])
        q["referenceSalinity"] = P("referenceSalinity", q["eutecticComposition"])
        q["thetaEutectic"] = (q["eutecticTemp"] - q["referenceTemperature"]) / q["deltaTemp"]
        q["ThetaEutectic"] = ((q["eutecticComposition"] - q["referenceSalinity"])
                              / q["deltaSalt"])
        q["ThetaInitial"] = ((q["initialComposition"] - q["referenceSalinity"])
                             / q["deltaSalt"])
        q["ThetaInitial"] = P("initialBulkConc", q["ThetaInitial"])
        q.update(self._transport(q))
        return q

    def _transport(self, q):
        """Coefficients of each nondimensionalisation
        (src/MushyLayerParams.cpp:705-828)."""
        nd = self.get("main.nondimensionalisation", 0, int)
        darcy, pr, le = q["darcy"], q["prandtl"], q["lewis"]
        ra_t, ra_c = q["rayleighTemp"], q["rayleighComposition"]
        darcy_brinkman = darcy > 1e-10
        if not darcy_brinkman and nd != 0:
            raise ValueError("Darcy flow needs the diffusive timescale / advective "
                             "velocity nondimensionalisation (0)")
        if nd == 1:      # Darcy timescale, advective velocity
            dh = 1.0 if darcy == pr else darcy / pr
            t = dict(heatDiffusionCoeff=dh, saltDiffusionCoeff=dh / le, viscosityCoeff=darcy,
                     buoyancyTCoeff=ra_t * darcy * darcy * pr,
                     buoyancySCoeff=ra_c * darcy * darcy * pr, darcyCoeff=1.0)
        elif nd == 0:    # diffusive timescale, advective velocity
            t = dict(heatDiffusionCoeff=1.0, saltDiffusionCoeff=1 / le, viscosityCoeff=pr,
                     buoyancyTCoeff=pr * ra_t, buoyancySCoeff=pr * ra_c,
                     darcyCoeff=pr / darcy)
            if not darcy_brinkman:
                t["buoyancyTCoeff"], t["buoyancySCoeff"] = ra_t, ra_c
        elif nd == 2:    # Darcy timescale, Darcy velocity
            dh = darcy / pr
            t = dict(heatDiffusionCoeff=dh, saltDiffusionCoeff=dh / le, viscosityCoeff=darcy,
                     buoyancyTCoeff=1.0, buoyancySCoeff=ra_c / ra_t, darcyCoeff=1.0)
        elif nd == 3:    # advective timescale, Darcy velocity
            dh = 1 / (darcy * ra_t)
            t = dict(heatDiffusionCoeff=dh, saltDiffusionCoeff=dh / le,
                     viscosityCoeff=pr / (darcy * ra_t), buoyancyTCoeff=pr / (darcy * ra_t),
                     darcyCoeff=pr / (darcy * darcy * ra_t))
            t["buoyancySCoeff"] = t["buoyancyTCoeff"] * (ra_c / ra_t)
        elif nd == 4:    # buoyancy timescale, advective velocity
            R = ra_c
            if R == 0:
                if ra_t == 0:
                    raise ValueError("buoyancy timescale needs RaT or RaC != 0")
                R = ra_t
            dh = 1 / np.sqrt(R * pr)
            t = dict(heatDiffusionCoeff=dh, saltDiffusionCoeff=dh / le,
                     viscosityCoeff=np.sqrt(pr / R), darcyCoeff=(1 / darcy) * np.sqrt(pr / R))
            if ra_c != 0:
                t["buoyancySCoeff"], t["buoyancyTCoeff"] = 1, ra_t / ra_c
            else:
                t["buoyancySCoeff"], t["buoyancyTCoeff"] = 0, 1
        else:
            raise ValueError("unknown nondimensionalisation %d" % nd)
        for k in ("heatDiffusionCoeff", "saltDiffusionCoeff", "viscosityCoeff",
                  "buoyancyTCoeff", "buoyancySCoeff", "darcyCoeff"):
            t[k] = self.get("main." + k, t[k])
        t["nondimensionalisation"] = nd
        return t

    def params(self):
        """mlgpu_params of the path, with the full table of derived
        quantities."""
        q = self.physical_parameters()
        p = abi.make_params(**{k: q[k] for k in (
            "compositionRatio", "waterDistributionCoeff", "specificHeatRatio", "stefan",
            "thetaEutectic", "ThetaEutectic", "heatConductivityRatio", "heatDiffusionCoeff",
            "saltDiffusionCoeff", "darcyCoeff", "viscosityCoeff")})
        return p, q

    # --------------------------------------------------------------- BCs
    def bc_types(self, name, target, required=False):
        """parseBCs: bc.<name> for every direction into `target` (a list)."""
        key = "bc." + name
        if key not in self.table:
            if required:
                raise ValueError("Couldn't find BC " + name)
            return
        toks = self.table[key]
        dim = len(target)
        if _all_digits(toks[0]):
            vals = [int(t) for t in toks[:dim]]
        else:
            vals = [_first_name(t) for t in toks[:dim]]
        if len(vals) < dim:
            raise ValueError("bc.%s needs %d values" % (name, dim))
        for d in range(dim):
            if vals[d] != -1:
                target[d] = vals[d]

    def bc_values(self, name, target, required=False):
        vals = self.getarr("bc." + name, len(target))
        if vals is None:
            if required:
                raise ValueError("Couldn't find BC " + name)
            return
        target[:] = vals

    def _bc_info(self, name, dim):
        """BCInfo: bc.<name>Lo / Hi per direction, through single precision."""
        out = [[0.0] * dim, [0.0] * dim]
        for s, lab in enumerate(("Lo", "Hi")):
            vals = self.getarr("bc." + name + lab, dim)
            if vals is not None:
                out[s] = [_to_float32(v) for v in vals]
        return out

    def scalar_bcs(self, dim=2, q=None):
        """Types and values of the scalar fields per side ([lo, hi] lists over
        directions), as MushyLayerParams holds them after getParameters."""
        if q is None:
            q = self.physical_parameters()
        T = {}
        scalar = {s: [DIRICHLET] * dim for s in ("Lo", "Hi")}
        scalar["Lo"][0] = scalar["Hi"][0] = NEUMANN
        self.bc_types("scalarLo", scalar["Lo"], True)
        self.bc_types("scalarHi", scalar["Hi"], True)
        for var in ("enthalpy", "bulkConcentration", "liquidConcentration", "temperature"):
            for s in ("Lo", "Hi"):
                T[var + s] = list(scalar[s])
        for var in ("enthalpy", "bulkConcentration", "liquidConcentration", "temperature"):
            for s in ("Lo", "Hi"):
                self.bc_types(var + s, T[var + s])
        V = {}
        for var in ("enthalpy", "bulkConcentration"):
            for s in ("Lo", "Hi"):
                V[var + s] = [0.0] * dim
                self.bc_values(var + s + "Val", V[var + s], True)
        # computeDerivedBCs: close the (H, C) wall values (a Neumann C wall
        # takes ThetaInitial) for the T, C_l, porosity wall values
        for var in ("temperature", "liquidConcentration", "porosity"):
            for s in ("Lo", "Hi"):
                V[var + s] = [0.0] * dim
        for d in range(dim):
            for s in ("Lo", "Hi"):
                C = V["bulkConcentration" + s][d]
                if T["bulkConcentration" + s][d] == NEUMANN:
                    C = q["ThetaInitial"]
                por, theta, cl, _ = phase_diagram_point(V["enthalpy" + s][d], C, q)
                V["porosity" + s][d], V["temperature" + s][d] = por, theta
                V["liquidConcentration" + s][d] = cl
        for var in ("liquidConcentration", "temperature"):
            for s in ("Lo", "Hi"):
                self.bc_values(var + s + "Val", V[var + s])
        return T, V

    def hc_bcs(self, grid):
        """(phi_bc, derived_bc, apply_derived_bc, nlbc) of the (H, C)
        operator on `grid`."""
        dim = grid.dim
        p, q = self.params()
        T, V = self.scalar_bcs(dim, q)
        apply_dbc = self.get("main.apply_diagnostic_bcs", True, bool)
        phi, der = {}, {}
        temp_type = {FIXED_TEMPERATURE: abi.BC_FIXED_TEMPERATURE,
                     TEMPERATURE_FLUX: abi.BC_TEMPERATURE_FLUX,
                     TEMPERATURE_FLUX_RADIATION: abi.BC_TEMPERATURE_FLUX_RADIATION}
        for d in range(dim):
            if grid.periodic[d]:
                continue
            for s, lab in enumerate(("Lo", "Hi")):
                th = T["enthalpy" + lab][d]
                if th in temp_type:
                    phi[(d, s, 0)] = (temp_type[th], V["enthalpy" + lab][d])
                if not apply_dbc:
                    continue
                for c, var in enumerate(("temperature", "liquidConcentration")):
                    t = T[var + lab][d]
                    if t == DIRICHLET:
                        der[(d, s, c)] = (abi.BC_DIRICHLET, V[var + lab][d])
                    elif t == NEUMANN:
                        der[(d, s, c)] = (abi.BC_NEUMANN, 0.0)
                    elif t == MIXED_T_S and c == 0:
                        # the Robin ghost on T with the radiation constants
                        # bc.a / bc.b / bc.TRef and the value as its flux
                        der[(d, s, c)] = (abi.BC_MIXED_TEMPERATURE_SALINITY,
                                          V[var + lab][d])
                    elif t == MIXED_T_S:
                        raise ValueError(
                            "bc type 9 (MixedBCTemperatureSalinity) of liquidConcentration "
                            "on side %s of direction %d is not on this path: the reference "
                            "then recomputes the temperature ghost with the liquid "
                            "concentration's value as the flux; give it to the temperature"
                            % (lab, d))
                    else:
                        raise ValueError(
                            "bc type %d of %s on side %s of direction %d is not on this "
                            "path (Dirichlet or Neumann diagnostic conditions, and the mixed "
                            "temperature condition on the temperature)"
                            % (t, var, lab, d))
        a, b = self._bc_info("a", dim), self._bc_info("b", dim)
        tref, lim = self._bc_info("TRef", dim), self._bc_info("NoFluxLimit", dim)
        nl = abi.make_nlbc(
            radiation={(d, s): (a[s][d], b[s][d], tref[s][d]) for d in range(dim)
                       for s in range(2)},
            no_flux_limit={(d, s): lim[s][d] for d in range(dim) for s in range(2)},
            method=self.get("main.nonlinear_bc_solve_method", 0, int),
            max_iter=self.get("main.max_bc_iter", 2, int),
            max_residual=self.get("main.max_bc_residual", 1e-5),
            relax_coeff=self.get("main.bc_relax_coeff", 0.5),
            dx=grid.dx)
        return abi.make_bc(phi), abi.make_bc(der), int(apply_dbc), nl

    # ----------------------------------------------------------- solvers
    def _options(self, hc, keys, **defaults):
        o = abi.MGOptions()
        abi.load().mlgpu_mg_default_options(ctypes.byref(o), int(hc))
        for field, v in defaults.items():
            setattr(o, field, v)
        for field, key, kind in keys:
            v = self.get(key, None, kind)
            if v is not None:
                setattr(o, field, v)
        return o

    def time_integration_order(self):
        """main.time_integration_order (srcSubcycle/MushyLayerSubcycleUtils.cpp:
        625-626, default 1): 1 takes the (H, C) step by backward Euler
        (mlgpu_hc_backward_euler / backwardEuler), 2 by the TGA scheme
        (mlgpu_hc_tga_step / tgaStep), as AMRLevelMushyLayer.cpp:1766-1779
        chooses."""
        order = self.get("main.time_integration_order", 1, int)
        if order not in (1, 2):
            raise ValueError("main.time_integration_order = %d: 1 (backward Euler) or 2 (TGA)"
                             % order)
        return order

    def hc_options(self):
        """HCMultigrid.* (srcSubcycle/MushyLayerSubcycleUtils.cpp:668-692)."""
        o = self._options(True, [
            ("num_smooth_up", "HCMultigrid.num_smooth_up", int),
            ("num_mg", "HCMultigrid.num_mg", int),
            ("hang", "HCMultigrid.hang_eps", float),
            ("norm_thresh", "HCMultigrid.norm_thresh", float),
            ("tolerance", "HCMultigrid.tolerance", float),
            ("max_iter", "HCMultigrid.max_iter", int),
            ("num_smooth_down", "HCMultigrid.numSmoothDown", int),
            ("relax_mode", "HCMultigrid.relaxMode", int),
            ("bottom_max_iter", "HCMultigrid.bottomSolveIterations", int)])
        # HCMultigrid.useRelaxBottomSolver = false would lend the FAS solve the
        # velocity solves' BiCGStab; the FAS bottom here is always relaxation
        return o

    def projection_options(self):
        """projection.* (srcSubcycle/Projector.cpp:44-64,434-443)."""
        o = self._options(False, [
            ("tolerance", "projection.solverTol", float),
            ("num_smooth_up", "projection.numSmoothUp", int),
            ("num_smooth_down", "projection.numSmoothDown", int),
            ("num_mg", "projection.numMG", int),
            ("max_iter", "projection.maxIter", int),
            ("bottom_max_iter", "projection.bottomSolveMaxIter", int),
            ("hang", "projection.solverHang", float),
            ("relax_mode", "projection.mg_relaxation", int)])
        # BiCGStab unless projection.relax_bottom_solver (Projector.cpp:58,440,
        # 2976-2986)
        relax = self.get("projection.relax_bottom_solver", False, bool)
        o.bottom_solver = abi.BOTTOM_RELAX if relax else abi.BOTTOM_BICGSTAB
        return o

    def velocity_options(self):
        """VelocityMultigrid.* (srcSubcycle/MushyLayerSubcycleUtils.cpp:654-665):
        num_smooth sets both sweep counts."""
        o = self._options(False, [
            ("tolerance", "VelocityMultigrid.tolerance", float),
            ("hang", "VelocityMultigrid.hang_eps", float),
            ("num_mg", "VelocityMultigrid.num_mg", int),
            ("norm_thresh", "VelocityMultigrid.norm_thresh", float),
            ("max_iter", "VelocityMultigrid.max_iter", int),
            ("num_smooth_down", "VelocityMultigrid.num_smooth", int),
            ("num_smooth_up", "VelocityMultigrid.num_smooth", int)],
            tolerance=1e-10, hang=1e-10, norm_thresh=1e-10, num_mg=1, max_iter=10,
            num_smooth_down=2, num_smooth_up=2)
        # the velocity solves' bottom is BiCGStab (s_botSolverUStar,
        # srcSubcycle/AMRLevelMushyLayerInit.cpp:738-739) at its default 80
        # iterations
        o.bottom_solver, o.bottom_max_iter = abi.BOTTOM_BICGSTAB, 80
        return o


def _convert(tok, kind):
    if kind is bool:
        t = tok.lower()
        if t in ("true", "1"):
            return True
        if t in ("false", "0"):
            return False
        raise ValueError("not a boolean: %r" % tok)
    if kind is int:
        return int(tok)
    return float(tok)


def _all_digits(s):
    return bool(s) and all(c.isdigit() for c in s)


def _first_name(tok):
    for name, v in _BC_NAMES:
        if tok == name:
            return v
    return 0  # "Unknown BC": Dirichlet


def _to_float32(v):
    return struct.unpack("f", struct.pack("f", v))[0]


def phase_diagram_point(H, C, q):
    """(porosity, theta, C_l, C_s) of one (H, C) by the scalar phase diagram
    used for boundary values: computeBoundingEnergy and computeEnthalpyVars
    (src/phaseDiagram.cpp:178-222,305-341), same operation order, IEEE
    arithmetic throughout."""
    with np.errstate(all="ignore"):
        return _phase_diagram_point(np.float64(H), np.float64(C), q)


def _phase_diagram_point(H, C, q):
    CR, k = q["compositionRatio"], q["waterDistributionCoeff"]
    cp, St = q["specificHeatRatio"], q["stefan"]
    te, Te = q["thetaEutectic"], q["ThetaEutectic"]
    H_s = cp * (te + max(0.0, (-C - CR) / k))
    chi_e = (CR + C) / (Te + CR)
    H_e = chi_e * (St + te * (1 - cp)) + cp * te
    H_l = St - C + te + Te
    if H <= H_s:
        return 0.0, H / cp, 0.0, C
    if H > H_s and H <= H_e:
        por = (H - te * cp) / (St + te * (1 - cp))
        return por, te, Te, C / (1 - por)
    if H > H_e and H < H_l:
        if St == 0:
            por = 1.0
        else:
            a = CR * (cp - 1) + St * (k - 1)
            b = CR * (1 - 2 * cp) + H * (1 - k) - C * (cp - 1) - k * St
            c = (C + CR) * cp + k * H
            por = (-b - np.sqrt(b * b - 4 * a * c)) / (2 * a)
        cl = (C + CR * (1 - por)) / (por + k * (1 - por))
        cs = (k * C - CR * por) / (por + k * (1 - por))
        return por, -cl, cl, cs
    return 1.0, H - St, C, 0.0


def hc_face_coefficients(porosity_faces, q):
    """bCoef of the (H, C) operator from face porosities, in the reference's
    operation order (srcSubcycle/AMRLevelMushyLayerInit.cpp:925-950):
    b_H = ((1 - chi) k_T + chi) (-D_H), b_C = (1 chi) (-D_C).  Returns, per
    direction, an array [2][faces]."""
    kT, DH, DC = q["heatConductivityRatio"], q["heatDiffusionCoeff"], q["saltDiffusionCoeff"]
    out = []
    for chi in porosity_faces:
        chi = np.asarray(chi, dtype=np.float64)
        bh = ((1.0 - chi) * kT + chi) * (-DH)
        bc = (1.0 * chi) * (-DC)
        out.append(np.ascontiguousarray(np.stack([bh, bc])))
    return out
