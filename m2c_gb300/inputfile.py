"""Reader for the reference's `.st` input files, restricted to the keys the
finite-volume step reads, plus the geometric initial conditions and the line
plots that go with them.

* `parse(text)`: the input grammar of parser/Dictionary.C and
  parser/AssignerCore.C -- `under Name { ... }` and `under Name[i] { ... }`
  blocks, `Key = value;` assignments (numbers, identifiers, quoted strings),
  `//` and `/* */` comments -- into nested dicts (indexed blocks become
  {index: dict}).
* `Case.from_tree(tree)`: the IoData fields of the path (IoData.cpp keyword
  tables; defaults of m2cg_config_default), the initial state of
  SpaceInitializer.cpp:99-143, 237-480, 1365-1512 (default state = the Inlet
  state unless DefaultInitialState is given, IoData.cpp:4032-4040; Plane and
  Sphere entities in OperationOrder slots, SpaceInitializer.cpp:147-230; phi
  starts at the domain diagonal, Main.cpp:207, and takes the signed distance
  to the level-set material's entities), and the line plots.
* `sample_line` / `write_line`: ProbeOutput.cpp:331-343, 360-597, 848-886 --
  points evenly spaced on the segment, trilinear interpolation over the
  ghosted cell-centre grid with unpopulated edge / corner ghosts replaced by
  the mean of the populated corners, output in the reference's format.
* `ProbeOutput`: time histories at the probe nodes of `Output.Probes`
  (ProbeOutput.cpp:14-350, 599-848; IoData.cpp:3152-3230), written when
  Utils.cpp:337-357 says so, one file per requested field.
* `MaterialVolumeOutput`: volume of every material over time
  (`Output.MaterialVolumes`; MaterialVolumeOutput.cpp:11-120).
* `EnergyIntegrationOutput`: per-material volume, mass and energies in a box
  (`Output.EnergyIntegration`; EnergyIntegrationOutput.cpp:13-245,
  IoData.cpp:3237-3281), from `Solver.integrate` on the device.

Anything the path does not implement (other EOS, non-uniform meshes, other
geometric entities, narrow bands, other reinitialization treatments) raises
NotImplementedError naming the key.
"""
import math
import re

import numpy as np

from . import abi

# ---------------------------------------------------------------------------
# Tokenizer and parser (parser/Lexer.l, parser/Parser.y)

_NUM = r"[+-]?(?:\d+\.\d*(?:[eEdD][+-]?\d+)?|\.\d+(?:[eEdD][+-]?\d+)?|\d+[eEdD][+-]?\d+|\d+)"
_TOKEN = re.compile(r'(\s+)|(//[^\n]*)|(/\*.*?\*/)|("[^"]*")|(' + _NUM + r')|([_A-Za-z][A-Za-z0-9_]*)|([-+*\[\]^{}=,():;./])',
                    re.S)


def _tokens(text):
    out, pos = [], 0
    while pos < len(text):
        m = _TOKEN.match(text, pos)
        if not m:
            raise ValueError(f"cannot read input near: {text[pos:pos + 40]!r}")
        pos = m.end()
        if m.group(1) or m.group(2) or m.group(3):
            continue
        if m.group(4):
            out.append(("str", m.group(4)[1:-1]))
        elif m.group(5):
            v = m.group(5)
            if re.fullmatch(r"[+-]?\d+", v):
                out.append(("int", int(v)))
            else:
                out.append(("dbl", float(re.sub("[dD]", "e", v))))
        elif m.group(6):
            w = m.group(6)
            if w == "end":
                break
            out.append(("under", w) if w == "under" else ("sym", w))
        else:
            out.append(("p", m.group(7)))
    return out


# Keys each block declares, for the blocks the path reads: a key assigned in a
# block that does not declare it belongs to the nearest enclosing block that
# does (Parser.y:65-75 searches the enclosing `under` scopes outward).
_STATE_KEYS = {"MaterialID", "Density", "VelocityX", "VelocityY", "VelocityZ", "Pressure", "Temperature",
               "InternalEnergyPerUnitMass"}
_SCHEMA = {
    "StiffenedGasModel": {"SpecificHeatRatio", "PressureConstant", "EnthalpyConstant", "SpecificHeatAtConstantVolume",
                          "ReferenceTemperature", "ReferenceSpecificInternalEnergy", "SpecificHeatAtConstantPressure",
                          "ReferenceSpecificEnthalpy", "ReferenceDensity"},
    "NobleAbelStiffenedGasModel": {"SpecificHeatRatio", "PressureConstant", "VolumeConstant", "EnergyConstant",
                                   "SpecificHeatAtConstantVolume", "TemperatureLawConstant"},
    "MieGruneisenModel": {"ReferenceDensity", "SpecificHeatAtConstantVolume", "BulkSpeedOfSound", "HugoniotSlope",
                          "ReferenceGamma", "ReferenceSpecificInternalEnergy", "SpecificHeatAtConstantPressure",
                          "ReferenceSpecificEnthalpy", "ReferenceTemperature"},
    "Material": {"EquationOfState", "DensityCutOff", "PressureCutOff", "DensityUpperLimit", "PressureUpperLimit",
                 "DensityPrescribedAtFailure"},
    "InitialState": _STATE_KEYS, "Inlet": _STATE_KEYS, "Inlet2": _STATE_KEYS, "Farfield": _STATE_KEYS,
    "Farfield2": _STATE_KEYS, "DefaultInitialState": _STATE_KEYS,
}


class _Parser:
    def __init__(self, text):
        self.toks = _tokens(text)
        self.i = 0
        self.root = {}
        self.scopes = [(None, self.root)]     # (block name, dict), outermost first

    def peek(self):
        return self.toks[self.i] if self.i < len(self.toks) else ("eof", None)

    def take(self, kind, val=None):
        t = self.peek()
        if t[0] != kind or (val is not None and t[1] != val):
            raise ValueError(f"expected {val or kind}, found {t[1]!r}")
        self.i += 1
        return t[1]

    # IntExpr / DblExpr: + - below * /, parentheses, C integer division
    def expr(self):
        v = self.term()
        while self.peek() in (("p", "+"), ("p", "-")):
            op = self.take("p")
            w = self.term()
            v = v + w if op == "+" else v - w
        return v

    def term(self):
        v = self.atom()
        while self.peek() in (("p", "*"), ("p", "/")):
            op = self.take("p")
            w = self.atom()
            if op == "*":
                v = v * w
            elif isinstance(v, int) and isinstance(w, int):
                v = int(v / w)
            else:
                v = v / w
        return v

    def atom(self):
        t = self.peek()
        if t == ("p", "("):
            self.i += 1
            v = self.expr()
            self.take("p", ")")
            return v
        if t[0] in ("int", "dbl"):
            self.i += 1
            return t[1]
        raise ValueError(f"expected a number, found {t[1]!r}")

    def assignable(self):
        path = [self.take("sym")]
        while self.peek() in (("p", "."), ("p", "[")):
            if self.take("p") == ".":
                path.append(self.take("sym"))
            else:
                path.append(int(self.expr()))
                self.take("p", "]")
        return path

    def target(self, path):
        """(dict, key) of an assignable path; its first name is looked up in
        the enclosing scopes outward (a new name opens in the innermost one)."""
        if len(path) == 1:
            return self.scopes[-1][1], path[0]
        d = self.scopes[-1][1]
        for _, blk in reversed(self.scopes):
            if path[0] in blk:
                d = blk
                break
        for k in path[:-1]:
            d = d.setdefault(k, {})
        return d, path[-1]

    def run(self):
        while self.i < len(self.toks):
            t = self.peek()
            if t == ("p", "}"):
                self.i += 1
                if len(self.scopes) == 1:
                    raise ValueError("unbalanced '}'")
                self.scopes.pop()
                continue
            if t[0] == "under":
                self.i += 1
                path = self.assignable()
                d, k = self.target(path)
                blk = d.setdefault(k, {})
                name = next(p for p in reversed(path) if isinstance(p, str))
                self.take("p", "{")
                self.scopes.append((name, blk))
                continue
            path = self.assignable()
            self.take("p", "=")
            t = self.peek()
            if t[0] in ("sym", "str"):
                self.i += 1
                val = t[1]
            else:
                val = self.expr()
            self.take("p", ";")
            d, k = self.target(path)
            if len(path) == 1:
                # a key the innermost block does not declare belongs to the
                # nearest enclosing block that does
                for depth in range(len(self.scopes) - 1, 0, -1):
                    name, blk = self.scopes[depth]
                    if name not in _SCHEMA or k in _SCHEMA[name]:
                        d = blk
                        break
                    d = self.scopes[depth - 1][1]
            d[k] = val
        if len(self.scopes) != 1:
            raise ValueError("missing '}'")
        return self.root


def parse(text):
    """Nested dict of an input file: blocks are dicts, indexed blocks are
    {index: dict}, values are int, float or str (a symbol or a string)."""
    return _Parser(text).run()


# ---------------------------------------------------------------------------
# IoData keyword tables (values as in the reference's enums)

_BC = {"Inlet": abi.BC_INLET, "Inlet2": abi.BC_INLET2, "Farfield": abi.BC_INLET, "Farfield2": abi.BC_INLET2,
       "Wall": abi.BC_SLIPWALL, "SlipWall": abi.BC_SLIPWALL,
       "StickWall": abi.BC_STICKWALL, "NoSlipWall": abi.BC_STICKWALL, "Symmetry": abi.BC_SYMMETRY,
       "Outlet": abi.BC_OUTLET}                                                   # IoData.cpp:527-535
_LSBC = {"ZeroNeumann": abi.LSBC_ZERO_NEUMANN, "LinearExtrapolation": abi.LSBC_LINEAR_EXTRAPOLATION,
         "NonNegative": abi.LSBC_NON_NEGATIVE}                                     # IoData.cpp:1561-1578
_FLUX = {"Roe": abi.FLUX_ROE, "LocalLaxFriedrichs": abi.FLUX_LLF, "HLLC": abi.FLUX_HLLC}   # IoData.cpp:1384-1387
_REC = {"Constant": abi.REC_CONSTANT, "Linear": abi.REC_LINEAR}
_LIM = {"None": abi.LIM_NONE, "GeneralizedMinMod": abi.LIM_GENERALIZED_MINMOD, "VanAlbada": abi.LIM_VANALBADA}
_VAR = {"Primitive": abi.VAR_PRIMITIVE, "Conservative": abi.VAR_CONSERVATIVE,
        "PrimitiveCharacteristic": abi.VAR_PRIMITIVE_CHARACTERISTIC,
        "ConservativeCharacteristic": abi.VAR_CONSERVATIVE_CHARACTERISTIC}
_SLOPE = {"Zero": abi.SLOPE_ZERO, "NonZero": abi.SLOPE_NONZERO}
_MPFLUX = {"Exact": abi.MPFLUX_EXACT, "Numerical": abi.MPFLUX_NUMERICAL, "LocalLaxFriedrichs": abi.MPFLUX_LLF}
_MPREC = {"Constant": abi.MPREC_CONSTANT, "Linear": abi.MPREC_LINEAR}
_PC = {"RiemannSolution": abi.PHASECHANGE_RIEMANN, "Extrapolation": abi.PHASECHANGE_EXTRAPOLATION}
_PCDIR = {"All": abi.PCDIR_ALL, "Upwind": abi.PCDIR_UPWIND}
_RNORMAL = {"Mesh": abi.RNORMAL_MESH, "LevelSet": abi.RNORMAL_LEVEL_SET, "Average": abi.RNORMAL_AVERAGE}
_TS = {"ForwardEuler": abi.TS_FORWARD_EULER, "RungeKutta2": abi.TS_RK2, "RungeKutta3": abi.TS_RK3}
_EOS = {"StiffenedGas": abi.EOS_SG, "NobleAbelStiffenedGas": abi.EOS_NASG, "MieGruneisen": abi.EOS_MG}
_LSSOLVER = {"FiniteVolume": abi.LS_FINITE_VOLUME, "FiniteDifference": abi.LS_FINITE_DIFFERENCE}   # IoData.cpp:1544-1547
_LSFLUX = {"Roe": abi.LSFLUX_ROE, "LocalLaxFriedrichs": abi.LSFLUX_LLF, "Upwind": abi.LSFLUX_UPWIND}


def _int_keys(t):
    """The tree with digit-string keys (indexed blocks after a JSON round trip) as ints."""
    if not isinstance(t, dict):
        return t
    return {(int(k) if isinstance(k, str) and k.isdigit() else k): _int_keys(v) for k, v in t.items()}


def _tok(table, v, key):
    if v not in table:
        raise NotImplementedError(f"{key} = {v} is not supported by this path")
    return table[v]


def _state(d, default=None):
    """StateVariable (IoData.cpp:60-100): density, velocity, pressure, material id."""
    base = default or {"MaterialID": 0, "Density": 1.0e-6, "VelocityX": 0.0, "VelocityY": 0.0,
                       "VelocityZ": 0.0, "Pressure": 0.0}
    s = dict(base)
    s.update({k: v for k, v in (d or {}).items() if k in base})
    return s


def _vec(s):
    return [s["Density"], s["VelocityX"], s["VelocityY"], s["VelocityZ"], s["Pressure"]]


class Case:
    """A configuration, its initial state and its outputs, read from an input tree."""

    def __init__(self):
        self.cfg = None
        self.V = self.ID = self.phi = None
        self.line_plots = []
        self.probes = None
        self.energy_integration = None
        self.material_volumes = None
        self.solution = {"base": "solution", "frequency": 0, "frequency_dt": -1.0, "fields": []}
        self.prefix = ""
        self.max_time = 1e10
        self.max_its = 2 ** 31 - 1
        self.variable_type = "Primitive"
        self.notes = []

    # -- configuration -------------------------------------------------------
    @classmethod
    def from_text(cls, text):
        return cls.from_tree(parse(text))

    @classmethod
    def from_tree(cls, t):
        t = _int_keys(t)
        self = cls()
        c = abi.default_config()
        mesh = t.get("Mesh", {})
        if mesh.get("Type", "ThreeDimensional") != "ThreeDimensional":
            raise NotImplementedError(f"Mesh.Type = {mesh['Type']}")
        for k in mesh:
            if k.startswith("ControlPoint"):
                raise NotImplementedError("non-uniform meshes (Mesh.ControlPoint*)")
        c.x0, c.xmax = float(mesh.get("X0", 0.0)), float(mesh.get("Xmax", 1.0))
        c.y0, c.ymax = float(mesh.get("Y0", 0.0)), float(mesh.get("Ymax", 1.0))
        c.z0, c.zmax = float(mesh.get("Z0", 0.0)), float(mesh.get("Zmax", 1.0))
        c.nx, c.ny, c.nz = (int(mesh.get(f"NumberOfCells{a}", 1)) for a in "XYZ")
        for s, key in enumerate(("X0", "Xmax", "Y0", "Ymax", "Z0", "Zmax")):
            v = mesh.get("BoundaryCondition" + key)
            if v is not None:
                c.bc[s] = _tok(_BC, v, "Mesh.BoundaryCondition" + key)

        mats = t.get("Equations", {}).get("Material", {})
        if not mats:
            raise ValueError("no Equations.Material")
        c.n_materials = len(mats)
        for m, d in sorted(mats.items()):
            eos = _tok(_EOS, d.get("EquationOfState", "StiffenedGas"), f"Material[{m}].EquationOfState")
            if eos == abi.EOS_SG:
                g = d.get("StiffenedGasModel", {})
                abi.set_material(c.mat[m], eos, gamma=g.get("SpecificHeatRatio", 1.4),
                                 pc=g.get("PressureConstant", 0.0))
            elif eos == abi.EOS_NASG:
                g = d.get("NobleAbelStiffenedGasModel", {})
                abi.set_material(c.mat[m], eos, gamma=g.get("SpecificHeatRatio", 1.4),
                                 pc=g.get("PressureConstant", 0.0), b=g.get("VolumeConstant", 0.0),
                                 q=g.get("EnergyConstant", 0.0))
            else:
                g = d.get("MieGruneisenModel", {})
                # MieGruneisenModelData defaults (IoData.cpp:708-722)
                abi.set_material(c.mat[m], eos, rho0=g.get("ReferenceDensity", 8.96e-3),
                                 c0=g.get("BulkSpeedOfSound", 3.933e6), s=g.get("HugoniotSlope", 1.5),
                                 Gamma0=g.get("ReferenceGamma", 1.99),
                                 e0=g.get("ReferenceSpecificInternalEnergy", 0.0))
            if "DensityCutOff" in d:
                c.mat[m].rhomin = float(d["DensityCutOff"])
            if "PressureCutOff" in d:
                c.mat[m].pmin = float(d["PressureCutOff"])

        bcs = t.get("BoundaryConditions", {})
        # Farfield / Farfield2 name the same states as Inlet / Inlet2 (IoData.cpp:1976-1979)
        inlet = _state({**bcs.get("Inlet", {}), **bcs.get("Farfield", {})})
        inlet2 = _state({**bcs.get("Inlet2", {}), **bcs.get("Farfield2", {})})
        for p, v in enumerate(_vec(inlet)):
            c.inlet[p] = v
        for p, v in enumerate(_vec(inlet2)):
            c.inlet2[p] = v

        ns = t.get("Space", {}).get("NavierStokes", {})
        c.flux = _tok(_FLUX, ns.get("Flux", "HLLC"), "Space.NavierStokes.Flux")
        if "EntropyFixCoefficient" in ns:
            c.roe_delta = float(ns["EntropyFixCoefficient"])
        rec = ns.get("Reconstruction", {})
        c.rec_type = _tok(_REC, rec.get("Type", "Linear"), "Reconstruction.Type")
        c.limiter = _tok(_LIM, rec.get("Limiter", "GeneralizedMinMod"), "Reconstruction.Limiter")
        self.variable_type = rec.get("VariableType", "Primitive")
        c.rec_var = _tok(_VAR, self.variable_type, "Reconstruction.VariableType")
        c.slope_near_interface = _tok(_SLOPE, rec.get("SlopeNearInterface", "NonZero"),
                                      "Reconstruction.SlopeNearInterface")
        if "GeneralizedMinModCoefficient" in rec:
            c.minmod_coeff = float(rec["GeneralizedMinModCoefficient"])

        ls = t.get("Space", {}).get("LevelSet", {})
        if len(ls) > 1:
            raise NotImplementedError("more than one level set")
        if ls:
            d = ls[min(ls)]
            c.n_levelsets = 1
            c.ls_matid = int(d.get("MaterialID", 1))
            c.ls_solver = _tok(_LSSOLVER, d.get("Solver", "FiniteDifference"), "LevelSet.Solver")
            c.ls_flux = _tok(_LSFLUX, d.get("Flux", "Roe"), "LevelSet.Flux")
            if "EntropyFixCoefficient" in d:
                c.ls_delta = float(d["EntropyFixCoefficient"])
            lrec = d.get("Reconstruction", {})
            c.ls_rec_type = _tok(_REC, lrec.get("Type", "Linear"), "LevelSet.Reconstruction.Type")
            c.ls_limiter = _tok(_LIM, lrec.get("Limiter", "GeneralizedMinMod"), "LevelSet.Reconstruction.Limiter")
            if "GeneralizedMinModCoefficient" in lrec:
                c.ls_minmod_coeff = float(lrec["GeneralizedMinModCoefficient"])
            if int(d.get("Bandwidth", 2 ** 31 - 1)) < 2 ** 31 - 1:
                raise NotImplementedError("narrow-band level set (LevelSet.Bandwidth)")
            if d.get("Initialization", "DistanceCalculation") != "DistanceCalculation":
                raise NotImplementedError(f"LevelSet.Initialization = {d['Initialization']}")
            for s, key in enumerate(("X0", "Xmax", "Y0", "Ymax", "Z0", "Zmax")):
                v = d.get("BoundaryCondition" + key)
                if v is not None:
                    c.ls_bc[s] = _tok(_LSBC, v, "LevelSet.BoundaryCondition" + key)
            re_ = d.get("Reinitialization", {})
            if re_:
                if re_.get("FirstLayerTreatment", "Fixed") != "Fixed":
                    raise NotImplementedError(f"Reinitialization.FirstLayerTreatment = {re_['FirstLayerTreatment']}")
                c.reinit_frequency_dt = float(re_.get("FrequencyDt", -1.0))
                c.reinit_frequency = int(re_.get("Frequency", -1))
                c.reinit_max_its = int(re_.get("MaxIts", 30))
                c.reinit_cfl = float(re_.get("CFL", 0.8))
                c.reinit_tol = float(re_.get("ConvergenceTolerance", 2.0e-4))

        mp = t.get("MultiPhase", {})
        c.mp_flux = _tok(_MPFLUX, mp.get("Flux", "Numerical"), "MultiPhase.Flux")
        c.mp_recon = _tok(_MPREC, mp.get("ReconstructionAtInterface", "Constant"),
                          "MultiPhase.ReconstructionAtInterface")
        c.mp_phasechange = _tok(_PC, mp.get("PhaseChange", "RiemannSolution"), "MultiPhase.PhaseChange")
        c.mp_phasechange_dir = _tok(_PCDIR, mp.get("PhaseChangeDirection", "Upwind"),
                                    "MultiPhase.PhaseChangeDirection")
        c.mp_riemann_normal = _tok(_RNORMAL, mp.get("RiemannNormal", "Mesh"), "MultiPhase.RiemannNormal")

        er = t.get("ExactRiemannSolution", {})
        for key, attr, typ in (("MaxIts", "maxits_main", int), ("MaxItsBracketing", "maxits_bracket", int),
                               ("MaxItsShock", "maxits_shock", int), ("IntegrationSteps", "numsteps_rarefaction", int),
                               ("Tolerance", "tol_main", float), ("ToleranceShock", "tol_shock", float),
                               ("ToleranceRarefaction", "tol_rarefaction", float),
                               ("MinPressure", "min_pressure", float), ("FailureThreshold", "failure_threshold", float),
                               ("PrescribedPressureUponFailure", "pressure_at_failure", float)):
            if key in er:
                setattr(c, attr, typ(er[key]))

        tm = t.get("Time", {})
        if tm.get("Type", "Explicit") != "Explicit":
            raise NotImplementedError(f"Time.Type = {tm['Type']}")
        c.ts_type = _tok(_TS, tm.get("Explicit", {}).get("Type", "RungeKutta2"), "Time.Explicit.Type")
        if "CFL" in tm:
            c.cfl = float(tm["CFL"])
        if "TimeStep" in tm:
            c.timestep = float(tm["TimeStep"])
        if "MaxTime" in tm:
            c.max_time = float(tm["MaxTime"])
        self.max_time = c.max_time
        if "MaxIts" in tm:
            self.max_its = int(tm["MaxIts"])
            c.max_its = self.max_its
        self.cfg = c

        ic = t.get("InitialCondition", {})
        self._initial_state(ic, inlet)
        out = t.get("Output", {})
        for k, d in sorted(out.get("LinePlot", {}).items()):
            if int(d.get("NumberOfPoints", 0)) == 1:
                # the reference spaces the points (x1 - x0) / (N - 1) apart
                # (ProbeOutput.cpp:335-337): one point has no defined position
                raise ValueError("Output.LinePlot[%s].NumberOfPoints = 1: a line plot needs 0 (off) or at "
                                 "least 2 points" % k)
            self.line_plots.append({"index": k, "FileName": d.get("FileName", ""),
                                    "NumberOfPoints": int(d.get("NumberOfPoints", 0)),
                                    "frequency": int(d.get("Frequency", -100)),
                                    "frequency_dt": float(d.get("TimeInterval", -1.0)),
                                    "x0": [float(d.get("X0", 0.0)), float(d.get("Y0", 0.0)), float(d.get("Z0", 0.0))],
                                    "x1": [float(d.get("Xmax", 0.0)), float(d.get("Ymax", 0.0)),
                                           float(d.get("Zmax", 0.0))]})
        self.prefix = str(out.get("Prefix", ""))
        # solution snapshots (OutputData, IoData.cpp:2970-2974, 3027-3031)
        self.solution = {"base": str(out.get("Solution", "solution")), "frequency": int(out.get("Frequency", 0)),
                         "frequency_dt": float(out.get("TimeInterval", -1.0)),
                         # fields switched On (all Off by default, IoData.cpp:2976-2994)
                         "fields": [name for key, name in (("Density", "density"), ("Velocity", "velocity"),
                                                           ("Pressure", "pressure"), ("MaterialID", "materialid"),
                                                           ("LevelSet0", "levelset0"))
                                    if out.get(key, "Off") == "On"]}
        if "Probes" in out:
            self.probes = _probes(out["Probes"])
        if "EnergyIntegration" in out:
            self.energy_integration = _energy_integration(out["EnergyIntegration"])
        mv = out.get("MaterialVolumes")
        if mv:   # MaterialVolumes::MaterialVolumes, IoData.cpp:2924-2938
            self.material_volumes = {"file": str(mv.get("FileName", "")), "frequency": int(mv.get("Frequency", 10)),
                                     "frequency_dt": float(mv.get("TimeInterval", -1.0))}
        return self

    # -- initial state -------------------------------------------------------
    def _initial_state(self, ic, inlet):
        c = self.cfg
        default = ic.get("DefaultInitialState")
        dstate = _state(default) if default else dict(inlet)   # IoData.cpp:4032-4040
        geo = ic.get("GeometricEntities", {})
        for k in geo:
            if k not in ("Plane", "Sphere"):
                raise NotImplementedError(f"InitialCondition.GeometricEntities.{k}")
        # operation order: each entity takes the first open slot at or after its
        # OperationOrder, entities taken plane-first (SpaceInitializer.cpp:147-230)
        ents = [("Plane", i, d) for i, d in sorted(geo.get("Plane", {}).items())] + \
               [("Sphere", i, d) for i, d in sorted(geo.get("Sphere", {}).items())]
        slots = [None] * len(ents)
        for kind, i, d in ents:
            o = int(d.get("OperationOrder", 0))
            if not 0 <= o < len(ents):
                raise ValueError(f"{kind}[{i}].OperationOrder = {o} outside [0, {len(ents)})")
            for s in range(o, len(ents)):
                if slots[s] is None:
                    slots[s] = (kind, i, d)
                    break
            else:
                raise ValueError("conflicting OperationOrder")
        for kind, i, d in ents:
            if d.get("Inclusion", "Override") != "Override":
                raise NotImplementedError(f"{kind}[{i}].Inclusion = {d['Inclusion']}")

        from .problems import cell_centers
        X, Y, Z = cell_centers(c)
        n = X.size
        V = np.tile(np.asarray(_vec(dstate), np.float64), (n, 1))
        ID = np.full(n, int(dstate["MaterialID"]), np.int32)
        diag = math.sqrt((c.xmax - c.x0) ** 2 + (c.ymax - c.y0) ** 2 + (c.zmax - c.z0) ** 2)   # Main.cpp:207
        phi = np.full(n, diag)

        def dist(kind, d):
            if kind == "Plane":   # GeoTools/DistancePointToPlane.h, GeoTools.h:121-129
                nrm = np.array([d.get("Normal_x", 0.0), d.get("Normal_y", 0.0), d.get("Normal_z", 0.0)], float)
                nrm = nrm / np.linalg.norm(nrm)
                return ((X - d.get("Point_x", 0.0)) * nrm[0] + (Y - d.get("Point_y", 0.0)) * nrm[1] +
                        (Z - d.get("Point_z", 0.0)) * nrm[2])
            cx, cy, cz = d.get("Center_x", 0.0), d.get("Center_y", 0.0), d.get("Center_z", 0.0)   # DistancePointToSphere.h
            return np.sqrt((X - cx) ** 2 + (Y - cy) ** 2 + (Z - cz) ** 2) - d.get("Radius", -1.0)

        for kind, i, d in slots:      # SpaceInitializer.cpp:346-480
            s = _state(d.get("InitialState"))
            dd = dist(kind, d)
            if kind == "Plane":
                inside = dd > 0
            else:
                interior = d.get("Side", "Interior") == "Interior"
                inside = dd < 0 if interior else dd > 0
            V[inside] = _vec(s)
            ID[inside] = int(s["MaterialID"])
        if c.n_levelsets:
            for kind, i, d in slots:  # SpaceInitializer.cpp:1392-1512
                s = _state(d.get("InitialState"))
                if int(s["MaterialID"]) != c.ls_matid:
                    continue
                dd = dist(kind, d)
                take = np.abs(dd) < np.abs(phi)
                if kind == "Plane":
                    val = -dd
                else:
                    val = dd if d.get("Side", "Interior") == "Interior" else -dd
                phi[take] = val[take]
        self.V, self.ID, self.phi = V, ID, phi


# ---------------------------------------------------------------------------
# Line plots


# probe files of the path (Probes::setup, IoData.cpp:3198-3230) and the column
# of each in the sampled values
_PROBE_FIELDS = {"Density": 0, "VelocityX": 1, "VelocityY": 2, "VelocityZ": 3, "Pressure": 4, "MaterialID": 5,
                 "LevelSet0": 6, "LevelSet1": 7, "LevelSet2": 8, "LevelSet3": 9, "LevelSet4": 10}
_PROBE_UNSUPPORTED = ("Temperature", "DeltaTemperature", "LaserRadiance", "LaserIrradiance", "IonizationResult",
                      "ReferenceMap", "PrincipalElasticStresses")


def _probes(pr):
    """Output.Probes: frequency (default -100: only forced writes), time
    interval, file per field, and the node locations (ProbeOutput.cpp:14-45)."""
    for k in _PROBE_UNSUPPORTED:
        if pr.get(k):
            raise NotImplementedError(f"Output.Probes.{k}")
    nodes = pr.get("Node", {})
    locs = [None] * len(nodes)
    for i, d in nodes.items():
        if not 0 <= int(i) < len(nodes):
            raise ValueError(f"Probe node index ({i}) out of range. Should be between 0 and {len(nodes) - 1}.")
        locs[int(i)] = (float(d.get("X", -1.0e20)), float(d.get("Y", -1.0e20)), float(d.get("Z", -1.0e20)))
    files = {k: str(pr[k]) for k in _PROBE_FIELDS if pr.get(k)}
    return {"frequency": int(pr.get("Frequency", -100)), "frequency_dt": float(pr.get("TimeInterval", -1.0)),
            "files": files, "nodes": locs}


# EnergyIntegrationData::setup (IoData.cpp:3256-3281): file per quantity and
# its column in the integrals
_INTEGRALS = {"Volume": 0, "Mass": 1, "TotalEnergy": 2, "TotalEnthalpy": 3, "KineticEnergy": 4,
              "InternalEnergy": 5}


def _energy_integration(ei):
    for k in ("PotentialEnergy", "LaserRadiation"):
        if ei.get(k):
            raise NotImplementedError(f"Output.EnergyIntegration.{k}")
    big = 1.7976931348623157e308
    box = [float(ei.get(k, v)) for k, v in (("Xmin", -big), ("Xmax", big), ("Ymin", -big), ("Ymax", big),
                                            ("Zmin", -big), ("Zmax", big))]
    return {"frequency": int(ei.get("Frequency", -100)), "frequency_dt": float(ei.get("TimeInterval", -1.0)),
            "files": {k: str(ei[k]) for k in _INTEGRALS if ei.get(k)}, "box": box}


def _ghost_coords(n, lo, hi):
    h = (hi - lo) / n
    return lo + 0.5 * h + np.arange(-1, n + 1) * h     # ghosted cell centres


def locate_points(cfg, points):
    """ProbeOutput::SetupInterpolation (ProbeOutput.cpp:360-480) for points on
    the ghosted cell-centre grid: per point the ghosted indices (i, j, k) of
    the lower corner, the trilinear coordinates and which of the eight corners
    are populated (edge and corner ghosts are not)."""
    nx, ny, nz = cfg.nx, cfg.ny, cfg.nz
    px, py, pz = nx + 2, ny + 2, nz + 2
    cx = _ghost_coords(nx, cfg.x0, cfg.xmax)
    cy = _ghost_coords(ny, cfg.y0, cfg.ymax)
    cz = _ghost_coords(nz, cfg.z0, cfg.zmax)

    def locate(c, v):
        # first ghosted index i with v < c[i+1] (ProbeOutput.cpp:392-413)
        for i in range(len(c) - 1):
            if v < c[i + 1]:
                return i, (v - c[i]) / (c[i + 1] - c[i])
        raise ValueError("probe point outside the mesh")

    def populated(i, j, k):
        out = (i == 0 or i == px - 1) + (j == 0 or j == py - 1) + (k == 0 or k == pz - 1)
        return out <= 1

    setup = []
    for q, p in enumerate(points):
        if (p[0] < cx[0] or p[0] >= cx[-1] or p[1] < cy[0] or p[1] >= cy[-1] or p[2] < cz[0] or p[2] >= cz[-1]):
            raise ValueError(f"cannot locate probe node {q} in the domain")
        (i, xi), (j, eta), (k, zeta) = locate(cx, p[0]), locate(cy, p[1]), locate(cz, p[2])
        corners = [(i, j, k), (i + 1, j, k), (i, j + 1, k), (i + 1, j + 1, k),
                   (i, j, k + 1), (i + 1, j, k + 1), (i, j + 1, k + 1), (i + 1, j + 1, k + 1)]
        valid = [populated(*cc) for cc in corners]
        if not any(valid):
            raise ValueError(f"probe node {q} is too close to the edges of the domain boundary")
        setup.append(((i, j, k), (xi, eta, zeta), valid))
    return setup


def interpolate_points(cfg, setup, fields):
    """ProbeOutput::InterpolateSolutionAtProbe (ProbeOutput.cpp:849-886): each
    field (a ghosted array, i fastest) at each located point; unpopulated
    corners take the mean of the populated ones.  Returns (points, fields)."""
    px, py = cfg.nx + 2, cfg.ny + 2
    out = np.zeros((len(setup), len(fields)))
    for q, ((i, j, k), (xi, eta, zeta), valid) in enumerate(setup):
        corners = [(i, j, k), (i + 1, j, k), (i, j + 1, k), (i + 1, j + 1, k),
                   (i, j, k + 1), (i + 1, j, k + 1), (i, j + 1, k + 1), (i + 1, j + 1, k + 1)]
        lin = [(kk * py + jj) * px + ii for ii, jj, kk in corners]
        for fi, f in enumerate(fields):
            cvals = [f[l] if v else 0.0 for l, v in zip(lin, valid)]
            if sum(valid) < 8:
                avg = sum(cvals) / sum(valid)
                cvals = [cv if v else avg for cv, v in zip(cvals, valid)]
            c000, c100, c010, c110, c001, c101, c011, c111 = cvals
            c00 = c000 * (1.0 - xi) + c100 * xi        # MathTools/trilinear_interpolation.h:50-62
            c01 = c001 * (1.0 - xi) + c101 * xi
            c10 = c010 * (1.0 - xi) + c110 * xi
            c11 = c011 * (1.0 - xi) + c111 * xi
            c0 = c00 * (1.0 - eta) + c10 * eta
            c1 = c01 * (1.0 - eta) + c11 * eta
            out[q, fi] = c0 * (1.0 - zeta) + c1 * zeta
    return out


def sample_line(cfg, plot, Vg, IDg, phig=None):
    """Values along a line plot from ghosted arrays (Vg: 5 x N planes, IDg,
    phig: N; N = (nx+2)(ny+2)(nz+2), i fastest).  Returns an array of rows
    {distance, rho, vx, vy, vz, p, T, ID, phi...} as the reference writes them;
    the temperature column is 0 (the path does not model temperature)."""
    npts = plot["NumberOfPoints"]
    if npts < 2:
        raise ValueError("a line plot needs more than one point")
    x0, x1 = np.asarray(plot["x0"], float), np.asarray(plot["x1"], float)
    dxyz = (x1 - x0) / (npts - 1)
    h = math.sqrt(float((dxyz ** 2).sum()))
    fields = [Vg[p] for p in range(5)] + [IDg.astype(np.float64)]
    if phig is not None and cfg.n_levelsets:
        fields.append(phig)
    vals = interpolate_points(cfg, locate_points(cfg, [x0 + q * dxyz for q in range(npts)]), fields)
    dist = np.array([q * h for q in range(npts)])[:, None]
    return np.hstack([dist, vals[:, :5], np.zeros((npts, 1)), vals[:, 5:]])   # temperature column: 0


def is_time_to_write(time, dt, step, frequency_dt, frequency, last, force):
    """Utils.cpp:337-357: forced writes unless one was made at this time; else
    the time interval when given, else the step count."""
    if force:
        return time > last + 0.1 * dt
    if frequency_dt > 0:
        return math.floor(time / frequency_dt) != math.floor((time - dt) / frequency_dt)
    return frequency > 0 and step % frequency == 0


class ProbeOutput:
    """Time histories at the probe nodes (ProbeOutput.cpp:14-350, 599-848): one
    file per requested field, named prefix + file name, one line per output:
    the step, the time and the field at every node.  `write` takes the
    ghosted state (Solver.get_state_ghosted, OracleSim.download_ghosted) or,
    with `solver=`, samples the nodes on the device (Solver.sample_points)."""

    def __init__(self, case, prefix=None):
        p = case.probes or {"frequency": -100, "frequency_dt": -1.0, "files": {}, "nodes": []}
        self.cfg = case.cfg
        self.frequency, self.frequency_dt = p["frequency"], p["frequency_dt"]
        self.nodes = [tuple(n) for n in p["nodes"]]
        self.setup = locate_points(self.cfg, self.nodes) if self.nodes else []
        self.last = -1.0
        pre = case.prefix if prefix is None else prefix
        self.files = {k: open(pre + name, "w") for k, name in p["files"].items()}

    def due(self, time, dt, step, force=False):
        return bool(self.nodes) and is_time_to_write(time, dt, step, self.frequency_dt, self.frequency,
                                                     self.last, force)

    def write(self, time, dt, step, Vg=None, IDg=None, phig=None, force=False, solver=None):
        """Appends a line to every file when the frequency says so; returns
        whether it wrote."""
        if not self.due(time, dt, step, force):
            return False
        if solver is not None:
            vals = solver.sample_points(self.nodes)
        else:
            fields = [Vg[q] for q in range(5)] + [np.asarray(IDg, np.float64)]
            if phig is not None and self.cfg.n_levelsets:
                fields.append(phig)
            vals = interpolate_points(self.cfg, self.setup, fields)
        for key, f in self.files.items():
            col = _PROBE_FIELDS[key]
            if col >= vals.shape[1]:   # LevelSet<n> beyond the level sets: file stays empty
                continue
            f.write(("%10d    %16.8e    " if key == "Density" else "%8d    %16.8e    ") % (step, time))
            for v in vals[:, col]:
                f.write("%16.8e    " % v)
            f.write("\n")
            f.flush()
        self.last = time
        return True

    def close(self):
        for f in self.files.values():
            f.close()


class MaterialVolumeOutput:
    """The volume of every material and of the ghost / inactive ID (none on
    this path: 0) with their sum, one line per output
    (MaterialVolumeOutput.cpp:11-85).  `write` takes any object with
    `integrate(box)`."""

    def __init__(self, case, prefix=None):
        mv = case.material_volumes or {"file": "", "frequency": 10, "frequency_dt": -1.0}
        self.frequency, self.frequency_dt = mv["frequency"], mv["frequency_dt"]
        self.last = -1.0
        self.f = None
        if mv["file"]:
            c = case.cfg
            pre = case.prefix if prefix is None else prefix
            self.f = open(pre + mv["file"], "w")
            n = c.n_materials + 1
            self.f.write("## Number of physical materials: %d (0 - %d); ID for ghost/inactive cells: %d.\n"
                         % (n - 1, n - 2, n - 1))
            self.f.write("## Total volume of computational domain: %e.\n"
                         % ((c.xmax - c.x0) * (c.ymax - c.y0) * (c.zmax - c.z0)))
            self.f.write("## The last column is the sum over all material subdomains (including ghost/inactive).\n")
            self.f.flush()

    def write(self, time, dt, step, sim, force=False):
        if self.f is None or not is_time_to_write(time, dt, step, self.frequency_dt, self.frequency, self.last, force):
            return False
        vol = list(sim.integrate(None)[:, 0]) + [0.0]
        self.f.write("%8d  %16.8e  " % (step, time))
        total = 0.0
        for v in vol:
            self.f.write("%16.8e  " % v)
            total += v
        self.f.write("%16.8e\n" % total)
        self.f.flush()
        self.last = time
        return True

    def close(self):
        if self.f is not None:
            self.f.close()


class EnergyIntegrationOutput:
    """Per-material integrals in the box of `Output.EnergyIntegration`
    (EnergyIntegrationOutput.cpp:126-245): one file per quantity, one line per
    output: the step, the time, the value of every material and their sum.
    `write` takes any object with `integrate(box)` (Solver: on the device;
    OracleSim: the CPU restatement)."""

    def __init__(self, case, prefix=None):
        e = case.energy_integration or {"frequency": -100, "frequency_dt": -1.0, "files": {}, "box": None}
        self.frequency, self.frequency_dt, self.box = e["frequency"], e["frequency_dt"], e["box"]
        self.last = -1.0
        pre = case.prefix if prefix is None else prefix
        self.files = {k: open(pre + name, "w") for k, name in e["files"].items()}

    def write(self, time, dt, step, sim, force=False):
        if not is_time_to_write(time, dt, step, self.frequency_dt, self.frequency, self.last, force):
            return False
        if self.files:
            vals = sim.integrate(self.box)
            for key, f in self.files.items():
                col = _INTEGRALS[key]
                f.write("%10d    %16.8e    " % (step, time))
                total = 0.0
                for v in vals[:, col]:
                    f.write("%16.8e  " % v)
                    total += v
                f.write("%16.8e\n" % total)
                f.flush()
        self.last = time
        return True

    def close(self):
        for f in self.files.values():
            f.close()


def write_line(path, plot, rows, time, step):
    """A line-plot file in the reference's layout (ProbeOutput.cpp:520-574)."""
    npts = plot["NumberOfPoints"]
    x0, x1 = plot["x0"], plot["x1"]
    d = [(b - a) / (npts - 1) for a, b in zip(x0, x1)]
    h = math.sqrt(sum(v * v for v in d))
    with open(path, "w") as f:
        f.write("## Line: (%e, %e, %e) -> (%e, %e, %e)\n" % (*x0, *x1))
        f.write("## Number of points: %d (h = %e)\n" % (npts, h))
        f.write("## Time: %e, Time step: %d.\n" % (time, step))
        f.write("## Coordinate  |  Density  |  Velocity (Vx,Vy,Vz)  |  Pressure  |  Temperature  |  Material ID  "
                "|  LevelSet(s)\n")
        for r in rows:
            f.write("%16.8e  %16.8e  %16.8e  %16.8e  %16.8e  %16.8e  %16.8e  %16.8e" % tuple(r[:8]))
            for v in r[8:]:
                f.write("%16.8e  " % v)
            f.write("\n")
