"""Probe time histories (ProbeOutput.cpp:14-350, 360-480, 599-886; IoData.cpp:
3152-3230; Utils.cpp:337-357): parsing of Output.Probes, the write schedule,
the file layout, the interpolation (exact on fields linear in x, y, z, and
the same numbers as the line-plot sampler), and the device sampler against
the host one on the same ghosted state."""
import numpy as np
import pytest

from m2c_gb300 import inputfile as inf

CASE = """
under Mesh { X0 = 0.0; Xmax = 1.0; Y0 = 0.0; Ymax = 0.5; Z0 = 0.0; Zmax = 0.25;
  NumberOfCellsX = 16; NumberOfCellsY = 8; NumberOfCellsZ = 4;
  BoundaryConditionX0 = Inlet; BoundaryConditionXmax = Outlet; BoundaryConditionY0 = Symmetry;
  BoundaryConditionYmax = Symmetry; BoundaryConditionZ0 = Symmetry; BoundaryConditionZmax = Symmetry; }
under Equations {
  under Material[0] { EquationOfState = StiffenedGas; under StiffenedGasModel { SpecificHeatRatio = 6.12;
                                                                               PressureConstant = 3.43e8; } }
  under Material[1] { EquationOfState = StiffenedGas; under StiffenedGasModel { SpecificHeatRatio = 1.4; } }
}
under InitialCondition { under GeometricEntities {
  under Sphere[0] { Center_x = 0.4; Center_y = 0.25; Center_z = 0.125; Radius = 0.12;
                    under InitialState { MaterialID = 1; Density = 1.2; Pressure = 1.0e5; } } } }
under BoundaryConditions { under Inlet { Density = 1050.0; Pressure = 5.0e7; VelocityX = 20.0; } }
under Space { under NavierStokes { Flux = HLLC; under Reconstruction { Type = Linear; Limiter = VanAlbada; } }
  under LevelSet[0] { MaterialID = 1; } }
under ExactRiemannSolution { Tolerance = 1.0e-10; }
under Time { MaxTime = 1.0; CFL = 0.4; MaxIts = 6; under Explicit { Type = RungeKutta2; } }
under Output { Prefix = "out_";
  under Probes { Frequency = 2; Density = "rho.txt"; Pressure = "p.txt"; VelocityX = "vx.txt";
                 MaterialID = "id.txt"; LevelSet0 = "phi.txt"; LevelSet1 = "phi1.txt";
                 under Node[0] { X = 0.41; Y = 0.26; Z = 0.13; }
                 under Node[2] { X = 0.0; Y = 0.0; Z = 0.0; }
                 under Node[1] { X = 0.97; Y = 0.49; Z = 0.01; } } }
"""

NODES = [(0.41, 0.26, 0.13), (0.97, 0.49, 0.01), (0.0, 0.0, 0.0)]


def test_probes_are_parsed():
    cs = inf.Case.from_text(CASE)
    p = cs.probes
    assert cs.prefix == "out_"
    assert p["frequency"] == 2 and p["frequency_dt"] == -1.0
    assert p["nodes"] == NODES
    assert p["files"] == {"Density": "rho.txt", "Pressure": "p.txt", "VelocityX": "vx.txt", "MaterialID": "id.txt",
                          "LevelSet0": "phi.txt", "LevelSet1": "phi1.txt"}


@pytest.mark.parametrize("bad", ["Temperature = \"t.txt\";", "under Node[5] { X = 0.5; }"])
def test_probe_inputs_outside_the_path_are_refused(bad):
    text = CASE.replace("Frequency = 2;", "Frequency = 2; " + bad)
    with pytest.raises((NotImplementedError, ValueError)):
        inf.Case.from_text(text)


def test_write_schedule():
    """Utils.cpp:337-357: forced writes skip a time already written; the time
    interval wins over the step count."""
    w = inf.is_time_to_write
    assert w(1.0, 0.1, 4, -1.0, 2, -1.0, False) and not w(1.0, 0.1, 3, -1.0, 2, -1.0, False)
    assert not w(1.0, 0.1, 3, -1.0, -100, -1.0, False)
    assert w(1.0, 0.1, 3, -1.0, -100, 0.5, True) and not w(1.0, 0.1, 3, -1.0, -100, 1.0, True)
    assert w(0.31, 0.02, 1, 0.1, 2, -1.0, False) and not w(0.33, 0.02, 2, 0.1, 2, -1.0, False)


def test_interpolation_is_exact_on_linear_fields_and_agrees_with_the_line_sampler():
    cs = inf.Case.from_text(CASE)
    c = cs.cfg
    px, py, pz = c.nx + 2, c.ny + 2, c.nz + 2
    h = np.array([(c.xmax - c.x0) / c.nx, (c.ymax - c.y0) / c.ny, (c.zmax - c.z0) / c.nz])
    ii, jj, kk = np.meshgrid(np.arange(px), np.arange(py), np.arange(pz), indexing="ij")
    xg = (c.x0 + (ii - 0.5) * h[0]).transpose(2, 1, 0).ravel()
    yg = (c.y0 + (jj - 0.5) * h[1]).transpose(2, 1, 0).ravel()
    zg = (c.z0 + (kk - 0.5) * h[2]).transpose(2, 1, 0).ravel()
    f = 1.0 + 2.0 * xg - 3.0 * yg + 0.5 * zg
    inner = [(0.41, 0.26, 0.13), (0.2, 0.1, 0.2), (0.95, 0.45, 0.2)]
    vals = inf.interpolate_points(c, inf.locate_points(c, inner), [f])
    exact = [1.0 + 2.0 * x - 3.0 * y + 0.5 * z for x, y, z in inner]
    np.testing.assert_allclose(vals[:, 0], exact, rtol=1e-12)
    # a point in a corner of the domain: its lower corners are edge / corner ghosts
    setup = inf.locate_points(c, [(0.0, 0.0, 0.0)])
    assert sum(setup[0][2]) == 4
    # the same numbers as the line sampler at the same points
    plot = {"NumberOfPoints": 2, "x0": list(inner[0]), "x1": list(inner[2])}
    Vg = np.stack([f, 2 * f, f, f, 3 * f])
    rows = inf.sample_line(c, plot, Vg, np.zeros(f.size, np.int32), f)
    pv = inf.interpolate_points(c, inf.locate_points(c, [inner[0], inner[2]]), [Vg[0], Vg[1], Vg[4], f])
    np.testing.assert_array_equal(rows[:, [1, 2, 5, 8]], pv)


def _run_oracle_with_probes(tmp_path):
    from oracle import binding as ob
    cs = inf.Case.from_text(CASE)
    o = ob.OracleSim(cs.cfg)
    o.upload(cs.V, cs.ID, cs.phi)
    pr = inf.ProbeOutput(cs, prefix=str(tmp_path) + "/")
    assert pr.write(0.0, 0.0, 0, *o.download_ghosted(), force=True)
    history = []
    for _ in range(cs.max_its):
        o.run(1)
        cnt = o.counters()
        history.append(pr.write(cnt["time"], cnt["dt"], cnt["steps"], *o.download_ghosted()))
    cnt = o.counters()
    assert not pr.write(cnt["time"], cnt["dt"], cnt["steps"], *o.download_ghosted(), force=True)   # step 6 written
    pr.close()
    return cs, o, history


def test_probe_files_follow_the_reference_layout(tmp_path):
    cs, o, history = _run_oracle_with_probes(tmp_path)
    assert history == [False, True, False, True, False, True]
    rho = (tmp_path / "rho.txt").read_text().splitlines()
    p = (tmp_path / "p.txt").read_text().splitlines()
    assert len(rho) == 4 and len(p) == 4
    assert (tmp_path / "phi1.txt").read_text() == ""   # one level set: LevelSet1 stays empty
    # "%10d    %16.8e    " + nodes x "%16.8e    " for density, "%8d" for the others
    assert rho[1][:10] == "%10d" % 2 and p[1][:8] == "%8d" % 2
    assert len(rho[1]) == 10 + 4 + (16 + 4) * 4 and len(p[1]) == 8 + 4 + (16 + 4) * 4
    last = [float(v) for v in rho[-1].split()]
    assert last[0] == 6 and last[1] == pytest.approx(o.counters()["time"], rel=1e-8)
    # node 0 sits in the gas bubble, node 1 in water
    Vg, IDg, pg = o.download_ghosted()
    vals = inf.interpolate_points(cs.cfg, inf.locate_points(cs.cfg, NODES), [Vg[0], IDg.astype(float), pg])
    np.testing.assert_allclose(last[2:], vals[:, 0], rtol=1e-8)
    ids = [float(v) for v in (tmp_path / "id.txt").read_text().splitlines()[-1].split()[2:]]
    np.testing.assert_allclose(ids, vals[:, 1], rtol=1e-8)
    assert vals[0, 2] < 0 < vals[1, 2]


@pytest.mark.gpu
def test_gpu_sampler_matches_the_host_sampler(tmp_path):
    from m2c_gb300.solver import FluidState, Solver
    cs = inf.Case.from_text(CASE)
    s = Solver(cs.cfg, FluidState(cs.V, cs.ID, cs.phi))
    s.run(3)
    Vg, IDg, pg = s.get_state_ghosted()
    rng = np.random.default_rng(7)
    c = cs.cfg
    lo = np.array([c.x0, c.y0, c.z0]) - 0.5 * np.array([1 / 16, 0.5 / 8, 0.25 / 4])
    hi = np.array([c.xmax, c.ymax, c.zmax]) + 0.49 * np.array([1 / 16, 0.5 / 8, 0.25 / 4])
    pts = [tuple(lo + (hi - lo) * rng.random(3)) for _ in range(200)] + NODES
    host = inf.interpolate_points(c, inf.locate_points(c, pts), [Vg[q] for q in range(5)] +
                                  [IDg.astype(np.float64), pg])
    dev = s.sample_points(pts)
    np.testing.assert_array_equal(dev, host)
    with pytest.raises(RuntimeError):
        s.sample_points([(2.0, 0.1, 0.1)])
    # the probe writer on the device path writes the same lines as on the host path
    (tmp_path / "d").mkdir()
    (tmp_path / "h").mkdir()
    a = inf.ProbeOutput(cs, prefix=str(tmp_path / "d") + "/")
    b = inf.ProbeOutput(cs, prefix=str(tmp_path / "h") + "/")
    assert a.write(1.0, 0.1, 2, solver=s) and b.write(1.0, 0.1, 2, Vg, IDg, pg)
    a.close()
    b.close()
    for name in ("rho.txt", "p.txt", "vx.txt", "id.txt", "phi.txt"):
        assert (tmp_path / "d" / name).read_text() == (tmp_path / "h" / name).read_text()


# ---------------------------------------------------------------------------
# Per-material integrals (EnergyIntegrationOutput.cpp:126-610)

EI = """under Output { Prefix = "out_";
  under EnergyIntegration { Frequency = 3; Volume = "vol.txt"; Mass = "mass.txt"; TotalEnergy = "E.txt";
                            TotalEnthalpy = "H.txt"; KineticEnergy = "K.txt"; InternalEnergy = "IE.txt";
                            Xmin = 0.1; Xmax = 0.7; Zmax = 0.2; } }
"""


def _ei_case():
    return inf.Case.from_text(CASE.split("under Output")[0] + EI)


def _sg_integrals(cfg, V, ID, box):
    """The integrals restated in numpy for stiffened gases: e = (p + gamma pc) / ((gamma - 1) rho)."""
    from m2c_gb300.problems import cell_centers
    X, Y, Z = cell_centers(cfg)
    vol = (cfg.xmax - cfg.x0) / cfg.nx * (cfg.ymax - cfg.y0) / cfg.ny * (cfg.zmax - cfg.z0) / cfg.nz
    inb = (X >= box[0]) & (X <= box[1]) & (Y >= box[2]) & (Y <= box[3]) & (Z >= box[4]) & (Z <= box[5])
    g = np.array([cfg.mat[m].gamma for m in range(cfg.n_materials)])[ID]
    pc = np.array([cfg.mat[m].pc for m in range(cfg.n_materials)])[ID]
    rho, p = V[:, 0], V[:, 4]
    e = (p + g * pc) / ((g - 1.0) * rho)
    vsq = (V[:, 1:4] ** 2).sum(1)
    q = np.stack([np.ones_like(rho), rho, rho * (0.5 * vsq + e), rho * (0.5 * vsq + e) + p, 0.5 * rho * vsq,
                  rho * e], 1) * vol
    return np.stack([q[inb & (ID == m)].sum(0) for m in range(cfg.n_materials)])


def test_energy_integration_is_parsed_and_refuses_potential_energy():
    cs = _ei_case()
    ei = cs.energy_integration
    assert ei["frequency"] == 3 and ei["box"][:5] == [0.1, 0.7, -1.7976931348623157e308, 1.7976931348623157e308,
                                                      -1.7976931348623157e308] and ei["box"][5] == 0.2
    assert set(ei["files"]) == {"Volume", "Mass", "TotalEnergy", "TotalEnthalpy", "KineticEnergy", "InternalEnergy"}
    with pytest.raises(NotImplementedError):
        inf.Case.from_text(CASE.split("under Output")[0] + EI.replace("Frequency = 3;",
                                                                       "Frequency = 3; PotentialEnergy = \"u.txt\";"))


def test_oracle_integrals_and_file_layout(tmp_path):
    from oracle import binding as ob
    cs = _ei_case()
    o = ob.OracleSim(cs.cfg)
    o.upload(cs.V, cs.ID, cs.phi)
    box = cs.energy_integration["box"]
    np.testing.assert_allclose(o.integrate(box), _sg_integrals(cs.cfg, cs.V, cs.ID, box), rtol=1e-12)
    full = o.integrate()
    assert full[:, 0].sum() == pytest.approx(1.0 * 0.5 * 0.25, rel=1e-12)
    # cell centres (i + 1/2) / 16 in [0.1, 0.7]: i = 2..10; (k + 1/2) / 16 <= 0.2: k = 0..2
    assert o.integrate(box)[:, 0].sum() == pytest.approx(0.125 * 9 / 16 * 3 / 4, rel=1e-12)
    w = inf.EnergyIntegrationOutput(cs, prefix=str(tmp_path) + "/")
    wrote = []
    for _ in range(6):
        o.run(1)
        c = o.counters()
        wrote.append(w.write(c["time"], c["dt"], c["steps"], o))
    w.close()
    assert wrote == [False, False, True, False, False, True]
    lines = (tmp_path / "mass.txt").read_text().splitlines()
    assert len(lines) == 2
    # "%10d    %16.8e    " + materials x "%16.8e  " + "%16.8e\n" (the sum)
    assert len(lines[1]) == 10 + 4 + 16 + 4 + (16 + 2) * 2 + 16
    vals = [float(v) for v in lines[1].split()]
    assert vals[0] == 6
    ref = o.integrate(box)
    np.testing.assert_allclose(vals[2:4], ref[:, 1], rtol=1e-8)
    assert vals[4] == pytest.approx(ref[:, 1].sum(), rel=1e-8)


@pytest.mark.gpu
def test_gpu_integrals_match_oracle():
    from m2c_gb300.solver import FluidState, Solver
    from oracle import binding as ob
    cs = _ei_case()
    s = Solver(cs.cfg, FluidState(cs.V, cs.ID, cs.phi))
    o = ob.OracleSim(cs.cfg)
    o.upload(cs.V, cs.ID, cs.phi)
    box = cs.energy_integration["box"]
    for b in (box, None):
        np.testing.assert_allclose(s.integrate(b), o.integrate(b), rtol=1e-12)   # same state: summation order only
    np.testing.assert_array_equal(s.integrate(box), s.integrate(box))   # fixed reduction order
    s.run(3)
    o.run(3)
    np.testing.assert_allclose(s.integrate(box), o.integrate(box), rtol=1e-9)


# ---------------------------------------------------------------------------
# The main loop with its outputs (Main.cpp:571-782)

RUN = """under Output { Prefix = "PREFIX"; Frequency = 3; Density = On; Pressure = On;
  under LinePlot[0] { FileName = "line"; NumberOfPoints = 9; Frequency = 2; X0 = 0.03; Xmax = 0.97;
                      Y0 = 0.25; Ymax = 0.25; Z0 = 0.1; Zmax = 0.1; }
  under Probes { Frequency = 2; Pressure = "p.txt"; under Node[0] { X = 0.41; Y = 0.26; Z = 0.13; } }
  under EnergyIntegration { Frequency = 3; Mass = "mass.txt"; }
  under MaterialVolumes { FileName = "volumes.txt"; Frequency = 2; } }
"""


class _OracleRun:
    """The oracle behind the Solver's stepping and output methods."""

    def __init__(self, cs):
        from oracle import binding as ob
        self.o = ob.OracleSim(cs.cfg)
        self.o.upload(cs.V, cs.ID, cs.phi)

    def run(self, n):
        self.o.run(n)
        return self.o.counters()

    def counters(self):
        return self.o.counters()

    def get_state(self):
        from m2c_gb300.solver import FluidState
        return FluidState(*self.o.download())

    def get_state_ghosted(self):
        return self.o.download_ghosted()

    def integrate(self, box=None):
        return self.o.integrate(box)


def _run_case(sim_factory, tmp_path):
    from m2c_gb300 import driver
    cs = inf.Case.from_text(CASE.split("under Output")[0] + RUN.replace("PREFIX", str(tmp_path) + "/r_"))
    sim = sim_factory(cs)
    return driver.run_case(cs, sim), sim


def test_run_case_writes_every_output_on_its_schedule(tmp_path):
    (c, written), sim = _run_case(_OracleRun, tmp_path)
    assert c["steps"] == 6
    # snapshots: 0 (initial), 3, 6; lines and probes: 0, 2, 4, 6; energy: 0, 3, 6
    assert written == {"snapshots": 3, "lines": 4, "probes": 4, "energy": 3, "volumes": 4}
    names = sorted(p.name for p in tmp_path.iterdir())
    assert names == ["r_line_0000.txt", "r_line_0001.txt", "r_line_0002.txt", "r_line_0003.txt", "r_mass.txt",
                     "r_p.txt", "r_solution.pvd", "r_solution_0000.vtr", "r_solution_0001.vtr",
                     "r_solution_0002.vtr", "r_volumes.txt"]
    vol = (tmp_path / "r_volumes.txt").read_text().splitlines()
    assert vol[0].startswith("## Number of physical materials: 2 (0 - 1); ID for ghost/inactive cells: 2.")
    rows = [[float(v) for v in l.split()] for l in vol[3:]]
    assert [int(r[0]) for r in rows] == [0, 2, 4, 6]
    for r in rows:   # step, time, material 0, material 1, ghost / inactive, sum = the domain's volume
        assert len(r) == 6 and r[4] == 0.0 and r[5] == pytest.approx(0.125, rel=1e-12) and r[3] > 0
    head = (tmp_path / "r_line_0003.txt").read_text().splitlines()
    assert head[2].startswith("## Time: ") and head[2].endswith("Time step: 6.")
    assert [int(l.split()[0]) for l in (tmp_path / "r_p.txt").read_text().splitlines()] == [0, 2, 4, 6]
    assert [int(l.split()[0]) for l in (tmp_path / "r_mass.txt").read_text().splitlines()] == [0, 3, 6]
    from m2c_gb300 import output
    snap = output.read_vtr(str(tmp_path / "r_solution_0002.vtr"))   # the final state
    np.testing.assert_array_equal(snap["density"], sim.get_state().V[:, 0])
    assert sorted(snap) == ["density", "pressure"]   # the fields switched On, as Output.cpp:268-330
    assert "<DataSet timestep" in (tmp_path / "r_solution.pvd").read_text()


@pytest.mark.gpu
def test_gpu_run_case_matches_oracle_outputs(tmp_path):
    from m2c_gb300.solver import FluidState, Solver
    (tmp_path / "o").mkdir()
    (tmp_path / "g").mkdir()
    (co, wo), _ = _run_case(_OracleRun, tmp_path / "o")
    (cg, wg), _ = _run_case(lambda cs: Solver(cs.cfg, FluidState(cs.V, cs.ID, cs.phi)), tmp_path / "g")
    assert wo == wg and co["steps"] == cg["steps"] == 6
    for name in ("r_line_0003.txt", "r_p.txt", "r_mass.txt"):
        a = np.loadtxt(tmp_path / "o" / name)
        b = np.loadtxt(tmp_path / "g" / name)
        np.testing.assert_allclose(b, a, rtol=1e-7, atol=1e-9 * np.abs(a).max())


def test_run_case_time_interval_outputs_step_one_at_a_time(tmp_path):
    """An output on a time interval is written after every step whose interval
    (t - dt, t] crosses a multiple of it (Utils.cpp:345-349), so the loop steps
    one at a time; the final forced write adds the last state unless it was
    just written."""
    from m2c_gb300 import driver
    text = CASE.split("under Output")[0] + RUN.replace("PREFIX", str(tmp_path) + "/t_")
    cs = inf.Case.from_text(text)
    sim = _OracleRun(cs)
    o2 = _OracleRun(cs)
    times = [0.0]
    for _ in range(cs.max_its):
        times.append(o2.run(1)["time"])
    interval = 2.5 * times[1]
    cs.probes["frequency"], cs.probes["frequency_dt"] = -100, interval
    c, written = driver.run_case(cs, sim, snapshots=False)
    t = np.array(times)
    crossing = [s for s in range(1, len(t)) if np.floor(t[s] / interval) != np.floor(t[s - 1] / interval)]
    steps = [int(l.split()[0]) for l in (tmp_path / "t_p.txt").read_text().splitlines()]
    expect = [0] + crossing + ([cs.max_its] if cs.max_its not in crossing else [])
    assert steps == expect and len(crossing) >= 1


def test_run_case_logs_the_reference_progress_line(tmp_path):
    from m2c_gb300 import driver
    cs = inf.Case.from_text(CASE.split("under Output")[0] + RUN.replace("PREFIX", str(tmp_path) + "/l_"))
    lines = []
    c, _ = driver.run_case(cs, _OracleRun(cs), snapshots=False, log=lines.append)
    assert len(lines) == c["steps"] == 6
    assert lines[0].startswith("Step 1: t = 0.000000e+00, dt = ") and ", cfl = 4.0000e-01. Computation time: " in lines[0]


def test_run_case_writes_the_reference_line_plot_of_test1(tmp_path):
    """The whole loop on the reference's Tests/RiemannProblems/Test1 input with
    the oracle: the final line plot is `line_0001.txt` (the initial state is
    frame 0), with the reference's header, and its columns match the
    reference's own final line plot (the committed golden columns)."""
    import json
    import os
    from m2c_gb300 import driver
    golden = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_lines.json")))["Test1"]
    cs = inf.Case.from_tree(golden["tree"])
    c, written = driver.run_case(cs, _OracleRun(cs), prefix=str(tmp_path) + "/", snapshots=False)
    assert c["steps"] == golden["step"] == 109 and written["lines"] == 2
    lines = (tmp_path / "line_0001.txt").read_text().splitlines()
    assert lines[0] == "## Line: (2.500000e-03, 0.000000e+00, 0.000000e+00) -> (9.975000e-01, 0.000000e+00, 0.000000e+00)"
    assert lines[1] == "## Number of points: 200 (h = 5.000000e-03)"
    assert lines[2] == "## Time: 2.000000e-01, Time step: 109."
    assert lines[3].startswith("## Coordinate  |  Density  |  Velocity (Vx,Vy,Vz)  |  Pressure  |  Temperature")
    rows = np.loadtxt(tmp_path / "line_0001.txt")
    for col, key in ((1, "rho"), (2, "vx"), (5, "p"), (8, "phi")):
        ref = np.asarray(golden[key])
        assert np.abs(rows[:, col] - ref).max() <= 1e-6 * np.abs(ref).max(), key
