"""The reference's main loop with its outputs (Main.cpp:571, 639-782;
Output.cpp:148-200): the initial state written, steps to MaxTime or MaxIts,
after every step each output written when its own frequency or time interval
says so (Utils.cpp:337-357), and a final forced write.

The outputs are the ones of `Output` in the input file: solution snapshots
(`<prefix><Solution>_NNNN.vtr` + `.pvd`), line plots (`<prefix><FileName>_NNNN.txt`,
ProbeOutput.cpp:483-597), probe histories, energy integrals and material volumes.  Steps run in
chunks of replayed step graphs up to the next step at which an output is due;
an output on a time interval makes every step its own chunk.

`sim` is a `Solver` (or any object with its `run`, `counters`, `get_state`,
`get_state_ghosted` and `integrate` methods; `sample_points` is used when
present).
"""
import os
import time as _time

from . import inputfile, output


class _LineSeries:
    def __init__(self, case, plot, prefix):
        self.case, self.plot, self.prefix = case, plot, prefix
        self.frame = 0
        self.last = -1.0

    def write(self, time, dt, step, ghosted, force):
        if self.plot["NumberOfPoints"] <= 0 or not inputfile.is_time_to_write(
                time, dt, step, self.plot["frequency_dt"], self.plot["frequency"], self.last, force):
            return False
        if not self.plot["FileName"]:
            return False
        rows = inputfile.sample_line(self.case.cfg, self.plot, *ghosted())
        inputfile.write_line("%s%s_%04d.txt" % (self.prefix, self.plot["FileName"], self.frame), self.plot, rows,
                             time, step)
        self.frame += 1
        self.last = time
        return True


def _due_steps(freq, step):
    """Steps to the next multiple of freq after step (None: never by step count)."""
    return None if freq <= 0 else freq - step % freq


def run_case(case, sim, prefix=None, snapshots=True, chunk=64, log=None):
    """Runs `case` on `sim` with the case's outputs; returns the final counters
    and the number of files written per kind.  With `log` (e.g. print) the
    steps run one at a time and each gets the reference's progress line
    (Main.cpp:699-701)."""
    start = _time.perf_counter()
    pre = case.prefix if prefix is None else prefix
    d = os.path.dirname(pre)
    if d:
        os.makedirs(d, exist_ok=True)
    sol = case.solution
    series = output.SolutionSeries(os.path.dirname(pre) + "/" if d else "", os.path.basename(pre) + sol["base"]) \
        if snapshots else None
    sol_last = [-1.0]
    lines = [_LineSeries(case, p, pre) for p in case.line_plots]
    probes = inputfile.ProbeOutput(case, prefix=pre)
    energy = inputfile.EnergyIntegrationOutput(case, prefix=pre)
    volumes = inputfile.MaterialVolumeOutput(case, prefix=pre)
    written = {"snapshots": 0, "lines": 0, "probes": 0, "energy": 0, "volumes": 0}
    cache = {}

    def ghosted():
        if "g" not in cache:
            cache["g"] = sim.get_state_ghosted()
        return cache["g"]

    def out(time, dt, step, force):
        cache.clear()
        if series is not None and inputfile.is_time_to_write(time, dt, step, sol["frequency_dt"], sol["frequency"],
                                                             sol_last[0], force):
            st = sim.get_state()
            series.write(case.cfg, st.V, st.ID, st.Phi, time, sol.get("fields"))
            sol_last[0] = time
            written["snapshots"] += 1
        for ln in lines:
            written["lines"] += ln.write(time, dt, step, ghosted, force)
        if probes.nodes and probes.due(time, dt, step, force):
            if hasattr(sim, "sample_points"):
                written["probes"] += probes.write(time, dt, step, solver=sim, force=force)
            else:
                written["probes"] += probes.write(time, dt, step, *ghosted(), force=force)
        written["energy"] += energy.write(time, dt, step, sim, force=force)
        written["volumes"] += volumes.write(time, dt, step, sim, force=force)

    c = sim.counters()
    out(c["time"], 0.0, c["steps"], True)                       # Main.cpp:571
    by_time = (sol["frequency_dt"] > 0 and series is not None) or any(p["frequency_dt"] > 0 for p in case.line_plots) \
        or probes.frequency_dt > 0 or energy.frequency_dt > 0 or (volumes.f is not None and volumes.frequency_dt > 0)
    freqs = ([sol["frequency"]] if series is not None else []) + [p["frequency"] for p in case.line_plots] + \
        [probes.frequency, energy.frequency] + ([volumes.frequency] if volumes.f is not None else [])
    while c["steps"] < case.max_its and c["time"] < case.max_time * (1.0 - 1e-12):
        n = 1 if (by_time or log is not None) else chunk
        for f in freqs:
            k = _due_steps(f, c["steps"])
            if k is not None:
                n = min(n, k)
        n = int(min(n, case.max_its - c["steps"]))
        before = c["steps"]
        c = sim.run(n)
        if c["steps"] == before:   # MaxTime reached
            break
        if log is not None:
            log("Step %d: t = %e, dt = %e, cfl = %.4e. Computation time: %.4e s."
                % (c["steps"], c["time"] - c["dt"], c["dt"], c["cfl"], _time.perf_counter() - start))
        out(c["time"], c["dt"], c["steps"], False)              # Main.cpp:769
    out(c["time"], c["dt"], c["steps"], True)                   # Main.cpp:782
    probes.close()
    energy.close()
    volumes.close()
    return c, written
