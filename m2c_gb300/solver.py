"""Host-side mirror of the reference's operator interface for the
finite-volume step, over the C ABI of libm2cg.so.

`FluidState` is the triple {V, ID, Phi} the reference's operators act on
(Main.cpp:283-327).  `Solver` exposes the reference's method names:
ComputeTimeStepSize (SpaceOperator.cpp:1298), ComputeResidual
(SpaceOperator.cpp:2573), LevelSetResidual (LevelSetOperator.cpp:768),
AdvanceOneTimeStep (TimeIntegrator.cpp:319/527) and the Main.cpp:653-771 loop
as run().  Everything executes on the GPU; there is no CPU fallback.
"""
import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import abi


@dataclass
class FluidState:
    V: np.ndarray      # (N, 5) primitive state rho, u, v, w, p, real cells k-major
    ID: np.ndarray     # (N,) int32 material IDs
    Phi: np.ndarray    # (N,) level set (negative inside the tracked material)


class Solver:
    def __init__(self, cfg, state=None, lib=None):
        self.lib = lib or abi.load()
        self.cfg = cfg
        self.n = cfg.nx * cfg.ny * cfg.nz
        h = C.c_void_p()
        abi.check(self.lib, self.lib.m2cg_create(C.byref(cfg), C.byref(h)), "m2cg_create")
        self.ctx = h
        if state is not None:
            self.set_state(state)

    @classmethod
    def member(cls, lib, cfg, ctx):
        """A view of a context owned elsewhere (an ensemble member): not destroyed by close()."""
        s = cls.__new__(cls)
        s.lib, s.cfg, s.n, s.ctx, s._owned = lib, cfg, cfg.nx * cfg.ny * cfg.nz, ctx, False
        return s

    def close(self):
        if getattr(self, "ctx", None):
            if getattr(self, "_owned", True):
                self.lib.m2cg_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        self.close()

    def set_state(self, s):
        V = np.ascontiguousarray(s.V, np.float64)
        ID = np.ascontiguousarray(s.ID, np.int32)
        Phi = None if s.Phi is None else np.ascontiguousarray(s.Phi, np.float64)
        assert V.shape == (self.n, 5) and ID.shape == (self.n,)
        abi.check(self.lib, self.lib.m2cg_upload_state(self.ctx, abi.dptr(V), abi.iptr(ID), abi.dptr(Phi)),
                  "m2cg_upload_state")

    def get_state(self):
        V = np.zeros((self.n, 5))
        ID = np.zeros(self.n, np.int32)
        Phi = np.zeros(self.n)
        abi.check(self.lib, self.lib.m2cg_download_state(self.ctx, abi.dptr(V), abi.iptr(ID), abi.dptr(Phi)),
                  "m2cg_download_state")
        return FluidState(V, ID, Phi)

    def get_state_ghosted(self):
        """(V planes 5 x N, ID, phi) with the ghost layer after the boundary
        conditions, N = (nx+2)(ny+2)(nz+2), i fastest (the probes' input)."""
        n = (self.cfg.nx + 2) * (self.cfg.ny + 2) * (self.cfg.nz + 2)
        V = np.zeros(5 * n)
        ID = np.zeros(n, np.int32)
        Phi = np.zeros(n)
        abi.check(self.lib, self.lib.m2cg_download_ghosted(self.ctx, abi.dptr(V), abi.iptr(ID), abi.dptr(Phi)),
                  "m2cg_download_ghosted")
        return V.reshape(5, n), ID, Phi

    def sample_points(self, points):
        """The solution at probe points (ProbeOutput.cpp:360-480, 849-886), on
        the device: rows of rho, vx, vy, vz, p, material ID, phi."""
        pts = np.ascontiguousarray(np.asarray(points, np.float64).reshape(-1, 3))
        nf = 6 + (1 if self.cfg.n_levelsets else 0)
        out = np.zeros((len(pts), nf))
        abi.check(self.lib, self.lib.m2cg_sample_points(self.ctx, len(pts), abi.dptr(pts), abi.dptr(out)),
                  "m2cg_sample_points")
        return out

    def integrate(self, box=None):
        """EnergyIntegrationOutput's per-material integrals on the device: rows
        per material of (volume, mass, total energy, total enthalpy, kinetic,
        internal) over the cells whose centres lie in box = (xmin, xmax, ymin,
        ymax, zmin, zmax), or everywhere."""
        out = np.zeros((self.cfg.n_materials, 6))
        b = None if box is None else np.ascontiguousarray(box, np.float64)
        abi.check(self.lib, self.lib.m2cg_integrate(self.ctx, abi.dptr(b), abi.dptr(out)), "m2cg_integrate")
        return out

    def run_to_end(self, max_time, max_its, chunk=64):
        """The Main.cpp:653-771 loop to MaxTime or MaxIts, whichever comes
        first, in chunks of graph-replayed steps; returns the counters."""
        c = self.counters()
        while c["steps"] < max_its and c["time"] < max_time * (1.0 - 1e-12):
            n = int(min(chunk, max_its - c["steps"]))
            before = c["steps"]
            c = self.run(n)
            if c["steps"] == before:   # MaxTime reached inside the chunk
                break
        return c

    def ComputeTimeStepSize(self):
        dt, cfl = C.c_double(), C.c_double()
        abi.check(self.lib, self.lib.m2cg_compute_dt(self.ctx, C.byref(dt), C.byref(cfl)), "m2cg_compute_dt")
        return dt.value, cfl.value

    def ComputeResidual(self):
        R = np.zeros((self.n, 5))
        abi.check(self.lib, self.lib.m2cg_compute_residual(self.ctx, abi.dptr(R)), "m2cg_compute_residual")
        return R

    def RiemannSolutions(self, cap=None):
        """The interface Riemann solutions of the last ComputeResidual (what the
        reference's RiemannSolutions argument receives): dict of ijkd (n x 4:
        plus cell i, j, k and direction), Vsm, Vsp (n x 5) and ids (n x 2)."""
        n = C.c_int64()
        abi.check(self.lib, self.lib.m2cg_riemann_solutions(self.ctx, 0, None, None, None, None, C.byref(n)),
                  "m2cg_riemann_solutions")
        m = n.value if cap is None else min(cap, n.value)
        ijkd = np.zeros((m, 4), np.int32)
        vsm, vsp = np.zeros((m, 5)), np.zeros((m, 5))
        ids = np.zeros((m, 2), np.int32)
        abi.check(self.lib, self.lib.m2cg_riemann_solutions(self.ctx, m, abi.iptr(ijkd), abi.dptr(vsm), abi.dptr(vsp),
                                                            abi.iptr(ids), C.byref(n)), "m2cg_riemann_solutions")
        return dict(ijkd=ijkd, Vsm=vsm, Vsp=vsp, ids=ids)

    def LevelSetResidual(self):
        R = np.zeros(self.n)
        abi.check(self.lib, self.lib.m2cg_levelset_residual(self.ctx, abi.dptr(R)), "m2cg_levelset_residual")
        return R

    def AdvanceOneTimeStep(self, dt):
        abi.check(self.lib, self.lib.m2cg_advance(self.ctx, float(dt)), "m2cg_advance")

    def run(self, nsteps):
        c = abi.Counters()
        abi.check(self.lib, self.lib.m2cg_run(self.ctx, int(nsteps), C.byref(c)), "m2cg_run")
        return c.as_dict()

    def counters(self):
        c = abi.Counters()
        abi.check(self.lib, self.lib.m2cg_get_counters(self.ctx, C.byref(c)), "m2cg_get_counters")
        return c.as_dict()

    def Reinitialize(self):
        """LevelSetOperator::Reinitialize with must_do (LevelSetOperator.cpp:1338-1361):
        one full-domain reinitialization now, first layer FIXED; returns the
        context's reinitialization totals."""
        st = abi.ReinitStats()
        abi.check(self.lib, self.lib.m2cg_reinitialize(self.ctx, C.byref(st)), "m2cg_reinitialize")
        return st.as_dict()

    def reinit_stats(self):
        st = abi.ReinitStats()
        abi.check(self.lib, self.lib.m2cg_get_reinit_stats(self.ctx, C.byref(st)), "m2cg_get_reinit_stats")
        return st.as_dict()

    def conserved_totals(self):
        t = np.zeros(5)
        abi.check(self.lib, self.lib.m2cg_conserved_totals(self.ctx, abi.dptr(t)), "m2cg_conserved_totals")
        return t

    def set_warm_start(self, net):
        """Warm-start the interface solves with a WarmStartMLP (None: cold start)."""
        abi.check(self.lib, self.lib.m2cg_set_warm_start(self.ctx, net.h if net is not None else None),
                  "m2cg_set_warm_start")
        self._warm_net = net  # the network must outlive its use by the context

    def riemann_batch(self, Vm, idm, Vp, idp, dirs):
        n = len(idm)
        Vs, Vsm, Vsp = np.zeros((n, 5)), np.zeros((n, 5)), np.zeros((n, 5))
        oid, it, err = np.zeros(n, np.int32), np.zeros(n, np.int32), np.zeros(n, np.int32)
        abi.check(self.lib, self.lib.m2cg_riemann_batch(
            self.ctx, n, abi.dptr(np.ascontiguousarray(Vm, np.float64)), abi.iptr(np.ascontiguousarray(idm, np.int32)),
            abi.dptr(np.ascontiguousarray(Vp, np.float64)), abi.iptr(np.ascontiguousarray(idp, np.int32)),
            abi.dptr(np.ascontiguousarray(dirs, np.float64)), abi.dptr(Vs), abi.iptr(oid), abi.dptr(Vsm),
            abi.dptr(Vsp), abi.iptr(it), abi.iptr(err)), "m2cg_riemann_batch")
        return dict(Vs=Vs, id=oid, Vsm=Vsm, Vsp=Vsp, iters=it, err=err)

    def flux_batch(self, dirs, Vm, Vp, ids):
        n = len(ids)
        F = np.zeros((n, 5))
        abi.check(self.lib, self.lib.m2cg_flux_batch(
            self.ctx, n, abi.iptr(np.ascontiguousarray(dirs, np.int32)), abi.dptr(np.ascontiguousarray(Vm, np.float64)),
            abi.dptr(np.ascontiguousarray(Vp, np.float64)), abi.iptr(np.ascontiguousarray(ids, np.int32)),
            abi.dptr(F)), "m2cg_flux_batch")
        return F
