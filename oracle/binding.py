"""ctypes binding of the oracle (liboracle.so) and of the reference build
(oracle/_ref/libm2cref.so).  Test infrastructure only."""
import ctypes as C
import os

import numpy as np

from m2c_gb300.abi import Config, Counters, dptr, iptr

HERE = os.path.dirname(os.path.abspath(__file__))
_P = C.c_void_p
_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int32)


def _load_oracle(fma=False):
    from oracle import build as ob
    lib = C.CDLL(ob.build(fma=fma))
    sig = {
        "orc_create": (_P, [C.POINTER(Config)]),
        "orc_destroy": (None, [_P]),
        "orc_set_threads": (None, [C.c_int]),
        "orc_max_threads": (C.c_int, []),
        "orc_upload": (None, [_P, _D, _I, _D]),
        "orc_download": (None, [_P, _D, _I, _D]),
        "orc_residual": (None, [_P, _D]),
        "orc_levelset_residual": (None, [_P, _D]),
        "orc_compute_dt": (None, [_P, _D, _D]),
        "orc_reinitialize": (C.c_int, [_P, _D]),
        "orc_download_ghosted": (None, [_P, _D, _I, _D]),
        "orc_advance": (None, [_P, C.c_double]),
        "orc_run": (C.c_int, [_P, C.c_int]),
        "orc_counters": (None, [_P, C.POINTER(Counters)]),
        "orc_conserved_totals": (None, [_P, _D]),
        "orc_integrate": (None, [_P, _D, _D]),
        "orc_riemann_normal": (None, [_P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _D]),
        "orc_riemann_batch": (None, [C.POINTER(Config), C.c_int64, _D, _I, _D, _I, _D, _D, _I, _D, _D, _I, _I, _D]),
        "orc_flux_batch": (None, [C.POINTER(Config), C.c_int64, _I, _D, _D, _I, _D]),
    }
    for k, (r, a) in sig.items():
        f = getattr(lib, k)
        f.restype, f.argtypes = r, a
    return lib


_orc = {}


def lib(fma=False):
    """The oracle library; fma=True: the same source compiled with fused
    multiply-add contraction (the reference's rounding under a contracting
    compiler)."""
    if fma not in _orc:
        _orc[fma] = _load_oracle(fma)
    return _orc[fma]


def ref_lib():
    """The reference's own classes compiled from its sources, or None when the
    reference tree is not available (e.g. on the GPU machine)."""
    from oracle import build_ref
    p = build_ref.build()
    if p is None:
        return None
    r = C.CDLL(p)
    r.ref_riemann_batch.restype = None
    r.ref_riemann_batch.argtypes = [C.POINTER(Config), C.c_int64, _D, _I, _D, _I, _D, _D, _I, _D, _D, _I]
    r.ref_flux_batch.restype = None
    r.ref_flux_batch.argtypes = [C.POINTER(Config), C.c_int64, _I, _D, _D, _I, _D]
    return r


class OracleSim:
    """The oracle's finite-volume state, mirroring the product context."""

    def __init__(self, cfg, fma=False):
        self.cfg = cfg
        self.n = cfg.nx * cfg.ny * cfg.nz
        self.L = lib(fma)
        self.h = self.L.orc_create(C.byref(cfg))

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_destroy(self.h)
            self.h = None

    def upload(self, V, ID, phi=None):
        V = np.ascontiguousarray(V, np.float64)
        ID = np.ascontiguousarray(ID, np.int32)
        phi = None if phi is None else np.ascontiguousarray(phi, np.float64)
        self.L.orc_upload(self.h, dptr(V), iptr(ID), dptr(phi))

    def download(self):
        V = np.zeros((self.n, 5))
        ID = np.zeros(self.n, np.int32)
        phi = np.zeros(self.n)
        self.L.orc_download(self.h, dptr(V), iptr(ID), dptr(phi))
        return V, ID, phi

    def residual(self):
        R = np.zeros((self.n, 5))
        self.L.orc_residual(self.h, dptr(R))
        return R

    def levelset_residual(self):
        R = np.zeros(self.n)
        self.L.orc_levelset_residual(self.h, dptr(R))
        return R

    def integrate(self, box=None):
        """Per-material (volume, mass, total energy, total enthalpy, kinetic,
        internal) over the cells whose centres lie in box (xmin, xmax, ymin,
        ymax, zmin, zmax)."""
        out = np.zeros((self.cfg.n_materials, 6))
        b = None if box is None else np.ascontiguousarray(box, np.float64)
        self.L.orc_integrate(self.h, dptr(b), dptr(out))
        return out

    def riemann_normal(self, d, i, j, k, myid, nid):
        out = np.zeros(3)
        self.L.orc_riemann_normal(self.h, d, i, j, k, myid, nid, dptr(out))
        return out

    def download_ghosted(self):
        """(V planes 5 x N, ID, phi) with the ghost layer, N = (nx+2)(ny+2)(nz+2), i fastest."""
        n = (self.cfg.nx + 2) * (self.cfg.ny + 2) * (self.cfg.nz + 2)
        V = np.zeros(5 * n)
        ID = np.zeros(n, np.int32)
        phi = np.zeros(n)
        self.L.orc_download_ghosted(self.h, dptr(V), iptr(ID), dptr(phi))
        return V.reshape(5, n), ID, phi

    def reinitialize(self):
        """One full-domain reinitialization; returns (found_interface, stats dict)."""
        st = np.zeros(5)
        r = self.L.orc_reinitialize(self.h, dptr(st))
        return bool(r), dict(calls=int(st[0]), iterations=int(st[1]), retries=int(st[2]), failures=int(st[3]),
                             cfl=float(st[4]))

    def compute_dt(self):
        dt, cfl = C.c_double(), C.c_double()
        self.L.orc_compute_dt(self.h, C.byref(dt), C.byref(cfl))
        return dt.value, cfl.value

    def advance(self, dt):
        self.L.orc_advance(self.h, dt)

    def run(self, nsteps):
        return self.L.orc_run(self.h, nsteps)

    def counters(self):
        c = Counters()
        self.L.orc_counters(self.h, C.byref(c))
        return c.as_dict()

    def conserved_totals(self):
        t = np.zeros(5)
        self.L.orc_conserved_totals(self.h, dptr(t))
        return t


def riemann_batch(cfg, Vm, idm, Vp, idp, dirs, warm_p=None, fma=False):
    n = len(idm)
    Vm = np.ascontiguousarray(Vm, np.float64); Vp = np.ascontiguousarray(Vp, np.float64)
    idm = np.ascontiguousarray(idm, np.int32); idp = np.ascontiguousarray(idp, np.int32)
    dirs = np.ascontiguousarray(dirs, np.float64)
    Vs, Vsm, Vsp = np.zeros((n, 5)), np.zeros((n, 5)), np.zeros((n, 5))
    oid, it, err = np.zeros(n, np.int32), np.zeros(n, np.int32), np.zeros(n, np.int32)
    w = None if warm_p is None else np.ascontiguousarray(warm_p, np.float64)
    lib(fma).orc_riemann_batch(C.byref(cfg), n, dptr(Vm), iptr(idm), dptr(Vp), iptr(idp), dptr(dirs), dptr(Vs), iptr(oid),
                            dptr(Vsm), dptr(Vsp), iptr(it), iptr(err), dptr(w))
    return dict(Vs=Vs, id=oid, Vsm=Vsm, Vsp=Vsp, iters=it, err=err)


def flux_batch(cfg, dirs, Vm, Vp, ids):
    n = len(ids)
    F = np.zeros((n, 5))
    lib().orc_flux_batch(C.byref(cfg), n, iptr(np.ascontiguousarray(dirs, np.int32)),
                         dptr(np.ascontiguousarray(Vm, np.float64)), dptr(np.ascontiguousarray(Vp, np.float64)),
                         iptr(np.ascontiguousarray(ids, np.int32)), dptr(F))
    return F


def ref_riemann_batch(rl, cfg, Vm, idm, Vp, idp, dirs):
    n = len(idm)
    Vs, Vsm, Vsp = np.zeros((n, 5)), np.zeros((n, 5)), np.zeros((n, 5))
    oid, err = np.zeros(n, np.int32), np.zeros(n, np.int32)
    rl.ref_riemann_batch(C.byref(cfg), n, dptr(np.ascontiguousarray(Vm, np.float64)),
                         iptr(np.ascontiguousarray(idm, np.int32)), dptr(np.ascontiguousarray(Vp, np.float64)),
                         iptr(np.ascontiguousarray(idp, np.int32)), dptr(np.ascontiguousarray(dirs, np.float64)),
                         dptr(Vs), iptr(oid), dptr(Vsm), dptr(Vsp), iptr(err))
    return dict(Vs=Vs, id=oid, Vsm=Vsm, Vsp=Vsp, err=err)


def ref_flux_batch(rl, cfg, dirs, Vm, Vp, ids):
    n = len(ids)
    F = np.zeros((n, 5))
    rl.ref_flux_batch(C.byref(cfg), n, iptr(np.ascontiguousarray(dirs, np.int32)),
                      dptr(np.ascontiguousarray(Vm, np.float64)), dptr(np.ascontiguousarray(Vp, np.float64)),
                      iptr(np.ascontiguousarray(ids, np.int32)), dptr(F))
    return F
