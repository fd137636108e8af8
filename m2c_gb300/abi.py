"""ctypes mirror of include/m2cg.h and the loader for the in-tree libm2cg.so.

The structs below follow the C header field for field; `load()` checks their
sizes against m2cg_config_size() / m2cg_counters_size() so a layout drift fails
loudly instead of passing garbage to the GPU.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libm2cg.so")

MAX_MATERIALS = 8

# enums (values follow the reference's IoData enums)
EOS_SG, EOS_NASG, EOS_MG = 0, 1, 2
BC_INLET, BC_INLET2, BC_SLIPWALL, BC_STICKWALL, BC_SYMMETRY, BC_OUTLET = 1, 2, 3, 4, 5, 7
LSBC_ZERO_NEUMANN, LSBC_LINEAR_EXTRAPOLATION, LSBC_NON_NEGATIVE = 1, 2, 3
FLUX_ROE, FLUX_LLF, FLUX_HLLC = 0, 1, 2
REC_CONSTANT, REC_LINEAR = 0, 1
LIM_NONE, LIM_GENERALIZED_MINMOD, LIM_VANALBADA = 0, 1, 2
SLOPE_ZERO, SLOPE_NONZERO = 0, 1
VAR_PRIMITIVE, VAR_CONSERVATIVE, VAR_PRIMITIVE_CHARACTERISTIC, VAR_CONSERVATIVE_CHARACTERISTIC = 0, 1, 2, 3
MPFLUX_EXACT, MPFLUX_NUMERICAL, MPFLUX_LLF = 0, 1, 2
MPREC_CONSTANT, MPREC_LINEAR = 0, 1
PHASECHANGE_RIEMANN, PHASECHANGE_EXTRAPOLATION = 0, 1
PCDIR_ALL, PCDIR_UPWIND = 0, 1
RNORMAL_LEVEL_SET, RNORMAL_MESH, RNORMAL_AVERAGE = 0, 1, 2
TS_FORWARD_EULER, TS_RK2, TS_RK3 = 0, 1, 2
LS_FINITE_VOLUME, LS_FINITE_DIFFERENCE = 0, 1
LSFLUX_ROE, LSFLUX_LLF, LSFLUX_UPWIND = 0, 1, 2

STATUS = {0: "OK", 1: "INVALID_ARG", 2: "CUDA", 3: "NONPHYSICAL", 4: "UNRESOLVED",
          5: "NO_DEVICE", 6: "CAPACITY"}


class Material(C.Structure):
    _fields_ = [("eos", C.c_int32), ("pad_", C.c_int32),
                ("gamma", C.c_double), ("pc", C.c_double), ("b", C.c_double), ("q", C.c_double),
                ("rho0", C.c_double), ("c0", C.c_double), ("Gamma0", C.c_double), ("s", C.c_double),
                ("e0", C.c_double),
                ("rhomin", C.c_double), ("pmin", C.c_double), ("rhomax", C.c_double), ("pmax", C.c_double),
                ("failsafe_density", C.c_double)]


class Config(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("pad0_", C.c_int32),
                ("x0", C.c_double), ("xmax", C.c_double), ("y0", C.c_double), ("ymax", C.c_double),
                ("z0", C.c_double), ("zmax", C.c_double),
                ("bc", C.c_int32 * 6),
                ("inlet", C.c_double * 5), ("inlet2", C.c_double * 5),
                ("n_materials", C.c_int32), ("pad1_", C.c_int32),
                ("mat", Material * MAX_MATERIALS),
                ("flux", C.c_int32), ("rec_type", C.c_int32), ("limiter", C.c_int32), ("rec_var", C.c_int32),
                ("slope_near_interface", C.c_int32), ("pad2_", C.c_int32),
                ("minmod_coeff", C.c_double), ("roe_delta", C.c_double),
                ("mp_flux", C.c_int32), ("mp_recon", C.c_int32), ("mp_phasechange", C.c_int32),
                ("mp_phasechange_dir", C.c_int32),
                ("maxits_main", C.c_int32), ("maxits_bracket", C.c_int32), ("maxits_shock", C.c_int32),
                ("numsteps_rarefaction", C.c_int32),
                ("tol_main", C.c_double), ("tol_shock", C.c_double), ("tol_rarefaction", C.c_double),
                ("min_pressure", C.c_double), ("failure_threshold", C.c_double),
                ("pressure_at_failure", C.c_double),
                ("n_levelsets", C.c_int32), ("ls_matid", C.c_int32), ("ls_bc", C.c_int32 * 6),
                ("ts_type", C.c_int32), ("max_its", C.c_int32),
                ("cfl", C.c_double), ("timestep", C.c_double), ("max_time", C.c_double),
                ("warm_start", C.c_int32), ("reinit_frequency", C.c_int32), ("reinit_max_its", C.c_int32),
                ("pad4_", C.c_int32), ("reinit_cfl", C.c_double), ("reinit_tol", C.c_double),
                ("ls_solver", C.c_int32), ("ls_flux", C.c_int32), ("ls_delta", C.c_double),
                ("ls_rec_type", C.c_int32), ("ls_limiter", C.c_int32), ("ls_minmod_coeff", C.c_double),
                ("reinit_frequency_dt", C.c_double), ("mp_riemann_normal", C.c_int32), ("pad5_", C.c_int32)]


class Counters(C.Structure):
    _fields_ = [("interface_faces", C.c_int64), ("riemann_errors", C.c_int64),
                ("riemann_iterations", C.c_int64), ("riemann_solves", C.c_int64),
                ("clipped_cells", C.c_int64), ("clipped_faces", C.c_int64), ("nonphysical", C.c_int64),
                ("swept_cells", C.c_int64), ("unresolved_cells", C.c_int64), ("steps", C.c_int64),
                ("time", C.c_double), ("dt", C.c_double), ("cfl", C.c_double),
                ("riemann_fallbacks", C.c_int64), ("path_capped", C.c_int64),
                ("unresolved_fixed", C.c_int64)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class ReinitStats(C.Structure):
    _fields_ = [("calls", C.c_int64), ("iterations", C.c_int64), ("retries", C.c_int64), ("failures", C.c_int64),
                ("loop_bodies", C.c_int64), ("cfl", C.c_double), ("last_residual", C.c_double),
                ("last_change", C.c_double)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


def default_config():
    """IoData defaults for the fields the hot path reads (IoData.cpp:1044-1055,
    1262-1272, 1368-1374, 1508-1530, 1618-1637, 1690-1710, 1838-1850)."""
    c = Config()
    c.nx = c.ny = c.nz = 1
    c.x0, c.xmax, c.y0, c.ymax, c.z0, c.zmax = 0.0, 1.0, 0.0, 1.0, 0.0, 1.0
    for s in range(6):
        c.bc[s] = BC_OUTLET
        c.ls_bc[s] = LSBC_ZERO_NEUMANN
    c.inlet[0] = c.inlet2[0] = 1.0e-6   # StateVariable's density (IoData.cpp:29-41)
    c.n_materials = 1
    for m in range(MAX_MATERIALS):
        set_material(c.mat[m], EOS_SG, gamma=1.4, pc=0.0)
    c.flux = FLUX_HLLC
    c.rec_type = REC_LINEAR
    c.limiter = LIM_GENERALIZED_MINMOD
    c.rec_var = 0
    c.slope_near_interface = SLOPE_NONZERO
    c.minmod_coeff = 1.2
    c.roe_delta = 0.2
    c.mp_flux = MPFLUX_NUMERICAL
    c.mp_recon = MPREC_CONSTANT
    c.mp_phasechange = PHASECHANGE_RIEMANN
    c.mp_phasechange_dir = PCDIR_UPWIND
    c.maxits_main, c.maxits_bracket, c.maxits_shock, c.numsteps_rarefaction = 200, 100, 200, 200
    c.tol_main, c.tol_shock, c.tol_rarefaction = 1.0e-5, 1.0e-12, 1.0e-8
    c.min_pressure, c.failure_threshold, c.pressure_at_failure = -1.0e8, 0.2, 1.0e-8
    c.n_levelsets = 0
    c.ls_matid = 1
    c.ts_type = TS_RK2
    c.max_its = 2 ** 31 - 1
    c.cfl = 0.5
    c.timestep = -1.0
    c.max_time = 1e10
    c.warm_start = 0
    c.reinit_frequency, c.reinit_max_its, c.reinit_cfl, c.reinit_tol = -1, 30, 0.8, 2.0e-4
    c.ls_solver, c.ls_flux, c.ls_delta = LS_FINITE_DIFFERENCE, LSFLUX_ROE, 0.2
    c.ls_rec_type, c.ls_limiter, c.ls_minmod_coeff = REC_LINEAR, LIM_GENERALIZED_MINMOD, 1.2
    c.reinit_frequency_dt = -1.0
    c.mp_riemann_normal = RNORMAL_MESH
    return c


def set_material(m, eos, gamma=1.4, pc=0.0, b=0.0, q=0.0, rho0=1.0, c0=1.0, Gamma0=1.0, s=1.0, e0=0.0):
    m.eos = eos
    m.gamma, m.pc, m.b, m.q = gamma, pc, b, q
    m.rho0, m.c0, m.Gamma0, m.s, m.e0 = rho0, c0, Gamma0, s, e0
    m.rhomin, m.pmin, m.rhomax, m.pmax = 0.0, -np.finfo(np.float64).max, np.finfo(np.float64).max, \
        np.finfo(np.float64).max
    m.failsafe_density = 1.0e-10


_P = C.c_void_p
_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int32)
_F = C.POINTER(C.c_float)


def dptr(a):
    return a.ctypes.data_as(_D) if a is not None else None


def iptr(a):
    return a.ctypes.data_as(_I) if a is not None else None


def fptr(a):
    return a.ctypes.data_as(_F) if a is not None else None


MLP_FEATURES = 16
MLP_PARAMS = 9473


_lib = None


def load(path=None):
    """Load libm2cg.so (built in-tree by m2c_gb300.build).  Raises if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"libm2cg.so not built at {p}; run python -c 'import __graft_entry__ as g; g.build()'")
    lib = C.CDLL(p)
    sig = {
        "m2cg_abi_version": (C.c_int32, []),
        "m2cg_config_size": (C.c_size_t, []),
        "m2cg_counters_size": (C.c_size_t, []),
        "m2cg_last_error": (C.c_char_p, []),
        "m2cg_config_default": (C.c_int, [C.POINTER(Config)]),
        "m2cg_create": (C.c_int, [C.POINTER(Config), C.POINTER(_P)]),
        "m2cg_destroy": (None, [_P]),
        "m2cg_upload_state": (C.c_int, [_P, _D, _I, _D]),
        "m2cg_download_state": (C.c_int, [_P, _D, _I, _D]),
        "m2cg_compute_dt": (C.c_int, [_P, _D, _D]),
        "m2cg_compute_residual": (C.c_int, [_P, _D]),
        "m2cg_riemann_solutions": (C.c_int, [_P, C.c_int64, _I, _D, _D, _I, C.POINTER(C.c_int64)]),
        "m2cg_levelset_residual": (C.c_int, [_P, _D]),
        "m2cg_advance": (C.c_int, [_P, C.c_double]),
        "m2cg_run": (C.c_int, [_P, C.c_int32, C.POINTER(Counters)]),
        "m2cg_get_counters": (C.c_int, [_P, C.POINTER(Counters)]),
        "m2cg_reinitialize": (C.c_int, [_P, C.POINTER(ReinitStats)]),
        "m2cg_fp64_peak": (C.c_int, [C.c_int32, _D, C.POINTER(C.c_float)]),
        "m2cg_selftest_quotient": (C.c_int, [C.c_int64, C.c_uint64, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
        "m2cg_download_ghosted": (C.c_int, [_P, _D, _I, _D]),
        "m2cg_sample_points": (C.c_int, [_P, C.c_int32, _D, _D]),
        "m2cg_integrate": (C.c_int, [_P, _D, _D]),
        "m2cg_get_reinit_stats": (C.c_int, [_P, C.POINTER(ReinitStats)]),
        "m2cg_conserved_totals": (C.c_int, [_P, _D]),
        "m2cg_riemann_batch": (C.c_int, [_P, C.c_int64, _D, _I, _D, _I, _D, _D, _I, _D, _D, _I, _I]),
        "m2cg_flux_batch": (C.c_int, [_P, C.c_int64, _I, _D, _D, _I, _D]),
        "m2cg_sync": (C.c_int, [_P]),
        "m2cg_event_record": (C.c_int, [_P, C.c_int32]),
        "m2cg_event_elapsed": (C.c_int, [_P, C.c_int32, C.c_int32, C.POINTER(C.c_float)]),
        "m2cg_kernel_launches": (C.c_int64, [_P]),
        "m2cg_host_alloc": (C.c_void_p, [C.c_size_t]),
        "m2cg_phase_times": (C.c_int, [_P, C.c_int32, _D]),
        "m2cg_riemann_batch_noalloc": (C.c_int, [C.POINTER(Config), C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                                 C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                 C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]),
        "m2cg_host_free": (None, [C.c_void_p]),
        "m2cg_riemann_batch_eos": (C.c_int, [_P, C.c_int64, _D, _D, _D, _D, _I, _I, _F]),
        "m2cg_mlp_create": (C.c_int, [C.c_uint64, C.POINTER(_P)]),
        "m2cg_mlp_destroy": (None, [_P]),
        "m2cg_mlp_set_params": (C.c_int, [_P, _F]),
        "m2cg_mlp_get_params": (C.c_int, [_P, _F]),
        "m2cg_mlp_features": (C.c_int, [C.c_int64, _D, _D, _D, _F, _F, _F]),
        "m2cg_mlp_set_data": (C.c_int, [_P, C.c_int64, _D, _D, _D]),
        "m2cg_mlp_train": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_float, C.c_uint64, _F, _F]),
        "m2cg_mlp_grad": (C.c_int, [_P, C.c_int64, _F, _F, _F, _F]),
        "m2cg_mlp_adam_step": (C.c_int, [_P, _F, C.c_float]),
        "m2cg_mlp_forward": (C.c_int, [_P, C.c_int64, _F, _F]),
        "m2cg_mlp_predict": (C.c_int, [_P, C.c_int64, _D, _D, _D, _F]),
        "m2cg_set_warm_start": (C.c_int, [_P, _P]),
        "m2cg_ensemble_create": (C.c_int, [C.POINTER(Config), C.c_int32, C.POINTER(_P)]),
        "m2cg_ensemble_destroy": (None, [_P]),
        "m2cg_ensemble_size": (C.c_int32, [_P]),
        "m2cg_ensemble_member": (_P, [_P, C.c_int32]),
        "m2cg_ensemble_run": (C.c_int, [_P, C.c_int32, _F]),
        "m2cg_ensemble_run_sequential": (C.c_int, [_P, C.c_int32, _F]),
        "m2cg_ensemble_kernel_launches": (C.c_int64, [_P]),
        "m2cg_ensemble_autotune": (C.c_int, [_P, C.c_int32, C.c_int32, _I, _I, _F]),
        "m2cg_ensemble_autotune_tiles": (C.c_int, [_P, C.c_int32, C.c_int32, _I, _I, _F]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if lib.m2cg_config_size() != C.sizeof(Config):
        raise RuntimeError(f"m2cg_config layout mismatch: C {lib.m2cg_config_size()} vs ctypes {C.sizeof(Config)}")
    if lib.m2cg_counters_size() != C.sizeof(Counters):
        raise RuntimeError("m2cg_counters layout mismatch")
    if path is None:
        _lib = lib
    return lib


def check(lib, status, what):
    if status != 0:
        msg = lib.m2cg_last_error()
        raise RuntimeError(f"{what} failed: {STATUS.get(status, status)}: {msg.decode() if msg else ''}")
