"""m2cg_riemann_batch_noalloc: the exact Riemann solves for callers that cannot
allocate device memory (they pass their own device buffers; the solver's scratch
is a static device array).  Checked through the C ABI against the allocating
entry point m2cg_riemann_batch, on two calls in a row.  This file is collected
last so a failure here leaves every other test already run."""
import ctypes as C

import numpy as np
import pytest

from helpers import config_for_materials, golden_riemann_cases, random_sg_states
from m2c_gb300 import abi
from m2c_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def _problems():
    rng = np.random.default_rng(21)
    cfg = abi.default_config()
    cfg.n_materials = 3
    abi.set_material(cfg.mat[0], abi.EOS_SG, gamma=6.12, pc=3.43e8)
    abi.set_material(cfg.mat[1], abi.EOS_SG, gamma=1.4, pc=0.0)
    abi.set_material(cfg.mat[2], abi.EOS_NASG, gamma=1.19, pc=6.2e8, b=6.61e-4, q=0.0)
    cfg.tol_main = 1e-10
    n = 3000
    Vm, Vp = random_sg_states(rng, n), random_sg_states(rng, n)
    idm = rng.integers(0, 3, n).astype(np.int32)
    idp = rng.integers(0, 3, n).astype(np.int32)
    for V, ids in ((Vm, idm), (Vp, idp)):
        sel = (ids == 2) & (V[:, 0] * 6.61e-4 > 0.5)
        V[sel, 0] = rng.uniform(50, 700, sel.sum())
    dirs = np.zeros((n, 3))
    dirs[np.arange(n), rng.integers(0, 3, n)] = 1.0
    return cfg, Vm, idm, Vp, idp, dirs


def _noalloc(lib, cfg, Vm, idm, Vp, idp, dirs, path_cap=1024):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    n = len(idm)
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev)
         for k, v in dict(Vm=Vm, idm=idm.astype(np.int32), Vp=Vp, idp=idp.astype(np.int32), dir=dirs).items()}
    out = dict(Vs=torch.zeros(n, 5, dtype=torch.float64, device=dev), id=torch.zeros(n, dtype=torch.int32, device=dev),
               Vsm=torch.zeros(n, 5, dtype=torch.float64, device=dev), Vsp=torch.zeros(n, 5, dtype=torch.float64, device=dev),
               iters=torch.zeros(n, dtype=torch.int32, device=dev), err=torch.zeros(n, dtype=torch.int32, device=dev))
    s = torch.cuda.current_stream()
    st = lib.m2cg_riemann_batch_noalloc(C.byref(cfg), n, t["Vm"].data_ptr(), t["idm"].data_ptr(), t["Vp"].data_ptr(),
                                        t["idp"].data_ptr(), t["dir"].data_ptr(), out["Vs"].data_ptr(),
                                        out["id"].data_ptr(), out["Vsm"].data_ptr(), out["Vsp"].data_ptr(),
                                        out["iters"].data_ptr(), out["err"].data_ptr(), path_cap, s.cuda_stream)
    abi.check(lib, st, "m2cg_riemann_batch_noalloc")
    s.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items()}


def _compare(a, b):
    np.testing.assert_array_equal(a["err"], b["err"])
    ok = a["err"] == 0
    np.testing.assert_array_equal(a["id"][ok], b["id"][ok])
    np.testing.assert_array_equal(a["iters"], b["iters"])
    for k in ("Vs", "Vsm", "Vsp"):
        np.testing.assert_allclose(a[k][ok], b[k][ok], rtol=1e-12, atol=0)


def test_noalloc_matches_allocating_entry_point_twice():
    cfg, Vm, idm, Vp, idp, dirs = _problems()
    s = Solver(cfg)
    ref = s.riemann_batch(Vm, idm, Vp, idp, dirs)
    for _ in range(2):
        got = _noalloc(s.lib, cfg, Vm, idm, Vp, idp, dirs)
        _compare(got, ref)


def test_noalloc_golden_cases_and_limits():
    lib = abi.load()
    for case in golden_riemann_cases():
        cfg = config_for_materials(case["materials"], tol=1e-10)
        Vm = np.array([[case["left"][0], case["left"][1], 0.0, 0.0, case["left"][2]]])
        Vp = np.array([[case["right"][0], case["right"][1], 0.0, 0.0, case["right"][2]]])
        idm, idp = np.array([case["idl"]], np.int32), np.array([case["idr"]], np.int32)
        dirs = np.array([[1.0, 0.0, 0.0]])
        ref = Solver(cfg).riemann_batch(Vm, idm, Vp, idp, dirs)
        for _ in range(2):
            _compare(_noalloc(lib, cfg, Vm, idm, Vp, idp, dirs), ref)
    cfg = config_for_materials(golden_riemann_cases()[0]["materials"])
    z = np.zeros((1, 5))
    with pytest.raises(RuntimeError, match="CAPACITY"):
        _noalloc(lib, cfg, z + 1, np.zeros(1, np.int32), z + 1, np.zeros(1, np.int32), np.array([[1.0, 0, 0]]),
                 path_cap=4096)


def test_noalloc_invalid_material_rows_are_marked():
    # a row whose material ID is outside the configuration is not solved: id -1,
    # err -2 and NaN star states, while the other rows match the allocating path
    cfg, Vm, idm, Vp, idp, dirs = _problems()
    n = 64
    Vm, idm, Vp, idp, dirs = Vm[:n], idm[:n].copy(), Vp[:n], idp[:n].copy(), dirs[:n]
    idm[5] = 7
    idp[9] = -1
    lib = abi.load()
    got = _noalloc(lib, cfg, Vm, idm, Vp, idp, dirs)
    for r in (5, 9):
        assert got["err"][r] == -2 and got["id"][r] == -1 and got["iters"][r] == 0
        for k in ("Vs", "Vsm", "Vsp"):
            assert np.isnan(got[k][r]).all()
    good = np.ones(n, bool)
    good[[5, 9]] = False
    ref = Solver(cfg).riemann_batch(Vm[good], idm[good], Vp[good], idp[good], dirs[good])
    _compare({k: v[good] for k, v in got.items()}, ref)
