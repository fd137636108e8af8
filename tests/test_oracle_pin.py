"""Pin the oracle: it must reproduce the reference's own compiled code
(oracle/_ref, built from the reference sources) and the reference's golden
exact-Riemann files (tests/golden, extracted by make_riemann_golden.py)."""
import numpy as np
import pytest

from helpers import config_for_materials, golden_problem, golden_riemann_cases, random_sg_states
from m2c_gb300 import abi
from oracle import binding as ob

CASES = golden_riemann_cases()
# cases whose 1- and 3-waves are both shocks: the reference's Hugoniot path is
# unchanged since the golden files were written, so they agree to print precision
SHOCK_SHOCK = {"Test4", "Test8", "Test9", "Test10"}


@pytest.fixture(scope="module")
def ref():
    r = ob.ref_lib()
    if r is None:
        pytest.skip("reference sources not available on this machine")
    return r


@pytest.mark.parametrize("case", CASES, ids=[c["test"] for c in CASES])
def test_oracle_equals_reference_build_on_golden_inputs(ref, case):
    for tol in (1e-5, 1e-10):
        cfg = config_for_materials(case["materials"], tol=tol)
        Vm, idm, Vp, idp, d = golden_problem(case)
        o = ob.riemann_batch(cfg, Vm, idm, Vp, idp, d)
        r = ob.ref_riemann_batch(ref, cfg, Vm, idm, Vp, idp, d)
        assert o["err"][0] == r["err"][0]
        np.testing.assert_array_equal(o["Vsm"], r["Vsm"])
        np.testing.assert_array_equal(o["Vsp"], r["Vsp"])
        np.testing.assert_array_equal(o["Vs"], r["Vs"])
        assert o["id"][0] == r["id"][0]


@pytest.mark.parametrize("case", CASES, ids=[c["test"] for c in CASES])
def test_oracle_against_golden_star_states(case):
    cfg = config_for_materials(case["materials"], tol=1e-10)
    Vm, idm, Vp, idp, d = golden_problem(case)
    o = ob.riemann_batch(cfg, Vm, idm, Vp, idp, d)
    assert o["err"][0] == 0
    got = dict(u_star=o["Vsm"][0, 1], p_star=o["Vsm"][0, 4], rho_l_star=o["Vsm"][0, 0], rho_r_star=o["Vsp"][0, 0])
    u_scale = max(abs(case["left"][1]), abs(case["right"][1]), abs(case["u_star"]), 1e-300)
    if case["test"] in SHOCK_SHOCK:
        tol = 2e-6   # 7 printed digits of the golden file and of its header inputs
    elif case["test"] in ("Test11", "Test12"):
        # near-vacuum rarefaction (rho_L = 1.2e-6): the current reference's
        # Cash-Karp stage pressure (ExactRiemannSolverBase.cpp:1809) moves p* far
        # from the older golden; the contact velocity and the right star density agree
        assert abs(got["u_star"] - case["u_star"]) / u_scale < 2e-3
        assert abs(got["rho_r_star"] - case["rho_r_star"]) / case["rho_r_star"] < 1e-6
        return
    else:
        tol = 3e-3   # rarefaction cases: same stage-pressure difference, bounded
    assert abs(got["u_star"] - case["u_star"]) / u_scale < tol
    for k in ("p_star", "rho_l_star", "rho_r_star"):
        assert abs(got[k] - case[k]) / abs(case[k]) < tol, k


def _random_two_material_cfg(rng):
    c = abi.default_config()
    c.n_materials = 3
    abi.set_material(c.mat[0], abi.EOS_SG, gamma=rng.uniform(1.1, 7.0), pc=rng.uniform(0, 6e8))
    abi.set_material(c.mat[1], abi.EOS_NASG, gamma=rng.uniform(1.1, 3.0), pc=rng.uniform(0, 6e8),
                     b=rng.uniform(0, 1e-3), q=0.0)
    abi.set_material(c.mat[2], abi.EOS_SG, gamma=1.4, pc=0.0)
    c.tol_main = 1e-10
    return c


def _make_physical(cfg, V, ids, rng):
    # Noble-Abel stiffened gas needs 1/rho > b (VarFcnNASG.h:55); the reference
    # stops the process on a nonphysical input, so keep the inputs physical.
    b = cfg.mat[1].b
    sel = (ids == 1) & (V[:, 0] * b > 0.5)
    V[sel, 0] = rng.uniform(0.05, 0.5, sel.sum()) / b


def test_oracle_equals_reference_build_random_riemann(ref):
    rng = np.random.default_rng(7)
    for trial in range(4):
        cfg = _random_two_material_cfg(rng)
        n = 200
        Vm = random_sg_states(rng, n)
        Vp = random_sg_states(rng, n)
        idm = rng.integers(0, 3, n).astype(np.int32)
        idp = rng.integers(0, 3, n).astype(np.int32)
        _make_physical(cfg, Vm, idm, rng)
        _make_physical(cfg, Vp, idp, rng)
        dirs = np.zeros((n, 3))
        dirs[np.arange(n), rng.integers(0, 3, n)] = 1.0
        o = ob.riemann_batch(cfg, Vm, idm, Vp, idp, dirs)
        r = ob.ref_riemann_batch(ref, cfg, Vm, idm, Vp, idp, dirs)
        # every solve, including the failures that go through the reference's
        # non-adaptive retry (ExactRiemannSolverBase.cpp:178-193, 323-337)
        np.testing.assert_array_equal(o["err"], r["err"])
        ok = o["err"] >= 0
        np.testing.assert_array_equal(o["Vsm"][ok], r["Vsm"][ok])
        np.testing.assert_array_equal(o["Vsp"][ok], r["Vsp"][ok])
        np.testing.assert_array_equal(o["Vs"][ok], r["Vs"][ok])
        assert ok.all()


def test_oracle_equals_reference_build_on_stalled_secant_cases(ref):
    # nearly-equal states across a gas/water interface whose secant iteration
    # stalls and falls back to the non-adaptive solver (seen in the shock-bubble run)
    from m2c_gb300 import problems
    cfg = problems.shock_bubble(n=8)[0]
    Vm = np.array([[998.20519390865695, 3.3314753181257264e-12, 0, 0, 99999.991927862167],
                   [1006.1150592521593, 1.8715164624221656e-14, 0, 0, 99999.991991758347]])
    Vp = np.array([[1.1938544441698975, -2.7841691152760676e-09, 0, 0, 99999.999999021107],
                   [1.2008467212565481, -3.0730441045384747e-11, 0, 0, 99999.999999807304]])
    idm, idp = np.zeros(2, np.int32), np.ones(2, np.int32)
    dirs = np.array([[1.0, 0, 0], [1.0, 0, 0]])
    o = ob.riemann_batch(cfg, Vm, idm, Vp, idp, dirs)
    r = ob.ref_riemann_batch(ref, cfg, Vm, idm, Vp, idp, dirs)
    np.testing.assert_array_equal(o["err"], r["err"])
    for k in ("Vsm", "Vsp", "Vs"):
        np.testing.assert_array_equal(o[k], r[k])


@pytest.mark.parametrize("flux", [abi.FLUX_HLLC, abi.FLUX_LLF, abi.FLUX_ROE])
def test_oracle_equals_reference_build_fluxes(ref, flux):
    rng = np.random.default_rng(11 + flux)
    cfg = _random_two_material_cfg(rng)
    cfg.flux = flux
    n = 2000
    Vm = random_sg_states(rng, n)
    Vp = Vm * (1 + 0.2 * rng.uniform(-1, 1, (n, 5)))
    Vp[:, 1:4] = Vm[:, 1:4] + rng.uniform(-50, 50, (n, 3))
    ids = rng.integers(0, 3, n).astype(np.int32)
    _make_physical(cfg, Vm, ids, rng)
    _make_physical(cfg, Vp, ids, rng)
    dirs = rng.integers(0, 3, n).astype(np.int32)
    np.testing.assert_array_equal(ob.flux_batch(cfg, dirs, Vm, Vp, ids), ob.ref_flux_batch(ref, cfg, dirs, Vm, Vp, ids))


def _assert_same_solutions(o, r):
    np.testing.assert_array_equal(o["err"], r["err"])
    np.testing.assert_array_equal(o["id"], r["id"])
    for k in ("Vsm", "Vsp", "Vs"):
        np.testing.assert_array_equal(o[k], r[k])


def test_oracle_equals_reference_build_on_tilted_directions(ref):
    # the LevelSet and Average interface normals (SpaceOperator.cpp:2186-2415)
    # hand the solver directions off the mesh axes: random unit vectors here
    rng = np.random.default_rng(17)
    for trial in range(3):
        cfg = _random_two_material_cfg(rng)
        n = 200
        Vm = random_sg_states(rng, n)
        Vp = random_sg_states(rng, n)
        idm = rng.integers(0, 3, n).astype(np.int32)
        idp = rng.integers(0, 3, n).astype(np.int32)
        _make_physical(cfg, Vm, idm, rng)
        _make_physical(cfg, Vp, idp, rng)
        dirs = rng.normal(size=(n, 3))
        dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
        _assert_same_solutions(ob.riemann_batch(cfg, Vm, idm, Vp, idp, dirs),
                               ob.ref_riemann_batch(ref, cfg, Vm, idm, Vp, idp, dirs))


def test_oracle_equals_reference_build_on_shock_bubble_interface_problems(ref):
    # every interface problem of a 24^3 shock-bubble after two RK3 steps with
    # level-set normals: mostly near-trivial gas/water states (equal
    # pressures, velocities differing in the last bits) along tilted normals,
    # many of which stall and go through the non-adaptive retry
    from m2c_gb300 import problems
    cfg, V, ID, phi = problems.shock_bubble(n=24)
    cfg.ts_type = abi.TS_RK3
    cfg.mp_riemann_normal = abi.RNORMAL_LEVEL_SET
    o = ob.OracleSim(cfg)
    o.upload(V, ID, phi)
    o.run(2)
    V, ID, _ = o.download()
    n = cfg.nx
    I3 = ID.reshape(n, n, n)
    rows = []
    for d, st in enumerate((1, n, n * n)):
        for k in range(n):
            for j in range(n):
                for i in range(n):
                    pos = (i, j, k)
                    if pos[d] == 0:
                        continue
                    c = (k * n + j) * n + i
                    m = c - st
                    if ID[m] != ID[c]:
                        rows.append((d, i, j, k, c, m))
    assert len(rows) > 200
    Vm = np.array([V[m] for *_, m in rows])
    Vp = np.array([V[c] for *_, c, m in rows])
    idm = np.array([ID[m] for *_, m in rows], np.int32)
    idp = np.array([ID[c] for *_, c, m in rows], np.int32)
    dirs = np.array([o.riemann_normal(d, i, j, k, ID[c], ID[m]) for d, i, j, k, c, m in rows])
    assert (np.abs(dirs).max(1) < 1.0 - 1e-6).mean() > 0.5   # mostly off the mesh axes
    res = ob.riemann_batch(cfg, Vm, idm, Vp, idp, dirs)
    assert (res["err"] != 0).sum() > 0   # stalled solves included
    _assert_same_solutions(res, ob.ref_riemann_batch(ref, cfg, Vm, idm, Vp, idp, dirs))
