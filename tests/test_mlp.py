"""Learned warm start: data sets, the tensor-core network against its CPU
reference (features, forward, gradients), the per-problem-EOS exact solver
against the oracle (cold and warm), training, and the warm start's effect on
the exact solve -- in batches and inside the finite-volume step."""
import ctypes as C

import numpy as np
import pytest

import mlp_ref
from m2c_gb300 import abi
from m2c_gb300 import warmstart as ws


def oracle_batch_eos(cfg, W, E, warm=None):
    from oracle import binding as ob
    lib = ob.lib()
    f = lib.orc_riemann_batch_eos
    f.restype = None
    f.argtypes = [C.POINTER(type(cfg)), C.c_int64, abi._D, abi._D, abi._D, abi._D, abi._I, abi._I]
    n = len(W)
    out = np.zeros((n, 4))
    it, err = np.zeros(n, np.int32), np.zeros(n, np.int32)
    f(C.byref(cfg), n, abi.dptr(np.ascontiguousarray(W)), abi.dptr(np.ascontiguousarray(E)),
      abi.dptr(None if warm is None else np.ascontiguousarray(warm, np.float64)), abi.dptr(out), abi.iptr(it),
      abi.iptr(err))
    return out, it, err


# ---------------------------------------------------------------- CPU ----------
def test_sample_problems_ranges_and_seed():
    W, E = ws.sample_problems(20000, 7)
    W2, E2 = ws.sample_problems(20000, 7)
    assert np.array_equal(W, W2) and np.array_equal(E, E2)
    for s in range(2):
        rho, u, p = W[:, 3 * s], W[:, 3 * s + 1], W[:, 3 * s + 2]
        assert rho.min() >= 0.1 and rho.max() <= 2000.0
        assert np.abs(u).max() <= 500.0
        assert p.min() >= 1e4 and p.max() <= 1e10
        typ, gam, pc, b = E[:, 5 * s], E[:, 5 * s + 1], E[:, 5 * s + 2], E[:, 5 * s + 3]
        assert set(np.unique(typ)) == {0.0, 1.0}
        assert gam.min() >= 1.1 and gam.max() <= 7.0 and pc.min() >= 0 and pc.max() <= 6e8
        assert np.all(b[typ == 0] == 0) and b.max() <= 1e-3
        c2 = gam * (p + pc) / (rho * (1 - b * rho))
        assert np.all(c2 > 0) and np.all(1 - b * rho > 0)
        # log-uniform density: median near the geometric mean of the bounds
        assert abs(np.log10(np.median(rho)) - 0.5 * (np.log10(0.1) + np.log10(2000.0))) < 0.3


def test_reference_backward_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = rng.normal(0, 0.3, mlp_ref.NPARAM)
    X = rng.normal(0, 1, (40, mlp_ref.NF))
    X[:, 12:] = 0
    t = rng.normal(0, 1, 40)
    _, loss, g = mlp_ref.forward_backward(p, X, t, rounding=False)
    idx = np.concatenate([rng.choice(np.arange(lo, hi), min(8, hi - lo), replace=False)
                          for lo, hi in mlp_ref.BLOCKS.values()])
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (mlp_ref.forward_backward(pp, X, t, False)[1] - mlp_ref.forward_backward(pm, X, t, False)[1]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_oracle_batch_eos_matches_oracle_batch():
    """The per-problem-EOS oracle entry equals the material-table one when the
    pair is the table's."""
    from oracle import binding as ob
    cfg = ws.solver_config(1e-10)
    abi.set_material(cfg.mat[0], abi.EOS_SG, gamma=6.12, pc=3.43e8)
    abi.set_material(cfg.mat[1], abi.EOS_NASG, gamma=1.19, pc=6.2e8, b=6.61e-4)
    rng = np.random.default_rng(5)
    n = 300
    W = np.column_stack([rng.uniform(900, 1100, n), rng.uniform(-50, 50, n), 10 ** rng.uniform(5, 9, n),
                         rng.uniform(900, 1100, n), rng.uniform(-50, 50, n), 10 ** rng.uniform(5, 9, n)])
    E = np.tile([0, 6.12, 3.43e8, 0, 0, 1, 1.19, 6.2e8, 6.61e-4, 0], (n, 1)).astype(float)
    out, it, err = oracle_batch_eos(cfg, W, E)
    Vm = np.column_stack([W[:, 0], W[:, 1], 0 * W[:, 0], 0 * W[:, 0], W[:, 2]])
    Vp = np.column_stack([W[:, 3], W[:, 4], 0 * W[:, 0], 0 * W[:, 0], W[:, 5]])
    dirs = np.tile([1.0, 0, 0], (n, 1))
    r = ob.riemann_batch(cfg, Vm, np.zeros(n, np.int32), Vp, np.ones(n, np.int32), dirs)
    assert np.array_equal(out[:, 0], r["Vsm"][:, 4]) and np.array_equal(out[:, 2], r["Vsm"][:, 0])
    assert np.array_equal(out[:, 3], r["Vsp"][:, 0]) and np.array_equal(err, r["err"])


def test_oracle_warm_start_keeps_the_stopping_rule():
    """A warm start at the exact root, or far off it, ends where the cold
    start ends, within the reference's stopping rule."""
    cfg = ws.solver_config(1e-10)
    W, E = ws.sample_problems(3000, 21)
    cold, cit, cerr = oracle_batch_eos(cfg, W, E)
    ok = (cerr == 0) & (cold[:, 0] > 0)
    for f in (1.0, 1.02, 0.5):
        warm, wit, werr = oracle_batch_eos(cfg, W, E, np.where(ok, cold[:, 0] * f, 0.0))
        both = ok & (werr == 0)
        assert both.sum() >= 0.99 * ok.sum()
        rel = np.abs(warm[both, 0] - cold[both, 0]) / cold[both, 0]
        assert np.median(rel) < 1e-5 and np.quantile(rel, 0.99) < 1e-3
    # started at the root, the warm start needs fewer evaluations
    warm, wit, werr = oracle_batch_eos(cfg, W, E, np.where(ok, cold[:, 0], 0.0))
    assert wit[ok].mean() < cit[ok].mean()


# ---------------------------------------------------------------- GPU ----------
gpu = pytest.mark.gpu


@gpu
def test_riemann_batch_eos_matches_oracle():
    W, E = ws.sample_problems(4000, 11)
    cfg = ws.solver_config(1e-10)
    solver = ws.BatchSolver(1e-10)
    g = solver.solve(W, E)
    o, oit, oerr = oracle_batch_eos(cfg, W, E)
    assert np.array_equal(g["err"], oerr)
    ok = oerr == 0
    rel = np.abs(g["pstar"][ok] - o[ok, 0]) / np.maximum(np.abs(o[ok, 0]), 1e-300)
    assert np.quantile(rel, 0.99) < 1e-11 and rel.max() < 1e-7
    assert np.mean(np.abs(g["iters"] - oit) <= 2) > 0.99
    # warm start from a perturbed root: GPU and oracle take the same path
    warm = np.where(ok, o[:, 0] * 1.01, 0.0)
    gw = solver.solve(W, E, warm_p=warm)
    ow, owit, owerr = oracle_batch_eos(cfg, W, E, warm)
    okw = (owerr == 0) & ok
    relw = np.abs(gw["pstar"][okw] - ow[okw, 0]) / np.abs(ow[okw, 0])
    assert np.quantile(relw, 0.99) < 1e-11
    assert np.mean(np.abs(gw["iters"] - owit) <= 2) > 0.99
    solver.close()


@gpu
def test_features_match_reference():
    W, E = ws.sample_problems(5000, 12)
    net = ws.WarmStartMLP(1)
    X, pref, _ = net.features(W, E)
    Xr, prefr = mlp_ref.features(W, E)
    assert np.allclose(pref, prefr, rtol=1e-6)
    ulp = np.abs(Xr) * 2.0 ** -7 + 1e-30
    assert np.all(np.abs(X - Xr) <= ulp)
    assert np.mean(X == Xr) > 0.999


@gpu
def test_forward_and_gradients_match_reference():
    rng = np.random.default_rng(13)
    net = ws.WarmStartMLP(3)
    p = net.params.astype(np.float64)
    p[mlp_ref.OFF_B1:mlp_ref.OFF_W2] = rng.normal(0, 0.1, 64)
    p[mlp_ref.OFF_B2:mlp_ref.OFF_W3] = rng.normal(0, 0.1, 64)
    p[mlp_ref.OFF_B3:mlp_ref.OFF_W4] = rng.normal(0, 0.1, 64)
    p[mlp_ref.OFF_B4] = 0.3
    net.params = p.astype(np.float32)
    p = net.params.astype(np.float64)
    for n in (128, 300, 1000):
        X = rng.normal(0, 1, (n, 16)).astype(np.float32)
        X[:, 12:] = 0
        t = rng.normal(0, 1, n).astype(np.float32)
        out_ref, loss_ref, g_ref = mlp_ref.forward_backward(p, X, t)
        out = net.forward(X)
        assert np.max(np.abs(out - out_ref)) < 2e-3 * max(1.0, np.max(np.abs(out_ref)))
        g, loss = net.grad(X, t)
        assert abs(loss - loss_ref) <= 1e-3 * loss_ref
        for name, (lo, hi) in mlp_ref.BLOCKS.items():
            err = np.max(np.abs(g[lo:hi] - g_ref[lo:hi])) / max(np.max(np.abs(g_ref[lo:hi])), 1e-30)
            assert err < 1e-2, (n, name, err)


@gpu
def test_adam_step_matches_numpy():
    # two updates: moments, bias corrections (1 - beta^t) and the parameter step
    rng = np.random.default_rng(29)
    net = ws.WarmStartMLP(5)
    p = rng.normal(0, 0.2, abi.MLP_PARAMS).astype(np.float32)
    net.params = p
    b1, b2, eps, lr = np.float32(0.9), np.float32(0.999), np.float32(1e-8), np.float32(3e-3)
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    for t in (1, 2):
        g = rng.normal(0, 1, abi.MLP_PARAMS).astype(np.float32) * np.float32(10.0) ** rng.uniform(-6, 1, abi.MLP_PARAMS).astype(np.float32)
        net.adam_step(g, lr)
        m = b1 * m + (np.float32(1) - b1) * g
        v = b2 * v + (np.float32(1) - b2) * g * g
        bc1 = np.float32(1) - b1 ** np.float32(t)
        bc2 = np.float32(1) - b2 ** np.float32(t)
        step = lr * (m / bc1) / (np.sqrt(v / bc2) + eps)
        p = p - step
        got = net.params
        # float32 arithmetic on both sides; the device contracts to FMA
        assert np.all(np.abs(got - p) <= 1e-5 * np.abs(step) + 2e-7 * np.abs(p)), t
    net.close()


@gpu
def test_training_and_warm_start():
    """The trained network predicts the star pressure better than the acoustic
    estimate the reference starts from on the problems with a strong acoustic
    jump (above 5 %); started from its predictions the exact solver needs no
    more wave-pair evaluations than the cold start (1-5 % fewer across six
    trained networks) and ends where the cold solve ends within the
    reference's stopping rule."""
    res = ws.study(n_train=1 << 20, n_test=1 << 15, epochs=60, batch=16384, lr=3e-3, seed=99)
    assert res["loss_last_epoch"] < 0.05 * res["loss_first_epoch"]
    assert res["pstar_rel_err_median"] < 0.03
    assert res["pstar_rel_err_median_strong"] < 0.5 * res["acoustic_rel_err_median_strong"]
    assert res["iters_warm_mean_converged"] <= res["iters_cold_mean_converged"]
    # the bound for any predictor: the same solver started at the converged root
    assert res["converged_set"]["iters_exact_start_mean"] < res["iters_cold_mean_converged"]
    assert res["warm_vs_cold_pstar_rel_median"] < 1e-5 and res["warm_vs_cold_pstar_rel_p99"] < 1e-3
    assert res["failed_warm"] <= res["failed_cold"] + 2


@gpu
def test_fv_step_with_warm_start():
    """Shock-bubble steps with the warm start enabled stay close to the
    cold-start run and solve the same faces."""
    from m2c_gb300 import problems
    from m2c_gb300.solver import FluidState, Solver
    cfg, V, ID, phi = problems.shock_bubble(n=32)
    W, E = ws.sample_problems(1 << 14, 5)
    solver = ws.BatchSolver(1e-10)
    lab = solver.solve(W, E)
    keep = (lab["err"] == 0) & (lab["pstar"] > 0)
    net = ws.WarmStartMLP(5)
    net.set_data(W[keep], E[keep], lab["pstar"][keep])
    net.train(8, 2048, 3e-3, 5)
    cold = Solver(cfg, FluidState(V, ID, phi))
    warm = Solver(cfg, FluidState(V, ID, phi))
    warm.set_warm_start(net)
    cc = cold.run(5)
    cw = warm.run(5)
    a, b = cold.get_state(), warm.get_state()
    assert np.array_equal(a.ID, b.ID)
    for k in (0, 4):
        rel = np.max(np.abs(a.V[:, k] - b.V[:, k])) / np.max(np.abs(a.V[:, k]))
        assert rel < 1e-7, (k, rel)
    assert cw["riemann_solves"] == cc["riemann_solves"]
    assert cw["riemann_iterations"] < 3 * cc["riemann_iterations"]
    warm.set_warm_start(None)
    cold.close(); warm.close(); net.close(); solver.close()
