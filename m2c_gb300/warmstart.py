"""Learned warm start for the exact two-material Riemann solve.

Data: independent interface problems drawn from a seed -- per side rho
log-uniform in [0.1, 2000] kg/m^3, u uniform in [-500, 500] m/s, p log-uniform
in [1e4, 1e10] Pa, and a stiffened gas (gamma in [1.1, 7], pc in [0, 6e8] Pa)
or a Noble-Abel stiffened gas (the same plus b in [0, 1e-3] m^3/kg, q = 0);
problems whose sound speed squared is not positive on either side are drawn
again.  Labels: the exact solver's FP64 star pressure at the configured
tolerance (1e-10 here), computed on the GPU (m2cg_riemann_batch_eos).

Model and training: the library's tensor-core MLP (m2cg_mlp_*).  Evaluation:
the same exact solver on held-out problems, cold (the reference's acoustic
starting pair) against warm (a starting pair bracketing the network's
prediction), comparing wave-pair evaluations per solve (bracketing + main
loop, the reference's iteration count) and device time, network inference
included in the warm time.
"""
import ctypes as C

import numpy as np

from . import abi


def sample_problems(n, seed):
    """n problems (W: n x 6 {rho_l, u_l, p_l, rho_r, u_r, p_r}, E: n x 10)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    W = np.empty((0, 6))
    E = np.empty((0, 10))
    while len(W) < n:
        m = int((n - len(W)) * 1.6) + 64
        w = np.empty((m, 6))
        e = np.zeros((m, 10))
        for s in range(2):
            w[:, 3 * s + 0] = 10.0 ** rng.uniform(-1.0, np.log10(2000.0), m)
            w[:, 3 * s + 1] = rng.uniform(-500.0, 500.0, m)
            w[:, 3 * s + 2] = 10.0 ** rng.uniform(4.0, 10.0, m)
            nasg = rng.random(m) < 0.5
            e[:, 5 * s + 0] = np.where(nasg, abi.EOS_NASG, abi.EOS_SG)
            e[:, 5 * s + 1] = rng.uniform(1.1, 7.0, m)
            e[:, 5 * s + 2] = rng.uniform(0.0, 6.0e8, m)
            e[:, 5 * s + 3] = np.where(nasg, rng.uniform(0.0, 1.0e-3, m), 0.0)
        ok = np.ones(m, bool)
        for s in range(2):
            rho, p = w[:, 3 * s], w[:, 3 * s + 2]
            gam, pc, b = e[:, 5 * s + 1], e[:, 5 * s + 2], e[:, 5 * s + 3]
            c2 = gam * (p + pc) / (rho * (1.0 - b * rho))
            ok &= (c2 > 0.0) & (1.0 - b * rho > 0.0)
        W = np.concatenate([W, w[ok]])
        E = np.concatenate([E, e[ok]])
    return np.ascontiguousarray(W[:n]), np.ascontiguousarray(E[:n])


def acoustic_estimate(W, E):
    """Acoustic-theory star pressure (ExactRiemannSolverBase.cpp:1107-1116) and
    the acoustic pressure jump relative to the impedance-weighted pressure."""
    rl, ul, pl, rr, ur, pr = (W[:, i] for i in range(6))
    c2l = E[:, 1] * (pl + E[:, 2]) / (rl * (1.0 - E[:, 3] * rl))
    c2r = E[:, 6] * (pr + E[:, 7]) / (rr * (1.0 - E[:, 8] * rr))
    Cl, Cr = rl * np.sqrt(c2l), rr * np.sqrt(c2r)
    pbar = (Cr * pl + Cl * pr) / (Cl + Cr)
    p0 = pbar + Cl * Cr * (ul - ur) / (Cl + Cr)
    return p0, np.abs(p0 - pbar) / np.abs(pbar)


def solver_config(tol=1e-10):
    c = abi.default_config()
    c.nx = c.ny = c.nz = 1
    c.x0, c.xmax, c.y0, c.ymax, c.z0, c.zmax = 0.0, 1.0, 0.0, 1.0, 0.0, 1.0
    c.n_materials = 2
    abi.set_material(c.mat[0], abi.EOS_SG, gamma=1.4)
    abi.set_material(c.mat[1], abi.EOS_SG, gamma=1.4)
    c.tol_main = tol
    return c


class BatchSolver:
    """Exact Riemann solves of W / E problems on the GPU (one context)."""

    def __init__(self, tol=1e-10, lib=None):
        self.lib = lib or abi.load()
        self.cfg = solver_config(tol)
        h = C.c_void_p()
        abi.check(self.lib, self.lib.m2cg_create(C.byref(self.cfg), C.byref(h)), "m2cg_create")
        self.ctx = h

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.m2cg_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        self.close()

    def solve(self, W, E, warm_p=None):
        n = len(W)
        W = np.ascontiguousarray(W, np.float64)
        E = np.ascontiguousarray(E, np.float64)
        wp = None if warm_p is None else np.ascontiguousarray(warm_p, np.float64)
        out = np.zeros((n, 4))
        it = np.zeros(n, np.int32)
        err = np.zeros(n, np.int32)
        ms = C.c_float()
        abi.check(self.lib, self.lib.m2cg_riemann_batch_eos(self.ctx, n, abi.dptr(W), abi.dptr(E), abi.dptr(wp),
                                                            abi.dptr(out), abi.iptr(it), abi.iptr(err),
                                                            C.byref(ms)), "m2cg_riemann_batch_eos")
        return dict(pstar=out[:, 0], ustar=out[:, 1], rhol=out[:, 2], rhor=out[:, 3], iters=it, err=err,
                    ms=ms.value)


class WarmStartMLP:
    """The library's warm-start network (m2cg_mlp_*)."""

    def __init__(self, seed=0, lib=None):
        self.lib = lib or abi.load()
        h = C.c_void_p()
        abi.check(self.lib, self.lib.m2cg_mlp_create(seed, C.byref(h)), "m2cg_mlp_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.m2cg_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    @property
    def params(self):
        p = np.zeros(abi.MLP_PARAMS, np.float32)
        abi.check(self.lib, self.lib.m2cg_mlp_get_params(self.h, abi.fptr(p)), "m2cg_mlp_get_params")
        return p

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.shape == (abi.MLP_PARAMS,)
        abi.check(self.lib, self.lib.m2cg_mlp_set_params(self.h, abi.fptr(p)), "m2cg_mlp_set_params")

    def features(self, W, E, pstar=None):
        """(X n x 16, p_ref n, targets t or None)."""
        n = len(W)
        X = np.zeros((n, abi.MLP_FEATURES), np.float32)
        pref = np.zeros(n, np.float32)
        t = np.zeros(n, np.float32) if pstar is not None else None
        ps = None if pstar is None else np.ascontiguousarray(pstar, np.float64)
        abi.check(self.lib, self.lib.m2cg_mlp_features(n, abi.dptr(np.ascontiguousarray(W, np.float64)),
                                                       abi.dptr(np.ascontiguousarray(E, np.float64)), abi.dptr(ps),
                                                       abi.fptr(X), abi.fptr(pref), abi.fptr(t)),
                  "m2cg_mlp_features")
        return X, pref, t

    def set_data(self, W, E, pstar):
        abi.check(self.lib, self.lib.m2cg_mlp_set_data(self.h, len(W), abi.dptr(np.ascontiguousarray(W, np.float64)),
                                                       abi.dptr(np.ascontiguousarray(E, np.float64)),
                                                       abi.dptr(np.ascontiguousarray(pstar, np.float64))),
                  "m2cg_mlp_set_data")

    def train(self, epochs, batch=16384, lr=3e-3, seed=0):
        loss = np.zeros(max(epochs, 1), np.float32)
        ms = C.c_float()
        abi.check(self.lib, self.lib.m2cg_mlp_train(self.h, epochs, batch, lr, seed, abi.fptr(loss), C.byref(ms)),
                  "m2cg_mlp_train")
        return loss[:epochs], ms.value

    def grad(self, X, t):
        X = np.ascontiguousarray(X, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        g = np.zeros(abi.MLP_PARAMS, np.float32)
        loss = C.c_float()
        abi.check(self.lib, self.lib.m2cg_mlp_grad(self.h, len(t), abi.fptr(X), abi.fptr(t), abi.fptr(g),
                                                   C.byref(loss)), "m2cg_mlp_grad")
        return g, loss.value

    def adam_step(self, grad, lr):
        """One Adam update with the given gradient (the training loop's update)."""
        g = np.ascontiguousarray(grad, np.float32)
        assert g.shape == (abi.MLP_PARAMS,)
        abi.check(self.lib, self.lib.m2cg_mlp_adam_step(self.h, abi.fptr(g), float(lr)), "m2cg_mlp_adam_step")

    def forward(self, X):
        X = np.ascontiguousarray(X, np.float32)
        t = np.zeros(len(X), np.float32)
        abi.check(self.lib, self.lib.m2cg_mlp_forward(self.h, len(X), abi.fptr(X), abi.fptr(t)), "m2cg_mlp_forward")
        return t

    def predict(self, W, E):
        n = len(W)
        p = np.zeros(n)
        ms = C.c_float()
        abi.check(self.lib, self.lib.m2cg_mlp_predict(self.h, n, abi.dptr(np.ascontiguousarray(W, np.float64)),
                                                      abi.dptr(np.ascontiguousarray(E, np.float64)), abi.dptr(p),
                                                      C.byref(ms)), "m2cg_mlp_predict")
        return p, ms.value


def study(n_train=1 << 22, n_test=1 << 22, epochs=60, batch=16384, lr=3e-3, seed=2024, tol=1e-10, log=None,
          keep_net=False):
    """Label a training set, train the network, compare warm and cold starts on
    a test set.  With keep_net the trained WarmStartMLP is returned as well."""
    say = log or (lambda *a: None)
    solver = BatchSolver(tol)
    Wtr, Etr = sample_problems(n_train, seed)
    Wte, Ete = sample_problems(n_test, seed + 1)
    lab = solver.solve(Wtr, Etr)
    keep = (lab["err"] == 0) & (lab["pstar"] > 0)
    say(f"train labels: {keep.sum()} of {n_train} usable ({(lab['err'] != 0).sum()} failed solves), "
        f"{lab['ms']:.1f} ms")
    net = WarmStartMLP(seed)
    net.set_data(Wtr[keep], Etr[keep], lab["pstar"][keep])
    loss, train_ms = net.train(epochs, batch, lr, seed)
    say(f"trained {epochs} epochs in {train_ms / 1e3:.1f} s, loss {loss[0]:.3e} -> {loss[-1]:.3e}")
    cold = solver.solve(Wte, Ete)
    pred, pred_ms = net.predict(Wte, Ete)
    warm = solver.solve(Wte, Ete, warm_p=pred)
    ok = (cold["err"] == 0) & (cold["pstar"] > 0)
    rel = np.abs(pred[ok] - cold["pstar"][ok]) / cold["pstar"][ok]
    # the method without the network: the acoustic estimate the reference starts from
    p_ac, jump = acoustic_estimate(Wte, Ete)
    rel_ac = np.abs(p_ac[ok] - cold["pstar"][ok]) / cold["pstar"][ok]
    strong = jump[ok] > 0.05
    both = (cold["err"] == 0) & (warm["err"] == 0)
    dp = np.abs(warm["pstar"][both] - cold["pstar"][both]) / np.maximum(np.abs(cold["pstar"][both]), 1e-300)
    # device time on the problems both starts solve: the whole-set time is set
    # by the few failing solves, which run the reference's MaxIts twice
    sub_cold = solver.solve(Wte[both], Ete[both])
    sub_pred, sub_pred_ms = net.predict(Wte[both], Ete[both])
    sub_warm = solver.solve(Wte[both], Ete[both], warm_p=sub_pred)
    # the same solver started at the converged root: the bound on any predictor
    exact = solver.solve(Wte[both], Ete[both], warm_p=np.where(cold["pstar"][both] > 0, cold["pstar"][both], 0.0))
    res = {
        "n_train": int(n_train), "n_test": int(n_test), "tolerance": tol,
        "train_usable": int(keep.sum()), "epochs": epochs, "batch": batch, "lr": lr,
        "loss_first_epoch": float(loss[0]), "loss_last_epoch": float(loss[-1]), "train_s": train_ms / 1e3,
        "pstar_rel_err_median": float(np.median(rel)), "pstar_rel_err_p90": float(np.percentile(rel, 90)),
        "pstar_rel_err_p99": float(np.percentile(rel, 99)),
        "acoustic_rel_err_median": float(np.median(rel_ac)),
        # problems whose acoustic pressure jump exceeds 5 % of p_ref, where the solver uses the network
        "strong_fraction": float(strong.mean()),
        "pstar_rel_err_median_strong": float(np.median(rel[strong])) if strong.any() else 0.0,
        "acoustic_rel_err_median_strong": float(np.median(rel_ac[strong])) if strong.any() else 0.0,
        "iters_cold_mean": float(cold["iters"].mean()), "iters_warm_mean": float(warm["iters"].mean()),
        "iters_ratio": float(cold["iters"].mean() / max(warm["iters"].mean(), 1e-30)),
        # problems both starts solve (failures run to MaxIts twice either way)
        "iters_cold_mean_converged": float(cold["iters"][both].mean()),
        "iters_warm_mean_converged": float(warm["iters"][both].mean()),
        "solve_ms_cold": cold["ms"], "solve_ms_warm": warm["ms"], "predict_ms": pred_ms,
        "time_ratio": cold["ms"] / max(warm["ms"] + pred_ms, 1e-30),
        "failed_cold": int((cold["err"] != 0).sum()), "failed_warm": int((warm["err"] != 0).sum()),
        "warm_vs_cold_pstar_rel_median": float(np.median(dp)) if len(dp) else 0.0,
        "warm_vs_cold_pstar_rel_p99": float(np.percentile(dp, 99)) if len(dp) else 0.0,
        "warm_vs_cold_pstar_rel_max": float(dp.max()) if len(dp) else 0.0,
        "converged_set": {"n": int(both.sum()), "solve_ms_cold": sub_cold["ms"], "solve_ms_warm": sub_warm["ms"],
                          "predict_ms": sub_pred_ms,
                          "time_ratio": sub_cold["ms"] / max(sub_warm["ms"] + sub_pred_ms, 1e-30),
                          "iters_cold_mean": float(sub_cold["iters"].mean()),
                          "iters_warm_mean": float(sub_warm["iters"].mean()),
                          "iters_exact_start_mean": float(exact["iters"].mean()),
                          "solve_ms_exact_start": exact["ms"]},
    }
    solver.close()
    if keep_net:
        return res, net
    net.close()
    return res
