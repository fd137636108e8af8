"""Shared test helpers: golden-case configs and parity metrics."""
import json
import os

import numpy as np

from m2c_gb300 import abi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_riemann_cases():
    return json.load(open(os.path.join(GOLDEN, "riemann_star_states.json")))


def config_for_materials(mats, tol=1e-10):
    c = abi.default_config()
    c.n_materials = len(mats)
    for i, m in enumerate(mats):
        if m["eos"] == "SG":
            abi.set_material(c.mat[i], abi.EOS_SG, gamma=m["gamma"], pc=m["pc"])
        elif m["eos"] == "NASG":
            abi.set_material(c.mat[i], abi.EOS_NASG, gamma=m["gamma"], pc=m["pc"], b=m["b"], q=m["q"])
        else:
            abi.set_material(c.mat[i], abi.EOS_MG, rho0=m["rho0"], c0=m["c0"], Gamma0=m["Gamma0"], s=m["s"], e0=m["e0"])
        if m.get("pmin") is not None:
            c.mat[i].pmin = m["pmin"]
        if m.get("rhomin") is not None:
            c.mat[i].rhomin = m["rhomin"]
    c.tol_main = tol
    return c


def golden_problem(case):
    Vm = np.array([[case["left"][0], case["left"][1], 0.0, 0.0, case["left"][2]]])
    Vp = np.array([[case["right"][0], case["right"][1], 0.0, 0.0, case["right"][2]]])
    return Vm, np.array([case["idl"]]), Vp, np.array([case["idr"]]), np.array([[1.0, 0.0, 0.0]])


def rel_linf(a, b, axis=0):
    """max|a-b| / max|b| per variable (the parity metric)."""
    a, b = np.asarray(a), np.asarray(b)
    den = np.abs(b).max(axis=axis)
    num = np.abs(a - b).max(axis=axis)
    return np.where(den > 0, num / np.where(den > 0, den, 1), num)


def random_sg_states(rng, n, nmat=2):
    """Random physical primitive states for stiffened-gas materials."""
    rho = 10 ** rng.uniform(-1, 3.3, n)
    u = rng.uniform(-500, 500, n)
    v = rng.uniform(-100, 100, n)
    w = rng.uniform(-100, 100, n)
    p = 10 ** rng.uniform(4, 10, n)
    return np.stack([rho, u, v, w, p], 1)
