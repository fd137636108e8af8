"""CPU reference of the warm-start network (test helper): features, forward and
backward in float64, with the same BF16 roundings as the GPU kernels -- the
network input, the hidden activations fed to the next GEMM and the
pre-activation gradients fed to the backward GEMMs are rounded to BF16; biases,
the head, the loss and the bias / head gradients stay in full precision.
"""
import numpy as np

NF, NH = 16, 64
OFF_W1 = 0
OFF_B1 = OFF_W1 + NH * NF
OFF_W2 = OFF_B1 + NH
OFF_B2 = OFF_W2 + NH * NH
OFF_W3 = OFF_B2 + NH
OFF_B3 = OFF_W3 + NH * NH
OFF_W4 = OFF_B3 + NH
OFF_B4 = OFF_W4 + NH
NPARAM = OFF_B4 + 1

BLOCKS = {"W1": (OFF_W1, OFF_B1), "b1": (OFF_B1, OFF_W2), "W2": (OFF_W2, OFF_B2), "b2": (OFF_B2, OFF_W3),
          "W3": (OFF_W3, OFF_B3), "b3": (OFF_B3, OFF_W4), "w4": (OFF_W4, OFF_B4), "b4": (OFF_B4, NPARAM)}


def bf16(x):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    x = np.ascontiguousarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def unpack(p):
    p = np.asarray(p, np.float64)
    return dict(W1=p[OFF_W1:OFF_B1].reshape(NH, NF), b1=p[OFF_B1:OFF_W2], W2=p[OFF_W2:OFF_B2].reshape(NH, NH),
                b2=p[OFF_B2:OFF_W3], W3=p[OFF_W3:OFF_B3].reshape(NH, NH), b3=p[OFF_B3:OFF_W4],
                w4=p[OFF_W4:OFF_B4], b4=p[OFF_B4])


def forward_backward(p, X, t, rounding=True):
    """Mean squared error of the output against t; returns (out, loss, grad)."""
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    q = unpack(p)
    W1, W2, W3 = r(q["W1"]), r(q["W2"]), r(q["W3"])
    X = r(X)
    Z1 = X @ W1.T + q["b1"]
    H1 = r(silu(Z1))
    Z2 = H1 @ W2.T + q["b2"]
    H2 = r(silu(Z2))
    Z3 = H2 @ W3.T + q["b3"]
    h3 = silu(Z3)
    out = h3 @ q["w4"] + q["b4"]
    n = len(t)
    e = out - np.asarray(t, np.float64)
    loss = float(np.mean(e * e))
    d = 2.0 * e / n
    g = np.zeros(NPARAM)
    dZ3 = d[:, None] * q["w4"][None, :] * dsilu(Z3)
    g[OFF_B3:OFF_W4] = dZ3.sum(0)
    g[OFF_W4:OFF_B4] = (d[:, None] * h3).sum(0)
    g[OFF_B4] = d.sum()
    dZ3 = r(dZ3)
    g[OFF_W3:OFF_B3] = (dZ3.T @ H2).ravel()
    dZ2 = (dZ3 @ W3) * dsilu(Z2)
    g[OFF_B2:OFF_W3] = dZ2.sum(0)
    dZ2 = r(dZ2)
    g[OFF_W2:OFF_B2] = (dZ2.T @ H1).ravel()
    dZ1 = (dZ2 @ W2) * dsilu(Z1)
    g[OFF_B1:OFF_W2] = dZ1.sum(0)
    dZ1 = r(dZ1)
    g[OFF_W1:OFF_B1] = (dZ1.T @ X).ravel()
    return out, loss, g


def features(W, E):
    """Network inputs (n x 16, BF16-rounded) and p_ref of problems W (n x 6), E (n x 10)."""
    rl, ul, pl = W[:, 0], W[:, 1], np.maximum(W[:, 2], 1.0)
    rr, ur, pr = W[:, 3], W[:, 4], np.maximum(W[:, 5], 1.0)
    gl, pcl, bl = E[:, 1], E[:, 2], E[:, 3]
    gr, pcr, br = E[:, 6], E[:, 7], E[:, 8]
    c2l = gl * (pl + pcl) / (rl * (1.0 - bl * rl))
    c2r = gr * (pr + pcr) / (rr * (1.0 - br * rr))
    c2l = np.where(c2l > 0, c2l, 1.0)
    c2r = np.where(c2r > 0, c2r, 1.0)
    Cl, Cr = rl * np.sqrt(c2l), rr * np.sqrt(c2r)
    pref = (Cr * pl + Cl * pr) / (Cl + Cr)
    a = (ul - ur) * Cl * Cr / ((Cl + Cr) * pref)
    f = [np.arcsinh(a) * 0.25, np.log(pl / pref) * 0.25, np.log(pr / pref) * 0.25, np.log(Cl / Cr) * 0.25,
         (gl - 4.0) / 1.7, (gr - 4.0) / 1.7, np.arcsinh(pcl / pref) * 0.125, np.arcsinh(pcr / pref) * 0.125,
         2.0 * bl * rl - 1.0, 2.0 * br * rr - 1.0, np.log(rl * c2l / pref) * 0.25, np.log(rr * c2r / pref) * 0.25]
    X = np.zeros((len(W), NF))
    for i, v in enumerate(f):
        X[:, i] = np.asarray(v, np.float32)
    return bf16(X), pref
