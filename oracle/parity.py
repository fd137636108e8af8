"""Parity metrics between the product's state and the oracle's (test
infrastructure only: used by tests/ and by bench.py's CPU-baseline leg).

rel_linf per variable is max|a - b| / max|b| over all real cells.  Two
refinements are reported beside it, never instead of it:
  * velocity components relative to the largest velocity magnitude (a
    component that stays near zero everywhere -- v, w of a planar shock --
    would otherwise be compared on rounding noise);
  * the same metric over the bulk (cells whose face neighbours all carry the
    cell's own material) and over the interface band (the rest), which
    separates the near-trivial interface Riemann problems -- whose outcome
    follows the last bits of their inputs -- from everything else.
"""
import numpy as np

NAMES = ("rho", "u", "v", "w", "p")


def rel_linf(a, b, axis=0):
    a, b = np.asarray(a), np.asarray(b)
    den = np.abs(b).max(axis=axis)
    num = np.abs(a - b).max(axis=axis)
    return np.where(den > 0, num / np.where(den > 0, den, 1), num)


def velocity_normalized(a, b):
    """rel_linf with u, v, w divided by the largest velocity magnitude of b."""
    e = rel_linf(a, b)
    vmax = np.sqrt((b[:, 1:4] ** 2).sum(1)).max()
    if vmax > 0:
        e[1:4] = np.abs(a[:, 1:4] - b[:, 1:4]).max(0) / vmax
    return e


def interface_band(ID, shape):
    """Cells with a face neighbour of another material (shape = (nz, ny, nx))."""
    I = ID.reshape(shape)
    band = np.zeros(shape, bool)
    for ax in range(3):
        d = np.diff(I, axis=ax) != 0
        lo = [slice(None)] * 3
        hi = [slice(None)] * 3
        lo[ax] = slice(0, -1)
        hi[ax] = slice(1, None)
        band[tuple(lo)] |= d
        band[tuple(hi)] |= d
    return band.ravel()


def compare(V, ID, phi, Vo, IDo, phio, shape):
    """All parity figures of one checkpoint as a JSON-ready dict."""
    out = {"rel_linf": dict(zip(NAMES, map(float, rel_linf(V, Vo)))),
           "rel_linf_velocity_magnitude": dict(zip(NAMES, map(float, velocity_normalized(V, Vo)))),
           "phi_rel_linf": float(rel_linf(phi, phio)),
           "ids_equal": bool(np.array_equal(ID, IDo)), "id_cells_differing": int((ID != IDo).sum())}
    band = interface_band(IDo, shape)
    den = np.abs(Vo).max(0)
    vden = den.copy()
    vden[1:4] = np.sqrt((Vo[:, 1:4] ** 2).sum(1)).max()
    for name, m in (("bulk", ~band), ("interface_band", band)):
        if m.any():
            num = np.abs(V[m] - Vo[m]).max(0)
            out[f"rel_linf_{name}"] = dict(zip(NAMES, map(float, num / np.where(den > 0, den, 1))))
            out[f"rel_linf_{name}_velocity_magnitude"] = dict(zip(NAMES, map(float, num / np.where(vden > 0, vden, 1))))
            out[f"cells_{name}"] = int(m.sum())
    return out


COUNTERS = ("interface_faces", "riemann_solves", "riemann_iterations", "riemann_errors", "swept_cells",
            "clipped_cells", "clipped_faces", "nonphysical", "unresolved_cells")


def counters_pair(cg, co):
    return {k: {"gpu": int(cg[k]), "oracle": int(co[k]), "diff": int(cg[k]) - int(co[k])} for k in COUNTERS}


TOTALS = ("mass", "momentum_x", "momentum_y", "momentum_z", "total_energy")


def totals_dict(t0, t, ref=None):
    """Conserved totals sum(U vol) now, their change since t0 relative to |t0|
    (or to the largest component for momentum), and the relative difference
    from the oracle's totals."""
    t0, t = np.asarray(t0), np.asarray(t)
    scale = np.abs(t0).copy()
    scale[1:4] = max(np.abs(t0[1:4]).max(), np.abs(t[1:4]).max(), 1e-300)
    out = {"totals": dict(zip(TOTALS, map(float, t))),
           "drift": dict(zip(TOTALS, map(float, (t - t0) / np.where(scale > 0, scale, 1))))}
    if ref is not None:
        ref = np.asarray(ref)
        rs = np.abs(ref).copy()
        rs[1:4] = max(np.abs(ref[1:4]).max(), 1e-300)
        out["rel_diff_from_oracle"] = dict(zip(TOTALS, map(float, np.abs(t - ref) / np.where(rs > 0, rs, 1))))
    return out
