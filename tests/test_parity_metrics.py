"""The parity metrics (oracle/parity.py) that the bench's parity leg and the
scale tests report, checked on small hand-made states (CPU)."""
import numpy as np

from oracle import parity


def test_rel_linf_is_per_variable_max_over_max():
    b = np.array([[1.0, 2.0], [4.0, -8.0]])
    a = b + np.array([[0.5, 0.0], [0.0, 0.4]])
    np.testing.assert_allclose(parity.rel_linf(a, b), [0.5 / 4.0, 0.4 / 8.0])
    # a variable that is zero in b: the absolute difference
    np.testing.assert_allclose(parity.rel_linf(np.array([[0.0, 1e-3]]), np.array([[0.0, 0.0]])), [0.0, 1e-3])


def test_velocity_normalized_uses_the_largest_speed():
    b = np.zeros((2, 5))
    b[:, 0] = 1.0
    b[:, 4] = 10.0
    b[0, 1:4] = [3.0, 4.0, 0.0]   # speed 5
    a = b.copy()
    a[1, 3] = 1e-6                # w is zero everywhere in b
    e = parity.velocity_normalized(a, b)
    assert e[3] == 1e-6 / 5.0 and e[0] == 0.0 and e[4] == 0.0
    assert parity.rel_linf(a, b)[3] == 1e-6   # the plain metric compares against 0


def test_interface_band_marks_both_sides_of_every_material_face():
    ID = np.zeros((3, 4, 5), np.int32)
    ID[1, 2, 3] = 1
    band = parity.interface_band(ID.ravel(), ID.shape).reshape(ID.shape)
    expect = np.zeros_like(band)
    expect[1, 2, 3] = True
    for dz, dy, dx in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)):
        expect[1 + dz, 2 + dy, 3 + dx] = True
    np.testing.assert_array_equal(band, expect)


def test_compare_splits_bulk_and_interface_band():
    rng = np.random.default_rng(0)
    shape = (4, 4, 4)
    n = 64
    Vo = np.column_stack([rng.uniform(1, 2, n), rng.uniform(-1, 1, (n, 3)), rng.uniform(1e5, 2e5, n)])
    IDo = np.zeros(n, np.int32)
    IDo[21] = 1                      # one cell of another material
    V = Vo.copy()
    V[21, 0] *= 1 + 1e-9             # the interface cell differs
    out = parity.compare(V, IDo, np.zeros(n), Vo, IDo, np.zeros(n), shape)
    assert out["ids_equal"] and out["id_cells_differing"] == 0
    assert out["rel_linf_bulk"]["rho"] == 0.0
    assert out["rel_linf_interface_band"]["rho"] > 0.0
    assert out["cells_bulk"] + out["cells_interface_band"] == n


def test_totals_drift_and_difference():
    t0 = np.array([10.0, 1.0, -2.0, 0.5, 100.0])
    t = t0 + np.array([1e-12, 0.0, 2e-3, 0.0, -1e-9])
    out = parity.totals_dict(t0, t, ref=t0)
    assert abs(out["drift"]["mass"] - 1e-13) < 1e-16      # 10 + 1e-12 carries an ulp of 10
    assert abs(out["drift"]["momentum_y"] - 1e-3) < 1e-15   # momentum relative to the largest component
    assert abs(out["rel_diff_from_oracle"]["total_energy"] - 1e-11) < 1e-15
