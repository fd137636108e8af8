"""Batched ensemble of uneven domains: every member, advanced with the others
in one launch per kernel and stage, ends bit for bit where the same domain
advanced alone ends (same arithmetic per cell and face, each member with its
own CFL step); the sequential baseline agrees too."""
import numpy as np
import pytest

from m2c_gb300 import abi, problems
from m2c_gb300.ensemble import Ensemble
from m2c_gb300.solver import FluidState, Solver

SMALL = [(16, 24, 20, 0.25, 1e7), (24, 16, 16, 0.2, 3e6), (20, 20, 28, 0.3, 1e8), (32, 16, 24, 0.15, 1e6),
         (16, 16, 16, 0.3, 5e7)]
KEYS = ("interface_faces", "riemann_solves", "riemann_iterations", "riemann_errors", "swept_cells",
        "clipped_cells", "nonphysical")


def test_ensemble_problem_shapes():
    doms = problems.bubble_collapse_ensemble(64, seed=3)
    for c, V, ID, phi in doms:
        assert c.nx in problems.EDGES and c.ny in problems.EDGES and c.nz in problems.EDGES
        n = c.nx * c.ny * c.nz
        assert V.shape == (n, 5) and ID.shape == (n,) and phi.shape == (n,)
        assert 0 < ID.sum() < n
        pw = V[ID == 0, 4][0]
        assert 1e6 <= pw <= 1e8 and np.all(V[ID == 1, 4] == 1e4)


@pytest.mark.gpu
@pytest.mark.parametrize("normal", [abi.RNORMAL_MESH, abi.RNORMAL_AVERAGE])
def test_ensemble_matches_members_run_alone(normal):
    doms = [problems.bubble_collapse(*d) for d in SMALL]
    for d in doms:
        d[0].mp_riemann_normal = normal   # interface normals from each member's own level set
    ens = Ensemble([d[0] for d in doms])
    for i, (c, V, ID, phi) in enumerate(doms):
        ens.member(i).set_state(FluidState(V, ID, phi))
    ens.run(3)
    ens.run(3)   # the graph replayed
    seq = Ensemble([d[0] for d in doms])
    for i, (c, V, ID, phi) in enumerate(doms):
        seq.member(i).set_state(FluidState(V, ID, phi))
    seq.run_sequential(6)
    for i, (c, V, ID, phi) in enumerate(doms):
        solo = Solver(c, FluidState(V, ID, phi))
        solo.run(6)
        a, b, q = ens.member(i).get_state(), solo.get_state(), seq.member(i).get_state()
        for x in (a, q):
            assert np.array_equal(x.ID, b.ID), i
            assert np.array_equal(x.V, b.V), i
            assert np.array_equal(x.Phi, b.Phi), i
        ca, cb = ens.member(i).counters(), solo.counters()
        for k in KEYS:
            assert ca[k] == cb[k], (i, k, ca[k], cb[k])
        assert cb["riemann_solves"] > 0
        solo.close()
    # and every member against the oracle directly
    from oracle import binding as ob
    from oracle import parity
    for i, (c, V, ID, phi) in enumerate(doms):
        o = ob.OracleSim(c)
        o.upload(V, ID, phi)
        o.run(6)
        Vo, IDo, po = o.download()
        a = ens.member(i).get_state()
        np.testing.assert_array_equal(a.ID, IDo)
        assert np.all(parity.velocity_normalized(a.V, Vo) < 1e-8), i
        assert parity.rel_linf(a.Phi, po) < 1e-8, i
    assert ens.kernel_launches() > 0
    ens.close()
    seq.close()


@pytest.mark.gpu
def test_autotuned_ensemble_matches_members_run_alone():
    """The autotuner's candidate budgets change the interface solves' schedule,
    not their results: after tuning (whose trial steps are real steps) every
    member ends bit for bit where it ends advanced alone."""
    doms = [problems.bubble_collapse(*d) for d in SMALL]
    ens = Ensemble([d[0] for d in doms])
    for i, (c, V, ID, phi) in enumerate(doms):
        ens.member(i).set_state(FluidState(V, ID, phi))
    budgets = (2, 8, 1 << 20)
    best, ms = ens.autotune(steps=1, budgets=budgets)
    assert best in budgets and ms > 0
    ens.run(2)   # 3 tuning steps + 2
    for i, (c, V, ID, phi) in enumerate(doms):
        solo = Solver(c, FluidState(V, ID, phi))
        solo.run(5)
        a, b = ens.member(i).get_state(), solo.get_state()
        assert np.array_equal(a.ID, b.ID), i
        assert np.array_equal(a.V, b.V), i
        assert np.array_equal(a.Phi, b.Phi), i
        solo.close()
    ens.close()


@pytest.mark.gpu
def test_tile_shapes_change_the_schedule_not_the_results():
    """The persistent batched kernels under every block shape the tile
    autotuner tries: after tuning (whose trial steps are real steps) every
    member ends bit for bit where it ends advanced alone, and the chosen shape
    is one of the candidates for every size class."""
    doms = [problems.bubble_collapse(*d) for d in SMALL]
    ens = Ensemble([d[0] for d in doms])
    for i, (c, V, ID, phi) in enumerate(doms):
        ens.member(i).set_state(FluidState(V, ID, phi))
    shapes = Ensemble.TILE_SHAPES
    chosen, ms = ens.autotune_tiles(steps=1, shapes=shapes)
    assert ms > 0 and set(chosen) == {d[0].nx for d in doms}
    assert all(s in shapes for s in chosen.values())
    ntrial = len(set(chosen)) * len(shapes)
    ens.run(2)
    for i, (c, V, ID, phi) in enumerate(doms):
        solo = Solver(c, FluidState(V, ID, phi))
        solo.run(ntrial + 2)
        a, b = ens.member(i).get_state(), solo.get_state()
        assert np.array_equal(a.ID, b.ID), i
        assert np.array_equal(a.V, b.V), i
        assert np.array_equal(a.Phi, b.Phi), i
        solo.close()
    ens.close()
