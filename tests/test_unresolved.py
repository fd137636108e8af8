"""Unresolved swept cells (TimeIntegrator.cpp:776-797): a cell whose material
ID changed in a step but that neither an interface Riemann solution nor an
extrapolation from same-material neighbours could fill.  With a reinitializer
configured the reference makes such cells' phi negative, reinitializes the
level set, moves the IDs with the sign changes and fills the cells by
MultiPhaseOperator::FixUnresolvedNodes (MultiPhaseOperator.cpp:1279-1480).

The case puts two planes of cells exactly on the zero set of phi in a uniform
flow in +x, with IDs that disagree with phi's sign next to the planes, so that
the first step leaves a known set of unresolved cells and reaches every branch
of the repair:
  * plane i = 5 (phi 0 -> -u dt, ID 0 -> 1, the level set's material): only
    rows j = 3, 4 touch an ID-1 column (i = 4), through a face; the others
    have no interface face, so they stay unresolved and take the upwind mean
    (rows 2, 5), the layered density (rows up to 14) or, 11 rows away from any
    ID-1 cell, the failsafe density (row 15);
  * plane i = 20 (phi 0 -> +u dt) inside an ID-1 block: the "remaining" cell
    has no other material around and becomes material 0 with no interface
    face; the repair flips its phi, the ID update returns it to material 1
    and it takes the upwind mean of its ID-1 neighbours."""
import numpy as np
import pytest

from helpers import rel_linf
from m2c_gb300 import abi
from oracle import binding as ob

NX, NY, NZ = 24, 16, 3
IC, IC2 = 5, 20


def unresolved_case(phase_change=abi.PHASECHANGE_RIEMANN, pcdir=abi.PCDIR_UPWIND, reinit=True):
    c = abi.default_config()
    c.nx, c.ny, c.nz = NX, NY, NZ
    h = 1.0 / 16.0
    c.x0, c.xmax = 0.0, NX * h
    c.y0, c.ymax = 0.0, NY * h
    c.z0, c.zmax = 0.0, NZ * h
    for s in range(6):
        c.bc[s] = abi.BC_OUTLET
    c.n_materials = 2
    abi.set_material(c.mat[0], abi.EOS_SG, gamma=6.12, pc=3.43e8)   # water
    abi.set_material(c.mat[1], abi.EOS_SG, gamma=1.4, pc=0.0)       # gas
    c.flux = abi.FLUX_HLLC
    c.rec_type = abi.REC_LINEAR
    c.limiter = abi.LIM_VANALBADA
    c.tol_main = 1e-10
    c.n_levelsets, c.ls_matid = 1, 1
    c.ts_type = abi.TS_RK2
    c.cfl = 0.4
    c.mp_phasechange = phase_change
    c.mp_phasechange_dir = pcdir
    if reinit:
        c.reinit_frequency = 1000   # configured, not due in the test's steps
    n = NX * NY * NZ
    K, J, I = np.meshgrid(np.arange(NZ), np.arange(NY), np.arange(NX), indexing="ij")
    I, J = I.ravel(), J.ravel()
    phi = np.minimum(I - IC, IC2 - I) * h     # exact multiples of h: 0 on both planes
    ID = np.zeros(n, np.int32)
    ID[(I == IC - 1) & ((J == 3) | (J == 4))] = 1
    ID[I >= IC2 - 1] = 1
    V = np.zeros((n, 5))
    V[:, 0] = np.where(ID == 1, 1.2, 1000.0)
    V[:, 1] = 50.0
    V[:, 4] = 1.0e5
    return c, V, ID, phi, I, J


def cells(I, J, i, js):
    return (I == i) & np.isin(J, js)


def test_oracle_repairs_unresolved_cells():
    c, V, ID, phi, I, J = unresolved_case()
    o = ob.OracleSim(c)
    o.upload(V, ID, phi)
    o.run(1)
    cnt = o.counters()
    Vo, IDo, phio = o.download()
    n_expect = (NY - 2) * NZ + NY * NZ
    assert cnt["unresolved_cells"] == n_expect
    assert cnt["unresolved_fixed"] == n_expect
    assert o.reinitialize()[1]["calls"] == 2   # the forced call and this one
    # the plane that went to material 0 without an interface is back in material 1
    p2 = cells(I, J, IC2, range(NY))
    assert np.all(IDo[p2] == 1) and np.all(phio[p2] < 0)
    # upwind means of gas neighbours: gas densities (the reset flag makes later
    # cells add their neighbours onto their own advected state, so the value is
    # not 1.2 itself)
    assert np.all(np.isfinite(Vo)) and np.all(Vo[p2, 0] > 0)
    # plane i = 5: material 1 everywhere; rows 0..14 filled from gas cells,
    # row 15 has no gas cell within 10 layers: failsafe density
    p1 = cells(I, J, IC, range(NY))
    assert np.all(IDo[p1] == 1)
    far = cells(I, J, IC, [15])
    assert np.all(Vo[far, 0] == c.mat[1].failsafe_density)
    layered = cells(I, J, IC, range(7, 15))
    assert np.all(np.abs(Vo[layered, 0] - 1.2) < 0.1)
    # velocity and pressure of the layered / failsafe cells stay as advected
    assert np.all(np.abs(Vo[far | layered, 4] / 1e5 - 1.0) < 1e-3)


def test_oracle_without_reinitializer_leaves_cells_as_advected():
    c, V, ID, phi, I, J = unresolved_case(reinit=False)
    o = ob.OracleSim(c)
    o.upload(V, ID, phi)
    o.run(1)
    cnt = o.counters()
    Vo, IDo, _ = o.download()
    assert cnt["unresolved_cells"] == (NY - 2) * NZ + NY * NZ and cnt["unresolved_fixed"] == 0
    assert np.all(IDo[cells(I, J, IC2, range(NY))] == 0)
    far = cells(I, J, IC, [15])
    assert np.all(np.abs(Vo[far, 0] / 1000.0 - 1.0) < 1e-3)   # water state under a gas ID


def test_oracle_extrapolation_path_repairs_the_rest():
    c, V, ID, phi, I, J = unresolved_case(phase_change=abi.PHASECHANGE_EXTRAPOLATION)
    o = ob.OracleSim(c)
    o.upload(V, ID, phi)
    o.run(1)
    cnt = o.counters()
    # rows 2..5 of plane 5 extrapolate from the ID-1 column; the rest do not
    assert cnt["unresolved_cells"] == (NY - 4) * NZ + NY * NZ == cnt["unresolved_fixed"]


@pytest.mark.gpu
@pytest.mark.parametrize("variant", ["riemann-upwind", "riemann-all", "extrapolation-upwind", "no-reinit"])
def test_gpu_repair_matches_oracle(variant):
    from m2c_gb300.solver import FluidState, Solver
    kw = {"riemann-upwind": {}, "riemann-all": {"pcdir": abi.PCDIR_ALL},
          "extrapolation-upwind": {"phase_change": abi.PHASECHANGE_EXTRAPOLATION},
          "no-reinit": {"reinit": False}}[variant]
    c, V, ID, phi, I, J = unresolved_case(**kw)
    o = ob.OracleSim(c)
    o.upload(V, ID, phi)
    o.run(1)
    s = Solver(c, FluidState(V, ID, phi))
    cnt = s.run(1)
    co = o.counters()
    g = s.get_state()
    Vo, IDo, phio = o.download()
    for k in ("unresolved_cells", "unresolved_fixed", "swept_cells"):
        assert cnt[k] == co[k], (k, cnt[k], co[k])
    np.testing.assert_array_equal(g.ID, IDo)
    assert rel_linf(g.Phi, phio) < 1e-10
    # densities span 1e-10 .. 1e3: each cell against its own scale; the
    # interface Riemann solves converge to 1e-10, so the bound is 1e-8
    rel = np.abs(g.V - Vo) / np.maximum(np.abs(Vo), 1e-300)
    worst = int(np.argmax(rel[:, 0]))
    assert rel[:, 0].max() <= 1e-8, (worst, g.V[worst], Vo[worst])
    # stiffened-gas pressure p = (gamma - 1) rho e - gamma p_inf: at 1e5 Pa in
    # water (p_inf 3.43e8) it carries the internal energy's error times
    # (p + gamma p_inf) / p, so it is compared on the scale p + p_inf
    pinf = np.array([c.mat[m].pc for m in range(c.n_materials)])[IDo]
    assert (np.abs(g.V[:, 4] - Vo[:, 4]) / (np.abs(Vo[:, 4]) + pinf)).max() <= 1e-8
    # velocities on the acoustic scale of the water (about 1.5e3 m/s)
    assert np.abs(g.V - Vo)[:, 1:4].max() <= 1e-8 * 1.5e3
    if variant != "no-reinit":
        assert s.reinit_stats()["calls"] == o.reinitialize()[1]["calls"] - 1 == 1
