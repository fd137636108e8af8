"""Boundary conditions on the GPU against the oracle
(SpaceOperator::ApplyBoundaryConditions, SpaceOperator.cpp:738-821, and the
ghost face states of Reconstructor.cpp:807-889): SlipWall (normal velocity
flipped), StickWall (every velocity component flipped) and Inlet2 (the
second inlet state), on a two-material box whose flow reaches every
boundary, one step at 1e-10 and ten steps at 1e-8."""
import numpy as np
import pytest

from m2c_gb300 import abi, problems
from m2c_gb300.solver import FluidState, Solver
from oracle import binding as ob
from oracle import parity

pytestmark = pytest.mark.gpu

LAYOUTS = {
    "slipwall": (abi.BC_INLET2, abi.BC_SLIPWALL, abi.BC_SLIPWALL, abi.BC_SLIPWALL, abi.BC_SLIPWALL, abi.BC_SLIPWALL),
    "stickwall": (abi.BC_STICKWALL, abi.BC_STICKWALL, abi.BC_STICKWALL, abi.BC_STICKWALL, abi.BC_OUTLET,
                  abi.BC_INLET2),
    "mixed": (abi.BC_INLET2, abi.BC_STICKWALL, abi.BC_SLIPWALL, abi.BC_STICKWALL, abi.BC_SLIPWALL, abi.BC_OUTLET),
}


def _case(layout, n=16, seed=3):
    cfg, V, ID, phi = problems.shock_bubble(n=n)
    for s, b in enumerate(LAYOUTS[layout]):
        cfg.bc[s] = b
    for p, v in enumerate((1100.0, 40.0, -15.0, 25.0, 3.0e8)):
        cfg.inlet2[p] = v
    rng = np.random.default_rng(seed)
    V[:, 1:4] += rng.uniform(-30, 30, (len(V), 3))   # flow through and along every wall
    return cfg, V, ID, phi


@pytest.mark.parametrize("layout", sorted(LAYOUTS))
@pytest.mark.parametrize("nsteps,tol", [(1, 1e-10), (10, 1e-8)])
def test_boundary_conditions_match_oracle(layout, nsteps, tol):
    cfg, V, ID, phi = _case(layout)
    g = Solver(cfg, FluidState(V, ID, phi))
    o = ob.OracleSim(cfg)
    o.upload(V, ID, phi)
    if nsteps == 1:
        R, Ro = g.ComputeResidual(), o.residual()
        assert np.all(parity.velocity_normalized(R, Ro) < 1e-10)
    g.run(nsteps)
    o.run(nsteps)
    s = g.get_state()
    Vo, IDo, pho = o.download()
    cmp = parity.compare(s.V, s.ID, s.Phi, Vo, IDo, pho, (cfg.nz, cfg.ny, cfg.nx))
    assert cmp["ids_equal"]
    assert max(cmp["rel_linf_velocity_magnitude"].values()) < tol, cmp
    assert cmp["phi_rel_linf"] < tol
    cg, co = g.counters(), o.counters()
    for k in ("interface_faces", "riemann_solves", "swept_cells", "clipped_faces", "nonphysical"):
        assert cg[k] == co[k], (k, cg[k], co[k])
    g.close()
