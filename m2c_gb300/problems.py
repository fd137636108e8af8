"""Problem set-ups with the shapes of the benchmark workloads: configuration
(IoData-equivalent fields) plus the initial FluidState {V, ID, phi}.

Geometry follows the reference's initializer conventions: a level set is
negative inside the material it tracks (SpaceInitializer.cpp:1407-1428), a
plane's signed distance is (x - x0).n with n normalized
(GeoTools/DistancePointToPlane.h:23-41).
"""
import numpy as np

from . import abi


def cell_centers(cfg):
    dx = (cfg.xmax - cfg.x0) / cfg.nx
    dy = (cfg.ymax - cfg.y0) / cfg.ny
    dz = (cfg.zmax - cfg.z0) / cfg.nz
    # MeshGenerator.cpp:166-171: x_i = x0 + 0.5h + i*h
    x = cfg.x0 + 0.5 * dx + np.arange(cfg.nx) * dx
    y = cfg.y0 + 0.5 * dy + np.arange(cfg.ny) * dy
    z = cfg.z0 + 0.5 * dz + np.arange(cfg.nz) * dz
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")   # k-major, then j, then i
    return X.ravel(), Y.ravel(), Z.ravel()


def uniform_noise(n, seed):
    """Seeded uniform [-1, 1) per global cell index (splitmix64 of index and seed)."""
    with np.errstate(over="ignore"):
        z = (np.arange(n, dtype=np.uint64) + np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15)) \
            * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (2.0 / 2.0 ** 53) - 1.0


def sg_post_shock(rho1, p1, u1, p2, gamma, pinf):
    """Post-shock state behind a right-moving shock into (rho1, p1, u1) for a
    stiffened gas: Rankine-Hugoniot density ratio and piston velocity."""
    a, b = p2 + pinf, p1 + pinf
    ratio = ((gamma + 1) * a + (gamma - 1) * b) / ((gamma - 1) * a + (gamma + 1) * b)
    rho2 = rho1 * ratio
    u2 = u1 + np.sqrt((p2 - p1) * (1.0 / rho1 - 1.0 / rho2))
    return rho2, u2


def riemann1d(nx=256, ny=8, nz=8):
    """Quasi-1D two-material Riemann problem: gas (SG 1.4, rho 1.2, p 1e9) for
    x < 0.5 tracked by the level set phi = x - 0.5 (Plane at x = 0.5, normal -x),
    water (SG 6.12, p_inf 3.43e8, rho 1000, p 1e5) elsewhere.  MUSCL / van Albada,
    HLLC, exact interface Riemann solver at 1e-10, RK2, CFL 0.5.
    Boundary conditions: Outlet in x, Symmetry in y and z."""
    c = abi.default_config()
    c.nx, c.ny, c.nz = nx, ny, nz
    c.x0, c.xmax = 0.0, 1.0
    c.y0, c.ymax = 0.0, 0.03125 * ny / 8.0
    c.z0, c.zmax = 0.0, 0.03125 * nz / 8.0
    c.bc[0] = c.bc[1] = abi.BC_OUTLET
    for s in range(2, 6):
        c.bc[s] = abi.BC_SYMMETRY
    c.n_materials = 2
    abi.set_material(c.mat[0], abi.EOS_SG, gamma=6.12, pc=3.43e8)   # water
    abi.set_material(c.mat[1], abi.EOS_SG, gamma=1.4, pc=0.0)       # gas
    c.flux = abi.FLUX_HLLC
    c.rec_type = abi.REC_LINEAR
    c.limiter = abi.LIM_VANALBADA
    c.tol_main = 1e-10
    c.n_levelsets, c.ls_matid = 1, 1
    c.ts_type = abi.TS_RK2
    c.cfl = 0.5
    X, Y, Z = cell_centers(c)
    n = X.size
    phi = X - 0.5
    gas = phi < 0
    V = np.zeros((n, 5))
    V[:, 0] = np.where(gas, 1.2, 1000.0)
    V[:, 4] = np.where(gas, 1.0e9, 1.0e5)
    ID = gas.astype(np.int32)
    return c, V, ID, phi


def shock_bubble(n=256, seed=2024, radius=0.15, noise=0.01):
    """3D shock-bubble: gas bubble (SG 1.4, rho 1.2, p 1e5) of radius 0.15 at the
    centre of [0,1]^3 in water (SG 6.12, p_inf 3.43e8, rho 1000, p 1e5); water
    for x < 0.1 carries the post-shock state of a 1e9 Pa shock (Rankine-Hugoniot);
    per-cell density times (1 + 0.01 U[-1,1)) from a seeded generator indexed by
    global cell id; phi = |x - c| - r.  MUSCL / van Albada, HLLC, exact interface
    Riemann solver at 1e-10, RK2, CFL 0.4.  Boundary conditions: Inlet (post-shock
    state) at x0, Outlet at xmax, Symmetry in y and z."""
    c = abi.default_config()
    c.nx = c.ny = c.nz = n
    c.x0, c.xmax, c.y0, c.ymax, c.z0, c.zmax = 0.0, 1.0, 0.0, 1.0, 0.0, 1.0
    c.n_materials = 2
    abi.set_material(c.mat[0], abi.EOS_SG, gamma=6.12, pc=3.43e8)
    abi.set_material(c.mat[1], abi.EOS_SG, gamma=1.4, pc=0.0)
    rho_s, u_s = sg_post_shock(1000.0, 1.0e5, 0.0, 1.0e9, 6.12, 3.43e8)
    c.bc[0] = abi.BC_INLET
    c.bc[1] = abi.BC_OUTLET
    for s in range(2, 6):
        c.bc[s] = abi.BC_SYMMETRY
    for p, v in enumerate((rho_s, u_s, 0.0, 0.0, 1.0e9)):
        c.inlet[p] = v
    c.flux = abi.FLUX_HLLC
    c.rec_type = abi.REC_LINEAR
    c.limiter = abi.LIM_VANALBADA
    c.tol_main = 1e-10
    c.n_levelsets, c.ls_matid = 1, 1
    c.ts_type = abi.TS_RK2
    c.cfl = 0.4
    X, Y, Z = cell_centers(c)
    N = X.size
    phi = np.sqrt((X - 0.5) ** 2 + (Y - 0.5) ** 2 + (Z - 0.5) ** 2) - radius
    gas = phi < 0
    shocked = (X < 0.1) & ~gas
    V = np.zeros((N, 5))
    V[:, 0] = np.where(gas, 1.2, np.where(shocked, rho_s, 1000.0))
    V[:, 1] = np.where(shocked, u_s, 0.0)
    V[:, 4] = np.where(gas, 1.0e5, np.where(shocked, 1.0e9, 1.0e5))
    V[:, 0] *= 1.0 + noise * uniform_noise(N, seed)
    ID = gas.astype(np.int32)
    return c, V, ID, phi


EDGES = (32, 48, 64, 96, 128)


def bubble_collapse(nx, ny, nz, radius_frac, p_water, h=1.0e-3):
    """One bubble-collapse domain: a gas bubble (SG 1.4, rho 0.12, p 1e4 Pa) of
    radius radius_frac times the box's shortest side at the box centre, in
    water (SG 6.12, p_inf 3.43e8, rho 1000) at p_water; cubic cells of side h;
    phi = |x - c| - r; MUSCL / van Albada, HLLC, exact interface Riemann at
    1e-10, RK2, CFL 0.4, Outlet on every side."""
    c = abi.default_config()
    c.nx, c.ny, c.nz = nx, ny, nz
    c.x0, c.xmax, c.y0, c.ymax, c.z0, c.zmax = 0.0, nx * h, 0.0, ny * h, 0.0, nz * h
    c.n_materials = 2
    abi.set_material(c.mat[0], abi.EOS_SG, gamma=6.12, pc=3.43e8)
    abi.set_material(c.mat[1], abi.EOS_SG, gamma=1.4, pc=0.0)
    for s in range(6):
        c.bc[s] = abi.BC_OUTLET
    c.flux = abi.FLUX_HLLC
    c.rec_type = abi.REC_LINEAR
    c.limiter = abi.LIM_VANALBADA
    c.tol_main = 1e-10
    c.n_levelsets, c.ls_matid = 1, 1
    c.ts_type = abi.TS_RK2
    c.cfl = 0.4
    X, Y, Z = cell_centers(c)
    ctr = np.array([nx, ny, nz]) * h * 0.5
    r = radius_frac * min(nx, ny, nz) * h
    phi = np.sqrt((X - ctr[0]) ** 2 + (Y - ctr[1]) ** 2 + (Z - ctr[2]) ** 2) - r
    gas = phi < 0
    V = np.zeros((X.size, 5))
    V[:, 0] = np.where(gas, 0.12, 1000.0)
    V[:, 4] = np.where(gas, 1.0e4, p_water)
    return c, V, gas.astype(np.int32), phi


def bubble_collapse_ensemble(n_domains=512, seed=4096, edges=EDGES):
    """Uneven ensemble: edges per axis drawn uniformly from `edges`, bubble
    radius uniform in [0.1, 0.3] of the box, water pressure log-uniform in
    [1e6, 1e8] Pa, gas at 1e4 Pa.  Returns a list of (cfg, V, ID, phi)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(n_domains):
        nx, ny, nz = (int(e) for e in rng.choice(edges, 3))
        rf = rng.uniform(0.1, 0.3)
        pw = 10.0 ** rng.uniform(6.0, 8.0)
        out.append(bubble_collapse(nx, ny, nz, rf, pw))
    return out


def nasg_post_shock(rho1, p1, p2, gamma, pinf, b):
    """Post-shock density and velocity behind a right-moving shock of pressure
    p2 into still Noble-Abel stiffened gas (q = 0) at (rho1, p1).  With
    e = (p + gamma pinf)(v - b) / (gamma - 1), v = 1/rho, the Hugoniot
    e2 - e1 + (p1 + p2)(v2 - v1) / 2 = 0 is linear in v2; u2 = sqrt((p2 - p1)(v1 - v2))."""
    v1 = 1.0 / rho1
    g1 = gamma - 1.0
    a = (p2 + gamma * pinf) / g1 + 0.5 * (p2 + p1)
    rhs = (p1 + gamma * pinf) * (v1 - b) / g1 + b * (p2 + gamma * pinf) / g1 + 0.5 * (p2 + p1) * v1
    v2 = rhs / a
    return 1.0 / v2, float(np.sqrt((p2 - p1) * (v1 - v2)))


def bubble_cluster_shock(n=512, seed=512, n_bubbles=8, p_shock=5.0e8):
    """Large production-shaped run: n^3 cells on [0,1]^3, n_bubbles gas bubbles
    (SG 1.4, rho 1.2, p 1e5) with seeded centres in [0.35,0.8] x [0.25,0.75]^2 and
    radii uniform in [0.04, 0.1], in NASG water (gamma 1.19, pinf 6.2e8,
    b 6.61e-4, rho 1000, p 1e5); water for x < 0.1 carries the post-shock state
    of a p_shock shock (Hugoniot above).  phi = min_i(|x - c_i| - r_i).  MUSCL /
    van Albada, HLLC, exact interface Riemann at 1e-10, RK3, CFL 0.4, level set
    reinitialized every 10 steps (full domain, first layer fixed, MaxIts 30,
    CFL 0.8, tolerance 2e-4); Inlet at x0 (post-shock state), Outlet at xmax,
    Symmetry on y and z."""
    rng = np.random.Generator(np.random.PCG64(seed))
    ctr = np.column_stack([rng.uniform(0.35, 0.8, n_bubbles), rng.uniform(0.25, 0.75, n_bubbles),
                           rng.uniform(0.25, 0.75, n_bubbles)])
    rad = rng.uniform(0.04, 0.1, n_bubbles)
    c = abi.default_config()
    c.nx = c.ny = c.nz = n
    c.x0, c.xmax, c.y0, c.ymax, c.z0, c.zmax = 0.0, 1.0, 0.0, 1.0, 0.0, 1.0
    c.n_materials = 2
    abi.set_material(c.mat[0], abi.EOS_NASG, gamma=1.19, pc=6.2e8, b=6.61e-4, q=0.0)
    abi.set_material(c.mat[1], abi.EOS_SG, gamma=1.4, pc=0.0)
    rho_s, u_s = nasg_post_shock(1000.0, 1.0e5, p_shock, 1.19, 6.2e8, 6.61e-4)
    c.bc[0] = abi.BC_INLET
    c.bc[1] = abi.BC_OUTLET
    for s in range(2, 6):
        c.bc[s] = abi.BC_SYMMETRY
    for p, v in enumerate((rho_s, u_s, 0.0, 0.0, p_shock)):
        c.inlet[p] = v
    c.flux = abi.FLUX_HLLC
    c.rec_type = abi.REC_LINEAR
    c.limiter = abi.LIM_VANALBADA
    c.tol_main = 1e-10
    c.n_levelsets, c.ls_matid = 1, 1
    c.ts_type = abi.TS_RK3
    c.cfl = 0.4
    c.reinit_frequency = 10
    h = 1.0 / n
    x = 0.5 * h + np.arange(n) * h
    phi = np.full((n, n, n), np.inf)
    for (cx, cy, cz), r in zip(ctr, rad):
        d = np.sqrt((x[None, None, :] - cx) ** 2 + (x[None, :, None] - cy) ** 2 + (x[:, None, None] - cz) ** 2) - r
        np.minimum(phi, d, out=phi)
    phi = phi.ravel()
    gas = phi < 0
    shocked = np.broadcast_to(x[None, None, :] < 0.1, (n, n, n)).ravel() & ~gas
    V = np.zeros((n * n * n, 5))
    V[:, 0] = np.where(gas, 1.2, np.where(shocked, rho_s, 1000.0))
    V[:, 1] = np.where(shocked, u_s, 0.0)
    V[:, 4] = np.where(gas, 1.0e5, np.where(shocked, p_shock, 1.0e5))
    return c, V, gas.astype(np.int32), phi
