// Internal definitions shared by the kernels and the host API of libm2cg.
#pragma once
#include <cstdint>
#include <cuda.h>   // CUtensorMap (encoded through the runtime's driver entry point)
#include <cuda_runtime.h>
#include "m2cg_device.cuh"
#include "m2cg_riemann.cuh"

namespace m2cg {

// Ghosted grid: one ghost layer on every side (the reference's DMDA stencil
// width for V, ID and phi; SpaceVariable.cpp:58-70).  Real cell (i,j,k) with
// i in [0,nx) sits at linear index ((k+1)*py + (j+1))*px + (i+1).
struct Grid {
  int nx, ny, nz;
  int px, py, pz;
  int64_t sy, sz, ntot;  // sx = 1
  double dx, dy, dz;
  double h_common;   // the spacing shared by every axis with more than one cell, 0 if they differ
  // Block shape of the cell and face kernels: tile[0] x tile[1] x tile[2] cells
  // per block of 128 threads (x fastest), or all zero: 128 consecutive cells of
  // the x-fastest order.  Set per ensemble member by the tile autotuner.
  int tile[3];
  M2CG_DEV int64_t at(int i, int j, int k) const { return ((int64_t)(k + 1) * py + (j + 1)) * px + (i + 1); }
};

// Cell (i, j, k) of thread th in block bx of an nx x ny x nz index space
// covered by tiles t[0] x t[1] x t[2] (x fastest, then the tiles in x, y, z).
M2CG_DEV bool tiled_index(int nx, int ny, int nz, const int* t, int64_t bx, int th, int& i, int& j, int& k) {
  const int ntx = (nx + t[0] - 1) / t[0], nty = (ny + t[1] - 1) / t[1];
  const int64_t per = (int64_t)ntx * nty;
  const int bz = (int)(bx / per);
  const int64_t r = bx - (int64_t)bz * per;
  const int by = (int)(r / ntx), bxx = (int)(r - (int64_t)by * ntx);
  i = bxx * t[0] + th % t[0];
  j = by * t[1] + (th / t[0]) % t[1];
  k = bz * t[2] + th / (t[0] * t[1]);
  return i < nx && j < ny && k < nz;
}
// Blocks of 128 threads covering an nx x ny x nz index space with the grid's shape.
inline int64_t shaped_blocks(const Grid& g, int nx, int ny, int nz) {
  if (g.tile[0] == 0) return ((int64_t)nx * ny * nz + 127) / 128;
  return (int64_t)((nx + g.tile[0] - 1) / g.tile[0]) * ((ny + g.tile[1] - 1) / g.tile[1]) *
         ((nz + g.tile[2] - 1) / g.tile[2]);
}

// Face-ghost cells: position and image (SpaceOperator.cpp:493-519).
M2CG_DEV bool ghost_face_cell(const Grid& g, int64_t t, int& side, int& i, int& j, int& k,
                                                int& ii, int& jj, int& kk) {
  int64_t nyz = (int64_t)g.ny * g.nz, nxz = (int64_t)g.nx * g.nz, nxy = (int64_t)g.nx * g.ny;
  if (t < 2 * nyz) {
    side = (int)(t / nyz); int64_t r = t % nyz;
    k = (int)(r / g.ny); j = (int)(r % g.ny);
    i = side == 0 ? -1 : g.nx;
    ii = side == 0 ? 0 : g.nx - 1; jj = j; kk = k;
    return true;
  }
  t -= 2 * nyz;
  if (t < 2 * nxz) {
    side = 2 + (int)(t / nxz); int64_t r = t % nxz;
    k = (int)(r / g.nx); i = (int)(r % g.nx);
    j = side == 2 ? -1 : g.ny;
    jj = side == 2 ? 0 : g.ny - 1; ii = i; kk = k;
    return true;
  }
  t -= 2 * nxz;
  if (t < 2 * nxy) {
    side = 4 + (int)(t / nxy); int64_t r = t % nxy;
    j = (int)(r / g.nx); i = (int)(r % g.nx);
    k = side == 4 ? -1 : g.nz;
    kk = side == 4 ? 0 : g.nz - 1; ii = i; jj = j;
    return true;
  }
  return false;
}

// Device counter slots (int64).
enum {
  CNT_IFACE = 0, CNT_RERR, CNT_RITER, CNT_RSOLVE, CNT_CLIPCELL, CNT_CLIPFACE, CNT_BAD, CNT_SWEPT, CNT_UNRES,
  CNT_IF_OVERFLOW, CNT_PATH_CAPPED, CNT_SWEPT_OVERFLOW, CNT_BADID, CNT_FALLBACK, CNT_UNRES_FIXED,
  CNT_UNRES_OVERFLOW, CNT_UNRES_REPAIRS, CNT_TILE_TIMEOUT, CNT_N
};

// Scalars that live on the device for the whole run (no host round trip per step).
struct DevScalars {
  unsigned long long min_dx_over_lambda;  // bit pattern of a positive double (atomicMin)
  double dt, cfl, time;
  int active;       // 0 once MaxTime has been reached
  int pad;
  long long steps;
  double dt_in;     // the time step a caller gave m2cg_advance (its step graph reads it here)
};

struct Params {
  Grid g;
  Mats mats;
  int n_mat;
  int flux, rec_type, limiter, slope_zero;
  int rec_var;          // M2CG_VAR_*: variables whose differences are limited
  int mp_flux, mp_recon, mp_phasechange, mp_pcdir;
  double minmod_coeff, roe_delta;
  int bc[6];
  double inlet[5], inlet2[5];
  int n_ls, ls_matid;
  int ls_bc[6];
  // unresolved swept cells of the current step, listed for the repair that
  // follows a step when reinitialization is configured (else NULL)
  int64_t* unres;
  unsigned long long* unres_count;
  int unres_cap;
  int riemann_normal;   // M2CG_RNORMAL_*: axis of the interface Riemann problems
  const double* phi_n;  // phi at the start of the step (the normals' input; NULL without a level set)
  double lo[3];         // domain origin: cell centres at lo + 0.5 h + i h
  int ls_fv;            // finite-volume level set (else finite difference)
  int ls_flux, ls_rec_linear, ls_limiter;
  double ls_delta, ls_minmod;
  RiemannPrm rp;
  double area[3];
  double inv_negvol;
  double fd3l[3][4], fd3r[3][4];
  double cfl, timestep, max_time;
  int ts_type;
};

// A primitive state set: rho, u, v, w, p, phi (SoA, ghosted).
struct StateSet {
  double* q[6];
};

// Interface-face work list (compacted each step).
struct IfaceList {
  int64_t* face;       // plus-cell index * 4 + direction
  double* lf1[5];      // flux contribution to the minus cell
  double* lf2[5];      // flux contribution to the plus cell
  double* vsm[5];      // stored star states (first stage only)
  double* vsp[5];
  int32_t* err;        // 0 ok / 1 failed: solution not stored (SpaceOperator.cpp:1661)
  int32_t* iters;
  int32_t* slot[3];    // per-cell slot of the face at the cell's minus side in each direction
  unsigned long long* count;
  int64_t cap;
};

// Level-set reinitialization (full domain, first layer held fixed): device
// state of the pseudo-time loop, written by the one-thread control kernel
// between the sub-stage launches and read by every launch of the loop body.
struct ReinitState {
  unsigned long long res_bits;   // max |grad phi| - 1 over untagged cells (first sub-stage), as bits
  unsigned long long dphi_bits;  // max relative change of the iteration, as bits
  unsigned int detected;         // an interior first-layer node exists
  int run;                       // the loop is running
  int restore;                   // the next first sub-stage restarts from the backup
  int iter;                      // iteration of the current attempt
  int body_runs;                 // loop-body executions of the current call (bounded)
  int keep;                      // write the backup even when the loop does not run
  double cfl;                    // pseudo-time CFL; reduced by 1.5 per retry and kept
  long long calls, iterations, retries, failures, bodies;
  double last_res, last_dphi;
};

// The repair of the step's unresolved swept cells (TimeIntegrator.cpp:776-797)
// after the reinitialization that it forces: the IDs follow the sign changes
// of phi (MultiPhaseOperator.cpp:153-357 against the phi before the repair),
// then FixUnresolvedNodes (MultiPhaseOperator.cpp:1279-1480) and clipping.
struct UnresArgs {
  Params P;
  double lo[3];                          // domain origin: cell centres at lo + 0.5 h + i h
  double failsafe[M2CG_MAX_MATERIALS];   // Material.FailSafeDensity
  StateSet S;                            // the solution (V and phi)
  double* bk;                            // phi before the repair (the reinitialization's backup)
  int32_t* id;
  int32_t* id_new;
  int32_t* cand;
  int64_t* swept;                        // cells whose sign changed in the repair
  unsigned long long* swept_count;
  int64_t swept_cap;
  const int64_t* list;                   // the unresolved cells, sorted by index
  const unsigned long long* count;
  const double* phi_old;                 // their phi before the sign flip
  unsigned long long* cnt;
  const DevScalars* sc;
};

struct ReinitArgs {
  Grid g;
  int ls_bc[6];
  double lo[3];        // domain origin: cell centres at lo + 0.5 h + i h
  double rh[3];        // 1/dx, 1/dy, 1/dz
  double hmin;         // min(dx, dy, dz)
  double tol;
  int max_its;
  int freq;            // gate: every freq-th completed step (<= 0: never) ...
  double freq_dt;      // ... or, when > 0, after every step crossing a multiple of freq_dt
  double* phi;         // the level set (ghosted), updated in place
  double* phi1;        // sub-stage states
  double* phi2;
  double* bk;          // backup for a retry
  double* sign;        // smoothed sign of the input
  uint8_t* tag;        // first-layer nodes (held fixed)
  ReinitState* st;
  const DevScalars* sc;
  // the step's unresolved swept cells (the repair's reinitialization runs when
  // there are any: the list is sorted, their phi saved and made negative)
  int64_t* unres;
  unsigned long long* unres_count;
  int unres_cap;
  double* unres_phi_old;
  unsigned long long* cnt;
};

// A probe point located on the ghosted cell-centre grid: lower corner
// (ghosted indices), populated corners (bit m: corner m in the order c000,
// c100, c010, c110, c001, c101, c011, c111) and trilinear coordinates.
struct ProbePoint {
  int i, j, k;
  unsigned valid;
  int nvalid;
  int pad;
  double w[3];
};

struct Box3 {
  double lo[3], hi[3];
};

struct StageArgs {
  // residual input (neighbors) and own-cell inputs of the stage combination
  StateSet in;          // V and phi of the stage input (residual evaluated here)
  StateSet out;         // output V and phi
  const double* phi_lsin;   // phi whose gradient drives the level-set residual (== in.q[5])
  const double* phi_own;    // phi combined with the stage weights (own cell)
  const double* phi_tmp;    // phi at t^n for the sign test (last stage only)
  double* Un[5];        // conservative state at t^n
  double* Us[5];        // conservative stage state (U1 / U2)
  int stage;            // 0, 1, 2
  int last;             // 1 on the final stage
  int store_un;         // write Un (first stage)
  double a_own, b_un, c_dt;   // U = a*Us + b*Un + c*dt*R  (first stage: a=0, b=1, c=1)
  double la, lb, lc;          // phi = la*phi_own_other + lb*phi_n + lc*dt*R (see kernel)
  int ls_use_updated_v;       // forward Euler: level set advected with the updated velocity
  double* R[5];               // residual output (residual-only mode)
  const double* rls_pre;      // level-set residual computed beforehand (finite volume), else NULL
  int residual_only;
};

// Tensor maps of the five primitive arrays of one state set for the fused
// reconstruction + flux kernel (m2cg_tile.cu): 3D (x, y, z) over the ghosted
// arrays, box 36 x 7 x 1.
struct TileMaps {
  CUtensorMap v[5];
};
bool tile_supported(const Params& P);
bool tile_maps(const Params& P, const StateSet& S, TileMaps* out);
cudaError_t tile_prepare();
void launch_recon_flux_tile(cudaStream_t s, const TileMaps& maps, const Params& P, const StateSet& S,
                            const int32_t* id, double* const* F, unsigned long long* cnt, int zchunk);

}  // namespace m2cg
