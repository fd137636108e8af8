// Interface kernels: the exact two-material Riemann solve on every material-
// interface face and the two one-sided fluxes built from its star states
// (SpaceOperator.cpp:1613-1690, 1772-1850, 1931-2009), plus the batched
// Riemann / flux entry points.
//
// This translation unit is compiled without floating-point contraction
// (-fmad=false) so that the iterative solver's branch decisions follow the
// same binary64 rounding as a CPU build of the same algorithm.
#include "m2cg_internal.h"
#include "m2cg_ens.h"

namespace m2cg {

__device__ __forceinline__ bool num_flux_if(const Params& P, int dir, const double* Vm, const double* Vp, int id,
                                            double* F) {
  const DevMat& M = P.mats.m[id];
  if (P.flux == M2CG_FLUX_HLLC) return flux_hllc(M, dir, Vm, Vp, F);
  if (P.flux == M2CG_FLUX_LLF) return flux_llf2(M, M, dir, Vm, Vp, F);
  return flux_genroe(M, dir, Vm, Vp, P.roe_delta, F);
}

// Loads the two states of interface face s (cell centres or reconstructed face
// states, SpaceOperator.cpp:1633-1639).
__device__ __forceinline__ void iface_inputs(const Params& P, const StateSet& S, const int32_t* __restrict__ id,
                                             double* const* fs, const IfaceList& L, int64_t s, int& d, int64_t& c,
                                             int& idm, int& idp, double* Vm, double* Vp) {
  const int64_t st[3] = {1, P.g.sy, P.g.sz};
  int64_t fc = L.face[s];
  d = (int)(fc & 3);
  c = fc >> 2;
  int64_t m = c - st[d];
  idm = id[m];
  idp = id[c];
  if (P.mp_recon == M2CG_MPREC_CONSTANT) {
    for (int p = 0; p < 5; p++) { Vm[p] = S.q[p][m]; Vp[p] = S.q[p][c]; }
  } else {
    for (int p = 0; p < 5; p++) { Vm[p] = fs[(2 * d + 1) * 5 + p][m]; Vp[p] = fs[(2 * d) * 5 + p][c]; }
  }
}

// Clip and check the star states, store them for the end-of-step update (first
// stage only) and form the two one-sided fluxes (SpaceOperator.cpp:1641-1690).
__device__ __forceinline__ int iface_finish(const Params& P, const IfaceList& L, int64_t s, int d, int idm, int idp,
                                            const double* Vm, const double* Vp, double* Vs, int midid, double* Vsm,
                                            double* Vsp, int err, int store) {
  int bad = 0;
  eos_clip(P.mats.m[idm], Vsm);
  bad += eos_bad5(P.mats.m[idm], Vsm);
  eos_clip(P.mats.m[idp], Vsp);
  bad += eos_bad5(P.mats.m[idp], Vsp);
  if (store) {
    L.err[s] = err ? 1 : 0;
    for (int p = 0; p < 5; p++) { L.vsm[p][s] = Vsm[p]; L.vsp[p][s] = Vsp[p]; }
  }
  double lf1[5], lf2[5];
  if (P.mp_flux == M2CG_MPFLUX_EXACT) {
    phys_flux(P.mats.m[midid], d, Vs, lf1);
    for (int p = 0; p < 5; p++) lf2[p] = lf1[p];
  } else {
    bad += !num_flux_if(P, d, Vm, Vsm, idm, lf1);
    bad += !num_flux_if(P, d, Vsp, Vp, idp, lf2);
  }
  for (int p = 0; p < 5; p++) { L.lf1[p][s] = lf1[p]; L.lf2[p][s] = lf2[p]; }
  return bad;
}

template <class Solver>
__device__ __forceinline__ void init_solver(Solver& rs, const Mats* md, const RiemannPrm& rp, double* scratch,
                                            int path_cap, int64_t tid, int64_t T) {
  rs.mats = md;
  rs.P = rp;
  rs.warm_p = 0.0;
  rs.nonadaptive = false;
  rs.fallback = 0;
  rs.path1.base = scratch + tid;
  rs.path1.stride = T;
  rs.path1.cap = path_cap;
  rs.path3.base = scratch + (int64_t)3 * path_cap * T + tid;
  rs.path3.stride = T;
  rs.path3.cap = path_cap;
}

// SpaceOperator::GetNormalForBimaterialRiemann with RiemannNormal = LevelSet or
// Average and one level set (SpaceOperator.cpp:2186-2415): the gradient of phi
// at the face between the plus cell c and its minus neighbour along d -- one-
// sided across the face, the tangential components by central differences in
// both cells (one-sided next to the ghost layer) interpolated to the face --
// normalized, reversed when the minus cell is material 0, its d component made
// non-negative; Average adds the mesh normal and normalizes again.  The
// reference asserts unless the two materials are 0 and the level set's; such
// faces keep the mesh normal here.  dir holds the mesh normal on entry.
__device__ __forceinline__ void riemann_normal_dir(const Params& P, int64_t c, int d, int idm, int idp, double* dir) {
  const int my_ls = idp == 0 ? idm : idp, nb_ls = idm == 0 ? idp : idm;
  if (my_ls != P.ls_matid || nb_ls != P.ls_matid || !P.phi_n) return;
  const Grid& g = P.g;
  const double* phi = P.phi_n;
  int64_t r = c;
  int pos[3];
  pos[0] = (int)(r % g.px) - 1; r /= g.px;
  pos[1] = (int)(r % g.py) - 1;
  pos[2] = (int)(r / g.py) - 1;
  const int64_t st[3] = {1, g.sy, g.sz};
  const int nn[3] = {g.nx, g.ny, g.nz};
  const double h[3] = {g.dx, g.dy, g.dz};
  auto X = [&](int a, int q) { return P.lo[a] + 0.5 * h[a] + q * h[a]; };   // MeshGenerator.cpp:166-171
  const int64_t m = c - st[d];
  double gr[3];
  gr[d] = (phi[c] - phi[m]) / (X(d, pos[d]) - X(d, pos[d] - 1));
  const double xmh = X(d, pos[d]) - 0.5 * h[d];
  const double dxd = X(d, pos[d]) - X(d, pos[d] - 1);
  const double c1 = (X(d, pos[d]) - xmh) / dxd, c2 = (xmh - X(d, pos[d] - 1)) / dxd;
  for (int a = 0; a < 3; a++) {
    if (a == d) continue;
    const int q = pos[a];
    double g1, g2;
    if (q < 0) {
      g1 = (phi[m + st[a]] - phi[m]) / (X(a, q + 1) - X(a, q));
      g2 = (phi[c + st[a]] - phi[c]) / (X(a, q + 1) - X(a, q));
    } else if (q >= nn[a]) {
      g1 = (phi[m] - phi[m - st[a]]) / (X(a, q) - X(a, q - 1));
      g2 = (phi[c] - phi[c - st[a]]) / (X(a, q) - X(a, q - 1));
    } else {   // SpaceOperator.h:223-228
      const double x0 = X(a, q - 1), x1 = X(a, q), x2 = X(a, q + 1);
      const double k0 = -(x2 - x1) / ((x1 - x0) * (x2 - x0));
      const double k1 = 1.0 / (x1 - x0) - 1.0 / (x2 - x1);
      const double k2 = (x1 - x0) / ((x2 - x0) * (x2 - x1));
      g1 = k0 * phi[m - st[a]] + k1 * phi[m] + k2 * phi[m + st[a]];
      g2 = k0 * phi[c - st[a]] + k1 * phi[c] + k2 * phi[c + st[a]];
    }
    gr[a] = c1 * g1 + c2 * g2;
  }
  double nrm = sqrt(gr[0] * gr[0] + gr[1] * gr[1] + gr[2] * gr[2]);
  if (nrm != 0.0) { const double inv = 1.0 / nrm; for (int a = 0; a < 3; a++) gr[a] *= inv; }
  if (idm == 0) for (int a = 0; a < 3; a++) gr[a] *= -1.0;
  if (sqrt(gr[0] * gr[0] + gr[1] * gr[1] + gr[2] * gr[2]) == 0.0) gr[d] = 1.0;
  if (gr[d] < 0.0) gr[d] *= -1.0;
  if (P.riemann_normal == M2CG_RNORMAL_AVERAGE) {
    gr[d] += 1.0;
    const double inv = 1.0 / sqrt(gr[0] * gr[0] + gr[1] * gr[1] + gr[2] * gr[2]);
    for (int a = 0; a < 3; a++) gr[a] *= inv;
  }
  for (int a = 0; a < 3; a++) dir[a] = gr[a];
}

// Solves interface face s and stores its fluxes; returns 2 without storing
// anything when the solver's evaluation budget ran out.
__device__ __forceinline__ int iface_solve(const Params& P, StateSet S, const int32_t* __restrict__ id,
                                           double* const* fs, const IfaceList& L, int store, const float* warm,
                                           int64_t s, ExactRiemannChainDev& rs, unsigned long long (&acc)[6]) {
  int d, idm, idp;
  int64_t c;
  double Vm[5], Vp[5];
  iface_inputs(P, S, id, fs, L, s, d, c, idm, idp, Vm, Vp);
  if (P.mp_flux == M2CG_MPFLUX_LLF) {   // SpaceOperator.cpp:1617-1626: no Riemann solve
    double lf[5];
    acc[3] += !flux_llf2(P.mats.m[idm], P.mats.m[idp], d, Vm, Vp, lf);
    for (int p = 0; p < 5; p++) { L.lf1[p][s] = lf[p]; L.lf2[p][s] = lf[p]; }
    if (store) L.err[s] = 1;  // no star states for the phase-change update
    return 0;
  }
  double dir[3] = {0.0, 0.0, 0.0};
  dir[d] = 1.0;  // RiemannNormal = Mesh (SpaceOperator.cpp:2186-2203)
  if (P.riemann_normal != M2CG_RNORMAL_MESH) riemann_normal_dir(P, c, d, idm, idp, dir);
  double Vs[5], Vsm[5], Vsp[5];
  int midid = idm;
  rs.warm_p = warm ? (double)warm[s] : 0.0;
  int err = rs.solve(dir, Vm, idm, Vp, idp, Vs, midid, Vsm, Vsp);
  if (err == 2) return 2;
  acc[0] += rs.evals;
  acc[1]++;
  acc[4] += rs.path1.capped | rs.path3.capped;
  acc[5] += rs.fallback;
  L.iters[s] = rs.evals;
  if (err) acc[2]++;
  if (err < 0) acc[3]++;
  acc[3] += iface_finish(P, L, s, d, idm, idp, Vm, Vp, Vs, midid, Vsm, Vsp, err, store);
  return err;
}

__device__ __forceinline__ void iface_counts(unsigned long long* cnt, const unsigned long long (&acc)[6]) {
  if (acc[1]) atomicAdd(&cnt[CNT_RSOLVE], acc[1]);
  if (acc[0]) atomicAdd(&cnt[CNT_RITER], acc[0]);
  if (acc[2]) atomicAdd(&cnt[CNT_RERR], acc[2]);
  if (acc[3]) atomicAdd(&cnt[CNT_BAD], acc[3]);
  if (acc[4]) atomicAdd(&cnt[CNT_PATH_CAPPED], acc[4]);
  if (acc[5]) atomicAdd(&cnt[CNT_FALLBACK], acc[5]);
}

// Interface Riemann solves, first pass: one thread per interface face
// (grid-stride over the device-side count), each solve limited to eval_limit
// wave-pair evaluations.  Nearly every face converges within a handful; the
// few that do not -- the reference's stalled secant iterations that run to
// MaxIts and then repeat with the non-adaptive solver (ExactRiemannSolverBase.cpp
// :178-193, 323-337), several hundred evaluations in sequence -- are listed in
// strag[] for k_riemann_stragglers.  scratch: 6 * path_cap doubles per thread.
__global__ void k_riemann_interfaces(Params P, const Mats* __restrict__ md, StateSet S, const int32_t* __restrict__ id,
                                     double* const* fs, IfaceList L, int store, double* scratch, int path_cap,
                                     int eval_limit, int32_t* strag, unsigned long long* strag_count,
                                     const float* warm, unsigned long long* cnt, const DevScalars* sc) {
  if (sc && !sc->active) return;
  int64_t n = (int64_t)min((unsigned long long)L.cap, *L.count);
  int64_t T = (int64_t)gridDim.x * blockDim.x;
  int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  ExactRiemannChainDev rs;
  init_solver(rs, md, P.rp, scratch, path_cap, tid, T);
  rs.eval_limit = eval_limit;
  if (tid == 0) atomicAdd(&cnt[CNT_IFACE], (unsigned long long)n);
  unsigned long long acc[6] = {0, 0, 0, 0, 0, 0};
  for (int64_t s = tid; s < n; s += T) {
    if (iface_solve(P, S, id, fs, L, store, warm, s, rs, acc) == 2) {
      unsigned long long k = atomicAdd(strag_count, 1ull);   // k < L.cap: each face is listed once
      strag[k] = (int32_t)s;
    }
  }
  iface_counts(cnt, acc);
}

// Warps the second pass spreads its n faces over: all W launched warps (one
// face per warp) when lanes <= 1, else just enough warps to hold `lanes` faces
// each.  Lanes of a warp that follow different faces take turns only where
// their control flow differs; the stalled solves that reach this pass mostly
// run the same secant loop, so packing several into one warp costs little
// latency and frees the SMs the pass would otherwise hold.  Face k runs on
// warp k mod W, lane k / W (k / W < 32 for every k < n).
__device__ __forceinline__ int64_t straggler_warps(int64_t n, int64_t W, int lanes) {
  if (lanes <= 1 || n <= 0) return W;
  int64_t need = (n + lanes - 1) / lanes;
  int64_t floor32 = (n + 31) / 32;   // never fewer warps than 32 lanes can hold
  need = need < floor32 ? floor32 : need;
  return need < W ? need : W;
}

// Second pass: the listed faces solved without a budget.  Each is one long
// chain of dependent binary64 operations, so the faces are dealt round-robin
// over the warps (lane-major), which puts as few as possible in one warp: lanes
// of a warp that follow different faces diverge and take turns.  The launch
// asks for (and never touches) nearly all of an SM's shared memory, so no block
// of another kernel shares an SM -- and its FP64 unit -- with these chains while
// the reconstruction and face-flux kernels run concurrently on the other SMs.
// That request also takes most of the SM's L1, so lane 0 of each warp -- the
// one lane in use while there are no more faces than warps -- keeps its
// integration-path caches in the reserved shared memory instead of going
// through L1 to the global scratch.
__global__ void __launch_bounds__(128) k_riemann_stragglers(Params P, const Mats* __restrict__ md, StateSet S,
                                                            const int32_t* __restrict__ id, double* const* fs,
                                                            IfaceList L, int store, double* scratch, int path_cap,
                                                            size_t reserve_bytes, const int32_t* __restrict__ strag,
                                                            const unsigned long long* strag_count, const float* warm,
                                                            unsigned long long* cnt, const DevScalars* sc, int lanes) {
  extern __shared__ __align__(16) double s_path[];
  if (sc && !sc->active) return;
  int64_t n = (int64_t)min((unsigned long long)L.cap, *strag_count);
  const int64_t W = straggler_warps(n, (int64_t)gridDim.x * (blockDim.x >> 5), lanes);
  const int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int64_t lane = threadIdx.x & 31;
  int64_t T = (int64_t)gridDim.x * blockDim.x;
  int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  ExactRiemannChainDev rs;
  init_solver(rs, md, P.rp, scratch, path_cap, tid, T);
  const size_t per_warp = (size_t)6 * path_cap;  // doubles: two waves x cap entries x {p, rho, u}
  if (lane == 0 && (size_t)(blockDim.x >> 5) * per_warp * sizeof(double) <= reserve_bytes) {
    rs.path1.base = s_path + (threadIdx.x >> 5) * per_warp;
    rs.path1.stride = 1;
    rs.path3.base = rs.path1.base + (size_t)3 * path_cap;
    rs.path3.stride = 1;
  }
  unsigned long long acc[6] = {0, 0, 0, 0, 0, 0};
  if (w < W)
    for (int64_t k = lane * W + w; k < n; k += 32 * W) iface_solve(P, S, id, fs, L, store, warm, strag[k], rs, acc);
  iface_counts(cnt, acc);
}

// ---- batched member domains (m2cg_ensemble) ----------------------------------
// One solve pass over the interface faces of every member domain: a global
// index runs over the concatenated per-domain lists (exclusive prefix `off`
// of the member counts), so the whole GPU works on all domains' faces at once
// and the integration-path scratch is one pool shared by the members.

// Prefix of the member interface counts (inactive members count zero) and
// the per-member face counter; clears the straggler count.  One thread.
__global__ void k_ens_iface_prefix(const RiemannEnsArgs* __restrict__ a, int D, int64_t* off,
                                   unsigned long long* strag_count) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int64_t t = 0;
  for (int d = 0; d < D; d++) {
    off[d] = t;
    int64_t n = (a[d].sc && !a[d].sc->active) ? 0 : (int64_t)min((unsigned long long)a[d].L.cap, *a[d].L.count);
    if (n) atomicAdd(&a[d].cnt[CNT_IFACE], (unsigned long long)n);
    t += n;
  }
  off[D] = t;
  *strag_count = 0;
}

__device__ __forceinline__ int ens_domain(const int64_t* off, int D, int64_t g) {
  int lo = 0, hi = D - 1;  // largest d with off[d] <= g
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= g) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ void ens_flush(unsigned long long* cnt, unsigned long long (&acc)[6]) {
  iface_counts(cnt, acc);
  for (int i = 0; i < 6; i++) acc[i] = 0;
}

__global__ void k_riemann_interfaces_ens(const RiemannEnsArgs* __restrict__ a, int D, const int64_t* __restrict__ off,
                                         double* scratch, int path_cap, int eval_limit, int64_t* strag,
                                         unsigned long long* strag_count) {
  const int64_t n = off[D];
  int64_t T = (int64_t)gridDim.x * blockDim.x;
  int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  ExactRiemannChainDev rs;
  init_solver(rs, a[0].md, a[0].P.rp, scratch, path_cap, tid, T);
  rs.eval_limit = eval_limit;
  unsigned long long acc[6] = {0, 0, 0, 0, 0, 0};
  int dcur = -1;
  for (int64_t g = tid; g < n; g += T) {
    int d = ens_domain(off, D, g);
    const RiemannEnsArgs& e = a[d];
    if (d != dcur) {
      if (dcur >= 0) ens_flush(a[dcur].cnt, acc);
      dcur = d;
    }
    rs.mats = e.md;
    rs.P = e.P.rp;
    int64_t s = g - off[d];
    if (iface_solve(e.P, e.S, e.id, e.fs, e.L, e.store, e.warm, s, rs, acc) == 2) {
      unsigned long long k = atomicAdd(strag_count, 1ull);  // k < n
      strag[k] = ((int64_t)d << 40) | s;
    }
  }
  if (dcur >= 0) ens_flush(a[dcur].cnt, acc);
}

// The listed faces of all members, dealt lane-major over the warps as in
// k_riemann_stragglers (one face per warp while there are no more faces than
// warps).
__global__ void __launch_bounds__(128) k_riemann_stragglers_ens(const RiemannEnsArgs* __restrict__ a, double* scratch,
                                                                int path_cap, size_t reserve_bytes,
                                                                const int64_t* __restrict__ strag,
                                                                const unsigned long long* strag_count, int lanes) {
  extern __shared__ __align__(16) double s_path[];
  const int64_t n = (int64_t)*strag_count;
  const int64_t W = straggler_warps(n, (int64_t)gridDim.x * (blockDim.x >> 5), lanes);
  const int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int64_t lane = threadIdx.x & 31;
  int64_t T = (int64_t)gridDim.x * blockDim.x;
  int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  ExactRiemannChainDev rs;
  init_solver(rs, a[0].md, a[0].P.rp, scratch, path_cap, tid, T);
  const size_t per_warp = (size_t)6 * path_cap;
  if (lane == 0 && (size_t)(blockDim.x >> 5) * per_warp * sizeof(double) <= reserve_bytes) {
    rs.path1.base = s_path + (threadIdx.x >> 5) * per_warp;
    rs.path1.stride = 1;
    rs.path3.base = rs.path1.base + (size_t)3 * path_cap;
    rs.path3.stride = 1;
  }
  unsigned long long acc[6] = {0, 0, 0, 0, 0, 0};
  for (int64_t k = lane * W + w; w < W && k < n; k += 32 * W) {
    int64_t v = strag[k];
    int d = (int)(v >> 40);
    int64_t s = v & ((1ll << 40) - 1);
    const RiemannEnsArgs& e = a[d];
    rs.mats = e.md;
    rs.P = e.P.rp;
    iface_solve(e.P, e.S, e.id, e.fs, e.L, e.store, e.warm, s, rs, acc);
    ens_flush(e.cnt, acc);
  }
}

void launch_riemann_ens(cudaStream_t s, const RiemannEnsArgs* a, int D, int64_t* off, double* scratch, int path_cap,
                        int blocks, int eval_limit, int64_t* strag, unsigned long long* strag_count, int sblocks,
                        size_t reserve_smem, int lanes) {
  k_ens_iface_prefix<<<1, 1, 0, s>>>(a, D, off, strag_count);
  k_riemann_interfaces_ens<<<blocks, 128, 0, s>>>(a, D, off, scratch, path_cap, eval_limit, strag, strag_count);
  k_riemann_stragglers_ens<<<sblocks, 128, reserve_smem, s>>>(a, scratch, path_cap, reserve_smem, strag, strag_count,
                                                              lanes);
}
cudaError_t riemann_stragglers_ens_reserve(size_t bytes) {
  return cudaFuncSetAttribute(k_riemann_stragglers_ens, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// Batched independent problems (device arrays, AoS rows of 5 / 3).
__global__ void k_riemann_batch(const Mats* __restrict__ md, RiemannPrm rp, int64_t n, const double* __restrict__ Vm,
                                const int32_t* __restrict__ idm, const double* __restrict__ Vp,
                                const int32_t* __restrict__ idp, const double* __restrict__ dir, double* Vs,
                                int32_t* id, double* Vsm, double* Vsp, int32_t* iters, int32_t* err, double* scratch,
                                int path_cap, const double* warm) {
  int64_t T = (int64_t)gridDim.x * blockDim.x;
  int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  ExactRiemannDev rs;
  rs.mats = md;
  rs.P = rp;
  rs.path1.base = scratch + tid;
  rs.path1.stride = T;
  rs.path1.cap = path_cap;
  rs.path3.base = scratch + (int64_t)3 * path_cap * T + tid;
  rs.path3.stride = T;
  rs.path3.cap = path_cap;
  for (int64_t q = tid; q < n; q += T) {
    int oid = 0;
    rs.warm_p = warm ? warm[q] : 0.0;
    int e = rs.solve(&dir[q * 3], &Vm[q * 5], idm[q], &Vp[q * 5], idp[q], &Vs[q * 5], oid, &Vsm[q * 5], &Vsp[q * 5]);
    id[q] = oid;
    if (iters) iters[q] = rs.evals;
    if (err) err[q] = e;
  }
}

// DevMat of a stiffened-gas / Noble-Abel stiffened-gas material from
// {type, gamma, pc, b, q}, with the reference's default (no-op) clipping; the
// same arithmetic as the host-side configuration (m2cg_fill_params).
__device__ __forceinline__ void make_devmat(const double* e, DevMat& d) {
  d.type = (int)e[0];
  d.gam = e[1];
  d.gam1 = e[1] - 1.0;
  d.Pstiff = e[2];
  d.gamPs = e[1] * e[2];
  d.invgam1 = 1.0 / (e[1] - 1.0);
  d.b = e[3];
  d.q = e[4];
  d.rho0 = 1.0; d.s = 0.0; d.e0 = 0.0; d.rho0_c0_c0 = 0.0; d.G0_half = 0.0; d.G0_rho0 = 0.0;
  d.rhomin = 0.0; d.pmin = -DBL_MAX; d.rhomax = DBL_MAX; d.pmax = DBL_MAX;
  d.clip_default = 1;
}

// Independent 1D problems, each with its own material pair (the warm-start
// training and evaluation sets): W rows {rho_l, u_l, p_l, rho_r, u_r, p_r},
// E rows {type, gamma, pc, b, q} left then right; out rows {p*, u*, rho*_l,
// rho*_r}.  One thread per problem, grid-stride.
__global__ void k_riemann_batch_eos(RiemannPrm rp, int64_t n, const double* __restrict__ W,
                                    const double* __restrict__ E, const double* __restrict__ warm, double* out,
                                    int32_t* iters, int32_t* err, double* scratch, int path_cap) {
  int64_t T = (int64_t)gridDim.x * blockDim.x;
  int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  Mats mats;
  ExactRiemannDev rs;
  init_solver(rs, &mats, rp, scratch, path_cap, tid, T);
  const double dir[3] = {1.0, 0.0, 0.0};
  for (int64_t q = tid; q < n; q += T) {
    make_devmat(&E[q * 10], mats.m[0]);
    make_devmat(&E[q * 10 + 5], mats.m[1]);
    const double* w = &W[q * 6];
    double Vm[5] = {w[0], w[1], 0.0, 0.0, w[2]}, Vp[5] = {w[3], w[4], 0.0, 0.0, w[5]};
    double Vs[5], Vsm[5], Vsp[5];
    int oid = 0;
    rs.warm_p = warm ? warm[q] : 0.0;
    int e = rs.solve(dir, Vm, 0, Vp, 1, Vs, oid, Vsm, Vsp);
    out[q * 4 + 0] = Vsm[4];
    out[q * 4 + 1] = Vsm[1];
    out[q * 4 + 2] = Vsm[0];
    out[q * 4 + 3] = Vsp[0];
    if (iters) iters[q] = rs.evals;
    if (err) err[q] = e;
  }
}

__global__ void k_flux_batch(Params P, int64_t n, const int32_t* __restrict__ dir, const double* __restrict__ Vm,
                             const double* __restrict__ Vp, const int32_t* __restrict__ id, double* F) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  num_flux_if(P, dir[q], &Vm[q * 5], &Vp[q * 5], id[q], &F[q * 5]);
}

void launch_riemann_interfaces(cudaStream_t s, const Params& P, const Mats* md, const StateSet& S, const int32_t* id,
                               double* const* fs, const IfaceList& L, int store, double* scratch, int path_cap,
                               int blocks, int threads, int eval_limit, int32_t* strag,
                               unsigned long long* strag_count, const float* warm, unsigned long long* cnt,
                               const DevScalars* sc) {
  cudaMemsetAsync(strag_count, 0, sizeof(unsigned long long), s);
  k_riemann_interfaces<<<blocks, threads, 0, s>>>(P, md, S, id, fs, L, store, scratch, path_cap, eval_limit, strag,
                                                  strag_count, warm, cnt, sc);
}
// blocks * 128 threads must not exceed the first pass's thread count (the
// path-cache scratch is shared); reserve_smem: dynamic shared memory per block.
void launch_riemann_stragglers(cudaStream_t s, const Params& P, const Mats* md, const StateSet& S, const int32_t* id,
                               double* const* fs, const IfaceList& L, int store, double* scratch, int path_cap,
                               int blocks, size_t reserve_smem, const int32_t* strag,
                               const unsigned long long* strag_count, const float* warm, unsigned long long* cnt,
                               const DevScalars* sc, int lanes) {
  k_riemann_stragglers<<<blocks, 128, reserve_smem, s>>>(P, md, S, id, fs, L, store, scratch, path_cap, reserve_smem,
                                                         strag, strag_count, warm, cnt, sc, lanes);
}
// One block that holds one SM for a fixed number of clock cycles (bounded
// loop, waits on nothing).  Launched on the main stream between the first
// Riemann pass and the reconstruction: without it the reconstruction's blocks,
// which become ready at the same moment as the straggler blocks, take every
// SM, and the straggler blocks -- which need an empty SM -- wait for the face
// fluxes to drain.
__global__ void k_hold(long long cycles) {
  long long t0 = clock64();
  for (int i = 0; i < (1 << 22); i++) {
    if (clock64() - t0 >= cycles) break;
  }
}
void launch_hold(cudaStream_t s, long long cycles) { k_hold<<<1, 32, 0, s>>>(cycles); }

cudaError_t riemann_stragglers_reserve(size_t bytes) {
  return cudaFuncSetAttribute(k_riemann_stragglers, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}
void launch_riemann_batch(cudaStream_t s, const Params& P, const Mats* md, int64_t n, const double* Vm, const int32_t* idm,
                          const double* Vp, const int32_t* idp, const double* dir, double* Vs, int32_t* id,
                          double* Vsm, double* Vsp, int32_t* iters, int32_t* err, double* scratch, int path_cap,
                          int blocks, int threads, const double* warm) {
  k_riemann_batch<<<blocks, threads, 0, s>>>(md, P.rp, n, Vm, idm, Vp, idp, dir, Vs, id, Vsm, Vsp, iters, err,
                                             scratch, path_cap, warm);
}
void launch_riemann_batch_eos(cudaStream_t s, const Params& P, int64_t n, const double* W, const double* E,
                              const double* warm, double* out, int32_t* iters, int32_t* err, double* scratch,
                              int path_cap, int blocks, int threads) {
  k_riemann_batch_eos<<<blocks, threads, 0, s>>>(P.rp, n, W, E, warm, out, iters, err, scratch, path_cap);
}
void launch_flux_batch(cudaStream_t s, const Params& P, int64_t n, const int32_t* dir, const double* Vm,
                       const double* Vp, const int32_t* id, double* F) {
  k_flux_batch<<<(int)((n + 127) / 128), 128, 0, s>>>(P, n, dir, Vm, Vp, id, F);
}

}  // namespace m2cg
