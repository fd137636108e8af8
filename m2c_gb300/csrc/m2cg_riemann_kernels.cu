// Interface kernels: the exact two-material Riemann solve on every material-
// interface face and the two one-sided fluxes built from its star states
// (SpaceOperator.cpp:1613-1690, 1772-1850, 1931-2009), plus the batched
// Riemann / flux entry points.
//
// This translation unit is compiled without floating-point contraction
// (-fmad=false) so that the iterative solver's branch decisions follow the
// same binary64 rounding as a CPU build of the same algorithm.
#include "m2cg_internal.h"

namespace m2cg {

__device__ __forceinline__ bool num_flux_if(const Params& P, int dir, const double* Vm, const double* Vp, int id,
                                            double* F) {
  const DevMat& M = P.mats.m[id];
  if (P.flux == M2CG_FLUX_HLLC) return flux_hllc(M, dir, Vm, Vp, F);
  if (P.flux == M2CG_FLUX_LLF) return flux_llf2(M, M, dir, Vm, Vp, F);
  return flux_genroe(M, dir, Vm, Vp, P.roe_delta, F);
}

// One thread per interface face (grid-stride over the device-side count).
// scratch: 6 * cap doubles per thread for the two integration-path caches.
__global__ void k_riemann_interfaces(Params P, const Mats* __restrict__ md, StateSet S, const int32_t* __restrict__ id,
                                     double* const* fs, IfaceList L, int store, double* scratch, int path_cap,
                                     const float* warm, unsigned long long* cnt, const DevScalars* sc) {
  if (sc && !sc->active) return;
  const Grid& g = P.g;
  int64_t n = (int64_t)min((unsigned long long)L.cap, *L.count);
  int64_t T = (int64_t)gridDim.x * blockDim.x;
  int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  ExactRiemannDev rs;
  rs.mats = md;
  rs.P = P.rp;
  rs.path1.base = scratch + tid;
  rs.path1.stride = T;
  rs.path1.cap = path_cap;
  rs.path3.base = scratch + (int64_t)3 * path_cap * T + tid;
  rs.path3.stride = T;
  rs.path3.cap = path_cap;
  const int64_t st[3] = {1, g.sy, g.sz};
  if (tid == 0) atomicAdd(&cnt[CNT_IFACE], (unsigned long long)n);
  unsigned long long iters = 0, solves = 0, errs = 0, bad = 0, capped = 0, fallbacks = 0;
  for (int64_t s = tid; s < n; s += T) {
    int64_t fc = L.face[s];
    int d = (int)(fc & 3);
    int64_t c = fc >> 2;
    int64_t m = c - st[d];
    int idm = id[m], idp = id[c];
    double Vm[5], Vp[5];
    if (P.mp_recon == M2CG_MPREC_CONSTANT) {
      for (int p = 0; p < 5; p++) { Vm[p] = S.q[p][m]; Vp[p] = S.q[p][c]; }
    } else {
      for (int p = 0; p < 5; p++) { Vm[p] = fs[(2 * d + 1) * 5 + p][m]; Vp[p] = fs[(2 * d) * 5 + p][c]; }
    }
    double lf1[5], lf2[5];
    if (P.mp_flux == M2CG_MPFLUX_LLF) {   // SpaceOperator.cpp:1617-1626
      bad += !flux_llf2(P.mats.m[idm], P.mats.m[idp], d, Vm, Vp, lf1);
      for (int p = 0; p < 5; p++) lf2[p] = lf1[p];
      if (store) L.err[s] = 1;  // no star states for the phase-change update
    } else {
      double dir[3] = {0.0, 0.0, 0.0};
      dir[d] = 1.0;  // RiemannNormal = Mesh (SpaceOperator.cpp:2186-2203)
      double Vs[5], Vsm[5], Vsp[5];
      int midid = idm;
      rs.warm_p = warm ? (double)warm[s] : 0.0;
      int err = rs.solve(dir, Vm, idm, Vp, idp, Vs, midid, Vsm, Vsp);
      solves++;
      iters += rs.evals;
      capped += rs.path1.capped | rs.path3.capped;
      fallbacks += rs.fallback;
      if (err) errs++;
      if (err < 0) bad++;
      eos_clip(P.mats.m[idm], Vsm);
      bad += eos_bad5(P.mats.m[idm], Vsm);
      eos_clip(P.mats.m[idp], Vsp);
      bad += eos_bad5(P.mats.m[idp], Vsp);
      if (store) {
        L.err[s] = err ? 1 : 0;
        L.iters[s] = rs.evals;
        for (int p = 0; p < 5; p++) { L.vsm[p][s] = Vsm[p]; L.vsp[p][s] = Vsp[p]; }
      }
      if (P.mp_flux == M2CG_MPFLUX_EXACT) {
        phys_flux(P.mats.m[midid], d, Vs, lf1);
        for (int p = 0; p < 5; p++) lf2[p] = lf1[p];
      } else {
        bad += !num_flux_if(P, d, Vm, Vsm, idm, lf1);
        bad += !num_flux_if(P, d, Vsp, Vp, idp, lf2);
      }
    }
    for (int p = 0; p < 5; p++) { L.lf1[p][s] = lf1[p]; L.lf2[p][s] = lf2[p]; }
  }
  if (solves) {
    atomicAdd(&cnt[CNT_RSOLVE], solves);
    atomicAdd(&cnt[CNT_RITER], iters);
  }
  if (errs) atomicAdd(&cnt[CNT_RERR], errs);
  if (bad) atomicAdd(&cnt[CNT_BAD], bad);
  if (capped) atomicAdd(&cnt[CNT_PATH_CAPPED], capped);
  if (fallbacks) atomicAdd(&cnt[CNT_FALLBACK], fallbacks);
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

__global__ void k_flux_batch(Params P, int64_t n, const int32_t* __restrict__ dir, const double* __restrict__ Vm,
                             const double* __restrict__ Vp, const int32_t* __restrict__ id, double* F) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  num_flux_if(P, dir[q], &Vm[q * 5], &Vp[q * 5], id[q], &F[q * 5]);
}

void launch_riemann_interfaces(cudaStream_t s, const Params& P, const Mats* md, const StateSet& S, const int32_t* id,
                               double* const* fs, const IfaceList& L, int store, double* scratch, int path_cap,
                               int blocks, int threads, const float* warm, unsigned long long* cnt,
                               const DevScalars* sc) {
  k_riemann_interfaces<<<blocks, threads, 0, s>>>(P, md, S, id, fs, L, store, scratch, path_cap, warm, cnt, sc);
}
void launch_riemann_batch(cudaStream_t s, const Params& P, const Mats* md, int64_t n, const double* Vm, const int32_t* idm,
                          const double* Vp, const int32_t* idp, const double* dir, double* Vs, int32_t* id,
                          double* Vsm, double* Vsp, int32_t* iters, int32_t* err, double* scratch, int path_cap,
                          int blocks, int threads, const double* warm) {
  k_riemann_batch<<<blocks, threads, 0, s>>>(md, P.rp, n, Vm, idm, Vp, idp, dir, Vs, id, Vsm, Vsp, iters, err,
                                             scratch, path_cap, warm);
}
void launch_flux_batch(cudaStream_t s, const Params& P, int64_t n, const int32_t* dir, const double* Vm,
                       const double* Vp, const int32_t* id, double* F) {
  k_flux_batch<<<(int)((n + 127) / 128), 128, 0, s>>>(P, n, dir, Vm, Vp, id, F);
}

}  // namespace m2cg
