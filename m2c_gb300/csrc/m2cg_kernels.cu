// Stage kernels of the GB300 finite-volume step: reconstruction, same-material
// face fluxes, residual gather + Runge-Kutta stage update + level-set update,
// boundary conditions, the CFL reduction and the end-of-step material update.
//
// One thread per cell (or per face-owning cell); every face flux is evaluated
// exactly once.  All arithmetic is binary64; the FP64 pipe, not HBM, bounds
// these kernels on GB300.
#include <algorithm>
#include "m2cg_internal.h"
#include "m2cg_ens.h"

namespace m2cg {

// Member owning flat block b of a batched launch: largest d with boff[d] <= b.
__device__ __forceinline__ int ens_member(const int64_t* __restrict__ boff, int D, int64_t b) {
  int lo = 0, hi = D - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (boff[mid] <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}


__device__ __forceinline__ void atomic_inc(unsigned long long* c, unsigned long long v = 1ull) {
  atomicAdd(c, v);
}

// Linear index of a real cell from a flat thread id over nx*ny*nz.
__device__ __forceinline__ bool real_cell(const Grid& g, int64_t t, int& i, int& j, int& k) {
  int64_t n = (int64_t)g.nx * g.ny * g.nz;
  if (t >= n) return false;
  int64_t nxy = (int64_t)g.nx * g.ny;
  k = (int)(t / nxy);
  int64_t r = t - (int64_t)k * nxy;
  j = (int)(r / g.nx);
  i = (int)(r - (int64_t)j * g.nx);
  return true;
}

// Real cell of this thread in block bx of a cell kernel (the grid's block shape).
__device__ __forceinline__ bool block_cell(const Grid& g, int64_t bx, int& i, int& j, int& k) {
  if (g.tile[0] == 0) return real_cell(g, bx * blockDim.x + threadIdx.x, i, j, k);
  return tiled_index(g.nx, g.ny, g.nz, g.tile, bx, threadIdx.x, i, j, k);
}

// CheckReconstructedStates (SpaceOperator.cpp:2446-2484): a face state that
// clipping would change reverts to the cell value; then the six face states
// are stored.
__device__ __forceinline__ void store_faces(const DevMat& M, const double* q, double (*face)[5], double* const* fs,
                                            int64_t c, unsigned long long* cnt) {
  int nclip = 0, nbad = 0;
#pragma unroll
  for (int f = 0; f < 6; f++) {
    double t[5] = {face[f][0], face[f][1], face[f][2], face[f][3], face[f][4]};
    if (eos_clip_fast(M, t)) {
#pragma unroll
      for (int p = 0; p < 5; p++) face[f][p] = q[p];
      nclip++;
    }
    nbad += eos_bad5_fast(M, face[f]);
  }
  if (nclip) atomic_inc(&cnt[CNT_CLIPFACE], nclip);
  if (nbad) atomic_inc(&cnt[CNT_BAD], nbad);
#pragma unroll
  for (int f = 0; f < 6; f++)
#pragma unroll
    for (int p = 0; p < 5; p++) fs[f * 5 + p][c] = face[f][p];
}

// ---------------------------------------------------------------------------
// K1: MUSCL reconstruction of the six face states of every real cell
// (Reconstructor.cpp:426-782) followed by CheckReconstructedStates
// (SpaceOperator.cpp:2446-2484).  fs[f*5+p]: f = vl, vr, vb, vt, vk, vf.
__device__ __forceinline__ void k_reconstruct_body(const Params& P, const StateSet& S, const int32_t* __restrict__ id, double* const* fs, unsigned long long* cnt, unsigned bx_, unsigned gx_) {
  int i, j, k;
  if (!block_cell(P.g, bx_, i, j, k)) return;
  const Grid& g = P.g;
  int64_t c = g.at(i, j, k);
  double q[5];
#pragma unroll
  for (int p = 0; p < 5; p++) q[p] = S.q[p][c];
  const int myid = id[c];
  const DevMat& M = P.mats.m[myid];
  double face[6][5];
  if (P.rec_type == M2CG_REC_CONSTANT) {
#pragma unroll
    for (int f = 0; f < 6; f++)
#pragma unroll
      for (int p = 0; p < 5; p++) face[f][p] = q[p];
  } else {
    const int64_t st[3] = {1, g.sy, g.sz};
#pragma unroll
    for (int d = 0; d < 3; d++) {
      bool zero = P.slope_zero && (id[c - st[d]] != myid || id[c + st[d]] != myid);
#pragma unroll
      for (int p = 0; p < 5; p++) {
        double dq0 = q[p] - S.q[p][c - st[d]];
        double dq1 = S.q[p][c + st[d]] - q[p];
        double s;
        if (P.limiter == M2CG_LIM_VANALBADA) s = van_albada_fast(dq0, dq1);
        else if (P.limiter == M2CG_LIM_GENERALIZED_MINMOD) s = gen_minmod(P.minmod_coeff, dq0, dq1);
        else s = 0.5 * (dq0 + dq1);
        if (zero) s = 0.0;
        face[2 * d][p] = fma(-0.5, s, q[p]);
        face[2 * d + 1][p] = fma(0.5, s, q[p]);
      }
    }
    // Reconstructor.cpp:722-778: the first nonphysical face state reverts to the cell value
    bool done = false;
#pragma unroll
    for (int f = 0; f < 6; f++) {
      bool bad = !done && eos_bad5_fast(M, face[f]);
      if (bad) {
#pragma unroll
        for (int p = 0; p < 5; p++) face[f][p] = q[p];
        done = true;
      }
    }
  }
  store_faces(M, q, face, fs, c, cnt);
}
__global__ void __launch_bounds__(128) k_reconstruct(Params P, StateSet S, const int32_t* __restrict__ id,
                                                     double* const* fs, unsigned long long* cnt) { k_reconstruct_body(P, S, id, fs, cnt, blockIdx.x, gridDim.x); }
// batched: the launch's blocks are the members' blocks back to back
// (boff: exclusive prefix of the members' block counts)
__global__ void __launch_bounds__(128) k_reconstruct_ens(const k_reconstruct_args* __restrict__ ea, const int64_t* __restrict__ boff, int D, int64_t nvb) {
  // persistent: the launch's blocks take the members' blocks in turn
  for (int64_t b = blockIdx.x; b < nvb; b += gridDim.x) {
    const int d = ens_member(boff, D, b);
    const k_reconstruct_args& e = ea[d];
    k_reconstruct_body(e.P, e.S, e.id, e.fs, e.cnt, (unsigned)(b - boff[d]), (unsigned)(boff[d + 1] - boff[d]));
  }
}



// ---------------------------------------------------------------------------
// K1 for the other reconstruction variable types (Reconstructor.cpp:335-918):
// conservative differences (each cell's U with its own material), or primitive
// / conservative differences projected on the characteristic fields of the
// cell's state in each direction (FluxFcnBase.h:308-517), limited, projected
// back; conservative face states convert back to primitive.  A nonphysical face
// state restarts the cell in primitive variables, where the first nonphysical
// face reverts to the cell value (Reconstructor.cpp:722-778).

// The EOS quantities and eigenvector products of the characteristic basis at V0.
struct CharBasis {
  double e0, c0, dpdrho0, Gamma0, kin0, alpha0, beta0, H0;
};
__device__ __forceinline__ void char_basis(const DevMat& M, const double* V0, CharBasis& b) {
  b.e0 = eos_e(M, V0[0], V0[4]);
  b.c0 = sqrt(eos_c2(M, V0[0], b.e0));
  b.dpdrho0 = eos_dpdrho(M, V0[0], b.e0);
  b.Gamma0 = eos_Gamma(M, V0[0]);
  b.kin0 = 0.5 * (V0[1] * V0[1] + V0[2] * V0[2] + V0[3] * V0[3]);
  b.alpha0 = V0[0] * b.Gamma0 / (V0[4] * b.Gamma0 + V0[0] * b.dpdrho0);
  b.beta0 = (b.e0 - b.kin0 + V0[4] / V0[0]) * b.alpha0;
  b.H0 = b.e0 + b.kin0 + V0[4] / V0[0];
}
// dW = R0^-1 x in direction d (rows: the u-c wave, three transverse / entropy
// fields, the u+c wave)
__device__ __forceinline__ void char_left(const CharBasis& b, const double* V0, int d, const double* x, double* w) {
  const double un = V0[1 + d], ic = 1.0 / b.c0, a = b.alpha0;
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < 3; j++) s += a * V0[1 + j] * x[1 + j];
  w[0] = 0.5 * (1.0 - b.beta0 + un * ic) * x[0] - 0.5 * s - 0.5 * ic * x[1 + d] + 0.5 * a * x[4];
  w[4] = 0.5 * (1.0 - b.beta0 - un * ic) * x[0] - 0.5 * s + 0.5 * ic * x[1 + d] + 0.5 * a * x[4];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    if (i == d) w[1 + i] = (b.beta0 + un - V0[1 + i]) * x[0] + s - a * x[4];
    else w[1 + i] = -V0[1 + i] * x[0] + x[1 + i];
  }
}
// x = R0 dW in direction d
__device__ __forceinline__ void char_right(const CharBasis& b, const double* V0, int d, const double* w, double* x) {
  const double un = V0[1 + d];
  const double param = b.e0 + b.kin0 - b.dpdrho0 / b.Gamma0 - un;
  x[0] = w[0] + w[1 + d] + w[4];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    // row 1+i of R0: (V_i - c n_i, delta_ij + V_i n_j - n_i n_j, V_i + c n_i)
    if (i == d) x[1 + i] = V0[1 + i] * (w[0] + w[4]) + b.c0 * (w[4] - w[0]) + V0[1 + i] * w[1 + d];
    else x[1 + i] = V0[1 + i] * (w[0] + w[4]) + w[1 + i] + V0[1 + i] * w[1 + d];
  }
  double t4 = (b.H0 - un * b.c0) * w[0] + (b.H0 + un * b.c0) * w[4];
#pragma unroll
  for (int j = 0; j < 3; j++) t4 += (V0[1 + j] + (j == d ? param : 0.0)) * w[1 + j];
  x[4] = t4;
}

template <int VT>
__device__ __forceinline__ void reconstruct_var_cell(const Params& P, const StateSet& S, const int32_t* __restrict__ id,
                                                     int64_t c, const double* q, int myid, double (*face)[5]) {
  const Grid& g = P.g;
  const DevMat& M = P.mats.m[myid];
  const int64_t st[3] = {1, g.sy, g.sz};
  CharBasis b;
  if (VT == M2CG_VAR_PRIMITIVE_CHARACTERISTIC || VT == M2CG_VAR_CONSERVATIVE_CHARACTERISTIC) char_basis(M, q, b);
  int vt = VT;
  for (int pass = 0; pass < 2; pass++) {
    const bool cons = (vt == M2CG_VAR_CONSERVATIVE || vt == M2CG_VAR_CONSERVATIVE_CHARACTERISTIC);
    double w[5];
    if (cons) prim_to_cons(M, q, w);
    else {
#pragma unroll
      for (int p = 0; p < 5; p++) w[p] = q[p];
    }
    double sig[3][5];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      double wm[5], wp[5], dq0[5], dq1[5];
#pragma unroll
      for (int p = 0; p < 5; p++) { wm[p] = S.q[p][c - st[d]]; wp[p] = S.q[p][c + st[d]]; }
      if (cons) {
        double t[5];
        prim_to_cons(P.mats.m[id[c - st[d]]], wm, t);
#pragma unroll
        for (int p = 0; p < 5; p++) wm[p] = t[p];
        prim_to_cons(P.mats.m[id[c + st[d]]], wp, t);
#pragma unroll
        for (int p = 0; p < 5; p++) wp[p] = t[p];
      }
#pragma unroll
      for (int p = 0; p < 5; p++) { dq0[p] = w[p] - wm[p]; dq1[p] = wp[p] - w[p]; }
      if (vt == M2CG_VAR_PRIMITIVE_CHARACTERISTIC) {
        // Q0: primitive -> conservative differential at q (FluxFcnBase.h:322-330)
        const double q51 = b.e0 + b.kin0 - b.dpdrho0 / b.Gamma0;
        double t0[5], t1[5];
        t0[0] = dq0[0]; t1[0] = dq1[0];
#pragma unroll
        for (int i = 1; i < 4; i++) { t0[i] = q[i] * dq0[0] + q[0] * dq0[i]; t1[i] = q[i] * dq1[0] + q[0] * dq1[i]; }
        t0[4] = q51 * dq0[0] + q[0] * q[1] * dq0[1] + q[0] * q[2] * dq0[2] + q[0] * q[3] * dq0[3] + dq0[4] / b.Gamma0;
        t1[4] = q51 * dq1[0] + q[0] * q[1] * dq1[1] + q[0] * q[2] * dq1[2] + q[0] * q[3] * dq1[3] + dq1[4] / b.Gamma0;
        char_left(b, q, d, t0, dq0);
        char_left(b, q, d, t1, dq1);
      } else if (vt == M2CG_VAR_CONSERVATIVE_CHARACTERISTIC) {
        double t0[5], t1[5];
        char_left(b, q, d, dq0, t0);
        char_left(b, q, d, dq1, t1);
#pragma unroll
        for (int p = 0; p < 5; p++) { dq0[p] = t0[p]; dq1[p] = t1[p]; }
      }
#pragma unroll
      for (int p = 0; p < 5; p++) {
        double s;
        if (P.limiter == M2CG_LIM_VANALBADA) s = van_albada_fast(dq0[p], dq1[p]);
        else if (P.limiter == M2CG_LIM_GENERALIZED_MINMOD) s = gen_minmod(P.minmod_coeff, dq0[p], dq1[p]);
        else s = 0.5 * (dq0[p] + dq1[p]);
        sig[d][p] = s;
      }
      if (vt == M2CG_VAR_PRIMITIVE_CHARACTERISTIC) {
        // R0 then Q0^-1 (FluxFcnBase.h:392-419)
        double t[5];
        char_right(b, q, d, sig[d], t);
        const double ir = 1.0 / q[0];
        sig[d][0] = t[0];
#pragma unroll
        for (int i = 1; i < 4; i++) sig[d][i] = -q[i] * ir * t[0] + t[i] * ir;
        sig[d][4] = ((-b.e0 + b.kin0) * b.Gamma0 + b.dpdrho0) * t[0] -
                    b.Gamma0 * (q[1] * t[1] + q[2] * t[2] + q[3] * t[3] - t[4]);
      } else if (vt == M2CG_VAR_CONSERVATIVE_CHARACTERISTIC) {
        double t[5];
        char_right(b, q, d, sig[d], t);
#pragma unroll
        for (int p = 0; p < 5; p++) sig[d][p] = t[p];
      }
      if (P.slope_zero && (id[c - st[d]] != myid || id[c + st[d]] != myid)) {
#pragma unroll
        for (int p = 0; p < 5; p++) sig[d][p] = 0.0;
      }
    }
#pragma unroll
    for (int f = 0; f < 6; f++) {
      const double h = (f & 1) ? 0.5 : -0.5;
      if (cons) {
        double u2[5];
#pragma unroll
        for (int p = 0; p < 5; p++) u2[p] = w[p] + h * sig[f >> 1][p];
        cons_to_prim(M, u2, face[f]);
      } else {
#pragma unroll
        for (int p = 0; p < 5; p++) face[f][p] = q[p] + h * sig[f >> 1][p];
      }
    }
    int bad = -1;
#pragma unroll
    for (int f = 0; f < 6; f++)
      if (bad < 0 && eos_bad5(M, face[f])) bad = f;
    if (bad < 0) return;
    if (vt == M2CG_VAR_PRIMITIVE) {
#pragma unroll
      for (int f = 0; f < 6; f++)
        if (f == bad) {
#pragma unroll
          for (int p = 0; p < 5; p++) face[f][p] = q[p];
        }
      return;
    }
    vt = M2CG_VAR_PRIMITIVE;
  }
}

template <int VT>
__global__ void __launch_bounds__(128) k_reconstruct_var(Params P, StateSet S, const int32_t* __restrict__ id,
                                                         double* const* fs, unsigned long long* cnt) {
  int i, j, k;
  if (!real_cell(P.g, (int64_t)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
  const int64_t c = P.g.at(i, j, k);
  double q[5];
#pragma unroll
  for (int p = 0; p < 5; p++) q[p] = S.q[p][c];
  const int myid = id[c];
  double face[6][5];
  reconstruct_var_cell<VT>(P, S, id, c, q, myid, face);
  store_faces(P.mats.m[myid], q, face, fs, c, cnt);
}

// K1b: face states of the face-ghost cells by boundary condition
// (Reconstructor.cpp:807-889), then the boundary branch of
// CheckReconstructedStates (SpaceOperator.cpp:2486-2535).
__device__ __forceinline__ void k_reconstruct_ghosts_body(const Params& P, const StateSet& S, const int32_t* __restrict__ id, double* const* fs, unsigned long long* cnt, unsigned bx_, unsigned gx_) {
  int side, i, j, k, ii, jj, kk;
  if (!ghost_face_cell(P.g, (int64_t)bx_ * blockDim.x + threadIdx.x, side, i, j, k, ii, jj, kk)) return;
  const Grid& g = P.g;
  int64_t c = g.at(i, j, k), im = g.at(ii, jj, kk);
  int inward = side ^ 1, src = side;
  int bc = P.bc[side];
  double t[5];
  if (bc == M2CG_BC_INLET || bc == M2CG_BC_INLET2) {
#pragma unroll
    for (int p = 0; p < 5; p++) t[p] = S.q[p][c];
  } else {
#pragma unroll
    for (int p = 0; p < 5; p++) t[p] = fs[src * 5 + p][im];
    if (bc == M2CG_BC_SYMMETRY || bc == M2CG_BC_SLIPWALL) t[1 + side / 2] *= -1.0;
    else if (bc == M2CG_BC_STICKWALL) { t[1] *= -1.0; t[2] *= -1.0; t[3] *= -1.0; }
  }
  const DevMat& M = P.mats.m[id[c]];
  double u[5] = {t[0], t[1], t[2], t[3], t[4]};
  if (eos_clip(M, u)) {
#pragma unroll
    for (int p = 0; p < 5; p++) t[p] = S.q[p][c];
    atomic_inc(&cnt[CNT_CLIPFACE]);
  }
  if (eos_bad5(M, t)) atomic_inc(&cnt[CNT_BAD]);
#pragma unroll
  for (int p = 0; p < 5; p++) fs[inward * 5 + p][c] = t[p];
}
__global__ void k_reconstruct_ghosts(Params P, StateSet S, const int32_t* __restrict__ id, double* const* fs,
                                     unsigned long long* cnt) { k_reconstruct_ghosts_body(P, S, id, fs, cnt, blockIdx.x, gridDim.x); }
// batched: the launch's blocks are the members' blocks back to back
// (boff: exclusive prefix of the members' block counts)
__global__ void k_reconstruct_ghosts_ens(const k_reconstruct_ghosts_args* __restrict__ ea, const int64_t* __restrict__ boff, int D) {
  const int d = ens_member(boff, D, blockIdx.x);
  const k_reconstruct_ghosts_args& e = ea[d];
  k_reconstruct_ghosts_body(e.P, e.S, e.id, e.fs, e.cnt, (unsigned)(blockIdx.x - boff[d]), (unsigned)(boff[d + 1] - boff[d]));
}


__device__ __forceinline__ bool num_flux(const Params& P, int dir, const double* Vm, const double* Vp, int id, double* F) {
  const DevMat& M = P.mats.m[id];
  if (P.flux == M2CG_FLUX_HLLC) return flux_hllc_fast(M, dir, Vm, Vp, F);
  if (P.flux == M2CG_FLUX_LLF) return flux_llf2(M, M, dir, Vm, Vp, F);
  return flux_genroe(M, dir, Vm, Vp, P.roe_delta, F);
}

// ---------------------------------------------------------------------------
// K2: numerical flux of every same-material face (SpaceOperator.cpp:1692-1701,
// 1852-1861, 2011-2020).  The thread of cell c owns the faces at its minus side.
__device__ __forceinline__ void k_face_flux_body(const Params& P, const int32_t* __restrict__ id, double* const* fs, double* const* F, unsigned long long* cnt, unsigned bx_, unsigned gx_) {
  const Grid& g = P.g;
  int i, j, k;
  if (g.tile[0]) {
    if (!tiled_index(g.nx + 1, g.ny + 1, g.nz + 1, g.tile, bx_, threadIdx.x, i, j, k)) return;
  } else {
    int64_t t = (int64_t)bx_ * blockDim.x + threadIdx.x;
    int64_t ex = g.nx + 1, ey = g.ny + 1;
    int64_t n = ex * ey * (g.nz + 1);
    if (t >= n) return;
    k = (int)(t / (ex * ey));
    int64_t r = t - (int64_t)k * ex * ey;
    j = (int)(r / ex);
    i = (int)(r - (int64_t)j * ex);
  }
  int64_t c = g.at(i, j, k);
  const int64_t st[3] = {1, g.sy, g.sz};
  bool has[3] = {j < g.ny && k < g.nz, i < g.nx && k < g.nz, i < g.nx && j < g.ny};
  int myid = id[c];
  int bad = 0;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (!has[d]) continue;
    int64_t m = c - st[d];
    if (id[m] != myid) continue;  // material interface: exact Riemann kernel
    double Vm[5], Vp[5], Fl[5];
#pragma unroll
    for (int p = 0; p < 5; p++) { Vm[p] = fs[(2 * d + 1) * 5 + p][m]; Vp[p] = fs[(2 * d) * 5 + p][c]; }
    bad += !num_flux(P, d, Vm, Vp, myid, Fl);
#pragma unroll
    for (int p = 0; p < 5; p++) F[d * 5 + p][c] = Fl[p];
  }
  if (bad) atomic_inc(&cnt[CNT_BAD], bad);
}
__global__ void __launch_bounds__(128) k_face_flux(Params P, const int32_t* __restrict__ id, double* const* fs, double* const* F,
                            unsigned long long* cnt) { k_face_flux_body(P, id, fs, F, cnt, blockIdx.x, gridDim.x); }
// batched: the launch's blocks are the members' blocks back to back
// (boff: exclusive prefix of the members' block counts)
__global__ void __launch_bounds__(128) k_face_flux_ens(const k_face_flux_args* __restrict__ ea, const int64_t* __restrict__ boff, int D, int64_t nvb) {
  // persistent: the launch's blocks take the members' blocks in turn
  for (int64_t b = blockIdx.x; b < nvb; b += gridDim.x) {
    const int d = ens_member(boff, D, b);
    const k_face_flux_args& e = ea[d];
    k_face_flux_body(e.P, e.id, e.fs, e.F, e.cnt, (unsigned)(b - boff[d]), (unsigned)(boff[d + 1] - boff[d]));
  }
}


// ---------------------------------------------------------------------------
// Level-set residual at one cell: LevelSetOperator.cpp:834-852 with the FD3
// coefficients of GradientCalculatorFD3.cpp:300-453 (uniform mesh).
__device__ __forceinline__ double ls_residual(const Params& P, const double* __restrict__ phi, int64_t c, int i, int j,
                                              int k, const double vel[3]) {
  const Grid& g = P.g;
  const int64_t st[3] = {1, g.sy, g.sz};
  const int pos[3] = {i, j, k};
  const int n[3] = {g.nx, g.ny, g.nz};
  const double h[3] = {g.dx, g.dy, g.dz};
  double term[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    int64_t s = st[d];
    double gr;
    if (vel[d] >= 0) {
      if (pos[d] - 2 >= -1)
        gr = P.fd3l[d][0] * phi[c - 2 * s] + P.fd3l[d][1] * phi[c - s] + P.fd3l[d][2] * phi[c] + P.fd3l[d][3] * phi[c + s];
      else
        gr = (phi[c] - phi[c - s]) / h[d];
    } else {
      if (pos[d] + 2 <= n[d]) {
        // the reference's right-biased y coefficients are 3rd order only when
        // i < NY-1 (GradientCalculatorFD3.cpp:409 tests i, not j)
        bool third = (d == 1) ? (i < g.ny - 1) : (pos[d] < n[d] - 1);
        if (third)
          gr = P.fd3r[d][0] * phi[c - s] + P.fd3r[d][1] * phi[c] + P.fd3r[d][2] * phi[c + s] + P.fd3r[d][3] * phi[c + 2 * s];
        else
          gr = 0.0 * phi[c - s] + (-1.0 / h[d]) * phi[c] + (1.0 / h[d]) * phi[c + s] + 0.0 * phi[c + 2 * s];
      } else
        gr = (phi[c + s] - phi[c]) / h[d];
    }
    term[d] = gr * vel[d];
  }
  return (term[0] + term[1] + term[2]) * -1.0;
}

// ---------------------------------------------------------------------------
// K3: residual gather in the reference's accumulation order
// (SpaceOperator.cpp:1703-1705, 1863-1865, 2022-2024, then r /= -vol at
// 2628-2632), the Runge-Kutta stage combination with clipping
// (TimeIntegrator.cpp:355-369, 409-417, 565-579, 617-631, 667-676), the
// level-set stage update and, on the final stage, the sign-change detection of
// MultiPhaseOperator::UpdateMaterialIDByLevelSet (MultiPhaseOperator.cpp:177-222).
__device__ __forceinline__ void k_update_body(const Params& P, const StageArgs& A, const int32_t* __restrict__ id, int32_t* __restrict__ id_new, double* const* F, const IfaceList& L, const DevScalars* __restrict__ sc, int64_t* __restrict__ swept, unsigned long long* swept_count, int64_t swept_cap, unsigned long long* cnt, unsigned bx_, unsigned gx_) {
  int i, j, k;
  if (!block_cell(P.g, bx_, i, j, k)) return;
  if (!sc->active && !A.residual_only) return;
  const Grid& g = P.g;
  int64_t c = g.at(i, j, k);
  const int64_t st[3] = {1, g.sy, g.sz};
  int myid = id[c];
  // f = sum_d (F(c + 1/2 e_d) - F(c - 1/2 e_d)) * A_d.  The reference accumulates
  // -F_minus*A (x, y, z) then +F_plus*A (SpaceOperator.cpp:1703-1705, 1863-1865,
  // 2022-2024); differencing first gives the same value to rounding and an exact
  // zero wherever the two fluxes of a direction are equal, as the reference does
  // for a uniform flux.
  double f[5] = {0, 0, 0, 0, 0};
#pragma unroll
  for (int d = 0; d < 3; d++) {
    int64_t m = c - st[d], pc = c + st[d];
    const double a = P.area[d];
    double fm[5], fp[5];
    if (id[m] != myid) {
      int s = L.slot[d][c];
#pragma unroll
      for (int p = 0; p < 5; p++) fm[p] = L.lf2[p][s];
    } else {
#pragma unroll
      for (int p = 0; p < 5; p++) fm[p] = F[d * 5 + p][c];
    }
    if (id[pc] != myid) {
      int s = L.slot[d][pc];
#pragma unroll
      for (int p = 0; p < 5; p++) fp[p] = L.lf1[p][s];
    } else {
#pragma unroll
      for (int p = 0; p < 5; p++) fp[p] = F[d * 5 + p][pc];
    }
#pragma unroll
    for (int p = 0; p < 5; p++) f[p] += (fp[p] - fm[p]) * a;
  }
  double R[5];
#pragma unroll
  for (int p = 0; p < 5; p++) R[p] = f[p] * P.inv_negvol;
  if (A.residual_only) {
#pragma unroll
    for (int p = 0; p < 5; p++) A.R[p][c] = R[p];
    return;
  }
  const double dt = sc->dt;
  const DevMat& M = P.mats.m[myid];
  double U[5];
  if (A.stage == 0) {
    double Vn[5], Un[5];
#pragma unroll
    for (int p = 0; p < 5; p++) Vn[p] = A.in.q[p][c];
    prim_to_cons_fast(M, Vn, Un);
    if (A.store_un) {
#pragma unroll
      for (int p = 0; p < 5; p++) A.Un[p][c] = Un[p];
    }
#pragma unroll
    for (int p = 0; p < 5; p++) U[p] = Un[p] + dt * R[p];
  } else {
    const double cdt = A.c_dt * dt;
#pragma unroll
    for (int p = 0; p < 5; p++) U[p] = (A.a_own * A.Us[p][c] + A.b_un * A.Un[p][c]) + cdt * R[p];
  }
  double V[5];
  cons_to_prim_fast(M, U, V);
  bool clipped = eos_clip_fast(M, V);
  if (clipped) atomic_inc(&cnt[CNT_CLIPCELL]);
  if (eos_bad5_fast(M, V)) atomic_inc(&cnt[CNT_BAD]);
  if (!A.last) {
    if (clipped) prim_to_cons_fast(M, V, U);
#pragma unroll
    for (int p = 0; p < 5; p++) A.Us[p][c] = U[p];
  }
#pragma unroll
  for (int p = 0; p < 5; p++) A.out.q[p][c] = V[p];
  // level set
  if (P.n_ls > 0) {
    double vel[3];
    if (A.ls_use_updated_v) { vel[0] = V[1]; vel[1] = V[2]; vel[2] = V[3]; }
    else { vel[0] = A.in.q[1][c]; vel[1] = A.in.q[2][c]; vel[2] = A.in.q[3][c]; }
    double rls = A.rls_pre ? A.rls_pre[c] : ls_residual(P, A.phi_lsin, c, i, j, k, vel);
    double ph;
    double phin = A.phi_tmp[c];
    if (A.stage == 0) ph = A.phi_own[c] + dt * rls;
    else ph = (A.la * A.phi_own[c] + A.lb * phin) + (A.lc * dt) * rls;
    A.out.q[5][c] = ph;
    if (A.last) {
      // sign change (MultiPhaseOperator.cpp:190-222) -> new ID or "remaining" tag (negative)
      int nid = myid;
      if (!(ph * phin > 0.0)) {
        if (ph < 0) nid = P.ls_matid;
        else nid = -1 - myid;  // resolved from the neighbors after this kernel
        unsigned long long s = atomicAdd(swept_count, 1ull);
        if ((int64_t)s < swept_cap) swept[s] = c;
        else atomic_inc(&cnt[CNT_SWEPT_OVERFLOW]);
      }
      id_new[c] = nid;
    }
  } else if (A.last) {
    id_new[c] = myid;
  }
}
__global__ void k_update(Params P, StageArgs A, const int32_t* __restrict__ id, int32_t* __restrict__ id_new,
                         double* const* F, IfaceList L, const DevScalars* __restrict__ sc,
                         int64_t* __restrict__ swept, unsigned long long* swept_count, int64_t swept_cap,
                         unsigned long long* cnt) { k_update_body(P, A, id, id_new, F, L, sc, swept, swept_count, swept_cap, cnt, blockIdx.x, gridDim.x); }
// batched: the launch's blocks are the members' blocks back to back
// (boff: exclusive prefix of the members' block counts)
__global__ void k_update_ens(const k_update_args* __restrict__ ea, const int64_t* __restrict__ boff, int D, int64_t nvb) {
  // persistent: the launch's blocks take the members' blocks in turn
  for (int64_t b = blockIdx.x; b < nvb; b += gridDim.x) {
    const int d = ens_member(boff, D, b);
    const k_update_args& e = ea[d];
    k_update_body(e.P, e.A, e.id, e.id_new, e.F, e.L, e.sc, e.swept, e.swept_count, e.swept_cap, e.cnt, (unsigned)(b - boff[d]), (unsigned)(boff[d + 1] - boff[d]));
  }
}


// Level-set residual only (LevelSetOperator::ComputeResidual).
// ---------------------------------------------------------------------------
// Finite-volume level set at one real cell (LevelSetOperator.cpp:966-1136,
// 1265-1324): face values from the level set's own reconstruction -- each
// velocity component along its direction (Reconstructor.cpp:922-1176) and phi
// (Reconstructor.cpp:335-918 with one DOF) -- for the cell and its neighbours,
// the neighbours beyond the boundary taking the ghost cells' inward values by
// boundary type; R = (F_lo,x + G_lo,y + H_lo,z - F_hi,x - G_hi,y - H_hi,z) +
// phi div(u), the reference's accumulation order.
__device__ __forceinline__ double ls_limit(const Params& P, double dq0, double dq1) {
  if (!P.ls_rec_linear) return 0.0;
  if (P.ls_limiter == M2CG_LIM_GENERALIZED_MINMOD) return gen_minmod(P.ls_minmod, dq0, dq1);
  if (P.ls_limiter == M2CG_LIM_VANALBADA) return van_albada_fast(dq0, dq1);
  return 0.5 * (dq0 + dq1);
}
__device__ __forceinline__ double ls_slope(const Params& P, const double* __restrict__ q, int64_t c, int64_t s) {
  return ls_limit(P, q[c] - q[c - s], q[c + s] - q[c]);
}
__device__ __forceinline__ double ls_fv_flux(const Params& P, double phim, double phip, double um, double up) {
  if (P.ls_flux == M2CG_LSFLUX_UPWIND) {
    const double vmid = 0.5 * (um + up);
    if (vmid > 0) return phim * um;
    if (vmid < 0) return phip * up;
    return 0.5 * (phim * um + phip * up);
  }
  if (P.ls_flux == M2CG_LSFLUX_LLF) return 0.5 * (phim * um + phip * up) - 0.5 * fmax(fabs(um), fabs(up)) * (phip - phim);
  double lam = fabs(0.5 * (um + up));
  const double tol = fmax(fabs(um), fabs(up)) * P.ls_delta;
  if (lam < tol) lam = (lam * lam + tol * tol) / (2 * tol);
  return 0.5 * (phim * um + phip * up) - 0.5 * lam * (phip - phim);
}
__device__ __forceinline__ double ls_fv_residual(const Params& P, const StateSet& S, int64_t c, int i, int j, int k) {
  const Grid& g = P.g;
  const int64_t st[3] = {1, g.sy, g.sz};
  const int pos[3] = {i, j, k};
  const int n[3] = {g.nx, g.ny, g.nz};
  const double h[3] = {g.dx, g.dy, g.dz};
  const double* __restrict__ phi = S.q[5];
  double flo[3], fhi[3], div = 0.0;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const double* __restrict__ u = S.q[1 + d];
    const int64_t s = st[d];
    const double su = ls_slope(P, u, c, s), sp = ls_slope(P, phi, c, s);
    div += su / h[d];
    const double u_m = u[c] - 0.5 * su, u_p = u[c] + 0.5 * su;
    const double p_m = phi[c] - 0.5 * sp, p_p = phi[c] + 0.5 * sp;
    double nu, np;
    if (pos[d] > 0) {
      nu = u[c - s] + 0.5 * ls_slope(P, u, c - s, s);
      np = phi[c - s] + 0.5 * ls_slope(P, phi, c - s, s);
    } else {   // the low ghost's inward values; its image is this cell
      const int bc = P.bc[2 * d];
      const bool inlet = (bc == M2CG_BC_INLET || bc == M2CG_BC_INLET2);
      nu = inlet ? u[c - s] : (bc == M2CG_BC_OUTLET ? u_m : -u_m);
      np = (inlet || !P.ls_rec_linear) ? phi[c - s] : p_m;
    }
    flo[d] = ls_fv_flux(P, np, p_m, nu, u_m) / h[d];
    if (pos[d] < n[d] - 1) {
      nu = u[c + s] - 0.5 * ls_slope(P, u, c + s, s);
      np = phi[c + s] - 0.5 * ls_slope(P, phi, c + s, s);
    } else {   // the high ghost's inward values
      const int bc = P.bc[2 * d + 1];
      const bool inlet = (bc == M2CG_BC_INLET || bc == M2CG_BC_INLET2);
      nu = inlet ? u[c + s] : (bc == M2CG_BC_OUTLET ? u_p : -u_p);
      np = (inlet || !P.ls_rec_linear) ? phi[c + s] : p_p;
    }
    fhi[d] = ls_fv_flux(P, p_p, np, u_p, nu) / h[d];
  }
  double r = flo[0];
  r += flo[1];
  r += flo[2];
  r -= fhi[0];
  r -= fhi[1];
  r -= fhi[2];
  return r + phi[c] * div;
}

__global__ void k_ls_residual(Params P, StateSet S, double* __restrict__ out) {
  int i, j, k;
  if (!real_cell(P.g, (int64_t)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
  int64_t c = P.g.at(i, j, k);
  if (P.ls_fv) {
    out[c] = ls_fv_residual(P, S, c, i, j, k);
    return;
  }
  double vel[3] = {S.q[1][c], S.q[2][c], S.q[3][c]};
  out[c] = ls_residual(P, S.q[5], c, i, j, k, vel);
}

// ---------------------------------------------------------------------------
// Boundary conditions on the face-ghost cells: SpaceOperator.cpp:738-821 (V),
// LevelSetOperator.cpp:408-508 (phi), MultiPhaseOperator.cpp:919-942 (ID).
__device__ __forceinline__ void k_bc_body(const Params& P, const StateSet& S, int do_v, int do_phi, int32_t* id, const DevScalars* sc, unsigned bx_, unsigned gx_) {
  int side, i, j, k, ii, jj, kk;
  if (!ghost_face_cell(P.g, (int64_t)bx_ * blockDim.x + threadIdx.x, side, i, j, k, ii, jj, kk)) return;
  if (sc && !sc->active) return;
  const Grid& g = P.g;
  int64_t c = g.at(i, j, k), im = g.at(ii, jj, kk);
  if (do_v) {
    int bc = P.bc[side];
    if (bc == M2CG_BC_INLET) {
#pragma unroll
      for (int p = 0; p < 5; p++) S.q[p][c] = P.inlet[p];
    } else if (bc == M2CG_BC_INLET2) {
#pragma unroll
      for (int p = 0; p < 5; p++) S.q[p][c] = P.inlet2[p];
    } else {
      double t[5];
#pragma unroll
      for (int p = 0; p < 5; p++) t[p] = S.q[p][im];
      if (bc == M2CG_BC_SYMMETRY || bc == M2CG_BC_SLIPWALL) t[1 + side / 2] *= -1.0;
      else if (bc == M2CG_BC_STICKWALL) { t[1] = -1.0 * t[1]; t[2] = -1.0 * t[2]; t[3] = -1.0 * t[3]; }
#pragma unroll
      for (int p = 0; p < 5; p++) S.q[p][c] = t[p];
    }
  }
  if (do_phi && P.n_ls > 0) {
    double* phi = S.q[5];
    int bc = P.ls_bc[side];
    if (bc == M2CG_LSBC_ZERO_NEUMANN) phi[c] = phi[im];
    else {
      int d = side / 2, sgn = (side % 2 == 0) ? 1 : -1;
      int pos[3] = {i, j, k};
      int n[3] = {g.nx, g.ny, g.nz};
      const double h[3] = {g.dx, g.dy, g.dz};
      const int64_t st[3] = {1, g.sy, g.sz};
      bool ok = (sgn > 0) ? (pos[d] + 2 < n[d]) : (pos[d] - 2 >= 0);
      double v;
      if (ok) {
        double r = pos[d] * h[d], r1 = (pos[d] + sgn) * h[d], r2 = (pos[d] + 2 * sgn) * h[d];
        double f1 = phi[c + sgn * st[d]], f2 = phi[c + 2 * sgn * st[d]];
        v = f1 + (f2 - f1) / (r2 - r1) * (r - r1);
      } else v = phi[im];
      if (bc == M2CG_LSBC_NON_NEGATIVE) v = fmax(-0.5 * h[d], v);
      phi[c] = v;
    }
  }
  if (id) id[c] = id[im];
}
__global__ void k_bc(Params P, StateSet S, int do_v, int do_phi, int32_t* id, const DevScalars* sc) { k_bc_body(P, S, do_v, do_phi, id, sc, blockIdx.x, gridDim.x); }
// batched: the launch's blocks are the members' blocks back to back
// (boff: exclusive prefix of the members' block counts)
__global__ void k_bc_ens(const k_bc_args* __restrict__ ea, const int64_t* __restrict__ boff, int D) {
  const int d = ens_member(boff, D, blockIdx.x);
  const k_bc_args& e = ea[d];
  k_bc_body(e.P, e.S, e.do_v, e.do_phi, e.id, e.sc, (unsigned)(blockIdx.x - boff[d]), (unsigned)(boff[d + 1] - boff[d]));
}


// ---------------------------------------------------------------------------
// CFL time step: FindExtremeValuesOfFlowVariables + ComputeTimeStepSize
// (SpaceOperator.cpp:1223-1330).  Warp-shuffle min, then one atomicMin per block
// on the bit pattern of the positive minimum.
__device__ __forceinline__ void k_dt_reduce_body(const Params& P, const StateSet& S, const int32_t* __restrict__ id, DevScalars* sc, unsigned bx_, unsigned gx_) {
  int i, j, k;
  double m = DBL_MAX;
  if (real_cell(P.g, (int64_t)bx_ * blockDim.x + threadIdx.x, i, j, k)) {
    const Grid& g = P.g;
    int64_t c = g.at(i, j, k);
    const DevMat& M = P.mats.m[id[c]];
    double V[5] = {S.q[0][c], S.q[1][c], S.q[2][c], S.q[3][c], S.q[4][c]};
    Side sd;
    side_eos(M, V, 0, sd);
    double cc = sd.c;
    if (g.h_common > 0.0) {
      // one spacing on every active axis: min_d h / (|u_d| + c) = h / (max_d |u_d| + c),
      // one reciprocal instead of three
      double v = 0.0;
      if (g.nx > 1) v = fabs(V[1]);
      if (g.ny > 1) v = fmax(v, fabs(V[2]));
      if (g.nz > 1) v = fmax(v, fabs(V[3]));
      m = g.h_common * rcp_fast(v + cc);
    } else {
      if (g.nx > 1) m = fmin(m, g.dx * rcp_fast(fabs(V[1]) + cc));
      if (g.ny > 1) m = fmin(m, g.dy * rcp_fast(fabs(V[2]) + cc));
      if (g.nz > 1) m = fmin(m, g.dz * rcp_fast(fabs(V[3]) + cc));
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmin(m, __shfl_xor_sync(0xffffffffu, m, o));
  __shared__ double wmin[32];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) wmin[w] = m;
  __syncthreads();
  if (w == 0) {
    int nw = (blockDim.x + 31) >> 5;
    m = lane < nw ? wmin[lane] : DBL_MAX;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmin(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0 && m < DBL_MAX) atomicMin(&sc->min_dx_over_lambda, (unsigned long long)__double_as_longlong(m));
  }
}
__global__ void k_dt_reduce(Params P, StateSet S, const int32_t* __restrict__ id, DevScalars* sc) { k_dt_reduce_body(P, S, id, sc, blockIdx.x, gridDim.x); }
// batched: the launch's blocks are the members' blocks back to back
// (boff: exclusive prefix of the members' block counts)
__global__ void k_dt_reduce_ens(const k_dt_reduce_args* __restrict__ ea, const int64_t* __restrict__ boff, int D) {
  const int d = ens_member(boff, D, blockIdx.x);
  const k_dt_reduce_args& e = ea[d];
  k_dt_reduce_body(e.P, e.S, e.id, e.sc, (unsigned)(blockIdx.x - boff[d]), (unsigned)(boff[d + 1] - boff[d]));
}


// dt, cfl and the MaxTime clamp of Main.cpp:653-681, kept on the device.
// mode 0: query (dt and cfl only); 1: CFL-driven step; 2: step with a given dt.
__device__ __forceinline__ void k_dt_finalize_body(const Params& P, DevScalars* sc, int mode, double fixed_dt, unsigned bx_, unsigned gx_) {
  double m = __longlong_as_double((long long)sc->min_dx_over_lambda);
  sc->min_dx_over_lambda = 0x7fefffffffffffffull;  // DBL_MAX for the next reduction
  double dt, cfl;
  if (mode == 2) { dt = fixed_dt; cfl = dt / m; }
  else if (mode == 3) { dt = sc->dt_in; cfl = dt / m; }   // mode 2 with the step given on the device
  else if (P.timestep > 0) { dt = P.timestep; cfl = dt / m; }
  else { cfl = P.cfl; dt = cfl * m; }
  if (mode == 0) { sc->dt = dt; sc->cfl = cfl; return; }
  double t = sc->time;
  if (mode == 1) {
    if (!(t < P.max_time - 1.0e-6 * dt)) { sc->active = 0; return; }
    if (t + dt > P.max_time) { cfl *= (P.max_time - t) / dt; dt = P.max_time - t; }
  }
  sc->active = 1;
  sc->dt = dt;
  sc->cfl = cfl;
  sc->time = t + dt;
  sc->steps += 1;
}
__global__ void k_dt_finalize(Params P, DevScalars* sc, int mode, double fixed_dt) { k_dt_finalize_body(P, sc, mode, fixed_dt, blockIdx.x, gridDim.x); }
// batched: the launch's blocks are the members' blocks back to back
// (boff: exclusive prefix of the members' block counts)
__global__ void k_dt_finalize_ens(const k_dt_finalize_args* __restrict__ ea, const int64_t* __restrict__ boff, int D) {
  const int d = ens_member(boff, D, blockIdx.x);
  const k_dt_finalize_args& e = ea[d];
  k_dt_finalize_body(e.P, e.sc, e.mode, e.fixed_dt, (unsigned)(blockIdx.x - boff[d]), (unsigned)(boff[d + 1] - boff[d]));
}


// ---------------------------------------------------------------------------
// End of step.  "Remaining" swept cells (phi >= 0 after a sign change) take the
// smallest material ID among their 26 neighbors that are decided and not the
// level-set material (MultiPhaseOperator.cpp:236-340).  Jacobi passes: each
// pass decides from the previous pass's IDs; the reference resolves in
// lexicographic order within a pass.
__device__ __forceinline__ void k_resolve_remaining_body(const Params& P, int32_t* id_new, const int64_t* swept, const unsigned long long* count, int64_t cap, int32_t* cand_out, int final_pass, const DevScalars* sc, unsigned bx_, unsigned gx_) {
  if (!sc->active) return;
  int64_t n = (int64_t)min((unsigned long long)cap, *count);
  const Grid& g = P.g;
  for (int64_t s = (int64_t)bx_ * blockDim.x + threadIdx.x; s < n; s += (int64_t)gx_ * blockDim.x) {
    int64_t c = swept[s];
    int cur = id_new[c];
    if (cur >= 0) { cand_out[s] = cur; continue; }
    int64_t r = c;
    int i = (int)(r % g.px) - 1; r /= g.px;
    int j = (int)(r % g.py) - 1;
    int k = (int)(r / g.py) - 1;
    int best = 0x7fffffff;
    for (int nk = k - 1; nk <= k + 1; nk++)
      for (int nj = j - 1; nj <= j + 1; nj++)
        for (int ni = i - 1; ni <= i + 1; ni++) {
          if (ni < 0 || ni >= g.nx || nj < 0 || nj >= g.ny || nk < 0 || nk >= g.nz) continue;
          int v = id_new[g.at(ni, nj, nk)];
          if (v < 0 || v == P.ls_matid) continue;
          best = min(best, v);
        }
    if (best != 0x7fffffff) cand_out[s] = best;
    else cand_out[s] = final_pass ? 0 : cur;  // orphans become material 0 (MultiPhaseOperator.cpp:327-334)
  }
}
__global__ void k_resolve_remaining(Params P, int32_t* id_new, const int64_t* swept, const unsigned long long* count,
                                    int64_t cap, int32_t* cand_out, int final_pass, const DevScalars* sc) { k_resolve_remaining_body(P, id_new, swept, count, cap, cand_out, final_pass, sc, blockIdx.x, gridDim.x); }
// batched: the launch's blocks are the members' blocks back to back
// (boff: exclusive prefix of the members' block counts)
__global__ void k_resolve_remaining_ens(const k_resolve_remaining_args* __restrict__ ea, const int64_t* __restrict__ boff, int D) {
  const int d = ens_member(boff, D, blockIdx.x);
  const k_resolve_remaining_args& e = ea[d];
  k_resolve_remaining_body(e.P, e.id_new, e.swept, e.count, e.cap, e.cand_out, e.final_pass, e.sc, (unsigned)(blockIdx.x - boff[d]), (unsigned)(boff[d + 1] - boff[d]));
}


__device__ __forceinline__ void k_commit_remaining_body(int32_t* id_new, const int64_t* swept, const unsigned long long* count, int64_t cap, const int32_t* cand, const DevScalars* sc, unsigned bx_, unsigned gx_) {
  if (!sc->active) return;
  int64_t n = (int64_t)min((unsigned long long)cap, *count);
  for (int64_t s = (int64_t)bx_ * blockDim.x + threadIdx.x; s < n; s += (int64_t)gx_ * blockDim.x)
    id_new[swept[s]] = cand[s];
}
__global__ void k_commit_remaining(int32_t* id_new, const int64_t* swept, const unsigned long long* count, int64_t cap,
                                   const int32_t* cand, const DevScalars* sc) { k_commit_remaining_body(id_new, swept, count, cap, cand, sc, blockIdx.x, gridDim.x); }
// batched: the launch's blocks are the members' blocks back to back
// (boff: exclusive prefix of the members' block counts)
__global__ void k_commit_remaining_ens(const k_commit_remaining_args* __restrict__ ea, const int64_t* __restrict__ boff, int D) {
  const int d = ens_member(boff, D, blockIdx.x);
  const k_commit_remaining_args& e = ea[d];
  k_commit_remaining_body(e.id_new, e.swept, e.count, e.cap, e.cand, e.sc, (unsigned)(blockIdx.x - boff[d]), (unsigned)(boff[d + 1] - boff[d]));
}


// UpdateStateVariablesByRiemannSolutions / LocalUpdateByRiemannSolutions
// (MultiPhaseOperator.cpp:980-1150) or by extrapolation (1155-1274) for every
// swept cell whose ID changed; then ClipDensityAndPressure (TimeIntegrator.cpp:800).
__device__ __forceinline__ void k_swept_update_body(const Params& P, const StateSet& S, const int32_t* __restrict__ id_old, const int32_t* __restrict__ id_new, const IfaceList& L, const int64_t* swept, const unsigned long long* count, int64_t cap, unsigned long long* cnt, const DevScalars* sc, unsigned bx_, unsigned gx_) {
  if (!sc->active) return;
  int64_t n = (int64_t)min((unsigned long long)cap, *count);
  const Grid& g = P.g;
  const int64_t st[3] = {1, g.sy, g.sz};
  for (int64_t s = (int64_t)bx_ * blockDim.x + threadIdx.x; s < n; s += (int64_t)gx_ * blockDim.x) {
    int64_t c = swept[s];
    int myid = id_new[c];
    if (myid == id_old[c]) continue;
    atomic_inc(&cnt[CNT_SWEPT]);
    double out[5];
    int counter = 0;
    if (P.mp_phasechange == M2CG_PHASECHANGE_RIEMANN) {
      for (int pass = 0; pass < 2 && counter == 0; pass++) {
        bool upwind = (pass == 0);
        double acc[5] = {0, 0, 0, 0, 0};
        double sum_w = 0.0;
        for (int d = 0; d < 3; d++)
          for (int side = 0; side < 2; side++) {
            int64_t fc = side == 0 ? c : c + st[d];
            int64_t nb = side == 0 ? c - st[d] : c + st[d];
            int idm = id_old[fc - st[d]], idp = id_old[fc];
            if (idm == idp) continue;           // not an interface face this step
            int sl = L.slot[d][fc];
            if (L.err[sl]) continue;            // solution not stored on failure
            int sid = side == 0 ? idm : idp;
            if (sid != myid) continue;
            double vel = S.q[1 + d][nb];
            bool upw_ok = side == 0 ? (vel > 0) : (vel < 0);
            if (upwind && !upw_ok) continue;
            double vx = S.q[1][nb], vy = S.q[2][nb], vz = S.q[3][nb];
            double nrm = sqrt(vx * vx + vy * vy + vz * vz);
            double w = upwind ? (side == 0 ? vel / nrm : -vel / nrm) : 1.0;
            sum_w += w;
            for (int p = 0; p < 5; p++) {
              double sv = side == 0 ? L.vsm[p][sl] : L.vsp[p][sl];
              if (counter == 0) acc[p] = w * sv;
              else acc[p] += w * sv;
            }
            counter++;
          }
        if (counter > 0) {
          if (sum_w > 0.0) { double inv = 1.0 / sum_w; for (int p = 0; p < 5; p++) out[p] = acc[p] * inv; }
          else for (int p = 0; p < 5; p++) out[p] = acc[p];
        }
      }
    } else {
      int64_t r = c;
      int i = (int)(r % g.px) - 1; r /= g.px;
      int j = (int)(r % g.py) - 1;
      int k = (int)(r / g.py) - 1;
      double sum_w = 0.0, vs[5] = {0, 0, 0, 0, 0};
      const double h[3] = {g.dx, g.dy, g.dz};
      for (int nk = k - 1; nk <= k + 1; nk++)
        for (int nj = j - 1; nj <= j + 1; nj++)
          for (int ni = i - 1; ni <= i + 1; ni++) {
            int64_t nc = g.at(ni, nj, nk);
            if (id_new[nc] != myid) continue;
            if (id_new[nc] != id_old[nc]) continue;
            if (ni < 0 || ni >= g.nx || nj < 0 || nj >= g.ny || nk < 0 || nk >= g.nz) continue;
            double x[3] = {(i - ni) * h[0], (j - nj) * h[1], (k - nk) * h[2]};
            double dist = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
            double w;
            if (P.mp_pcdir == M2CG_PCDIR_ALL) w = 1.0 / dist;
            else {
              double v1[3] = {S.q[1][nc], S.q[2][nc], S.q[3][nc]};
              double vn = sqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
              if (vn != 0) for (int m = 0; m < 3; m++) v1[m] /= vn;
              for (int m = 0; m < 3; m++) x[m] /= dist;
              w = fmax(0.0, x[0] * v1[0] + x[1] * v1[1] + x[2] * v1[2]);
            }
            if (w > 0) { sum_w += w; for (int p = 0; p < 5; p++) vs[p] += w * S.q[p][nc]; }
          }
      if (sum_w > 0) { counter = 1; for (int p = 0; p < 5; p++) out[p] = vs[p] / sum_w; }
    }
    if (counter == 0) {
      atomic_inc(&cnt[CNT_UNRES]);
      if (P.unres) {
        const unsigned long long u = atomicAdd(P.unres_count, 1ull);
        if (u < (unsigned long long)P.unres_cap) P.unres[u] = c;
      }
      continue;
    }
    const DevMat& M = P.mats.m[myid];
    eos_clip(M, out);
    if (eos_bad5(M, out)) atomic_inc(&cnt[CNT_BAD]);
    for (int p = 0; p < 5; p++) S.q[p][c] = out[p];
  }
}
__global__ void k_swept_update(Params P, StateSet S, const int32_t* __restrict__ id_old, const int32_t* __restrict__ id_new,
                               IfaceList L, const int64_t* swept, const unsigned long long* count, int64_t cap,
                               unsigned long long* cnt, const DevScalars* sc) { k_swept_update_body(P, S, id_old, id_new, L, swept, count, cap, cnt, sc, blockIdx.x, gridDim.x); }
// batched: the launch's blocks are the members' blocks back to back
// (boff: exclusive prefix of the members' block counts)
__global__ void k_swept_update_ens(const k_swept_update_args* __restrict__ ea, const int64_t* __restrict__ boff, int D) {
  const int d = ens_member(boff, D, blockIdx.x);
  const k_swept_update_args& e = ea[d];
  k_swept_update_body(e.P, e.S, e.id_old, e.id_new, e.L, e.swept, e.count, e.cap, e.cnt, e.sc, (unsigned)(blockIdx.x - boff[d]), (unsigned)(boff[d + 1] - boff[d]));
}


__device__ __forceinline__ void k_commit_ids_body(int32_t* id, const int32_t* id_new, const int64_t* swept, const unsigned long long* count, int64_t cap, const DevScalars* sc, unsigned bx_, unsigned gx_) {
  if (!sc->active) return;
  int64_t n = (int64_t)min((unsigned long long)cap, *count);
  for (int64_t s = (int64_t)bx_ * blockDim.x + threadIdx.x; s < n; s += (int64_t)gx_ * blockDim.x)
    id[swept[s]] = id_new[swept[s]];
}
__global__ void k_commit_ids(int32_t* id, const int32_t* id_new, const int64_t* swept, const unsigned long long* count,
                             int64_t cap, const DevScalars* sc) { k_commit_ids_body(id, id_new, swept, count, cap, sc, blockIdx.x, gridDim.x); }
// batched: the launch's blocks are the members' blocks back to back
// (boff: exclusive prefix of the members' block counts)
__global__ void k_commit_ids_ens(const k_commit_ids_args* __restrict__ ea, const int64_t* __restrict__ boff, int D) {
  const int d = ens_member(boff, D, blockIdx.x);
  const k_commit_ids_args& e = ea[d];
  k_commit_ids_body(e.id, e.id_new, e.swept, e.count, e.cap, e.sc, (unsigned)(blockIdx.x - boff[d]), (unsigned)(boff[d + 1] - boff[d]));
}


// ---------------------------------------------------------------------------
// Interface-face compaction: every face whose two cells carry different IDs
// (SpaceOperator.cpp:1613, 1772, 1931) gets a slot in the work list.
__device__ __forceinline__ void k_compact_interfaces_body(const Params& P, const int32_t* __restrict__ id, const IfaceList& L, unsigned long long* cnt, const DevScalars* sc, unsigned bx_, unsigned gx_) {
  if (sc && !sc->active) return;
  const Grid& g = P.g;
  int64_t t = (int64_t)bx_ * blockDim.x + threadIdx.x;
  int64_t ex = g.nx + 1, ey = g.ny + 1;
  int64_t n = ex * ey * (g.nz + 1);
  bool valid = t < n;
  int i = 0, j = 0, k = 0;
  if (valid) {
    k = (int)(t / (ex * ey));
    int64_t r = t - (int64_t)k * ex * ey;
    j = (int)(r / ex); i = (int)(r - (int64_t)j * ex);
  }
  const int64_t st[3] = {1, g.sy, g.sz};
  for (int d = 0; d < 3; d++) {
    bool is_if = false;
    int64_t c = 0;
    if (valid) {
      bool has = d == 0 ? (j < g.ny && k < g.nz) : d == 1 ? (i < g.nx && k < g.nz) : (i < g.nx && j < g.ny);
      c = g.at(i, j, k);
      is_if = has && id[c - st[d]] != id[c];
    }
    // warp-aggregated slot allocation
    unsigned mask = __ballot_sync(0xffffffffu, is_if);
    if (!mask) continue;
    int lane = threadIdx.x & 31;
    int leader = __ffs(mask) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(L.count, (unsigned long long)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (is_if) {
      unsigned long long s = base + __popc(mask & ((1u << lane) - 1u));
      if ((int64_t)s < L.cap) {
        L.face[s] = c * 4 + d;
        L.slot[d][c] = (int32_t)s;
      } else if (lane == leader) {
        atomic_inc(&cnt[CNT_IF_OVERFLOW]);
      }
    }
  }
}
__global__ void k_compact_interfaces(Params P, const int32_t* __restrict__ id, IfaceList L, unsigned long long* cnt,
                                     const DevScalars* sc) { k_compact_interfaces_body(P, id, L, cnt, sc, blockIdx.x, gridDim.x); }
// batched: the launch's blocks are the members' blocks back to back
// (boff: exclusive prefix of the members' block counts)
__global__ void k_compact_interfaces_ens(const k_compact_interfaces_args* __restrict__ ea, const int64_t* __restrict__ boff, int D) {
  const int d = ens_member(boff, D, blockIdx.x);
  const k_compact_interfaces_args& e = ea[d];
  k_compact_interfaces_body(e.P, e.id, e.L, e.cnt, e.sc, (unsigned)(blockIdx.x - boff[d]), (unsigned)(boff[d + 1] - boff[d]));
}


// Sum of U * vol over real cells (conserved totals), per block partials.
__global__ void k_conserved(Params P, StateSet S, const int32_t* __restrict__ id, double* partial) {
  int i, j, k;
  double u[5] = {0, 0, 0, 0, 0};
  if (real_cell(P.g, (int64_t)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) {
    int64_t c = P.g.at(i, j, k);
    double V[5] = {S.q[0][c], S.q[1][c], S.q[2][c], S.q[3][c], S.q[4][c]};
    prim_to_cons(P.mats.m[id[c]], V, u);
  }
  __shared__ double red[5][256];
  for (int p = 0; p < 5; p++) red[p][threadIdx.x] = u[p];
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o)
      for (int p = 0; p < 5; p++) red[p][threadIdx.x] += red[p][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int p = 0; p < 5; p++) partial[(int64_t)blockIdx.x * 5 + p] = red[p][0];
}

// Pack / unpack between the AoS host layout (real cells) and the ghosted SoA device layout.
__global__ void k_unpack(Params P, const double* __restrict__ Vh, const int32_t* __restrict__ idh,
                         const double* __restrict__ phih, StateSet S, int32_t* id, unsigned long long* cnt) {
  int i, j, k;
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (!real_cell(P.g, t, i, j, k)) return;
  int64_t c = P.g.at(i, j, k);
  for (int p = 0; p < 5; p++) S.q[p][c] = Vh[t * 5 + p];
  int v = idh[t];
  if (v < 0 || v >= P.n_mat) { atomic_inc(&cnt[CNT_BADID]); v = 0; }
  id[c] = v;
  if (phih) S.q[5][c] = phih[t];
}
__global__ void k_pack(Params P, StateSet S, const int32_t* id, double* Vh, int32_t* idh, double* phih, double* const* R,
                       double* Rh, const double* rphi, double* rphih) {
  int i, j, k;
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (!real_cell(P.g, t, i, j, k)) return;
  int64_t c = P.g.at(i, j, k);
  if (Vh) for (int p = 0; p < 5; p++) Vh[t * 5 + p] = S.q[p][c];
  if (idh) idh[t] = id[c];
  if (phih) phih[t] = S.q[5][c];
  if (Rh) for (int p = 0; p < 5; p++) Rh[t * 5 + p] = R[p][c];
  if (rphih) rphih[t] = rphi[c];
}

// ---------------------------------------------------------------------------
// Host-side launchers
static inline int nblk(int64_t n, int b) { return (int)((n + b - 1) / b); }

void launch_reconstruct(cudaStream_t s, const Params& P, const StateSet& S, const int32_t* id, double* const* fs,
                        unsigned long long* cnt) {
  int64_t n = (int64_t)P.g.nx * P.g.ny * P.g.nz;
  if (P.rec_type == M2CG_REC_CONSTANT || P.rec_var == M2CG_VAR_PRIMITIVE)
    k_reconstruct<<<(unsigned)shaped_blocks(P.g, P.g.nx, P.g.ny, P.g.nz), 128, 0, s>>>(P, S, id, fs, cnt);
  else if (P.rec_var == M2CG_VAR_CONSERVATIVE)
    k_reconstruct_var<M2CG_VAR_CONSERVATIVE><<<nblk(n, 128), 128, 0, s>>>(P, S, id, fs, cnt);
  else if (P.rec_var == M2CG_VAR_PRIMITIVE_CHARACTERISTIC)
    k_reconstruct_var<M2CG_VAR_PRIMITIVE_CHARACTERISTIC><<<nblk(n, 128), 128, 0, s>>>(P, S, id, fs, cnt);
  else
    k_reconstruct_var<M2CG_VAR_CONSERVATIVE_CHARACTERISTIC><<<nblk(n, 128), 128, 0, s>>>(P, S, id, fs, cnt);
  int64_t ng = 2 * ((int64_t)P.g.ny * P.g.nz + (int64_t)P.g.nx * P.g.nz + (int64_t)P.g.nx * P.g.ny);
  k_reconstruct_ghosts<<<nblk(ng, 128), 128, 0, s>>>(P, S, id, fs, cnt);
}
void launch_face_flux(cudaStream_t s, const Params& P, const int32_t* id, double* const* fs, double* const* F,
                      unsigned long long* cnt) {
  k_face_flux<<<(unsigned)shaped_blocks(P.g, P.g.nx + 1, P.g.ny + 1, P.g.nz + 1), 128, 0, s>>>(P, id, fs, F, cnt);
}
void launch_update(cudaStream_t s, const Params& P, const StageArgs& A, const int32_t* id, int32_t* id_new,
                   double* const* F, const IfaceList& L, const DevScalars* sc, int64_t* swept,
                   unsigned long long* swept_count, int64_t swept_cap, unsigned long long* cnt) {
  k_update<<<(unsigned)shaped_blocks(P.g, P.g.nx, P.g.ny, P.g.nz), 128, 0, s>>>(P, A, id, id_new, F, L, sc, swept,
                                                                                swept_count, swept_cap, cnt);
}
void launch_ls_residual(cudaStream_t s, const Params& P, const StateSet& S, double* out) {
  int64_t n = (int64_t)P.g.nx * P.g.ny * P.g.nz;
  k_ls_residual<<<nblk(n, 128), 128, 0, s>>>(P, S, out);
}
void launch_bc(cudaStream_t s, const Params& P, const StateSet& S, int do_v, int do_phi, int32_t* id,
               const DevScalars* sc) {
  int64_t ng = 2 * ((int64_t)P.g.ny * P.g.nz + (int64_t)P.g.nx * P.g.nz + (int64_t)P.g.nx * P.g.ny);
  k_bc<<<nblk(ng, 128), 128, 0, s>>>(P, S, do_v, do_phi, id, sc);
}
void launch_dt(cudaStream_t s, const Params& P, const StateSet& S, const int32_t* id, DevScalars* sc, int mode,
               double fixed_dt) {
  int64_t n = (int64_t)P.g.nx * P.g.ny * P.g.nz;
  k_dt_reduce<<<nblk(n, 256), 256, 0, s>>>(P, S, id, sc);
  k_dt_finalize<<<1, 1, 0, s>>>(P, sc, mode, fixed_dt);
}
void launch_compact(cudaStream_t s, const Params& P, const int32_t* id, const IfaceList& L, unsigned long long* cnt,
                    const DevScalars* sc) {
  int64_t n = (int64_t)(P.g.nx + 1) * (P.g.ny + 1) * (P.g.nz + 1);
  k_compact_interfaces<<<nblk(n, 256), 256, 0, s>>>(P, id, L, cnt, sc);
}
// The "remaining" cells of a swept list take their IDs from their neighbours
// (three passes; six launches).
void launch_resolve_remaining(cudaStream_t s, const Params& P, int32_t* id_new, const int64_t* swept,
                              const unsigned long long* swept_count, int64_t swept_cap, int32_t* cand,
                              const DevScalars* sc, int nsm) {
  const int passes = 3;
  for (int p = 0; p < passes; p++) {
    k_resolve_remaining<<<nsm * 2, 256, 0, s>>>(P, id_new, swept, swept_count, swept_cap, cand, p == passes - 1, sc);
    k_commit_remaining<<<nsm * 2, 256, 0, s>>>(id_new, swept, swept_count, swept_cap, cand, sc);
  }
}
void launch_commit_ids(cudaStream_t s, int32_t* id, const int32_t* id_new, const int64_t* swept,
                       const unsigned long long* swept_count, int64_t swept_cap, const DevScalars* sc, int nsm) {
  k_commit_ids<<<nsm * 2, 256, 0, s>>>(id, id_new, swept, swept_count, swept_cap, sc);
}
void launch_end_of_step(cudaStream_t s, const Params& P, const StateSet& S, int32_t* id, int32_t* id_new,
                        const IfaceList& L, const int64_t* swept, const unsigned long long* swept_count,
                        int64_t swept_cap, int32_t* cand, unsigned long long* cnt, const DevScalars* sc, int nsm) {
  launch_resolve_remaining(s, P, id_new, swept, swept_count, swept_cap, cand, sc, nsm);
  k_swept_update<<<nsm * 2, 128, 0, s>>>(P, S, id, id_new, L, swept, swept_count, swept_cap, cnt, sc);
  launch_commit_ids(s, id, id_new, swept, swept_count, swept_cap, sc, nsm);
  launch_bc(s, P, S, 1, 1, id, sc);
}
void launch_conserved(cudaStream_t s, const Params& P, const StateSet& S, const int32_t* id, double* partial,
                      int* nblocks) {
  int64_t n = (int64_t)P.g.nx * P.g.ny * P.g.nz;
  *nblocks = nblk(n, 256);
  k_conserved<<<*nblocks, 256, 0, s>>>(P, S, id, partial);
}
void launch_unpack(cudaStream_t s, const Params& P, const double* Vh, const int32_t* idh, const double* phih,
                   const StateSet& S, int32_t* id, unsigned long long* cnt) {
  int64_t n = (int64_t)P.g.nx * P.g.ny * P.g.nz;
  k_unpack<<<nblk(n, 256), 256, 0, s>>>(P, Vh, idh, phih, S, id, cnt);
}
void launch_pack(cudaStream_t s, const Params& P, const StateSet& S, const int32_t* id, double* Vh, int32_t* idh,
                 double* phih, double* const* R, double* Rh, const double* rphi, double* rphih) {
  int64_t n = (int64_t)P.g.nx * P.g.ny * P.g.nz;
  k_pack<<<nblk(n, 256), 256, 0, s>>>(P, S, id, Vh, idh, phih, R, Rh, rphi, rphih);
}

// ---- batched launchers: the members' blocks back to back ---------------------------
__global__ void k_reset_counters_ens(const CounterResetArgs* __restrict__ ea) {
  const CounterResetArgs& e = ea[blockIdx.y];
  if (threadIdx.x == 0) { *e.a = 0; *e.b = 0; }
}
#define M2CG_ENS_LAUNCHER(K, B)                                                                        \
  void launch_##K##_ens(cudaStream_t s, int64_t blocks, const K##_args* t, const int64_t* boff, int D) { \
    if (blocks > 0 && D > 0) K##_ens<<<(unsigned)blocks, B, 0, s>>>(t, boff, D);                       \
  }
// The per-stage cell and face kernels of a batch run persistent: as many
// blocks as fit on the GPU at once (occupancy x SMs), each looping over the
// members' blocks (a work queue in member order, boff).
template <class KF>
static int persistent_grid(KF kernel, int block) {
  int dev = 0, nsm = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, block, 0) != cudaSuccess || per < 1) {
    cudaGetLastError();
    per = 1;
  }
  return std::max(1, nsm * per);
}
#define M2CG_ENS_PERSISTENT_LAUNCHER(K, B)                                                             \
  void launch_##K##_ens(cudaStream_t s, int64_t blocks, const K##_args* t, const int64_t* boff, int D) { \
    static const int grid = persistent_grid(K##_ens, B);                                                \
    if (blocks > 0 && D > 0) K##_ens<<<(unsigned)std::min<int64_t>(blocks, grid), B, 0, s>>>(t, boff, D, blocks); \
  }
M2CG_ENS_PERSISTENT_LAUNCHER(k_reconstruct, 128)
M2CG_ENS_LAUNCHER(k_reconstruct_ghosts, 128)
M2CG_ENS_PERSISTENT_LAUNCHER(k_face_flux, 128)
M2CG_ENS_PERSISTENT_LAUNCHER(k_update, 128)
M2CG_ENS_LAUNCHER(k_bc, 128)
M2CG_ENS_LAUNCHER(k_dt_reduce, 256)
M2CG_ENS_LAUNCHER(k_dt_finalize, 1)
M2CG_ENS_LAUNCHER(k_compact_interfaces, 256)
M2CG_ENS_LAUNCHER(k_resolve_remaining, 256)
M2CG_ENS_LAUNCHER(k_commit_remaining, 256)
M2CG_ENS_LAUNCHER(k_swept_update, 128)
M2CG_ENS_LAUNCHER(k_commit_ids, 256)
void launch_reset_counters_ens(cudaStream_t s, const CounterResetArgs* t, int D) {
  if (D > 0) k_reset_counters_ens<<<dim3(1, (unsigned)D), 32, 0, s>>>(t);
}

}  // namespace m2cg
