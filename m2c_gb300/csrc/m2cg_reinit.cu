// Level-set reinitialization over the full domain with the first layer held
// fixed (the default FirstLayerTreatment FIXED): LevelSetReinitializer.cpp:76-176
// (ReinitializeFullDomain), :304-437 (TagFirstLayerNodes), :601-623 (sign
// function, eps = 1), :960-1041 (ComputeResidualFullDomain), :1249-1362 (ghost
// values), :1966-1991 (largest relative change).
//
// The pseudo-time loop runs on the device as a CUDA graph: a one-thread gate
// kernel and a preparation pass, then a WHILE conditional node whose body is one
// RK3 iteration (three fused residual + stage-combination passes, each followed
// by the ghost pass) and a one-thread control kernel that decides continue /
// converged / retry-with-smaller-CFL and sets the loop condition.  No host round
// trip happens inside a call; the stepping launches the graph after the steps
// whose number is a multiple of the frequency.
//
// Compiled without floating-point contraction: the stage combinations, the sign
// function and the ghost extrapolation follow the reference's operation order
// in plain binary64.  The residual is written for GB300's FP64 pipe, which
// bounds this loop: the one-sided differences are multiplied by 1/h where the
// reference divides by the difference of two cell-centre coordinates (equal to
// h up to the rounding of those coordinates), signs flip and maxima are taken
// on the integer pipe through the bit patterns, and the square root and the
// relative change use a refined hardware reciprocal (square root) estimate.
// The result differs from the reference's operation order by a few ulps.
#include <algorithm>
#include "m2cg_internal.h"

namespace m2cg {

void launch_bc(cudaStream_t, const Params&, const StateSet&, int, int, int32_t*, const DevScalars*);
void launch_resolve_remaining(cudaStream_t, const Params&, int32_t*, const int64_t*, const unsigned long long*,
                              int64_t, int32_t*, const DevScalars*, int);
void launch_commit_ids(cudaStream_t, int32_t*, const int32_t*, const int64_t*, const unsigned long long*, int64_t,
                       const DevScalars*, int);

namespace {

constexpr int RI_THREADS = 128;

M2CG_DEV double as_dbl(unsigned long long b) { return __longlong_as_double((long long)b); }
M2CG_DEV unsigned long long as_bits(double x) { return (unsigned long long)__double_as_longlong(x); }

M2CG_DEV bool ri_live(const ReinitState* st) { return st->run && st->detected; }

// max(x, y, 0) through the bit patterns: non-negative doubles order like their
// signed 64-bit patterns and every negative one (-0 included) falls below the
// pattern of +0, so the comparison runs on the integer pipe.
M2CG_DEV double max_with_zero(double x, double y) {
  long long a = __double_as_longlong(x), b = __double_as_longlong(y);
  long long m = a > b ? a : b;
  return __longlong_as_double(m > 0 ? m : 0);
}

// x with its sign bit xor-ed with sb (0 or the sign bit): an exact negation
// when sb is set, on the integer pipe.
M2CG_DEV double flip(double x, long long sb) { return __longlong_as_double(__double_as_longlong(x) ^ sb); }

// sqrt(x) for x >= 0 as x * rsqrt(x), the reciprocal square root from the
// hardware estimate refined by Newton's iteration (one step, cubic term).
M2CG_DEV double sqrt_nr(double x) {
  if (!(x > 1e-300)) return sqrt(x);   // zero, subnormal (the estimate flushes it), NaN
  double y;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  const double e = fma(-x, y * y, 1.0);
  y = fma(y * e, fma(e, 0.375, 0.5), y);
  return x * y;
}

// 1/x for x > 0 from the hardware estimate refined by Newton's iteration.
M2CG_DEV double rcp_nr(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  const double e = fma(-x, r, 1.0);
  return fma(r, fma(e, e, e), r);
}

// |grad phi| - 1 by Godunov's upwind rule (LevelSetReinitializer.cpp:1009-1026).
// For phi >= 0 the x term is max(max(a,0)^2, min(b,0)^2) with a, b the backward
// and forward differences; it equals (max(p - p_{i-1}, p - p_{i+1}, 0) / h)^2.
// For phi < 0 the differences change sign (phi = -0 counts as >= 0, as there).
M2CG_DEV double ri_res(const double* __restrict__ q, int64_t c, int64_t sy, int64_t sz, const double* rh) {
  const double p = q[c];
  const long long pb = __double_as_longlong(p);
  const long long sb = (pb < 0 && pb != (long long)0x8000000000000000ull) ? (long long)0x8000000000000000ull : 0ll;
  const double gx = max_with_zero(flip(p - q[c - 1], sb), flip(p - q[c + 1], sb)) * rh[0];
  const double gy = max_with_zero(flip(p - q[c - sy], sb), flip(p - q[c + sy], sb)) * rh[1];
  const double gz = max_with_zero(flip(p - q[c - sz], sb), flip(p - q[c + sz], sb)) * rh[2];
  return sqrt_nr(fma(gz, gz, fma(gy, gy, gx * gx))) - 1.0;
}

// Block maximum of non-negative bit patterns, one atomic per block.
M2CG_DEV void block_max_atomic(unsigned long long v, unsigned long long* dst) {
  __shared__ unsigned long long red[RI_THREADS / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m = red[0];
    for (int w = 1; w < RI_THREADS / 32; w++) m = red[w] > m ? red[w] : m;
    if (m) atomicMax(dst, m);
  }
}

// Gate: run this call?  gated = 1: after every freq-th completed step, or after
// every step that crosses a multiple of freq_dt; gated = 2: when the step left
// unresolved swept cells (TimeIntegrator.cpp:776-797), whose list is then
// sorted into the reference's (k, j, i) order, their phi saved, and made
// negative where it is not (MultiPhaseOperator.cpp:1364-1420); never with
// MaxIts <= 0, where the reference's loop does not execute and the failsafe
// accepts the input.
__global__ void k_ri_begin(ReinitArgs a, cudaGraphConditionalHandle h, int gated) {
  ReinitState* st = a.st;
  bool go = a.max_its > 0;
  st->keep = 0;
  if (gated == 1) {   // Utils.cpp:337-357: the time interval when given, else the step count
    bool due;
    if (a.freq_dt > 0) due = floor(a.sc->time / a.freq_dt) != floor((a.sc->time - a.sc->dt) / a.freq_dt);
    else due = a.freq > 0 && (a.sc->steps % a.freq) == 0;
    go = go && a.sc && a.sc->active && due;
  } else if (gated == 2) {
    unsigned long long n = *a.unres_count;
    if (n > (unsigned long long)a.unres_cap) {
      a.cnt[CNT_UNRES_OVERFLOW] += 1;
      n = (unsigned long long)a.unres_cap;
      *a.unres_count = n;
    }
    int64_t* L = a.unres;
    for (unsigned long long s = 1; s < n; s++) {   // insertion sort: the list is short
      const int64_t v = L[s];
      unsigned long long t = s;
      for (; t > 0 && L[t - 1] > v; t--) L[t] = L[t - 1];
      L[t] = v;
    }
    for (unsigned long long s = 0; s < n; s++) {
      const double p = a.phi[L[s]];
      a.unres_phi_old[s] = p;
      if (!(p < 0)) a.phi[L[s]] = -p;
    }
    st->keep = n > 0 ? 1 : 0;
    go = go && n > 0;
  }
  st->run = go ? 1 : 0;
  st->detected = 0;
  st->restore = 0;
  st->iter = 0;
  st->body_runs = 0;
  st->res_bits = 0;
  st->dphi_bits = 0;
  cudaGraphSetConditional(h, go ? 1u : 0u);
}

// Backup of the whole ghosted array (the retry restores it), first-layer tags
// and the smoothed sign phi / sqrt(phi^2 + h_min^2) on the interior.
__global__ void __launch_bounds__(RI_THREADS) k_ri_prep(ReinitArgs a) {
  ReinitState* st = a.st;
  if (!st->run && !st->keep) return;
  const Grid& g = a.g;
  for (int64_t t = (int64_t)blockIdx.x * RI_THREADS + threadIdx.x; t < g.ntot; t += (int64_t)gridDim.x * RI_THREADS)
    a.bk[t] = a.phi[t];
  const int64_t rows = (int64_t)g.ny * g.nz;
  const double f = a.hmin;   // eps = 1: factor = 1.0 * min(dx, dy, dz)
  unsigned found = 0;
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    const int k = (int)(r / g.ny), j = (int)(r - (int64_t)k * g.ny);
    const int64_t base = g.at(0, j, k);
    for (int i = threadIdx.x; i < g.nx; i += RI_THREADS) {
      const int64_t c = base + i;
      const double p = a.phi[c];
      const bool t = p * a.phi[c - 1] <= 0.0 || p * a.phi[c + 1] <= 0.0 || p * a.phi[c - g.sy] <= 0.0 ||
                     p * a.phi[c + g.sy] <= 0.0 || p * a.phi[c - g.sz] <= 0.0 || p * a.phi[c + g.sz] <= 0.0;
      a.tag[c] = t ? 1 : 0;
      a.sign[c] = p / sqrt(p * p + f * f);
      found |= t ? 1u : 0u;
    }
  }
  if (__syncthreads_or(found) && threadIdx.x == 0) atomicOr(&st->detected, 1u);
}

// One RK3 sub-stage: R = R(src) on the interior (0 on first-layer nodes), then
//   S = 1: phi1 = src + R                       (src = phi, or the backup on a retry)
//   S = 2: phi2 = (0.25 phi1 + 0.75 phi) + 0.25 R
//   S = 3: phi  = (phi/3 + 2 phi2/3) + 2 R/3, and the largest relative change
// S = 1 also records max |res| over the untagged nodes; later sub-stages stop
// once that is below the tolerance (the reference's loop exit).
template <int S>
__global__ void __launch_bounds__(RI_THREADS) k_ri_stage(ReinitArgs a) {
  ReinitState* st = a.st;
  if (!ri_live(st)) return;
  if (S > 1 && as_dbl(st->res_bits) < a.tol) return;
  const bool restore = (S == 1) && st->restore;
  const double* __restrict__ src = S == 1 ? (restore ? a.bk : a.phi) : (S == 2 ? a.phi1 : a.phi2);
  double* out = S == 1 ? a.phi1 : (S == 2 ? a.phi2 : a.phi);
  const double mdt = -(st->cfl * a.hmin);
  const Grid& g = a.g;
  const int64_t rows = (int64_t)g.ny * g.nz;
  unsigned long long mx = 0;
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    const int k = (int)(r / g.ny), j = (int)(r - (int64_t)k * g.ny);
    const int64_t base = g.at(0, j, k);
    for (int i = threadIdx.x; i < g.nx; i += RI_THREADS) {
      const int64_t c = base + i;
      double R = 0.0;
      if (!a.tag[c]) {
        const double res = ri_res(src, c, g.sy, g.sz, a.rh);
        const double f = mdt * a.sign[c];
        const double ares = fabs(res);
        R = ares <= 1.0 ? f * res : (f * res) / ares;
        if (S == 1) { const unsigned long long b = as_bits(ares); mx = b > mx ? b : mx; }
      }
      if (S == 1) {
        const double p = src[c];
        if (restore) a.phi[c] = p;
        out[c] = p + R;
      } else if (S == 2) {
        out[c] = (0.25 * src[c] + 0.75 * a.phi[c]) + 0.25 * R;
      } else {
        const double old = out[c];
        const double nw = ((1.0 / 3.0) * old + (2.0 / 3.0) * src[c]) + (2.0 / 3.0) * R;
        out[c] = nw;
        double e = fabs(nw - old);
        const double anw = fabs(nw);
        if (anw > 1e-300) e *= rcp_nr(anw);
        else if (nw != 0.0) e /= anw;
        const unsigned long long b = as_bits(e);
        mx = b > mx ? b : mx;
      }
    }
  }
  if (S == 1) block_max_atomic(mx, &st->res_bits);
  if (S == 3) block_max_atomic(mx, &st->dphi_bits);
}

// Face-ghost values of phi1 (which = 1), phi2 (2) or phi (0) from the interior:
// zero-Neumann copy or linear extrapolation from the two nearest interior
// nodes (cell-centre coordinates lo + 0.5 h + i h), clamped at -h/2 for
// NON_NEGATIVE.  On a retry the pass after the first sub-stage also restores
// phi's face ghosts from the backup.
__global__ void k_ri_bc(ReinitArgs a, int which) {
  ReinitState* st = a.st;
  if (!ri_live(st) || as_dbl(st->res_bits) < a.tol) return;
  double* q = which == 1 ? a.phi1 : (which == 2 ? a.phi2 : a.phi);
  const bool restore = which == 1 && st->restore;
  const Grid& g = a.g;
  const int64_t n = 2 * ((int64_t)g.ny * g.nz + (int64_t)g.nx * g.nz + (int64_t)g.nx * g.ny);
  const double h[3] = {g.dx, g.dy, g.dz};
  const int64_t strd[3] = {1, g.sy, g.sz};
  const int nn[3] = {g.nx, g.ny, g.nz};
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    int side, i, j, k, ii, jj, kk;
    ghost_face_cell(g, t, side, i, j, k, ii, jj, kk);
    const int64_t c = g.at(i, j, k);
    if (restore) a.phi[c] = a.bk[c];
    const int bc = a.ls_bc[side];
    if (bc == M2CG_LSBC_ZERO_NEUMANN) { q[c] = q[g.at(ii, jj, kk)]; continue; }
    const int d = side / 2, sgn = (side % 2 == 0) ? 1 : -1;
    const int pos[3] = {i, j, k};
    const bool ok = sgn > 0 ? (pos[d] + 2 < nn[d]) : (pos[d] - 2 >= 0);
    double v;
    if (ok) {
      const double r = a.lo[d] + 0.5 * h[d] + pos[d] * h[d];
      const double r1 = a.lo[d] + 0.5 * h[d] + (pos[d] + sgn) * h[d];
      const double r2 = a.lo[d] + 0.5 * h[d] + (pos[d] + 2 * sgn) * h[d];
      const double f1 = q[c + sgn * strd[d]], f2 = q[c + 2 * sgn * strd[d]];
      v = f1 + (f2 - f1) / (r2 - r1) * (r - r1);
    } else {
      v = q[g.at(ii, jj, kk)];
    }
    if (bc == M2CG_LSBC_NON_NEGATIVE) v = fmax(-(0.5 * h[d]), v);
    q[c] = v;
  }
}

// End of one loop-body execution (LevelSetReinitializer.cpp:113-175): converged
// on the residual or on the relative change, or after MaxIts either accept
// (change < 0.02), give up (CFL < 0.02; the reference stops the program, here
// counted in failures) or restart from the backup with CFL / 1.5.  A call
// never runs more than 64 MaxIts bodies.
__global__ void k_ri_ctl(ReinitArgs a, cudaGraphConditionalHandle h) {
  ReinitState* st = a.st;
  st->body_runs += 1;
  st->bodies += 1;
  bool more = false;
  if (st->run && st->detected) {
    const double res = as_dbl(st->res_bits);
    const int idx = st->iter;
    st->last_res = res;
    bool done = false;
    int restore = 0;
    if (res < a.tol) {
      done = true;
    } else {
      const double dphi = as_dbl(st->dphi_bits);
      st->last_dphi = dphi;
      if (dphi < a.tol) {
        done = true;
      } else if (idx + 1 >= a.max_its) {
        st->iter = a.max_its;
        if (dphi < 0.02) done = true;
        else if (st->cfl < 0.02) { st->failures += 1; done = true; }
        else {
          st->cfl /= 1.5;
          st->retries += 1;
          st->iterations += a.max_its;
          st->iter = 0;
          restore = 1;
        }
      } else {
        st->iter = idx + 1;
      }
    }
    if (!done && st->body_runs >= 64 * a.max_its) { st->failures += 1; done = true; }
    if (done) {
      st->iterations += st->iter;
      st->calls += 1;
      st->run = 0;
    }
    st->restore = restore;
    st->res_bits = 0;
    st->dphi_bits = 0;
    more = !done;
  } else {
    st->run = 0;
  }
  cudaGraphSetConditional(h, more ? 1u : 0u);
}

// ---------------------------------------------------------------------------
// Repair of the step's unresolved swept cells, after the reinitialization that
// the gate of mode 2 ran.  One graph: a one-thread gate, then an IF node whose
// body restores the saved phi of the listed cells into the backup (which then
// holds phi as it was before the repair), moves the IDs of the cells whose
// sign changed, repairs the listed cells' states and clips them.

M2CG_DEV void cell_ijk(const Grid& g, int64_t c, int& i, int& j, int& k) {
  int64_t r = c;
  i = (int)(r % g.px) - 1; r /= g.px;
  j = (int)(r % g.py) - 1;
  k = (int)(r / g.py) - 1;
}

// whether c is in the sorted list
M2CG_DEV bool listed(const int64_t* L, int64_t n, int64_t c) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    const int64_t m = (lo + hi) >> 1;
    if (L[m] < c) lo = m + 1;
    else hi = m;
  }
  return lo < n && L[lo] == c;
}

__global__ void k_ur_begin(UnresArgs a, cudaGraphConditionalHandle h) {
  const bool go = *a.count > 0;
  if (go) {
    *a.swept_count = 0;
    a.cnt[CNT_UNRES_REPAIRS] += 1;
  }
  cudaGraphSetConditional(h, go ? 1u : 0u);
}

__global__ void k_ur_restore(UnresArgs a) {
  const int64_t n = (int64_t)*a.count;
  for (int64_t s = threadIdx.x; s < n; s += blockDim.x) a.bk[a.list[s]] = a.phi_old[s];
}

// MultiPhaseOperator::UpdateMaterialIDByLevelSet against the phi before the
// repair (MultiPhaseOperator.cpp:190-222): a sign change makes the cell the
// level set's material when phi < 0, else a "remaining" cell resolved from its
// neighbours by the passes that follow.
__global__ void __launch_bounds__(256) k_ur_mark(UnresArgs a) {
  const Grid& g = a.P.g;
  const double* phi = a.S.q[5];
  const int64_t rows = (int64_t)g.ny * g.nz;
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    const int k = (int)(r / g.ny), j = (int)(r - (int64_t)k * g.ny);
    const int64_t base = g.at(0, j, k);
    for (int i = threadIdx.x; i < g.nx; i += blockDim.x) {
      const int64_t c = base + i;
      const double ph = phi[c];
      if (ph * a.bk[c] > 0.0) continue;
      const int nid = ph < 0 ? a.P.ls_matid : -1 - a.id[c];
      const unsigned long long s = atomicAdd(a.swept_count, 1ull);
      if ((int64_t)s < a.swept_cap) a.swept[s] = c;
      else atomicAdd(&a.cnt[CNT_SWEPT_OVERFLOW], 1ull);
      a.id_new[c] = nid;
    }
  }
}

// MultiPhaseOperator::FixUnresolvedNodes (MultiPhaseOperator.cpp:1279-1480, no
// embedded surfaces), one thread in list order: each cell takes the upwind-
// weighted mean of its resolved same-material neighbours (weight = max(0,
// unit neighbour velocity . unit direction from the neighbour to the cell)),
// else their inverse-distance mean, else keeps velocity and pressure and
// takes an inverse-distance density over up to 10 layers, else the material's
// failsafe density.  The flag that marks the first accumulated neighbour is
// set once for the whole list, as in the reference (line 1296): later cells
// accumulate onto their own advected state.
__global__ void k_ur_fix(UnresArgs a) {
  const int64_t n = (int64_t)*a.count;
  const Grid& g = a.P.g;
  const double h[3] = {g.dx, g.dy, g.dz};
  double* const* q = a.S.q;
  const int32_t* id = a.id;
  bool reset = false;
  for (int64_t s = 0; s < n; s++) {
    const int64_t c = a.list[s];
    int i, j, k;
    cell_ijk(g, c, i, j, k);
    const int myid = id[c];
    const int pos[3] = {i, j, k};
    double x0[3];
    for (int d = 0; d < 3; d++) x0[d] = a.lo[d] + 0.5 * h[d] + pos[d] * h[d];
    double sw = 0.0, sw2 = 0.0, vt[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int nk = k - 1; nk <= k + 1; nk++)
      for (int nj = j - 1; nj <= j + 1; nj++)
        for (int ni = i - 1; ni <= i + 1; ni++) {
          if (ni < 0 || ni >= g.nx || nj < 0 || nj >= g.ny || nk < 0 || nk >= g.nz) continue;
          const int64_t nc = g.at(ni, nj, nk);
          if (id[nc] != myid || nc == c || listed(a.list, n, nc)) continue;
          const int npos[3] = {ni, nj, nk};
          double x1[3], v1[3], dv[3];
          for (int d = 0; d < 3; d++) x1[d] = a.lo[d] + 0.5 * h[d] + npos[d] * h[d];
          for (int d = 0; d < 3; d++) v1[d] = q[1 + d][nc];
          const double v1norm = sqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
          if (v1norm != 0) { const double r = 1.0 / v1norm; for (int d = 0; d < 3; d++) v1[d] *= r; }
          for (int d = 0; d < 3; d++) dv[d] = x0[d] - x1[d];
          const double dn = sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
          { const double r = 1.0 / dn; for (int d = 0; d < 3; d++) dv[d] *= r; }
          const double dot = dv[0] * v1[0] + dv[1] * v1[1] + dv[2] * v1[2];
          const double w = 0.0 < dot ? dot : 0.0;
          if (w > 0) {
            sw += w;
            for (int p = 0; p < 5; p++) {
              if (reset) q[p][c] += w * q[p][nc];
              else q[p][c] = w * q[p][nc];
            }
            reset = true;
          }
          for (int p = 0; p < 5; p++) vt[p] += 1.0 / dn * q[p][nc];
          sw2 += 1.0 / dn;
        }
    if (a.P.mp_pcdir == M2CG_PCDIR_UPWIND && sw > 0) {
      const double r = 1.0 / sw;
      for (int p = 0; p < 5; p++) q[p][c] *= r;
      continue;
    }
    if (sw2 > 0) {
      for (int p = 0; p < 5; p++) q[p][c] = vt[p] / sw2;
      continue;
    }
    double density = 0.0;
    for (int layer = 1; layer <= 10; layer++) {
      for (int nk = k - layer; nk <= k + layer; nk++)
        for (int nj = j - layer; nj <= j + layer; nj++)
          for (int ni = i - layer; ni <= i + layer; ni++) {
            if (ni < 0 || ni >= g.nx || nj < 0 || nj >= g.ny || nk < 0 || nk >= g.nz) continue;
            const int64_t nc = g.at(ni, nj, nk);
            if (id[nc] != myid || nc == c || listed(a.list, n, nc)) continue;
            const int npos[3] = {ni, nj, nk};
            double x1[3];
            for (int d = 0; d < 3; d++) x1[d] = a.lo[d] + 0.5 * h[d] + npos[d] * h[d];
            const double dist = sqrt((x1[0] - x0[0]) * (x1[0] - x0[0]) + (x1[1] - x0[1]) * (x1[1] - x0[1]) +
                                     (x1[2] - x0[2]) * (x1[2] - x0[2]));
            sw += 1.0 / dist;
            density += (1.0 / dist) * q[0][nc];
          }
      if (sw > 0) { q[0][c] = density / sw; break; }
    }
    if (sw == 0) q[0][c] = a.failsafe[myid];
  }
  a.cnt[CNT_UNRES_FIXED] += (unsigned long long)n;
}

// ClipDensityAndPressure (TimeIntegrator.cpp:800) of the repaired cells and of
// the cells whose ID the repair changed.
__global__ void k_ur_clip(UnresArgs a) {
  const int64_t n = (int64_t)*a.count;
  const int64_t m = (int64_t)min((unsigned long long)a.swept_cap, *a.swept_count);
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n + m; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = t < n ? a.list[t] : a.swept[t - n];
    const DevMat& M = a.P.mats.m[a.id[c]];
    double V[5];
    for (int p = 0; p < 5; p++) V[p] = a.S.q[p][c];
    eos_clip(M, V);
    if (t < n && eos_bad5(M, V)) atomicAdd(&a.cnt[CNT_BAD], 1ull);
    for (int p = 0; p < 5; p++) a.S.q[p][c] = V[p];
  }
}

}  // namespace

// The reinitialization graph: gate, preparation, then the WHILE loop.
cudaError_t reinit_build_graph(cudaStream_t s, const ReinitArgs& a, int nsm, int gated, cudaGraphExec_t* out) {
  *out = nullptr;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaGraphCreate(&g, 0);
  if (e != cudaSuccess) return e;
  cudaGraphConditionalHandle h;
  const int64_t rows = (int64_t)a.g.ny * a.g.nz;
  const int sblocks = (int)std::min<int64_t>(rows, (int64_t)nsm * 16);
  const int64_t nghost = 2 * ((int64_t)a.g.ny * a.g.nz + (int64_t)a.g.nx * a.g.nz + (int64_t)a.g.nx * a.g.ny);
  const int gblocks = (int)std::max<int64_t>(1, std::min<int64_t>((nghost + 255) / 256, (int64_t)nsm * 4));
  cudaGraphNodeParams np = {};
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  cudaStreamCaptureStatus cs;
  cudaGraph_t cap = nullptr, body = nullptr;
  cudaGraphNode_t cn;
#define RI_CK(x) do { e = (x); if (e != cudaSuccess) goto fail; } while (0)
  RI_CK(cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault));
  RI_CK(cudaStreamBeginCaptureToGraph(s, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  k_ri_begin<<<1, 1, 0, s>>>(a, h, gated);
  k_ri_prep<<<sblocks, RI_THREADS, 0, s>>>(a);
  e = cudaStreamGetCaptureInfo(s, &cs, nullptr, nullptr, &deps, nullptr, &nd);
  if (e == cudaSuccess) {
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    e = cudaGraphAddNode(&cn, g, deps, nullptr, nd, &np);
  }
  if (e == cudaSuccess) e = cudaStreamUpdateCaptureDependencies(s, &cn, nullptr, 1, cudaStreamSetCaptureDependencies);
  {
    cudaError_t e2 = cudaStreamEndCapture(s, &cap);
    if (e == cudaSuccess) e = e2;
  }
  if (e != cudaSuccess) goto fail;
  body = np.conditional.phGraph_out[0];
  RI_CK(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  k_ri_stage<1><<<sblocks, RI_THREADS, 0, s>>>(a);
  k_ri_bc<<<gblocks, 256, 0, s>>>(a, 1);
  k_ri_stage<2><<<sblocks, RI_THREADS, 0, s>>>(a);
  k_ri_bc<<<gblocks, 256, 0, s>>>(a, 2);
  k_ri_stage<3><<<sblocks, RI_THREADS, 0, s>>>(a);
  k_ri_bc<<<gblocks, 256, 0, s>>>(a, 0);
  k_ri_ctl<<<1, 1, 0, s>>>(a, h);
  {
    cudaError_t e2 = cudaStreamEndCapture(s, &cap);
    if (e == cudaSuccess) e = e2;
  }
  if (e != cudaSuccess) goto fail;
  RI_CK(cudaGraphInstantiate(out, g, 0));
  cudaGraphDestroy(g);
  return cudaSuccess;
fail:
#undef RI_CK
  cudaGraphDestroy(g);
  return e;
}

// The repair graph: gate, then the IF node with the repair passes.
cudaError_t unres_build_graph(cudaStream_t s, const UnresArgs& a, int nsm, cudaGraphExec_t* out) {
  *out = nullptr;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaGraphCreate(&g, 0);
  if (e != cudaSuccess) return e;
  cudaGraphConditionalHandle h;
  const int64_t rows = (int64_t)a.P.g.ny * a.P.g.nz;
  const int mblocks = (int)std::min<int64_t>(rows, (int64_t)nsm * 8);
  cudaGraphNodeParams np = {};
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  cudaStreamCaptureStatus cs;
  cudaGraph_t cap = nullptr, body = nullptr;
  cudaGraphNode_t cn;
#define UR_CK(x) do { e = (x); if (e != cudaSuccess) goto fail; } while (0)
  UR_CK(cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault));
  UR_CK(cudaStreamBeginCaptureToGraph(s, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  k_ur_begin<<<1, 1, 0, s>>>(a, h);
  e = cudaStreamGetCaptureInfo(s, &cs, nullptr, nullptr, &deps, nullptr, &nd);
  if (e == cudaSuccess) {
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeIf;
    np.conditional.size = 1;
    e = cudaGraphAddNode(&cn, g, deps, nullptr, nd, &np);
  }
  if (e == cudaSuccess) e = cudaStreamUpdateCaptureDependencies(s, &cn, nullptr, 1, cudaStreamSetCaptureDependencies);
  {
    cudaError_t e2 = cudaStreamEndCapture(s, &cap);
    if (e == cudaSuccess) e = e2;
  }
  if (e != cudaSuccess) goto fail;
  body = np.conditional.phGraph_out[0];
  UR_CK(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  k_ur_restore<<<1, 256, 0, s>>>(a);
  k_ur_mark<<<mblocks, 256, 0, s>>>(a);
  launch_resolve_remaining(s, a.P, a.id_new, a.swept, a.swept_count, a.swept_cap, a.cand, a.sc, nsm);
  launch_commit_ids(s, a.id, a.id_new, a.swept, a.swept_count, a.swept_cap, a.sc, nsm);
  launch_bc(s, a.P, a.S, 0, 0, a.id, a.sc);   // ID ghosts (MultiPhaseOperator.cpp:919-942)
  k_ur_fix<<<1, 1, 0, s>>>(a);
  k_ur_clip<<<nsm, 256, 0, s>>>(a);
  launch_bc(s, a.P, a.S, 1, 0, nullptr, a.sc);   // V ghosts
  {
    cudaError_t e2 = cudaStreamEndCapture(s, &cap);
    if (e == cudaSuccess) e = e2;
  }
  if (e != cudaSuccess) goto fail;
  UR_CK(cudaGraphInstantiate(out, g, 0));
  cudaGraphDestroy(g);
  return cudaSuccess;
fail:
#undef UR_CK
  cudaGraphDestroy(g);
  return e;
}

}  // namespace m2cg
