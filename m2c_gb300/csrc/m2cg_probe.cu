// Solution values at probe points on the device: ProbeOutput::
// InterpolateSolutionAtProbe (ProbeOutput.cpp:849-886) -- trilinear
// interpolation over the ghosted cell-centre grid, corners that are edge or
// corner ghosts (never populated) replaced by the mean of the populated ones.
// The points are located on the host (ProbeOutput::SetupInterpolation,
// ProbeOutput.cpp:360-480); one thread per point gathers its eight corners of
// V, ID and phi, so a probe line costs a few hundred bytes instead of a
// download of the state.  Compiled without floating-point contraction: the
// interpolation rounds as the reference's MathTools/trilinear_interpolation.h.
//
// Also the per-material integrals of EnergyIntegrationOutput (EnergyIntegration
// Output.cpp:247-610, Cartesian meshes): volume, mass, total energy, total
// enthalpy, kinetic and internal energy of the cells whose centres lie in a
// box, reduced per block in a fixed order and summed over the blocks on the
// host, so repeated calls give identical sums.
#include <algorithm>
#include "m2cg_internal.h"

namespace m2cg {

namespace {

constexpr int INT_THREADS = 128;
constexpr int INT_Q = 6;   // volume, mass, total energy, total enthalpy, kinetic, internal
static_assert(INT_Q == M2CG_N_INTEGRALS, "integral count");

__global__ void __launch_bounds__(INT_THREADS) k_integrate(Params P, StateSet S, const int32_t* __restrict__ id,
                                                          Box3 box, double lo0, double lo1, double lo2,
                                                          double* __restrict__ partial) {
  const Grid& g = P.g;
  double acc[M2CG_MAX_MATERIALS * INT_Q];
  for (int m = 0; m < M2CG_MAX_MATERIALS * INT_Q; m++) acc[m] = 0.0;
  const double cell = g.dx * g.dy * g.dz;
  const int64_t n = (int64_t)g.nx * g.ny * g.nz;
  for (int64_t t = (int64_t)blockIdx.x * INT_THREADS + threadIdx.x; t < n; t += (int64_t)gridDim.x * INT_THREADS) {
    const int k = (int)(t / ((int64_t)g.nx * g.ny));
    const int64_t r = t - (int64_t)k * g.nx * g.ny;
    const int j = (int)(r / g.nx), i = (int)(r - (int64_t)j * g.nx);
    const double x = lo0 + 0.5 * g.dx + i * g.dx, y = lo1 + 0.5 * g.dy + j * g.dy, z = lo2 + 0.5 * g.dz + k * g.dz;
    if (!(x >= box.lo[0] && x <= box.hi[0] && y >= box.lo[1] && y <= box.hi[1] && z >= box.lo[2] && z <= box.hi[2]))
      continue;
    const int64_t c = g.at(i, j, k);
    const int m = id[c];
    if (m < 0 || m >= P.n_mat) continue;
    const double rho = S.q[0][c], vx = S.q[1][c], vy = S.q[2][c], vz = S.q[3][c], p = S.q[4][c];
    const double vsq = vx * vx + vy * vy + vz * vz;
    const double e = eos_e(P.mats.m[m], rho, p);
    double* a = acc + m * INT_Q;
    a[0] += cell;
    a[1] += rho * cell;
    a[2] += rho * (0.5 * vsq + e) * cell;
    a[3] += (rho * (0.5 * vsq + e) + p) * cell;
    a[4] += 0.5 * rho * vsq * cell;
    a[5] += rho * e * cell;
  }
  __shared__ double red[INT_THREADS / 32][M2CG_MAX_MATERIALS * INT_Q];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int q = 0; q < M2CG_MAX_MATERIALS * INT_Q; q++) {
    double v = acc[q];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[w][q] = v;
  }
  __syncthreads();
  for (int q = threadIdx.x; q < M2CG_MAX_MATERIALS * INT_Q; q += INT_THREADS) {
    double v = 0.0;
    for (int ww = 0; ww < INT_THREADS / 32; ww++) v += red[ww][q];
    partial[(int64_t)blockIdx.x * M2CG_MAX_MATERIALS * INT_Q + q] = v;
  }
}

__global__ void k_sample_points(StateSet S, const int32_t* __restrict__ id, int with_phi, int64_t px, int64_t py,
                                const ProbePoint* __restrict__ pts, int n, double* __restrict__ out) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const ProbePoint& p = pts[q];
  const int64_t base = ((int64_t)p.k * py + p.j) * px + p.i;
  // corners c000, c100, c010, c110, c001, c101, c011, c111
  const int64_t off[8] = {0, 1, px, px + 1, px * py, px * py + 1, px * py + px, px * py + px + 1};
  const int nf = 6 + (with_phi ? 1 : 0);
  for (int f = 0; f < nf; f++) {
    double c[8];
    double sum = 0.0;
    for (int m = 0; m < 8; m++) {
      const int64_t l = base + off[m];
      double v = 0.0;
      if (p.valid & (1u << m)) v = f < 5 ? S.q[f][l] : (f == 5 ? (double)id[l] : S.q[5][l]);
      c[m] = v;
      sum += v;
    }
    if (p.nvalid < 8) {
      const double avg = sum / p.nvalid;
      for (int m = 0; m < 8; m++)
        if (!(p.valid & (1u << m))) c[m] = avg;
    }
    const double xi = p.w[0], eta = p.w[1], zeta = p.w[2];
    const double c00 = c[0] * (1.0 - xi) + c[1] * xi;
    const double c01 = c[4] * (1.0 - xi) + c[5] * xi;
    const double c10 = c[2] * (1.0 - xi) + c[3] * xi;
    const double c11 = c[6] * (1.0 - xi) + c[7] * xi;
    const double c0 = c00 * (1.0 - eta) + c10 * eta;
    const double c1 = c01 * (1.0 - eta) + c11 * eta;
    out[(int64_t)q * nf + f] = c0 * (1.0 - zeta) + c1 * zeta;
  }
}

}  // namespace

int launch_integrate(cudaStream_t s, const Params& P, const StateSet& S, const int32_t* id, const Box3& box,
                     const double lo[3], int nsm, double* partial) {
  const int64_t n = (int64_t)P.g.nx * P.g.ny * P.g.nz;
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((n + INT_THREADS - 1) / INT_THREADS, (int64_t)nsm * 4));
  if (partial) k_integrate<<<blocks, INT_THREADS, 0, s>>>(P, S, id, box, lo[0], lo[1], lo[2], partial);
  return blocks;
}

void launch_sample_points(cudaStream_t s, const Params& P, const StateSet& S, const int32_t* id,
                          const ProbePoint* pts, int n, double* out) {
  k_sample_points<<<(n + 127) / 128, 128, 0, s>>>(S, id, P.n_ls > 0 ? 1 : 0, P.g.px, P.g.py, pts, n, out);
}

}  // namespace m2cg
