// Solution values at probe points on the device: ProbeOutput::
// InterpolateSolutionAtProbe (ProbeOutput.cpp:849-886) -- trilinear
// interpolation over the ghosted cell-centre grid, corners that are edge or
// corner ghosts (never populated) replaced by the mean of the populated ones.
// The points are located on the host (ProbeOutput::SetupInterpolation,
// ProbeOutput.cpp:360-480); one thread per point gathers its eight corners of
// V, ID and phi, so a probe line costs a few hundred bytes instead of a
// download of the state.  Compiled without floating-point contraction: the
// interpolation rounds as the reference's MathTools/trilinear_interpolation.h.
#include "m2cg_internal.h"

namespace m2cg {

namespace {

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

void launch_sample_points(cudaStream_t s, const Params& P, const StateSet& S, const int32_t* id,
                          const ProbePoint* pts, int n, double* out) {
  k_sample_points<<<(n + 127) / 128, 128, 0, s>>>(S, id, P.n_ls > 0 ? 1 : 0, P.g.px, P.g.py, pts, n, out);
}

}  // namespace m2cg
