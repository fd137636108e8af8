// ORACLE -- test infrastructure only.
//
// CPU restatement of M2C's explicit multi-material finite-volume step, used by
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
// checker for the GPU library.  No product code links, loads or calls it.
//
// What it restates (reference file:line):
//   SpaceOperator::ComputeAdvectionFluxes   SpaceOperator.cpp:1432-2076
//   SpaceOperator::CheckReconstructedStates SpaceOperator.cpp:2420-2569
//   SpaceOperator::ComputeResidual          SpaceOperator.cpp:2573-2641
//   SpaceOperator::ApplyBoundaryConditions  SpaceOperator.cpp:738-821
//   SpaceOperator::ClipDensityAndPressure   SpaceOperator.cpp:647-693
//   SpaceOperator::ComputeTimeStepSize      SpaceOperator.cpp:1223-1330
//   Reconstructor::Reconstruct              Reconstructor.cpp:335-918 (all four variable types), limiters
//                                           Reconstructor.h:96-111, characteristic transforms FluxFcnBase.h:308-517
//   LevelSetReinitializer (full, FIXED)     LevelSetReinitializer.cpp:76-176, 304-437, 601-623, 960-1041, 1966-1991
//   LevelSetOperator FD residual + BCs      LevelSetOperator.cpp:796-870, 408-508
//   GradientCalculatorFD3 coefficients      GradientCalculatorFD3.cpp:300-470
//   TimeIntegratorFE/RK2/RK3                TimeIntegrator.cpp:167-250, 319-455, 527-715
//   UpdateSolutionAfterTimeStepping         TimeIntegrator.cpp:720-843
//   MultiPhaseOperator ID / state updates   MultiPhaseOperator.cpp:153-357, 919-1274
//   Main step loop dt clamp                 Main.cpp:653-712
// EOS, fluxes and the exact Riemann solver are in oracle_eos_flux.h and
// oracle_riemann.h.  Compiled with -ffp-contract=off (reference order of
// operations, no fused multiply-add) and optionally OpenMP.
#include <cstdio>
#include <cstring>
#include <cstdint>
#include <vector>
#include <set>
#include <map>
#include <memory>
#include <chrono>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "oracle_riemann.h"

using namespace orc;

namespace {

struct Counters {
  int64_t interface_faces = 0, riemann_errors = 0, riemann_iterations = 0, riemann_solves = 0;
  int64_t clipped_cells = 0, clipped_faces = 0, nonphysical = 0, swept_cells = 0, unresolved_cells = 0, steps = 0;
  int64_t unresolved_fixed = 0;
  int64_t fallbacks = 0;
};

// Star states stored at one face (RiemannSolutions.h:12-30; SpaceOperator.cpp:1661-1666).
struct FaceSol { bool valid = false; double Vsm[5], Vsp[5]; int idm = 0, idp = 0; };

struct Oracle {
  m2cg_config cfg;
  int NX, NY, NZ, PX, PY, PZ;  // padded dims (ghost width 1)
  double dx, dy, dz, vol;
  std::vector<Eos> vf;
  RiemannParams rp;
  // state (ghosted, AoS for V)
  std::vector<double> V, Phi;
  std::vector<int> ID;
  std::vector<FaceSol> sol[3];   // per-face stored star states, indexed by the plus cell
  Counters cnt;
  double time = 0.0, last_dt = 0.0, last_cfl = 0.0;
  int time_step = 0;
  double fd3_left[4], fd3_right[4][3];  // uniform-mesh FD3 coefficients per direction (set in setup)
  double cl_[3][4], cr_[3][4];

  size_t idx(int i, int j, int k) const { return ((size_t)(k + 1) * PY + (j + 1)) * PX + (i + 1); }
  size_t N() const { return (size_t)PX * PY * PZ; }
  bool outside(int i, int j, int k) const { return i < 0 || i >= NX || j < 0 || j >= NY || k < 0 || k >= NZ; }
  int nface_ghost(int i, int j, int k) const {
    return (i < 0 || i >= NX) + (j < 0 || j >= NY) + (k < 0 || k >= NZ);
  }

  void setup(const m2cg_config& c);
  void ApplyBC(std::vector<double>& v);
  void ApplyLSBC(std::vector<double>& phi);
  void UpdateIDGhosts(std::vector<int>& id);
  int  ClipAll(std::vector<double>& v, const std::vector<int>& id);
  bool Reconstruct(const std::vector<double>& v, const std::vector<int>& id, std::vector<double> fs[6]);
  void CheckReconstructed(const std::vector<double>& v, const std::vector<int>& id, std::vector<double> fs[6]);
  void ComputeResidual(const std::vector<double>& v, const std::vector<int>& id, std::vector<double>& R, bool store);
  void LevelSetResidual(const std::vector<double>& v, const std::vector<double>& phi, std::vector<double>& R);
  void LevelSetResidualFV(const std::vector<double>& v, const std::vector<double>& phi, std::vector<double>& R);
  void ComputeDt(const std::vector<double>& v, const std::vector<int>& id, double& dt, double& cfl);
  void Advance(double dt);
  void P2C(const std::vector<double>& v, const std::vector<int>& id, std::vector<double>& u);
  void C2P(const std::vector<double>& u, const std::vector<int>& id, std::vector<double>& v);
  void EndOfStep(std::vector<double>& phi0);
  void UpdateIDByLevelSet(const std::vector<double>& phi_old);
  void FixUnresolvedNodes(const std::vector<std::array<int, 3>>& unresolved);
  void RiemannNormal(int d, int i, int j, int k, int myid, int nid, double dir[3]) const;
  // level-set reinitialization (full domain, first layer FIXED)
  double reinit_cfl = 0.8;
  int reinit_retries = 0, reinit_failures = 0, reinit_calls = 0, reinit_iters = 0;
  bool Reinitialize();
  double ReinitResidual(const std::vector<double>& phi, const std::vector<char>& tag, const std::vector<double>& sign,
                        std::vector<double>& R, double cfl);
  bool NumFlux(int dir, const double* Vm, const double* Vp, int id, double* F);
};

// Solve the 4x4 Taylor system of GradientCalculatorFD3.cpp:455-470 by Gaussian
// elimination with partial pivoting.
void TaylorCoeffs(double d0, double d1, double d2, double d3, double* c) {
  double A[4][5] = {{1, 1, 1, 1, 0}, {d0, d1, d2, d3, 1}, {d0 * d0, d1 * d1, d2 * d2, d3 * d3, 0},
                    {d0 * d0 * d0, d1 * d1 * d1, d2 * d2 * d2, d3 * d3 * d3, 0}};
  for (int col = 0; col < 4; col++) {
    int piv = col;
    for (int r = col + 1; r < 4; r++) if (std::fabs(A[r][col]) > std::fabs(A[piv][col])) piv = r;
    for (int k = 0; k < 5; k++) std::swap(A[col][k], A[piv][k]);
    for (int r = col + 1; r < 4; r++) {
      double f = A[r][col] / A[col][col];
      for (int k = col; k < 5; k++) A[r][k] -= f * A[col][k];
    }
  }
  for (int r = 3; r >= 0; r--) {
    double s = A[r][4];
    for (int k = r + 1; k < 4; k++) s -= A[r][k] * c[k];
    c[r] = s / A[r][r];
  }
}

void Oracle::setup(const m2cg_config& c) {
  cfg = c;
  NX = c.nx; NY = c.ny; NZ = c.nz;
  PX = NX + 2; PY = NY + 2; PZ = NZ + 2;
  dx = (c.xmax - c.x0) / NX; dy = (c.ymax - c.y0) / NY; dz = (c.zmax - c.z0) / NZ;  // MeshGenerator.cpp:166
  vol = dx * dy * dz;                                                              // SpaceOperator.cpp:217
  vf.resize(c.n_materials);
  for (int m = 0; m < c.n_materials; m++) vf[m].setup(c.mat[m]);
  rp.maxIts_main = c.maxits_main; rp.maxIts_bracket = c.maxits_bracket; rp.maxIts_shock = c.maxits_shock;
  rp.numSteps_rarefaction = c.numsteps_rarefaction; rp.tol_main = c.tol_main; rp.tol_shock = c.tol_shock;
  rp.tol_rarefaction = c.tol_rarefaction; rp.min_pressure = c.min_pressure; rp.failure_threshold = c.failure_threshold;
  rp.pressure_at_failure = c.pressure_at_failure;
  V.assign(N() * 5, 0.0); Phi.assign(N(), 0.0); ID.assign(N(), 0);
  for (int d = 0; d < 3; d++) sol[d].assign(N(), FaceSol());
  double h[3] = {dx, dy, dz};
  for (int d = 0; d < 3; d++) {
    // left-biased: nodes i-2, i-1, i, i+1 (GradientCalculatorFD3.cpp:318-324)
    TaylorCoeffs(-2 * h[d], -h[d], 0.0, h[d], cl_[d]);
    // right-biased: nodes i-1, i, i+1, i+2 (GradientCalculatorFD3.cpp:395-401)
    TaylorCoeffs(-h[d], 0.0, h[d], 2 * h[d], cr_[d]);
  }
}

// SpaceOperator.cpp:738-821 (FACE ghosts only; edges and corners stay untouched).
void Oracle::ApplyBC(std::vector<double>& v) {
  for (int k = -1; k <= NZ; k++)
    for (int j = -1; j <= NY; j++)
      for (int i = -1; i <= NX; i++) {
        if (nface_ghost(i, j, k) != 1) continue;
        int side = (i < 0) ? 0 : (i >= NX) ? 1 : (j < 0) ? 2 : (j >= NY) ? 3 : (k < 0) ? 4 : 5;
        int ii = i < 0 ? -i - 1 : i >= NX ? NX + (i - NX) - 1 : i;   // SpaceOperator.cpp:493-519
        int jj = j < 0 ? -j - 1 : j >= NY ? NY + (j - NY) - 1 : j;
        int kk = k < 0 ? -k - 1 : k >= NZ ? NZ + (k - NZ) - 1 : k;
        double* g = &v[idx(i, j, k) * 5];
        const double* im = &v[idx(ii, jj, kk) * 5];
        int bc = cfg.bc[side];
        if (bc == M2CG_BC_INLET) for (int p = 0; p < 5; p++) g[p] = cfg.inlet[p];
        else if (bc == M2CG_BC_INLET2) for (int p = 0; p < 5; p++) g[p] = cfg.inlet2[p];
        else if (bc == M2CG_BC_SLIPWALL || bc == M2CG_BC_SYMMETRY) {
          for (int p = 0; p < 5; p++) g[p] = im[p];
          g[1 + side / 2] *= -1.0;
        } else if (bc == M2CG_BC_STICKWALL) {
          g[0] = im[0]; g[1] = -1.0 * im[1]; g[2] = -1.0 * im[2]; g[3] = -1.0 * im[3]; g[4] = im[4];
        } else {  // OUTLET
          for (int p = 0; p < 5; p++) g[p] = im[p];
        }
      }
}

// LevelSetOperator.cpp:408-508
void Oracle::ApplyLSBC(std::vector<double>& phi) {
  double h[3] = {dx, dy, dz};
  for (int k = -1; k <= NZ; k++)
    for (int j = -1; j <= NY; j++)
      for (int i = -1; i <= NX; i++) {
        if (nface_ghost(i, j, k) != 1) continue;
        int side = (i < 0) ? 0 : (i >= NX) ? 1 : (j < 0) ? 2 : (j >= NY) ? 3 : (k < 0) ? 4 : 5;
        int ii = i < 0 ? -i - 1 : i >= NX ? NX + (i - NX) - 1 : i;
        int jj = j < 0 ? -j - 1 : j >= NY ? NY + (j - NY) - 1 : j;
        int kk = k < 0 ? -k - 1 : k >= NZ ? NZ + (k - NZ) - 1 : k;
        int bc = cfg.ls_bc[side];
        double& g = phi[idx(i, j, k)];
        if (bc == M2CG_LSBC_ZERO_NEUMANN) { g = phi[idx(ii, jj, kk)]; continue; }
        int d = side / 2, sgn = (side % 2 == 0) ? +1 : -1;  // direction into the domain
        int n[3] = {NX, NY, NZ};
        int pos[3] = {i, j, k};
        int ok = (sgn > 0) ? (pos[d] + 2 < n[d]) : (pos[d] - 2 >= 0);
        if (ok) {
          int p1[3] = {i, j, k}, p2[3] = {i, j, k};
          p1[d] += sgn; p2[d] += 2 * sgn;
          // coordinates along d (uniform): r = x0 + (pos+0.5)h
          double lo[3] = {cfg.x0, cfg.y0, cfg.z0};
          double r = lo[d] + 0.5 * h[d] + pos[d] * h[d];
          double r1 = lo[d] + 0.5 * h[d] + p1[d] * h[d];
          double r2 = lo[d] + 0.5 * h[d] + p2[d] * h[d];
          double f1 = phi[idx(p1[0], p1[1], p1[2])], f2 = phi[idx(p2[0], p2[1], p2[2])];
          g = f1 + (f2 - f1) / (r2 - r1) * (r - r1);
        } else g = phi[idx(ii, jj, kk)];
        if (bc == M2CG_LSBC_NON_NEGATIVE) {
          double d2wall = 0.5 * h[d];  // 0.5*|x_image - x_ghost| for the first ghost layer
          g = std::max(-d2wall, g);
        }
      }
}

// MultiPhaseOperator.cpp:919-942
void Oracle::UpdateIDGhosts(std::vector<int>& id) {
  for (int k = -1; k <= NZ; k++)
    for (int j = -1; j <= NY; j++)
      for (int i = -1; i <= NX; i++) {
        if (nface_ghost(i, j, k) != 1) continue;
        int ii = i < 0 ? -i - 1 : i >= NX ? NX + (i - NX) - 1 : i;
        int jj = j < 0 ? -j - 1 : j >= NY ? NY + (j - NY) - 1 : j;
        int kk = k < 0 ? -k - 1 : k >= NZ ? NZ + (k - NZ) - 1 : k;
        id[idx(i, j, k)] = id[idx(ii, jj, kk)];
      }
}

// SpaceOperator.cpp:647-693 (real cells)
int Oracle::ClipAll(std::vector<double>& v, const std::vector<int>& id) {
  int n = 0;
  for (int k = 0; k < NZ; k++)
    for (int j = 0; j < NY; j++)
      for (int i = 0; i < NX; i++) {
        size_t c = idx(i, j, k);
        n += vf[id[c]].ClipDensityAndPressure(&v[c * 5]);
        if (vf[id[c]].CheckState(&v[c * 5])) cnt.nonphysical++;
      }
  return n;
}

void Oracle::P2C(const std::vector<double>& v, const std::vector<int>& id, std::vector<double>& u) {
#pragma omp parallel for schedule(static)
  for (int k = 0; k < NZ; k++)
    for (int j = 0; j < NY; j++)
      for (int i = 0; i < NX; i++) {
        size_t c = idx(i, j, k);
        vf[id[c]].PrimitiveToConservative(&v[c * 5], &u[c * 5]);
      }
}
void Oracle::C2P(const std::vector<double>& u, const std::vector<int>& id, std::vector<double>& v) {
#pragma omp parallel for schedule(static)
  for (int k = 0; k < NZ; k++)
    for (int j = 0; j < NY; j++)
      for (int i = 0; i < NX; i++) {
        size_t c = idx(i, j, k);
        vf[id[c]].ConservativeToPrimitive(&u[c * 5], &v[c * 5]);
      }
}

inline double GenMinMod(double A, double B, double alpha, double dq0, double dq1) {  // Reconstructor.h:96-103
  if (dq0 < 0.0 && dq1 < 0.0) return std::max(alpha * dq0, std::max(B / (A + 1.0) * (dq0 + dq1), alpha * dq1));
  else if (dq0 > 0.0 && dq1 > 0.0) return std::min(alpha * dq0, std::min(B / (A + 1.0) * (dq0 + dq1), alpha * dq1));
  return 0.0;
}
inline double VanAlbada(double A, double B, int k, double dq0, double dq1) {  // Reconstructor.h:105-111
  if (dq0 * dq1 <= 0) return 0.0;
  if (std::fabs(dq0 * dq1) < 1e-16) return 0.0;
  double a = std::pow(dq0, k), b = std::pow(dq1, k);
  return B * (dq1 * a + dq0 * b) / (a + A * b);
}

// Characteristic variables about a reference primitive state V0, direction
// dir (FluxFcnBase.h:308-517): the EOS quantities at V0, the left (R0^-1) and
// right (R0) eigenvector matrices of the Euler flux Jacobian in conservative
// form, and the primitive <-> conservative differential Q0.  Every entry and
// product follows the reference's expression order.
struct CharBasis {
  double e0, c0, dpdrho0, Gamma0, kin0;
};
static CharBasis char_basis(const Eos& e, const double* V0) {
  CharBasis b;
  b.e0 = e.GetInternalEnergyPerUnitMass(V0[0], V0[4]);
  b.c0 = std::sqrt(e.ComputeSoundSpeedSquare(V0[0], b.e0));   // the reference stops if c0^2 < 0
  b.dpdrho0 = e.GetDpdrho(V0[0], b.e0);
  b.Gamma0 = e.GetBigGamma(V0[0], b.e0);
  b.kin0 = 0.5 * (V0[1] * V0[1] + V0[2] * V0[2] + V0[3] * V0[3]);
  return b;
}
static void char_left(const CharBasis& b, const double* V0, int dir, double L[5][5]) {
  double n[3] = {0, 0, 0};
  n[dir] = 1.0;
  const double un0 = V0[dir + 1];
  const double alpha0 = V0[0] * b.Gamma0 / (V0[4] * b.Gamma0 + V0[0] * b.dpdrho0);
  const double beta0 = (b.e0 - b.kin0 + V0[4] / V0[0]) * alpha0;
  L[0][0] = 0.5 * (1.0 - beta0 + un0 / b.c0);
  L[4][0] = 0.5 * (1.0 - beta0 - un0 / b.c0);
  L[0][4] = L[4][4] = alpha0 / 2.0;
  for (int i = 0; i < 3; i++) {
    L[0][1 + i] = -0.5 * (alpha0 * V0[1 + i] + n[i] / b.c0);
    L[4][1 + i] = -0.5 * (alpha0 * V0[1 + i] - n[i] / b.c0);
    L[1 + i][0] = -V0[1 + i] + (beta0 + un0) * n[i];
    L[1 + i][4] = -alpha0 * n[i];
    for (int j = 0; j < 3; j++) L[1 + i][1 + j] = (i == j) + alpha0 * n[i] * V0[1 + j] - n[i] * n[j];
  }
}
static void char_right(const CharBasis& b, const double* V0, int dir, double R[5][5]) {
  double n[3] = {0, 0, 0};
  n[dir] = 1.0;
  const double un0 = V0[dir + 1];
  const double H0 = b.e0 + b.kin0 + V0[4] / V0[0];
  const double param = b.e0 + b.kin0 - b.dpdrho0 / b.Gamma0 - un0;
  R[0][0] = 1.0;
  R[0][4] = 1.0;
  R[4][0] = H0 - un0 * b.c0;
  R[4][4] = H0 + un0 * b.c0;
  for (int i = 0; i < 3; i++) {
    R[0][1 + i] = n[i];
    R[1 + i][0] = V0[1 + i] - b.c0 * n[i];
    R[1 + i][4] = V0[1 + i] + b.c0 * n[i];
    R[4][1 + i] = V0[1 + i] + param * n[i];
    for (int j = 0; j < 3; j++) R[1 + i][1 + j] = (i == j) + V0[1 + i] * n[j] - n[i] * n[j];
  }
}
static void matvec5(const double M[5][5], const double* x, double* y) {
  for (int i = 0; i < 5; i++) {
    y[i] = 0.0;
    for (int j = 0; j < 5; j++) y[i] += M[i][j] * x[j];
  }
}
// FluxFcnBase.h:308-359
static void PrimToPrimChar(const Eos& e, int dir, const double* V0, const double* dV, double* dW) {
  CharBasis b = char_basis(e, V0);
  const double Q0_51 = b.e0 + b.kin0 - b.dpdrho0 / b.Gamma0;
  double t[5];
  t[0] = dV[0];
  t[1] = V0[1] * dV[0] + V0[0] * dV[1];
  t[2] = V0[2] * dV[0] + V0[0] * dV[2];
  t[3] = V0[3] * dV[0] + V0[0] * dV[3];
  t[4] = Q0_51 * dV[0] + V0[0] * V0[1] * dV[1] + V0[0] * V0[2] * dV[2] + V0[0] * V0[3] * dV[3] + 1.0 / b.Gamma0 * dV[4];
  double L[5][5];
  char_left(b, V0, dir, L);
  matvec5(L, t, dW);
}
// FluxFcnBase.h:364-420
static void PrimCharToPrim(const Eos& e, int dir, const double* V0, const double* dW, double* dV) {
  CharBasis b = char_basis(e, V0);
  double R[5][5], t[5];
  char_right(b, V0, dir, R);
  matvec5(R, dW, t);
  dV[0] = t[0];
  dV[1] = -V0[1] / V0[0] * t[0] + t[1] / V0[0];
  dV[2] = -V0[2] / V0[0] * t[0] + t[2] / V0[0];
  dV[3] = -V0[3] / V0[0] * t[0] + t[3] / V0[0];
  dV[4] = ((-b.e0 + b.kin0) * b.Gamma0 + b.dpdrho0) * t[0] - b.Gamma0 * (V0[1] * t[1] + V0[2] * t[2] + V0[3] * t[3] - t[4]);
}
// FluxFcnBase.h:424-467
static void ConsToConsChar(const Eos& e, int dir, const double* V0, const double* dU, double* dW) {
  CharBasis b = char_basis(e, V0);
  double L[5][5];
  char_left(b, V0, dir, L);
  matvec5(L, dU, dW);
}
// FluxFcnBase.h:471-517
static void ConsCharToCons(const Eos& e, int dir, const double* V0, const double* dW, double* dU) {
  CharBasis b = char_basis(e, V0);
  double R[5][5];
  char_right(b, V0, dir, R);
  matvec5(R, dW, dU);
}

// Reconstructor.cpp:335-918.  fs[0..5] = vl, vr, vb, vt, vk, vf (ghosted, AoS).
// Slopes of primitive, conservative, primitive-characteristic or
// conservative-characteristic differences; a nonphysical face state restarts
// the cell with primitive variables, and in primitive variables the first
// nonphysical face reverts to the cell value (Reconstructor.cpp:722-778).
bool Oracle::Reconstruct(const std::vector<double>& v, const std::vector<int>& id, std::vector<double> fs[6]) {
  for (int f = 0; f < 6; f++) fs[f].assign(N() * 5, 0.0);
  const double A = 1.0, B = 1.0;   // uniform mesh: Reconstructor.cpp:78-84 give exactly 1
  int kay = 2;                     // CalculateSlopeLimiterCoefficientK(1,1) -> 2
  if (cfg.limiter == M2CG_LIM_VANALBADA) {
    for (kay = 2; kay < 1000; kay++) {
      double rhs = 2.0 / (1.0 + std::pow((kay - 1.0) / kay, kay - 1) / kay) * std::min(A, 1.0);
      if (B <= rhs) break;
    }
  }
  double alpha = cfg.minmod_coeff;
  int64_t sx = 5, sy = (int64_t)PX * 5, sz = (int64_t)PX * PY * 5;
  const int var0 = cfg.rec_var;
  // conservative state of the real and face-ghost cells, with each cell's own
  // material (Reconstructor.cpp:400-408; edge and corner ghosts are not read)
  std::vector<double> u;
  if (cfg.rec_type != M2CG_REC_CONSTANT && (var0 == M2CG_VAR_CONSERVATIVE || var0 == M2CG_VAR_CONSERVATIVE_CHARACTERISTIC)) {
    u.assign(N() * 5, 0.0);
    for (int k = -1; k <= NZ; k++)
      for (int j = -1; j <= NY; j++)
        for (int i = -1; i <= NX; i++) {
          if (nface_ghost(i, j, k) > 1) continue;
          size_t c = idx(i, j, k);
          vf[id[c]].PrimitiveToConservative(&v[c * 5], &u[c * 5]);
        }
  }
#pragma omp parallel for schedule(static)
  for (int k = 0; k < NZ; k++)
    for (int j = 0; j < NY; j++)
      for (int i = 0; i < NX; i++) {
        size_t c = idx(i, j, k);
        const double* q = &v[c * 5];
        if (cfg.rec_type == M2CG_REC_CONSTANT) {
          for (int f = 0; f < 6; f++) for (int p = 0; p < 5; p++) fs[f][c * 5 + p] = q[p];
          continue;
        }
        const Eos& e = vf[id[c]];
        int vt = var0;
        while (true) {
          const bool cons = (vt == M2CG_VAR_CONSERVATIVE || vt == M2CG_VAR_CONSERVATIVE_CHARACTERISTIC);
          const double* w = cons ? &u[c * 5] : q;   // the variables whose differences are limited
          double sig[3][5];
          int64_t st[3] = {sx, sy, sz};
          for (int d = 0; d < 3; d++) {
            double dq0[5], dq1[5];
            for (int p = 0; p < 5; p++) {
              dq0[p] = w[p] - w[p - st[d]];
              dq1[p] = w[p + st[d]] - w[p];
            }
            if (vt == M2CG_VAR_PRIMITIVE_CHARACTERISTIC) {
              double t[5];
              PrimToPrimChar(e, d, q, dq0, t); for (int p = 0; p < 5; p++) dq0[p] = t[p];
              PrimToPrimChar(e, d, q, dq1, t); for (int p = 0; p < 5; p++) dq1[p] = t[p];
            } else if (vt == M2CG_VAR_CONSERVATIVE_CHARACTERISTIC) {
              double t[5];
              ConsToConsChar(e, d, q, dq0, t); for (int p = 0; p < 5; p++) dq0[p] = t[p];
              ConsToConsChar(e, d, q, dq1, t); for (int p = 0; p < 5; p++) dq1[p] = t[p];
            }
            for (int p = 0; p < 5; p++) {
              double s;
              if (cfg.limiter == M2CG_LIM_GENERALIZED_MINMOD) s = GenMinMod(A, B, alpha, dq0[p], dq1[p]);
              else if (cfg.limiter == M2CG_LIM_VANALBADA) s = VanAlbada(A, B, kay, dq0[p], dq1[p]);
              else s = 0.5 * (dq0[p] + dq1[p]);
              sig[d][p] = s;
            }
          }
          // Reconstructor.cpp:620-644: back to primitive / conservative differences
          for (int d = 0; d < 3; d++) {
            double t[5];
            if (vt == M2CG_VAR_PRIMITIVE_CHARACTERISTIC) PrimCharToPrim(e, d, q, sig[d], t);
            else if (vt == M2CG_VAR_CONSERVATIVE_CHARACTERISTIC) ConsCharToCons(e, d, q, sig[d], t);
            else continue;
            for (int p = 0; p < 5; p++) sig[d][p] = t[p];
          }
          if (cfg.slope_near_interface == M2CG_SLOPE_ZERO) {   // Reconstructor.cpp:649-658
            size_t cs[3] = {1, (size_t)PX, (size_t)PX * PY};
            for (int d = 0; d < 3; d++)
              if (id[c] != id[c - cs[d]] || id[c] != id[c + cs[d]])
                for (int p = 0; p < 5; p++) sig[d][p] = 0.0;
          }
          if (!cons) {
            for (int p = 0; p < 5; p++) {   // Reconstructor.cpp:676-688
              fs[0][c * 5 + p] = q[p] - 0.5 * sig[0][p];
              fs[1][c * 5 + p] = q[p] + 0.5 * sig[0][p];
              fs[2][c * 5 + p] = q[p] - 0.5 * sig[1][p];
              fs[3][c * 5 + p] = q[p] + 0.5 * sig[1][p];
              fs[4][c * 5 + p] = q[p] - 0.5 * sig[2][p];
              fs[5][c * 5 + p] = q[p] + 0.5 * sig[2][p];
            }
          } else {                          // Reconstructor.cpp:689-716
            for (int f = 0; f < 6; f++) {
              double u2[5];
              for (int p = 0; p < 5; p++) u2[p] = (f % 2 == 0) ? w[p] - 0.5 * sig[f / 2][p] : w[p] + 0.5 * sig[f / 2][p];
              e.ConservativeToPrimitive(u2, &fs[f][c * 5]);
            }
          }
          // Reconstructor.cpp:722-778
          int bad = -1;
          for (int f = 0; f < 6 && bad < 0; f++)
            if (e.CheckState(&fs[f][c * 5])) bad = f;
          if (bad < 0) break;
          if (vt == M2CG_VAR_PRIMITIVE) {
            for (int p = 0; p < 5; p++) fs[bad][c * 5 + p] = q[p];
            break;
          }
          vt = M2CG_VAR_PRIMITIVE;
        }
      }
  // Ghost faces by boundary condition, Reconstructor.cpp:807-889
  for (int k = -1; k <= NZ; k++)
    for (int j = -1; j <= NY; j++)
      for (int i = -1; i <= NX; i++) {
        if (nface_ghost(i, j, k) != 1) continue;
        int side = (i < 0) ? 0 : (i >= NX) ? 1 : (j < 0) ? 2 : (j >= NY) ? 3 : (k < 0) ? 4 : 5;
        int ii = i < 0 ? -i - 1 : i >= NX ? NX + (i - NX) - 1 : i;
        int jj = j < 0 ? -j - 1 : j >= NY ? NY + (j - NY) - 1 : j;
        int kk = k < 0 ? -k - 1 : k >= NZ ? NZ + (k - NZ) - 1 : k;
        size_t g = idx(i, j, k), im = idx(ii, jj, kk);
        int inward = side ^ 1;      // face state of the ghost facing the domain: vr for the x0 ghost, ...
        int src = side;             // face state of the image on the boundary: vl of the image for x0
        int bc = cfg.bc[side];
        double* dst = &fs[inward][g * 5];
        if (bc == M2CG_BC_INLET || bc == M2CG_BC_INLET2) {
          for (int p = 0; p < 5; p++) dst[p] = v[g * 5 + p];
        } else if (bc == M2CG_BC_OUTLET) {
          for (int p = 0; p < 5; p++) dst[p] = fs[src][im * 5 + p];
        } else if (bc == M2CG_BC_SYMMETRY || bc == M2CG_BC_SLIPWALL) {
          for (int p = 0; p < 5; p++) dst[p] = fs[src][im * 5 + p];
          dst[1 + side / 2] *= -1.0;
        } else {  // STICKWALL: copyarray_flip(.., 1, 3) flips all three velocity components
          for (int p = 0; p < 5; p++) dst[p] = fs[src][im * 5 + p];
          dst[1] *= -1.0; dst[2] *= -1.0; dst[3] *= -1.0;
        }
      }
  return true;
}

// SpaceOperator.cpp:2420-2569
void Oracle::CheckReconstructed(const std::vector<double>& v, const std::vector<int>& id, std::vector<double> fs[6]) {
  int64_t nclip = 0, nbad = 0;
#pragma omp parallel for schedule(static) reduction(+ : nclip, nbad)
  for (int k = -1; k <= NZ; k++)
    for (int j = -1; j <= NY; j++)
      for (int i = -1; i <= NX; i++) {
        int boundary = (k == -1 || k == NZ) + (j == -1 || j == NY) + (i == -1 || i == NX);
        if (boundary >= 2) continue;
        size_t c = idx(i, j, k);
        const Eos& e = vf[id[c]];
        auto clip_one = [&](int f) {
          double* s = &fs[f][c * 5];
          double tmp[5];
          for (int p = 0; p < 5; p++) tmp[p] = s[p];
          if (e.ClipDensityAndPressure(tmp)) {
            for (int p = 0; p < 5; p++) s[p] = v[c * 5 + p];
            nclip++;
          }
          if (e.CheckState(s)) nbad++;
        };
        if (boundary == 0) { for (int f = 0; f < 6; f++) clip_one(f); }
        else {
          if (i == -1) clip_one(1);
          else if (i == NX) clip_one(0);
          else if (j == -1) clip_one(3);
          else if (j == NY) clip_one(2);
          else if (k == -1) clip_one(5);
          else if (k == NZ) clip_one(4);
        }
      }
  cnt.clipped_faces += nclip;
  cnt.nonphysical += nbad;
}

bool Oracle::NumFlux(int dir, const double* Vm, const double* Vp, int id, double* F) {
  if (cfg.flux == M2CG_FLUX_HLLC) return FluxHLLC(vf[id], dir, Vm, Vp, F);
  if (cfg.flux == M2CG_FLUX_LLF) return FluxLLF2(vf[id], vf[id], dir, Vm, Vp, F);
  return FluxGenRoe(vf[id], dir, Vm, Vp, cfg.roe_delta, F);
}

// SpaceOperator.cpp:1432-2076 then 2573-2641.  R is ghosted AoS; only real cells are meaningful.
// SpaceOperator::GetNormalForBimaterialRiemann (SpaceOperator.cpp:2186-2203)
// with CalculateGradPhiAtCellInterface (2208-2266, one level set) and
// CalculateGradientAtCellInterface (2270-2415) on the uniform mesh, for the face
// between cell (i,j,k) (material myid) and its minus neighbour along d (nid).
// Phi is phi at the start of the step while the residuals of a step are formed
// (TimeIntegrator.cpp:350, 403).  Faces whose materials are not 0 and the level
// set's (where the reference asserts) keep the mesh normal.
void Oracle::RiemannNormal(int d, int i, int j, int k, int myid, int nid, double dir[3]) const {
  dir[0] = dir[1] = dir[2] = 0.0;
  dir[d] = 1.0;
  const int my_ls = (myid == 0) ? nid : myid, neigh_ls = (nid == 0) ? myid : nid;
  if (cfg.mp_riemann_normal == M2CG_RNORMAL_MESH || my_ls != cfg.ls_matid || neigh_ls != cfg.ls_matid) return;
  const double lo[3] = {cfg.x0, cfg.y0, cfg.z0}, h[3] = {dx, dy, dz};
  const int n[3] = {NX, NY, NZ};
  auto X = [&](int a, int q) { return lo[a] + 0.5 * h[a] + q * h[a]; };   // coords (MeshGenerator.cpp:166-171)
  auto P = [&](const int* q) { return Phi[idx(q[0], q[1], q[2])]; };
  auto central = [](double p0, double p1, double p2, double x0, double x1, double x2) {   // SpaceOperator.h:223-228
    double c0 = -(x2 - x1) / ((x1 - x0) * (x2 - x0));
    double c1 = 1.0 / (x1 - x0) - 1.0 / (x2 - x1);
    double c2 = (x1 - x0) / ((x2 - x0) * (x2 - x1));
    return c0 * p0 + c1 * p1 + c2 * p2;
  };
  const int pc[3] = {i, j, k};
  int pm[3] = {i, j, k};
  pm[d] -= 1;
  double g[3];
  g[d] = (P(pc) - P(pm)) / (X(d, pc[d]) - X(d, pm[d]));
  const double x_minus_half = X(d, pc[d]) - 0.5 * h[d];
  const double dxd = X(d, pc[d]) - X(d, pm[d]);
  const double c1 = (X(d, pc[d]) - x_minus_half) / dxd;
  const double c2 = (x_minus_half - X(d, pm[d])) / dxd;
  for (int a = 0; a < 3; a++) {
    if (a == d) continue;
    const int q = pc[a];
    int mp[3] = {pm[0], pm[1], pm[2]}, mm[3] = {pm[0], pm[1], pm[2]}, cp[3] = {pc[0], pc[1], pc[2]},
        cmn[3] = {pc[0], pc[1], pc[2]};
    mp[a] += 1; mm[a] -= 1; cp[a] += 1; cmn[a] -= 1;
    double g1, g2;
    if (q < 0) {
      g1 = (P(mp) - P(pm)) / (X(a, q + 1) - X(a, q));
      g2 = (P(cp) - P(pc)) / (X(a, q + 1) - X(a, q));
    } else if (q >= n[a]) {
      g1 = (P(pm) - P(mm)) / (X(a, q) - X(a, q - 1));
      g2 = (P(pc) - P(cmn)) / (X(a, q) - X(a, q - 1));
    } else {
      g1 = central(P(mm), P(pm), P(mp), X(a, q - 1), X(a, q), X(a, q + 1));
      g2 = central(P(cmn), P(pc), P(cp), X(a, q - 1), X(a, q), X(a, q + 1));
    }
    g[a] = c1 * g1 + c2 * g2;
  }
  auto norm = [](const double* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); };
  double nrm = norm(g);
  if (nrm != 0.0) { double r = 1.0 / nrm; for (int a = 0; a < 3; a++) g[a] *= r; }   // Vec3D::operator/=
  if (nid == 0) for (int a = 0; a < 3; a++) g[a] *= -1.0;
  if (norm(g) == 0.0) g[d] = 1.0;
  if (g[d] < 0.0) g[d] *= -1.0;
  if (cfg.mp_riemann_normal == M2CG_RNORMAL_AVERAGE) {
    g[d] += 1.0;
    double r = 1.0 / norm(g);
    for (int a = 0; a < 3; a++) g[a] *= r;
  }
  for (int a = 0; a < 3; a++) dir[a] = g[a];
}

void Oracle::ComputeResidual(const std::vector<double>& v, const std::vector<int>& id, std::vector<double>& R, bool store) {
  std::vector<double> fs[6];
  Reconstruct(v, id, fs);
  CheckReconstructed(v, id, fs);
  if (store) for (int d = 0; d < 3; d++) for (auto& s : sol[d]) s.valid = false;
  // Per-face fluxes: lf1 goes to the minus cell, lf2 to the plus cell.  Face d of
  // cell c (plus cell) sits between c - e_d and c.
  std::vector<double> lf1[3], lf2[3];
  for (int d = 0; d < 3; d++) { lf1[d].assign(N() * 5, 0.0); lf2[d].assign(N() * 5, 0.0); }
  size_t cs[3] = {1, (size_t)PX, (size_t)PX * PY};
  int64_t n_if = 0, n_err = 0, n_iter = 0, n_solve = 0, n_fb = 0;
#pragma omp parallel reduction(+ : n_if, n_err, n_iter, n_solve, n_fb)
  {
    ExactRiemann riemann(vf, rp);
    Counters local;
#pragma omp for schedule(dynamic, 1)
    for (int k = 0; k <= NZ; k++)
      for (int j = 0; j <= NY; j++)
        for (int i = 0; i <= NX; i++) {
          int lim[3] = {(k != NZ && j != NY), (k != NZ && i != NX), (j != NY && i != NX)};
          size_t c = idx(i, j, k);
          int myid = id[c];
          for (int d = 0; d < 3; d++) {
            if (!lim[d]) continue;
            size_t m = c - cs[d];
            int nid = id[m];
            double* L1 = &lf1[d][c * 5];
            double* L2 = &lf2[d][c * 5];
            const double* vm_face = &fs[2 * d + 1][m * 5];   // vr / vt / vf of the minus cell
            const double* vp_face = &fs[2 * d][c * 5];       // vl / vb / vk of the plus cell
            if (nid != myid) {
              n_if++;
              const double* Vm = (cfg.mp_recon == M2CG_MPREC_CONSTANT) ? &v[m * 5] : vm_face;
              const double* Vp = (cfg.mp_recon == M2CG_MPREC_CONSTANT) ? &v[c * 5] : vp_face;
              if (cfg.mp_flux == M2CG_MPFLUX_LLF) {   // SpaceOperator.cpp:1617-1626
                FluxLLF2(vf[nid], vf[myid], d, Vm, Vp, L1);
                for (int p = 0; p < 5; p++) L2[p] = L1[p];
              } else {
                double dirv[3];
                RiemannNormal(d, i, j, k, myid, nid, dirv);
                double Vmid[5], Vsm[5], Vsp[5];
                int midid = 0;
                int err = riemann.Solve(dirv, Vm, nid, Vp, myid, Vmid, midid, Vsm, Vsp);
                n_solve++;
                n_iter += riemann.evals;
                n_fb += riemann.fallbacks;
                if (err) n_err++;
                vf[nid].ClipDensityAndPressure(Vsm);
                if (vf[nid].CheckState(Vsm)) local.nonphysical++;
                vf[myid].ClipDensityAndPressure(Vsp);
                if (vf[myid].CheckState(Vsp)) local.nonphysical++;
                if (store && !err) {
                  FaceSol& s = sol[d][c];
                  s.valid = true;
                  for (int p = 0; p < 5; p++) { s.Vsm[p] = Vsm[p]; s.Vsp[p] = Vsp[p]; }
                  s.idm = nid; s.idp = myid;
                }
                if (cfg.mp_flux == M2CG_MPFLUX_EXACT) {
                  EvaluateFlux(vf[midid], d, Vmid, L1);
                  for (int p = 0; p < 5; p++) L2[p] = L1[p];
                } else {
                  if (!NumFlux(d, Vm, Vsm, nid, L1)) local.nonphysical++;
                  if (!NumFlux(d, Vsp, Vp, myid, L2)) local.nonphysical++;
                }
              }
            } else {
              if (!NumFlux(d, vm_face, vp_face, myid, L1)) local.nonphysical++;
              for (int p = 0; p < 5; p++) L2[p] = L1[p];
            }
          }
        }
#pragma omp critical
    cnt.nonphysical += local.nonphysical;
  }
  cnt.interface_faces += n_if;
  cnt.riemann_errors += n_err;
  cnt.riemann_iterations += n_iter;
  cnt.riemann_solves += n_solve;
  cnt.fallbacks += n_fb;
  // Gather in the reference's accumulation order: -x, -y, -z faces, then +x, +y, +z.
  R.assign(N() * 5, 0.0);
  double area[3] = {dy * dz, dx * dz, dx * dy};
  double inv = 1.0 / (-vol);   // Vector5D.h:174-183 (r /= -vol multiplies by the reciprocal)
#pragma omp parallel for schedule(static)
  for (int k = 0; k < NZ; k++)
    for (int j = 0; j < NY; j++)
      for (int i = 0; i < NX; i++) {
        size_t c = idx(i, j, k);
        double f[5] = {0, 0, 0, 0, 0};
        for (int d = 0; d < 3; d++)
          for (int p = 0; p < 5; p++) f[p] -= lf2[d][c * 5 + p] * area[d];
        for (int d = 0; d < 3; d++)
          for (int p = 0; p < 5; p++) f[p] += lf1[d][(c + cs[d]) * 5 + p] * area[d];
        for (int p = 0; p < 5; p++) R[c * 5 + p] = f[p] * inv;
      }
}

// LevelSetOperator::ComputeLocalAdvectionFlux (LevelSetOperator.cpp:1265-1296)
static double LsFlux(int type, double delta, double phim, double phip, double um, double up) {
  if (type == M2CG_LSFLUX_UPWIND) {
    double vmid = 0.5 * (um + up);
    if (vmid > 0) return phim * um;
    if (vmid < 0) return phip * up;
    return 0.5 * (phim * um + phip * up);
  }
  if (type == M2CG_LSFLUX_LLF)
    return 0.5 * (phim * um + phip * up) - 0.5 * std::max(std::fabs(um), std::fabs(up)) * (phip - phim);
  double lam = std::fabs(0.5 * (um + up));
  double tol = std::max(std::fabs(um), std::fabs(up)) * delta;
  if (lam < tol) lam = (lam * lam + tol * tol) / (2 * tol);
  return 0.5 * (phim * um + phip * up) - 0.5 * lam * (phip - phim);
}

// Finite-volume level set (LevelSetOperator.cpp:966-1136, 1265-1324): the
// level set's own reconstructor gives face values of each velocity component
// along its direction (Reconstructor::ReconstructIn1D, Reconstructor.cpp:922-1176)
// and of phi in all directions (Reconstructor::Reconstruct with one DOF and no
// material IDs, Reconstructor.cpp:335-918); boundary faces take the ghost
// cells' inward values by boundary type; R = sum of the face fluxes (in the
// reference's loop order) + phi div(u).
void Oracle::LevelSetResidualFV(const std::vector<double>& v, const std::vector<double>& phi, std::vector<double>& R) {
  const size_t n = N();
  const double h[3] = {dx, dy, dz};
  const size_t cs[3] = {1, (size_t)PX, (size_t)PX * PY};
  const bool linear = (cfg.ls_rec_type == M2CG_REC_LINEAR);
  auto limit = [&](double dq0, double dq1) {
    if (cfg.ls_limiter == M2CG_LIM_GENERALIZED_MINMOD) return GenMinMod(1.0, 1.0, cfg.ls_minmod_coeff, dq0, dq1);
    if (cfg.ls_limiter == M2CG_LIM_VANALBADA) return VanAlbada(1.0, 1.0, 2, dq0, dq1);
    return 0.5 * (dq0 + dq1);
  };
  std::vector<double> um[3], up[3], slope[3], pf[6];
  for (int d = 0; d < 3; d++) { um[d].assign(n, 0.0); up[d].assign(n, 0.0); slope[d].assign(n, 0.0); }
  for (int f = 0; f < 6; f++) pf[f].assign(n, 0.0);
  // real cells
  for (int k = 0; k < NZ; k++)
    for (int j = 0; j < NY; j++)
      for (int i = 0; i < NX; i++) {
        size_t c = idx(i, j, k);
        for (int d = 0; d < 3; d++) {
          const double* u = &v[1 + d];   // velocity component d, stride 5
          double sig = 0.0;
          if (linear) sig = limit(u[c * 5] - u[(c - cs[d]) * 5], u[(c + cs[d]) * 5] - u[c * 5]);
          um[d][c] = u[c * 5] - 0.5 * sig;
          up[d][c] = u[c * 5] + 0.5 * sig;
          slope[d][c] = sig / h[d];
          double sp = 0.0;
          if (linear) sp = limit(phi[c] - phi[c - cs[d]], phi[c + cs[d]] - phi[c]);
          pf[2 * d][c] = phi[c] - 0.5 * sp;
          pf[2 * d + 1][c] = phi[c] + 0.5 * sp;
        }
      }
  // face-ghost cells: the inward face values
  for (int k = -1; k <= NZ; k++)
    for (int j = -1; j <= NY; j++)
      for (int i = -1; i <= NX; i++) {
        if (nface_ghost(i, j, k) != 1) continue;
        int side = (i < 0) ? 0 : (i >= NX) ? 1 : (j < 0) ? 2 : (j >= NY) ? 3 : (k < 0) ? 4 : 5;
        int ii = i < 0 ? 0 : i >= NX ? NX - 1 : i;
        int jj = j < 0 ? 0 : j >= NY ? NY - 1 : j;
        int kk = k < 0 ? 0 : k >= NZ ? NZ - 1 : k;
        size_t g = idx(i, j, k), im = idx(ii, jj, kk);
        int d = side / 2;
        bool low = (side % 2 == 0);
        int bc = cfg.bc[side];
        const double ug = v[g * 5 + 1 + d];
        // velocity along d (Reconstructor.cpp:1056-1152)
        double& uin = low ? up[d][g] : um[d][g];
        const double uimg = low ? um[d][im] : up[d][im];
        if (bc == M2CG_BC_INLET || bc == M2CG_BC_INLET2) uin = ug;
        else if (bc == M2CG_BC_OUTLET) uin = uimg;
        else uin = -uimg;
        // phi (Reconstructor.cpp:807-889; with one DOF the walls' sign flip touches nothing)
        double& pin = pf[low ? 2 * d + 1 : 2 * d][g];
        if (!linear || bc == M2CG_BC_INLET || bc == M2CG_BC_INLET2) pin = phi[g];
        else pin = pf[low ? 2 * d : 2 * d + 1][im];
      }
  // fluxes over the interior and the upper ghost layers (LevelSetOperator.cpp:1091-1122)
  std::vector<double> res(n, 0.0);
  for (int k = 0; k <= NZ; k++)
    for (int j = 0; j <= NY; j++)
      for (int i = 0; i <= NX; i++) {
        size_t c = idx(i, j, k);
        if (k != NZ && j != NY) {
          double f = LsFlux(cfg.ls_flux, cfg.ls_delta, pf[1][c - cs[0]], pf[0][c], up[0][c - cs[0]], um[0][c]) / h[0];
          res[c - cs[0]] -= f;
          res[c] += f;
        }
        if (k != NZ && i != NX) {
          double f = LsFlux(cfg.ls_flux, cfg.ls_delta, pf[3][c - cs[1]], pf[2][c], up[1][c - cs[1]], um[1][c]) / h[1];
          res[c - cs[1]] -= f;
          res[c] += f;
        }
        if (j != NY && i != NX) {
          double f = LsFlux(cfg.ls_flux, cfg.ls_delta, pf[5][c - cs[2]], pf[4][c], up[2][c - cs[2]], um[2][c]) / h[2];
          res[c - cs[2]] -= f;
          res[c] += f;
        }
      }
  R.assign(n, 0.0);
  for (int k = 0; k < NZ; k++)
    for (int j = 0; j < NY; j++)
      for (int i = 0; i < NX; i++) {
        size_t c = idx(i, j, k);
        R[c] = res[c] + phi[c] * (slope[0][c] + slope[1][c] + slope[2][c]);   // LevelSetOperator.cpp:1300-1324
      }
}

// LevelSetOperator.cpp:796-870 (full domain, finite difference)
void Oracle::LevelSetResidual(const std::vector<double>& v, const std::vector<double>& phi, std::vector<double>& R) {
  if (cfg.ls_solver == M2CG_LS_FINITE_VOLUME) { LevelSetResidualFV(v, phi, R); return; }
  R.assign(N(), 0.0);
  double h[3] = {dx, dy, dz};
  size_t cs[3] = {1, (size_t)PX, (size_t)PX * PY};
  int n[3] = {NX, NY, NZ};
#pragma omp parallel for schedule(static)
  for (int k = 0; k < NZ; k++)
    for (int j = 0; j < NY; j++)
      for (int i = 0; i < NX; i++) {
        size_t c = idx(i, j, k);
        int pos[3] = {i, j, k};
        double res = 0.0;
        double term[3];
        for (int d = 0; d < 3; d++) {
          size_t s = cs[d];
          // left-biased derivative (a, c, e): 3rd order if pos >= 1, else one-sided first order
          double gm, gp;
          if (pos[d] - 2 >= -1)
            gm = cl_[d][0] * phi[c - 2 * s] + cl_[d][1] * phi[c - s] + cl_[d][2] * phi[c] + cl_[d][3] * phi[c + s];
          else
            gm = (phi[c] - phi[c - s]) / h[d];
          // right-biased (b, d, f): 3rd order if pos + 2 <= N.  The reference's
          // right-biased y coefficients are 3rd order only when i < NY-1
          // (GradientCalculatorFD3.cpp:409, tests i instead of j).
          bool third = (pos[d] + 2 <= n[d]);
          if (third) {
            bool coeff3 = (d == 1) ? (i < NY - 1) : (pos[d] < n[d] - 1);
            if (coeff3)
              gp = cr_[d][0] * phi[c - s] + cr_[d][1] * phi[c] + cr_[d][2] * phi[c + s] + cr_[d][3] * phi[c + 2 * s];
            else
              gp = 0.0 * phi[c - s] + (-1.0 / h[d]) * phi[c] + (1.0 / h[d]) * phi[c + s] + 0.0 * phi[c + 2 * s];
          } else
            gp = (phi[c + s] - phi[c]) / h[d];
          double vel = v[c * 5 + 1 + d];
          term[d] = (vel >= 0 ? gm * vel : gp * vel);
        }
        res = term[0] + term[1] + term[2];
        R[c] = res * -1.0;
      }
}

// SpaceOperator.cpp:1223-1330
void Oracle::ComputeDt(const std::vector<double>& v, const std::vector<int>& id, double& dt, double& cfl) {
  double m = DBL_MAX;
  for (int k = 0; k < NZ; k++)
    for (int j = 0; j < NY; j++)
      for (int i = 0; i < NX; i++) {
        size_t c = idx(i, j, k);
        const double* q = &v[c * 5];
        const Eos& e = vf[id[c]];
        double cc = e.ComputeSoundSpeedSquare(q[0], e.GetInternalEnergyPerUnitMass(q[0], q[4]));
        cc = std::sqrt(std::max(cc, 0.0));
        // FluxFcnBase::EvaluateMaxEigenvalues (FluxFcnBase.h:286-303) recomputes c the same way
        double lf = std::fabs(q[1]) + cc, lg = std::fabs(q[2]) + cc, lh = std::fabs(q[3]) + cc;
        if (NX > 1) m = std::min(m, dx / lf);
        if (NY > 1) m = std::min(m, dy / lg);
        if (NZ > 1) m = std::min(m, dz / lh);
      }
  if (cfg.timestep > 0) { dt = cfg.timestep; cfl = dt / m; }
  else { cfl = cfg.cfl; dt = cfl * m; }
}

void Oracle::Advance(double dt) {
  // TimeIntegrator.cpp:333-339: Phi_tmp = Phi (including ghosts)
  std::vector<double> phi0 = Phi;
  size_t n5 = N() * 5;
  std::vector<double> R, Un(n5, 0.0), U1(n5, 0.0), V1 = V, V2, Rls, Phi1 = Phi;
  bool ls = cfg.n_levelsets > 0;
  int64_t nclip = 0;
  auto axpby = [&](std::vector<double>& x, double a, double b, const std::vector<double>& y, int dof) {
    for (int k = 0; k < NZ; k++)
      for (int j = 0; j < NY; j++)
        for (int i = 0; i < NX; i++) {
          size_t c = idx(i, j, k);
          for (int p = 0; p < dof; p++) x[c * dof + p] = a * x[c * dof + p] + b * y[c * dof + p];
        }
  };
  // Stage 1 (all schemes): U1 = Un + dt R(V)
  ComputeResidual(V, ID, R, true);
  P2C(V, ID, Un);
  axpby(U1, 0.0, 1.0, Un, 5);
  axpby(U1, 1.0, dt, R, 5);
  if (cfg.ts_type == M2CG_TS_FORWARD_EULER) {  // TimeIntegrator.cpp:167-250
    C2P(U1, ID, V);
    nclip += ClipAll(V, ID);
    ApplyBC(V);
    if (ls) {
      LevelSetResidual(V, Phi, Rls);   // FE uses the updated V (TimeIntegrator.cpp:215)
      axpby(Phi, 1.0, dt, Rls, 1);
      ApplyLSBC(Phi);
    }
  } else {
    C2P(U1, ID, V1);
    int clipped = ClipAll(V1, ID);
    nclip += clipped;
    if (clipped) P2C(V1, ID, U1);
    ApplyBC(V1);
    if (ls) {
      LevelSetResidual(V, Phi, Rls);
      axpby(Phi1, 0.0, 1.0, Phi, 1);
      axpby(Phi1, 1.0, dt, Rls, 1);
      ApplyLSBC(Phi1);
    }
    if (cfg.ts_type == M2CG_TS_RK2) {  // TimeIntegrator.cpp:400-428
      ComputeResidual(V1, ID, R, false);
      axpby(U1, 0.5, 0.5, Un, 5);
      axpby(U1, 1.0, 0.5 * dt, R, 5);
      C2P(U1, ID, V);
      nclip += ClipAll(V, ID);
      ApplyBC(V);
      if (ls) {
        LevelSetResidual(V1, Phi1, Rls);
        axpby(Phi, 0.5, 0.5, Phi1, 1);
        axpby(Phi, 1.0, 0.5 * dt, Rls, 1);
        ApplyLSBC(Phi);
      }
    } else {  // RK3, TimeIntegrator.cpp:602-680
      ComputeResidual(V1, ID, R, false);
      axpby(U1, 0.25, 0.75, Un, 5);
      axpby(U1, 1.0, 0.25 * dt, R, 5);
      V2 = V1;
      C2P(U1, ID, V2);
      clipped = ClipAll(V2, ID);
      nclip += clipped;
      if (clipped) P2C(V2, ID, U1);
      ApplyBC(V2);
      if (ls) {
        LevelSetResidual(V1, Phi1, Rls);
        axpby(Phi1, 0.25, 0.75, Phi, 1);
        axpby(Phi1, 1.0, 0.25 * dt, Rls, 1);
        ApplyLSBC(Phi1);
      }
      ComputeResidual(V2, ID, R, false);
      axpby(U1, 2.0 / 3.0, 1.0 / 3.0, Un, 5);
      axpby(U1, 1.0, 2.0 / 3.0 * dt, R, 5);
      C2P(U1, ID, V);
      nclip += ClipAll(V, ID);
      ApplyBC(V);
      if (ls) {
        LevelSetResidual(V2, Phi1, Rls);
        axpby(Phi, 1.0 / 3.0, 2.0 / 3.0, Phi1, 1);
        axpby(Phi, 1.0, 2.0 / 3.0 * dt, Rls, 1);
        ApplyLSBC(Phi);
      }
    }
  }
  cnt.clipped_cells += nclip;
  if (ls) EndOfStep(phi0);
  cnt.steps++;
}

// LevelSetReinitializer.cpp:960-1041 (ComputeResidualFullDomain): first-order
// Godunov upwind |grad phi| - 1 on the interior, R = -dt S (|grad phi| - 1)
// with dt = cfl min(dx, dy, dz) (scaled back where |res| > 1), first-layer
// nodes held (R = 0).  Returns the largest |res| over the other nodes.
double Oracle::ReinitResidual(const std::vector<double>& phi, const std::vector<char>& tag,
                              const std::vector<double>& sign, std::vector<double>& R, double cfl) {
  const double xlo[3] = {cfg.x0, cfg.y0, cfg.z0}, h[3] = {dx, dy, dz};
  auto coord = [&](int d, int i) { return xlo[d] + 0.5 * h[d] + i * h[d]; };  // MeshGenerator.cpp:166-171
  double max_res = 0.0;
  for (int k = 0; k < NZ; k++)
    for (int j = 0; j < NY; j++)
      for (int i = 0; i < NX; i++) {
        size_t c = idx(i, j, k);
        if (tag[c]) { R[c] = 0.0; continue; }
        double hmin = std::min(dx, std::min(dy, dz));
        double dt = cfl * hmin;
        double p = phi[c];
        double a = (p - phi[idx(i - 1, j, k)]) / (coord(0, i) - coord(0, i - 1));
        double b = (phi[idx(i + 1, j, k)] - p) / (coord(0, i + 1) - coord(0, i));
        double cc = (p - phi[idx(i, j - 1, k)]) / (coord(1, j) - coord(1, j - 1));
        double d = (phi[idx(i, j + 1, k)] - p) / (coord(1, j + 1) - coord(1, j));
        double e = (p - phi[idx(i, j, k - 1)]) / (coord(2, k) - coord(2, k - 1));
        double f = (phi[idx(i, j, k + 1)] - p) / (coord(2, k + 1) - coord(2, k));
        double ap = std::max(a, 0.0), am = std::min(a, 0.0), bp = std::max(b, 0.0), bm = std::min(b, 0.0);
        double cp = std::max(cc, 0.0), cm = std::min(cc, 0.0), dp = std::max(d, 0.0), dm = std::min(d, 0.0);
        double ep = std::max(e, 0.0), em = std::min(e, 0.0), fp = std::max(f, 0.0), fm = std::min(f, 0.0);
        double res;
        if (p >= 0) res = std::sqrt(std::max(ap * ap, bm * bm) + std::max(cp * cp, dm * dm) + std::max(ep * ep, fm * fm)) - 1.0;
        else res = std::sqrt(std::max(am * am, bp * bp) + std::max(cm * cm, dp * dp) + std::max(em * em, fp * fp)) - 1.0;
        if (std::fabs(res) <= 1.0) R[c] = -dt * sign[c] * res;
        else R[c] = -dt * sign[c] * res / std::fabs(res);
        max_res = std::max(max_res, std::fabs(res));
      }
  return max_res;
}

// LevelSetReinitializer.cpp:76-176 (ReinitializeFullDomain) with the default
// first-layer treatment FIXED (IoData.cpp:1428): tag the first layer
// (:304-437), sign function with eps = 1 (:601-623), RK3 in pseudo time until
// the residual or the largest relative change drops below the tolerance;
// after MaxIts without it, accept if the change is below 0.02, else restart
// from the input with CFL / 1.5 (the CFL stays reduced for later calls), and
// give up below CFL 0.02 (the reference stops the program; counted here).
bool Oracle::Reinitialize() {
  std::vector<char> tag(N(), 0);
  bool detected = false;
  for (int k = -1; k <= NZ; k++)
    for (int j = -1; j <= NY; j++)
      for (int i = -1; i <= NX; i++) {
        if (nface_ghost(i, j, k) > 1) continue;  // edge and corner ghosts are not populated
        double p = Phi[idx(i, j, k)];
        bool t = (i - 1 >= -1 && p * Phi[idx(i - 1, j, k)] <= 0) || (i + 1 <= NX && p * Phi[idx(i + 1, j, k)] <= 0) ||
                 (j - 1 >= -1 && p * Phi[idx(i, j - 1, k)] <= 0) || (j + 1 <= NY && p * Phi[idx(i, j + 1, k)] <= 0) ||
                 (k - 1 >= -1 && p * Phi[idx(i, j, k - 1)] <= 0) || (k + 1 <= NZ && p * Phi[idx(i, j, k + 1)] <= 0);
        // neighbours that are edge ghosts are not populated either; a face ghost's neighbours along the
        // face are edge ghosts, whose values the reference leaves untouched (zero here)
        tag[idx(i, j, k)] = t;
        if (t && !outside(i, j, k)) detected = true;
      }
  if (!detected) return false;
  reinit_calls++;
  std::vector<double> sign(N(), 0.0);
  double factor = 1.0 * std::min(dx, std::min(dy, dz));
  for (int k = -1; k <= NZ; k++)
    for (int j = -1; j <= NY; j++)
      for (int i = -1; i <= NX; i++) {
        size_t c = idx(i, j, k);
        sign[c] = Phi[c] / std::sqrt(Phi[c] * Phi[c] + factor * factor);
      }
  auto axpby = [&](std::vector<double>& x, double a, double b, const std::vector<double>& y) {
    for (int k = 0; k < NZ; k++)
      for (int j = 0; j < NY; j++)
        for (int i = 0; i < NX; i++) {
          size_t c = idx(i, j, k);
          x[c] = a * x[c] + b * y[c];
        }
  };
  std::vector<double> Phibk = Phi, Phi0(N(), 0.0), Phi1(N(), 0.0), R(N(), 0.0);
  const int maxIts = cfg.reinit_max_its;
  const double tol = cfg.reinit_tol;
  while (true) {
    double dphi_max = 0.0;
    int iter;
    for (iter = 0; iter < maxIts; iter++) {
      axpby(Phi0, 0.0, 1.0, Phi);
      double residual = ReinitResidual(Phi, tag, sign, R, reinit_cfl);
      if (residual < tol) break;
      axpby(Phi1, 0.0, 1.0, Phi);
      axpby(Phi1, 1.0, 1.0, R);
      ApplyLSBC(Phi1);
      ReinitResidual(Phi1, tag, sign, R, reinit_cfl);
      axpby(Phi1, 0.25, 0.75, Phi);
      axpby(Phi1, 1.0, 0.25, R);
      ApplyLSBC(Phi1);
      ReinitResidual(Phi1, tag, sign, R, reinit_cfl);
      axpby(Phi, 1.0 / 3.0, 2.0 / 3.0, Phi1);
      axpby(Phi, 1.0, 2.0 / 3.0, R);
      ApplyLSBC(Phi);
      dphi_max = 0.0;  // CalculateMaximumRelativeErrorFullDomain (:1966-1991)
      for (int k = 0; k < NZ; k++)
        for (int j = 0; j < NY; j++)
          for (int i = 0; i < NX; i++) {
            size_t c = idx(i, j, k);
            double e = std::fabs(Phi[c] - Phi0[c]);
            if (Phi[c] != 0) e /= std::fabs(Phi[c]);
            dphi_max = std::max(dphi_max, e);
          }
      if (dphi_max < tol) break;
    }
    reinit_iters += iter;
    if (iter < maxIts) return true;
    if (dphi_max < 0.02) return true;
    if (reinit_cfl < 0.02) { reinit_failures++; return true; }
    reinit_cfl /= 1.5;
    reinit_retries++;
    Phi = Phibk;
  }
}

// MultiPhaseOperator::UpdateMaterialIDByLevelSet (MultiPhaseOperator.cpp:153-357,
// one level set) from phi_old to Phi, then the ID ghosts.
void Oracle::UpdateIDByLevelSet(const std::vector<double>& phi_old) {
  int lsmat = cfg.ls_matid;
  std::vector<char> tag(N(), 0);
  std::vector<std::array<int, 3>> remaining;
  for (int k = 0; k < NZ; k++)
    for (int j = 0; j < NY; j++)
      for (int i = 0; i < NX; i++) {
        size_t c = idx(i, j, k);
        if (Phi[c] * phi_old[c] > 0.0) continue;
        if (Phi[c] < 0) ID[c] = lsmat;
        else { tag[c] = 1; remaining.push_back({i, j, k}); }
      }
  for (int iter = 0; iter < 100 && !remaining.empty(); iter++) {
    int progress = 0;
    auto tmp = remaining;
    std::vector<std::array<int, 3>> still;
    std::set<std::array<int, 3>> done;
    // the reference walks a std::set<Int3> ordered by (i, j, k) components
    std::sort(tmp.begin(), tmp.end());
    for (auto& p : tmp) {
      int i = p[0], j = p[1], k = p[2];
      std::set<int> cands;
      for (int nk = k - 1; nk <= k + 1; nk++)
        for (int nj = j - 1; nj <= j + 1; nj++)
          for (int ni = i - 1; ni <= i + 1; ni++) {
            if (outside(ni, nj, nk)) continue;
            size_t nc = idx(ni, nj, nk);
            if (tag[nc] == 1) continue;
            int nid = ID[nc];
            if (nid == lsmat) continue;
            cands.insert(nid);
          }
      if (cands.empty()) continue;
      size_t c = idx(i, j, k);
      ID[c] = *cands.begin();
      tag[c] = 0;
      done.insert(p);
      progress++;
    }
    for (auto& p : remaining) if (!done.count(p)) still.push_back(p);
    remaining.swap(still);
    if (progress == 0) {
      for (auto& p : tmp) ID[idx(p[0], p[1], p[2])] = 0;
      remaining.clear();
      break;
    }
  }
  UpdateIDGhosts(ID);
}

// MultiPhaseOperator::FixUnresolvedNodes (MultiPhaseOperator.cpp:1279-1480; no
// embedded surfaces, failsafe density applied): each unresolved cell takes the
// upwind-weighted mean of its resolved same-material neighbours (weight =
// max(0, unit neighbour velocity . unit direction from the neighbour to the
// cell)), else their inverse-distance mean, else keeps pressure and velocity
// and takes an inverse-distance density from up to 10 layers, else the
// material's failsafe density.  As in the reference, the flag marking the
// first accumulated neighbour is set once for the whole list (line 1296), so
// later cells add their upwind neighbours onto their own advected state.
void Oracle::FixUnresolvedNodes(const std::vector<std::array<int, 3>>& unresolved) {
  const double lo[3] = {cfg.x0, cfg.y0, cfg.z0}, h[3] = {dx, dy, dz};
  auto coord = [&](int i, int j, int k, double* x) {
    const int q[3] = {i, j, k};
    for (int d = 0; d < 3; d++) x[d] = lo[d] + 0.5 * h[d] + q[d] * h[d];
  };
  auto listed = [&](int i, int j, int k) {
    for (auto& p : unresolved) if (p[0] == i && p[1] == j && p[2] == k) return true;
    return false;
  };
  bool reset = false;
  for (auto& p : unresolved) {
    const int i = p[0], j = p[1], k = p[2];
    const size_t c = idx(i, j, k);
    double x0[3];
    coord(i, j, k, x0);
    double sum_weight = 0.0, sum_weight2 = 0.0, vtmp[5] = {0, 0, 0, 0, 0};
    for (int nk = k - 1; nk <= k + 1; nk++)
      for (int nj = j - 1; nj <= j + 1; nj++)
        for (int ni = i - 1; ni <= i + 1; ni++) {
          if (outside(ni, nj, nk)) continue;
          const size_t nc = idx(ni, nj, nk);
          if (ID[nc] != ID[c]) continue;
          if (ni == i && nj == j && nk == k) continue;
          if (listed(ni, nj, nk)) continue;
          double x1[3], v1[3], d[3];
          coord(ni, nj, nk, x1);
          for (int q = 0; q < 3; q++) v1[q] = V[nc * 5 + 1 + q];
          double v1norm = std::sqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
          if (v1norm != 0) { double r = 1.0 / v1norm; for (int q = 0; q < 3; q++) v1[q] *= r; }
          for (int q = 0; q < 3; q++) d[q] = x0[q] - x1[q];
          double dn = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
          { double r = 1.0 / dn; for (int q = 0; q < 3; q++) d[q] *= r; }
          double weight = std::max(0.0, d[0] * v1[0] + d[1] * v1[1] + d[2] * v1[2]);
          if (weight > 0) {
            sum_weight += weight;
            for (int q = 0; q < 5; q++) {
              if (reset) V[c * 5 + q] += weight * V[nc * 5 + q];
              else V[c * 5 + q] = weight * V[nc * 5 + q];
            }
            reset = true;
          }
          for (int q = 0; q < 5; q++) vtmp[q] += 1.0 / dn * V[nc * 5 + q];
          sum_weight2 += 1.0 / dn;
        }
    if (cfg.mp_phasechange_dir == M2CG_PCDIR_UPWIND && sum_weight > 0) {
      double r = 1.0 / sum_weight;
      for (int q = 0; q < 5; q++) V[c * 5 + q] *= r;
      continue;
    }
    if (sum_weight2 > 0) {
      for (int q = 0; q < 5; q++) V[c * 5 + q] = vtmp[q] / sum_weight2;
      continue;
    }
    double density = 0.0;
    for (int layer = 1; layer <= 10; layer++) {
      for (int nk = k - layer; nk <= k + layer; nk++)
        for (int nj = j - layer; nj <= j + layer; nj++)
          for (int ni = i - layer; ni <= i + layer; ni++) {
            if (outside(ni, nj, nk)) continue;
            if (ni < -1 || ni > NX || nj < -1 || nj > NY || nk < -1 || nk > NZ) continue;
            const size_t nc = idx(ni, nj, nk);
            if (ID[nc] != ID[c]) continue;
            if (ni == i && nj == j && nk == k) continue;
            if (listed(ni, nj, nk)) continue;
            double x1[3];
            coord(ni, nj, nk, x1);
            double dist = std::sqrt((x1[0] - x0[0]) * (x1[0] - x0[0]) + (x1[1] - x0[1]) * (x1[1] - x0[1]) +
                                    (x1[2] - x0[2]) * (x1[2] - x0[2]));
            sum_weight += 1.0 / dist;
            density += (1.0 / dist) * V[nc * 5];
          }
      if (sum_weight > 0) { V[c * 5] = density / sum_weight; break; }
    }
    if (sum_weight == 0) V[c * 5] = cfg.mat[ID[c]].failsafe_density;
  }
}

// TimeIntegrator.cpp:720-843 with MultiPhaseOperator.cpp:153-357, 947-1274.
void Oracle::EndOfStep(std::vector<double>& phi0) {
  std::vector<int> IDn = ID;
  int lsmat = cfg.ls_matid;
  UpdateIDByLevelSet(phi0);
  // level-set reinitialization at the user frequency (TimeIntegrator.cpp:756-768,
  // LevelSetOperator.cpp:1338-1361, Utils.cpp:337-357 with frequency_dt unset)
  bool due = (cfg.reinit_frequency_dt > 0)
                 ? std::floor(time / cfg.reinit_frequency_dt) != std::floor((time - last_dt) / cfg.reinit_frequency_dt)
                 : (cfg.reinit_frequency > 0 && time_step % cfg.reinit_frequency == 0);
  if (due) Reinitialize();
  // UpdateStateVariablesAfterInterfaceMotion
  std::vector<std::array<int, 3>> unresolved;
  std::vector<double> Vold = V;
  size_t cs[3] = {1, (size_t)PX, (size_t)PX * PY};
  for (int k = 0; k < NZ; k++)
    for (int j = 0; j < NY; j++)
      for (int i = 0; i < NX; i++) {
        size_t c = idx(i, j, k);
        if (ID[c] == IDn[c]) continue;
        cnt.swept_cells++;
        int myid = ID[c];
        if (cfg.mp_phasechange == M2CG_PHASECHANGE_RIEMANN) {
          // LocalUpdateByRiemannSolutions, MultiPhaseOperator.cpp:1039-1150 (upwind, then not)
          int counter = 0;
          for (int pass = 0; pass < 2 && counter == 0; pass++) {
            bool upwind = (pass == 0);
            double acc[5] = {0, 0, 0, 0, 0};
            double sum_weight = 0;
            for (int d = 0; d < 3; d++)
              for (int side = 0; side < 2; side++) {
                // side 0: face at c - e_d (left/bottom/back entry: Vsm, id of the minus cell)
                // side 1: face at c + e_d (right/top/front entry: Vsp, id of the plus cell)
                size_t fc = side == 0 ? c : c + cs[d];
                const FaceSol& s = sol[d][fc];
                if (!s.valid) continue;
                int sid = side == 0 ? s.idm : s.idp;
                const double* sv = side == 0 ? s.Vsm : s.Vsp;
                size_t nb = side == 0 ? c - cs[d] : c + cs[d];
                const double* vn = &V[nb * 5];
                double vel = vn[1 + d];
                bool upw_ok = side == 0 ? (vel > 0) : (vel < 0);
                if (sid != myid || (upwind && !upw_ok)) continue;
                double nrm = std::sqrt(vn[1] * vn[1] + vn[2] * vn[2] + vn[3] * vn[3]);
                double weight = upwind ? (side == 0 ? vel / nrm : -vel / nrm) : 1.0;
                sum_weight += weight;
                for (int p = 0; p < 5; p++) {
                  if (counter == 0) acc[p] = weight * sv[p];
                  else acc[p] += weight * sv[p];
                }
                counter++;
              }
            if (counter > 0) {
              double* dst = &V[c * 5];
              if (sum_weight > 0.0) { double inv = 1.0 / sum_weight; for (int p = 0; p < 5; p++) dst[p] = acc[p] * inv; }
              else for (int p = 0; p < 5; p++) dst[p] = acc[p];
            }
          }
          if (counter == 0) unresolved.push_back({i, j, k});
        } else {
          // UpdateStateVariablesByExtrapolation, MultiPhaseOperator.cpp:1155-1274
          double sum_weight = 0.0, vsum[5] = {0, 0, 0, 0, 0};
          double hx[3] = {dx, dy, dz};
          for (int nk = k - 1; nk <= k + 1; nk++)
            for (int nj = j - 1; nj <= j + 1; nj++)
              for (int ni = i - 1; ni <= i + 1; ni++) {
                size_t nc = idx(ni, nj, nk);
                if (ID[nc] != ID[c]) continue;
                if (ID[nc] != IDn[nc]) continue;
                if (outside(ni, nj, nk)) continue;
                double x1x0[3] = {(i - ni) * hx[0], (j - nj) * hx[1], (k - nk) * hx[2]};
                double dist = std::sqrt(x1x0[0] * x1x0[0] + x1x0[1] * x1x0[1] + x1x0[2] * x1x0[2]);
                double weight;
                if (cfg.mp_phasechange_dir == M2CG_PCDIR_ALL) weight = 1.0 / dist;
                else {
                  const double* q = &V[nc * 5];
                  double v1[3] = {q[1], q[2], q[3]};
                  double v1n = std::sqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
                  if (v1n != 0) for (int m = 0; m < 3; m++) v1[m] /= v1n;
                  for (int m = 0; m < 3; m++) x1x0[m] /= dist;
                  weight = std::max(0.0, x1x0[0] * v1[0] + x1x0[1] * v1[1] + x1x0[2] * v1[2]);
                }
                if (weight > 0) {
                  sum_weight += weight;
                  for (int p = 0; p < 5; p++) vsum[p] += weight * V[nc * 5 + p];
                }
              }
          if (sum_weight == 0) unresolved.push_back({i, j, k});
          else for (int p = 0; p < 5; p++) V[c * 5 + p] = vsum[p] / sum_weight;  // Vector5D.h:190-200
        }
      }
  cnt.unresolved_cells += (int64_t)unresolved.size();
  // Unresolved cells (TimeIntegrator.cpp:776-797): background cells among them
  // return to the level set's material (phi -> -phi), the level set is
  // reinitialized, the IDs follow the sign changes, and the states are
  // extrapolated from resolved neighbours.  The reinitialization is
  // mandatory there; without a configured reinitializer the reference stops,
  // and the oracle counts the cells and leaves their state as advected.
  if (!unresolved.empty() && (cfg.reinit_frequency > 0 || cfg.reinit_frequency_dt > 0)) {
    std::vector<double> phi_tmp = Phi;
    for (auto& p : unresolved) {   // UpdateLevelSetsInUnresolvedCells, MultiPhaseOperator.cpp:1364-1420
      size_t c = idx(p[0], p[1], p[2]);
      if (!(Phi[c] < 0)) Phi[c] = -Phi[c];
    }
    Reinitialize();
    UpdateIDByLevelSet(phi_tmp);
    FixUnresolvedNodes(unresolved);
    cnt.unresolved_fixed += (int64_t)unresolved.size();
  }
  ClipAll(V, ID);
  ApplyBC(V);
}

}  // namespace

// ---------------------------------------------------------------------------
// C API for the tests (ctypes).
extern "C" {

void* orc_create(const m2cg_config* cfg) {
  Oracle* o = new Oracle();
  o->setup(*cfg);
  o->reinit_cfl = cfg->reinit_cfl;
  return o;
}
void orc_destroy(void* h) { delete (Oracle*)h; }

void orc_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n);
#else
  (void)n;
#endif
}
int orc_max_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_upload(void* h, const double* V, const int32_t* id, const double* phi) {
  Oracle* o = (Oracle*)h;
  size_t n = 0;
  for (int k = 0; k < o->NZ; k++)
    for (int j = 0; j < o->NY; j++)
      for (int i = 0; i < o->NX; i++, n++) {
        size_t c = o->idx(i, j, k);
        for (int p = 0; p < 5; p++) o->V[c * 5 + p] = V[n * 5 + p];
        o->ID[c] = id[n];
        if (phi) o->Phi[c] = phi[n];
      }
  o->UpdateIDGhosts(o->ID);
  o->ApplyBC(o->V);
  if (o->cfg.n_levelsets > 0) o->ApplyLSBC(o->Phi);
}

void orc_download(void* h, double* V, int32_t* id, double* phi) {
  Oracle* o = (Oracle*)h;
  size_t n = 0;
  for (int k = 0; k < o->NZ; k++)
    for (int j = 0; j < o->NY; j++)
      for (int i = 0; i < o->NX; i++, n++) {
        size_t c = o->idx(i, j, k);
        if (V) for (int p = 0; p < 5; p++) V[n * 5 + p] = o->V[c * 5 + p];
        if (id) id[n] = o->ID[c];
        if (phi) phi[n] = o->Phi[c];
      }
}

// The ghosted arrays (ghost width 1, i fastest): V as 5 planes, id, phi.
void orc_download_ghosted(void* h, double* V, int32_t* id, double* phi) {
  Oracle* o = (Oracle*)h;
  const size_t n = o->N();
  for (size_t c = 0; c < n; c++) {
    if (V) for (int p = 0; p < 5; p++) V[(size_t)p * n + c] = o->V[c * 5 + p];
    if (id) id[c] = o->ID[c];
    if (phi) phi[c] = o->Phi[c];
  }
}

void orc_residual(void* h, double* Rout) {
  Oracle* o = (Oracle*)h;
  std::vector<double> R;
  o->ComputeResidual(o->V, o->ID, R, true);
  size_t n = 0;
  for (int k = 0; k < o->NZ; k++)
    for (int j = 0; j < o->NY; j++)
      for (int i = 0; i < o->NX; i++, n++)
        for (int p = 0; p < 5; p++) Rout[n * 5 + p] = R[o->idx(i, j, k) * 5 + p];
}

void orc_levelset_residual(void* h, double* Rout) {
  Oracle* o = (Oracle*)h;
  std::vector<double> R;
  o->LevelSetResidual(o->V, o->Phi, R);
  size_t n = 0;
  for (int k = 0; k < o->NZ; k++)
    for (int j = 0; j < o->NY; j++)
      for (int i = 0; i < o->NX; i++, n++) Rout[n] = R[o->idx(i, j, k)];
}

// One full-domain reinitialization of the level set now (the call the
// stepping makes every reinit_frequency steps); returns 1 if an interface was
// found.  stats (optional): {calls, iterations, retries, failures, cfl}.
int orc_reinitialize(void* h, double* stats) {
  Oracle* o = (Oracle*)h;
  int r = o->Reinitialize() ? 1 : 0;
  if (stats) {
    stats[0] = o->reinit_calls; stats[1] = o->reinit_iters; stats[2] = o->reinit_retries;
    stats[3] = o->reinit_failures; stats[4] = o->reinit_cfl;
  }
  return r;
}

void orc_compute_dt(void* h, double* dt, double* cfl) {
  Oracle* o = (Oracle*)h;
  o->ComputeDt(o->V, o->ID, *dt, *cfl);
}

void orc_advance(void* h, double dt) {
  Oracle* o = (Oracle*)h;
  o->time_step++;
  o->time += dt;
  o->last_dt = dt;
  o->Advance(dt);
}

// Main.cpp:653-712 for n steps; returns steps taken.
int orc_run(void* h, int nsteps) {
  Oracle* o = (Oracle*)h;
  int s = 0;
  double tmax = o->cfg.max_time;
  for (; s < nsteps; s++) {
    double dt, cfl;
    o->ComputeDt(o->V, o->ID, dt, cfl);
    if (!(o->time < tmax - 1.0e-6 * dt)) break;
    if (o->time + dt > tmax) { cfl *= (tmax - o->time) / dt; dt = tmax - o->time; }
    o->last_cfl = cfl;
    orc_advance(h, dt);
  }
  return s;
}

void orc_counters(void* h, m2cg_counters* c) {
  Oracle* o = (Oracle*)h;
  std::memset(c, 0, sizeof(*c));
  c->interface_faces = o->cnt.interface_faces;
  c->riemann_errors = o->cnt.riemann_errors;
  c->riemann_iterations = o->cnt.riemann_iterations;
  c->riemann_solves = o->cnt.riemann_solves;
  c->clipped_cells = o->cnt.clipped_cells;
  c->clipped_faces = o->cnt.clipped_faces;
  c->nonphysical = o->cnt.nonphysical;
  c->swept_cells = o->cnt.swept_cells;
  c->unresolved_cells = o->cnt.unresolved_cells;
  c->steps = o->cnt.steps;
  c->time = o->time;
  c->dt = o->last_dt;
  c->cfl = o->last_cfl;
  c->riemann_fallbacks = o->cnt.fallbacks;
  c->unresolved_fixed = o->cnt.unresolved_fixed;
}

// The interface Riemann normal of the face between cell (i,j,k) and its minus
// neighbour along d, from the current level set (unit tests of RiemannNormal).
void orc_riemann_normal(void* h, int d, int i, int j, int k, int myid, int nid, double* dir) {
  ((Oracle*)h)->RiemannNormal(d, i, j, k, myid, nid, dir);
}

// Compensated (Neumaier) sums: a plain running sum over 16.8M cells drifts by
// ~1e-10 relative, larger than the differences the totals are compared for.
void orc_conserved_totals(void* h, double* tot) {
  Oracle* o = (Oracle*)h;
  double sum[5] = {0, 0, 0, 0, 0}, comp[5] = {0, 0, 0, 0, 0};
  for (int k = 0; k < o->NZ; k++)
    for (int j = 0; j < o->NY; j++)
      for (int i = 0; i < o->NX; i++) {
        size_t c = o->idx(i, j, k);
        double U[5];
        o->vf[o->ID[c]].PrimitiveToConservative(&o->V[c * 5], U);
        for (int p = 0; p < 5; p++) {
          double x = U[p] * o->vol, t = sum[p] + x;
          comp[p] += (std::fabs(sum[p]) >= std::fabs(x)) ? (sum[p] - t) + x : (x - t) + sum[p];
          sum[p] = t;
        }
      }
  for (int p = 0; p < 5; p++) tot[p] = sum[p] + comp[p];
}

// EnergyIntegrationOutput::IntegrateVolume / Mass / TotalEnergy / TotalEnthalpy /
// KineticEnergy / InternalEnergy (EnergyIntegrationOutput.cpp:247-610, Cartesian
// mesh): per material, over the cells whose centres lie in the box, in (k, j, i)
// order.  out[n_materials * 6].
void orc_integrate(void* h, const double* box, double* out) {
  Oracle* o = (Oracle*)h;
  const int nm = o->cfg.n_materials;
  for (int q = 0; q < nm * 6; q++) out[q] = 0.0;
  const double lo[3] = {o->cfg.x0, o->cfg.y0, o->cfg.z0}, hh[3] = {o->dx, o->dy, o->dz};
  for (int k = 0; k < o->NZ; k++)
    for (int j = 0; j < o->NY; j++)
      for (int i = 0; i < o->NX; i++) {
        const int q3[3] = {i, j, k};
        bool in = true;
        for (int d = 0; d < 3; d++) {
          const double x = lo[d] + 0.5 * hh[d] + q3[d] * hh[d];   // MeshGenerator.cpp:166-171
          if (box && !(x >= box[2 * d] && x <= box[2 * d + 1])) in = false;
        }
        if (!in) continue;
        const size_t c = o->idx(i, j, k);
        const int m = o->ID[c];
        const double* v = &o->V[c * 5];
        const double vsq = v[1] * v[1] + v[2] * v[2] + v[3] * v[3];
        const double e = o->vf[m].GetInternalEnergyPerUnitMass(v[0], v[4]);
        double* a = out + m * 6;
        a[0] += o->vol;
        a[1] += v[0] * o->vol;
        a[2] += v[0] * (0.5 * vsq + e) * o->vol;
        a[3] += (v[0] * (0.5 * vsq + e) + v[4]) * o->vol;
        a[4] += 0.5 * v[0] * vsq * o->vol;
        a[5] += v[0] * e * o->vol;
      }
}

// Batched exact Riemann solves (ExactRiemannSolverBase.cpp:59-347).
void orc_riemann_batch(const m2cg_config* cfg, int64_t n, const double* Vm, const int32_t* idm, const double* Vp,
                       const int32_t* idp, const double* dir, double* Vs, int32_t* id, double* Vsm, double* Vsp,
                       int32_t* iters, int32_t* err, const double* warm_p) {
  std::vector<Eos> vf(cfg->n_materials);
  for (int m = 0; m < cfg->n_materials; m++) vf[m].setup(cfg->mat[m]);
  RiemannParams rp;
  rp.maxIts_main = cfg->maxits_main; rp.maxIts_bracket = cfg->maxits_bracket; rp.maxIts_shock = cfg->maxits_shock;
  rp.numSteps_rarefaction = cfg->numsteps_rarefaction; rp.tol_main = cfg->tol_main; rp.tol_shock = cfg->tol_shock;
  rp.tol_rarefaction = cfg->tol_rarefaction; rp.min_pressure = cfg->min_pressure;
  rp.failure_threshold = cfg->failure_threshold; rp.pressure_at_failure = cfg->pressure_at_failure;
#pragma omp parallel
  {
    ExactRiemann rs(vf, rp);
#pragma omp for schedule(dynamic, 16)
    for (int64_t q = 0; q < n; q++) {
      int oid = 0;
      rs.warm_p = warm_p ? warm_p[q] : 0.0;
      int e = rs.Solve(&dir[q * 3], &Vm[q * 5], idm[q], &Vp[q * 5], idp[q], &Vs[q * 5], oid, &Vsm[q * 5], &Vsp[q * 5]);
      id[q] = oid;
      if (iters) iters[q] = rs.evals;
      if (err) err[q] = e;
    }
  }
}

// Batched 1D problems with a material pair each (the warm-start data sets):
// W rows {rho_l, u_l, p_l, rho_r, u_r, p_r}, E rows {type, gamma, pc, b, q}
// left then right, out rows {p*, u*, rho*_l, rho*_r}; the solver parameters
// come from cfg.
void orc_riemann_batch_eos(const m2cg_config* cfg, int64_t n, const double* W, const double* E, const double* warm_p,
                           double* out, int32_t* iters, int32_t* err) {
  RiemannParams rp;
  rp.warm_gate = 0.0;   // given starting pressures are used on every problem
  rp.maxIts_main = cfg->maxits_main; rp.maxIts_bracket = cfg->maxits_bracket; rp.maxIts_shock = cfg->maxits_shock;
  rp.numSteps_rarefaction = cfg->numsteps_rarefaction; rp.tol_main = cfg->tol_main; rp.tol_shock = cfg->tol_shock;
  rp.tol_rarefaction = cfg->tol_rarefaction; rp.min_pressure = cfg->min_pressure;
  rp.failure_threshold = cfg->failure_threshold; rp.pressure_at_failure = cfg->pressure_at_failure;
#pragma omp parallel
  {
    std::vector<Eos> vf(2);
    ExactRiemann rs(vf, rp);
#pragma omp for schedule(dynamic, 16)
    for (int64_t q = 0; q < n; q++) {
      for (int side = 0; side < 2; side++) {
        const double* e = &E[q * 10 + side * 5];
        m2cg_material m;
        memset(&m, 0, sizeof(m));
        m.eos = (int32_t)e[0]; m.gamma = e[1]; m.pc = e[2]; m.b = e[3]; m.q = e[4];
        m.rhomin = 0.0; m.pmin = -DBL_MAX; m.rhomax = DBL_MAX; m.pmax = DBL_MAX;
        vf[side].setup(m);
      }
      const double* w = &W[q * 6];
      double Vm[5] = {w[0], w[1], 0.0, 0.0, w[2]}, Vp[5] = {w[3], w[4], 0.0, 0.0, w[5]};
      double dir[3] = {1.0, 0.0, 0.0}, Vs[5], Vsm[5], Vsp[5];
      int oid = 0;
      rs.warm_p = warm_p ? warm_p[q] : 0.0;
      int e = rs.Solve(dir, Vm, 0, Vp, 1, Vs, oid, Vsm, Vsp);
      out[q * 4 + 0] = Vsm[4]; out[q * 4 + 1] = Vsm[1]; out[q * 4 + 2] = Vsm[0]; out[q * 4 + 3] = Vsp[0];
      if (iters) iters[q] = rs.evals;
      if (err) err[q] = e;
    }
  }
}

// Batched numerical fluxes (FluxFcnHLLC.h:196-245, FluxFcnLLF.h:80-111, FluxFcnGenRoe.h:183-213).
void orc_flux_batch(const m2cg_config* cfg, int64_t n, const int32_t* dir, const double* Vm, const double* Vp,
                    const int32_t* id, double* F) {
  std::vector<Eos> vf(cfg->n_materials);
  for (int m = 0; m < cfg->n_materials; m++) vf[m].setup(cfg->mat[m]);
  for (int64_t q = 0; q < n; q++) {
    const Eos& e = vf[id[q]];
    if (cfg->flux == M2CG_FLUX_HLLC) FluxHLLC(e, dir[q], &Vm[q * 5], &Vp[q * 5], &F[q * 5]);
    else if (cfg->flux == M2CG_FLUX_LLF) FluxLLF2(e, e, dir[q], &Vm[q * 5], &Vp[q * 5], &F[q * 5]);
    else FluxGenRoe(e, dir[q], &Vm[q * 5], &Vp[q * 5], cfg->roe_delta, &F[q * 5]);
  }
}

}  // extern "C"
