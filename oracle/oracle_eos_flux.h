// ORACLE -- test infrastructure only.  CPU restatement of M2C's equations of
// state and numerical fluxes, used by the tests, smoke() and the bench's CPU
// baseline leg to check the GPU library.  Nothing in the product links it.
//
// Arithmetic is written in the reference's order of operations and compiled
// with -ffp-contract=off so that it follows the reference's IEEE double
// rounding on any host.
#pragma once
#include <cmath>
#include <cfloat>
#include <algorithm>
#include "../include/m2cg.h"

namespace orc {

// One material's equation of state.  Formulas: VarFcnSG.h:64-68, 96-108;
// VarFcnNASG.h:55-59, 73-85; VarFcnMG.h:70-87; VarFcnBase.h:120-151 (CheckState),
// 173-201 (conversions), 219-223 (c^2), 262-298 (clipping).
struct Eos {
  int type = M2CG_EOS_SG;
  // SG
  double gam = 1.4, Pstiff = 0, gam1 = 0.4;
  // NASG
  double pc = 0, b = 0, q = 0, gam_pc = 0, invgam1 = 0;
  // MG
  double rho0 = 1, c0 = 1, Gamma0 = 1, s = 1, e0 = 0, rho0_c0_c0 = 1, Gamma0_over_2 = 0.5, Gamma0_rho0 = 1;
  // clipping
  double rhomin = 0, pmin = -DBL_MAX, rhomax = DBL_MAX, pmax = DBL_MAX;

  void setup(const m2cg_material& m) {
    type = m.eos;
    rhomin = m.rhomin; pmin = m.pmin; rhomax = m.rhomax; pmax = m.pmax;
    if (type == M2CG_EOS_SG) {            // VarFcnSG.h:128-134
      gam = m.gamma; gam1 = gam - 1.0; Pstiff = m.pc;
    } else if (type == M2CG_EOS_NASG) {   // VarFcnNASG.h:101-111
      gam = m.gamma; pc = m.pc; q = m.q; b = m.b;
      gam1 = gam - 1.0; invgam1 = 1.0 / gam1; gam_pc = gam * pc;
    } else {                              // VarFcnMG.h:104-125
      rho0 = m.rho0; c0 = m.c0; Gamma0 = m.Gamma0; s = m.s; e0 = m.e0;
      rho0_c0_c0 = rho0 * c0 * c0; Gamma0_over_2 = 0.5 * Gamma0; Gamma0_rho0 = Gamma0 * rho0;
    }
  }

  double GetPressure(double rho, double e) const {
    if (type == M2CG_EOS_SG) return gam1 * rho * e - gam * Pstiff;
    if (type == M2CG_EOS_NASG) return gam1 * (e - q) / (1.0 / rho - b) - gam_pc;
    double eta = 1.0 - rho0 / rho;
    return rho0_c0_c0 * eta * (1.0 - Gamma0_over_2 * eta) / ((1.0 - s * eta) * (1.0 - s * eta)) + Gamma0_rho0 * (e - e0);
  }
  double GetInternalEnergyPerUnitMass(double rho, double p) const {
    if (type == M2CG_EOS_SG) return (p + gam * Pstiff) / (gam1 * rho);
    if (type == M2CG_EOS_NASG) return invgam1 * (p + gam_pc) * (1.0 / rho - b) + q;
    double eta = 1.0 - rho0 / rho;
    return (p - rho0_c0_c0 * eta * (1.0 - Gamma0_over_2 * eta) / ((1.0 - s * eta) * (1.0 - s * eta))) / Gamma0_rho0 + e0;
  }
  double GetDpdrho(double rho, double e) const {
    if (type == M2CG_EOS_SG) return gam1 * e;
    if (type == M2CG_EOS_NASG) { double V = 1.0 / rho; return gam1 * V * V * (e - q) / ((V - b) * (V - b)); }
    double eta = 1.0 - rho0 / rho;
    double S = 1.0 - s * eta;
    return rho0_c0_c0 * (1.0 + (s - Gamma0) * eta) / (S * S * S) * rho0 / (rho * rho);
  }
  double GetBigGamma(double rho, double /*e*/) const {
    if (type == M2CG_EOS_SG) return gam1;
    if (type == M2CG_EOS_NASG) return gam1 / (1.0 - b * rho);
    return Gamma0_rho0 / rho;
  }
  // VarFcnBase.h:219-223
  double ComputeSoundSpeedSquare(double rho, double e) const {
    return GetDpdrho(rho, e) + GetPressure(rho, e) / rho * GetBigGamma(rho, e);
  }
  // true = nonphysical.  SG: VarFcnSG.h:96-108; NASG: VarFcnNASG.h:73-85; MG: VarFcnBase.h:120-140
  bool CheckState(double rho, double p) const {
    if (!std::isfinite(rho) || !std::isfinite(p)) return true;
    if (type == M2CG_EOS_SG) return (rho <= 0.0 || p + Pstiff <= 0.0);
    if (type == M2CG_EOS_NASG) return (rho <= 0.0 || p + pc <= 0.0);
    if (rho <= 0.0) return true;
    double e = GetInternalEnergyPerUnitMass(rho, p);
    double c2 = GetDpdrho(rho, e) + p / rho * GetBigGamma(rho, e);
    return c2 <= 0;
  }
  bool CheckState(const double* V) const {   // VarFcnBase.h:143-151
    for (int i = 0; i < 5; i++) if (!std::isfinite(V[i])) return true;
    return CheckState(V[0], V[4]);
  }
  void ConservativeToPrimitive(const double* U, double* V) const {  // VarFcnBase.h:173-186
    V[0] = U[0];
    double invRho = 1.0 / U[0];
    V[1] = U[1] * invRho; V[2] = U[2] * invRho; V[3] = U[3] * invRho;
    double e = (U[4] - 0.5 * V[0] * (V[1] * V[1] + V[2] * V[2] + V[3] * V[3])) * invRho;
    V[4] = GetPressure(V[0], e);
  }
  void PrimitiveToConservative(const double* V, double* U) const {  // VarFcnBase.h:190-201
    U[0] = V[0];
    U[1] = V[0] * V[1]; U[2] = V[0] * V[2]; U[3] = V[0] * V[3];
    double e = GetInternalEnergyPerUnitMass(V[0], V[4]);
    U[4] = V[0] * (e + 0.5 * (V[1] * V[1] + V[2] * V[2] + V[3] * V[3]));
  }
  double ComputeTotalEnthalpyPerUnitMass(const double* V) const {   // VarFcnBase.h:253-258
    double e = GetInternalEnergyPerUnitMass(V[0], V[4]);
    return e + 0.5 * (V[1] * V[1] + V[2] * V[2] + V[3] * V[3]) + V[4] / V[0];
  }
  // VarFcnBase.h:262-298 (U not modified here; callers recompute it).
  bool ClipDensityAndPressure(double* V) const {
    bool clip = false;
    if (V[0] < rhomin) { V[0] = rhomin; clip = true; }
    if (V[4] < pmin) { V[4] = pmin; clip = true; }
    if (V[0] > rhomax) { V[0] = rhomax; clip = true; }
    if (V[4] > pmax) { V[4] = pmax; clip = true; }
    return clip;
  }
};

// Physical flux in direction dir (FluxFcnBase.h:82-123).
inline void EvaluateFlux(const Eos& vf, int dir, const double* V, double* F) {
  double H = vf.ComputeTotalEnthalpyPerUnitMass(V);
  double rhou = V[0] * V[dir + 1];
  F[0] = rhou;
  F[1] = rhou * V[1]; F[2] = rhou * V[2]; F[3] = rhou * V[3];
  F[dir + 1] = rhou * V[dir + 1] + V[4];
  F[4] = rhou * H;
}

inline double Average(double w1, double f1, double w2, double f2) {  // FluxFcnHLLC.h:51-54
  return (w1 * f1 + w2 * f2) / (w1 + w2);
}

// Generalized Roe-averaged sound speed of Hu et al. (FluxFcnHLLC.h:57-126 and
// FluxFcnGenRoe.h:63-136 share this block).
struct RoeHat {
  double rho_hat, sqrt_rhom, sqrt_rhop, em, ep, de, e_hat, c_hat, c_hat_square, dpdrho_hat, Gamma_hat, p_over_rho_hat;
};
inline void ComputeRoeHat(const Eos& vf, int dir, const double* Vm, const double* Vp, double eps, RoeHat& r) {
  r.rho_hat = std::sqrt(Vm[0] * Vp[0]);
  r.sqrt_rhom = std::sqrt(Vm[0]);
  r.sqrt_rhop = std::sqrt(Vp[0]);
  double drho = Vp[0] - Vm[0];
  double dp = Vp[4] - Vm[4];
  double diffvelo = Vp[dir + 1] - Vm[dir + 1];
  double diff = diffvelo / (r.sqrt_rhom + r.sqrt_rhop);
  r.p_over_rho_hat = Average(r.sqrt_rhom, Vm[4] / Vm[0], r.sqrt_rhop, Vp[4] / Vp[0]) + 0.5 * diff * diff;
  r.em = vf.GetInternalEnergyPerUnitMass(Vm[0], Vm[4]);
  r.ep = vf.GetInternalEnergyPerUnitMass(Vp[0], Vp[4]);
  r.de = r.ep - r.em;
  r.e_hat = Average(r.sqrt_rhom, r.em, r.sqrt_rhop, r.ep);
  double w_rho = drho * drho / (r.rho_hat * r.rho_hat);
  double w_e = r.de * r.de / (r.e_hat * r.e_hat);
  double denominator = w_rho + w_e + eps;
  double dpdrho_roeavg = Average(r.sqrt_rhom, vf.GetDpdrho(Vm[0], r.em), r.sqrt_rhop, vf.GetDpdrho(Vp[0], r.ep));
  double Gamma_roeavg = Average(r.sqrt_rhom, vf.GetBigGamma(Vm[0], r.em), r.sqrt_rhop, vf.GetBigGamma(Vp[0], r.ep));
  double t1 = (w_e + eps) * dpdrho_roeavg;
  double t2 = (dp - Gamma_roeavg * r.rho_hat * r.de) * drho / (r.rho_hat * r.rho_hat);
  r.dpdrho_hat = (t1 + t2) / denominator;
  double g1 = (w_rho + eps) * Gamma_roeavg;
  double g2 = (dp - dpdrho_roeavg * drho) * r.de / (r.rho_hat * r.e_hat * r.e_hat);
  r.Gamma_hat = (g1 + g2) / denominator;
  r.c_hat_square = r.dpdrho_hat + r.Gamma_hat * r.p_over_rho_hat;
  if (r.c_hat_square <= 0) { r.c_hat = eps; r.c_hat_square = r.c_hat * r.c_hat; }
  else r.c_hat = std::sqrt(r.c_hat_square);
}

// FluxFcnHLLC.h:158-192
inline void HLLCFstar(const Eos& vf, int dir, const double* V, double S, double Sstar, double* Fstar) {
  double velo = V[dir + 1];
  double rhostar = V[0] * (S - velo) / (S - Sstar);
  double U[5];
  vf.PrimitiveToConservative(V, U);
  double Ustar[5];
  Ustar[0] = 1.0;
  Ustar[1] = (dir == 0) ? Sstar : V[1];
  Ustar[2] = (dir == 1) ? Sstar : V[2];
  Ustar[3] = (dir == 2) ? Sstar : V[3];
  Ustar[4] = U[4] / V[0] + (Sstar - velo) * (Sstar + V[4] / (V[0] * (S - velo)));
  for (int i = 0; i < 5; i++) Ustar[i] *= rhostar;
  EvaluateFlux(vf, dir, V, Fstar);
  for (int i = 0; i < 5; i++) Fstar[i] += S * (Ustar[i] - U[i]);
}

// FluxFcnHLLC.h:57-154 + 196-245.  Returns false when c^2 < 0 (reference: exit).
inline bool FluxHLLC(const Eos& vf, int dir, const double* Vm, const double* Vp, double* flux) {
  const double eps = 1e-10;
  RoeHat r;
  ComputeRoeHat(vf, dir, Vm, Vp, eps, r);
  double cm = vf.ComputeSoundSpeedSquare(Vm[0], r.em);
  double cp = vf.ComputeSoundSpeedSquare(Vp[0], r.ep);
  bool ok = !(cm < 0) && !(cp < 0);
  cm = std::sqrt(std::max(cm, 0.0));
  cp = std::sqrt(std::max(cp, 0.0));
  double vel_hat = Average(r.sqrt_rhom, Vm[dir + 1], r.sqrt_rhop, Vp[dir + 1]);
  double Sm = std::min(Vm[dir + 1] - cm, vel_hat - r.c_hat);
  double Sp = std::max(Vp[dir + 1] + cp, vel_hat + r.c_hat);
  if (0.0 <= Sm) EvaluateFlux(vf, dir, Vm, flux);
  else if (0.0 >= Sp) EvaluateFlux(vf, dir, Vp, flux);
  else {
    double velo_m = Vm[dir + 1], velo_p = Vp[dir + 1];
    double Sstar = (Vp[4] - Vm[4] + Vm[0] * velo_m * (Sm - velo_m) - Vp[0] * velo_p * (Sp - velo_p))
                 / (Vm[0] * (Sm - velo_m) - Vp[0] * (Sp - velo_p));
    if (Sstar >= 0.0) HLLCFstar(vf, dir, Vm, Sm, Sstar, flux);
    else HLLCFstar(vf, dir, Vp, Sp, Sstar, flux);
  }
  return ok;
}

// FluxFcnLLF.h:46-111 (single material) and 118-185 (two materials).
inline bool FluxLLF2(const Eos& vfm, const Eos& vfp, int dir, const double* Vm, const double* Vp, double* flux) {
  double e_m = vfm.GetInternalEnergyPerUnitMass(Vm[0], Vm[4]);
  double e_p = vfp.GetInternalEnergyPerUnitMass(Vp[0], Vp[4]);
  double c_m = vfm.ComputeSoundSpeedSquare(Vm[0], e_m);
  double c_p = vfp.ComputeSoundSpeedSquare(Vp[0], e_p);
  bool ok = !(c_m < 0) && !(c_p < 0);
  c_m = std::sqrt(std::max(c_m, 0.0));
  c_p = std::sqrt(std::max(c_p, 0.0));
  double a = std::max(std::fabs(Vm[dir + 1]) + c_m, std::fabs(Vp[dir + 1]) + c_p);
  double fm[5], fp[5], Um[5], Up[5];
  EvaluateFlux(vfm, dir, Vm, fm);
  EvaluateFlux(vfp, dir, Vp, fp);
  vfm.PrimitiveToConservative(Vm, Um);
  vfp.PrimitiveToConservative(Vp, Up);
  for (int i = 0; i < 5; i++) flux[i] = 0.5 * ((fm[i] + fp[i]) - a * (Up[i] - Um[i]));
  return ok;
}

// FluxFcnGenRoe.h:63-221, with FluxFcnBase.h:154-176 (eigenvectors of F; G and H
// permute the velocity components).
inline bool FluxGenRoe(const Eos& vf, int dir, const double* Vm, const double* Vp, double del, double* flux) {
  const double eps = 1e-10;
  double sqrt_rhom = std::sqrt(Vm[0]), sqrt_rhop = std::sqrt(Vp[0]);
  double rho_hat = std::sqrt(Vm[0] * Vp[0]);
  double u_hat = Average(sqrt_rhom, Vm[1], sqrt_rhop, Vp[1]);
  double v_hat = Average(sqrt_rhom, Vm[2], sqrt_rhop, Vp[2]);
  double w_hat = Average(sqrt_rhom, Vm[3], sqrt_rhop, Vp[3]);
  double Hm = vf.ComputeTotalEnthalpyPerUnitMass(Vm);
  double Hp = vf.ComputeTotalEnthalpyPerUnitMass(Vp);
  double H_hat = Average(sqrt_rhom, Hm, sqrt_rhop, Hp);
  double du = Vp[1] - Vm[1], dv = Vp[2] - Vm[2], dw = Vp[3] - Vm[3], dp = Vp[4] - Vm[4];
  double drho = Vp[0] - Vm[0];
  RoeHat r;
  ComputeRoeHat(vf, dir, Vm, Vp, eps, r);
  double c_hat = r.c_hat, c2 = r.c_hat_square;
  double vel2 = u_hat * u_hat + v_hat * v_hat + w_hat * w_hat;
  double vn = (dir == 0) ? u_hat : (dir == 1) ? v_hat : w_hat;
  double lam[5] = {vn - c_hat, vn, vn, vn, vn + c_hat};
  // eigenvectors r[p][i]
  double R[5][5];
  double e_term = r.e_hat + 0.5 * vel2 - r.dpdrho_hat / r.Gamma_hat;
  double vel[3] = {u_hat, v_hat, w_hat};
  for (int p = 0; p < 5; p++) for (int i = 0; i < 5; i++) R[p][i] = 0.0;
  // r1, r5
  R[0][0] = 1; R[4][0] = 1;
  for (int m = 0; m < 3; m++) { R[0][m + 1] = vel[m]; R[4][m + 1] = vel[m]; }
  R[0][dir + 1] = vn - c_hat; R[4][dir + 1] = vn + c_hat;
  R[0][4] = H_hat - vn * c_hat; R[4][4] = H_hat + vn * c_hat;
  // the three middle eigenvectors: the "density" wave sits at slot dir+1
  // (FluxFcnBase.h:170-174 for F; 219-223 for G; 268-272 for H)
  for (int p = 1; p <= 3; p++) {
    int m = p - 1;  // velocity component associated with this slot
    if (m == dir) {  // entropy wave
      R[p][0] = 1; R[p][1] = u_hat; R[p][2] = v_hat; R[p][3] = w_hat; R[p][4] = e_term;
    } else {         // shear wave in component m
      R[p][m + 1] = 1; R[p][4] = vel[m];
    }
  }
  double dvel[3] = {du, dv, dw};
  double a[5];
  double dvn = dvel[dir];
  a[0] = (dp - rho_hat * c_hat * dvn) / (2 * c2);
  a[4] = (dp + rho_hat * c_hat * dvn) / (2 * c2);
  for (int p = 1; p <= 3; p++) {
    int m = p - 1;
    a[p] = (m == dir) ? (-dp / c2 + drho) : rho_hat * dvel[m];
  }
  double tol = lam[0];
  for (int i = 1; i < 5; i++) if (std::fabs(lam[i]) > tol) tol = std::fabs(lam[i]);
  tol *= del;
  for (int i = 0; i < 5; i++) if (std::fabs(lam[i]) < tol) lam[i] = (lam[i] * lam[i] + tol * tol) / (2 * tol);
  double fm[5], fp[5];
  EvaluateFlux(vf, dir, Vm, fm);
  EvaluateFlux(vf, dir, Vp, fp);
  for (int i = 0; i < 5; i++) {
    flux[i] = 0.5 * (fm[i] + fp[i]);
    for (int p = 0; p < 5; p++) flux[i] -= 0.5 * std::fabs(lam[p]) * a[p] * R[p][i];
  }
  return true;
}

}  // namespace orc
