// Device-side equations of state, numerical fluxes and slope limiters for the
// GB300 finite-volume step.  All arithmetic is IEEE binary64.
//
// Reference formulas: VarFcnSG.h:64-68, VarFcnNASG.h:55-59, VarFcnMG.h:70-87,
// VarFcnBase.h:120-298, FluxFcnBase.h:82-123, FluxFcnHLLC.h:51-245,
// FluxFcnLLF.h:46-185, FluxFcnGenRoe.h:63-221, Reconstructor.h:96-111.
#pragma once
#include <cstdint>
#include <cfloat>
#include "../../include/m2cg.h"

#define M2CG_DEV __device__ __forceinline__

namespace m2cg {

// Material constants precomputed on the host (one entry per material ID).
struct DevMat {
  int type;                      // M2CG_EOS_*
  int clip_default;              // rhomin = 0, pmin = -DBL_MAX, rhomax = pmax = DBL_MAX
  double gam, gam1, Pstiff, gamPs, invgam1;   // SG / NASG (Pstiff = pc for NASG)
  double b, q;                                // NASG
  double rho0, s, e0, rho0_c0_c0, G0_half, G0_rho0;  // MG
  double rhomin, pmin, rhomax, pmax;
};

struct Mats {
  DevMat m[M2CG_MAX_MATERIALS];
};

// ---- binary64 building blocks on the integer and FP64 pipes -----------------
// GB300 runs binary64 at 2 FMA/clk/SM; comparisons, min/max and divisions cost
// FP64-pipe slots too.  Sign and range tests on a double's bit pattern run on
// the integer pipe instead (IEEE-754 binary64 orders like a sign-magnitude
// integer).
M2CG_DEV long long bits(double x) { return __double_as_longlong(x); }
M2CG_DEV bool is_finite_bits(double x) { return (bits(x) & 0x7ff0000000000000ll) != 0x7ff0000000000000ll; }
// x <= 0 (both zeros included)
M2CG_DEV bool le_zero_bits(double x) { return bits(x) <= 0; }
// x < 0 (negative zero excluded)
M2CG_DEV bool lt_zero_bits(double x) { long long b = bits(x); return b < 0 && b != (long long)0x8000000000000000ull; }
// |x| < c for a positive constant c
M2CG_DEV bool abs_lt_bits(double x, double c) { return (bits(x) & 0x7fffffffffffffffll) < bits(c); }
M2CG_DEV bool is_pos_inf(double x) { return bits(x) == 0x7ff0000000000000ll; }
M2CG_DEV bool is_neg_inf(double x) { return bits(x) == (long long)0xfff0000000000000ull; }

// Reciprocal and reciprocal square root: the hardware approximations of the
// PTX ISA (rcp.approx.ftz.f64, rsqrt.approx.ftz.f64; about 2^-20 relative
// error) refined by one third-order Householder step,
//   r' = r (1 + e + e^2),            e = 1 - x r
//   y' = y (1 + e/2 + 3 e^2 / 8),    e = 1 - x y^2,
// which leaves at most about one ulp of error (checked on the device against
// correctly rounded 1/x over 1e-20..1e20: max 2.2e-16).  Call sites pass
// finite, positive, normal arguments.
M2CG_DEV double rcp_fast(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  double e = fma(-x, r, 1.0);
  return fma(r, fma(e, e, e), r);
}
M2CG_DEV double rsqrt_fast(double x) {
  double y;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  double e = fma(-x, y * y, 1.0);
  return fma(y * e, fma(e, 0.375, 0.5), y);
}

// Correctly rounded quotients a / b for several numerators over one divisor,
// after P. Markstein, "Computation of elementary functions on the IBM RISC
// System/6000 processor", IBM J. Res. Dev. 34(1), 1990 (theorems restated in
// Muller et al., Handbook of Floating-Point Arithmetic, ch. on division with
// an FMA).  In round-to-nearest binary64 without underflow or overflow:
//   (1) if y1 is within one ulp of 1/b and the significand of b is not all
//       ones, y = y1 + y1 (1 - b y1) (two FMAs) is RN(1/b);
//   (2) if y = RN(1/b) and q is within one ulp of a/b, the remainder
//       a - b q is exact in one FMA and q + (a - b q) y rounds to RN(a/b).
// q0 = RN(a y) can be 1.5 ulp off, so one remainder step brings it within
// half an ulp first: five FP64 operations per quotient against the ~9 of a
// full division, which pays from the second quotient of a divisor on
// (measured on GB300, one dependent chain: 590 cycles for a / b, 321 for the
// five operations, 372 for y).  Operands outside the range where the theorems
// hold -- zero, subnormal, infinite or NaN operands, quotients near the
// exponent limits, divisors with an all-ones significand -- take the IEEE
// division instead, so every result equals a / b bit for bit
// (m2cg_selftest_quotient checks that on random and edge-case operands).
struct Quot {
  double b, y;
  bool fast;
};
M2CG_DEV int exp_field(double x) { return (int)((bits(x) >> 52) & 0x7ff); }
M2CG_DEV Quot quot_of(double b) {
  Quot q;
  q.b = b;
  const int eb = exp_field(b);
  q.fast = (unsigned)(eb - 128) <= 1792u && (bits(b) & 0xfffffffffffffll) != 0xfffffffffffffll;
  q.y = 0.0;
  if (q.fast) {
    const double y1 = rcp_fast(b);
    q.y = fma(fma(-b, y1, 1.0), y1, y1);
  }
  return q;
}
// the IEEE division out of line: one copy of its code however many quotients
// fall back, which keeps the solver's hot loops small in the instruction cache
static __device__ __noinline__ double ieee_div(double a, double b) { return a / b; }
M2CG_DEV double qdiv(double a, const Quot& d) {
  const int ea = exp_field(a), eq = ea - exp_field(d.b) + 1023;
  if (!d.fast || (unsigned)(ea - 128) > 1792u || (unsigned)(eq - 128) > 1792u) return ieee_div(a, d.b);
  double q = __dmul_rn(a, d.y);
  q = fma(fma(-d.b, q, a), d.y, q);
  return fma(fma(-d.b, q, a), d.y, q);
}
// 1 / b from the same divisor: y itself is RN(1/b)
M2CG_DEV double qrcp(const Quot& d) { return d.fast ? d.y : ieee_div(1.0, d.b); }
// The same calls with Shared = false are plain IEEE divisions.  The shared
// reciprocal shortens a dependent chain (a lone solve on an otherwise idle
// FP64 pipe) but issues a few more FP64-pipe slots per divisor than the
// divisions it replaces, so code whose pipe is full (a warp of independent
// solves per lane) keeps the divisions.  Both give the same bits.
template <bool Shared> M2CG_DEV Quot quot_of_t(double b) {
  if constexpr (Shared) return quot_of(b);
  Quot q;
  q.b = b;
  q.y = 0.0;
  q.fast = false;
  return q;
}
template <bool Shared> M2CG_DEV double qdiv_t(double a, const Quot& d) {
  if constexpr (Shared) return qdiv(a, d);
  return a / d.b;
}
template <bool Shared> M2CG_DEV double qrcp_t(const Quot& d) {
  if constexpr (Shared) return qrcp(d);
  return 1.0 / d.b;
}

// ---- equation of state ----------------------------------------------------
M2CG_DEV double eos_p(const DevMat& M, double rho, double e) {
  if (M.type == M2CG_EOS_SG) return M.gam1 * rho * e - M.gamPs;   // gamPs = RN(gamma * pc), the same product
  if (M.type == M2CG_EOS_NASG) return M.gam1 * (e - M.q) / (1.0 / rho - M.b) - M.gamPs;
  double eta = 1.0 - M.rho0 / rho;
  return M.rho0_c0_c0 * eta * (1.0 - M.G0_half * eta) / ((1.0 - M.s * eta) * (1.0 - M.s * eta)) + M.G0_rho0 * (e - M.e0);
}
M2CG_DEV double eos_e(const DevMat& M, double rho, double p) {
  if (M.type == M2CG_EOS_SG) return (p + M.gamPs) / (M.gam1 * rho);
  if (M.type == M2CG_EOS_NASG) return M.invgam1 * (p + M.gamPs) * (1.0 / rho - M.b) + M.q;
  double eta = 1.0 - M.rho0 / rho;
  return (p - M.rho0_c0_c0 * eta * (1.0 - M.G0_half * eta) / ((1.0 - M.s * eta) * (1.0 - M.s * eta))) / M.G0_rho0 + M.e0;
}
M2CG_DEV double eos_dpdrho(const DevMat& M, double rho, double e) {
  if (M.type == M2CG_EOS_SG) return M.gam1 * e;
  if (M.type == M2CG_EOS_NASG) { double V = 1.0 / rho; return M.gam1 * V * V * (e - M.q) / ((V - M.b) * (V - M.b)); }
  double eta = 1.0 - M.rho0 / rho;
  double S = 1.0 - M.s * eta;
  return M.rho0_c0_c0 * (1.0 + (M.s - 2.0 * M.G0_half) * eta) / (S * S * S) * M.rho0 / (rho * rho);
}
M2CG_DEV double eos_Gamma(const DevMat& M, double rho) {
  if (M.type == M2CG_EOS_SG) return M.gam1;
  if (M.type == M2CG_EOS_NASG) return M.gam1 / (1.0 - M.b * rho);
  return M.G0_rho0 / rho;
}
// VarFcnBase.h:219-223
M2CG_DEV double eos_c2(const DevMat& M, double rho, double e) {
  return eos_dpdrho(M, rho, e) + eos_p(M, rho, e) / rho * eos_Gamma(M, rho);
}
// eos_c2 with its division by rho through a reciprocal the caller shares (same bits)
template <bool Shared> M2CG_DEV double eos_c2_q(const DevMat& M, double rho, const Quot& R, double e) {
  return eos_dpdrho(M, rho, e) + qdiv_t<Shared>(eos_p(M, rho, e), R) * eos_Gamma(M, rho);
}
// CheckState: true = nonphysical (VarFcnSG.h:96-108, VarFcnNASG.h:73-85, VarFcnBase.h:120-140)
M2CG_DEV bool eos_bad(const DevMat& M, double rho, double p) {
  if (!isfinite(rho) || !isfinite(p)) return true;
  if (M.type == M2CG_EOS_SG || M.type == M2CG_EOS_NASG) return (rho <= 0.0 || p + M.Pstiff <= 0.0);
  if (rho <= 0.0) return true;
  double e = eos_e(M, rho, p);
  return eos_dpdrho(M, rho, e) + p / rho * eos_Gamma(M, rho) <= 0.0;
}
M2CG_DEV bool eos_bad5(const DevMat& M, const double* V) {
  if (!isfinite(V[1]) || !isfinite(V[2]) || !isfinite(V[3])) return true;
  return eos_bad(M, V[0], V[4]);
}
// VarFcnBase.h:262-298 (returns whether it clipped)
M2CG_DEV bool eos_clip(const DevMat& M, double* V) {
  bool c = false;
  if (V[0] < M.rhomin) { V[0] = M.rhomin; c = true; }
  if (V[4] < M.pmin) { V[4] = M.pmin; c = true; }
  if (V[0] > M.rhomax) { V[0] = M.rhomax; c = true; }
  if (V[4] > M.pmax) { V[4] = M.pmax; c = true; }
  return c;
}
// CheckState and ClipDensityAndPressure with the integer-pipe tests above
// (same results for finite and infinite inputs).
M2CG_DEV bool eos_bad5_fast(const DevMat& M, const double* V) {
  if (!is_finite_bits(V[0]) || !is_finite_bits(V[1]) || !is_finite_bits(V[2]) || !is_finite_bits(V[3]) ||
      !is_finite_bits(V[4]))
    return true;
  if (M.type == M2CG_EOS_SG || M.type == M2CG_EOS_NASG) return le_zero_bits(V[0]) || le_zero_bits(V[4] + M.Pstiff);
  return eos_bad(M, V[0], V[4]);
}
M2CG_DEV bool eos_clip_fast(const DevMat& M, double* V) {
  if (!M.clip_default) return eos_clip(M, V);
  bool c = false;
  if (lt_zero_bits(V[0])) { V[0] = 0.0; c = true; }
  if (is_neg_inf(V[4])) { V[4] = M.pmin; c = true; }
  if (is_pos_inf(V[0])) { V[0] = M.rhomax; c = true; }
  if (is_pos_inf(V[4])) { V[4] = M.pmax; c = true; }
  return c;
}

// VarFcnBase.h:190-201
M2CG_DEV void prim_to_cons(const DevMat& M, const double* V, double* U) {
  U[0] = V[0];
  U[1] = V[0] * V[1]; U[2] = V[0] * V[2]; U[3] = V[0] * V[3];
  double e = eos_e(M, V[0], V[4]);
  U[4] = V[0] * (e + 0.5 * (V[1] * V[1] + V[2] * V[2] + V[3] * V[3]));
}
// Conversions with one reciprocal and no division (SG and NASG closed forms);
// equal to prim_to_cons / cons_to_prim to rounding.
M2CG_DEV void prim_to_cons_fast(const DevMat& M, const double* V, double* U) {
  double k2 = V[1] * V[1] + V[2] * V[2] + V[3] * V[3];
  U[0] = V[0];
  U[1] = V[0] * V[1]; U[2] = V[0] * V[2]; U[3] = V[0] * V[3];
  if (M.type == M2CG_EOS_SG) U[4] = fma(0.5 * V[0], k2, (V[4] + M.gamPs) * M.invgam1);
  else U[4] = V[0] * (eos_e(M, V[0], V[4]) + 0.5 * k2);
}
M2CG_DEV void cons_to_prim_fast(const DevMat& M, const double* U, double* V) {
  V[0] = U[0];
  double ir = rcp_fast(U[0]);
  V[1] = U[1] * ir; V[2] = U[2] * ir; V[3] = U[3] * ir;
  double rhoe = U[4] - 0.5 * V[0] * (V[1] * V[1] + V[2] * V[2] + V[3] * V[3]);
  if (M.type == M2CG_EOS_SG) V[4] = fma(M.gam1, rhoe, -M.gamPs);
  else V[4] = eos_p(M, V[0], rhoe * ir);
}
// VarFcnBase.h:173-186
M2CG_DEV void cons_to_prim(const DevMat& M, const double* U, double* V) {
  V[0] = U[0];
  double invRho = 1.0 / U[0];
  V[1] = U[1] * invRho; V[2] = U[2] * invRho; V[3] = U[3] * invRho;
  double e = (U[4] - 0.5 * V[0] * (V[1] * V[1] + V[2] * V[2] + V[3] * V[3])) * invRho;
  V[4] = eos_p(M, V[0], e);
}
M2CG_DEV double total_enthalpy(const DevMat& M, const double* V) {
  double e = eos_e(M, V[0], V[4]);
  return e + 0.5 * (V[1] * V[1] + V[2] * V[2] + V[3] * V[3]) + V[4] / V[0];
}

// ---- physical flux (FluxFcnBase.h:82-123) ------------------------------------
M2CG_DEV void phys_flux(const DevMat& M, int dir, const double* V, double* F) {
  double H = total_enthalpy(M, V);
  double vn = V[1 + dir];
  double rhou = V[0] * vn;
  F[0] = rhou;
  F[1] = rhou * V[1]; F[2] = rhou * V[2]; F[3] = rhou * V[3];
  F[1 + dir] = rhou * vn + V[4];
  F[4] = rhou * H;
}

M2CG_DEV double avg(double w1, double f1, double w2, double f2) { return (w1 * f1 + w2 * f2) / (w1 + w2); }

// Generalized Roe-averaged state of Hu et al. (FluxFcnHLLC.h:57-126)
struct RoeHat {
  double rho_hat, srm, srp, em, ep, e_hat, c_hat, c2_hat, dpdrho_hat, Gamma_hat, p_over_rho_hat;
};
M2CG_DEV void roe_hat(const DevMat& M, int dir, const double* Vm, const double* Vp, RoeHat& r) {
  const double eps = 1e-10;
  r.rho_hat = sqrt(Vm[0] * Vp[0]);
  r.srm = sqrt(Vm[0]);
  r.srp = sqrt(Vp[0]);
  double drho = Vp[0] - Vm[0];
  double dp = Vp[4] - Vm[4];
  double diff = (Vp[1 + dir] - Vm[1 + dir]) / (r.srm + r.srp);
  r.p_over_rho_hat = avg(r.srm, Vm[4] / Vm[0], r.srp, Vp[4] / Vp[0]) + 0.5 * diff * diff;
  r.em = eos_e(M, Vm[0], Vm[4]);
  r.ep = eos_e(M, Vp[0], Vp[4]);
  double de = r.ep - r.em;
  r.e_hat = avg(r.srm, r.em, r.srp, r.ep);
  double w_rho = drho * drho / (r.rho_hat * r.rho_hat);
  double w_e = de * de / (r.e_hat * r.e_hat);
  double denom = w_rho + w_e + eps;
  double dpdrho_avg = avg(r.srm, eos_dpdrho(M, Vm[0], r.em), r.srp, eos_dpdrho(M, Vp[0], r.ep));
  double Gamma_avg = avg(r.srm, eos_Gamma(M, Vm[0]), r.srp, eos_Gamma(M, Vp[0]));
  double t1 = (w_e + eps) * dpdrho_avg;
  double t2 = (dp - Gamma_avg * r.rho_hat * de) * drho / (r.rho_hat * r.rho_hat);
  r.dpdrho_hat = (t1 + t2) / denom;
  double g1 = (w_rho + eps) * Gamma_avg;
  double g2 = (dp - dpdrho_avg * drho) * de / (r.rho_hat * r.e_hat * r.e_hat);
  r.Gamma_hat = (g1 + g2) / denom;
  r.c2_hat = r.dpdrho_hat + r.Gamma_hat * r.p_over_rho_hat;
  if (r.c2_hat <= 0) { r.c_hat = eps; r.c2_hat = eps * eps; }
  else r.c_hat = sqrt(r.c2_hat);
}

// FluxFcnHLLC.h:158-192
M2CG_DEV void hllc_fstar(const DevMat& M, int dir, const double* V, double S, double Sstar, double* F) {
  double velo = V[1 + dir];
  double rhostar = V[0] * (S - velo) / (S - Sstar);
  double U[5];
  prim_to_cons(M, V, U);
  double Us[5];
  Us[0] = 1.0; Us[1] = V[1]; Us[2] = V[2]; Us[3] = V[3];
  Us[1 + dir] = Sstar;
  Us[4] = U[4] / V[0] + (Sstar - velo) * (Sstar + V[4] / (V[0] * (S - velo)));
  phys_flux(M, dir, V, F);
#pragma unroll
  for (int i = 0; i < 5; i++) F[i] += S * (Us[i] * rhostar - U[i]);
}

// FluxFcnHLLC.h:196-245.  Returns false if c^2 < 0 on either side.
M2CG_DEV bool flux_hllc(const DevMat& M, int dir, const double* Vm, const double* Vp, double* F) {
  RoeHat r;
  roe_hat(M, dir, Vm, Vp, r);
  double cm = eos_c2(M, Vm[0], r.em);
  double cp = eos_c2(M, Vp[0], r.ep);
  bool ok = !(cm < 0.0) && !(cp < 0.0);
  cm = sqrt(fmax(cm, 0.0));
  cp = sqrt(fmax(cp, 0.0));
  double vm = Vm[1 + dir], vp = Vp[1 + dir];
  double vh = avg(r.srm, vm, r.srp, vp);
  double Sm = fmin(vm - cm, vh - r.c_hat);
  double Sp = fmax(vp + cp, vh + r.c_hat);
  if (0.0 <= Sm) phys_flux(M, dir, Vm, F);
  else if (0.0 >= Sp) phys_flux(M, dir, Vp, F);
  else {
    double Sstar = (Vp[4] - Vm[4] + Vm[0] * vm * (Sm - vm) - Vp[0] * vp * (Sp - vp)) /
                   (Vm[0] * (Sm - vm) - Vp[0] * (Sp - vp));
    if (Sstar >= 0.0) hllc_fstar(M, dir, Vm, Sm, Sstar, F);
    else hllc_fstar(M, dir, Vp, Sp, Sstar, F);
  }
  return ok;
}

// ---- HLLC with shared reciprocals ------------------------------------------
// The same flux as flux_hllc (FluxFcnHLLC.h:57-245) with every division of the
// reference rewritten as a product with a reciprocal that is computed once:
// 1/rho and sqrt(rho) come from one rsqrt per side, the Roe-average weight
// 1/(sqrt(rho_m)+sqrt(rho_p)) is shared by all five averages, and the star-state
// algebra uses three more reciprocals.  Results agree with the reference order
// to a few ulps.
struct Side {
  double rho, vn, p, inv_rho, sr, e, dpdrho, Gamma, c2, c;
};
M2CG_DEV void side_eos(const DevMat& M, const double* V, int dir, Side& S) {
  S.rho = V[0];
  S.vn = V[1 + dir];
  S.p = V[4];
  double y = rsqrt_fast(S.rho);
  S.sr = S.rho * y;
  S.inv_rho = y * y;
  if (M.type == M2CG_EOS_SG) {
    // c^2 = dp/drho + p/rho Gamma = gamma (p + p_inf) / rho (VarFcnSG.h:64-68,
    // VarFcnBase.h:219-223), the same value to rounding without the
    // cancellation of the two terms near p = -p_inf
    S.e = (S.p + M.gamPs) * M.invgam1 * S.inv_rho;
    S.dpdrho = M.gam1 * S.e;
    S.Gamma = M.gam1;
    S.c2 = M.gam * (S.p + M.Pstiff) * S.inv_rho;
    S.c = (S.c2 > 0.0) ? S.c2 * rsqrt_fast(S.c2) : 0.0;
    return;
  } else if (M.type == M2CG_EOS_NASG) {
    double vb = S.inv_rho - M.b;
    S.e = M.invgam1 * (S.p + M.gamPs) * vb + M.q;
    double r = S.inv_rho * rcp_fast(vb);
    S.dpdrho = M.gam1 * (S.e - M.q) * r * r;
    S.Gamma = M.gam1 * rcp_fast(1.0 - M.b * S.rho);
  } else {
    S.e = eos_e(M, S.rho, S.p);
    S.dpdrho = eos_dpdrho(M, S.rho, S.e);
    S.Gamma = eos_Gamma(M, S.rho);
  }
  S.c2 = S.dpdrho + S.p * S.inv_rho * S.Gamma;
  S.c = (S.c2 > 0.0) ? S.c2 * rsqrt_fast(S.c2) : 0.0;
}
M2CG_DEV void phys_flux_side(int dir, const double* V, const Side& S, double* F) {
  double k2 = V[1] * V[1] + V[2] * V[2] + V[3] * V[3];
  double H = S.e + 0.5 * k2 + S.p * S.inv_rho;
  double m = S.rho * S.vn;
  F[0] = m;
  F[1] = m * V[1]; F[2] = m * V[2]; F[3] = m * V[3];
  F[1 + dir] = fma(m, S.vn, S.p);
  F[4] = m * H;
}
M2CG_DEV void hllc_fstar_side(int dir, const double* V, const Side& S, double Sw, double Sstar, double* F) {
  double t = Sw - S.vn;
  double rhostar = S.rho * t * rcp_fast(Sw - Sstar);
  double k2 = V[1] * V[1] + V[2] * V[2] + V[3] * V[3];
  double Eo = S.e + 0.5 * k2;   // U[4] / rho
  double U[5] = {S.rho, S.rho * V[1], S.rho * V[2], S.rho * V[3], S.rho * Eo};
  double Us[5] = {1.0, V[1], V[2], V[3], Eo + (Sstar - S.vn) * (Sstar + S.p * S.inv_rho * rcp_fast(t))};
  Us[1 + dir] = Sstar;
  phys_flux_side(dir, V, S, F);
#pragma unroll
  for (int i = 0; i < 5; i++) F[i] = fma(Sw, fma(Us[i], rhostar, -U[i]), F[i]);
}
M2CG_DEV bool flux_hllc_fast(const DevMat& M, int dir, const double* Vm, const double* Vp, double* F) {
  const double eps = 1e-10;
  Side A, B;
  side_eos(M, Vm, dir, A);
  side_eos(M, Vp, dir, B);
  double inv_s = rcp_fast(A.sr + B.sr);
  double rho_hat = A.sr * B.sr;
  double irr = A.inv_rho * B.inv_rho;          // 1 / rho_hat^2
  double drho = B.rho - A.rho;
  double dp = B.p - A.p;
  double diff = (B.vn - A.vn) * inv_s;
  double p_over_rho_hat = (A.sr * (A.p * A.inv_rho) + B.sr * (B.p * B.inv_rho)) * inv_s + 0.5 * diff * diff;
  double e_hat = (A.sr * A.e + B.sr * B.e) * inv_s;
  double c2_hat;
  if (M.type == M2CG_EOS_SG) {
    // Stiffened gas: p is linear in rho e with the constant Gamma = gamma - 1,
    // and the Roe-averaged jumps satisfy d(rho e) = rho_hat de + e_hat drho
    // exactly, so the generalized averages of FluxFcnHLLC.h:99-119 reduce to
    // Gamma_hat = gamma - 1 and dp/drho_hat = (gamma - 1) e_hat: the same value
    // without the weights w_rho, w_e and two reciprocals (the reference's form
    // carries its rounding through a cancellation when dp ~ Gamma rho_hat de).
    c2_hat = M.gam1 * (e_hat + p_over_rho_hat);
  } else {
    double de = B.e - A.e;
    double inv_e = rcp_fast(e_hat);
    double w_rho = drho * drho * irr;
    double de_e = de * inv_e;
    double w_e = de_e * de_e;
    double inv_den = rcp_fast(w_rho + w_e + eps);
    double dpdrho_avg = (A.sr * A.dpdrho + B.sr * B.dpdrho) * inv_s;
    double Gamma_avg = (A.sr * A.Gamma + B.sr * B.Gamma) * inv_s;
    double dpdrho_hat = ((w_e + eps) * dpdrho_avg + (dp - Gamma_avg * rho_hat * de) * drho * irr) * inv_den;
    double Gamma_hat = ((w_rho + eps) * Gamma_avg + (dp - dpdrho_avg * drho) * de_e * inv_e * (A.inv_rho * B.sr * B.inv_rho * A.sr)) * inv_den;
    c2_hat = dpdrho_hat + Gamma_hat * p_over_rho_hat;
  }
  double c_hat = (c2_hat <= 0.0) ? eps : c2_hat * rsqrt_fast(c2_hat);
  double vh = (A.sr * A.vn + B.sr * B.vn) * inv_s;
  double Sm = fmin(A.vn - A.c, vh - c_hat);
  double Sp = fmax(B.vn + B.c, vh + c_hat);
  bool ok = !(A.c2 < 0.0) && !(B.c2 < 0.0);
  // FluxFcnHLLC.h:226-241: F_L, F_R, F*_L or F*_R.  The side is selected
  // first and its flux evaluated once, so lanes of a warp whose faces pick
  // different sides do not run both branches (the same operations as
  // phys_flux_side / hllc_fstar_side on the chosen side).
  const bool sup_l = 0.0 <= Sm, sup_r = 0.0 >= Sp;
  const double am = A.rho * (Sm - A.vn), bp = B.rho * (Sp - B.vn);
  const double Sstar = (dp + am * A.vn - bp * B.vn) * rcp_fast(am - bp);
  const bool left = sup_l || (!sup_r && Sstar >= 0.0);
  // value selects (no pointer to either side, which would put them in memory)
  Side K;
  K.rho = left ? A.rho : B.rho;
  K.vn = left ? A.vn : B.vn;
  K.p = left ? A.p : B.p;
  K.inv_rho = left ? A.inv_rho : B.inv_rho;
  K.e = left ? A.e : B.e;
  double V[5];
#pragma unroll
  for (int i = 0; i < 5; i++) V[i] = left ? Vm[i] : Vp[i];
  phys_flux_side(dir, V, K, F);
  if (!sup_l && !sup_r) {
    const double Sw = left ? Sm : Sp;
    double t = Sw - K.vn;
    double rhostar = K.rho * t * rcp_fast(Sw - Sstar);
    double k2 = V[1] * V[1] + V[2] * V[2] + V[3] * V[3];
    double Eo = K.e + 0.5 * k2;   // U[4] / rho
    double U[5] = {K.rho, K.rho * V[1], K.rho * V[2], K.rho * V[3], K.rho * Eo};
    double Us[5] = {1.0, V[1], V[2], V[3], Eo + (Sstar - K.vn) * (Sstar + K.p * K.inv_rho * rcp_fast(t))};
    Us[1 + dir] = Sstar;
#pragma unroll
    for (int i = 0; i < 5; i++) F[i] = fma(Sw, fma(Us[i], rhostar, -U[i]), F[i]);
  }
  return ok;
}

// FluxFcnLLF.h:46-111 and 118-185 (two materials)
M2CG_DEV bool flux_llf2(const DevMat& Mm, const DevMat& Mp, int dir, const double* Vm, const double* Vp, double* F) {
  double em = eos_e(Mm, Vm[0], Vm[4]);
  double ep = eos_e(Mp, Vp[0], Vp[4]);
  double cm = eos_c2(Mm, Vm[0], em);
  double cp = eos_c2(Mp, Vp[0], ep);
  bool ok = !(cm < 0.0) && !(cp < 0.0);
  cm = sqrt(fmax(cm, 0.0));
  cp = sqrt(fmax(cp, 0.0));
  double a = fmax(fabs(Vm[1 + dir]) + cm, fabs(Vp[1 + dir]) + cp);
  double fm[5], fp[5], Um[5], Up[5];
  phys_flux(Mm, dir, Vm, fm);
  phys_flux(Mp, dir, Vp, fp);
  prim_to_cons(Mm, Vm, Um);
  prim_to_cons(Mp, Vp, Up);
#pragma unroll
  for (int i = 0; i < 5; i++) F[i] = 0.5 * ((fm[i] + fp[i]) - a * (Up[i] - Um[i]));
  return ok;
}

// FluxFcnGenRoe.h:63-221 with the eigenvectors of FluxFcnBase.h:154-176 (F),
// 203-225 (G), 252-274 (H).
M2CG_DEV bool flux_genroe(const DevMat& M, int dir, const double* Vm, const double* Vp, double del, double* F) {
  double srm = sqrt(Vm[0]), srp = sqrt(Vp[0]);
  double rho_hat = sqrt(Vm[0] * Vp[0]);
  double vel[3];
#pragma unroll
  for (int m = 0; m < 3; m++) vel[m] = avg(srm, Vm[1 + m], srp, Vp[1 + m]);
  double H_hat = avg(srm, total_enthalpy(M, Vm), srp, total_enthalpy(M, Vp));
  double dvel[3] = {Vp[1] - Vm[1], Vp[2] - Vm[2], Vp[3] - Vm[3]};
  double dp = Vp[4] - Vm[4], drho = Vp[0] - Vm[0];
  RoeHat r;
  roe_hat(M, dir, Vm, Vp, r);
  double c = r.c_hat, c2 = r.c2_hat;
  double vn = vel[dir];
  double vel2 = vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2];
  double e_term = r.e_hat + 0.5 * vel2 - r.dpdrho_hat / r.Gamma_hat;
  double lam[5] = {vn - c, vn, vn, vn, vn + c};
  double a[5];
  a[0] = (dp - rho_hat * c * dvel[dir]) / (2 * c2);
  a[4] = (dp + rho_hat * c * dvel[dir]) / (2 * c2);
#pragma unroll
  for (int p = 1; p <= 3; p++) a[p] = (p - 1 == dir) ? (-dp / c2 + drho) : rho_hat * dvel[p - 1];
  double tol = lam[0];
#pragma unroll
  for (int i = 1; i < 5; i++) if (fabs(lam[i]) > tol) tol = fabs(lam[i]);
  tol *= del;
#pragma unroll
  for (int i = 0; i < 5; i++) if (fabs(lam[i]) < tol) lam[i] = (lam[i] * lam[i] + tol * tol) / (2 * tol);
  double fm[5], fp[5];
  phys_flux(M, dir, Vm, fm);
  phys_flux(M, dir, Vp, fp);
#pragma unroll
  for (int i = 0; i < 5; i++) F[i] = 0.5 * (fm[i] + fp[i]);
  // subtract 0.5|lam_p| a_p r_p in the order p = 0..4 for every component
#pragma unroll
  for (int p = 0; p < 5; p++) {
    double coef = 0.5 * fabs(lam[p]) * a[p];
    double R[5] = {0, 0, 0, 0, 0};
    if (p == 0 || p == 4) {
      R[0] = 1; R[1] = vel[0]; R[2] = vel[1]; R[3] = vel[2];
      R[1 + dir] = (p == 0) ? vn - c : vn + c;
      R[4] = (p == 0) ? H_hat - vn * c : H_hat + vn * c;
    } else if (p - 1 == dir) {
      R[0] = 1; R[1] = vel[0]; R[2] = vel[1]; R[3] = vel[2]; R[4] = e_term;
    } else {
      R[p] = 1; R[4] = vel[p - 1];
    }
#pragma unroll
    for (int i = 0; i < 5; i++) F[i] -= coef * R[i];
  }
  return true;
}

// ---- slope limiters (Reconstructor.h:96-111) ------------------------------------
M2CG_DEV double gen_minmod(double alpha, double dq0, double dq1) {
  // uniform mesh: A = B = 1, so B/(A+1) = 0.5
  if (dq0 < 0.0 && dq1 < 0.0) return fmax(alpha * dq0, fmax(0.5 * (dq0 + dq1), alpha * dq1));
  if (dq0 > 0.0 && dq1 > 0.0) return fmin(alpha * dq0, fmin(0.5 * (dq0 + dq1), alpha * dq1));
  return 0.0;
}
// van Albada with the sign / magnitude tests on the integer pipe and one
// reciprocal (same value as van_albada to an ulp).  a = dq0^2 and b = dq1^2
// come in precomputed (a difference shared by two neighbouring cells is squared
// once); every operation is pinned (no contraction), so the split and fused
// stage kernels produce the same bits.
M2CG_DEV double van_albada_sq(double dq0, double dq1, double a, double b) {
  double pr = __dmul_rn(dq0, dq1);
  if (le_zero_bits(pr) || abs_lt_bits(pr, 1e-16)) return 0.0;
  return __dmul_rn(fma(dq1, a, __dmul_rn(dq0, b)), rcp_fast(__dadd_rn(a, b)));
}
M2CG_DEV double van_albada_fast(double dq0, double dq1) {
  return van_albada_sq(dq0, dq1, __dmul_rn(dq0, dq0), __dmul_rn(dq1, dq1));
}
// k = 2 on a uniform mesh (Reconstructor.cpp:103-121 with A = B = 1)
M2CG_DEV double van_albada(double dq0, double dq1) {
  double pr = dq0 * dq1;
  if (pr <= 0.0) return 0.0;
  if (fabs(pr) < 1e-16) return 0.0;
  double a = dq0 * dq0, b = dq1 * dq1;
  return (dq1 * a + dq0 * b) / (a + b);
}

}  // namespace m2cg
