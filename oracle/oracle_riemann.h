// ORACLE -- test infrastructure only.  CPU restatement of the reference's
// two-material exact Riemann solver (ExactRiemannSolverBase.cpp), adaptive
// Runge-Kutta rarefaction path with its integration-path cache, and the
// secant/bisection Hugoniot root (the reference's WITHOUT_BOOST branch,
// ExactRiemannSolverBase.cpp:1545-1587).  Nothing in the product links it.
#pragma once
#include <vector>
#include <array>
#include "oracle_eos_flux.h"

namespace orc {

struct RiemannParams {
  int maxIts_main = 200, maxIts_bracket = 100, maxIts_shock = 200, numSteps_rarefaction = 200;
  double tol_main = 1e-5, tol_shock = 1e-12, tol_rarefaction = 1e-8;
  double min_pressure = -1e8, failure_threshold = 0.2, pressure_at_failure = 1e-8;
  double warm_delta = 1e-5;  // learned warm start (not in the reference)
  int warm_tries = 3;
  double warm_gate = 0.05;
};

class ExactRiemann {
 public:
  ExactRiemann(const std::vector<Eos>& vf, const RiemannParams& prm) : vf_(vf), P(prm) {
    path1_.reserve(600); path3_.reserve(600);
  }
  // Number of wave-pair evaluations (bracketing + main loop) in the last solve.
  int evals = 0;
  int main_iters = 0;
  // Optional warm start (the learned warm start; the reference path passes 0):
  // when > 0 on a problem whose acoustic pressure jump exceeds P.warm_gate
  // times the mean pressure, the starting pair is warm_p (1 -+ P.warm_delta) instead of the
  // acoustic-theory pair; if that pair is not physical, or P.warm_tries secant
  // expansions do not bracket the root, the solve restarts cold (SolveOnce
  // returns 3 to Solve).
  double warm_p = 0.0;
  bool warm_used = false;
  bool warm_miss = false;
  // true while running as ExactRiemannSolverNonAdaptive (fixed-step RK4
  // rarefactions, ExactRiemannSolverBase.cpp:2243-2990)
  bool nonadaptive = false;
  int fallbacks = 0;

  // ExactRiemannSolverBase.cpp:59-347 including the retries with the
  // non-adaptive solver after a failure (lines 178-193 and 323-337).
  int Solve(const double* dir, const double* Vm, int idl, const double* Vp, int idr,
            double* Vs, int& id, double* Vsm, double* Vsp) {
    nonadaptive = false;
    fallbacks = 0;
    int e = SolveOnce(dir, Vm, idl, Vp, idr, Vs, id, Vsm, Vsp);
    if (e == 3) {  // the warm start did not bracket the root quickly: cold start
      int ev = evals;
      double w = warm_p;
      warm_p = 0.0;
      e = SolveOnce(dir, Vm, idl, Vp, idr, Vs, id, Vsm, Vsp);
      evals += ev;
      warm_p = w;
    }
    if (e == 1) {
      int ev = evals;
      double w = warm_p;
      warm_p = 0.0;  // the fallback solver starts from acoustic theory
      nonadaptive = true;
      fallbacks = 1;
      e = SolveOnce(dir, Vm, idl, Vp, idr, Vs, id, Vsm, Vsp);
      evals += ev;
      nonadaptive = false;
      warm_p = w;
    }
    return e;
  }

  // One pass of ComputeRiemannSolution (ExactRiemannSolverBase.cpp:59-347, or
  // 2243-2519 when nonadaptive).  Returns 0 on success, 1 on failure.
  int SolveOnce(const double* dir, const double* Vm, int idl, const double* Vp, int idr,
                double* Vs, int& id, double* Vsm, double* Vsp) {
    evals = 0; main_iters = 0;
    double rhol = Vm[0];
    double ul = Vm[1] * dir[0] + Vm[2] * dir[1] + Vm[3] * dir[2];
    double pl = Vm[4];
    double rhor = Vp[0];
    double ur = Vp[1] * dir[0] + Vp[2] * dir[1] + Vp[3] * dir[2];
    double pr = Vp[4];
    path1_.clear(); path3_.clear();
    path1_.push_back({pl, rhol, ul});
    path3_.push_back({pr, rhor, ur});

    double el = vf_[idl].GetInternalEnergyPerUnitMass(rhol, pl);
    double cl = vf_[idl].ComputeSoundSpeedSquare(rhol, el);
    if (rhol <= 0 || cl < 0) return -1;  // reference: exit(-1)
    cl = std::sqrt(cl);
    double er = vf_[idr].GetInternalEnergyPerUnitMass(rhor, pr);
    double cr = vf_[idr].ComputeSoundSpeedSquare(rhor, er);
    if (rhor <= 0 || cr < 0) return -1;
    cr = std::sqrt(cr);

    double p0 = DBL_MIN, ul0 = 0, ur0 = 0, rhol0 = DBL_MIN, rhor0 = DBL_MIN;
    double p1 = DBL_MIN, ul1 = 0, ur1 = 0, rhol1 = DBL_MIN, rhor1 = DBL_MIN;
    double p2 = DBL_MIN, ul2 = 0, ur2 = 0, rhol2 = DBL_MIN, rhor2 = DBL_MIN;
    double f0 = 0, f1 = 0, f2 = 0;
    bool trans_rare = false;
    double Vrare_x0[3] = {0, 0, 0};

    if (ul == ur && pl == pr) {  // :134-139
      Finalize(dir, Vm, Vp, rhol, ul, pl, idl, rhor, ur, pr, idr, rhol, rhor, ul, pl, trans_rare, Vrare_x0, Vs, id, Vsm, Vsp);
      return 0;
    }

    warm_miss = false;
    warm_used = false;
    bool success = FindInitialInterval(rhol, ul, pl, el, cl, idl, rhor, ur, pr, er, cr, idr,
                                       p0, rhol0, rhor0, ul0, ur0, p1, rhol1, rhor1, ul1, ur1);
    if (warm_miss) return 3;
    if (!success) {  // :150-194 (the caller retries with the non-adaptive solver)
      success = RhoUStar(1, path1_, rhol, ul, pl, p1, idl, rhol0, rhol0 * 1.1, rhol2, ul2, &trans_rare, Vrare_x0);
      success = success && RhoUStar(3, path3_, rhor, ur, pr, p1, idr, rhor0, rhol0 * 1.1, rhor2, ur2, &trans_rare, Vrare_x0);
      if (!success) {
        for (int i = 0; i < 5; i++) { Vsm[i] = Vm[i]; Vsp[i] = Vp[i]; }
        double u_avg = 0.5 * (ul + ur);
        if (u_avg >= 0) { id = idl; for (int i = 0; i < 5; i++) Vs[i] = Vm[i]; }
        else { id = idr; for (int i = 0; i < 5; i++) Vs[i] = Vp[i]; }
        return 1;
      }
      Finalize(dir, Vm, Vp, rhol, ul, pl, idl, rhor, ur, pr, idr, rhol2, rhor2, 0.5 * (ul2 + ur2), p1,
               trans_rare, Vrare_x0, Vs, id, Vsm, Vsp);
      return 1;
    }

    f0 = ul0 - ur0;
    f1 = ul1 - ur1;
    double denom = 0;
    int iter = 0;
    double err_p = 1.0, err_u = 1.0;
    p2 = p1;
    f2 = f1;
    for (iter = 0; iter < P.maxIts_main; iter++) {  // :219-311
      denom = f1 - f0;
      if (denom == 0) p2 = p0 + 0.5 * (p1 - p0);
      else {
        p2 = p2 - f2 * (p1 - p0) / denom;
        if (p2 <= p0 || p2 >= p1) p2 = p0 + 0.5 * (p1 - p0);
      }
    try_again:
      evals++;
      success = RhoUStar(1, path1_, rhol, ul, pl, p2, idl, rhol0, rhol1, rhol2, ul2, &trans_rare, Vrare_x0);
      if (!success) {
        p2 = 0.5 * (p2 + p0);
        iter++;
        if (iter < P.maxIts_main) goto try_again;
        else break;
      }
      success = RhoUStar(3, path3_, rhor, ur, pr, p2, idr, rhor0, rhor1, rhor2, ur2, &trans_rare, Vrare_x0);
      if (!success) {
        p2 = 0.5 * (p2 + p1);
        iter++;
        if (iter < P.maxIts_main) goto try_again;
        else break;
      }
      f2 = ul2 - ur2;
      if (f0 * f2 < 0.0) { p1 = p2; f1 = f2; rhol1 = rhol2; rhor1 = rhor2; }
      else { p0 = p2; f0 = f2; rhol0 = rhol2; rhor0 = rhor2; }
      err_p = std::fabs(p1 - p0) / std::max(std::fabs(pl + 0.5 * rhol * ul * ul), std::fabs(pr + 0.5 * rhor * ur * ur));
      err_u = std::fabs(f2) / std::max(cl, cr);
      if ((err_p < P.tol_main && err_u < P.tol_main) || (err_p < P.tol_main * 1e-3) || (err_u < P.tol_main * 1e-3))
        break;
      trans_rare = false;
    }
    main_iters = iter;
    double u2 = 0.5 * (ul2 + ur2);
    Finalize(dir, Vm, Vp, rhol, ul, pl, idl, rhor, ur, pr, idr, rhol2, rhor2, u2, p2, trans_rare, Vrare_x0, Vs, id, Vsm, Vsp);
    if (iter == P.maxIts_main) return 1;  // :323-337 (the caller retries non-adaptively)
    return 0;
  }

 private:
  const std::vector<Eos>& vf_;
  RiemannParams P;
  std::vector<std::array<double, 3>> path1_, path3_;  // {p, rho, u}

  // ExactRiemannSolverBase.cpp:351-558
  void Finalize(const double* dir, const double* Vm, const double* Vp, double rhol, double ul, double pl, int idl,
                double rhor, double ur, double pr, int idr, double rhol2, double rhor2, double u2, double p2,
                bool trans_rare, const double* Vrare_x0, double* Vs, int& id, double* Vsm, double* Vsp) {
    double utanl[3] = {Vm[1] - ul * dir[0], Vm[2] - ul * dir[1], Vm[3] - ul * dir[2]};
    double utanr[3] = {Vp[1] - ur * dir[0], Vp[2] - ur * dir[1], Vp[3] - ur * dir[2]};
    id = (u2 >= 0) ? idl : idr;
    Vs[0] = Vs[1] = Vs[2] = Vs[3] = Vs[4] = 0.0;
    if (trans_rare) {
      Vs[0] = Vrare_x0[0];
      Vs[1] = Vrare_x0[1] * dir[0]; Vs[2] = Vrare_x0[1] * dir[1]; Vs[3] = Vrare_x0[1] * dir[2];
      Vs[4] = Vrare_x0[2];
    } else {
      if (u2 >= 0) {
        bool is_star = false;
        if (pl >= p2) {
          double el2 = vf_[idl].GetInternalEnergyPerUnitMass(rhol2, p2);
          double cl2 = vf_[idl].ComputeSoundSpeedSquare(rhol2, el2);
          cl2 = std::sqrt(std::max(cl2, 0.0));
          if (u2 - cl2 <= 0) is_star = true;
        } else {
          double us = (rhol2 * u2 - rhol * ul) / (rhol2 - rhol);
          if (us <= 0) is_star = true;
        }
        if (is_star) { Vs[0] = rhol2; Vs[1] = u2 * dir[0]; Vs[2] = u2 * dir[1]; Vs[3] = u2 * dir[2]; Vs[4] = p2; }
        else { Vs[0] = rhol; Vs[1] = ul * dir[0]; Vs[2] = ul * dir[1]; Vs[3] = ul * dir[2]; Vs[4] = pl; }
      } else {
        bool is_star = false;
        if (pr >= p2) {
          double er2 = vf_[idr].GetInternalEnergyPerUnitMass(rhor2, p2);
          double cr2 = vf_[idr].ComputeSoundSpeedSquare(rhor2, er2);
          cr2 = std::sqrt(std::max(cr2, 0.0));
          if (u2 - cr2 >= 0) is_star = true;
        } else {
          double us = (rhor2 * u2 - rhor * ur) / (rhor2 - rhor);
          if (us >= 0) is_star = true;
        }
        if (is_star) { Vs[0] = rhor2; Vs[1] = u2 * dir[0]; Vs[2] = u2 * dir[1]; Vs[3] = u2 * dir[2]; Vs[4] = p2; }
        else { Vs[0] = rhor; Vs[1] = ur * dir[0]; Vs[2] = ur * dir[1]; Vs[3] = ur * dir[2]; Vs[4] = pr; }
      }
    }
    if (u2 > 0) { for (int i = 1; i <= 3; i++) Vs[i] += utanl[i - 1]; }
    else if (u2 < 0) { for (int i = 1; i <= 3; i++) Vs[i] += utanr[i - 1]; }
    else { for (int i = 1; i <= 3; i++) Vs[i] += 0.5 * (utanl[i - 1] + utanr[i - 1]); }
    Vsm[0] = rhol2;
    Vsm[1] = utanl[0] + u2 * dir[0]; Vsm[2] = utanl[1] + u2 * dir[1]; Vsm[3] = utanl[2] + u2 * dir[2];
    Vsm[4] = p2;
    Vsp[0] = rhor2;
    Vsp[1] = utanr[0] + u2 * dir[0]; Vsp[2] = utanr[1] + u2 * dir[1]; Vsp[3] = utanr[2] + u2 * dir[2];
    Vsp[4] = p2;
  }

  bool Pair(double p, double rhol, double ul, double pl, int idl, double rhor, double ur, double pr, int idr,
            double gl0, double gl1, double gr0, double gr1, double& rl, double& uL, double& rr, double& uR) {
    evals++;
    bool s = RhoUStar(1, path1_, rhol, ul, pl, p, idl, gl0, gl1, rl, uL, nullptr, nullptr);
    return s && RhoUStar(3, path3_, rhor, ur, pr, p, idr, gr0, gr1, rr, uR, nullptr, nullptr);
  }

  // ExactRiemannSolverBase.cpp:674-839
  bool FindInitialInterval(double rhol, double ul, double pl, double el, double cl, int idl,
                           double rhor, double ur, double pr, double er, double cr, int idr,
                           double& p0, double& rhol0, double& rhor0, double& ul0, double& ur0,
                           double& p1, double& rhol1, double& rhor1, double& ul1, double& ur1) {
    bool success = FindInitialFeasiblePoints(rhol, ul, pl, el, cl, idl, rhor, ur, pr, er, cr, idr,
                                             p0, rhol0, rhor0, ul0, ur0, p1, rhol1, rhor1, ul1, ur1);
    if (!success) { p0 = p1 = P.pressure_at_failure; return false; }
    double p2, rhol2, rhor2, ul2, ur2, f0, f1;
    int i;
    double fmin, p_fmin, rhol_fmin, rhor_fmin, ul_fmin, ur_fmin;
    if (std::fabs(ul0 - ur0) < std::fabs(ul1 - ur1)) {
      fmin = std::fabs(ul0 - ur0); p_fmin = p0; rhol_fmin = rhol0; rhor_fmin = rhor0; ul_fmin = ul0; ur_fmin = ur0;
    } else {
      fmin = std::fabs(ul1 - ur1); p_fmin = p1; rhol_fmin = rhol1; rhor_fmin = rhor1; ul_fmin = ul1; ur_fmin = ur1;
    }
    for (i = 0; i < P.maxIts_bracket; i++) {
      f0 = ul0 - ur0;
      f1 = ul1 - ur1;
      if (f0 * f1 <= 0.0) return true;
      if (warm_used && i >= P.warm_tries) { warm_miss = true; return false; }
      if (std::fabs(f0 - f1) > 1e-9) {
        p2 = p1 - f1 * (p1 - p0) / (f1 - f0);
        if (p2 < p0) p2 -= 0.1 * (p1 - p0);
        else p2 += 0.1 * (p1 - p0);
      } else p2 = 1.1 * p1;
      if (p2 < P.min_pressure || i == int(P.maxIts_bracket / 2)) p2 = 1.0e-8;
      success = Pair(p2, rhol, ul, pl, idl, rhor, ur, pr, idr, rhol0, rhol1, rhor0, rhor1, rhol2, ul2, rhor2, ur2);
      if (!success) {
        for (int j = 0; j < P.maxIts_bracket / 2; j++) {
          if (p2 < p0) p2 = p0 - 0.5 * (p0 - p2);
          else p2 = p1 + 0.5 * (p2 - p1);
          success = Pair(p2, rhol, ul, pl, idl, rhor, ur, pr, idr, rhol0, rhol1, rhor0, rhor1, rhol2, ul2, rhor2, ur2);
          if (success) break;
        }
      }
      if (!success) break;
      if (std::fabs(ul2 - ur2) < fmin) {
        fmin = std::fabs(ul2 - ur2); p_fmin = p2; rhol_fmin = rhol2; rhor_fmin = rhor2; ul_fmin = ul2; ur_fmin = ur2;
      }
      if (p2 < p0) {
        p1 = p0; rhol1 = rhol0; rhor1 = rhor0; ul1 = ul0; ur1 = ur0;
        p0 = p2; rhol0 = rhol2; rhor0 = rhor2; ul0 = ul2; ur0 = ur2;
      } else {
        p0 = p1; rhol0 = rhol1; rhor0 = rhor1; ul0 = ul1; ur0 = ur1;
        p1 = p2; rhol1 = rhol2; rhor1 = rhor2; ul1 = ul2; ur1 = ur2;
      }
    }
    if (!success || i == P.maxIts_bracket) {
      if (fmin < P.failure_threshold * std::fabs(ul - ur)) {
        p0 = p1 = p_fmin; rhol0 = rhol1 = rhol_fmin; rhor0 = rhor1 = rhor_fmin; ul0 = ul1 = ul_fmin; ur0 = ur1 = ur_fmin;
      } else {
        p2 = P.pressure_at_failure;
        success = Pair(p2, rhol, ul, pl, idl, rhor, ur, pr, idr, rhol0, rhol1, rhor0, rhor1, rhol2, ul2, rhor2, ur2);
        if (success) {
          p0 = p1 = p2; rhol0 = rhol1 = rhol2; rhor0 = rhor1 = rhor2; ul0 = ul1 = ul2; ur0 = ur1 = ur2;
        } else {
          p0 = p1 = p_fmin; rhol0 = rhol1 = rhol_fmin; rhor0 = rhor1 = rhor_fmin; ul0 = ul1 = ul_fmin; ur0 = ur1 = ur_fmin;
        }
      }
      return false;
    }
    return true;
  }

  // ExactRiemannSolverBase.cpp:1002-1103
  bool FindInitialFeasiblePoints(double rhol, double ul, double pl, double el, double cl, int idl,
                                 double rhor, double ur, double pr, double er, double cr, int idr,
                                 double& p0, double& rhol0, double& rhor0, double& ul0, double& ur0,
                                 double& p1, double& rhol1, double& rhor1, double& ul1, double& ur1) {
    double dp;
    bool success = true;
    int found = Acoustic(rhol, ul, pl, el, cl, idl, rhor, ur, pr, er, cr, idr, p0, rhol0, rhor0, ul0, ur0, p1, rhol1, rhor1, ul1, ur1);
    if (found == 2) return true;
    if (warm_used) { warm_miss = true; return false; }
    if (found != 1) {
      dp = (pl != pr) ? std::fabs(pl - pr) : 0.5 * pl;
      for (int i = 0; i < P.maxIts_bracket; i++) {
        p0 = std::min(pl, pr) + 0.01 * (i + 1) * (i + 1) * std::min(dp, std::min(std::fabs(pl), std::fabs(pr)));
        if (p0 < P.min_pressure) p0 = P.pressure_at_failure;
        success = Pair(p0, rhol, ul, pl, idl, rhor, ur, pr, idr, rhol, (p0 > pl) ? rhol * 1.1 : rhol * 0.9,
                       rhor, (p0 > pr) ? rhor * 1.1 : rhor * 0.9, rhol0, ul0, rhor0, ur0);
        if (success) break;
      }
      if (!success) {
        for (int i = 0; i < P.maxIts_bracket; i++) {
          p0 = std::min(pl, pr) - 0.01 * (i + 1) * (i + 1) * std::min(dp, std::min(std::fabs(pl), std::fabs(pr)));
          if (p0 < P.min_pressure || i == (int)(P.maxIts_bracket / 2)) p0 = P.pressure_at_failure;
          success = Pair(p0, rhol, ul, pl, idl, rhor, ur, pr, idr, rhol, (p0 > pl) ? rhol * 1.1 : rhol * 0.9,
                         rhor, (p0 > pr) ? rhor * 1.1 : rhor * 0.9, rhol0, ul0, rhor0, ur0);
          if (success) break;
        }
      }
      if (!success) return false;
    }
    dp = std::min(std::fabs(p0 - pl), std::fabs(p0 - pr));
    for (int i = 0; i < P.maxIts_bracket; i++) {
      p1 = p0 + 0.01 * (i + 1) * (i + 1) * dp;
      success = Pair(p1, rhol, ul, pl, idl, rhor, ur, pr, idr, rhol, rhol0, rhor, rhor0, rhol1, ul1, rhor1, ur1);
      if (success) break;
    }
    if (!success) {
      for (int i = 0; i < P.maxIts_bracket; i++) {
        p1 = p0 - 0.01 * (i + 1) * (i + 1) * dp;
        if (p1 < P.min_pressure) p1 = P.pressure_at_failure * 1000.0;
        success = Pair(p1, rhol, ul, pl, idl, rhor, ur, pr, idr, rhol, rhol0, rhor, rhor0, rhol1, ul1, rhor1, ur1);
        if (success) break;
      }
    }
    if (!success) return false;
    if (p0 > p1) {
      std::swap(p0, p1); std::swap(rhol0, rhol1); std::swap(rhor0, rhor1); std::swap(ul0, ul1); std::swap(ur0, ur1);
    }
    return true;
  }

  // ExactRiemannSolverBase.cpp:1107-1158
  int Acoustic(double rhol, double ul, double pl, double /*el*/, double cl, int idl,
               double rhor, double ur, double pr, double /*er*/, double cr, int idr,
               double& p0, double& rhol0, double& rhor0, double& ul0, double& ur0,
               double& p1, double& rhol1, double& rhor1, double& ul1, double& ur1) {
    int found = 0;
    double Cl = rhol * cl, Cr = rhor * cr;
    p0 = (Cr * pl + Cl * pr + Cl * Cr * (ul - ur)) / (Cl + Cr);
    // warm start only where the acoustic pressure jump exceeds warm_gate times
    // the impedance-weighted pressure
    const double pbar = (Cr * pl + Cl * pr) / (Cl + Cr);
    warm_used = warm_p > 0.0 && std::fabs(p0 - pbar) > P.warm_gate * std::fabs(pbar);
    if (warm_used) {
      // learned warm start (not in the reference): the starting pair brackets
      // the prediction, warm_p (1 -+ warm_delta), in place of the acoustic pair
      p0 = warm_p * (1.0 - P.warm_delta);
      p1 = warm_p * (1.0 + P.warm_delta);
      evals++;
      if (!RhoUStar(1, path1_, rhol, ul, pl, p0, idl, rhol, (p0 > pl) ? rhol * 1.1 : rhol * 0.9, rhol0, ul0, nullptr, nullptr)) return found;
      if (!RhoUStar(3, path3_, rhor, ur, pr, p0, idr, rhor, (p0 > pr) ? rhor * 1.1 : rhor * 0.9, rhor0, ur0, nullptr, nullptr)) return found;
      found = 1;
      evals++;
      if (!RhoUStar(1, path1_, rhol, ul, pl, p1, idl, rhol, (p1 > pl) ? rhol * 1.1 : rhol * 0.9, rhol1, ul1, nullptr, nullptr)) return found;
      if (!RhoUStar(3, path3_, rhor, ur, pr, p1, idr, rhor, (p1 > pr) ? rhor * 1.1 : rhor * 0.9, rhor1, ur1, nullptr, nullptr)) return found;
      return 2;
    }
    evals++;
    if (!RhoUStar(1, path1_, rhol, ul, pl, p0, idl, rhol, (p0 > pl) ? rhol * 1.1 : rhol * 0.9, rhol0, ul0, nullptr, nullptr)) return found;
    if (!RhoUStar(3, path3_, rhor, ur, pr, p0, idr, rhor, (p0 > pr) ? rhor * 1.1 : rhor * 0.9, rhor0, ur0, nullptr, nullptr)) return found;
    found = 1;
    double Clbar = (ul0 == ul) ? Cl : std::fabs(p0 - pl) / std::fabs(ul0 - ul);
    double Crbar = (ur0 == ur) ? Cr : std::fabs(p0 - pr) / std::fabs(ur0 - ur);
    p1 = (Crbar * pl + Clbar * pr + Clbar * Crbar * (ul - ur)) / (Clbar + Crbar);
    double tmp = std::max(std::fabs(p0), std::fabs(p1));
    if (std::fabs(p1 - p0) / tmp < 1.0e-8) p1 = p0 + 1.0e-8 * tmp;
    evals++;
    if (!RhoUStar(1, path1_, rhol, ul, pl, p1, idl, rhol, rhol0, rhol1, ul1, nullptr, nullptr)) return found;
    if (!RhoUStar(3, path3_, rhor, ur, pr, p1, idr, rhor, rhor0, rhor1, ur1, nullptr, nullptr)) return found;
    return 2;
  }

  // Hugoniot equation, ExactRiemannSolverBase.h:66-83
  struct Hugo {
    const Eos* vf; double e, pavg, one_over_rho, ps;
    Hugo(const Eos& v, double rho, double p, double ps_) : vf(&v), ps(ps_) {
      e = v.GetInternalEnergyPerUnitMass(rho, p);
      pavg = 0.5 * (p + ps_);
      one_over_rho = 1.0 / rho;
    }
    double operator()(double rhos) const {
      double es = vf->GetInternalEnergyPerUnitMass(rhos, ps);
      return es - e + pavg * (1.0 / rhos - one_over_rho);
    }
  };

  // ExactRiemannSolverBase.cpp:1212-1624
  bool RhoUStar(int wavenumber, std::vector<std::array<double, 3>>& path, double rho, double u, double p, double ps, int id,
                double rhos0, double rhos1, double& rhos, double& us, bool* trans_rare, double* Vrare_x0) {
    const Eos& vf = vf_[id];
    rhos = rho;
    us = u;
    if (p > ps && nonadaptive) return RarefactionFixed(wavenumber, path, rho, u, p, ps, id, rhos, us, trans_rare, Vrare_x0);
    if (p > ps) {  // rarefaction
      double rhos_0 = rho, us_0 = u, ps_0 = p, xi_0;
      double rhos_1 = rho, us_1 = u, ps_1 = p, xi_1 = 0;
      double dp = (p - ps) / P.numSteps_rarefaction;
      double dp_min_adaption = dp / 2.5;
      double pressure_endpoint_tol = P.tol_rarefaction * std::max(1.0, std::fabs(p));
      double e = vf.GetInternalEnergyPerUnitMass(rho, p);
      double c = vf.ComputeSoundSpeedSquare(rho, e);
      if (rho <= 0 || c < 0) return false;
      c = std::sqrt(c);
      int index0 = 0;
      if (path.size() > 1) {
        for (int j = (int)path.size() - 1; j >= 0; j--) {
          if (path[j][0] > ps) { index0 = j; break; }
        }
        ps_0 = path[index0][0];
        rhos_0 = path[index0][1];
        us_0 = path[index0][2];
        dp_min_adaption = (ps_0 - ps) / P.numSteps_rarefaction / 2.5;
        if (index0 != (int)path.size() - 1) dp = ps_0 - ps;
        else dp = std::min(path[index0 - 1][0] - path[index0][0], ps_0 - ps);
      }
      double xi = (wavenumber == 1) ? u - c : u + c;
      xi_0 = xi;
      bool done = false;
      double uErr = 0., rhoErr = 0.;
      int moreSteps = 3;
      for (int i = 0; i < P.numSteps_rarefaction * moreSteps; i++) {
        if (std::fabs(ps_1 - ps) <= pressure_endpoint_tol) {
          rhos = rhos_1;
          us = us_1;
          if (vf.CheckState(rhos, ps)) return false;
          done = true;
          break;
        }
        bool success = RK45(wavenumber, vf, rhos_0, us_0, ps_0, dp, rhos_1, us_1, ps_1, xi_1, uErr, rhoErr);
        if (!success) { dp = dp / 2.0; continue; }
        if (ps_1 - ps < -pressure_endpoint_tol) { dp = ps_0 - ps; continue; }
        double tiny = 1.e-30;
        double errBar = std::max(1.0e-8, std::min(1.0e-5, 100.0 * P.tol_rarefaction));
        double uErrScaled = uErr / c + tiny;
        double rhoErrScaled = rhoErr / rho + tiny;
        if (std::isnan(rhoErrScaled) || std::isnan(uErrScaled)) return false;  // reference: exit(-1)
        double dpTemp = dp;
        double safety = 0.9;
        if (rhoErrScaled >= errBar && dp > dp_min_adaption) {
          dpTemp = safety * dp * std::pow(std::fabs(errBar / rhoErrScaled), 0.25);
          dpTemp = std::max(std::max(dpTemp, 0.2 * dp), dp_min_adaption);
          dp = std::min(dpTemp, ps_0 - ps);
          continue;
        }
        if (uErrScaled >= errBar && dp > dp_min_adaption) {
          dpTemp = safety * dp * std::pow(std::fabs(errBar / uErrScaled), 0.25);
          dpTemp = std::max(std::max(dpTemp, 0.2 * dp), dp_min_adaption);
          dp = std::min(dpTemp, ps_0 - ps);
          continue;
        }
        if (ps_1 < path.back()[0]) path.push_back({ps_1, rhos_1, us_1});
        if (trans_rare && Vrare_x0 && xi_0 * xi_1 <= 0) {
          *trans_rare = true;
          double w0 = std::fabs(xi_1), w1 = std::fabs(xi_0);
          double ww = w0 + w1;
          w0 /= ww;
          w1 /= ww;
          Vrare_x0[0] = w0 * rhos_0 + w1 * rhos_1;
          Vrare_x0[1] = w0 * us_0 + w1 * us_1;
          Vrare_x0[2] = w0 * ps_0 + w1 * ps_1;
        }
        double dpTemp_rho = safety * dp * std::pow(std::fabs(errBar / rhoErrScaled), 0.2);
        double dpTemp_u = safety * dp * std::pow(std::fabs(errBar / uErrScaled), 0.2);
        dpTemp = std::min(dpTemp_rho, dpTemp_u);
        dpTemp = std::min(dpTemp, 10 * dp);
        dpTemp = std::max(dpTemp, dp_min_adaption);
        dp = std::min(dpTemp, ps_1 - ps);
        rhos_0 = rhos_1; us_0 = us_1; ps_0 = ps_1; xi_0 = xi_1;
      }
      if (!done) return false;
    } else {  // shock
      Hugo hugo(vf, rho, p, ps);
      double f0, f1;
      double drho = std::max(std::fabs(rhos0 - rhos1), 0.001 * rhos0);
      bool found_rhos0 = false, found_rhos1 = false;
      if (std::min(rhos0, rhos1) >= rho) {
        f0 = hugo(rhos0);
        f1 = hugo(rhos1);
        if (f0 * f1 <= 0) {
          if (rhos0 > rhos1) { std::swap(rhos0, rhos1); std::swap(f0, f1); }
          found_rhos0 = found_rhos1 = true;
        } else { rhos0 = rhos1; f0 = f1; }
      } else {
        if (rhos1 > rhos0) { rhos0 = rhos1; f0 = hugo(rhos0); }
        if (rhos0 < rho) { rhos0 = rho; f0 = hugo(rhos0); found_rhos0 = true; }
        else f0 = hugo(rhos0);
      }
      if (!found_rhos0 || !found_rhos1) {
        int i = 0;
        double factor = 1.5;
        double tmp, ftmp;
        rhos1 = rhos0;
        f1 = f0;
        while (!found_rhos0) {
          if (++i >= P.maxIts_shock) return false;
          tmp = rhos1; ftmp = f1;
          rhos1 = rhos0; f1 = f0;
          rhos0 = rhos1 - factor * drho;
          if (rhos0 <= rho) { rhos0 = rho; found_rhos0 = true; }
          f0 = hugo(rhos0);
          if (f0 * f1 <= 0) found_rhos0 = found_rhos1 = true;
          else {
            rhos1 = tmp; f1 = ftmp;
            tmp = rhos0; ftmp = f0;
            rhos0 = rhos1; f0 = f1;
            rhos1 = rhos0 + factor * drho;
            f1 = hugo(rhos1);
            if (f0 * f1 <= 0) found_rhos0 = found_rhos1 = true;
            else { rhos0 = tmp; f0 = ftmp; drho = rhos1 - rhos0; }
          }
        }
        if (!found_rhos1) {
          i = 0;
          double factor2 = 2.5;
          while (!found_rhos1) {
            if (++i >= P.maxIts_shock) return false;
            rhos0 = rhos1; f0 = f1;
            rhos1 = rhos0 + factor2 * drho;
            f1 = hugo(rhos1);
            if (f0 * f1 <= 0) found_rhos1 = true;
            else drho = rhos1 - rhos0;
          }
        }
      }
      double loc_tol_shock = P.tol_shock * std::min(rhos0, rhos1);
      double sol_first = 0, sol_second = 0;
      if (f0 == 0.0) sol_first = sol_second = rhos0;
      else if (f1 == 0.0) sol_first = sol_second = rhos1;
      else {
        double rhos2 = rhos1, f2 = f1;
        int it;
        for (it = 0; it < P.maxIts_shock; it++) {
          drho = rhos1 - rhos0;
          rhos2 = rhos2 - f2 * (rhos1 - rhos0) / (f1 - f0);
          if (rhos2 >= rhos1 || rhos2 <= rhos0) rhos2 = rhos0 + 0.5 * (rhos1 - rhos0);
          f2 = hugo(rhos2);
          if (f2 == 0.0) { sol_first = sol_second = rhos2; break; }
          if (f2 * f0 < 0) { rhos1 = rhos2; f1 = f2; }
          else { rhos0 = rhos2; f0 = f2; }
          if (rhos1 - rhos0 < loc_tol_shock) { sol_first = rhos0; sol_second = rhos1; break; }
        }
        if (it == P.maxIts_shock) return false;
      }
      rhos = 0.5 * (sol_first + sol_second);
      double du = -(ps - p) * (1.0 / rhos - 1.0 / rho);
      if (du < 0) return false;
      if (vf.CheckState(rhos, ps)) return false;
      us = (wavenumber == 1) ? u - std::sqrt(du) : u + std::sqrt(du);
    }
    return true;
  }

  // Non-adaptive rarefaction integration, ExactRiemannSolverBase.cpp:2534-2651
  bool RarefactionFixed(int wavenumber, std::vector<std::array<double, 3>>& path, double rho, double u, double p,
                        double ps, int id, double& rhos, double& us, bool* trans_rare, double* Vrare_x0) {
    const Eos& vf = vf_[id];
    double rhos_0 = rho, us_0 = u, ps_0 = p, xi_0;
    double rhos_1 = rho, us_1 = u, ps_1 = p, xi_1 = 0;
    double dp_target = (p - ps) / P.numSteps_rarefaction;
    double e = vf.GetInternalEnergyPerUnitMass(rho, p);
    double dpdrho = vf.GetDpdrho(rho, e);
    double drho_op1 = (p - ps) / dpdrho / P.numSteps_rarefaction;
    double drho_op2 = rho / (2.5 * P.numSteps_rarefaction);
    double drho_target = std::min(drho_op1, drho_op2);
    double dp = std::min(dp_target, drho_target * dpdrho);
    double pressure_endpoint_tol = P.tol_rarefaction * std::max(1.0, std::fabs(p));
    double c = vf.ComputeSoundSpeedSquare(rho, e);
    if (rho <= 0 || c < 0) return false;
    c = std::sqrt(c);
    int index0 = 0;
    if (path.size() > 1) {
      for (int j = (int)path.size() - 1; j >= 0; j--) {
        if (path[j][0] > ps) { index0 = j; break; }
      }
      ps_0 = path[index0][0];
      rhos_0 = path[index0][1];
      us_0 = path[index0][2];
      dp = std::min((p - ps) / P.numSteps_rarefaction, ps_0 - ps);
    }
    double xi = (wavenumber == 1) ? u - c : u + c;
    xi_0 = xi;
    bool done = false;
    for (int i = 0; i < P.numSteps_rarefaction * 5; i++) {
      if (std::fabs(ps_1 - ps) <= pressure_endpoint_tol) {
        rhos = rhos_1;
        us = us_1;
        if (vf.CheckState(rhos, ps)) return false;
        done = true;
        break;
      }
      bool success = RK4(wavenumber, vf, rhos_0, us_0, ps_0, dp, rhos_1, us_1, ps_1, xi_1);
      if (!success) {
        dp = dp / 2.0;
        if (dp == 0.0) break;
        continue;
      }
      if (ps_1 - ps < -pressure_endpoint_tol) { dp = ps_0 - ps; continue; }
      if (ps_1 < path.back()[0]) path.push_back({ps_1, rhos_1, us_1});
      if (trans_rare && Vrare_x0 && xi_0 * xi_1 <= 0) {
        *trans_rare = true;
        double w0 = std::fabs(xi_1), w1 = std::fabs(xi_0);
        double ww = w0 + w1;
        w0 /= ww;
        w1 /= ww;
        Vrare_x0[0] = w0 * rhos_0 + w1 * rhos_1;
        Vrare_x0[1] = w0 * us_0 + w1 * us_1;
        Vrare_x0[2] = w0 * ps_0 + w1 * ps_1;
      }
      dp = std::min(std::min(dp_target, ps_1 - ps), 4.0 * dp);
      rhos_0 = rhos_1; us_0 = us_1; ps_0 = ps_1; xi_0 = xi_1;
    }
    return done;
  }

  // Classical RK4 step, ExactRiemannSolverBase.cpp:2896-2990
  bool RK4(int wavenumber, const Eos& vf, double rho_0, double u_0, double p_0, double dp, double& rho, double& u,
           double& p, double& xi) {
    dp = -dp;
    double e_0 = vf.GetInternalEnergyPerUnitMass(rho_0, p_0);
    double c_0_square = vf.ComputeSoundSpeedSquare(rho_0, e_0);
    if (rho_0 <= 0 || c_0_square < 0) return false;
    double c_0 = std::sqrt(c_0_square);
    double rho_1 = rho_0 + 0.5 * dp / c_0_square;
    double p_1 = p_0 + 0.5 * dp;
    double e_1 = vf.GetInternalEnergyPerUnitMass(rho_1, p_1);
    double c_1_square = vf.ComputeSoundSpeedSquare(rho_1, e_1);
    if (rho_1 <= 0 || c_1_square < 0) return false;
    double c_1 = std::sqrt(c_1_square);
    double rho_2 = rho_0 + 0.5 * dp / c_1_square;
    double p_2 = p_1;
    double e_2 = vf.GetInternalEnergyPerUnitMass(rho_2, p_2);
    double c_2_square = vf.ComputeSoundSpeedSquare(rho_2, e_2);
    if (rho_2 <= 0 || c_2_square < 0) return false;
    double c_2 = std::sqrt(c_2_square);
    double rho_3 = rho_0 + dp / c_2_square;
    double p_3 = p_0 + dp;
    double e_3 = vf.GetInternalEnergyPerUnitMass(rho_3, p_3);
    double c_3_square = vf.ComputeSoundSpeedSquare(rho_3, e_3);
    if (rho_3 <= 0 || c_3_square < 0) return false;
    double c_3 = std::sqrt(c_3_square);
    double drho = 1.0 / 6.0 * dp * (1. / c_0_square + 2.0 * (1. / c_1_square + 1. / c_2_square) + 1. / c_3_square);
    double du = 1.0 / 6.0 * dp * (1. / c_0 / rho_0 + 2.0 * (1. / c_1 / rho_1 + 1. / c_2 / rho_2) + 1. / c_3 / rho_3);
    if (std::isnan(du)) return false;
    rho = rho_0 + drho;
    p = p_0 + dp;
    u = (wavenumber == 1) ? u_0 - du : u_0 + du;
    double e = vf.GetInternalEnergyPerUnitMass(rho, p);
    double c = vf.ComputeSoundSpeedSquare(rho, e);
    if (rho <= 0 || c < 0) return false;
    c = std::sqrt(c);
    xi = (wavenumber == 1) ? u - c : u + c;
    return true;
  }

  // Cash-Karp embedded Runge-Kutta step, ExactRiemannSolverBase.cpp:1771-1896
  bool RK45(int wavenumber, const Eos& vf, double rho_0, double u_0, double p_0, double dp,
            double& rho, double& u, double& p, double& xi, double& uErr, double& rhoErr) {
    dp = -dp;
    double e_0 = vf.GetInternalEnergyPerUnitMass(rho_0, p_0);
    double c_0_square = vf.ComputeSoundSpeedSquare(rho_0, e_0);
    if (rho_0 <= 0 || c_0_square < 0) return false;
    double c_0 = std::sqrt(c_0_square);
    double rho_1 = rho_0 + 0.2 * dp / c_0_square;
    double p_1 = p_0 + 0.2 * dp;
    double e_1 = vf.GetInternalEnergyPerUnitMass(rho_1, p_1);
    double c_1_square = vf.ComputeSoundSpeedSquare(rho_1, e_1);
    if (rho_1 <= 0 || c_1_square < 0) return false;
    double rho_2 = rho_0 + 3. / 40. * dp / c_0_square + 9. / 40. * dp / c_1_square;
    double p_2 = p_1 + 3. / 10. * dp;
    double e_2 = vf.GetInternalEnergyPerUnitMass(rho_2, p_2);
    double c_2_square = vf.ComputeSoundSpeedSquare(rho_2, e_2);
    if (rho_2 <= 0 || c_2_square < 0) return false;
    double c_2 = std::sqrt(c_2_square);
    double rho_3 = rho_0 + 3. / 10. * dp / c_0_square - 9. / 10. * dp / c_1_square + 6. / 5. * dp / c_2_square;
    double p_3 = p_0 + 3. / 5. * dp;
    double e_3 = vf.GetInternalEnergyPerUnitMass(rho_3, p_3);
    double c_3_square = vf.ComputeSoundSpeedSquare(rho_3, e_3);
    if (rho_3 <= 0 || c_3_square < 0) return false;
    double c_3 = std::sqrt(c_3_square);
    double rho_4 = rho_0 - 11. / 54. * dp / c_0_square + 2.5 * dp / c_1_square - 70. / 27. * dp / c_2_square + 35. / 27. * dp / c_3_square;
    double p_4 = p_0 + dp;
    double e_4 = vf.GetInternalEnergyPerUnitMass(rho_4, p_4);
    double c_4_square = vf.ComputeSoundSpeedSquare(rho_4, e_4);
    if (rho_4 <= 0 || c_4_square < 0) return false;
    double c_4 = std::sqrt(c_4_square);
    double rho_5 = rho_0 + 1631. / 55296. * dp / c_0_square + 175. / 512. * dp / c_1_square + 575. / 13824. * dp / c_2_square +
                   44275. / 110592. * dp / c_3_square + 253. / 4096. * dp / c_4_square;
    double p_5 = p_0 + 7. / 8. * dp;
    double e_5 = vf.GetInternalEnergyPerUnitMass(rho_5, p_5);
    double c_5_square = vf.ComputeSoundSpeedSquare(rho_5, e_5);
    if (rho_5 <= 0 || c_5_square < 0) return false;
    double c_5 = std::sqrt(c_5_square);
    double drho = (37. / 378. / c_0_square + 250. / 621. / c_2_square + 125. / 594. / c_3_square + 512. / 1771. / c_5_square) * dp;
    double drho_err = (2825. / 27648. / c_0_square + 18575. / 48384. / c_2_square + 13525. / 55296. / c_3_square +
                       277. / 14336. / c_4_square + 0.25 / c_5_square) * dp;
    double du = (37. / 378. / c_0 / rho_0 + 250. / 621. / c_2 / rho_2 + 125. / 594. / c_3 / rho_3 + 512. / 1771. / c_5 / rho_5) * dp;
    double du_err = (2825. / 27648. / c_0 / rho_0 + 18575. / 48384. / c_2 / rho_2 + 13525. / 55296. / c_3 / rho_3 +
                     277. / 14336. / c_4 / rho_4 + 0.25 / c_5 / rho_5) * dp;
    if (std::isnan(du) || std::isnan(du_err)) return false;
    rhoErr = std::fabs(drho_err - drho);
    uErr = std::fabs(du_err - du);
    rho = rho_0 + drho;
    p = p_0 + dp;
    u = (wavenumber == 1) ? u_0 - du : u_0 + du;
    double e = vf.GetInternalEnergyPerUnitMass(rho, p);
    double c = vf.ComputeSoundSpeedSquare(rho, e);
    if (rho <= 0 || c < 0) return false;
    c = std::sqrt(c);
    xi = (wavenumber == 1) ? u - c : u + c;
    return true;
  }
};

}  // namespace orc
