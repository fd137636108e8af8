// Device exact two-material Riemann solver: the algorithm of
// ExactRiemannSolverBase::ComputeRiemannSolution (ExactRiemannSolverBase.cpp:59-347)
// -- acoustic-theory start, bracketing, safeguarded secant on p*, adaptive
// Cash-Karp rarefaction integration with the per-solve integration-path cache,
// secant/bisection Hugoniot root (the reference's WITHOUT_BOOST branch,
// ExactRiemannSolverBase.cpp:1545-1587) and the xi = 0 sampling.
//
// One thread solves one problem.  Every loop is bounded by the reference's own
// caps (MaxIts, MaxItsBracketing, MaxItsShock, 3 x IntegrationSteps), so a
// solve always ends.  The integration-path cache lives in global scratch:
// `cap` entries of {p, rho, u} per wave, strided by `stride` doubles so that
// the lanes of a warp touch adjacent words.
#pragma once
#include "m2cg_device.cuh"

namespace m2cg {

struct RiemannPrm {
  int maxIts_main, maxIts_bracket, maxIts_shock, numSteps;
  double tol_main, tol_shock, tol_rare, min_pressure, failure_threshold, pressure_at_failure;
  // learned warm start: half-width of the starting pair and the number of
  // secant expansions allowed before a cold restart
  double warm_delta;
  int warm_tries;
  double warm_gate;  // the prediction is used only where the acoustic jump / pressure exceeds this
};

// Status bits returned alongside the reference's error code.
enum { RS_PATH_CAPPED = 1 };

struct PathCache {
  double* base;    // entry e, component c at base[(e * 3 + c) * stride]
  int64_t stride;
  int cap;
  int n;
  int capped;
  M2CG_DEV double get(int e, int c) const { return base[(int64_t)(e * 3 + c) * stride]; }
  M2CG_DEV void put(int e, double p, double rho, double u) {
    base[(int64_t)(e * 3 + 0) * stride] = p;
    base[(int64_t)(e * 3 + 1) * stride] = rho;
    base[(int64_t)(e * 3 + 2) * stride] = u;
  }
  M2CG_DEV void reset(double p, double rho, double u) { n = 1; capped = 0; put(0, p, rho, u); }
  M2CG_DEV void push(double p, double rho, double u) {
    if (n < cap) { put(n, p, rho, u); n++; }
    else capped = 1;
  }
  // Largest entry index whose pressure exceeds ps, or 0 if there is none --
  // what the reference's backward linear scan of the path returns
  // (ExactRiemannSolverBase.cpp:1246-1251, 2567-2572).  Entries are pushed only
  // below the last one, so the pressures strictly decrease and a binary search
  // finds the same index.
  M2CG_DEV int last_above(double ps) const {
    if (!(get(0, 0) > ps)) return 0;
    int lo = 0, hi = n - 1;  // get(lo, 0) > ps
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (get(mid, 0) > ps) lo = mid;
      else hi = mid - 1;
    }
    return lo;
  }
};

// SharedDiv: the Cash-Karp and RK4 steps form each repeated divisor's
// reciprocal once (qdiv), for the latency-bound solves of the finite-volume
// step; false keeps the IEEE divisions (batched independent problems).
template <bool SharedDiv>
struct ExactRiemannDevT {
  const Mats* mats;
  RiemannPrm P;
  PathCache path1, path3;
  int evals;
  // Learned warm start: with warm_p > 0 on a face whose acoustic pressure
  // jump exceeds P.warm_gate times the mean pressure, the starting pair is
  // warm_p (1 -+ P.warm_delta) instead of the acoustic-theory pair; if that
  // pair is not physical or P.warm_tries secant expansions do not bracket the
  // root, solve_once returns 3 and solve restarts cold (the reference's path).
  double warm_p;
  bool warm_used = false;  // this pass started from the prediction
  bool warm_miss = false;
  bool nonadaptive;  // running as the reference's non-adaptive fallback solver
  int fallback;      // 1 if the last solve needed the non-adaptive retry
  // Evaluation budget: with eval_limit > 0 a solve that reaches eval_limit
  // wave-pair evaluations stops and returns 2 ("suspended"); its outputs are
  // then meaningless and the caller solves the problem again without a limit.
  // The evaluations themselves are untouched, so a solve that finishes within
  // the budget returns exactly what an unlimited solve returns.
  int eval_limit = 0;
  bool suspended = false;

  M2CG_DEV bool over_budget() {
    if (eval_limit > 0 && evals >= eval_limit) suspended = true;
    return suspended;
  }

  M2CG_DEV const DevMat& mat(int id) const { return mats->m[id]; }
  // the division policy (shared reciprocals or IEEE divisions, same bits)
  M2CG_DEV static Quot qof(double b) { return quot_of_t<SharedDiv>(b); }
  M2CG_DEV static double qd(double a, const Quot& d) { return qdiv_t<SharedDiv>(a, d); }
  M2CG_DEV static double qr(const Quot& d) { return qrcp_t<SharedDiv>(d); }

  // The sound speed of the state a Runge-Kutta step starts from.  The next
  // step of an integration starts where the last one ended (an accepted step)
  // or where it started (a rejected one), and the same state and material give
  // the same bits, so the step keeps those two evaluations and reuses them:
  // a fixed-step non-adaptive rarefaction runs thousands of RK4 steps in a
  // stalled solve, each of whose first stage is an evaluation already made.
  struct EosMemo {
    const DevMat* M;
    double rho, p, c2, c;
  };
  mutable EosMemo memo_start, memo_end;
  // The states a solve starts from are the same at every evaluation, so their
  // internal energy, sound speed, dp/drho and 1/rho are kept from the first
  // evaluation that needs each of them (keyed on the exact state and material).
  struct SideMemo {
    const DevMat* M;
    double rho, p, e, c2, c, dpdrho, oor;
    unsigned have;   // bits: 1 e, 2 c2, 4 c, 8 dpdrho, 16 oor
  };
  mutable SideMemo side_memo[2];
  M2CG_DEV void memo_clear() const {
    memo_start.M = nullptr;
    memo_end.M = nullptr;
    side_memo[0].M = nullptr;
    side_memo[1].M = nullptr;
  }
  M2CG_DEV SideMemo& side(int wave, const DevMat& M, double rho, double p) const {
    SideMemo& m = side_memo[wave == 1 ? 0 : 1];
    if (!(m.M == &M && __double_as_longlong(m.rho) == __double_as_longlong(rho) &&
          __double_as_longlong(m.p) == __double_as_longlong(p))) {
      m.M = &M;
      m.rho = rho;
      m.p = p;
      m.have = 0;
    }
    return m;
  }
  M2CG_DEV static double side_e(SideMemo& m) {
    if (!(m.have & 1u)) { m.e = eos_e(*m.M, m.rho, m.p); m.have |= 1u; }
    return m.e;
  }
  M2CG_DEV static double side_c2(SideMemo& m) {
    if (!(m.have & 2u)) { m.c2 = eos_c2(*m.M, m.rho, side_e(m)); m.have |= 2u; }
    return m.c2;
  }
  // only after the caller has checked c^2 >= 0
  M2CG_DEV static double side_c(SideMemo& m) {
    if (!(m.have & 4u)) { m.c = sqrt(side_c2(m)); m.have |= 4u; }
    return m.c;
  }
  M2CG_DEV static double side_dpdrho(SideMemo& m) {
    if (!(m.have & 8u)) { m.dpdrho = eos_dpdrho(*m.M, m.rho, side_e(m)); m.have |= 8u; }
    return m.dpdrho;
  }
  M2CG_DEV static double side_oor(SideMemo& m) {
    if (!(m.have & 16u)) { m.oor = 1.0 / m.rho; m.have |= 16u; }
    return m.oor;
  }
  M2CG_DEV static bool memo_hit(const EosMemo& m, const DevMat& M, double rho, double p) {
    return m.M == &M && __double_as_longlong(m.rho) == __double_as_longlong(rho) &&
           __double_as_longlong(m.p) == __double_as_longlong(p);
  }
  // c^2 and c of (rho, p) from a kept evaluation; false if there is none
  M2CG_DEV bool memo_get(const DevMat& M, double rho, double p, double& c2, double& c) const {
    if (memo_hit(memo_end, M, rho, p)) { c2 = memo_end.c2; c = memo_end.c; return true; }
    if (memo_hit(memo_start, M, rho, p)) { c2 = memo_start.c2; c = memo_start.c; return true; }
    return false;
  }

  // Cash-Karp step, ExactRiemannSolverBase.cpp:1771-1896.  The same
  // operations in the same order; a divisor that serves several quotients
  // (c_k^2, c_k, rho_k) takes its correctly rounded reciprocal once and each
  // quotient comes out of qdiv bit-identical to the division.
  __device__ __noinline__ bool rk45(int wave, const DevMat& M, double rho_0, double u_0, double p_0, double dp,
                     double& rho, double& u, double& p, double& xi, double& uErr, double& rhoErr) const {
    dp = -dp;
    const Quot R0 = qof(rho_0);
    double c_0_square, c_0;
    if (!memo_get(M, rho_0, p_0, c_0_square, c_0)) {
      double e_0 = eos_e(M, rho_0, p_0);
      c_0_square = eos_c2_q<SharedDiv>(M, rho_0, R0, e_0);
      if (rho_0 <= 0 || c_0_square < 0) return false;
      c_0 = sqrt(c_0_square);
      memo_start = EosMemo{&M, rho_0, p_0, c_0_square, c_0};
    }
    const Quot C0 = qof(c_0_square);
    double rho_1 = rho_0 + qd(0.2 * dp, C0);
    double p_1 = p_0 + 0.2 * dp;
    double e_1 = eos_e(M, rho_1, p_1);
    double c_1_square = eos_c2(M, rho_1, e_1);
    if (rho_1 <= 0 || c_1_square < 0) return false;
    const Quot C1 = qof(c_1_square);
    double rho_2 = rho_0 + qd(3. / 40. * dp, C0) + qd(9. / 40. * dp, C1);
    double p_2 = p_1 + 3. / 10. * dp;
    double e_2 = eos_e(M, rho_2, p_2);
    const Quot R2 = qof(rho_2);
    double c_2_square = eos_c2_q<SharedDiv>(M, rho_2, R2, e_2);
    if (rho_2 <= 0 || c_2_square < 0) return false;
    double c_2 = sqrt(c_2_square);
    const Quot C2 = qof(c_2_square);
    double rho_3 = rho_0 + qd(3. / 10. * dp, C0) - qd(9. / 10. * dp, C1) + qd(6. / 5. * dp, C2);
    double p_3 = p_0 + 3. / 5. * dp;
    double e_3 = eos_e(M, rho_3, p_3);
    const Quot R3 = qof(rho_3);
    double c_3_square = eos_c2_q<SharedDiv>(M, rho_3, R3, e_3);
    if (rho_3 <= 0 || c_3_square < 0) return false;
    double c_3 = sqrt(c_3_square);
    const Quot C3 = qof(c_3_square);
    double rho_4 = rho_0 - qd(11. / 54. * dp, C0) + qd(2.5 * dp, C1) - qd(70. / 27. * dp, C2) +
                   qd(35. / 27. * dp, C3);
    double p_4 = p_0 + dp;
    double e_4 = eos_e(M, rho_4, p_4);
    const Quot R4 = qof(rho_4);
    double c_4_square = eos_c2_q<SharedDiv>(M, rho_4, R4, e_4);
    if (rho_4 <= 0 || c_4_square < 0) return false;
    double c_4 = sqrt(c_4_square);
    const Quot C4 = qof(c_4_square);
    double rho_5 = rho_0 + qd(1631. / 55296. * dp, C0) + qd(175. / 512. * dp, C1) +
                   qd(575. / 13824. * dp, C2) + qd(44275. / 110592. * dp, C3) + qd(253. / 4096. * dp, C4);
    double p_5 = p_0 + 7. / 8. * dp;
    double e_5 = eos_e(M, rho_5, p_5);
    const Quot R5 = qof(rho_5);
    double c_5_square = eos_c2_q<SharedDiv>(M, rho_5, R5, e_5);
    if (rho_5 <= 0 || c_5_square < 0) return false;
    double c_5 = sqrt(c_5_square);
    const Quot C5 = qof(c_5_square);
    double drho = (qd(37. / 378., C0) + qd(250. / 621., C2) + qd(125. / 594., C3) + qd(512. / 1771., C5)) * dp;
    double drho_err = (qd(2825. / 27648., C0) + qd(18575. / 48384., C2) + qd(13525. / 55296., C3) +
                       qd(277. / 14336., C4) + qd(0.25, C5)) * dp;
    const Quot S0 = qof(c_0), S2 = qof(c_2), S3 = qof(c_3), S5 = qof(c_5);
    double du = (qd(qd(37. / 378., S0), R0) + qd(qd(250. / 621., S2), R2) + qd(qd(125. / 594., S3), R3) +
                 qd(qd(512. / 1771., S5), R5)) * dp;
    double du_err = (qd(qd(2825. / 27648., S0), R0) + qd(qd(18575. / 48384., S2), R2) +
                     qd(qd(13525. / 55296., S3), R3) + qd(277. / 14336. / c_4, R4) + qd(qd(0.25, S5), R5)) * dp;
    if (isnan(du) || isnan(du_err)) return false;
    rhoErr = fabs(drho_err - drho);
    uErr = fabs(du_err - du);
    rho = rho_0 + drho;
    p = p_0 + dp;
    u = (wave == 1) ? u_0 - du : u_0 + du;
    double e = eos_e(M, rho, p);
    double c = eos_c2(M, rho, e);
    if (rho <= 0 || c < 0) return false;
    const double c2 = c;
    c = sqrt(c);
    memo_end = EosMemo{&M, rho, p, c2, c};
    xi = (wave == 1) ? u - c : u + c;
    return true;
  }

  // Classical RK4 step of the non-adaptive solver, ExactRiemannSolverBase.cpp:2896-2990
  // (shared reciprocals as in rk45)
  __device__ __noinline__ bool rk4(int wave, const DevMat& M, double rho_0, double u_0, double p_0, double dp,
                                   double& rho, double& u, double& p, double& xi) const {
    dp = -dp;
    const Quot R0 = qof(rho_0);
    double c_0_square, c_0;
    if (!memo_get(M, rho_0, p_0, c_0_square, c_0)) {
      double e_0 = eos_e(M, rho_0, p_0);
      c_0_square = eos_c2_q<SharedDiv>(M, rho_0, R0, e_0);
      if (rho_0 <= 0 || c_0_square < 0) return false;
      c_0 = sqrt(c_0_square);
      memo_start = EosMemo{&M, rho_0, p_0, c_0_square, c_0};
    }
    const Quot C0 = qof(c_0_square);
    double rho_1 = rho_0 + qd(0.5 * dp, C0);
    double p_1 = p_0 + 0.5 * dp;
    double e_1 = eos_e(M, rho_1, p_1);
    const Quot R1 = qof(rho_1);
    double c_1_square = eos_c2_q<SharedDiv>(M, rho_1, R1, e_1);
    if (rho_1 <= 0 || c_1_square < 0) return false;
    double c_1 = sqrt(c_1_square);
    const Quot C1 = qof(c_1_square);
    double rho_2 = rho_0 + qd(0.5 * dp, C1);
    double p_2 = p_1;
    double e_2 = eos_e(M, rho_2, p_2);
    const Quot R2 = qof(rho_2);
    double c_2_square = eos_c2_q<SharedDiv>(M, rho_2, R2, e_2);
    if (rho_2 <= 0 || c_2_square < 0) return false;
    double c_2 = sqrt(c_2_square);
    const Quot C2 = qof(c_2_square);
    double rho_3 = rho_0 + qd(dp, C2);
    double p_3 = p_0 + dp;
    double e_3 = eos_e(M, rho_3, p_3);
    const Quot R3 = qof(rho_3);
    double c_3_square = eos_c2_q<SharedDiv>(M, rho_3, R3, e_3);
    if (rho_3 <= 0 || c_3_square < 0) return false;
    double c_3 = sqrt(c_3_square);
    double drho = 1.0 / 6.0 * dp * (qr(C0) + 2.0 * (qr(C1) + qr(C2)) + 1. / c_3_square);
    double du = 1.0 / 6.0 * dp *
                (qd(1. / c_0, R0) + 2.0 * (qd(1. / c_1, R1) + qd(1. / c_2, R2)) + qd(1. / c_3, R3));
    if (isnan(du)) return false;
    rho = rho_0 + drho;
    p = p_0 + dp;
    u = (wave == 1) ? u_0 - du : u_0 + du;
    double e = eos_e(M, rho, p);
    double c = eos_c2(M, rho, e);
    if (rho <= 0 || c < 0) return false;
    const double c2 = c;
    c = sqrt(c);
    memo_end = EosMemo{&M, rho, p, c2, c};
    xi = (wave == 1) ? u - c : u + c;
    return true;
  }

  // Fixed-step rarefaction of the non-adaptive solver, ExactRiemannSolverBase.cpp:2534-2651
  __device__ __noinline__ bool rarefaction_fixed(int wave, PathCache& path, const DevMat& M, double rho, double u,
                                                 double p, double ps, double& rhos, double& us, bool* trans_rare,
                                                 double* Vrare) {
    double rhos_0 = rho, us_0 = u, ps_0 = p, xi_0;
    double rhos_1 = rho, us_1 = u, ps_1 = p, xi_1 = 0;
    double dp_target = (p - ps) / P.numSteps;
    SideMemo& sm = side(wave, M, rho, p);
    double dpdrho = side_dpdrho(sm);
    double drho_op1 = (p - ps) / dpdrho / P.numSteps;
    double drho_op2 = rho / (2.5 * P.numSteps);
    double drho_target = fmin(drho_op1, drho_op2);
    double dp = fmin(dp_target, drho_target * dpdrho);
    double tol_end = P.tol_rare * fmax(1.0, fabs(p));
    double c = side_c2(sm);
    if (rho <= 0 || c < 0) return false;
    c = side_c(sm);
    if (path.n > 1) {
      int index0 = path.last_above(ps);
      ps_0 = path.get(index0, 0);
      rhos_0 = path.get(index0, 1);
      us_0 = path.get(index0, 2);
      dp = fmin((p - ps) / P.numSteps, ps_0 - ps);
    }
    xi_0 = (wave == 1) ? u - c : u + c;
    for (int i = 0; i < P.numSteps * 5; i++) {
      if (fabs(ps_1 - ps) <= tol_end) {
        rhos = rhos_1;
        us = us_1;
        return !eos_bad(M, rhos, ps);
      }
      bool ok = rk4(wave, M, rhos_0, us_0, ps_0, dp, rhos_1, us_1, ps_1, xi_1);
      if (!ok) {
        dp = dp / 2.0;
        if (dp == 0.0) break;
        continue;
      }
      if (ps_1 - ps < -tol_end) { dp = ps_0 - ps; continue; }
      if (ps_1 < path.get(path.n - 1, 0)) path.push(ps_1, rhos_1, us_1);
      if (trans_rare && Vrare && xi_0 * xi_1 <= 0) {
        *trans_rare = true;
        double w0 = fabs(xi_1), w1 = fabs(xi_0);
        double ww = w0 + w1;
        w0 /= ww;
        w1 /= ww;
        Vrare[0] = w0 * rhos_0 + w1 * rhos_1;
        Vrare[1] = w0 * us_0 + w1 * us_1;
        Vrare[2] = w0 * ps_0 + w1 * ps_1;
      }
      dp = fmin(fmin(dp_target, ps_1 - ps), 4.0 * dp);
      rhos_0 = rhos_1; us_0 = us_1; ps_0 = ps_1; xi_0 = xi_1;
    }
    return false;
  }

  // Hugoniot residual, ExactRiemannSolverBase.h:66-83
  M2CG_DEV double hugo(const DevMat& M, double e, double pavg, double one_over_rho, double ps, double rhos) const {
    double es = eos_e(M, rhos, ps);
    return es - e + pavg * (1.0 / rhos - one_over_rho);
  }

  // ExactRiemannSolverBase.cpp:1212-1624
  __device__ __noinline__ bool rho_u_star(int wave, PathCache& path, double rho, double u, double p, double ps, int id,
                           double rhos0, double rhos1, double& rhos, double& us, bool* trans_rare, double* Vrare) {
    const DevMat& M = mat(id);
    rhos = rho;
    us = u;
    if (p > ps && nonadaptive) return rarefaction_fixed(wave, path, M, rho, u, p, ps, rhos, us, trans_rare, Vrare);
    if (p > ps) {
      double rhos_0 = rho, us_0 = u, ps_0 = p, xi_0;
      double rhos_1 = rho, us_1 = u, ps_1 = p, xi_1 = 0;
      double dp = (p - ps) / P.numSteps;
      double dp_min = dp / 2.5;
      double tol_end = P.tol_rare * fmax(1.0, fabs(p));
      SideMemo& sm = side(wave, M, rho, p);
      double c = side_c2(sm);
      if (rho <= 0 || c < 0) return false;
      c = side_c(sm);
      int index0 = 0;
      if (path.n > 1) {
        index0 = path.last_above(ps);
        ps_0 = path.get(index0, 0);
        rhos_0 = path.get(index0, 1);
        us_0 = path.get(index0, 2);
        dp_min = (ps_0 - ps) / P.numSteps / 2.5;
        if (index0 != path.n - 1) dp = ps_0 - ps;
        else dp = fmin(path.get(index0 - 1, 0) - path.get(index0, 0), ps_0 - ps);
      }
      double xi = (wave == 1) ? u - c : u + c;
      xi_0 = xi;
      bool done = false;
      double uErr = 0., rhoErr = 0.;
      const double errBar = fmax(1.0e-8, fmin(1.0e-5, 100.0 * P.tol_rare));
      for (int i = 0; i < P.numSteps * 3; i++) {
        if (fabs(ps_1 - ps) <= tol_end) {
          rhos = rhos_1;
          us = us_1;
          if (eos_bad(M, rhos, ps)) return false;
          done = true;
          break;
        }
        bool ok = rk45(wave, M, rhos_0, us_0, ps_0, dp, rhos_1, us_1, ps_1, xi_1, uErr, rhoErr);
        if (!ok) { dp = dp / 2.0; continue; }
        if (ps_1 - ps < -tol_end) { dp = ps_0 - ps; continue; }
        double uS = uErr / c + 1.e-30;
        double rS = rhoErr / rho + 1.e-30;
        if (isnan(rS) || isnan(uS)) return false;
        if (rS >= errBar && dp > dp_min) {
          double t = 0.9 * dp * pow(fabs(errBar / rS), 0.25);
          t = fmax(fmax(t, 0.2 * dp), dp_min);
          dp = fmin(t, ps_0 - ps);
          continue;
        }
        if (uS >= errBar && dp > dp_min) {
          double t = 0.9 * dp * pow(fabs(errBar / uS), 0.25);
          t = fmax(fmax(t, 0.2 * dp), dp_min);
          dp = fmin(t, ps_0 - ps);
          continue;
        }
        if (ps_1 < path.get(path.n - 1, 0)) path.push(ps_1, rhos_1, us_1);
        if (trans_rare && Vrare && xi_0 * xi_1 <= 0) {
          *trans_rare = true;
          double w0 = fabs(xi_1), w1 = fabs(xi_0);
          double ww = w0 + w1;
          w0 /= ww;
          w1 /= ww;
          Vrare[0] = w0 * rhos_0 + w1 * rhos_1;
          Vrare[1] = w0 * us_0 + w1 * us_1;
          Vrare[2] = w0 * ps_0 + w1 * ps_1;
        }
        // the next step size; skipped when the next pass ends the loop and
        // never reads it (the common case of a solve that restarts from the
        // path cache: one step to the end point)
        if (!(fabs(ps_1 - ps) <= tol_end) && i + 1 < P.numSteps * 3) {
          double tr = 0.9 * dp * pow(fabs(errBar / rS), 0.2);
          double tu = 0.9 * dp * pow(fabs(errBar / uS), 0.2);
          double t = fmin(tr, tu);
          t = fmin(t, 10 * dp);
          t = fmax(t, dp_min);
          dp = fmin(t, ps_1 - ps);
        }
        rhos_0 = rhos_1; us_0 = us_1; ps_0 = ps_1; xi_0 = xi_1;
      }
      if (!done) return false;
    } else {
      SideMemo& sm = side(wave, M, rho, p);
      double e = side_e(sm);
      double pavg = 0.5 * (p + ps);
      double oor = side_oor(sm);
      double f0, f1;
      double drho = fmax(fabs(rhos0 - rhos1), 0.001 * rhos0);
      bool found0 = false, found1 = false;
      if (fmin(rhos0, rhos1) >= rho) {
        f0 = hugo(M, e, pavg, oor, ps, rhos0);
        f1 = hugo(M, e, pavg, oor, ps, rhos1);
        if (f0 * f1 <= 0) {
          if (rhos0 > rhos1) { double t = rhos0; rhos0 = rhos1; rhos1 = t; t = f0; f0 = f1; f1 = t; }
          found0 = found1 = true;
        } else { rhos0 = rhos1; f0 = f1; }
      } else {
        if (rhos1 > rhos0) { rhos0 = rhos1; f0 = hugo(M, e, pavg, oor, ps, rhos0); }
        if (rhos0 < rho) { rhos0 = rho; f0 = hugo(M, e, pavg, oor, ps, rhos0); found0 = true; }
        else f0 = hugo(M, e, pavg, oor, ps, rhos0);
      }
      if (!found0 || !found1) {
        int i = 0;
        const double factor = 1.5;
        double tmp, ftmp;
        rhos1 = rhos0;
        f1 = f0;
        while (!found0) {
          if (++i >= P.maxIts_shock) return false;
          tmp = rhos1; ftmp = f1;
          rhos1 = rhos0; f1 = f0;
          rhos0 = rhos1 - factor * drho;
          if (rhos0 <= rho) { rhos0 = rho; found0 = true; }
          f0 = hugo(M, e, pavg, oor, ps, rhos0);
          if (f0 * f1 <= 0) found0 = found1 = true;
          else {
            rhos1 = tmp; f1 = ftmp;
            tmp = rhos0; ftmp = f0;
            rhos0 = rhos1; f0 = f1;
            rhos1 = rhos0 + factor * drho;
            f1 = hugo(M, e, pavg, oor, ps, rhos1);
            if (f0 * f1 <= 0) found0 = found1 = true;
            else { rhos0 = tmp; f0 = ftmp; drho = rhos1 - rhos0; }
          }
        }
        if (!found1) {
          i = 0;
          while (!found1) {
            if (++i >= P.maxIts_shock) return false;
            rhos0 = rhos1; f0 = f1;
            rhos1 = rhos0 + 2.5 * drho;
            f1 = hugo(M, e, pavg, oor, ps, rhos1);
            if (f0 * f1 <= 0) found1 = true;
            else drho = rhos1 - rhos0;
          }
        }
      }
      double loc_tol = P.tol_shock * fmin(rhos0, rhos1);
      double s_first = 0, s_second = 0;
      if (f0 == 0.0) s_first = s_second = rhos0;
      else if (f1 == 0.0) s_first = s_second = rhos1;
      else {
        double rhos2 = rhos1, f2 = f1;
        int it;
        for (it = 0; it < P.maxIts_shock; it++) {
          drho = rhos1 - rhos0;
          rhos2 = rhos2 - f2 * (rhos1 - rhos0) / (f1 - f0);
          if (rhos2 >= rhos1 || rhos2 <= rhos0) rhos2 = rhos0 + 0.5 * (rhos1 - rhos0);
          f2 = hugo(M, e, pavg, oor, ps, rhos2);
          if (f2 == 0.0) { s_first = s_second = rhos2; break; }
          if (f2 * f0 < 0) { rhos1 = rhos2; f1 = f2; }
          else { rhos0 = rhos2; f0 = f2; }
          if (rhos1 - rhos0 < loc_tol) { s_first = rhos0; s_second = rhos1; break; }
        }
        if (it == P.maxIts_shock) return false;
      }
      rhos = 0.5 * (s_first + s_second);
      double du = -(ps - p) * (1.0 / rhos - 1.0 / rho);
      if (du < 0) return false;
      if (eos_bad(M, rhos, ps)) return false;
      us = (wave == 1) ? u - sqrt(du) : u + sqrt(du);
    }
    return true;
  }

  M2CG_DEV bool pair(double p, double rhol, double ul, double pl, int idl, double rhor, double ur, double pr, int idr,
                     double gl0, double gl1, double gr0, double gr1, double& rl, double& uL, double& rr, double& uR) {
    if (over_budget()) return false;
    evals++;
    bool s = rho_u_star(1, path1, rhol, ul, pl, p, idl, gl0, gl1, rl, uL, nullptr, nullptr);
    return s && rho_u_star(3, path3, rhor, ur, pr, p, idr, gr0, gr1, rr, uR, nullptr, nullptr);
  }

  // ExactRiemannSolverBase.cpp:1107-1158
  __device__ __noinline__ int acoustic(double rhol, double ul, double pl, double cl, int idl, double rhor, double ur, double pr,
                        double cr, int idr, double& p0, double& rhol0, double& rhor0, double& ul0, double& ur0,
                        double& p1, double& rhol1, double& rhor1, double& ul1, double& ur1) {
    double Cl = rhol * cl, Cr = rhor * cr;
    p0 = (Cr * pl + Cl * pr + Cl * Cr * (ul - ur)) / (Cl + Cr);
    // the prediction replaces the acoustic estimate only where the acoustic
    // pressure jump exceeds warm_gate times the impedance-weighted pressure:
    // the linearization's error grows like the square of that ratio, and
    // below it acoustic theory is closer than the network
    const double pbar = (Cr * pl + Cl * pr) / (Cl + Cr);
    warm_used = warm_p > 0.0 && fabs(p0 - pbar) > P.warm_gate * fabs(pbar);
    if (warm_used) {
      // learned warm start: the two starting points bracket the prediction,
      // p_hat (1 -+ warm_delta), in place of the acoustic-theory pair; the
      // bracketing and the secant loop that follow are the reference's
      p0 = warm_p * (1.0 - P.warm_delta);
      p1 = warm_p * (1.0 + P.warm_delta);
      evals++;
      if (!rho_u_star(1, path1, rhol, ul, pl, p0, idl, rhol, (p0 > pl) ? rhol * 1.1 : rhol * 0.9, rhol0, ul0, nullptr, nullptr)) return 0;
      if (!rho_u_star(3, path3, rhor, ur, pr, p0, idr, rhor, (p0 > pr) ? rhor * 1.1 : rhor * 0.9, rhor0, ur0, nullptr, nullptr)) return 0;
      evals++;
      if (!rho_u_star(1, path1, rhol, ul, pl, p1, idl, rhol, (p1 > pl) ? rhol * 1.1 : rhol * 0.9, rhol1, ul1, nullptr, nullptr)) return 1;
      if (!rho_u_star(3, path3, rhor, ur, pr, p1, idr, rhor, (p1 > pr) ? rhor * 1.1 : rhor * 0.9, rhor1, ur1, nullptr, nullptr)) return 1;
      return 2;
    }
    evals++;
    if (!rho_u_star(1, path1, rhol, ul, pl, p0, idl, rhol, (p0 > pl) ? rhol * 1.1 : rhol * 0.9, rhol0, ul0, nullptr, nullptr)) return 0;
    if (!rho_u_star(3, path3, rhor, ur, pr, p0, idr, rhor, (p0 > pr) ? rhor * 1.1 : rhor * 0.9, rhor0, ur0, nullptr, nullptr)) return 0;
    double Clbar = (ul0 == ul) ? Cl : fabs(p0 - pl) / fabs(ul0 - ul);
    double Crbar = (ur0 == ur) ? Cr : fabs(p0 - pr) / fabs(ur0 - ur);
    p1 = (Crbar * pl + Clbar * pr + Clbar * Crbar * (ul - ur)) / (Clbar + Crbar);
    double tmp = fmax(fabs(p0), fabs(p1));
    if (fabs(p1 - p0) / tmp < 1.0e-8) p1 = p0 + 1.0e-8 * tmp;
    evals++;
    if (!rho_u_star(1, path1, rhol, ul, pl, p1, idl, rhol, rhol0, rhol1, ul1, nullptr, nullptr)) return 1;
    if (!rho_u_star(3, path3, rhor, ur, pr, p1, idr, rhor, rhor0, rhor1, ur1, nullptr, nullptr)) return 1;
    return 2;
  }

  // ExactRiemannSolverBase.cpp:1002-1103
  __device__ __noinline__ bool feasible(double rhol, double ul, double pl, double cl, int idl, double rhor, double ur, double pr,
                         double cr, int idr, double& p0, double& rhol0, double& rhor0, double& ul0, double& ur0,
                         double& p1, double& rhol1, double& rhor1, double& ul1, double& ur1) {
    int found = acoustic(rhol, ul, pl, cl, idl, rhor, ur, pr, cr, idr, p0, rhol0, rhor0, ul0, ur0, p1, rhol1, rhor1, ul1, ur1);
    if (found == 2) return true;
    if (warm_used) { warm_miss = true; return false; }
    bool ok = true;
    double dp;
    if (found != 1) {
      dp = (pl != pr) ? fabs(pl - pr) : 0.5 * pl;
      for (int i = 0; i < P.maxIts_bracket; i++) {
        p0 = fmin(pl, pr) + 0.01 * (i + 1) * (i + 1) * fmin(dp, fmin(fabs(pl), fabs(pr)));
        if (p0 < P.min_pressure) p0 = P.pressure_at_failure;
        ok = pair(p0, rhol, ul, pl, idl, rhor, ur, pr, idr, rhol, (p0 > pl) ? rhol * 1.1 : rhol * 0.9, rhor,
                  (p0 > pr) ? rhor * 1.1 : rhor * 0.9, rhol0, ul0, rhor0, ur0);
        if (ok || suspended) break;
      }
      if (!ok) {
        for (int i = 0; i < P.maxIts_bracket; i++) {
          p0 = fmin(pl, pr) - 0.01 * (i + 1) * (i + 1) * fmin(dp, fmin(fabs(pl), fabs(pr)));
          if (p0 < P.min_pressure || i == P.maxIts_bracket / 2) p0 = P.pressure_at_failure;
          ok = pair(p0, rhol, ul, pl, idl, rhor, ur, pr, idr, rhol, (p0 > pl) ? rhol * 1.1 : rhol * 0.9, rhor,
                    (p0 > pr) ? rhor * 1.1 : rhor * 0.9, rhol0, ul0, rhor0, ur0);
          if (ok || suspended) break;
        }
      }
      if (!ok) return false;
    }
    dp = fmin(fabs(p0 - pl), fabs(p0 - pr));
    for (int i = 0; i < P.maxIts_bracket; i++) {
      p1 = p0 + 0.01 * (i + 1) * (i + 1) * dp;
      ok = pair(p1, rhol, ul, pl, idl, rhor, ur, pr, idr, rhol, rhol0, rhor, rhor0, rhol1, ul1, rhor1, ur1);
      if (ok || suspended) break;
    }
    if (!ok) {
      for (int i = 0; i < P.maxIts_bracket; i++) {
        p1 = p0 - 0.01 * (i + 1) * (i + 1) * dp;
        if (p1 < P.min_pressure) p1 = P.pressure_at_failure * 1000.0;
        ok = pair(p1, rhol, ul, pl, idl, rhor, ur, pr, idr, rhol, rhol0, rhor, rhor0, rhol1, ul1, rhor1, ur1);
        if (ok || suspended) break;
      }
    }
    if (!ok) return false;
    if (p0 > p1) {
      double t;
      t = p0; p0 = p1; p1 = t;
      t = rhol0; rhol0 = rhol1; rhol1 = t;
      t = rhor0; rhor0 = rhor1; rhor1 = t;
      t = ul0; ul0 = ul1; ul1 = t;
      t = ur0; ur0 = ur1; ur1 = t;
    }
    return true;
  }

  // ExactRiemannSolverBase.cpp:674-839
  __device__ __noinline__ bool bracket(double rhol, double ul, double pl, double cl, int idl, double rhor, double ur, double pr,
                        double cr, int idr, double& p0, double& rhol0, double& rhor0, double& ul0, double& ur0,
                        double& p1, double& rhol1, double& rhor1, double& ul1, double& ur1) {
    bool ok = feasible(rhol, ul, pl, cl, idl, rhor, ur, pr, cr, idr, p0, rhol0, rhor0, ul0, ur0, p1, rhol1, rhor1, ul1, ur1);
    if (!ok) { p0 = p1 = P.pressure_at_failure; return false; }
    if (suspended) return false;
    double p2 = 0, rhol2 = 0, rhor2 = 0, ul2 = 0, ur2 = 0, f0, f1;
    double fmin_, p_f, rl_f, rr_f, ul_f, ur_f;
    if (fabs(ul0 - ur0) < fabs(ul1 - ur1)) { fmin_ = fabs(ul0 - ur0); p_f = p0; rl_f = rhol0; rr_f = rhor0; ul_f = ul0; ur_f = ur0; }
    else { fmin_ = fabs(ul1 - ur1); p_f = p1; rl_f = rhol1; rr_f = rhor1; ul_f = ul1; ur_f = ur1; }
    int i;
    for (i = 0; i < P.maxIts_bracket; i++) {
      f0 = ul0 - ur0;
      f1 = ul1 - ur1;
      if (f0 * f1 <= 0.0) return true;
      if (warm_used && i >= P.warm_tries) { warm_miss = true; return false; }
      if (fabs(f0 - f1) > 1e-9) {
        p2 = p1 - f1 * (p1 - p0) / (f1 - f0);
        if (p2 < p0) p2 -= 0.1 * (p1 - p0);
        else p2 += 0.1 * (p1 - p0);
      } else p2 = 1.1 * p1;
      if (p2 < P.min_pressure || i == P.maxIts_bracket / 2) p2 = 1.0e-8;
      ok = pair(p2, rhol, ul, pl, idl, rhor, ur, pr, idr, rhol0, rhol1, rhor0, rhor1, rhol2, ul2, rhor2, ur2);
      if (!ok) {
        for (int j = 0; j < P.maxIts_bracket / 2; j++) {
          if (p2 < p0) p2 = p0 - 0.5 * (p0 - p2);
          else p2 = p1 + 0.5 * (p2 - p1);
          ok = pair(p2, rhol, ul, pl, idl, rhor, ur, pr, idr, rhol0, rhol1, rhor0, rhor1, rhol2, ul2, rhor2, ur2);
          if (ok || suspended) break;
        }
      }
      if (!ok) break;
      if (suspended) return false;
      if (fabs(ul2 - ur2) < fmin_) { fmin_ = fabs(ul2 - ur2); p_f = p2; rl_f = rhol2; rr_f = rhor2; ul_f = ul2; ur_f = ur2; }
      if (p2 < p0) {
        p1 = p0; rhol1 = rhol0; rhor1 = rhor0; ul1 = ul0; ur1 = ur0;
        p0 = p2; rhol0 = rhol2; rhor0 = rhor2; ul0 = ul2; ur0 = ur2;
      } else {
        p0 = p1; rhol0 = rhol1; rhor0 = rhor1; ul0 = ul1; ur0 = ur1;
        p1 = p2; rhol1 = rhol2; rhor1 = rhor2; ul1 = ul2; ur1 = ur2;
      }
    }
    if (fmin_ < P.failure_threshold * fabs(ul - ur)) {
      p0 = p1 = p_f; rhol0 = rhol1 = rl_f; rhor0 = rhor1 = rr_f; ul0 = ul1 = ul_f; ur0 = ur1 = ur_f;
    } else {
      p2 = P.pressure_at_failure;
      ok = pair(p2, rhol, ul, pl, idl, rhor, ur, pr, idr, rhol0, rhol1, rhor0, rhor1, rhol2, ul2, rhor2, ur2);
      if (ok) { p0 = p1 = p2; rhol0 = rhol1 = rhol2; rhor0 = rhor1 = rhor2; ul0 = ul1 = ul2; ur0 = ur1 = ur2; }
      else { p0 = p1 = p_f; rhol0 = rhol1 = rl_f; rhor0 = rhor1 = rr_f; ul0 = ul1 = ul_f; ur0 = ur1 = ur_f; }
    }
    return false;
  }

  // ExactRiemannSolverBase.cpp:351-558
  __device__ __noinline__ void finalize(const double* dir, const double* Vm, const double* Vp, double rhol, double ul, double pl,
                         int idl, double rhor, double ur, double pr, int idr, double rhol2, double rhor2, double u2,
                         double p2, bool trans_rare, const double* Vrare, double* Vs, int& id, double* Vsm, double* Vsp) {
    double utl[3] = {Vm[1] - ul * dir[0], Vm[2] - ul * dir[1], Vm[3] - ul * dir[2]};
    double utr[3] = {Vp[1] - ur * dir[0], Vp[2] - ur * dir[1], Vp[3] - ur * dir[2]};
    id = (u2 >= 0) ? idl : idr;
    if (trans_rare) {
      Vs[0] = Vrare[0]; Vs[1] = Vrare[1] * dir[0]; Vs[2] = Vrare[1] * dir[1]; Vs[3] = Vrare[1] * dir[2]; Vs[4] = Vrare[2];
    } else if (u2 >= 0) {
      bool star = false;
      if (pl >= p2) {
        const DevMat& M = mat(idl);
        double cl2 = sqrt(fmax(eos_c2(M, rhol2, eos_e(M, rhol2, p2)), 0.0));
        if (u2 - cl2 <= 0) star = true;
      } else if ((rhol2 * u2 - rhol * ul) / (rhol2 - rhol) <= 0) star = true;
      if (star) { Vs[0] = rhol2; Vs[1] = u2 * dir[0]; Vs[2] = u2 * dir[1]; Vs[3] = u2 * dir[2]; Vs[4] = p2; }
      else { Vs[0] = rhol; Vs[1] = ul * dir[0]; Vs[2] = ul * dir[1]; Vs[3] = ul * dir[2]; Vs[4] = pl; }
    } else {
      bool star = false;
      if (pr >= p2) {
        const DevMat& M = mat(idr);
        double cr2 = sqrt(fmax(eos_c2(M, rhor2, eos_e(M, rhor2, p2)), 0.0));
        if (u2 - cr2 >= 0) star = true;
      } else if ((rhor2 * u2 - rhor * ur) / (rhor2 - rhor) >= 0) star = true;
      if (star) { Vs[0] = rhor2; Vs[1] = u2 * dir[0]; Vs[2] = u2 * dir[1]; Vs[3] = u2 * dir[2]; Vs[4] = p2; }
      else { Vs[0] = rhor; Vs[1] = ur * dir[0]; Vs[2] = ur * dir[1]; Vs[3] = ur * dir[2]; Vs[4] = pr; }
    }
    for (int i = 1; i <= 3; i++) {
      if (u2 > 0) Vs[i] += utl[i - 1];
      else if (u2 < 0) Vs[i] += utr[i - 1];
      else Vs[i] += 0.5 * (utl[i - 1] + utr[i - 1]);
    }
    Vsm[0] = rhol2; Vsm[1] = utl[0] + u2 * dir[0]; Vsm[2] = utl[1] + u2 * dir[1]; Vsm[3] = utl[2] + u2 * dir[2]; Vsm[4] = p2;
    Vsp[0] = rhor2; Vsp[1] = utr[0] + u2 * dir[0]; Vsp[2] = utr[1] + u2 * dir[1]; Vsp[3] = utr[2] + u2 * dir[2]; Vsp[4] = p2;
  }

  // ExactRiemannSolverBase.cpp:59-347 with the non-adaptive retry after a failure
  // (lines 178-193 and 323-337), preceded by a cold restart when a warm start
  // misses.  Returns 0 (ok), 1 (failed), -1 (nonphysical input) or 2
  // (evaluation budget spent, see eval_limit).
  __device__ __noinline__ int solve(const double* dir, const double* Vm, int idl, const double* Vp, int idr, double* Vs,
                                    int& id, double* Vsm, double* Vsp) {
    nonadaptive = false;
    fallback = 0;
    suspended = false;
    int e = solve_once(dir, Vm, idl, Vp, idr, Vs, id, Vsm, Vsp);
    if (e == 2) return 2;
    if (e == 3) {  // the warm start did not bracket the root quickly: cold start
      int ev = evals;
      double w = warm_p;
      warm_p = 0.0;
      e = solve_once(dir, Vm, idl, Vp, idr, Vs, id, Vsm, Vsp);
      evals += ev;
      warm_p = w;
      if (e == 2) return 2;
    }
    if (e == 1) {
      int ev = evals;
      double w = warm_p;
      warm_p = 0.0;   // the fallback solver starts from acoustic theory
      nonadaptive = true;
      fallback = 1;
      e = solve_once(dir, Vm, idl, Vp, idr, Vs, id, Vsm, Vsp);
      evals += ev;
      nonadaptive = false;
      warm_p = w;
    }
    return e;
  }

  // One pass of ComputeRiemannSolution (the adaptive solver, or the
  // non-adaptive one of ExactRiemannSolverBase.cpp:2243-2519).
  __device__ __noinline__ int solve_once(const double* dir, const double* Vm, int idl, const double* Vp, int idr,
                                         double* Vs, int& id, double* Vsm, double* Vsp) {
    evals = 0;
    memo_clear();
    double rhol = Vm[0], ul = Vm[1] * dir[0] + Vm[2] * dir[1] + Vm[3] * dir[2], pl = Vm[4];
    double rhor = Vp[0], ur = Vp[1] * dir[0] + Vp[2] * dir[1] + Vp[3] * dir[2], pr = Vp[4];
    path1.reset(pl, rhol, ul);
    path3.reset(pr, rhor, ur);
    const DevMat& ML = mat(idl);
    const DevMat& MR = mat(idr);
    double cl = eos_c2(ML, rhol, eos_e(ML, rhol, pl));
    double cr = eos_c2(MR, rhor, eos_e(MR, rhor, pr));
    if (rhol <= 0 || cl < 0 || rhor <= 0 || cr < 0) {
      for (int i = 0; i < 5; i++) { Vsm[i] = Vm[i]; Vsp[i] = Vp[i]; Vs[i] = Vm[i]; }
      id = idl;
      return -1;
    }
    cl = sqrt(cl);
    cr = sqrt(cr);
    double p0 = DBL_MIN, ul0 = 0, ur0 = 0, rhol0 = DBL_MIN, rhor0 = DBL_MIN;
    double p1 = DBL_MIN, ul1 = 0, ur1 = 0, rhol1 = DBL_MIN, rhor1 = DBL_MIN;
    double p2 = DBL_MIN, ul2 = 0, ur2 = 0, rhol2 = DBL_MIN, rhor2 = DBL_MIN;
    bool trans_rare = false;
    double Vrare[3] = {0, 0, 0};
    if (ul == ur && pl == pr) {
      finalize(dir, Vm, Vp, rhol, ul, pl, idl, rhor, ur, pr, idr, rhol, rhor, ul, pl, false, Vrare, Vs, id, Vsm, Vsp);
      return 0;
    }
    warm_miss = false;
    warm_used = false;
    bool ok = bracket(rhol, ul, pl, cl, idl, rhor, ur, pr, cr, idr, p0, rhol0, rhor0, ul0, ur0, p1, rhol1, rhor1, ul1, ur1);
    if (suspended) return 2;
    if (warm_miss) return 3;
    if (!ok) {
      ok = rho_u_star(1, path1, rhol, ul, pl, p1, idl, rhol0, rhol0 * 1.1, rhol2, ul2, &trans_rare, Vrare);
      ok = ok && rho_u_star(3, path3, rhor, ur, pr, p1, idr, rhor0, rhol0 * 1.1, rhor2, ur2, &trans_rare, Vrare);
      if (!ok) {
        for (int i = 0; i < 5; i++) { Vsm[i] = Vm[i]; Vsp[i] = Vp[i]; }
        double ua = 0.5 * (ul + ur);
        id = (ua >= 0) ? idl : idr;
        for (int i = 0; i < 5; i++) Vs[i] = (ua >= 0) ? Vm[i] : Vp[i];
        return 1;
      }
      finalize(dir, Vm, Vp, rhol, ul, pl, idl, rhor, ur, pr, idr, rhol2, rhor2, 0.5 * (ul2 + ur2), p1, trans_rare,
               Vrare, Vs, id, Vsm, Vsp);
      return 1;
    }
    double f0 = ul0 - ur0, f1 = ul1 - ur1, f2;
    p2 = p1;
    f2 = f1;
    // the stopping rule's two denominators do not change during the loop
    const Quot Qp = qof(fmax(fabs(pl + 0.5 * rhol * ul * ul), fabs(pr + 0.5 * rhor * ur * ur)));
    const Quot Qc = qof(fmax(cl, cr));
    int iter;
    for (iter = 0; iter < P.maxIts_main; iter++) {
      double denom = f1 - f0;
      if (denom == 0) p2 = p0 + 0.5 * (p1 - p0);
      else {
        p2 = p2 - f2 * (p1 - p0) / denom;
        if (p2 <= p0 || p2 >= p1) p2 = p0 + 0.5 * (p1 - p0);
      }
      // the reference's "try_again" loop (ExactRiemannSolverBase.cpp:239-278)
      bool pass = false;
      while (true) {
        if (over_budget()) return 2;
        evals++;
        if (!rho_u_star(1, path1, rhol, ul, pl, p2, idl, rhol0, rhol1, rhol2, ul2, &trans_rare, Vrare)) {
          p2 = 0.5 * (p2 + p0);
          iter++;
          if (iter < P.maxIts_main) continue;
          break;
        }
        if (!rho_u_star(3, path3, rhor, ur, pr, p2, idr, rhor0, rhor1, rhor2, ur2, &trans_rare, Vrare)) {
          p2 = 0.5 * (p2 + p1);
          iter++;
          if (iter < P.maxIts_main) continue;
          break;
        }
        pass = true;
        break;
      }
      if (!pass) break;
      f2 = ul2 - ur2;
      if (f0 * f2 < 0.0) { p1 = p2; f1 = f2; rhol1 = rhol2; rhor1 = rhor2; }
      else { p0 = p2; f0 = f2; rhol0 = rhol2; rhor0 = rhor2; }
      double err_p = qd(fabs(p1 - p0), Qp);
      double err_u = qd(fabs(f2), Qc);
      if ((err_p < P.tol_main && err_u < P.tol_main) || (err_p < P.tol_main * 1e-3) || (err_u < P.tol_main * 1e-3)) break;
      trans_rare = false;
    }
    finalize(dir, Vm, Vp, rhol, ul, pl, idl, rhor, ur, pr, idr, rhol2, rhor2, 0.5 * (ul2 + ur2), p2, trans_rare, Vrare,
             Vs, id, Vsm, Vsp);
    return (iter == P.maxIts_main) ? 1 : 0;
  }
};
using ExactRiemannDev = ExactRiemannDevT<false>;
using ExactRiemannChainDev = ExactRiemannDevT<true>;

}  // namespace m2cg
