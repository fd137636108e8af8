/* C++ adapter over the C ABI of m2cg.h with the reference's operator method
 * names, so a driver shaped like the reference's Main.cpp keeps its calls:
 *
 *   SpaceOperator::ComputeTimeStepSize(V, ID, dt, cfl)       (SpaceOperator.h:135-136)
 *   SpaceOperator::ComputeResidual(V, ID, R, time, ...)      (SpaceOperator.h:144-149)
 *   LevelSetOperator::ComputeResidual(V, Phi, R, time)       (LevelSetOperator.cpp:768-781)
 *   TimeIntegratorBase::AdvanceOneTimeStep(V, ID, Phi, ...)  (TimeIntegrator.h:77-88)
 *   LevelSetOperator::Reinitialize(...)                      (LevelSetOperator.cpp:1338-1361)
 *   ExactRiemannSolverBase::ComputeRiemannSolution(dir, Vm, idm, Vp, idp, Vs, id, Vsm, Vsp)
 *                                                            (ExactRiemannSolverBase.h:42-47)
 *   FluxFcnBase::ComputeNumericalFluxAtCellInterface(dir, Vm, Vp, id, F)  (FluxFcnBase.h:65-69)
 *
 * The state (V, ID, Phi) lives on the device between calls; Upload / Download
 * move it in the reference's host layout (real cells, k-major, V as 5
 * interleaved primitives per cell).  Errors throw m2cg::Error with the
 * library's message where the reference would print and exit.  Header-only:
 * link against libm2cg.so. */
#pragma once
#include <stdexcept>
#include <string>
#include <vector>

#include "m2cg.h"

namespace m2cg {

class Error : public std::runtime_error {
 public:
  Error(m2cg_status s, const std::string& what)
      : std::runtime_error(what + ": " + (m2cg_last_error() ? m2cg_last_error() : "")), status(s) {}
  m2cg_status status;
};

inline void check(m2cg_status s, const char* what) {
  if (s != M2CG_OK) throw Error(s, what);
}

inline m2cg_config DefaultConfig() {
  m2cg_config c;
  check(m2cg_config_default(&c), "m2cg_config_default");
  return c;
}

class Solver {
 public:
  explicit Solver(const m2cg_config& cfg) : cfg_(cfg) {
    if (m2cg_abi_version() != M2CG_ABI_VERSION || m2cg_config_size() != sizeof(m2cg_config) ||
        m2cg_counters_size() != sizeof(m2cg_counters))
      throw std::runtime_error("libm2cg does not match this header");
    check(m2cg_create(&cfg_, &ctx_), "m2cg_create");
  }
  ~Solver() { m2cg_destroy(ctx_); }
  Solver(const Solver&) = delete;
  Solver& operator=(const Solver&) = delete;

  int64_t NumberOfCells() const { return (int64_t)cfg_.nx * cfg_.ny * cfg_.nz; }
  m2cg_ctx* Context() { return ctx_; }

  /* State in the host layout: V[5 N], ID[N], Phi[N] (Phi ignored without a level set). */
  void Upload(const double* V, const int32_t* ID, const double* Phi) {
    check(m2cg_upload_state(ctx_, V, ID, Phi), "m2cg_upload_state");
  }
  void Download(double* V, int32_t* ID, double* Phi) {
    check(m2cg_download_state(ctx_, V, ID, Phi), "m2cg_download_state");
  }

  void ComputeTimeStepSize(double& dt, double& cfl) { check(m2cg_compute_dt(ctx_, &dt, &cfl), "m2cg_compute_dt"); }
  /* R[5 N] for the current state (NULL keeps it on the device). */
  void ComputeResidual(double* R) { check(m2cg_compute_residual(ctx_, R), "m2cg_compute_residual"); }
  void ComputeLevelSetResidual(double* Rphi) {
    check(m2cg_levelset_residual(ctx_, Rphi), "m2cg_levelset_residual");
  }
  /* One step of the configured explicit integrator with this dt, including
   * the end-of-step material-ID update and, when configured, reinitialization. */
  void AdvanceOneTimeStep(double dt) { check(m2cg_advance(ctx_, dt), "m2cg_advance"); }
  /* The Main.cpp step loop for n steps (dt from the CFL, clamped at MaxTime). */
  m2cg_counters Run(int32_t n_steps) {
    m2cg_counters c;
    check(m2cg_run(ctx_, n_steps, &c), "m2cg_run");
    return c;
  }
  m2cg_counters Counters() {
    m2cg_counters c;
    check(m2cg_get_counters(ctx_, &c), "m2cg_get_counters");
    return c;
  }
  m2cg_reinit_stats Reinitialize() {
    m2cg_reinit_stats s;
    check(m2cg_reinitialize(ctx_, &s), "m2cg_reinitialize");
    return s;
  }

  /* One exact two-material Riemann problem; returns the reference's code
   * (0 ok, 1 failed).  Batches go through m2cg_riemann_batch directly. */
  int ComputeRiemannSolution(const double* dir, const double* Vm, int idm, const double* Vp, int idp, double* Vs,
                             int& id, double* Vsm, double* Vsp) {
    int32_t im = idm, ip = idp, ido = 0, iters = 0, err = 0;
    check(m2cg_riemann_batch(ctx_, 1, Vm, &im, Vp, &ip, dir, Vs, &ido, Vsm, Vsp, &iters, &err), "m2cg_riemann_batch");
    id = ido;
    return err;
  }
  void ComputeNumericalFluxAtCellInterface(int dir, const double* Vm, const double* Vp, int id, double* F) {
    int32_t d = dir, i = id;
    check(m2cg_flux_batch(ctx_, 1, &d, Vm, Vp, &i, F), "m2cg_flux_batch");
  }

  /* Diagnostics: probe points (n x 6, or n x 7 with a level set) and the
   * per-material integrals (n_materials x M2CG_N_INTEGRALS) in a box. */
  std::vector<double> SamplePoints(const std::vector<double>& xyz) {
    const int32_t n = (int32_t)(xyz.size() / 3);
    std::vector<double> out((size_t)n * (cfg_.n_levelsets > 0 ? 7 : 6));
    check(m2cg_sample_points(ctx_, n, xyz.data(), out.data()), "m2cg_sample_points");
    return out;
  }
  std::vector<double> Integrate(const double* box = nullptr) {
    std::vector<double> out((size_t)cfg_.n_materials * M2CG_N_INTEGRALS);
    check(m2cg_integrate(ctx_, box, out.data()), "m2cg_integrate");
    return out;
  }

 private:
  m2cg_config cfg_;
  m2cg_ctx* ctx_ = nullptr;
};

}  // namespace m2cg
