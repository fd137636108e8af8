// Test infrastructure only.  A C entry layer over the reference's own classes
// (VarFcnSG/NASG/MG, FluxFcnHLLC/LLF/GenRoe, ExactRiemannSolverBase), compiled
// from the reference sources by oracle/build_ref.py, so the tests can check
// the oracle restatement against the reference code on the same inputs.
#include <VarFcnSG.h>
#include <VarFcnNASG.h>
#include <VarFcnMG.h>
#include <FluxFcnHLLC.h>
#include <FluxFcnLLF.h>
#include <FluxFcnGenRoe.h>
#include <ExactRiemannSolverBase.h>
#include <memory>
#include <vector>
#include "../../include/m2cg.h"

int verbose = 0;
int INACTIVE_MATERIAL_ID = -1;

namespace {
struct RefSet {
  std::vector<std::unique_ptr<MaterialModelData>> md;
  std::vector<VarFcnBase*> vf;
  ~RefSet() { for (auto p : vf) delete p; }
};
void make(const m2cg_config* c, RefSet& r) {
  for (int m = 0; m < c->n_materials; m++) {
    auto d = std::make_unique<MaterialModelData>();
    const m2cg_material& s = c->mat[m];
    d->rhomin = s.rhomin; d->pmin = s.pmin; d->rhomax = s.rhomax; d->pmax = s.pmax;
    if (s.eos == M2CG_EOS_SG) {
      d->eos = MaterialModelData::STIFFENED_GAS;
      d->sgModel.specificHeatRatio = s.gamma; d->sgModel.pressureConstant = s.pc;
      r.vf.push_back(new VarFcnSG(*d));
    } else if (s.eos == M2CG_EOS_NASG) {
      d->eos = MaterialModelData::NOBLE_ABEL_STIFFENED_GAS;
      d->nasgModel.specificHeatRatio = s.gamma; d->nasgModel.pressureConstant = s.pc;
      d->nasgModel.volumeConstant = s.b; d->nasgModel.energyConstant = s.q;
      r.vf.push_back(new VarFcnNASG(*d));
    } else {
      d->eos = MaterialModelData::MIE_GRUNEISEN;
      d->mgModel.rho0 = s.rho0; d->mgModel.c0 = s.c0; d->mgModel.Gamma0 = s.Gamma0; d->mgModel.s = s.s;
      d->mgModel.e0 = s.e0;
      r.vf.push_back(new VarFcnMG(*d));
    }
    r.md.push_back(std::move(d));
  }
}
}  // namespace

extern "C" {

void ref_riemann_batch(const m2cg_config* c, int64_t n, const double* Vm, const int32_t* idm, const double* Vp,
                       const int32_t* idp, const double* dir, double* Vs, int32_t* id, double* Vsm, double* Vsp,
                       int32_t* err) {
  RefSet r;
  make(c, r);
  ExactRiemannSolverData rd;
  rd.maxIts_main = c->maxits_main; rd.maxIts_bracket = c->maxits_bracket; rd.maxIts_shock = c->maxits_shock;
  rd.numSteps_rarefaction = c->numsteps_rarefaction; rd.tol_main = c->tol_main; rd.tol_shock = c->tol_shock;
  rd.tol_rarefaction = c->tol_rarefaction; rd.min_pressure = c->min_pressure;
  rd.failure_threshold = c->failure_threshold; rd.pressure_at_failure = c->pressure_at_failure;
  ExactRiemannSolverBase rs(r.vf, rd);
  for (int64_t q = 0; q < n; q++) {
    double a[5], b[5], d3[3];
    for (int p = 0; p < 5; p++) { a[p] = Vm[q * 5 + p]; b[p] = Vp[q * 5 + p]; }
    for (int p = 0; p < 3; p++) d3[p] = dir[q * 3 + p];
    int oid = 0;
    err[q] = rs.ComputeRiemannSolution(d3, a, idm[q], b, idp[q], &Vs[q * 5], oid, &Vsm[q * 5], &Vsp[q * 5]);
    id[q] = oid;
  }
}

void ref_flux_batch(const m2cg_config* c, int64_t n, const int32_t* dir, const double* Vm, const double* Vp,
                    const int32_t* id, double* F) {
  RefSet r;
  make(c, r);
  // The flux constructors read only iod.schemes.ns.delta (FluxFcnGenRoe.h:29-30);
  // IoData's own constructor parses an input file, so hand them zeroed storage
  // with that one field set.
  alignas(IoData) static char storage[sizeof(IoData)];
  IoData* iod = reinterpret_cast<IoData*>(storage);
  iod->schemes.ns.delta = c->roe_delta;
  std::unique_ptr<FluxFcnBase> ff;
  if (c->flux == M2CG_FLUX_HLLC) ff.reset(new FluxFcnHLLC(r.vf, *iod));
  else if (c->flux == M2CG_FLUX_LLF) ff.reset(new FluxFcnLLF(r.vf, *iod));
  else ff.reset(new FluxFcnGenRoe(r.vf, *iod));
  for (int64_t q = 0; q < n; q++) {
    double a[5], b[5];
    for (int p = 0; p < 5; p++) { a[p] = Vm[q * 5 + p]; b[p] = Vp[q * 5 + p]; }
    ff->ComputeNumericalFluxAtCellInterface(dir[q], a, b, id[q], &F[q * 5]);
  }
}

}  // extern "C"
