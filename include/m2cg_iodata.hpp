/* The reference-side binding: m2c's parsed input (IoData) to the library's
 * configuration.  Compiled inside m2c (or against its headers): include after
 * IoData.h.  It reads exactly the IoData fields the finite-volume step uses
 * (IoData.h:274-284 mesh, 550-565 materials, 655-730 schemes, 800-830 level
 * set, 880-905 multiphase, 920-1000 time) and refuses, with a reason, what the
 * library does not run: non-uniform meshes, other equations of state, more than
 * one level set, implicit time integration. */
#pragma once
#include <cstring>
#include "m2cg.h"

namespace m2cg {

inline void state_from(const StateVariable& s, double* v) {
  v[0] = s.density;
  v[1] = s.velocity_x;
  v[2] = s.velocity_y;
  v[3] = s.velocity_z;
  v[4] = s.pressure;
}

/* Fills *c from iod; returns false and sets *why when the input asks for
 * something outside the library's scope. */
inline bool config_from_iodata(const IoData& iod, m2cg_config* c, const char** why) {
  const char* dummy = nullptr;
  if (!why) why = &dummy;
  *why = nullptr;
  m2cg_config_default(c);
  // Mesh (uniform: no control points)
  const MeshData& m = iod.mesh;
  if (!m.xpoints_map.dataMap.empty() || !m.ypoints_map.dataMap.empty() || !m.zpoints_map.dataMap.empty()) {
    *why = "non-uniform mesh (Mesh.ControlPoint*)";
    return false;
  }
  if (m.type != MeshData::THREEDIMENSIONAL) { *why = "Mesh.Type other than ThreeDimensional"; return false; }
  c->nx = m.Nx; c->ny = m.Ny; c->nz = m.Nz;
  c->x0 = m.x0; c->xmax = m.xmax; c->y0 = m.y0; c->ymax = m.ymax; c->z0 = m.z0; c->zmax = m.zmax;
  const MeshData::BcType bc[6] = {m.bc_x0, m.bc_xmax, m.bc_y0, m.bc_ymax, m.bc_z0, m.bc_zmax};
  for (int s = 0; s < 6; s++) {
    if (bc[s] == MeshData::OVERSET || bc[s] == MeshData::NONE || bc[s] == MeshData::SIZE) {
      *why = "boundary condition other than Inlet, Inlet2, SlipWall, StickWall, Symmetry, Outlet";
      return false;
    }
    c->bc[s] = (int32_t)bc[s];   // the same values (IoData.h:283-284)
  }
  state_from(iod.bc.inlet, c->inlet);
  state_from(iod.bc.inlet2, c->inlet2);
  // Equations.Material[i]
  const auto& mats = iod.eqs.materials.dataMap;
  if (mats.empty() || (int)mats.size() > M2CG_MAX_MATERIALS) { *why = "material count"; return false; }
  c->n_materials = (int32_t)mats.size();
  for (const auto& kv : mats) {
    if (kv.first < 0 || kv.first >= (int)mats.size()) { *why = "material indices must run 0..n-1"; return false; }
    const MaterialModelData& d = *kv.second;
    m2cg_material& t = c->mat[kv.first];
    if (d.eos == MaterialModelData::STIFFENED_GAS) {
      t.eos = M2CG_EOS_SG;
      t.gamma = d.sgModel.specificHeatRatio;
      t.pc = d.sgModel.pressureConstant;
    } else if (d.eos == MaterialModelData::NOBLE_ABEL_STIFFENED_GAS) {
      t.eos = M2CG_EOS_NASG;
      t.gamma = d.nasgModel.specificHeatRatio;
      t.pc = d.nasgModel.pressureConstant;
      t.b = d.nasgModel.volumeConstant;
      t.q = d.nasgModel.energyConstant;
    } else if (d.eos == MaterialModelData::MIE_GRUNEISEN) {
      t.eos = M2CG_EOS_MG;
      t.rho0 = d.mgModel.rho0;
      t.c0 = d.mgModel.c0;
      t.Gamma0 = d.mgModel.Gamma0;
      t.s = d.mgModel.s;
      t.e0 = d.mgModel.e0;
    } else {
      *why = "equation of state other than StiffenedGas, NobleAbelStiffenedGas, MieGruneisen";
      return false;
    }
    t.rhomin = d.rhomin; t.pmin = d.pmin; t.rhomax = d.rhomax; t.pmax = d.pmax;
    t.failsafe_density = d.failsafe_density;
  }
  // Space.NavierStokes
  const SchemeData& ns = iod.schemes.ns;
  if (ns.flux == SchemeData::GODUNOV) { *why = "Flux = Godunov"; return false; }
  c->flux = (int32_t)ns.flux;
  c->roe_delta = ns.delta;
  c->rec_type = (int32_t)ns.rec.type;
  c->limiter = (int32_t)ns.rec.limiter;
  c->rec_var = (int32_t)ns.rec.varType;
  c->slope_near_interface = (int32_t)ns.rec.slopeNearInterface;
  c->minmod_coeff = ns.rec.generalized_minmod_coeff;
  // MultiPhase
  const MultiPhaseData& mp = iod.multiphase;
  c->mp_flux = (int32_t)mp.flux;
  c->mp_recon = (int32_t)mp.recon;
  c->mp_phasechange = (int32_t)mp.phasechange_type;
  c->mp_phasechange_dir = (int32_t)mp.phasechange_dir;
  c->mp_riemann_normal = (int32_t)mp.riemann_normal;
  // ExactRiemannSolution
  const ExactRiemannSolverData& er = iod.exact_riemann;
  c->maxits_main = er.maxIts_main; c->maxits_bracket = er.maxIts_bracket; c->maxits_shock = er.maxIts_shock;
  c->numsteps_rarefaction = er.numSteps_rarefaction;
  c->tol_main = er.tol_main; c->tol_shock = er.tol_shock; c->tol_rarefaction = er.tol_rarefaction;
  c->min_pressure = er.min_pressure; c->failure_threshold = er.failure_threshold;
  c->pressure_at_failure = er.pressure_at_failure;
  // Space.LevelSet[0]
  const auto& lss = iod.schemes.ls.dataMap;
  if (lss.size() > 1) { *why = "more than one level set"; return false; }
  c->n_levelsets = (int32_t)lss.size();
  if (!lss.empty()) {
    const LevelSetSchemeData& ls = *lss.begin()->second;
    c->ls_matid = ls.materialid;
    const LevelSetSchemeData::BcType lb[6] = {ls.bc_x0, ls.bc_xmax, ls.bc_y0, ls.bc_ymax, ls.bc_z0, ls.bc_zmax};
    for (int s = 0; s < 6; s++) c->ls_bc[s] = (int32_t)lb[s];   // IoData.h:814
    c->ls_solver = (int32_t)ls.solver;
    c->ls_flux = (int32_t)ls.flux;
    c->ls_delta = ls.delta;
    c->ls_rec_type = (int32_t)ls.rec.type;
    c->ls_limiter = (int32_t)ls.rec.limiter;
    c->ls_minmod_coeff = ls.rec.generalized_minmod_coeff;
    c->reinit_frequency = ls.reinit.frequency;
    c->reinit_frequency_dt = ls.reinit.frequency_dt;
    c->reinit_max_its = ls.reinit.maxIts;
    c->reinit_cfl = ls.reinit.cfl;
    c->reinit_tol = ls.reinit.convergence_tolerance;
  }
  // Time (explicit only)
  const TsData& ts = iod.ts;
  if (ts.type != TsData::EXPLICIT) { *why = "Time.Type other than Explicit"; return false; }
  c->ts_type = (int32_t)ts.expl.type;
  c->max_its = ts.maxIts;
  c->cfl = ts.cfl;
  c->timestep = ts.timestep;
  c->max_time = ts.maxTime;
  c->warm_start = 0;
  return true;
}

}  // namespace m2cg
