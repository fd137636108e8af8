/*
 * m2cg.h -- C ABI of the GB300 multi-material finite-volume step (libm2cg.so).
 *
 * The library computes M2C's explicit multi-material finite-volume time step on
 * one GPU: MUSCL reconstruction, HLLC / local Lax-Friedrichs / generalized Roe
 * fluxes, stiffened-gas / Noble-Abel stiffened-gas / Mie-Gruneisen equations of
 * state, the exact two-material Riemann solver at material interfaces, the
 * level-set advection residual, the SSP Runge-Kutta stage update and the CFL
 * time-step reduction.
 *
 * Every entry point takes plain pointers and sizes.  Host pointers are copied;
 * the context owns all device memory.  Integer enum values follow the
 * reference's IoData enums so a reference config maps field-for-field.
 *
 * Threading: one context per host thread; every call is issued on the
 * context's own CUDA stream.  Calls that return host data synchronize that
 * stream.  No entry point aborts the process: failures come back as an
 * m2cg_status and per-step counters.
 */
#ifndef M2CG_H
#define M2CG_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define M2CG_ABI_VERSION 1
#define M2CG_MAX_MATERIALS 8

typedef enum {
  M2CG_OK = 0,
  M2CG_ERR_INVALID_ARG = 1,    /* null pointer, bad size, unsupported option */
  M2CG_ERR_CUDA = 2,           /* a CUDA runtime call failed (message via m2cg_last_error) */
  M2CG_ERR_NONPHYSICAL = 3,    /* reserved: where the reference calls exit(-1) on a failed CheckState the
                                  library counts the state (m2cg_counters.nonphysical) and goes on */
  M2CG_ERR_UNRESOLVED = 4,     /* reserved: unresolved swept cells without a reinitializer, where the
                                  reference stops, are counted (unresolved_cells - unresolved_fixed) */
  M2CG_ERR_NO_DEVICE = 5,      /* no CUDA device visible */
  M2CG_ERR_CAPACITY = 6        /* a fixed-size buffer would overflow */
} m2cg_status;

/* Equation of state (VarFcnBase::Type, VarFcnBase.h:40-42). */
enum { M2CG_EOS_SG = 0, M2CG_EOS_NASG = 1, M2CG_EOS_MG = 2 };
/* Boundary conditions (MeshData::BcType, IoData.h:283-284). */
enum { M2CG_BC_INLET = 1, M2CG_BC_INLET2 = 2, M2CG_BC_SLIPWALL = 3, M2CG_BC_STICKWALL = 4,
       M2CG_BC_SYMMETRY = 5, M2CG_BC_OUTLET = 7 };
/* Level-set boundary conditions (LevelSetSchemeData::BcType, IoData.h:814). */
enum { M2CG_LSBC_ZERO_NEUMANN = 1, M2CG_LSBC_LINEAR_EXTRAPOLATION = 2, M2CG_LSBC_NON_NEGATIVE = 3 };
/* Numerical flux (SchemeData::Flux, IoData.h:710). */
enum { M2CG_FLUX_ROE = 0, M2CG_FLUX_LLF = 1, M2CG_FLUX_HLLC = 2 };
/* Reconstruction (ReconstructionData, IoData.h:660-671). */
enum { M2CG_REC_CONSTANT = 0, M2CG_REC_LINEAR = 1 };
enum { M2CG_LIM_NONE = 0, M2CG_LIM_GENERALIZED_MINMOD = 1, M2CG_LIM_VANALBADA = 2 };
enum { M2CG_SLOPE_ZERO = 0, M2CG_SLOPE_NONZERO = 1 };
/* Reconstruction.VariableType (IoData.cpp:1300-1304). */
enum { M2CG_VAR_PRIMITIVE = 0, M2CG_VAR_CONSERVATIVE = 1, M2CG_VAR_PRIMITIVE_CHARACTERISTIC = 2,
       M2CG_VAR_CONSERVATIVE_CHARACTERISTIC = 3 };
/* Level-set solver and finite-volume flux (LevelSetSchemeData, IoData.cpp:1544-1556). */
enum { M2CG_LS_FINITE_VOLUME = 0, M2CG_LS_FINITE_DIFFERENCE = 1 };
enum { M2CG_LSFLUX_ROE = 0, M2CG_LSFLUX_LLF = 1, M2CG_LSFLUX_UPWIND = 2 };
/* Multiphase (MultiPhaseData, IoData.h:893-903). */
enum { M2CG_MPFLUX_EXACT = 0, M2CG_MPFLUX_NUMERICAL = 1, M2CG_MPFLUX_LLF = 2 };
enum { M2CG_MPREC_CONSTANT = 0, M2CG_MPREC_LINEAR = 1 };
enum { M2CG_PHASECHANGE_RIEMANN = 0, M2CG_PHASECHANGE_EXTRAPOLATION = 1 };
enum { M2CG_PCDIR_ALL = 0, M2CG_PCDIR_UPWIND = 1 };
enum { M2CG_RNORMAL_LEVEL_SET = 0, M2CG_RNORMAL_MESH = 1, M2CG_RNORMAL_AVERAGE = 2 };
/* Time integrator (ExplicitData::Type, IoData.h:931). */
enum { M2CG_TS_FORWARD_EULER = 0, M2CG_TS_RK2 = 1, M2CG_TS_RK3 = 2 };

/* One material: Equations.Material[i] (MaterialModelData, IoData.cpp:1044-1055;
 * StiffenedGasModel / NobleAbelStiffenedGasModel / MieGruneisenModel). */
typedef struct {
  int32_t eos;                 /* M2CG_EOS_* */
  int32_t pad_;
  double gamma;                /* SG, NASG: SpecificHeatRatio */
  double pc;                   /* SG, NASG: PressureConstant */
  double b;                    /* NASG: VolumeConstant */
  double q;                    /* NASG: EnergyConstant */
  double rho0, c0, Gamma0, s, e0; /* MG: ReferenceDensity, BulkSpeedOfSound, GruneisenParameter,
                                     HugoniotSlope, ReferenceSpecificInternalEnergy */
  double rhomin, pmin, rhomax, pmax; /* DensityCutOff, PressureCutOff and the upper clips */
  double failsafe_density;
} m2cg_material;

/* The subset of IoData the hot path reads, with the reference keys noted. */
typedef struct {
  /* Mesh: uniform Cartesian (MeshGenerator::ComputeMesh1DUniform, MeshGenerator.cpp:160-171) */
  int32_t nx, ny, nz;
  int32_t pad0_;
  double x0, xmax, y0, ymax, z0, zmax;
  int32_t bc[6];               /* BoundaryConditionX0, Xmax, Y0, Ymax, Z0, Zmax: M2CG_BC_* */
  double inlet[5];             /* BoundaryConditions.Inlet  {Density, VelocityX/Y/Z, Pressure} */
  double inlet2[5];            /* BoundaryConditions.Inlet2 */
  /* Equations */
  int32_t n_materials;         /* 1..M2CG_MAX_MATERIALS */
  int32_t pad1_;
  m2cg_material mat[M2CG_MAX_MATERIALS];
  /* Space.NavierStokes */
  int32_t flux;                /* Flux: M2CG_FLUX_* (default HLLC) */
  int32_t rec_type;            /* Reconstruction.Type (default Linear) */
  int32_t limiter;             /* Reconstruction.Limiter (default GeneralizedMinMod) */
  int32_t rec_var;             /* Reconstruction.VariableType: M2CG_VAR_* (default Primitive) */
  int32_t slope_near_interface;/* Reconstruction.SlopeNearInterface (default NonZero) */
  int32_t pad2_;
  double minmod_coeff;         /* GeneralizedMinModCoefficient (1.2) */
  double roe_delta;            /* EntropyFixCoefficient (0.2) */
  /* MultiPhase */
  int32_t mp_flux;             /* Flux (default Numerical) */
  int32_t mp_recon;            /* ReconstructionAtInterface (default Constant) */
  int32_t mp_phasechange;      /* PhaseChange (default RiemannSolution) */
  int32_t mp_phasechange_dir;  /* PhaseChangeDirection (default Upwind) */
  /* ExactRiemannSolution (ExactRiemannSolverData, IoData.cpp:1622-1637) */
  int32_t maxits_main, maxits_bracket, maxits_shock, numsteps_rarefaction;
  double tol_main, tol_shock, tol_rarefaction;
  double min_pressure, failure_threshold, pressure_at_failure;
  /* Space.LevelSet[0] (one level set; finite-difference solver) */
  int32_t n_levelsets;         /* 0 or 1 */
  int32_t ls_matid;            /* LevelSet[0].MaterialID */
  int32_t ls_bc[6];            /* BoundaryConditionX0..Zmax: M2CG_LSBC_* */
  /* Time */
  int32_t ts_type;             /* Explicit.Type: M2CG_TS_* */
  int32_t max_its;             /* MaxIts */
  double cfl;                  /* CFL (0.5) */
  double timestep;             /* TimeStep (<=0: CFL-driven) */
  double max_time;             /* MaxTime */
  /* Learned warm start for the interface Riemann solve (no reference counterpart) */
  int32_t warm_start;          /* 0 = cold start (reference), 1 = MLP warm start */
  /* LevelSet[0].Reinitialization (IoData.cpp:1421-1429): full domain, first layer FIXED */
  int32_t reinit_frequency;    /* Frequency: every that many steps (<= 0: never, the default) */
  int32_t reinit_max_its;      /* MaxIts (30) */
  int32_t pad4_;
  double reinit_cfl;           /* CFL (0.8) */
  double reinit_tol;           /* ConvergenceTolerance (2e-4) */
  /* LevelSet[0] solver and its own reconstruction (LevelSetSchemeData, IoData.cpp:1513-1590) */
  int32_t ls_solver;           /* Solver: M2CG_LS_FINITE_VOLUME / M2CG_LS_FINITE_DIFFERENCE (default) */
  int32_t ls_flux;             /* Flux (finite volume): M2CG_LSFLUX_* (default Roe) */
  double ls_delta;             /* EntropyFixCoefficient of the Roe flux (0.2) */
  int32_t ls_rec_type;         /* Reconstruction.Type (default Linear) */
  int32_t ls_limiter;          /* Reconstruction.Limiter (default GeneralizedMinMod) */
  double ls_minmod_coeff;      /* Reconstruction.GeneralizedMinModCoefficient (1.2) */
  double reinit_frequency_dt;  /* Reinitialization.FrequencyDt: after every step that crosses a multiple of
                                  this time (> 0 takes precedence over Frequency, Utils.cpp:344-349) */
  int32_t mp_riemann_normal;   /* MultiPhase.RiemannNormal (default Mesh): axis of the interface Riemann
                                  problems (SpaceOperator.cpp:2186-2415) */
  int32_t pad5_;
} m2cg_config;

/* Per-step counters (the reference prints these as warnings; SpaceOperator.cpp:681-683,
 * 2031-2034, 2557-2559). */
typedef struct {
  int64_t interface_faces;     /* faces whose two cells carry different material IDs */
  int64_t riemann_errors;      /* ComputeRiemannSolution returned non-zero */
  int64_t riemann_iterations;  /* secant iterations + bracketing evaluations, summed */
  int64_t riemann_solves;      /* exact solves performed (faces x stages) */
  int64_t clipped_cells;       /* ClipDensityAndPressure hits in stage updates */
  int64_t clipped_faces;       /* clipped reconstructed face states */
  int64_t nonphysical;         /* CheckState failures (reference: exit(-1)) */
  int64_t swept_cells;         /* cells whose material ID changed this step */
  int64_t unresolved_cells;    /* swept cells with no Riemann solution / extrapolation */
  int64_t steps;               /* time steps taken on this context */
  double time;                 /* simulated time */
  double dt;                   /* last time step */
  double cfl;                  /* last CFL number */
  int64_t riemann_fallbacks;   /* solves retried with the non-adaptive solver (ExactRiemannSolverBase.cpp:178-193, 323-337) */
  int64_t path_capped;         /* solves whose integration-path cache reached its capacity */
  int64_t unresolved_fixed;    /* unresolved cells repaired after a forced reinitialization
                                  (TimeIntegrator.cpp:776-797; needs reinitialization configured) */
} m2cg_counters;

typedef struct m2cg_ctx m2cg_ctx;

/* ---- library ---------------------------------------------------------- */
int32_t     m2cg_abi_version(void);
/* sizeof(m2cg_config) and sizeof(m2cg_counters), for bindings that mirror the structs. */
size_t      m2cg_config_size(void);
size_t      m2cg_counters_size(void);
const char* m2cg_last_error(void);
/* IoData defaults (IoData.cpp:1044-1055, 1262-1272, 1368-1374, 1508-1530, 1618-1637,
 * 1690-1710, 1838-1850). */
m2cg_status m2cg_config_default(m2cg_config* cfg);

/* ---- context ---------------------------------------------------------- */
/* Replaces the construction in Main.cpp:88-222 and 475-491 (VarFcn, FluxFcn,
 * ExactRiemannSolverBase, SpaceOperator, LevelSetOperator, TimeIntegrator). */
m2cg_status m2cg_create(const m2cg_config* cfg, m2cg_ctx** out);
void        m2cg_destroy(m2cg_ctx* ctx);

/* State upload / download over the real cells, k-major then j then i.
 * V: N x 5 doubles, dof-interleaved like SpaceVariable3D (rho, u, v, w, p).
 * id: N material IDs.  phi: N doubles (ignored when n_levelsets == 0).
 * Ghost cells are filled by the boundary conditions. */
m2cg_status m2cg_upload_state(m2cg_ctx* ctx, const double* V, const int32_t* id, const double* phi);
m2cg_status m2cg_download_state(m2cg_ctx* ctx, double* V, int32_t* id, double* phi);

/* SpaceOperator::ComputeTimeStepSize (SpaceOperator.cpp:1298-1330). */
m2cg_status m2cg_compute_dt(m2cg_ctx* ctx, double* dt, double* cfl);

/* The state with its ghost layer, as the reference's ghosted local arrays hold
 * it after the boundary conditions (SpaceOperator.cpp:738-821; edge and corner
 * ghosts are not populated, as there): (nx+2) x (ny+2) x (nz+2) cells, i
 * fastest, real cell (i,j,k) at ((k+1)(ny+2) + j+1)(nx+2) + i+1.  V: 5 planes of
 * that size (rho, u, v, w, p); id, phi: one plane each (phi ignored without a
 * level set).  Any pointer may be NULL.  Used by probes and line plots
 * (ProbeOutput.cpp:360-597, 848-886), which interpolate across the boundary. */
m2cg_status m2cg_download_ghosted(m2cg_ctx* ctx, double* V, int32_t* id, double* phi);
/* Solution at n probe points xyz[3n] (ProbeOutput::SetupInterpolation and
 * InterpolateSolutionAtProbe, ProbeOutput.cpp:360-480, 849-886): trilinear over the
 * ghosted cell-centre grid; out[n * 6] (n * 7 with a level set) per point: rho, vx, vy,
 * vz, p, material ID (interpolated), phi.  A point outside the ghosted grid, or one whose
 * eight corners are all edge / corner ghosts, is M2CG_ERR_INVALID_ARG. */
m2cg_status m2cg_sample_points(m2cg_ctx* ctx, int32_t n, const double* xyz, double* out);
/* Per-material integrals over the real cells whose centres lie in box = {xmin, xmax,
 * ymin, ymax, zmin, zmax} (NULL: everywhere), as EnergyIntegrationOutput computes them
 * on a Cartesian mesh (EnergyIntegrationOutput.cpp:247-610): out[n_materials *
 * M2CG_N_INTEGRALS], per material: volume, mass, total energy rho (|u|^2/2 + e), total
 * enthalpy rho (|u|^2/2 + e) + p, kinetic energy, internal energy rho e (each times the
 * cell volume, summed). */
#define M2CG_N_INTEGRALS 6
m2cg_status m2cg_integrate(m2cg_ctx* ctx, const double* box, double* out);

/* SpaceOperator::ComputeResidual on the current state with the stored
 * Riemann solutions refreshed (SpaceOperator.cpp:2573-2641, first RK stage).
 * R: N x 5 doubles (real cells), may be NULL to keep the residual on device. */
m2cg_status m2cg_compute_residual(m2cg_ctx* ctx, double* R);

/* The interface Riemann solutions the last m2cg_compute_residual (or the first
 * stage of the last step) stored: what ComputeResidual's RiemannSolutions
 * argument receives (SpaceOperator.h:144-149, filled at SpaceOperator.cpp:
 * 1661-1666, 1821-1826, 1980-1985).  Row r: the face between cell
 * (i - e_d) and cell (i, j, k) = ijkd[4r .. 4r+2] in direction d = ijkd[4r+3]
 * (0 x, 1 y, 2 z); vsm[5r..] the star state on the minus side with material
 * ids[2r] -- the reference's left / bottom / back entry of cell (i, j, k) --
 * and vsp[5r..] on the plus side with material ids[2r+1] -- the right / top /
 * front entry of cell (i, j, k) - e_d.  Only solves that succeeded are listed,
 * as in the reference; the IDs are the cells' current ones.  At most cap rows
 * are written; *n receives the number of stored solutions (host arrays). */
m2cg_status m2cg_riemann_solutions(m2cg_ctx* ctx, int64_t cap, int32_t* ijkd, double* vsm, double* vsp,
                                   int32_t* ids, int64_t* n);

/* LevelSetOperator::ComputeResidual, finite-difference solver
 * (LevelSetOperator.cpp:768-870). Rphi: N doubles. */
m2cg_status m2cg_levelset_residual(m2cg_ctx* ctx, double* Rphi);

/* TimeIntegratorBase::AdvanceOneTimeStep with a given dt, including the
 * end-of-step material-ID and interface-state update (TimeIntegrator.cpp:319-455,
 * 527-715, 720-843). */
m2cg_status m2cg_advance(m2cg_ctx* ctx, double dt);

/* The step loop of Main.cpp:653-771: n_steps x (ComputeTimeStepSize, clamp to
 * MaxTime, AdvanceOneTimeStep).  dt stays on the device; nothing is copied to
 * the host until the call returns.  Counters are summed over the steps. */
m2cg_status m2cg_run(m2cg_ctx* ctx, int32_t n_steps, m2cg_counters* counters);

m2cg_status m2cg_get_counters(m2cg_ctx* ctx, m2cg_counters* counters);

/* Level-set reinitialization statistics of a context (summed over its calls). */
typedef struct {
  int64_t calls;               /* reinitializations that found an interface and ran */
  int64_t iterations;          /* pseudo-time RK3 iterations, summed over attempts */
  int64_t retries;             /* restarts with CFL / 1.5 (LevelSetReinitializer.cpp:157-174) */
  int64_t failures;            /* gave up below CFL 0.02 (the reference stops the program) */
  int64_t loop_bodies;         /* executions of the device loop body */
  double cfl;                  /* current pseudo-time CFL (kept reduced after a retry) */
  double last_residual;        /* max |grad phi| - 1 of the last iteration's first sub-stage */
  double last_change;          /* largest relative change of the last completed iteration */
} m2cg_reinit_stats;

/* LevelSetOperator::Reinitialize with must_do (LevelSetOperator.cpp:1338-1361):
 * one full-domain reinitialization of the level set now, first layer FIXED
 * (LevelSetReinitializer.cpp:76-176), with the context's MaxIts / CFL /
 * ConvergenceTolerance.  The stepping (m2cg_run, m2cg_advance) calls the same
 * after every reinit_frequency-th step (TimeIntegrator.cpp:756-768).  stats
 * (optional) receives the context's totals. */
m2cg_status m2cg_reinitialize(m2cg_ctx* ctx, m2cg_reinit_stats* stats);
m2cg_status m2cg_get_reinit_stats(m2cg_ctx* ctx, m2cg_reinit_stats* stats);

/* Conserved totals sum(U * vol) over real cells: mass, momentum x/y/z, energy. */
m2cg_status m2cg_conserved_totals(m2cg_ctx* ctx, double totals[5]);

/* ---- batched device kernels (unit-level parity surface) ---------------- */
/* ExactRiemannSolverBase::ComputeRiemannSolution (ExactRiemannSolverBase.cpp:59-347)
 * for n independent problems, host arrays:
 *   Vm, Vp: n x 5; idm, idp: n; dir: n x 3 (unit normals)
 *   Vs, Vsm, Vsp: n x 5 outputs; id: n; iters: n (secant + bracketing evaluations);
 *   err: n (the reference's return code: 0 ok, 1 failed). */
m2cg_status m2cg_riemann_batch(m2cg_ctx* ctx, int64_t n,
                               const double* Vm, const int32_t* idm,
                               const double* Vp, const int32_t* idp, const double* dir,
                               double* Vs, int32_t* id, double* Vsm, double* Vsp,
                               int32_t* iters, int32_t* err);

/* Exact Riemann solves of independent 1D problems, each with its own pair of
 * stiffened-gas / Noble-Abel stiffened-gas materials -- the learned warm
 * start's training and evaluation sets (no reference counterpart: the
 * reference solver is configured with one material table,
 * ExactRiemannSolverBase.cpp:34-50).  Host arrays:
 *   W      n x 6  {rho_l, u_l, p_l, rho_r, u_r, p_r}
 *   eos    n x 10 {type (M2CG_EOS_SG / M2CG_EOS_NASG), gamma, pc, b, q} left, then right
 *   warm_p n starting pressures (> 0: learned warm start, see m2cg_mlp_*) or NULL; used on every
 *          problem that has one (the in-step warm start of m2cg_set_warm_start uses its predictions
 *          only where the acoustic pressure jump exceeds 5 % of the mean pressure)
 *   out    n x 4  {p*, u*, rho*_l, rho*_r}
 *   iters  wave-pair evaluations (bracketing + main loop), err as m2cg_riemann_batch (optional)
 *   kernel_ms  device time of the solve kernel alone (optional). */
m2cg_status m2cg_riemann_batch_eos(m2cg_ctx* ctx, int64_t n, const double* W, const double* eos,
                                   const double* warm_p, double* out, int32_t* iters, int32_t* err,
                                   float* kernel_ms);
/* FluxFcn*::ComputeNumericalFluxAtCellInterface (FluxFcnHLLC.h:196-245,
 * FluxFcnLLF.h:80-111, FluxFcnGenRoe.h:183-213) with the context's flux type,
 * host arrays: dir n; Vm, Vp n x 5; id n; F n x 5 output. */
m2cg_status m2cg_flux_batch(m2cg_ctx* ctx, int64_t n, const int32_t* dir,
                            const double* Vm, const double* Vp, const int32_t* id, double* F);

/* No counterpart in the reference.  The exact Riemann solves of
 * m2cg_riemann_batch for callers that cannot allocate device memory (a host that
 * hands the library only its own pre-allocated buffers, or code running where
 * new allocations are forbidden).  Needs no context and allocates nothing: the
 * solver's scratch is a 32 MiB file-scope device array that every GPU loading
 * the library keeps until exit.  Every array argument is a DEVICE pointer with
 * the layout of m2cg_riemann_batch; iters and err may be NULL; cfg is a host
 * pointer (materials and ExactRiemannSolution fields are read); stream is a
 * cudaStream_t (NULL: default stream).  path_cap is the integration-path cache
 * capacity per wave, 2..1024 (M2CG_ERR_CAPACITY beyond); m2cg_riemann_batch
 * uses 1024, and results equal m2cg_riemann_batch's bit for bit at 1024 (a
 * smaller cache can cap a long rarefaction path; capped solves are not
 * reported separately here).  Solver concurrency is 32 MiB / (48 * path_cap)
 * threads: 682 threads (5 blocks of 128) at 1024, while path_cap <= 32 gives
 * 21,845 threads, enough for every SM of a 152-SM GB300.  A row with an
 * invalid material ID is not solved: id = -1, err = -2 (when err is given),
 * iters = 0 and NaN in its Vs, Vsm and Vsp.  Asynchronous on `stream`.  All
 * calls share the scratch array: calls that overlap on one GPU race, so
 * serialize them.  The first call on a device looks up the array's address;
 * make it before any stream capture.  After a device reset the next call looks
 * the address up again in the new context. */
m2cg_status m2cg_riemann_batch_noalloc(const m2cg_config* cfg, int64_t n,
                                       const double* Vm, const int32_t* idm,
                                       const double* Vp, const int32_t* idp, const double* dir,
                                       double* Vs, int32_t* id, double* Vsm, double* Vsp,
                                       int32_t* iters, int32_t* err, int32_t path_cap, void* stream);

/* ---- learned warm start for the interface Riemann solve -----------------
 * No reference counterpart: a 16 -> 64 -> 64 -> 64 -> 1 SiLU MLP (BF16
 * tensor-core GEMMs, FP32 accumulate, FP32 Adam) predicts the star pressure
 * from the two states and their EOS parameters; the exact solver starts from
 * a pair bracketing the prediction instead of the acoustic pair
 * (ExactRiemannSolverBase.cpp:1107-1158), falls back to the acoustic start
 * when that pair does not bracket the root within three secant expansions,
 * and converges with the reference's stopping rule.  Problems use the
 * m2cg_riemann_batch_eos row layout (W n x 6, eos n x 10). */
#define M2CG_MLP_FEATURES 16
#define M2CG_MLP_PARAMS 9473   /* W1[64][16] b1[64] W2[64][64] b2 W3[64][64] b3 w4[64] b4 (FP32) */
typedef struct m2cg_mlp m2cg_mlp;
m2cg_status m2cg_mlp_create(uint64_t seed, m2cg_mlp** out);
void m2cg_mlp_destroy(m2cg_mlp* mlp);
m2cg_status m2cg_mlp_set_params(m2cg_mlp* mlp, const float* params);
m2cg_status m2cg_mlp_get_params(m2cg_mlp* mlp, float* params);
/* Network inputs (n x 16, BF16-rounded, returned as float), the reference
 * pressure p_ref of each problem (optional) and, when pstar and t are given,
 * the targets t = ln(p* / p_ref) / 4 (the prediction is p_ref exp(4 t)). */
m2cg_status m2cg_mlp_features(int64_t n, const double* W, const double* eos, const double* pstar, float* X,
                              float* pref, float* t);
/* Keeps features and targets of a labelled set on the device for training. */
m2cg_status m2cg_mlp_set_data(m2cg_mlp* mlp, int64_t n, const double* W, const double* eos, const double* pstar);
/* Mini-batch Adam (cosine learning-rate decay to lr / 20) on the squared error
 * of t over the stored set, reshuffled every epoch, whole batches only.
 * loss_per_epoch (optional, epochs entries): mean loss during each epoch;
 * ms: device time. */
m2cg_status m2cg_mlp_train(m2cg_mlp* mlp, int32_t epochs, int32_t batch, float lr, uint64_t seed,
                           float* loss_per_epoch, float* ms);
/* One forward + backward pass over X (n x 16) and targets t without an update:
 * gradient of the mean squared error (M2CG_MLP_PARAMS floats) and the loss. */
m2cg_status m2cg_mlp_grad(m2cg_mlp* mlp, int64_t n, const float* X, const float* t, float* grad, float* loss);
/* One Adam update of the parameters with the given gradient (M2CG_MLP_PARAMS
 * floats, host), the moments and step count that m2cg_mlp_train keeps
 * (beta1 0.9, beta2 0.999, eps 1e-8, bias-corrected; m2cg_mlp_set_params
 * resets them), at learning rate lr. */
m2cg_status m2cg_mlp_adam_step(m2cg_mlp* mlp, const float* grad, float lr);
/* Network output t for features X (n x 16). */
m2cg_status m2cg_mlp_forward(m2cg_mlp* mlp, int64_t n, const float* X, float* t);
/* Predicted star pressures (0 where the prediction is not positive) for
 * problems W / eos; kernel_ms: device time of features + network. */
m2cg_status m2cg_mlp_predict(m2cg_mlp* mlp, int64_t n, const double* W, const double* eos, double* p_pred,
                             float* kernel_ms);
/* Warm-start the interface solves of the finite-volume step with this network
 * (NULL: cold start, the reference behaviour).  The network must outlive its
 * use by the context; the step's CUDA graph is captured again. */
m2cg_status m2cg_set_warm_start(m2cg_ctx* ctx, m2cg_mlp* mlp);

/* ---- batched ensemble of independent domains ----------------------------
 * No reference counterpart (the reference runs one domain per program): n
 * member domains, each an ordinary context (m2cg_ensemble_member returns it;
 * upload / download / counters work on it as on any context), advanced
 * together with one launch per kernel and Runge-Kutta stage for all members
 * (persistent cell and face kernels whose blocks take the members' blocks in
 * turn, the interface Riemann solves of all members as one pool) inside one
 * CUDA graph.  Members may differ in mesh, materials,
 * boundary conditions and state; they must share the time integrator (RK2 or
 * RK3), the level-set count and the interface reconstruction.  Each member
 * keeps its own CFL time step.  m2cg_ensemble_run_sequential advances the
 * members one after another with their own per-domain launches (the baseline
 * the batched step is compared with); ms: elapsed milliseconds. */
typedef struct m2cg_ensemble m2cg_ensemble;
m2cg_status m2cg_ensemble_create(const m2cg_config* cfgs, int32_t n, m2cg_ensemble** out);
void m2cg_ensemble_destroy(m2cg_ensemble* ens);
int32_t m2cg_ensemble_size(const m2cg_ensemble* ens);
m2cg_ctx* m2cg_ensemble_member(m2cg_ensemble* ens, int32_t i);
m2cg_status m2cg_ensemble_run(m2cg_ensemble* ens, int32_t n_steps, float* ms);
m2cg_status m2cg_ensemble_run_sequential(m2cg_ensemble* ens, int32_t n_steps, float* ms);
int64_t m2cg_ensemble_kernel_launches(const m2cg_ensemble* ens);
/* No reference counterpart: tunes the batched step's interface-solve schedule.
 * Each candidate first-pass evaluation budget cand[0..n_cand) runs `steps`
 * real steps of the run (the members' states advance; the budget changes the
 * schedule, not the results); the fastest is kept for later m2cg_ensemble_run
 * calls.  best / ms_per_step (optional) receive the choice and its time. */
m2cg_status m2cg_ensemble_autotune(m2cg_ensemble* ens, int32_t steps, int32_t n_cand, const int32_t* cand,
                                   int32_t* best, float* ms_per_step);
/* No reference counterpart: tunes the block shape of the batched cell and face
 * kernels per size class (members with the same cell count along x).  shapes:
 * n_shapes rows {tx, ty, tz} with tx * ty * tz = 128 cells per block, or
 * {0, 0, 0} for 128 consecutive cells in x-fastest order (the default).  For
 * each class in turn, every shape runs `steps` real batched steps with the
 * other classes at their choice so far, and the fastest is kept; the shape
 * changes the schedule, not the results.  member_shape (optional, one entry
 * per member) receives the chosen row; ms_per_step the last class's best. */
m2cg_status m2cg_ensemble_autotune_tiles(m2cg_ensemble* ens, int32_t steps, int32_t n_shapes,
                                         const int32_t* shapes, int32_t* member_shape, float* ms_per_step);

/* ---- timing on the context stream -------------------------------------- */
m2cg_status m2cg_sync(m2cg_ctx* ctx);
/* Records CUDA event `slot` (0..15) on the context stream. */
m2cg_status m2cg_event_record(m2cg_ctx* ctx, int32_t slot);
/* Milliseconds between two recorded events (synchronizes on the second). */
m2cg_status m2cg_event_elapsed(m2cg_ctx* ctx, int32_t slot0, int32_t slot1, float* ms);
/* Runs n_steps CFL-driven steps launch by launch with a CUDA event pair around
 * every kernel and returns the summed device milliseconds per phase:
 * [0] dt reduction, [1] interface compaction, [2] reconstruction, [3] face fluxes,
 * [4] interface Riemann solves (first, budgeted pass), [5] residual gather +
 * stage update, [6] boundary conditions, [7] end-of-step material update,
 * [8] interface Riemann solves that outlasted the first pass (these run
 * concurrently with [2] and [3], so the phases overlap in time). */
#define M2CG_N_PHASES 9
m2cg_status m2cg_phase_times(m2cg_ctx* ctx, int32_t n_steps, double ms[M2CG_N_PHASES]);
/* Kernel launches issued on this context since creation (all kernels are this library's). */
int64_t     m2cg_kernel_launches(m2cg_ctx* ctx);
/* No reference counterpart (measurement helper): binary64 FMA throughput of
 * this GPU -- eight independent FMA chains per thread, 8 blocks of 256 threads
 * per SM, `iters` FMAs per chain (1 .. 2^22) -- in thread-level FMAs per second;
 * ms (optional) receives the timed kernel's duration.  The FP64-pipe roofline's
 * denominator. */
m2cg_status m2cg_fp64_peak(int32_t iters, double* dfma_per_s, float* ms);
/* No reference counterpart (self-check of the device solver's arithmetic): the
 * exact interface Riemann solver divides several numerators by one divisor
 * through a shared, correctly rounded reciprocal (Markstein's method), which
 * must give IEEE a / b bit for bit.  This runs that code on n (1 .. 2^36)
 * operand pairs drawn from `seed` -- random bit patterns, wide and physical
 * exponent ranges, all-ones significands, zeros, subnormals, infinities, NaNs,
 * exponent-limit quotients, exact quotients -- and compares each quotient with
 * a / b and each reciprocal it forms with 1 / b.  mismatches receives the number
 * of differing results (0 expected); fast (optional) the number of quotients
 * that took the shared-reciprocal path rather than the IEEE fallback. */
m2cg_status m2cg_selftest_quotient(int64_t n, uint64_t seed, int64_t* mismatches, int64_t* fast);
/* Page-locked host memory for fast upload / download (NULL on failure). */
void*       m2cg_host_alloc(size_t bytes);
void        m2cg_host_free(void* ptr);

#ifdef __cplusplus
}
#endif
#endif /* M2CG_H */
