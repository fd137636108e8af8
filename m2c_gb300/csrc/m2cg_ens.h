// Per-member argument records of the batched (m2cg_ensemble) launches: one
// record per member domain, read by block row blockIdx.y; the fields are the
// single-domain kernels' arguments.
#pragma once
#include "m2cg_internal.h"

namespace m2cg {

struct k_reconstruct_args {
  Params P;
  StateSet S;
  const int32_t* id;
  double* const* fs;
  unsigned long long* cnt;
};
struct k_reconstruct_ghosts_args {
  Params P;
  StateSet S;
  const int32_t* id;
  double* const* fs;
  unsigned long long* cnt;
};
struct k_face_flux_args {
  Params P;
  const int32_t* id;
  double* const* fs;
  double* const* F;
  unsigned long long* cnt;
};
struct k_update_args {
  Params P;
  StageArgs A;
  const int32_t* id;
  int32_t* id_new;
  double* const* F;
  IfaceList L;
  const DevScalars* sc;
  int64_t* swept;
  unsigned long long* swept_count;
  int64_t swept_cap;
  unsigned long long* cnt;
};
struct k_bc_args {
  Params P;
  StateSet S;
  int do_v;
  int do_phi;
  int32_t* id;
  const DevScalars* sc;
};
struct k_dt_reduce_args {
  Params P;
  StateSet S;
  const int32_t* id;
  DevScalars* sc;
};
struct k_dt_finalize_args {
  Params P;
  DevScalars* sc;
  int mode;
  double fixed_dt;
};
struct k_resolve_remaining_args {
  Params P;
  int32_t* id_new;
  const int64_t* swept;
  const unsigned long long* count;
  int64_t cap;
  int32_t* cand_out;
  int final_pass;
  const DevScalars* sc;
};
struct k_commit_remaining_args {
  int32_t* id_new;
  const int64_t* swept;
  const unsigned long long* count;
  int64_t cap;
  const int32_t* cand;
  const DevScalars* sc;
};
struct k_swept_update_args {
  Params P;
  StateSet S;
  const int32_t* id_old;
  const int32_t* id_new;
  IfaceList L;
  const int64_t* swept;
  const unsigned long long* count;
  int64_t cap;
  unsigned long long* cnt;
  const DevScalars* sc;
};
struct k_commit_ids_args {
  int32_t* id;
  const int32_t* id_new;
  const int64_t* swept;
  const unsigned long long* count;
  int64_t cap;
  const DevScalars* sc;
};
struct k_compact_interfaces_args {
  Params P;
  const int32_t* id;
  IfaceList L;
  unsigned long long* cnt;
  const DevScalars* sc;
};

struct RiemannEnsArgs {
  Params P;
  const Mats* md;
  StateSet S;
  const int32_t* id;
  double* const* fs;
  IfaceList L;
  int store;
  const float* warm;
  unsigned long long* cnt;
  const DevScalars* sc;
};

struct CounterResetArgs {
  unsigned long long* a;
  unsigned long long* b;
};

}  // namespace m2cg
