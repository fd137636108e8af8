// Learned warm start for the exact two-material Riemann solve: a
// 16 -> 64 -> 64 -> 64 -> 1 SiLU MLP that predicts the star pressure from the
// two states and their EOS parameters.  The exact solver starts from a pair
// bracketing the prediction (in place of the acoustic pair,
// ExactRiemannSolverBase.cpp:1107-1158) and still converges to the same
// tolerance, so its answer, not the prediction, is the result.
//
// The three 64-wide layers run on the tensor cores: tcgen05.mma with BF16
// operands staged in shared memory and FP32 accumulators in tensor memory, one
// 128-row tile per CTA pass.  The scalar head (64 -> 1), biases, SiLU, the
// loss and Adam run on the CUDA cores in FP32.  Training runs forward and
// backward for a tile in one kernel, keeping the three pre-activations in
// TMEM for the backward pass, and accumulates the weight gradients with FP32
// atomics; Adam then updates the FP32 master weights and k_pack_bf16 writes
// the BF16 copies the GEMMs read.
//
// Inputs are dimensionless groups of the two states relative to the
// impedance-weighted pressure p_ref = (C_r p_l + C_l p_r) / (C_l + C_r), with
// c^2 = gamma (p + pc) / (rho (1 - b rho)) and C = rho c (12 used, padded to 16):
//   asinh(a) / 4 with a = (u_l - u_r) C_l C_r / ((C_l + C_r) p_ref), the
//     acoustic pressure jump;
//   ln(p_l / p_ref) / 4, ln(p_r / p_ref) / 4, ln(C_l / C_r) / 4;
//   (gamma_s - 4) / 1.7, asinh(pc_s / p_ref) / 8, 2 b_s rho_s - 1,
//     ln(rho_s c_s^2 / p_ref) / 4 for each side s.
// Target: t = ln(p* / p_ref) / 4, i.e. p* = p_ref exp(4 t).  (Pressures below
// 1 Pa enter the inputs as 1 Pa.)
#include <cstdio>
#include <cstring>
#include <cmath>
#include <vector>
#include <random>
#include <algorithm>
#include "m2cg_internal.h"
#include "m2cg_umma.cuh"

void m2cg_set_error(const char* fmt, ...);

#define MCK(call)                                                                                  \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) {                                                                       \
      m2cg_set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
      return M2CG_ERR_CUDA;                                                                        \
    }                                                                                              \
  } while (0)

namespace m2cg {
namespace mlp {

constexpr int NF = M2CG_MLP_FEATURES;  // 16
constexpr int NH = 64;
constexpr int TILE = 128;
// flat FP32 parameter vector: W1 [64][16], b1, W2 [64][64], b2, W3 [64][64], b3, w4 [64], b4
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + NH * NF, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH,
              OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + NH * NH, OFF_W4 = OFF_B3 + NH, OFF_B4 = OFF_W4 + NH,
              NPARAM = OFF_B4 + 1;
static_assert(NPARAM == M2CG_MLP_PARAMS, "parameter count");
// BF16 GEMM operands: W1f [64][16], W2f, W3f [64][64] (out x in, the forward
// B operands) and W2b, W3b [64][64] (in x out, the backward B operands)
constexpr int BF_W1F = 0, BF_W2F = BF_W1F + NH * NF, BF_W3F = BF_W2F + NH * NH, BF_W2B = BF_W3F + NH * NH,
              BF_W3B = BF_W2B + NH * NH, NBF = BF_W3B + NH * NH;

constexpr long long MAX_POLLS = 1ll << 26;  // mbarrier wait limit (the MMAs take microseconds)

// shared-memory layout of the tile kernels (byte offsets, 1024-aligned)
constexpr int S_W1F = 0, S_W2F = S_W1F + 2048, S_W3F = S_W2F + 8192, S_W2B = S_W3F + 8192, S_W3B = S_W2B + 8192,
              S_XA = S_W3B + 8192, S_H1A = S_XA + 4096, S_H2A = S_H1A + 16384, S_HT = S_H2A + 16384,
              S_DZA = S_HT + 32768, S_DZT = S_DZA + 16384, S_F32 = S_DZT + 16384,
              // fp32: b1 b2 b3 w4 (4 x 64), reductions db1 db2 db3 dw4 (4 x 64), b4, loss, db4
              S_END = S_F32 + (8 * 64 + 4) * 4;
constexpr int SMEM_FWD = S_H2A + 16384 + (8 * 64 + 4) * 4;  // forward: weights, Xa, H1a, H2a (+ floats)
constexpr int SMEM_TRAIN = S_END;

__device__ __forceinline__ float silu(float z) { return z / (1.0f + expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
  float s = 1.0f / (1.0f + expf(-z));
  return s * (1.0f + z * (1.0f - s));
}
__device__ __forceinline__ void st_bf16(unsigned char* base, uint32_t off, float v) {
  *reinterpret_cast<__nv_bfloat16*>(base + off) = __float2bfloat16_rn(v);
}

// ---- features ---------------------------------------------------------------
// f[0..15] and p_ref of one problem: states (rho, u, p) per side, EOS rows
// {type, gamma, pc, b, q}.
__device__ double problem_features(double rl, double ul, double pl, const double* el, double rr, double ur,
                                   double pr, const double* er, float* f) {
  pl = fmax(pl, 1.0);
  pr = fmax(pr, 1.0);
  double c2l = el[1] * (pl + el[2]) / (rl * (1.0 - el[3] * rl));
  double c2r = er[1] * (pr + er[2]) / (rr * (1.0 - er[3] * rr));
  c2l = c2l > 0.0 ? c2l : 1.0;
  c2r = c2r > 0.0 ? c2r : 1.0;
  double Cl = rl * sqrt(c2l), Cr = rr * sqrt(c2r);
  double pref = (Cr * pl + Cl * pr) / (Cl + Cr);
  double a = (ul - ur) * Cl * Cr / ((Cl + Cr) * pref);
  f[0] = (float)(asinh(a) * 0.25);
  f[1] = (float)(log(pl / pref) * 0.25);
  f[2] = (float)(log(pr / pref) * 0.25);
  f[3] = (float)(log(Cl / Cr) * 0.25);
  f[4] = (float)((el[1] - 4.0) / 1.7);
  f[5] = (float)((er[1] - 4.0) / 1.7);
  f[6] = (float)(asinh(el[2] / pref) * 0.125);
  f[7] = (float)(asinh(er[2] / pref) * 0.125);
  f[8] = (float)(2.0 * el[3] * rl - 1.0);
  f[9] = (float)(2.0 * er[3] * rr - 1.0);
  f[10] = (float)(log(rl * c2l / pref) * 0.25);
  f[11] = (float)(log(rr * c2r / pref) * 0.25);
  for (int i = 12; i < NF; i++) f[i] = 0.f;
  return pref;
}

// 1D problems: W rows {rho_l, u_l, p_l, rho_r, u_r, p_r}, E rows {type, gamma,
// pc, b, q} x 2.  X: n x 16 bf16; pref: n; t (optional): targets from pstar.
__global__ void k_features(int64_t n, const double* __restrict__ W, const double* __restrict__ E,
                           const double* __restrict__ pstar, __nv_bfloat16* X, float* pref, float* t) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const double* w = &W[q * 6];
  float f[NF];
  double pr = problem_features(w[0], w[1], w[2], &E[q * 10], w[3], w[4], w[5], &E[q * 10 + 5], f);
  for (int i = 0; i < NF; i++) X[q * NF + i] = __float2bfloat16_rn(f[i]);
  if (pref) pref[q] = (float)pr;
  if (t && pstar) t[q] = (float)(log(fmax(pstar[q], 1e-300) / pr) * 0.25);
}

// Interface faces of the finite-volume step: inputs as the interface solve
// reads them (cell-centre states, Constant reconstruction at the interface),
// normal velocity along the face's axis.
__global__ void k_features_faces(Params P, StateSet S, const int32_t* __restrict__ id, const IfaceList L,
                                 __nv_bfloat16* X, float* pref, const DevScalars* sc) {
  if (sc && !sc->active) return;
  int64_t n = (int64_t)min((unsigned long long)L.cap, *L.count);
  const int64_t st[3] = {1, P.g.sy, P.g.sz};
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
    int64_t fc = L.face[s];
    int d = (int)(fc & 3);
    int64_t c = fc >> 2, m = c - st[d];
    const DevMat& ML = P.mats.m[id[m]];
    const DevMat& MR = P.mats.m[id[c]];
    double el[5] = {(double)ML.type, ML.gam, ML.Pstiff, ML.type == M2CG_EOS_NASG ? ML.b : 0.0, 0.0};
    double er[5] = {(double)MR.type, MR.gam, MR.Pstiff, MR.type == M2CG_EOS_NASG ? MR.b : 0.0, 0.0};
    float f[NF];
    double pr = problem_features(S.q[0][m], S.q[1 + d][m], S.q[4][m], el, S.q[0][c], S.q[1 + d][c], S.q[4][c], er, f);
    for (int i = 0; i < NF; i++) X[s * NF + i] = __float2bfloat16_rn(f[i]);
    pref[s] = (float)pr;
  }
}

// Network output -> starting pressure p_ref exp(4 t) (0 = no warm start).
__global__ void k_to_pressure(int64_t n, const float* __restrict__ t, const float* __restrict__ pref, double* pd,
                              float* pf, const DevScalars* sc, const unsigned long long* count) {
  if (sc && !sc->active) return;
  if (count) n = min((unsigned long long)n, *count);
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    double p = (double)pref[q] * exp(4.0 * (double)t[q]);
    if (!(p > 0.0) || !(p < 1e300)) p = 0.0;
    if (pd) pd[q] = p;
    if (pf) pf[q] = (float)p;
  }
}

// ---- tile machinery -----------------------------------------------------------
struct TileCtx {
  unsigned char* sm;
  float* f32;  // b1 b2 b3 w4 | db1 db2 db3 dw4 | b4, loss, db4
  uint64_t* bar;
  uint32_t tm;
  uint32_t phase;
  bool ok;
};

__device__ void load_weights(TileCtx& c, const __nv_bfloat16* __restrict__ wbf, const float* __restrict__ prm,
                             bool backward) {
  int t = threadIdx.x;
  for (int i = t; i < NH * NF; i += blockDim.x) {
    int n = i / NF, k = i % NF;
    *reinterpret_cast<__nv_bfloat16*>(c.sm + S_W1F + umma::kmajor_offset(n, k, NF)) = wbf[BF_W1F + i];
  }
  for (int i = t; i < NH * NH; i += blockDim.x) {
    int n = i / NH, k = i % NH;
    uint32_t o = umma::kmajor_offset(n, k, NH);
    *reinterpret_cast<__nv_bfloat16*>(c.sm + S_W2F + o) = wbf[BF_W2F + i];
    *reinterpret_cast<__nv_bfloat16*>(c.sm + S_W3F + o) = wbf[BF_W3F + i];
    if (backward) {
      *reinterpret_cast<__nv_bfloat16*>(c.sm + S_W2B + o) = wbf[BF_W2B + i];
      *reinterpret_cast<__nv_bfloat16*>(c.sm + S_W3B + o) = wbf[BF_W3B + i];
    }
  }
  for (int i = t; i < NH; i += blockDim.x) {
    c.f32[i] = prm[OFF_B1 + i];
    c.f32[64 + i] = prm[OFF_B2 + i];
    c.f32[128 + i] = prm[OFF_B3 + i];
    c.f32[192 + i] = prm[OFF_W4 + i];
  }
  if (t == 0) c.f32[512] = prm[OFF_B4];
}

// Orders generic shared-memory writes before MMAs issued after the barrier,
// and TMEM reads before MMAs that overwrite the same columns.
__device__ __forceinline__ void sync_for_mma() {
  umma::fence_async_smem();
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
}

__device__ __forceinline__ void commit_wait(TileCtx& c) {
  if (threadIdx.x == 0) umma::mma_commit(c.bar);
  bool ok = umma::mbar_wait(c.bar, c.phase, MAX_POLLS);
  c.phase ^= 1u;
  c.ok = __syncthreads_and(ok) && c.ok;
  umma::fence_after_sync();
}

// TMEM address of this thread's row (lane) at column col.
__device__ __forceinline__ uint32_t trow(const TileCtx& c, int col) {
  return c.tm + ((uint32_t)(threadIdx.x & ~31) << 16) + (uint32_t)col;
}

// Layer epilogue: H = bf16(SiLU(acc + bias)) into an A tile (K = 64).
__device__ void epilogue_silu(const TileCtx& c, int col, const float* bias, unsigned char* dst) {
  const int r = threadIdx.x;
  for (int j0 = 0; j0 < NH; j0 += 16) {
    float v[16];
    umma::tmem_ld16(trow(c, col + j0), v);
#pragma unroll
    for (int i = 0; i < 16; i++) st_bf16(dst, umma::kmajor_offset(r, j0 + i, NH), silu(v[i] + bias[j0 + i]));
  }
}

// Forward through the three GEMM layers for the tile already in S_XA; leaves
// Z1..Z3 accumulators (bias not added) in TMEM columns 0, 64, 128.
__device__ void forward_tile(TileCtx& c) {
  sync_for_mma();
  if (threadIdx.x == 0) umma::gemm_128xN(c.tm + 0, c.sm + S_XA, c.sm + S_W1F, NH, NF, false);
  commit_wait(c);
  epilogue_silu(c, 0, c.f32 + 0, c.sm + S_H1A);
  sync_for_mma();
  if (threadIdx.x == 0) umma::gemm_128xN(c.tm + 64, c.sm + S_H1A, c.sm + S_W2F, NH, NH, false);
  commit_wait(c);
  epilogue_silu(c, 64, c.f32 + 64, c.sm + S_H2A);
  sync_for_mma();
  if (threadIdx.x == 0) umma::gemm_128xN(c.tm + 128, c.sm + S_H2A, c.sm + S_W3F, NH, NH, false);
  commit_wait(c);
}

// Scalar head on the CUDA cores: out = b4 + sum_j SiLU(z3_j + b3_j) w4_j.
__device__ float head(const TileCtx& c) {
  float out = c.f32[512];
  for (int j0 = 0; j0 < NH; j0 += 16) {
    float v[16];
    umma::tmem_ld16(trow(c, 128 + j0), v);
#pragma unroll
    for (int i = 0; i < 16; i++) out += silu(v[i] + c.f32[128 + j0 + i]) * c.f32[192 + j0 + i];
  }
  return out;
}

__device__ void load_x_row(TileCtx& c, const __nv_bfloat16* __restrict__ X, int64_t row, bool valid) {
  const int r = threadIdx.x;
  for (int k = 0; k < NF; k++) {
    __nv_bfloat16 v = valid ? X[row * NF + k] : __float2bfloat16_rn(0.f);
    *reinterpret_cast<__nv_bfloat16*>(c.sm + S_XA + umma::kmajor_offset(r, k, NF)) = v;
  }
}

__device__ void tile_setup(TileCtx& c, unsigned char* sm, uint64_t* bar, uint32_t* tslot) {
  c.sm = sm;
  c.bar = bar;
  c.phase = 0;
  c.ok = true;
  if (threadIdx.x == 0) umma::mbar_init(bar, 1);
  if (threadIdx.x < 32) umma::tmem_alloc(tslot, 256);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  c.tm = *tslot;
}

__device__ void tile_teardown(TileCtx& c) {
  umma::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) umma::tmem_dealloc(c.tm, 256);
}

// ---- inference ----------------------------------------------------------------
// Persistent: CTA b handles tiles b, b + grid, ...  out[row] = network output.
// rows = min(n, *count) when count is given (the device-side interface count).
__global__ void __launch_bounds__(TILE, 1) k_forward(int64_t n, const unsigned long long* count,
                                                      const __nv_bfloat16* __restrict__ X,
                                                      const __nv_bfloat16* __restrict__ wbf,
                                                      const float* __restrict__ prm, float* out, int* err,
                                                      const DevScalars* sc) {
  if (sc && !sc->active) return;
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tslot;
  if (count) n = (int64_t)min((unsigned long long)n, *count);
  int64_t ntiles = (n + TILE - 1) / TILE;
  if ((int64_t)blockIdx.x >= ntiles) return;
  TileCtx c;
  c.f32 = reinterpret_cast<float*>(sm + SMEM_FWD - (8 * 64 + 4) * 4);
  tile_setup(c, sm, &bar, &tslot);
  load_weights(c, wbf, prm, false);
  for (int64_t tile = blockIdx.x; tile < ntiles && c.ok; tile += gridDim.x) {
    int64_t row = tile * TILE + threadIdx.x;
    load_x_row(c, X, row, row < n);
    forward_tile(c);
    float o = head(c);
    if (row < n) out[row] = o;
    umma::fence_before_sync();
    __syncthreads();  // TMEM reads done before the next tile's MMAs
    umma::fence_after_sync();
  }
  if (!c.ok && threadIdx.x == 0) atomicExch(err, 1);
  tile_teardown(c);
}

// ---- training -------------------------------------------------------------------
// Warp-reduce v over the 32 rows of this warp, then add into s[j] (shared).
__device__ __forceinline__ void col_reduce_add(float* s, int j, float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(&s[j], v);
}

// dZ (fp32, per row) -> bf16 A tile dZa [row][j] and B tile dZT [j][row].
__device__ __forceinline__ void store_dz(const TileCtx& c, int j, float dz) {
  const int r = threadIdx.x;
  st_bf16(c.sm + S_DZA, umma::kmajor_offset(r, j, NH), dz);
  st_bf16(c.sm + S_DZT, umma::kmajor_offset(j, r, TILE), dz);
}

// Weight-gradient readout: TMEM columns 192..255 hold D[i][j] for input
// feature i = row (< n_in); grad[off + j * n_in + i] += D[i][j].
__device__ void dw_readout(const TileCtx& c, float* grad, int off, int n_in) {
  const int i = threadIdx.x;
  if ((threadIdx.x >> 5) * 32 >= n_in) return;  // warp-uniform: no rows of interest in this warp
  for (int j0 = 0; j0 < NH; j0 += 16) {
    float v[16];
    umma::tmem_ld16(trow(c, 192 + j0), v);
    if (i < n_in) {
#pragma unroll
      for (int q = 0; q < 16; q++) atomicAdd(&grad[off + (j0 + q) * n_in + i], v[q]);
    }
  }
}

// One 128-row tile of the batch: forward, squared-error loss on the target,
// backward; gradients (of the mean loss over the batch) and the loss sum are
// accumulated into grad[] and loss[0].
__global__ void __launch_bounds__(TILE, 1) k_train(int64_t batch, const int32_t* __restrict__ idx,
                                                    const __nv_bfloat16* __restrict__ X, const float* __restrict__ y,
                                                    const __nv_bfloat16* __restrict__ wbf,
                                                    const float* __restrict__ prm, float* grad, float* loss,
                                                    int* err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tslot;
  TileCtx c;
  c.f32 = reinterpret_cast<float*>(sm + S_F32);
  const int r = threadIdx.x;
  const int64_t brow = (int64_t)blockIdx.x * TILE + r;
  const bool valid = brow < batch;
  const int64_t row = valid ? (idx ? (int64_t)idx[brow] : brow) : 0;
  tile_setup(c, sm, &bar, &tslot);
  load_weights(c, wbf, prm, true);
  for (int i = r; i < 4 * 64; i += TILE) c.f32[256 + i] = 0.f;  // reductions db1 db2 db3 dw4
  if (r == 0) { c.f32[513] = 0.f; c.f32[514] = 0.f; }             // loss, db4 (f32[512] holds b4)
  // HT rows 64..127 (padding of the feature dimension) stay zero
  for (int i = r; i < 32768 / 4; i += TILE) reinterpret_cast<uint32_t*>(sm + S_HT)[i] = 0u;
  load_x_row(c, X, row, valid);
  forward_tile(c);
  // head, loss and dOut
  float out = head(c);
  float d = 0.f;
  if (valid) {
    float e = out - y[row];
    d = 2.f * e / (float)batch;
    atomicAdd(&c.f32[513], e * e);
    atomicAdd(&c.f32[514], d);
  }
  float* sdb1 = c.f32 + 256;
  float* sdb2 = c.f32 + 320;
  float* sdb3 = c.f32 + 384;
  float* sdw4 = c.f32 + 448;
  // layer 3: dZ3 = d w4 SiLU'(z3); dw4 = sum d h3; H2^T into HT
  for (int j0 = 0; j0 < NH; j0 += 16) {
    float v[16];
    umma::tmem_ld16(trow(c, 128 + j0), v);
#pragma unroll
    for (int q = 0; q < 16; q++) {
      int j = j0 + q;
      float z = v[q] + c.f32[128 + j];
      float dz = d * c.f32[192 + j] * dsilu(z);
      store_dz(c, j, dz);
      col_reduce_add(sdb3, j, dz);
      col_reduce_add(sdw4, j, d * silu(z));
    }
  }
  for (int i = 0; i < NH; i++)
    *reinterpret_cast<__nv_bfloat16*>(sm + S_HT + umma::kmajor_offset(i, r, TILE)) =
        *reinterpret_cast<const __nv_bfloat16*>(sm + S_H2A + umma::kmajor_offset(r, i, NH));
  sync_for_mma();
  if (r == 0) {
    umma::gemm_128xN(c.tm + 192, sm + S_HT, sm + S_DZT, NH, TILE, false);  // dW3[i][j]
    umma::gemm_128xN(c.tm + 128, sm + S_DZA, sm + S_W3B, NH, NH, false);  // dH2[r][i]
  }
  commit_wait(c);
  dw_readout(c, grad, OFF_W3, NH);
  // layer 2: dZ2 = dH2 SiLU'(z2); H1^T into HT
  for (int j0 = 0; j0 < NH; j0 += 16) {
    float g[16], v[16];
    umma::tmem_ld16(trow(c, 128 + j0), g);
    umma::tmem_ld16(trow(c, 64 + j0), v);
#pragma unroll
    for (int q = 0; q < 16; q++) {
      int j = j0 + q;
      float dz = g[q] * dsilu(v[q] + c.f32[64 + j]);
      store_dz(c, j, dz);
      col_reduce_add(sdb2, j, dz);
    }
  }
  for (int i = 0; i < NH; i++)
    *reinterpret_cast<__nv_bfloat16*>(sm + S_HT + umma::kmajor_offset(i, r, TILE)) =
        *reinterpret_cast<const __nv_bfloat16*>(sm + S_H1A + umma::kmajor_offset(r, i, NH));
  sync_for_mma();
  if (r == 0) {
    umma::gemm_128xN(c.tm + 192, sm + S_HT, sm + S_DZT, NH, TILE, false);  // dW2
    umma::gemm_128xN(c.tm + 64, sm + S_DZA, sm + S_W2B, NH, NH, false);   // dH1
  }
  commit_wait(c);
  dw_readout(c, grad, OFF_W2, NH);
  // layer 1: dZ1 = dH1 SiLU'(z1); X^T into HT (feature rows 16..63 zeroed)
  for (int j0 = 0; j0 < NH; j0 += 16) {
    float g[16], v[16];
    umma::tmem_ld16(trow(c, 64 + j0), g);
    umma::tmem_ld16(trow(c, 0 + j0), v);
#pragma unroll
    for (int q = 0; q < 16; q++) {
      int j = j0 + q;
      float dz = g[q] * dsilu(v[q] + c.f32[j]);
      st_bf16(sm + S_DZT, umma::kmajor_offset(j, r, TILE), dz);
      col_reduce_add(sdb1, j, dz);
    }
  }
  for (int i = 0; i < NH; i++) {
    __nv_bfloat16 v = (i < NF) ? *reinterpret_cast<const __nv_bfloat16*>(sm + S_XA + umma::kmajor_offset(r, i, NF))
                               : __float2bfloat16_rn(0.f);
    *reinterpret_cast<__nv_bfloat16*>(sm + S_HT + umma::kmajor_offset(i, r, TILE)) = v;
  }
  sync_for_mma();
  if (r == 0) umma::gemm_128xN(c.tm + 192, sm + S_HT, sm + S_DZT, NH, TILE, false);  // dW1
  commit_wait(c);
  dw_readout(c, grad, OFF_W1, NF);
  __syncthreads();
  if (r < NH) {
    atomicAdd(&grad[OFF_B1 + r], sdb1[r]);
    atomicAdd(&grad[OFF_B2 + r], sdb2[r]);
    atomicAdd(&grad[OFF_B3 + r], sdb3[r]);
    atomicAdd(&grad[OFF_W4 + r], sdw4[r]);
  }
  if (r == 0) {
    atomicAdd(&grad[OFF_B4], c.f32[514]);
    atomicAdd(loss, c.f32[513]);
    if (!c.ok) atomicExch(err, 1);
  }
  tile_teardown(c);
}

// Adam on the FP32 master weights; clears the gradient.  bc1 = 1 - beta1^step,
// bc2 = 1 - beta2^step.  k_pack_bf16 then refreshes the BF16 GEMM copies.
__global__ void k_adam(float* prm, float* grad, float* m, float* v, float lr, float b1, float b2, float eps, float bc1,
                       float bc2) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NPARAM) return;
  float g = grad[i];
  float mi = b1 * m[i] + (1.f - b1) * g;
  float vi = b2 * v[i] + (1.f - b2) * g * g;
  m[i] = mi;
  v[i] = vi;
  prm[i] = prm[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  grad[i] = 0.f;
}

// BF16 copies of the three GEMM weight matrices (forward and transposed).
__global__ void k_pack_bf16(const float* __restrict__ prm, __nv_bfloat16* wbf) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < NH * NF) wbf[BF_W1F + i] = __float2bfloat16_rn(prm[OFF_W1 + i]);
  if (i < NH * NH) {
    int o = i / NH, in = i % NH;  // W[o][in]
    __nv_bfloat16 w2 = __float2bfloat16_rn(prm[OFF_W2 + i]), w3 = __float2bfloat16_rn(prm[OFF_W3 + i]);
    wbf[BF_W2F + i] = w2;
    wbf[BF_W3F + i] = w3;
    wbf[BF_W2B + in * NH + o] = w2;
    wbf[BF_W3B + in * NH + o] = w3;
  }
}

}  // namespace mlp
}  // namespace m2cg

using namespace m2cg;
using namespace m2cg::mlp;

struct m2cg_mlp {
  cudaStream_t stream = nullptr;
  int nsm = 0;
  float* prm = nullptr;  // FP32 master weights
  float* grad = nullptr;
  float* adam_m = nullptr;
  float* adam_v = nullptr;
  __nv_bfloat16* wbf = nullptr;
  float* loss = nullptr;
  int* err = nullptr;
  int64_t step = 0;
  // training set on the device
  int64_t n_data = 0;
  __nv_bfloat16* X = nullptr;
  float* y = nullptr;
  int32_t* perm = nullptr;
};

namespace {
m2cg_status mlp_check(m2cg_mlp* m) {
  int herr = 0;
  MCK(cudaMemcpyAsync(&herr, m->err, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
  MCK(cudaStreamSynchronize(m->stream));
  if (herr) {
    m2cg_set_error("MLP kernel: tensor-core completion wait timed out");
    return M2CG_ERR_CUDA;
  }
  return M2CG_OK;
}
cudaError_t mlp_set_smem() {
  static bool done = false;
  if (done) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(k_train, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_TRAIN);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_FWD);
  done = (e == cudaSuccess);
  return e;
}
}  // namespace

extern "C" {

m2cg_status m2cg_mlp_create(uint64_t seed, m2cg_mlp** out) {
  if (!out) { m2cg_set_error("null argument"); return M2CG_ERR_INVALID_ARG; }
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { m2cg_set_error("no CUDA device"); return M2CG_ERR_NO_DEVICE; }
  m2cg_mlp* m = new m2cg_mlp();
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&m->nsm, cudaDevAttrMultiProcessorCount, dev);
  if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&m->prm, NPARAM * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&m->grad, NPARAM * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&m->adam_m, NPARAM * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&m->adam_v, NPARAM * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&m->wbf, NBF * sizeof(__nv_bfloat16)) != cudaSuccess ||
      cudaMalloc(&m->loss, sizeof(float)) != cudaSuccess || cudaMalloc(&m->err, sizeof(int)) != cudaSuccess ||
      mlp_set_smem() != cudaSuccess) {
    m2cg_set_error("MLP allocation failed: %s", cudaGetErrorString(cudaGetLastError()));
    m2cg_mlp_destroy(m);
    return M2CG_ERR_CUDA;
  }
  // He-uniform initial weights for the SiLU layers, zero biases
  std::vector<float> h(NPARAM, 0.f);
  std::mt19937_64 rng(seed);
  auto fill = [&](int off, int fan_out, int fan_in) {
    float a = std::sqrt(6.0f / (float)fan_in);
    std::uniform_real_distribution<float> u(-a, a);
    for (int i = 0; i < fan_out * fan_in; i++) h[off + i] = u(rng);
  };
  fill(OFF_W1, NH, NF);
  for (int o = 0; o < NH; o++)
    for (int k = 12; k < NF; k++) h[OFF_W1 + o * NF + k] = 0.f;  // 12 of the 16 inputs are used
  fill(OFF_W2, NH, NH);
  fill(OFF_W3, NH, NH);
  fill(OFF_W4, 1, NH);
  for (int i = 0; i < NH; i++) h[OFF_W4 + i] *= 0.5f;
  m2cg_status st = m2cg_mlp_set_params(m, h.data());
  if (st != M2CG_OK) { m2cg_mlp_destroy(m); return st; }
  *out = m;
  return M2CG_OK;
}

void m2cg_mlp_destroy(m2cg_mlp* m) {
  if (!m) return;
  if (m->stream) cudaStreamSynchronize(m->stream);
  for (void* p : {(void*)m->prm, (void*)m->grad, (void*)m->adam_m, (void*)m->adam_v, (void*)m->wbf, (void*)m->loss,
                  (void*)m->err, (void*)m->X, (void*)m->y, (void*)m->perm})
    if (p) cudaFree(p);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
}

m2cg_status m2cg_mlp_set_params(m2cg_mlp* m, const float* params) {
  if (!m || !params) { m2cg_set_error("null argument"); return M2CG_ERR_INVALID_ARG; }
  MCK(cudaMemcpyAsync(m->prm, params, NPARAM * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  MCK(cudaMemsetAsync(m->grad, 0, NPARAM * sizeof(float), m->stream));
  MCK(cudaMemsetAsync(m->adam_m, 0, NPARAM * sizeof(float), m->stream));
  MCK(cudaMemsetAsync(m->adam_v, 0, NPARAM * sizeof(float), m->stream));
  MCK(cudaMemsetAsync(m->err, 0, sizeof(int), m->stream));
  k_pack_bf16<<<(NH * NH + 255) / 256, 256, 0, m->stream>>>(m->prm, m->wbf);
  MCK(cudaGetLastError());
  m->step = 0;
  MCK(cudaStreamSynchronize(m->stream));
  return M2CG_OK;
}

m2cg_status m2cg_mlp_adam_step(m2cg_mlp* m, const float* grad, float lr) {
  if (!m || !grad || !(lr > 0.f)) { m2cg_set_error("null argument or non-positive rate"); return M2CG_ERR_INVALID_ARG; }
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;   // as m2cg_mlp_train
  MCK(cudaMemcpyAsync(m->grad, grad, NPARAM * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  m->step++;
  const float bc1 = 1.f - std::pow(b1, (float)m->step), bc2 = 1.f - std::pow(b2, (float)m->step);
  k_adam<<<(NPARAM + 255) / 256, 256, 0, m->stream>>>(m->prm, m->grad, m->adam_m, m->adam_v, lr, b1, b2, eps, bc1, bc2);
  k_pack_bf16<<<(NH * NH + 255) / 256, 256, 0, m->stream>>>(m->prm, m->wbf);
  MCK(cudaGetLastError());
  MCK(cudaStreamSynchronize(m->stream));
  return M2CG_OK;
}

m2cg_status m2cg_mlp_get_params(m2cg_mlp* m, float* params) {
  if (!m || !params) { m2cg_set_error("null argument"); return M2CG_ERR_INVALID_ARG; }
  MCK(cudaMemcpyAsync(params, m->prm, NPARAM * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
  MCK(cudaStreamSynchronize(m->stream));
  return M2CG_OK;
}

m2cg_status m2cg_mlp_features(int64_t n, const double* W, const double* eos, const double* pstar, float* X,
                              float* pref, float* t) {
  if (n < 0 || !W || !eos || !X) { m2cg_set_error("null argument"); return M2CG_ERR_INVALID_ARG; }
  if (n == 0) return M2CG_OK;
  double *dW, *dE, *dp = nullptr;
  __nv_bfloat16* dX;
  float *dt = nullptr, *dref;
  MCK(cudaMalloc(&dW, n * 6 * sizeof(double)));
  MCK(cudaMalloc(&dE, n * 10 * sizeof(double)));
  MCK(cudaMalloc(&dX, n * NF * sizeof(__nv_bfloat16)));
  MCK(cudaMalloc(&dref, n * sizeof(float)));
  MCK(cudaMemcpy(dW, W, n * 6 * sizeof(double), cudaMemcpyHostToDevice));
  MCK(cudaMemcpy(dE, eos, n * 10 * sizeof(double), cudaMemcpyHostToDevice));
  if (pstar && t) {
    MCK(cudaMalloc(&dp, n * sizeof(double)));
    MCK(cudaMalloc(&dt, n * sizeof(float)));
    MCK(cudaMemcpy(dp, pstar, n * sizeof(double), cudaMemcpyHostToDevice));
  }
  k_features<<<(unsigned)((n + 255) / 256), 256>>>(n, dW, dE, dp, dX, dref, dt);
  MCK(cudaGetLastError());
  std::vector<__nv_bfloat16> h(n * NF);
  MCK(cudaMemcpy(h.data(), dX, n * NF * sizeof(__nv_bfloat16), cudaMemcpyDeviceToHost));
  for (int64_t i = 0; i < n * NF; i++) X[i] = __bfloat162float(h[i]);
  if (dt) MCK(cudaMemcpy(t, dt, n * sizeof(float), cudaMemcpyDeviceToHost));
  if (pref) MCK(cudaMemcpy(pref, dref, n * sizeof(float), cudaMemcpyDeviceToHost));
  cudaFree(dW); cudaFree(dE); cudaFree(dX); cudaFree(dref);
  if (dp) cudaFree(dp);
  if (dt) cudaFree(dt);
  return M2CG_OK;
}

m2cg_status m2cg_mlp_set_data(m2cg_mlp* m, int64_t n, const double* W, const double* eos, const double* pstar) {
  if (!m || n <= 0 || !W || !eos || !pstar) { m2cg_set_error("null argument or empty set"); return M2CG_ERR_INVALID_ARG; }
  if (n > (int64_t)INT32_MAX) { m2cg_set_error("training set too large"); return M2CG_ERR_CAPACITY; }
  for (void* p : {(void*)m->X, (void*)m->y, (void*)m->perm}) if (p) cudaFree(p);
  m->X = nullptr; m->y = nullptr; m->perm = nullptr;
  double *dW, *dE, *dp;
  MCK(cudaMalloc(&m->X, n * NF * sizeof(__nv_bfloat16)));
  MCK(cudaMalloc(&m->y, n * sizeof(float)));
  MCK(cudaMalloc(&m->perm, n * sizeof(int32_t)));
  MCK(cudaMalloc(&dW, n * 6 * sizeof(double)));
  MCK(cudaMalloc(&dE, n * 10 * sizeof(double)));
  MCK(cudaMalloc(&dp, n * sizeof(double)));
  MCK(cudaMemcpyAsync(dW, W, n * 6 * sizeof(double), cudaMemcpyHostToDevice, m->stream));
  MCK(cudaMemcpyAsync(dE, eos, n * 10 * sizeof(double), cudaMemcpyHostToDevice, m->stream));
  MCK(cudaMemcpyAsync(dp, pstar, n * sizeof(double), cudaMemcpyHostToDevice, m->stream));
  k_features<<<(unsigned)((n + 255) / 256), 256, 0, m->stream>>>(n, dW, dE, dp, m->X, nullptr, m->y);
  MCK(cudaGetLastError());
  MCK(cudaStreamSynchronize(m->stream));
  cudaFree(dW); cudaFree(dE); cudaFree(dp);
  m->n_data = n;
  return M2CG_OK;
}

m2cg_status m2cg_mlp_train(m2cg_mlp* m, int32_t epochs, int32_t batch, float lr, uint64_t seed, float* loss_per_epoch,
                           float* ms) {
  if (!m || epochs < 0 || batch < 1 || !(lr > 0.f)) { m2cg_set_error("bad training arguments"); return M2CG_ERR_INVALID_ARG; }
  if (m->n_data == 0) { m2cg_set_error("no training data (m2cg_mlp_set_data)"); return M2CG_ERR_INVALID_ARG; }
  const int64_t n = m->n_data;
  if (batch > n) batch = (int32_t)n;
  std::vector<int32_t> perm(n);
  for (int64_t i = 0; i < n; i++) perm[i] = (int32_t)i;
  std::mt19937_64 rng(seed);
  cudaEvent_t e0, e1;
  MCK(cudaEventCreate(&e0));
  MCK(cudaEventCreate(&e1));
  MCK(cudaEventRecord(e0, m->stream));
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int ep = 0; ep < epochs; ep++) {
    // cosine decay from lr to lr / 20 over the epochs
    const float lr_ep = lr * (0.05f + 0.95f * 0.5f * (1.f + std::cos(3.14159265f * (float)ep / (float)epochs)));
    std::shuffle(perm.begin(), perm.end(), rng);
    MCK(cudaMemcpyAsync(m->perm, perm.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, m->stream));
    MCK(cudaMemsetAsync(m->loss, 0, sizeof(float), m->stream));
    for (int64_t b0 = 0; b0 + batch <= n; b0 += batch) {  // whole batches only
      k_train<<<(unsigned)((batch + TILE - 1) / TILE), TILE, SMEM_TRAIN, m->stream>>>(
          batch, m->perm + b0, m->X, m->y, m->wbf, m->prm, m->grad, m->loss, m->err);
      m->step++;
      float bc1 = 1.f - std::pow(b1, (float)m->step), bc2 = 1.f - std::pow(b2, (float)m->step);
      k_adam<<<(NPARAM + 255) / 256, 256, 0, m->stream>>>(m->prm, m->grad, m->adam_m, m->adam_v, lr_ep, b1, b2,
                                                          eps, bc1, bc2);
      k_pack_bf16<<<(NH * NH + 255) / 256, 256, 0, m->stream>>>(m->prm, m->wbf);
    }
    MCK(cudaGetLastError());
    if (loss_per_epoch) {
      float l = 0.f;
      MCK(cudaMemcpyAsync(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream));
      MCK(cudaStreamSynchronize(m->stream));
      loss_per_epoch[ep] = l / (float)((n / batch) * batch);
    }
  }
  MCK(cudaEventRecord(e1, m->stream));
  MCK(cudaStreamSynchronize(m->stream));
  if (ms) MCK(cudaEventElapsedTime(ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return mlp_check(m);
}

m2cg_status m2cg_mlp_grad(m2cg_mlp* m, int64_t n, const float* X, const float* t, float* grad, float* loss) {
  if (!m || n <= 0 || !X || !t || !grad) { m2cg_set_error("null argument"); return M2CG_ERR_INVALID_ARG; }
  std::vector<__nv_bfloat16> h(n * NF);
  for (int64_t i = 0; i < n * NF; i++) h[i] = __float2bfloat16_rn(X[i]);
  __nv_bfloat16* dX;
  float* dt;
  MCK(cudaMalloc(&dX, n * NF * sizeof(__nv_bfloat16)));
  MCK(cudaMalloc(&dt, n * sizeof(float)));
  MCK(cudaMemcpyAsync(dX, h.data(), n * NF * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice, m->stream));
  MCK(cudaMemcpyAsync(dt, t, n * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  MCK(cudaMemsetAsync(m->grad, 0, NPARAM * sizeof(float), m->stream));
  MCK(cudaMemsetAsync(m->loss, 0, sizeof(float), m->stream));
  k_train<<<(unsigned)((n + TILE - 1) / TILE), TILE, SMEM_TRAIN, m->stream>>>(n, nullptr, dX, dt, m->wbf, m->prm,
                                                                              m->grad, m->loss, m->err);
  MCK(cudaGetLastError());
  MCK(cudaMemcpyAsync(grad, m->grad, NPARAM * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
  if (loss) MCK(cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream));
  MCK(cudaMemsetAsync(m->grad, 0, NPARAM * sizeof(float), m->stream));
  MCK(cudaStreamSynchronize(m->stream));
  cudaFree(dX);
  cudaFree(dt);
  if (loss) *loss /= (float)n;
  return mlp_check(m);
}

m2cg_status m2cg_mlp_forward(m2cg_mlp* m, int64_t n, const float* X, float* t) {
  if (!m || n < 0 || !X || !t) { m2cg_set_error("null argument"); return M2CG_ERR_INVALID_ARG; }
  if (n == 0) return M2CG_OK;
  std::vector<__nv_bfloat16> h(n * NF);
  for (int64_t i = 0; i < n * NF; i++) h[i] = __float2bfloat16_rn(X[i]);
  __nv_bfloat16* dX;
  float* dt;
  MCK(cudaMalloc(&dX, n * NF * sizeof(__nv_bfloat16)));
  MCK(cudaMalloc(&dt, n * sizeof(float)));
  MCK(cudaMemcpyAsync(dX, h.data(), n * NF * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice, m->stream));
  int64_t ntiles = (n + TILE - 1) / TILE;
  int grid = (int)std::min<int64_t>(ntiles, m->nsm);
  k_forward<<<grid, TILE, SMEM_FWD, m->stream>>>(n, nullptr, dX, m->wbf, m->prm, dt, m->err, nullptr);
  MCK(cudaGetLastError());
  MCK(cudaMemcpyAsync(t, dt, n * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
  MCK(cudaStreamSynchronize(m->stream));
  cudaFree(dX);
  cudaFree(dt);
  return mlp_check(m);
}

m2cg_status m2cg_mlp_predict(m2cg_mlp* m, int64_t n, const double* W, const double* eos, double* p_pred,
                             float* kernel_ms) {
  if (!m || n < 0 || !W || !eos || !p_pred) { m2cg_set_error("null argument"); return M2CG_ERR_INVALID_ARG; }
  if (n == 0) return M2CG_OK;
  double *dW, *dE, *dp;
  __nv_bfloat16* dX;
  float *dt, *dref;
  MCK(cudaMalloc(&dW, n * 6 * sizeof(double)));
  MCK(cudaMalloc(&dE, n * 10 * sizeof(double)));
  MCK(cudaMalloc(&dp, n * sizeof(double)));
  MCK(cudaMalloc(&dX, n * NF * sizeof(__nv_bfloat16)));
  MCK(cudaMalloc(&dt, n * sizeof(float)));
  MCK(cudaMalloc(&dref, n * sizeof(float)));
  MCK(cudaMemcpyAsync(dW, W, n * 6 * sizeof(double), cudaMemcpyHostToDevice, m->stream));
  MCK(cudaMemcpyAsync(dE, eos, n * 10 * sizeof(double), cudaMemcpyHostToDevice, m->stream));
  cudaEvent_t e0, e1;
  MCK(cudaEventCreate(&e0));
  MCK(cudaEventCreate(&e1));
  MCK(cudaEventRecord(e0, m->stream));
  k_features<<<(unsigned)((n + 255) / 256), 256, 0, m->stream>>>(n, dW, dE, nullptr, dX, dref, nullptr);
  int64_t ntiles = (n + TILE - 1) / TILE;
  int grid = (int)std::min<int64_t>(ntiles, m->nsm);
  k_forward<<<grid, TILE, SMEM_FWD, m->stream>>>(n, nullptr, dX, m->wbf, m->prm, dt, m->err, nullptr);
  k_to_pressure<<<(unsigned)std::min<int64_t>((n + 255) / 256, 65535), 256, 0, m->stream>>>(n, dt, dref, dp,
                                                                                              nullptr, nullptr, nullptr);
  MCK(cudaEventRecord(e1, m->stream));
  MCK(cudaGetLastError());
  MCK(cudaMemcpyAsync(p_pred, dp, n * sizeof(double), cudaMemcpyDeviceToHost, m->stream));
  MCK(cudaStreamSynchronize(m->stream));
  if (kernel_ms) MCK(cudaEventElapsedTime(kernel_ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  for (void* p : {(void*)dW, (void*)dE, (void*)dp, (void*)dX, (void*)dt, (void*)dref}) cudaFree(p);
  return mlp_check(m);
}

}  // extern "C"

// ---- use inside the finite-volume step (m2cg_api.cu) -----------------------------
namespace m2cg {
// Features of the interface faces, network, starting pressures (float) for
// the interface solve; all device-side, sized by the interface list capacity.
void mlp_warm_faces(m2cg_mlp* m, cudaStream_t s, int nsm, const Params& P, const StateSet& S, const int32_t* id,
                    const IfaceList& L, __nv_bfloat16* X, float* t, float* pref, float* warm, const DevScalars* sc) {
  k_features_faces<<<nsm * 4, 128, 0, s>>>(P, S, id, L, X, pref, sc);
  int64_t ntiles = (L.cap + TILE - 1) / TILE;
  int grid = (int)std::min<int64_t>(ntiles, nsm);
  k_forward<<<grid, TILE, SMEM_FWD, s>>>(L.cap, L.count, X, m->wbf, m->prm, t, m->err, sc);
  k_to_pressure<<<nsm * 4, 128, 0, s>>>(L.cap, t, pref, nullptr, warm, sc, L.count);
}
cudaError_t mlp_prepare() { return mlp_set_smem(); }
}  // namespace m2cg
