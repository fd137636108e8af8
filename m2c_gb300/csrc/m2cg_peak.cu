// Measurement and self-check helpers: the FP64 pipe peak of this GPU (eight
// independent binary64 FMA chains per thread, enough warps per SM to hide the
// pipe's latency; the denominator of the FP64 roofline of the stage kernels)
// and the bit-exactness check of the shared-reciprocal quotients.
#include <algorithm>
#include <cuda_runtime.h>
#include "m2cg.h"
#include "m2cg_device.cuh"

namespace {

constexpr int PEAK_THREADS = 256;
constexpr int PEAK_CHAINS = 8;

__global__ void __launch_bounds__(PEAK_THREADS) k_dfma_peak(double* out, int iters, double b, double c) {
  double a[PEAK_CHAINS];
#pragma unroll
  for (int q = 0; q < PEAK_CHAINS; q++) a[q] = 1.0e-3 * (threadIdx.x + q);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int q = 0; q < PEAK_CHAINS; q++) a[q] = fma(a[q], b, c);   // converges to c / (1 - b)
  }
  double s = 0.0;
#pragma unroll
  for (int q = 0; q < PEAK_CHAINS; q++) s += a[q];
  if (s == -1.0) out[blockIdx.x] = s;   // never true: keeps the chains live
}

}  // namespace

extern "C" m2cg_status m2cg_fp64_peak(int32_t iters, double* dfma_per_s, float* ms_out) {
  if (!dfma_per_s || iters < 1 || iters > (1 << 22)) return M2CG_ERR_INVALID_ARG;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return M2CG_ERR_NO_DEVICE;
  const int blocks = nsm * 8;
  double* out = nullptr;
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  m2cg_status st = M2CG_ERR_CUDA;
  float ms = 0.0f;
  if (cudaMalloc(&out, blocks * sizeof(double)) != cudaSuccess) return M2CG_ERR_CUDA;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess && cudaEventCreate(&e0) == cudaSuccess &&
      cudaEventCreate(&e1) == cudaSuccess) {
    k_dfma_peak<<<blocks, PEAK_THREADS, 0, s>>>(out, std::max(1, iters / 16), 0.999999, 1.0e-6);   // warm-up
    cudaEventRecord(e0, s);
    k_dfma_peak<<<blocks, PEAK_THREADS, 0, s>>>(out, iters, 0.999999, 1.0e-6);
    cudaEventRecord(e1, s);
    if (cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess &&
        cudaGetLastError() == cudaSuccess && ms > 0.0f) {
      *dfma_per_s = (double)blocks * PEAK_THREADS * PEAK_CHAINS * (double)iters / (ms * 1e-3);
      if (ms_out) *ms_out = ms;
      st = M2CG_OK;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (s) cudaStreamDestroy(s);
  cudaFree(out);
  return st;
}

// ---- m2cg_selftest_quotient ---------------------------------------------------
namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {   // splitmix64 finalizer
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
// a double with sign and significand from r and the given biased exponent field
__device__ __forceinline__ double with_exp(uint64_t r, int e) {
  return __longlong_as_double((long long)((r & 0x800fffffffffffffull) | ((uint64_t)(e & 0x7ff) << 52)));
}

__global__ void k_selftest_quotient(int64_t n, uint64_t seed, unsigned long long* out) {
  unsigned long long bad = 0, fast = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t r1 = mix64(seed ^ (uint64_t)i * 0xd1342543de82ef95ull), r2 = mix64(r1 ^ 0x2545f4914f6cdd1dull);
    const uint64_t r3 = mix64(r2);
    double a, b;
    switch (i & 7) {
      case 0: a = __longlong_as_double((long long)r1); b = __longlong_as_double((long long)r2); break;   // any bits
      case 1: a = with_exp(r1, 1023 - 90 + (int)(r3 % 181)); b = with_exp(r2, 1023 - 90 + (int)((r3 >> 16) % 181)); break;
      case 2: a = with_exp(r1, 1023 - 40 + (int)(r3 % 81)); b = with_exp(r2, 1023 - 40 + (int)((r3 >> 16) % 81)); break;
      case 3: {   // divisors with all-ones (or nearly) significands, and powers of two
        const uint64_t sig[4] = {0xfffffffffffffull, 0xffffffffffffeull, 0x0000000000001ull, 0ull};
        b = __longlong_as_double((long long)((r2 & 0x8000000000000000ull) | ((uint64_t)(1023 - 30 + (int)(r3 % 61)) << 52) |
                                             sig[(r3 >> 20) & 3]));
        a = with_exp(r1, 1023 - 30 + (int)((r3 >> 32) % 61));
        break;
      }
      case 4: {   // zeros, subnormals, infinities and NaNs as numerator or divisor
        const double sp[6] = {0.0, -0.0, 4.9e-324, -2.2e-308, __longlong_as_double(0x7ff0000000000000ll),
                              __longlong_as_double(0x7ff8000000000000ll)};
        const double x = sp[r3 % 6], y = with_exp(r2, 1023 - 60 + (int)((r3 >> 8) % 121));
        if ((r3 >> 40) & 1) { a = x; b = y; } else { a = y; b = x; }
        break;
      }
      case 5: {   // exponents at and around the limits of the shared-reciprocal path
        const int ea = ((r3 & 1) ? 128 : 1920) + (int)((r3 >> 1) % 9) - 4;
        const int eb = ((r3 >> 8) & 1) ? 1023 + (int)((r3 >> 9) % 1000) - 500 : ((r3 >> 20) & 1 ? 128 : 1920) + (int)((r3 >> 21) % 9) - 4;
        a = with_exp(r1, ea); b = with_exp(r2, eb);
        break;
      }
      case 6: {   // exact quotients: a = b * m for a small integer m
        b = with_exp(r2, 1023 - 30 + (int)(r3 % 61));
        a = b * (double)(1 + (int)((r3 >> 16) % 4096));
        break;
      }
      default: {   // quotients near 1 and near a power of two
        b = with_exp(r2, 1023 - 20 + (int)(r3 % 41));
        a = b * (1.0 + ((double)(int)((r3 >> 16) & 0xff) - 128.0) * 0x1p-52) * (double)(1 << ((r3 >> 30) & 7));
        break;
      }
    }
    const m2cg::Quot d = m2cg::quot_of(b);
    const double q = m2cg::qdiv(a, d), ref = a / b;
    const bool both_nan = isnan(q) && isnan(ref);
    if (!both_nan && __double_as_longlong(q) != __double_as_longlong(ref)) bad++;
    if (d.fast && __double_as_longlong(d.y) != __double_as_longlong(1.0 / b)) bad++;
    const int ea = m2cg::exp_field(a), eq = ea - m2cg::exp_field(b) + 1023;
    fast += (d.fast && ea >= 128 && ea <= 1920 && eq >= 128 && eq <= 1920) ? 1 : 0;
  }
  if (bad) atomicAdd(&out[0], bad);
  if (fast) atomicAdd(&out[1], fast);
}

}  // namespace

extern "C" m2cg_status m2cg_selftest_quotient(int64_t n, uint64_t seed, int64_t* mismatches, int64_t* fast) {
  if (!mismatches || n < 1 || n > (1ll << 36)) return M2CG_ERR_INVALID_ARG;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return M2CG_ERR_NO_DEVICE;
  unsigned long long* d = nullptr;
  unsigned long long h[2] = {0, 0};
  if (cudaMalloc(&d, sizeof(h)) != cudaSuccess) return M2CG_ERR_CUDA;
  m2cg_status st = M2CG_ERR_CUDA;
  if (cudaMemset(d, 0, sizeof(h)) == cudaSuccess) {
    k_selftest_quotient<<<nsm * 8, 256>>>(n, seed, d);
    if (cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost) == cudaSuccess && cudaGetLastError() == cudaSuccess) {
      *mismatches = (int64_t)h[0];
      if (fast) *fast = (int64_t)h[1];
      st = M2CG_OK;
    }
  }
  cudaFree(d);
  return st;
}
