// FP64 pipe peak of this GPU, measured: eight independent binary64 FMA chains
// per thread, enough warps per SM to hide the pipe's latency.  The rate is the
// denominator of the FP64 roofline of the stage kernels (the HBM and tensor
// peaks are measured elsewhere; no FP64 figure is).
#include <algorithm>
#include <cuda_runtime.h>
#include "m2cg.h"

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
