// Blackwell (sm_100-family) tensor-core building blocks for the warm-start
// MLP: tcgen05 MMA with accumulators in tensor memory (TMEM), operands in
// shared memory in the canonical K-major layout without swizzle, completion
// tracked by an mbarrier.  Only the MLP's BF16 GEMMs use these.
//
// Operand layout (K-major, no swizzle).  An R x K tile of bf16 is stored as
// "core matrices" of 8 rows x 8 elements (8 rows of 16 bytes, 128 contiguous
// bytes); core matrix (r/8, k/8) sits at byte ((r/8) * (K/8) + k/8) * 128 and
// element (r, k) at + (r%8) * 16 + (k%8) * 2.  In the matrix descriptor the
// leading-dimension byte offset (LBO) is the step between core matrices
// adjacent in K (128 B) and the stride-dimension byte offset (SBO) the step
// between 8-row groups ((K/8) * 128 B).
//
// D[M x N] (fp32, TMEM lanes = rows, columns = n) += A[M x K] * B[N x K]^T
// with one tcgen05.mma per 16 elements of K.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>

namespace m2cg {
namespace umma {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Byte offset of element (r, k) in an R x K K-major tile.
__device__ __forceinline__ uint32_t kmajor_offset(int r, int k, int K) {
  return (uint32_t)((((r >> 3) * (K >> 3) + (k >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1));
}

// Shared-memory matrix descriptor: start address, LBO and SBO in 16-byte
// units, descriptor version 1 (bits 46-47), base offset 0, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor for kind::f16 with BF16 A and B, FP32 D, both
// operands K-major, dense: D format bits 4-5 (1 = F32), A format bits 7-9 and
// B format bits 10-12 (1 = BF16), N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// ---- TMEM allocation (one full warp executes these) -------------------------
__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes become visible to the tensor core's async proxy
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// ---- mbarrier ---------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Waits for the phase with the given parity to complete; gives up after
// max_polls polls and returns false.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long max_polls) {
  uint32_t a = smem_u32(bar);
  for (long long i = 0; i < max_polls; i++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// ---- MMA --------------------------------------------------------------------
// One tcgen05.mma (single issuing thread): D(tmem) (+)= A(desc) * B(desc)^T.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// Arrives on the mbarrier once every MMA issued so far by this thread is done.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// D[128 x N] (+)= A[128 x K] * B[N x K]^T, A and B K-major tiles in shared
// memory (K a multiple of 16).  Issued by one thread.
__device__ __forceinline__ void gemm_128xN(uint32_t d_tmem, const void* a, const void* b, int N, int K,
                                           bool accumulate) {
  const uint32_t ia = smem_u32(a), ib = smem_u32(b);
  const uint32_t sbo = (uint32_t)(K >> 3) << 7;
  const uint32_t idesc = idesc_bf16_f32(128, N);
  for (int kk = 0; kk < K / 16; kk++) {
    // a K step of 16 elements spans two core matrices: 256 bytes
    mma_bf16(d_tmem, smem_desc(ia + kk * 256, 128, sbo), smem_desc(ib + kk * 256, 128, sbo), idesc,
             (accumulate || kk > 0) ? 1u : 0u);
  }
}

// ---- TMEM -> registers ------------------------------------------------------
// Warp q (of a 4-warp group) reads TMEM lanes 32q..32q+31; lane i receives 16
// consecutive fp32 columns of row 32q+i starting at column col.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

}  // namespace umma
}  // namespace m2cg
