// Fifth-generation tensor-core primitives for sm_103a in inline PTX: tensor-memory (TMEM)
// allocation, shared-memory matrix descriptors, tcgen05.mma of kind::f16 (BF16 operands, FP32
// accumulation) issued by one thread, completion through tcgen05.commit on an mbarrier, and
// TMEM -> register loads.  Operand tiles are kept in shared memory in the canonical K-major
// layout without swizzle: 8 x 8 core matrices of 128 contiguous bytes (row r of a core matrix
// at byte 16 r), core matrices adjacent along K 128 bytes apart (the descriptor's leading
// byte offset), 8-row groups along M or N `sbo` bytes apart (its stride byte offset).
#pragma once
#include <stdint.h>

namespace tc {

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// byte offset of element (r, k) of a BF16 tile with `kdim` columns in the canonical layout
__device__ __forceinline__ constexpr int kmajor_offset(int r, int k, int kdim) {
  return (r >> 3) * (kdim / 8) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

// shared-memory matrix descriptor: start address, leading / stride byte offsets (>> 4), the
// fixed version field of sm_100-class descriptors (bits 46-48 = 0b001), base offset 0, no
// swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), A and B BF16 (bits
// 7-9 and 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28
__device__ __forceinline__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// TMEM columns for the CTA (power of two, >= 32), written to *holder by the whole warp
__device__ __forceinline__ void tmem_alloc(uint32_t *holder, uint32_t cols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(holder)),
               "r"(cols));
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t cols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
  asm volatile("fence.mbarrier_init.release.cluster;");
}

// wait for the completion of phase `parity` of the barrier, giving up after `tries` polls;
// returns whether the phase completed
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int tries) {
  uint32_t done = 0;
  for (int it = 0; it < tries && !done; it++) {
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
  }
  return done != 0;
}

// generic-proxy shared-memory writes made visible to the tensor cores' async proxy
__device__ __forceinline__ void fence_async_shared() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// D[tmem] (+)= A[smem] x B[smem]^T, one instruction (K = 16 for BF16)
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         bool accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accumulate));
}

// arrive on the barrier once every tcgen05.mma issued so far by this thread has completed
__device__ __forceinline__ void commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_addr(bar))
               : "memory");
}

// 16 consecutive FP32 columns of the warp's 32 TMEM lanes (lane i of the warp gets lane
// 32 (warp % 4) + i), then the wait for the load
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 16; j++) v[j] = __uint_as_float(r[j]);
}

}  // namespace tc
