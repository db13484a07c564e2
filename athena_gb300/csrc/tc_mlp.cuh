// Fifth-generation tensor-core (tcgen05) evaluation of the con2prim network for a tile of
// 128 cells: one CTA of 128 threads, thread t = cell t = row t of the M = 128 tiles.
//
//   layer 1: D0[128 x 64]  = X[128 x 16] . W1^T       (K = 16: inputs zero-padded)
//   layer 2: D1[128 x 64]  = silu(D0 + b1) . W2^T     (K = 64: four K = 16 steps)
//   layer 3: D0[128 x 16]  = silu(D1 + b2) . W3^T     (N = 16: outputs zero-padded)
//
// Operands are BF16 in shared memory in the no-swizzle K-major core-matrix layout (a core
// matrix is 8 rows x 16 bytes, rows 16 bytes apart; along K core matrices are LBO bytes
// apart, along M/N SBO bytes apart), accumulators FP32 in tensor memory (TMEM: lane = row,
// column = output).  One elected thread issues tcgen05.mma and tcgen05.commit, which
// arrives on an mbarrier when the MMAs are done; every thread then reads its own row back
// with tcgen05.ld (warp w reads TMEM lanes 32w..32w+31), applies bias and SiLU in FP32 and
// writes the next layer's A operand.  Waits on the mbarrier are bounded (0.1 s of SM
// clock): on timeout the CTA records an error flag and stops issuing work.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace athgpu {
namespace tc {

constexpr int M = 128;       // cells per tile = threads per CTA
constexpr int TMEM_COLS = 128;
constexpr uint32_t LBO = 128;  // core matrices adjacent along K

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor: start >> 4 [0,14), LBO >> 4 [16,30), SBO >> 4 [32,46),
// descriptor version 1 [46,48), base offset 0, no swizzle [61,64) = 0
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: D FP32 [4,6) = 1, A BF16 [7,10) = 1, B BF16
// [10,13) = 1, both K-major (bits 15, 16 = 0), N >> 3 at [17,23), M >> 4 at [24,29)
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}

// byte offset of element (row r, k) in a K-major no-swizzle tile with kdim columns
__device__ __forceinline__ uint32_t kmajor_off(int r, int k, int kdim) {
  return (uint32_t)((r >> 3) * (kdim / 8) * 128 + (k >> 3) * LBO + (r & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                   dst_smem),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}
// generic-proxy shared-memory writes -> visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void commit(uint32_t mbar_smem) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
          mbar_smem)
      : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar_smem, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(mbar_smem), "r"(count)
               : "memory");
}
// one test of the mbarrier phase with the given parity (true once it has completed)
__device__ __forceinline__ bool mbar_try(uint32_t mbar_smem, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(done)
      : "r"(mbar_smem), "r"(parity)
      : "memory");
  return done != 0;
}

// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  // the registers are tied to the wait so that no use is scheduled before it
  asm volatile("tcgen05.wait::ld.sync.aligned;\n"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]),
                 "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]),
                 "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15])
               :
               : "memory");
#pragma unroll
  for (int q = 0; q < 16; ++q) v[q] = __uint_as_float(r[q]);
}

}  // namespace tc
}  // namespace athgpu
