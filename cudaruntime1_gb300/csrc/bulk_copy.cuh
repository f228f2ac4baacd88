// bulk_copy.cuh -- one-dimensional bulk copies from global to shared memory
// (cp.async.bulk: the tensor memory accelerator's untiled copy), completing
// on a shared-memory mbarrier, and waits on that barrier with an iteration
// limit.
//
// A copy needs a 16-byte aligned source and destination and a size that is
// a multiple of 16 bytes; the callers round a float2 range out to an even
// start and an even count and check that the rounded range stays inside its
// array.  A barrier counts one arrival (the issuing thread's, with the
// transaction's byte count) and the copy's bytes; its phase flips when both
// are in, and a waiter names the parity of the phase it waits for.
#pragma once
#include <cstdint>

namespace tsim {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// makes initialised barriers visible to the copy engine (before a CTA-wide sync)
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// one thread: expect `bytes` on `bar` and start the copy (after a proxy
// fence: the buffer's earlier reads, ordered by the caller's warp barrier,
// come before the copy engine's writes)
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// true once the phase of parity `parity` has completed; false after `limit`
// attempts (each attempt may suspend the thread for a short, bounded time)
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit) {
  for (uint32_t it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

}  // namespace tsim
