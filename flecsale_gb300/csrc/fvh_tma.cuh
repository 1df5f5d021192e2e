// Shared-memory staging with the bulk-copy (TMA) engine: mbarrier and
// cp.async.bulk wrappers (inline PTX, sm_90+; used here on sm_103a).
//
// A copy global -> shared of `bytes` (a multiple of 16, both addresses 16-byte
// aligned) completes on an mbarrier; the thread that posts the copies first
// announces their total size with arrive.expect_tx, and the barrier's phase
// completes once that arrival and all the announced bytes have landed.  Every
// wait here is bounded: it gives up after a fixed number of polls and reports
// failure, so a kernel never spins forever on a copy that does not arrive.
#pragma once

#include <cstdint>

namespace fvh {
namespace tma {

__device__ __forceinline__ unsigned smem_addr(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

// make barrier initialisation visible to the async proxy (the copy engine)
__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// order this thread's earlier shared-memory accesses (generic proxy) before
// later bulk copies into shared memory (async proxy)
__device__ __forceinline__ void fence_proxy_async_shared() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *bar, unsigned bytes) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(smem_addr(bar)),
      "r"(bytes)
      : "memory");
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes,
                                         unsigned long long *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for the phase of `parity` to complete; false after `polls` polls.
// (try_wait itself may suspend the thread for a while before it returns.)
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned parity,
                                                  int polls) {
  for (int k = 0; k < polls; ++k)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

}  // namespace tma
}  // namespace fvh
