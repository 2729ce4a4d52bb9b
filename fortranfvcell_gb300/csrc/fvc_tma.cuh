// fvc_tma.cuh -- bulk asynchronous copies global -> shared memory (the
// non-tensor form of the Tensor Memory Accelerator, cp.async.bulk) with
// mbarrier completion, for the staged streaming loops of the persistent
// solvers (sm_90 and later; built for sm_103a).
//
// Rules the callers keep:
//  * source and destination addresses are 16-byte aligned and every size
//    is a multiple of 16 bytes (SELL-32 slices are 32 rows or 32 slots, so
//    chunks of whole slices always are);
//  * data written with ordinary stores and read by a bulk copy in a later
//    phase is published by the grid barrier between the phases and a
//    fence.proxy.async.global by the issuing thread;
//  * a stage buffer is re-filled only after every thread of the block has
//    finished reading it (a __syncthreads between chunks);
//  * every wait is bounded: a copy that has not landed after
//    kBarrierTimeoutNs sets the launch's error flag, and the next grid
//    barrier ends the launch.
#pragma once
#include <cstdint>

#include "fvc_device.cuh"

namespace fvc {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

// Makes initialised mbarriers visible to the async proxy.
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One arrival that also announces `bytes` of copies completing on `bar`.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for phase `parity` of `bar`.  Returns false (and sets *err)
// when the copies have not landed within kBarrierTimeoutNs.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int *err) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (unsigned int spins = 1;; ++spins) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((spins & 63u) == 0) {
      if (*(volatile int *)err != 0) return false;
      if (global_ns() - t0 > kBarrierTimeoutNs) {
        atomicExch(err, 7 /* FVC_ERR_TIMEOUT */);
        return false;
      }
    }
  }
}

// Waits for the copies an mbarrier phase counts even when the error word is
// set (before a block leaves with copies in flight); bounded by the same
// time limit.  Returns false if they did not arrive in time.
__device__ __forceinline__ bool mbar_drain(uint64_t *bar, uint32_t parity) {
  const uint64_t t0 = global_ns();
  for (unsigned int spins = 0;; ++spins) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((spins & 63u) == 63u && global_ns() - t0 > kBarrierTimeoutNs) return false;
  }
}

// Orders this thread's earlier (generic-proxy) view of global memory --
// including what the last grid barrier acquired -- before its later bulk
// copies.
__device__ __forceinline__ void fence_proxy_async_global() {
  asm volatile("fence.proxy.async.global;" ::: "memory");
}

// Orders earlier generic accesses to shared memory before later bulk
// copies into it.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

}  // namespace fvc
