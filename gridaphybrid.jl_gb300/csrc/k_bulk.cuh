// k_bulk.cuh -- bulk asynchronous global->shared copies completed on an
// mbarrier (cp.async.bulk, sm_90+ / sm_103a), with bounded waits.
//
// A copy must start and end on 16-byte boundaries (both addresses and the size).
// Waits give up after a fixed number of polls so that a copy that never
// lands cannot hang the GPU: the caller records an error and returns.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace hdg {

// One mbarrier try_wait suspends for up to a few microseconds (3.8 us measured on
// a GB300), so 2^18 polls give up after about one second.
constexpr uint32_t kBulkWaitPolls = 1u << 18;

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// make initialised barriers visible to the async proxy
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// order this thread's earlier generic-proxy shared accesses before later bulk copies
__device__ __forceinline__ void async_proxy_fence() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ uint64_t l2_evict_first_policy() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}

// bytes from global src to shared dst; completion is signalled on bar
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar,
                                              uint64_t policy) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar)), "l"(policy)
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// true once phase `parity` of bar has completed; false after `polls` polls
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity,
                                                  uint32_t polls = kBulkWaitPolls) {
  for (uint32_t i = 0; i < polls; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Grid barriers of co-resident (cooperative) grids wait on a generation word;
// a poll takes about 0.2 us, so 2^22 polls give up after about one second.
constexpr uint32_t kGridWaitPolls = 1u << 22;

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// true once *word differs from `old`; false after `polls` polls (32 ns apart)
__device__ __forceinline__ bool wait_word_change(const unsigned *word, unsigned old,
                                                 uint32_t polls = kGridWaitPolls) {
  for (uint32_t i = 0; i < polls; ++i) {
    if (ld_acquire_u32(word) != old) return true;
    __nanosleep(32);
  }
  return false;
}

}  // namespace hdg
