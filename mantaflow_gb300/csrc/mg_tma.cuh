// Bulk asynchronous copies (the TMA engine's untiled form) into shared
// memory, completed on shared-memory mbarriers: the staging of the plane-
// streaming stencil kernels.
//
// Every wait is bounded by the global timer: a wait that runs out returns
// false and the kernel reports the error instead of spinning on.  A bulk copy
// needs 16-byte aligned source and destination addresses and a size that is
// a multiple of 16 bytes.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mgpu {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// one thread: an mbarrier expecting `count` arrivals per phase
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count = 1) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// a plain arrival (no transaction bytes)
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  uint64_t state;
  asm volatile("mbarrier.arrive.shared::cta.b64 %0, [%1];" : "=l"(state) : "r"(smem_addr(bar)) : "memory");
  (void)state;
}

// after every mbar_init of the block, before any thread uses the barriers
// (the bulk-copy engine included)
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// the one arrival of this phase, announcing `bytes` of copies that complete it
__device__ __forceinline__ void mbar_arrive_expect(uint64_t* bar, uint32_t bytes) {
  uint64_t state;
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;"
               : "=l"(state)
               : "r"(smem_addr(bar)), "r"(bytes)
               : "memory");
  (void)state;
}

// bulk copy of `bytes` from global memory into shared memory, counted on bar
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// wait until the phase of the given parity has completed; false after
// limitNs nanoseconds
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limitNs) {
  if (mbar_try(bar, parity)) return true;
  const unsigned long long t0 = gtimer();
  for (;;) {
    if (mbar_try(bar, parity)) return true;
    if (gtimer() - t0 > (unsigned long long)limitNs) return false;
  }
}

}  // namespace mgpu
