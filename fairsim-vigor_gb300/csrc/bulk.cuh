// Bulk global -> shared copies tracked by shared-memory mbarriers (sm_90+ PTX: cp.async.bulk,
// mbarrier.arrive.expect_tx, mbarrier.test_wait.parity), for kernels that stage contiguous
// runs of HBM into a ring of shared-memory slots ahead of their use.
//
// A copy needs 16-byte aligned source and destination and a size that is a multiple of 16.
// Waits are bounded: bulk_wait returns false after `limit` polls (about 100 ns each), and
// the caller records the expiry in the device status word (FSIM_STATUS_BULK_WAIT) instead of
// spinning forever.
#pragma once

#include <cstdint>

namespace fsim {

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
// makes initialised barriers visible to the bulk-copy (async) proxy
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// orders this thread's earlier generic-proxy shared-memory accesses before later bulk copies
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// one arrival that also announces `bytes` of copies completing on the barrier's current phase
__device__ __forceinline__ void mbar_arrive_expect(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// waits for the phase with parity `parity` to complete; false when `limit` polls expired
__device__ __forceinline__ bool bulk_wait(uint64_t* bar, uint32_t parity, int limit) {
  for (int k = 0; k < limit; k++) {
    if (mbar_test(bar, parity)) return true;
    if (k >= 8) __nanosleep(100);
  }
  return false;
}

}  // namespace fsim
