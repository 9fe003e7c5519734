// Bulk copies (cp.async.bulk, non-tensor TMA) from global to shared memory
// completing on an mbarrier, and the bounded waits on them.
#pragma once
#include <cstdint>

#include "fvg_internal.cuh"

namespace fvg {

__device__ __forceinline__ unsigned smem_u32(const void* ptr) { return (unsigned)__cvta_generic_to_shared(ptr); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// One poll: the thread may sleep in the barrier until the phase completes,
// for at most kCopyPollNs (a suspend-time hint), instead of spinning.
constexpr unsigned kCopyPollNs = 20000;
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(kCopyPollNs)
      : "memory");
  return ok != 0;
}
// global -> shared, both addresses 16-byte aligned, size a multiple of 16
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar, uint64_t pol) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(pol)
      : "memory");
}
__device__ __forceinline__ uint64_t policy_evict_first() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// Bounded wait of a whole warp: gives up after `limit` polls (by default
// 2^16 polls of up to kCopyPollNs each, far beyond any copy's time) and reports it in the device error word
// instead of spinning forever.  The lanes vote on every poll (a completed
// phase stays completed), so the outcome is the same for the whole warp.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity, unsigned* err, unsigned limit) {
  for (unsigned it = 0; it < limit; it++)
    if (__any_sync(0xffffffffu, mbar_try_wait(bar, parity))) return true;
  if (err) atomicOr(err, 2u);
  return false;
}

}  // namespace fvg
