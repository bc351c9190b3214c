// Device helpers for asynchronous global->shared copies completed on
// mbarriers (cp.async.bulk / cp.async.bulk.tensor), with bounded waits.
//
// Every wait here gives up after a fixed number of polls and reports it, so a
// copy that never lands ends the kernel with an error code instead of a hang.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace risa_gb {
namespace async {

constexpr uint32_t kSpinLimit = 1u << 26;  // ~ seconds of polling

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
   return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
   asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes initialised mbarriers visible to the async proxy; follow with a CTA barrier.
__device__ __forceinline__ void mbar_init_fence() {
   asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
   asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
   asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
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

// Bounded wait; returns false when it gives up.
__device__ __forceinline__ bool mbar_wait_quiet(uint64_t* bar, uint32_t parity) {
   for (uint32_t i = 0; i < kSpinLimit; ++i)
      if (mbar_try_wait(bar, parity)) return true;
   return false;
}

// Bounded wait; returns false (and records `code` in the global *err) when it gives up.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err, int code) {
   if (mbar_wait_quiet(bar, parity)) return true;
   atomicCAS(err, 0, code);
   return false;
}

// Contiguous global -> shared copy of `bytes` (multiple of 16; both addresses
// 16-byte aligned) that completes `bytes` transactions on `bar`.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
   asm volatile(
       "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
           smem_u32(dst)),
       "l"(src), "r"(bytes), "r"(smem_u32(bar))
       : "memory");
}

// 4-, 8- or 16-byte global -> shared copy (cp.async, both addresses aligned to
// its size). Copies are grouped by cp_async_commit; cp_async_wait_all makes
// the issuing thread's own copies visible to it.
template <int BYTES>
__device__ __forceinline__ void cp_async(void* dst, const void* src) {
   static_assert(BYTES == 4 || BYTES == 8 || BYTES == 16, "cp.async copies 4, 8 or 16 bytes");
   asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(smem_u32(dst)), "l"(src), "n"(BYTES) : "memory");
}
// 16-byte copy that bypasses L1 (cp.async.cg), for data read once from shared memory
__device__ __forceinline__ void cp_async_cg16(uint32_t dst, const void* src) {
   asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
// waits until at most N of the issuing thread's committed groups are pending
template <int N>
__device__ __forceinline__ void cp_async_wait() {
   asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

}  // namespace async
}  // namespace risa_gb
