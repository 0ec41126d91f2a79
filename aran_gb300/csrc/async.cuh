// async.cuh -- asynchronous copy and mbarrier primitives (inline PTX, sm_90+)
// shared by the M2L kernels: bulk (TMA) global->shared copies completed on
// an mbarrier, bounded mbarrier waits, and per-thread cp.async copies.
#pragma once

#include <cstdint>

namespace aran {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *mb, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mb)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *mb, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mb)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *mb) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(mb)) : "memory");
}

// bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned)
// completing as transaction bytes on mbarrier `mb`
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *mb) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(mb))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *mb, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(mb)), "r"(parity)
      : "memory");
  return ok != 0;
}

constexpr int kWaitPolls = 1 << 20;

// bounded wait: gives up after `polls` polls (each poll may itself suspend)
__device__ __forceinline__ bool mbar_wait(uint64_t *mb, uint32_t parity, int polls = kWaitPolls) {
  for (int i = 0; i < polls; ++i)
    if (mbar_try_wait(mb, parity)) return true;
  return false;
}

// bounded wait that also gives up once the error word `flag` is non-zero
// (another warp or CTA stopped: the phase it was to complete may never come)
__device__ __forceinline__ bool mbar_wait_or_flag(uint64_t *mb, uint32_t parity, const int *flag,
                                                  int polls = kWaitPolls) {
  for (int i = 0; i < polls; ++i) {
    if (mbar_try_wait(mb, parity)) return true;
    if ((i & 63) == 63 && *(const volatile int *)flag) return false;
  }
  return false;
}

// per-thread asynchronous global -> shared copies of 8 or 16 bytes (both
// addresses aligned to the size)
__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;" ::: "memory");
}

}  // namespace aran
