// TMA (cp.async.bulk.tensor) and mbarrier helpers, inline PTX for sm_103a.
#pragma once
#include <cuda.h>
#include <stdint.h>

namespace enl {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait on an mbarrier phase.  Returns false after max_iter polls
// (each try_wait itself suspends for a hardware-defined interval), so that a
// copy that never lands turns into an error status instead of a hang.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int max_iter) {
  for (int it = 0; it < max_iter; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Nanoseconds of the GPU's global timer.
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Wait on an mbarrier phase for at most max_ns nanoseconds of wall time:
// false when the phase has not completed by then (a copy that never lands
// becomes an error status within that time, whatever try_wait's own
// suspension interval is).
__device__ __forceinline__ bool mbar_wait_timed(uint64_t* bar, uint32_t parity, unsigned long long max_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (int it = 0; it < (1 << 26); ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > max_ns) return false;
  }
  return false;
}

// 3-D tiled TMA load global -> shared, completion signalled on an mbarrier.
// c0 (innermost) must be a multiple of 2 for 8-byte elements (16-byte rule).
__device__ __forceinline__ void tma_load_3d(void* smem_dst, const CUtensorMap* map, int c0, int c1, int c2,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(smem_dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}

// Untiled bulk copy global -> shared (cp.async.bulk): both addresses 16-byte
// aligned and bytes a multiple of 16; completion signalled on an mbarrier.
__device__ __forceinline__ void bulk_load(void* smem_dst, const void* gsrc, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(smem_dst)),
      "l"(static_cast<uint64_t>(__cvta_generic_to_global(gsrc))), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

}  // namespace enl
