// Bulk asynchronous copies (TMA, cp.async.bulk) from global to shared memory
// completing on shared-memory mbarriers, for sm_100-family GPUs.
//
// A warp that stages data for itself uses one mbarrier per buffer with an
// arrival count of 1: one lane arrives with the expected byte count and
// issues the copies; every lane then waits on the barrier's phase.  Waits
// are bounded: after kMbarMaxPolls unsuccessful polls they give up and the
// caller reports MPM_STATUS_TIMEOUT instead of spinning forever.
#pragma once

#include <cuda.h>
#include <stdint.h>

namespace mpm {

constexpr int kMbarMaxPolls = 1 << 22;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// makes mbarrier initialisation visible to the asynchronous proxy
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// orders this thread's earlier shared-memory accesses before later
// asynchronous-proxy accesses (a bulk copy into a buffer that was just read)
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n"
      "  .reg .pred p;\n"
      "  mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "  selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits until the phase with the given parity of `bar` has completed;
// false when it has not after kMbarMaxPolls polls.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, uint32_t parity) {
  for (int k = 0; k < kMbarMaxPolls; ++k)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// One contiguous global -> shared copy of `bytes` (a multiple of 16; both
// addresses 16-byte aligned) that completes `bytes` transactions on `bar`.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, unsigned long long *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// One tiled tensor copy (a box of a 2-D tensor map) global -> shared at box
// origin (x, y) in elements; x * element size must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y,
                                            unsigned long long *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

}  // namespace mpm
