// mbarrier and bulk-tensor (TMA) primitives with bounded waits: a CTA that
// waits for an asynchronous copy polls its mbarrier a limited number of
// times, and when the phase never completes it records an error in a status
// word and returns instead of hanging the GPU.
#pragma once
#include <cuda.h>
#include <stdint.h>

#include "ribo_dev.cuh"

namespace ribo {

// Bounded waits: a phase that has not completed after this many polls is
// reported in the status word and the CTA stops.
constexpr uint32_t TMA_WAIT_POLLS = 1u << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t arrivals) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(arrivals) : "memory");
  // make the initialised barrier visible to the asynchronous (TMA) proxy
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// The calling thread's arrival, announcing `bytes` of transactions.
__device__ __forceinline__ void mbar_arrive_expect(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// Box (x, y) of tensor map `map` (generic address of a map in global
// memory) into shared memory at `dst` (16-byte aligned), completing on `bar`.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// Waits for phase `parity` of `bar` to complete; false after `polls` polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t polls = TMA_WAIT_POLLS) {
  for (uint32_t i = 0; i < polls; i++) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

}  // namespace ribo
