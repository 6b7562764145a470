// Tensor-memory-accelerator (TMA) tile loads for the stencil kernels.
//
// A 2-D tile (box) of a row-major array is copied from global to shared
// memory by one elected thread with cp.async.bulk.tensor; completion is
// tracked by an mbarrier transaction count.  Out-of-range parts of the box
// (negative or past-the-end coordinates) are filled with zeros by the
// hardware, which is exactly the "outside the grid" value the kernels need.
//
// Alignment rules the callers respect: the box's first coordinate x times
// the element size is a multiple of 16 bytes, the array base is 16-byte
// aligned, the row pitch is a multiple of 16 bytes, and the shared-memory
// destination is 128-byte aligned.
//
// Waits are bounded: a wait that does not complete within RIBO_TMA_SPIN
// polls records RIBO_ERR_TMA_TIMEOUT in the world's status word and the
// kernel returns instead of hanging.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace ribo {

constexpr uint32_t RIBO_TMA_SPIN = 1u << 26;
constexpr uint32_t RIBO_ERR_TMA_TIMEOUT = 1u;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}

// Waits for phase `phase` of `bar`; false (and an error flag) on timeout.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t phase, uint32_t* status) {
  for (uint32_t i = 0; i < RIBO_TMA_SPIN; i++)
    if (mbar_try_wait(bar, phase)) return true;
  if (status) atomicOr(status, RIBO_ERR_TMA_TIMEOUT);
  return false;
}

// Host: encodes a 2-D tiled tensor map over a row-major array of `w` x `h`
// elements with row pitch `pitch_elems`, box `box_w` x `box_h`.  Returns
// false when the driver entry point is unavailable or the layout breaks the
// alignment rules.
bool make_tensor_map_2d(CUtensorMap* out, void* base, CUtensorMapDataType type, int elem_bytes, uint64_t w, uint64_t h,
                        uint64_t pitch_elems, uint32_t box_w, uint32_t box_h);

}  // namespace ribo
