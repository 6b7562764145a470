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

// ---- Stencil-pass tiles ----------------------------------------------------
// A PASS_BX x PASS_BY tile of fluid cells with its one-cell ring, staged as a
// 36 x 10 box of 8-byte elements whose origin is (x0 - 2, y0 - 1): x0 is a
// multiple of 32, so the box starts on a 16-byte boundary, and a box row is
// 288 bytes.  Elements outside the field read as zero (the passes index
// clamped coordinates, which lie inside the field).
constexpr int ST_OX = 2, ST_OY = 1;
constexpr int ST_BW = PASS_BX + 2 * ST_OX, ST_BH = PASS_BY + 2 * ST_OY, ST_BOX = ST_BW * ST_BH;
static_assert((ST_OX * 8) % 16 == 0 && (PASS_BX * 8) % 16 == 0 && (ST_BW * 8) % 16 == 0, "16-byte box origins and rows");
// The world's descriptors (device memory, 64-byte aligned), by field: the
// gathered forces, whose 3 x 3 average add_forces takes from the staged box.
// (Staging the velocities of the diffusion and curl passes the same way was
// slower: their 3 x 3 and 5-point neighbours are cheap L1 hits, and a box
// makes every thread wait for the copy before it computes.)
enum StencilMap : int { SM_FORCES = 0, SM_COUNT };
constexpr size_t STENCIL_TMAP_BYTES = SM_COUNT * 128;

// Box index of field cell (gx, gy) for the tile at (x0, y0).
__device__ __forceinline__ int st_at(int x0, int y0, int gx, int gy) { return (gy - (y0 - ST_OY)) * ST_BW + (gx - (x0 - ST_OX)); }

// Stages the boxes of NF 8-byte fields around the tile at (x0, y0): one TMA
// copy per field when the world has descriptors (tmap non-null; map[k] is
// the field's index), else plain loads of the in-grid elements.  Every
// thread of the CTA calls it.  Returns false (after recording a timeout in
// `status`) when a copy never completed; the caller then returns.
template <int NF>
__device__ __forceinline__ bool stage_stencil(const void* tmap, const int (&map)[NF], const uint2* const (&src)[NF],
                                              uint2* const (&box)[NF], int x0, int y0, int fw, int fh, uint64_t* bar,
                                              uint32_t* status) {
  const int tid = (int)(threadIdx.y * blockDim.x + threadIdx.x), nt = (int)(blockDim.x * blockDim.y);
  if (tmap) {
    const CUtensorMap* maps = reinterpret_cast<const CUtensorMap*>(tmap);
    if (tid == 0) mbar_init(bar, 1);
    __syncthreads();
    if (tid == 0) {
      mbar_arrive_expect(bar, (uint32_t)(NF * ST_BOX * 8));
#pragma unroll
      for (int k = 0; k < NF; k++) tma_load_2d(box[k], maps + map[k], x0 - ST_OX, y0 - ST_OY, bar);
    }
    const bool late = !mbar_wait(bar, 0u);
    if (__syncthreads_or(late)) {
      if (tid == 0 && status) atomicOr(status, ERR_TIMEOUT);
      mbar_wait(bar, 0u);  // the copy may still be in flight: wait once more before leaving
      return false;
    }
    return true;
  }
  for (int i = tid; i < ST_BOX; i += nt) {
    const int gx = x0 - ST_OX + i % ST_BW, gy = y0 - ST_OY + i / ST_BW;
    if (gx < 0 || gy < 0 || gx >= fw || gy >= fh) continue;
    const size_t g = (size_t)gy * fw + gx;
#pragma unroll
    for (int k = 0; k < NF; k++) box[k][i] = __ldg(src[k] + g);
  }
  __syncthreads();
  return true;
}

}  // namespace ribo
