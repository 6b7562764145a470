// Allocation-free pressure solve.
//
// ribo_pressure_solve_noalloc runs the same multigrid V-cycles as the world
// step's pressure solve on buffers the caller owns, for callers that must
// not allocate device memory while they run: for example an engine or
// plugin host that reserves its whole device-memory budget at start-up and
// forbids allocations afterwards, or a frame loop that cannot afford the
// implicit device synchronisation cudaMalloc / cudaFree may cause.  The
// multigrid hierarchy (all levels of p, rhs, water flags, the pre-smoothed
// copies) lives in the file-scope array below, which every GPU that loads
// this library holds until the process exits.
#include <cuda_runtime.h>
#include <string.h>

#include <atomic>

#include "../../include/ribo_world.h"
#include "ribo_dev.cuh"
#include "ribo_launch.h"
#include "ribo_world_impl.h"

namespace ribo {
namespace {

// Largest fluid grid the fixed scratch can hold: 512 x 512 cells.
constexpr uint64_t NOALLOC_MAX_CELLS = 512ull * 512ull;
// Level arrays of the hierarchy: sum over levels of cells rounded up to 64,
// at most 4/3 of the finest level plus one 64-cell pad per level.
constexpr uint64_t NOALLOC_MAX_LEVEL_CELLS = NOALLOC_MAX_CELLS * 4 / 3 + 64 * 16;
// p, rhs, p2 (floats, all levels) + p_tmp (floats, level 0) + water flags
// (bytes, all levels) + wall mask (bytes, level 0), plus 256-byte alignment
// of each of the six blocks.
constexpr uint64_t NOALLOC_SCRATCH_BYTES =
    3 * 4 * NOALLOC_MAX_LEVEL_CELLS + 4 * NOALLOC_MAX_CELLS + NOALLOC_MAX_LEVEL_CELLS + NOALLOC_MAX_CELLS + 256 * 6;

// ~6.2 MB per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

// Device address of the scratch array, looked up once per device.  In host
// code `g_noalloc_scratch` only names a host-side stand-in, so kernels are
// always given this address instead.
constexpr int MAX_DEVICES = 64;
std::atomic<unsigned char*> g_scratch_addr[MAX_DEVICES];

__global__ void k_noalloc_flags(const uint32_t* __restrict__ solid, uint8_t* __restrict__ mask, uint8_t* __restrict__ water,
                                size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const bool s = solid[i] != 0u;
  mask[i] = s ? 1 : 0;
  water[i] = s ? 0 : 1;
}

inline size_t up256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace
}  // namespace ribo

extern "C" ribo_status ribo_pressure_solve_noalloc(uint32_t fluid_w, uint32_t fluid_h, const float* d_divergence,
                                                   const uint32_t* d_solid_mask, float* d_pressure, uint32_t mg_min_size,
                                                   uint32_t mg_pre, uint32_t mg_post, uint32_t mg_coarse, uint32_t mg_cycles,
                                                   void* stream_handle) {
  using namespace ribo;
  if (!d_divergence || !d_solid_mask || !d_pressure) return set_error(RIBO_INVALID_ARG, "null buffer");
  if (fluid_w < 2 || fluid_h < 2) return set_error(RIBO_INVALID_ARG, "fluid sides must be >= 2");
  const uint64_t cells = (uint64_t)fluid_w * fluid_h;
  if (cells > NOALLOC_MAX_CELLS)
    return set_error(RIBO_INVALID_ARG,
                     "ribo_pressure_solve_noalloc: %ux%u fluid cells exceed the fixed scratch limit of %llu cells (512x512)",
                     fluid_w, fluid_h, (unsigned long long)NOALLOC_MAX_CELLS);
  if (!mg_min_size) mg_min_size = 8;
  if (!mg_pre) mg_pre = 2;
  if (!mg_post) mg_post = 2;
  if (!mg_coarse) mg_coarse = 30;
  if (!mg_cycles) mg_cycles = 1;
  cudaStream_t stream = (cudaStream_t)stream_handle;

  // once per device: the device address of the scratch array
  int dev = 0;
  ribo_status st = cuda_status(cudaGetDevice(&dev), "device");
  if (st != RIBO_OK) return st;
  if (dev < 0 || dev >= MAX_DEVICES) return set_error(RIBO_INVALID_ARG, "device ordinal %d out of range", dev);
  unsigned char* base = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (!base) {
    void* p = nullptr;
    st = cuda_status(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress");
    if (st != RIBO_OK) return st;
    base = static_cast<unsigned char*>(p);
    g_scratch_addr[dev].store(base, std::memory_order_release);
  }

  // multigrid levels (src/world/mod.rs:637-671), on the stack
  MgLevel levels[16];
  int nl = 0;
  size_t off = 0;
  {
    int nx = (int)fluid_w, ny = (int)fluid_h, l = 0;
    for (;;) {
      if (nl == 16) return set_error(RIBO_INVALID_ARG, "too many multigrid levels");
      levels[nl++] = MgLevel{nx, ny, off, (float)1e-4 * (float)(1u << l)};
      off += ((size_t)nx * ny + 63) & ~(size_t)63;
      if ((uint32_t)nx > mg_min_size && (uint32_t)ny > mg_min_size && nx % 2 == 0 && ny % 2 == 0) {
        nx /= 2;
        ny /= 2;
        l++;
      } else {
        break;
      }
    }
  }
  MgConfig c{(int)mg_pre, (int)mg_post, (int)mg_coarse, (int)mg_cycles};
  if (!multigrid_fused_ok(levels, nl, c))
    return set_error(RIBO_INVALID_ARG,
                     "ribo_pressure_solve_noalloc: the coarsest level must hold at most 4096 cells and 1 <= pre, post <= 7");

  // carve the scratch
  MgBufs b{};
  size_t at = 0;
  auto take = [&](size_t bytes) {
    unsigned char* p = base + at;
    at += up256(bytes);
    return p;
  };
  b.p = reinterpret_cast<float*>(take(off * 4));
  b.rhs = reinterpret_cast<float*>(take(off * 4));
  b.p2 = reinterpret_cast<float*>(take(off * 4));
  b.p_tmp = reinterpret_cast<float*>(take(cells * 4));
  b.fluid = take(off);
  uint8_t* mask = take(cells);
  if (at > NOALLOC_SCRATCH_BYTES) return set_error(RIBO_INVALID_ARG, "scratch layout overflow");

  Dev d{};
  memset(&d, 0, sizeof d);
  d.fw = d.gw = (int)fluid_w;
  d.fh = d.gh = (int)fluid_h;
  d.mask = mask;
  d.div = const_cast<float*>(d_divergence);
  d.pa = d_pressure;
  d.fluid0 = b.fluid + levels[0].off;
  // No kernel of the solve waits on anything or reports through a status
  // word, so none is passed.  Every scratch word the solve reads is written
  // earlier in the same call, so nothing needs clearing between calls.
  d.status = nullptr;
  k_noalloc_flags<<<(unsigned)((cells + 255) / 256), 256, 0, stream>>>(d_solid_mask, mask, d.fluid0, cells);
  launch_multigrid_fused(d, levels, nl, b, c, stream);
  return cuda_status(cudaGetLastError(), "noalloc pressure solve");
}
