// Host-side launchers of the world-step kernels (one per pass).  The world
// orchestration in world.cu and the batch orchestration in batch.cu call
// them in the reference's dispatch order.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <atomic>

#include "ribo_dev.cuh"

namespace ribo {

// Per-device one-time set-up (kernel attributes and the like) that may be
// reached from several host threads: `pending()` says whether the current
// device still needs it, `done()` records it.  Two threads that race both
// run the set-up, which is idempotent; no bit is ever lost.
struct DeviceOnce {
  std::atomic<uint64_t> bits{0};
  static int device() {
    int dev = 0;
    cudaGetDevice(&dev);
    return dev & 63;
  }
  bool pending(int dev) const { return !((bits.load(std::memory_order_acquire) >> dev) & 1ull); }
  void done(int dev) { bits.fetch_or(1ull << dev, std::memory_order_release); }
};

// Streaming multiprocessors of the current device, queried once per device
// (grid sizes and tile choices scale with it).  Without an answering device
// (a host-only size computation) it is the GB300's 152.
inline int device_sm_count() {
  static std::atomic<int> cache[64];
  const int dev = DeviceOnce::device();
  int v = cache[dev].load(std::memory_order_relaxed);
  if (v <= 0) {
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) {
      cudaGetLastError();
      return 152;
    }
    cache[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}

// Per-launch instrumentation: every kernel launch of the library goes
// through RB_LAUNCH, which counts it and, when kernel timing is enabled on
// the world being stepped, brackets it with CUDA events on its stream.
// `bytes` is the launch's algorithmic traffic (compulsory reads + writes).
void ktime_begin(const char* label, double bytes, cudaStream_t s);
void ktime_end(cudaStream_t s);
#define RB_LAUNCH(label, bytes, s, ...)      \
  do {                                        \
    ::ribo::ktime_begin((label), (bytes), (s)); \
    __VA_ARGS__;                              \
    ::ribo::ktime_end(s);                     \
  } while (0)

// Launch geometries of the passes: how many CTAs one world's grid needs.
enum Geo : int {
  GEO_FLUID = 0,    // fluid grid, PASS_BX x PASS_BY cells per CTA
  GEO_ENV,          // environment grid, PASS_BX x PASS_BY cells per CTA
  GEO_ENV_LINEAR,   // environment cells, LINEAR_THREADS per CTA (1-D)
  GEO_SCATTER,      // environment grid, SCATTER_TX x SCATTER_TY tiles
  GEO_NET_FLUX,     // fluid rows then columns, NET_FLUX_LINES per CTA (1-D)
  GEO_LEDGER,       // environment cells, LEDGER_CELLS_PER_CTA per CTA (1-D)
  GEO_LIGHT,        // light grid (grid / LIGHT_DIV), PASS_BX x PASS_BY cells per CTA
  GEO_FLUID_TALL,   // fluid grid, PASS_BX x (PASS_BY * FLUID_ROWS) cells per CTA
  GEO_ENV_TALL,     // environment grid, PASS_BX x (PASS_BY * FLUID_ROWS) cells per CTA
  GEO_ENV_LINEAR4,  // environment cells, 4 * LINEAR_THREADS per CTA (1-D)
  GEO_COUNT
};
void geo_blocks(Geo g, const Dev& d, int* nbx, int* nby);

// Where a pass runs: one world (its Dev by value), or a batch of worlds
// through device tables (see WorldSet).
struct Target {
  Dev one{};
  const ribo_sim_params* P = nullptr;  // device: the world's params, or [n] params of the batch's step
  int n = 0;                           // 0: one world; > 0: a batch of n worlds
  const Dev* devs = nullptr;           // device [n]
  const int* start[GEO_COUNT] = {};    // device [n + 1] per geometry
  const int* nbx[GEO_COUNT] = {};      // device [n] per geometry
  int total[GEO_COUNT] = {};           // CTAs of a batched launch per geometry
  double fcells = 0.0, cells = 0.0;    // fluid / environment cells over all worlds (byte models)
  bool batch() const { return n > 0; }
  WorldSet set(Geo g, uint32_t* out) const { return WorldSet{devs, start[g], nbx[g], P, out, n}; }
  OneWorld single(uint32_t* out) const { return OneWorld{one, P, out}; }
  dim3 grid(Geo g) const {
    int x = 0, y = 0;
    geo_blocks(g, one, &x, &y);
    return dim3((unsigned)x, (unsigned)y);
  }
};
Target target_one(const Dev& d, const ribo_sim_params* P);

// Launches pass kernel template `kern` over target `t`: kern<OneWorld> on the
// world's own grid, or kern<WorldSet> over the CTAs of geometry `geo` of all
// worlds of the batch.  `out` is the pass-specific output pointer.
#define RB_PASS(label, bytes, s, t, geo, blk, smem, kern, out, ...)                                             \
  do {                                                                                                         \
    if ((t).batch()) {                                                                                         \
      if ((t).total[geo] > 0)                                                                                  \
        RB_LAUNCH(label, bytes, s,                                                                             \
                  kern<WorldSet><<<(unsigned)(t).total[geo], blk, smem, s>>>((t).set(geo, out), ##__VA_ARGS__)); \
    } else {                                                                                                   \
      RB_LAUNCH(label, bytes, s, kern<OneWorld><<<(t).grid(geo), blk, smem, s>>>((t).single(out), ##__VA_ARGS__)); \
    }                                                                                                          \
  } while (0)

// Velocity ping-pong direction of a pass: reads velocity_a, writes
// velocity_b (A_TO_B) or the reverse (B_TO_A).
enum : int { A_TO_B = 0, B_TO_A = 1 };

// light.cu (light_mode 1)
void launch_light_transmit(const Target& t, cudaStream_t s);
void launch_light_sweep(const Dev& d, const ribo_sim_params* P, cudaStream_t s);
void launch_light_propagate(const Target& t, cudaStream_t s);
void launch_light_commit(const Target& t, cudaStream_t s);

// terrain.cu (terrain_mode 1, and the terrain brush)
struct TerrainBufs {
  uint32_t* gamma;  // grains per cell, updated in place
  uint8_t* code;    // per cell: 0 = its grain stays; 1 + k = it moves to the k-th of its 8 neighbours
                    // in ascending cell index (centre skipped)
  uint8_t* arrivals;  // per cell that received grains: bit k = the grain of its k-th neighbour arrived
  uint32_t* list;   // cells that received a grain (relax) or were painted, each at most once, in nine
                    // segments by class (x mod 3 + 3 (y mod 3)) of terrain_list_entries / 9 entries
  uint32_t* count;  // [9] entries per segment (the eviction kernel empties them)
};
size_t terrain_list_entries(int gw, int gh);
// One relax pass (relax_gamma_a for phase 0, _b for phase 1): decisions,
// moves, eviction loops.
void launch_relax(const Dev& d, const ribo_sim_params* P, const TerrainBufs& t, uint32_t phase, cudaStream_t s);
// grain_fall: three launches (columns x mod 3); each returns at once on steps
// the fall clock does not tick.
void launch_grain_fall(const Dev& d, const ribo_sim_params* P, const TerrainBufs& t, cudaStream_t s);
void launch_paint(const Dev& d, const TerrainBufs& t, float cx, float cy, float radius, uint32_t grains, cudaStream_t s);

// fluid.cu
void launch_solid_mask(const Target& t, cudaStream_t s);
void launch_temperature(const Target& t, cudaStream_t s);
void launch_forces(const Target& t, cudaStream_t s);
void launch_add_forces(const Target& t, int dir, cudaStream_t s);
void launch_diffuse(const Target& t, int dir, cudaStream_t s);
void launch_advect(const Target& t, int dir, cudaStream_t s);
void launch_vorticity(const Target& t, int dir, cudaStream_t s);
void launch_divergence(const Target& t, int dir, cudaStream_t s);
void launch_subtract_gradient(const Target& t, int dir, cudaStream_t s);
void launch_net_flux(const Target& t, int dir, cudaStream_t s);
void launch_boundaries(const Target& t, int dir, cudaStream_t s);
void launch_smooth(const Target& t, int dir, cudaStream_t s);
// TMA descriptors of a world's stencil-pass tiles (the gathered forces),
// written to `dst` (device, STENCIL_TMAP_BYTES, 64-byte aligned) on stream
// s; false where the field cannot be described (the pass then stages its
// tile with plain loads).
struct StencilFields {
  const void* forces;
  int fw, fh;
};
constexpr size_t STENCIL_TMAP_BYTES_HOST = 128;
bool stencil_tensor_maps(void* dst, const StencilFields& f, cudaStream_t s);
// A bounded mbarrier wait that runs out, on `device` (ribo_selftest_bounded_wait).
ribo_status selftest_bounded_wait(int device, uint32_t polls, uint32_t* bits);

// multigrid.cu
struct MgLevel {
  int nx, ny;
  size_t off;  // element offset of the level in the level arrays
  float eps;
};
struct MgBufs {
  float* p;         // all levels, contiguous (64-element aligned level offsets)
  float* rhs;       // all levels
  uint8_t* fluid;   // all levels: 1 = water
  float* p_tmp;     // level-0 ping-pong partner of pressure_a (fused path)
  float* p2;        // all levels: pre-smoothed p (fused path)
  uint8_t* code;    // all levels: neighbour codes from the water flags (null: built per box)
};
struct MgConfig {
  int pre, post, coarse, cycles;
  int cluster = 0;  // ribo_world_cfg::mg_cluster
};
// One dispatch per half-sweep, restrict and prolong, as the reference records them.
void launch_multigrid(const Dev& d, const MgLevel* levels, int nlevels, const MgBufs& b, const MgConfig& c, cudaStream_t s);
// The same V-cycles, bit-identical: fused tile kernels per fine level and one
// shared-memory kernel for the coarse levels.  Usable when the coarsest level
// fits in shared memory and 1 <= pre <= 7, 1 <= post <= 8.
// Neighbour codes of every level (0: not water, else 1 + water neighbours)
// and the water flags of levels >= 1, from the level-0 flags; run after every
// wall-mask build.
void launch_mg_codes(const MgLevel* levels, int nlevels, const MgBufs& b, cudaStream_t s);
bool multigrid_fused_ok(const MgLevel* levels, int nlevels, const MgConfig& c);
int multigrid_first_coarse_level(const MgLevel* levels, int nlevels);
void launch_multigrid_fused(const Dev& d, const MgLevel* levels, int nlevels, const MgBufs& b, const MgConfig& c,
                            cudaStream_t s);
void launch_jacobi(const Dev& d, int iters, cudaStream_t s);

// The fused V-cycles of several worlds advanced together: every fine-level
// launch covers the tiles of that level in all worlds, and one coarse launch
// runs one CTA per world.  Built once per batch membership (device tables).
struct MgWorld {
  Dev d;  // pressure_a, divergence, mask, status of the world (fixed buffers)
  const MgLevel* levels;
  int nlevels;
  MgBufs b;
};
struct MgBatchPlan;
// Tile shape per fine level index: 0 = by level size (the one-world rule),
// 1 = 64x32 tiles everywhere, 2 = 32x16 tiles everywhere.
MgBatchPlan* multigrid_batch_plan(const MgWorld* worlds, int n, const MgConfig& c, const int* tile_mode, int nmodes,
                                  cudaStream_t s);
void multigrid_batch_free(MgBatchPlan* plan);
int multigrid_batch_levels(const MgBatchPlan* plan);  // fine level indices in the plan
void launch_multigrid_batch(const MgBatchPlan* plan, cudaStream_t s);
// Pre-smooth launches of one fine level index only (side-effect free: their
// outputs are rewritten before they are read in the next V-cycle); used to
// time tile shapes.
void launch_multigrid_batch_pre(const MgBatchPlan* plan, int level, cudaStream_t s);

// Buffers of the mixed-precision preconditioner V-cycle (owned by the world;
// see mixed.cu).  Fine level l (below the first coarse level) stores its
// right-hand side (l >= 1) and pre-smoothed correction as FP16 when
// l < nhalf, else FP32, and its total correction E (l >= 1) as FP32.
struct MpHierarchy {
  int nhalf;
  struct Fine {
    void* ef;
    void* rhs;
    float* E;
  } fine[16];
  const float* r;            // level-0 input: the CG residual
  const int* label;          // water component per fluid cell (-1: wall)
  const float* comp_mean;    // mean residual per component (FP32 copy of the FP64 mean)
  const float* scale;        // [0] scale, [1] inverse scale
  float* z;                  // level-0 output
  double* comp_sum_z;        // per-component sums of z (cells outside a tile's dominant component)
  double* part_c;            // per level-0 tile: sum of z over its dominant component
  int* part_dom;             // per level-0 tile: that component (-1: none)
  const double* coarse_inv;  // dense FP64 inverse of the coarsest operator
  float alpha;               // coarse-correction over-relaxation
  int pre, post;
};
// Sets the kernel attributes of the mixed V-cycle (call before capturing it).
void multigrid_prepare_mixed();
// Level-0 tiles of the mixed V-cycle's post pass (entries of part_c /
// part_dom it writes).
size_t mixed_vcycle_tiles(const MgLevel* levels, int nlevels, const MgConfig& c);
// Launches one V-cycle of the preconditioner; returns the number of level-0
// tiles (entries of part_c / part_dom it wrote).
int launch_mixed_vcycle(const Dev& d, const MgLevel* levels, int nlevels, const MgBufs& b, const MpHierarchy& h,
                        cudaStream_t s);

// transport.cu
void launch_slope(const Dev& d, float world_units_per_cell, cudaStream_t s);
void launch_thermal(const Target& t, cudaStream_t s);
void launch_agg(const Target& t, cudaStream_t s);
void launch_scatter(const Target& t, bool simple, cudaStream_t s);
// Zeroes chem_next of every world of the target (batched form of the memset).
void launch_zero_next(const Target& t, cudaStream_t s);
// Ledger of each world's current chem: 12 words at `out` (one world) or at
// out + 12 * w (world w of a batch).  The words must be zero beforehand.
void launch_ledger(const Target& t, uint32_t* out, cudaStream_t s);

}  // namespace ribo
