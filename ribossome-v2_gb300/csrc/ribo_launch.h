// Host-side launchers of the world-step kernels (one per pass).  The world
// orchestration in world.cu calls them in the reference's dispatch order.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include "ribo_dev.cuh"

namespace ribo {

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

// fluid.cu
void launch_solid_mask(const Dev& d, cudaStream_t s);
void launch_temperature(const Dev& d, const ribo_sim_params* P, cudaStream_t s);
void launch_forces(const Dev& d, const ribo_sim_params* P, cudaStream_t s);
void launch_add_forces(const Dev& d, const ribo_sim_params* P, const float2* vin, float2* vout, cudaStream_t s);
void launch_diffuse(const Dev& d, const ribo_sim_params* P, const float2* vin, float2* vout, cudaStream_t s);
void launch_advect(const Dev& d, const ribo_sim_params* P, const float2* vin, float2* vout, cudaStream_t s);
void launch_vorticity(const Dev& d, const ribo_sim_params* P, const float2* vin, float2* vout, cudaStream_t s);
void launch_divergence(const Dev& d, const float2* vin, cudaStream_t s);
void launch_subtract_gradient(const Dev& d, const float2* vin, float2* vout, cudaStream_t s);
void launch_net_flux(const Dev& d, const float2* vin, cudaStream_t s);
void launch_boundaries(const Dev& d, const float2* vin, float2* vout, cudaStream_t s);
void launch_smooth(const Dev& d, const float2* vin, cudaStream_t s);

// multigrid.cu
struct MgLevel {
  int nx, ny;
  size_t off;  // element offset of the level in the level arrays
  float eps;
};
// TMA tensor maps of one fine level of the fused V-cycle: the boxes the
// pre-smooth kernel loads (p only on level 0, rhs, water flags) and the
// boxes the post-smooth kernel loads (pre-smoothed p, rhs, water flags).
struct MgLevelMaps {
  CUtensorMap pre_p, pre_rhs, pre_fl, post_p, post_rhs, post_fl;
  int ok;
};
struct MgBufs {
  float* p;         // all levels, contiguous (64-element aligned level offsets)
  float* rhs;       // all levels
  uint8_t* fluid;   // all levels: 1 = water
  float* p_tmp;     // level-0 ping-pong partner of pressure_a (fused path)
  float* p2;        // all levels: pre-smoothed p (fused path)
  const MgLevelMaps* maps;  // host array, one per level, or null (plain loads)
};
struct MgConfig {
  int pre, post, coarse, cycles;
};
// One dispatch per half-sweep, restrict and prolong, as the reference records them.
void launch_multigrid(const Dev& d, const MgLevel* levels, int nlevels, const MgBufs& b, const MgConfig& c, cudaStream_t s);
// The same V-cycles, bit-identical: fused tile kernels per fine level and one
// shared-memory kernel for the coarse levels.  Usable when the coarsest level
// fits in shared memory and 1 <= pre, post <= 8.
bool multigrid_fused_ok(const MgLevel* levels, int nlevels, const MgConfig& c);
int multigrid_first_coarse_level(const MgLevel* levels, int nlevels);
// Encodes the tensor maps of the fine levels; false when some level cannot
// use TMA (its kernels then load with plain loads).
bool multigrid_make_maps(const MgLevel* levels, int nlevels, const MgConfig& c, const MgBufs& b, const Dev& d,
                         MgLevelMaps* out);
void launch_multigrid_fused(const Dev& d, const MgLevel* levels, int nlevels, const MgBufs& b, const MgConfig& c,
                            cudaStream_t s);
void launch_jacobi(const Dev& d, int iters, cudaStream_t s);

// transport.cu
void launch_slope(const Dev& d, float world_units_per_cell, cudaStream_t s);
void launch_thermal(const Dev& d, const ribo_sim_params* P, cudaStream_t s);
void launch_agg(const Dev& d, cudaStream_t s);
void launch_scatter(const Dev& d, const ribo_sim_params* P, bool simple, cudaStream_t s);
void launch_ledger(const Dev& d, const uint32_t* chem, uint32_t* out12, cudaStream_t s);

}  // namespace ribo
