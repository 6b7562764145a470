// The World object behind the C handle (host side; see world.cu).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/ribo_world.h"
#include "ribo_dev.cuh"
#include "ribo_launch.h"

namespace ribo {

ribo_status set_error(ribo_status st, const char* fmt, ...);
ribo_status cuda_status(cudaError_t e, const char* what);

// Events bracketing each kernel launch of one step call (kernel timing).
struct KTimer {
  struct Rec {
    const char* label;
    double bytes;
    cudaEvent_t a, b;
  };
  std::vector<cudaEvent_t> pool;
  size_t used = 0;
  std::vector<Rec> recs;
  cudaEvent_t event();
  ~KTimer();
};

// Device bytes a world with configuration `c` allocates (defaults applied).
size_t world_footprint(const ribo_world_cfg& c);
// Bytes of field `f` of a world with configuration `c` (0: no such field).
size_t field_bytes_of(const ribo_world_cfg& c, ribo_field f);

struct World;
struct MixedSolver;
// Mixed-precision pressure solver of a world (mixed.cu).
ribo_status mixed_init(World& w);
ribo_status mixed_setup(World& w);
ribo_status mixed_solve(World& w);
ribo_status mixed_info(World& w, uint32_t* outer, uint32_t* inner, double* rho);
void mixed_free(World& w);
float* mixed_pressure_lo(World& w);
size_t mixed_footprint(const ribo_world_cfg& c, const std::vector<MgLevel>& levels);

uint64_t ktime_launch_count();
void ktime_add_launches(uint64_t n);
// Makes `t` (cleared) the timer of the following launches on this thread, or none.
void ktime_set_active(KTimer* t);
// Sums a finished timer's records per kernel name (its stream must be idle).
ribo_status ktimer_read(const KTimer& t, ribo_kernel_timing* out, uint32_t cap, uint32_t* count);

// A captured step sequence and the ping-pong state it leaves.
struct GraphEntry {
  std::string key;
  cudaGraphExec_t exec = nullptr;
  uint32_t *chem_end = nullptr;
  float *temp_end = nullptr, *redox_end = nullptr;
  uint64_t kernels = 0, uses = 0;
};

struct World {
  ribo_world_cfg cfg{};
  ribo_world_settings st{};
  int gw = 0, gh = 0, fw = 0, fh = 0;
  bool fluid_was_on = true;
  void* batch = nullptr;  // the ribo_batch this world belongs to (its work then runs on the batch's stream)
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  std::vector<void*> allocs;

  // environment resolution
  uint32_t *chem_a = nullptr, *chem_b = nullptr, *chem_cur = nullptr, *chem_nxt = nullptr;
  uint32_t* gamma = nullptr;
  float* light = nullptr;
  float* light_next = nullptr;  // light_propagate's output (light_mode 1)
  bool light_dirty = true;      // the next light block is a full sweep (creation, gamma upload, light turned on)
  uint32_t* shade = nullptr;
  float2* slope = nullptr;
  uint32_t* agg_nb = nullptr;
  // terrain grains (terrain_mode 1 and the brush)
  uint8_t* terrain_code = nullptr;
  uint8_t* terrain_arrivals = nullptr;
  uint32_t* terrain_list = nullptr;
  uint32_t* terrain_count = nullptr;
  TerrainBufs terrain_bufs() const {
    return TerrainBufs{gamma, terrain_code, terrain_arrivals, terrain_list, terrain_count};
  }
  // fluid resolution
  uint8_t* mask = nullptr;
  float2* normal = nullptr;
  float* curl = nullptr;
  void* tmaps = nullptr;  // TMA descriptors of the stencil passes' tiles (null: plain loads)
  uint32_t* mask32 = nullptr;
  float2 *va = nullptr, *vb = nullptr, *vsmooth = nullptr;
  float *pa = nullptr, *pb = nullptr, *div = nullptr;
  float *temp_a = nullptr, *temp_b = nullptr, *temp_cur = nullptr, *temp_nxt = nullptr;
  float *redox_a = nullptr, *redox_b = nullptr, *redox_cur = nullptr, *redox_nxt = nullptr;
  uint32_t* redox_eaten = nullptr;
  uint32_t* force_vec = nullptr;
  float2* forces = nullptr;
  float2* heat = nullptr;
  float* net_flux = nullptr;
  uint32_t* ledger = nullptr;
  uint32_t* step_ledgers = nullptr;  // 64 x 12 words (ledger_each_step)
  // asynchronous ledger readback (encode_ledger_readback / poll_ledger)
  uint32_t* ledger_async = nullptr;  // device, 12 words
  uint32_t* ledger_host = nullptr;   // pinned, 12 words (inside the pinned params block)
  cudaEvent_t ledger_ev = nullptr;
  bool ledger_pending = false;
  uint32_t last_steps = 0;
  // multigrid
  std::vector<MgLevel> levels;
  size_t mg_total = 0;
  size_t device_bytes = 0;  // sum of the world's device buffers
  MixedSolver* mixed = nullptr;      // precision_mode = RIBO_PRECISION_MIXED
  ribo_status solve_error = RIBO_OK;  // a pressure solve that failed to record
  MgBufs mg{};
  uint32_t* status = nullptr;  // kernel error bits (RIBO_ERR_*)
  // per-step parameters: two slots of 64 copies, device + pinned staging
  ribo_sim_params* d_params = nullptr;
  ribo_sim_params* h_params = nullptr;
  cudaEvent_t param_ev[2] = {nullptr, nullptr};
  int param_slot = 0;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  cudaEvent_t marks[8] = {};
  bool timing = false;
  KTimer timer;

  size_t cells() const { return (size_t)gw * gh; }
  size_t fcells() const { return (size_t)fw * fh; }
  size_t lcells() const { return (size_t)(gw / 2) * (gh / 2); }
  size_t field_bytes(ribo_field f) const;
  void* field_ptr(ribo_field f);
  Dev dev() const;

  ribo_status alloc(void** p, size_t bytes, const char* what);
  ribo_status init(const ribo_world_cfg& c);
  ~World();
  ribo_status upload(ribo_field f, const void* host, size_t bytes);
  ribo_status paint_terrain(float cx, float cy, float radius, uint32_t grains);
  // re-derives what the world keeps from gamma (slope, wall mask, the mixed
  // solver's setup) after gamma changed outside a step
  ribo_status terrain_changed();
  ribo_status read(ribo_field f, void* host, size_t bytes);
  ribo_status step(const ribo_sim_params* per_step, uint32_t n);
  ribo_status ledger_read(uint32_t out[12]);
  ribo_status ledger_request();
  ribo_status ledger_poll(uint32_t out[12], uint32_t* ready);
  ribo_status check_status();
  // CUDA-graph replay of repeated step sequences
  std::vector<GraphEntry> graphs;
  std::vector<std::string> seen_keys;
  std::string graph_key(const ribo_sim_params* per_step, uint32_t n, int slot) const;
  ribo_status record_steps_graphed(const ribo_sim_params* per_step, const ribo_sim_params* ds, uint32_t n, int slot);
  ribo_status read_timing(ribo_kernel_timing* out, uint32_t cap, uint32_t* count);
  void record_step(const ribo_sim_params& hp, const ribo_sim_params* P, uint32_t i);
  // light_mode 1: whether the light block of a step with these parameters is
  // a full sweep (else rows of propagation), given the dirty flag before it
  bool light_sweeps(const ribo_sim_params& hp, bool dirty) const;
  cudaError_t bind() const;
  void pressure_solve(const Dev& d);
};

}  // namespace ribo

// The C handle of a world.
struct ribo_world {
  ribo::World w;
};
