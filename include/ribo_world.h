// C ABI of the GB300 world-step library (libribo_world.so).
//
// The library replaces the GPU side of the reference's world step: the
// `World` methods in src/world/mod.rs that own the device buffers and record
// the fluid / multigrid / transport / ledger dispatches.  Every entry point
// takes plain pointers and sizes; nothing here depends on CUDA or PyTorch
// headers.  A `ribo_world` handle is thread-affine (like the reference's
// `World`, which is not Sync): all calls on one handle come from one thread,
// and all device work of a handle is ordered on one CUDA stream.
#pragma once
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

// Status codes.  Setup errors in the reference are `Result<_, String>`
// (src/gpu/mod.rs:15-41); the text of the last error is kept per thread and
// returned by ribo_last_error().
typedef enum ribo_status {
  RIBO_OK = 0,
  RIBO_INVALID_ARG = 1,
  RIBO_OOM = 2,
  RIBO_OVER_BUDGET = 3,
  RIBO_TIMEOUT = 4,
  RIBO_CUDA_ERROR = 5,
} ribo_status;

// Per-step parameters: the reference's `SimParams` (src/params.rs:86-487),
// 116 four-byte fields in the same order and with the same names, 464 bytes.
// One copy per simulated step, as in the reference's uniform buffer
// (src/world/mod.rs:1431-1445).  Only the fields the world hot path reads are
// interpreted here; the others travel unchanged.
typedef struct ribo_sim_params {
  uint32_t  epoch;
  uint32_t  seed;
  float     dt;
  float     diffusion;
  float     settle;
  float     fluid_dt;
  float     fluid_decay;
  float     fluid_vorticity;
  float     fluid_viscosity;
  uint32_t  fumarole_count;
  float     uv_strength;
  float     uv_depth;
  uint32_t  fluid_enabled;
  float     fluid_obstacle_strength;
  float     slope_steer_rate;
  float     cohesion;
  uint32_t  spawn_count;
  uint32_t  max_agents;
  float     death_probability;
  float     spawn_energy;
  float     food_power;
  float     maintenance_cost;
  float     pairing_rate;
  float     mutation_rate;
  float     uv_damage;
  float     uptake_rate;
  float     brownian;
  float     phoretic_gain;
  float     chain_stiffness;
  float     thermal_kt;
  float     motor_amplitude;
  uint32_t  rft_enabled;
  uint32_t  require_start;
  float     joint_coupling;
  uint32_t  hunger_regulation;
  float     pairing_cost;
  float     reactivation_rate;
  float     swim_gain;
  float     bioturbation;
  float     bioturbation_cost;
  float     monomer_uv_absorb;
  float     sedimentation;
  float     direct_photoactivation;
  float     activation_decay;
  float     monomer_pressure;
  float     agent_fluid_push;
  float     swim_wobble;
  uint32_t  fluid_swim_only;
  float     motion_cost;
  float     bond_rate;
  float     bond_energy_share;
  float     bond_signal;
  float     aggregation;
  float     photo_yield;
  float     heat_kill;
  float     flow_coupling;
  float     inertia;
  float     death_energy_cap;
  float     chemo_yield;
  float     redox_decay;
  float     thermal_activation;
  float     denature_temp;
  float     day_period;
  float     sun_slope;
  float     sun_now;
  float     sun_angle;
  float     day_fraction;
  float     metabolic_q10;
  float     metabolic_span;
  float     metabolic_ref;
  float     sun_heat;
  float     sediment_transport;
  float     sediment_threshold;
  float     sediment_settle;
  float     signal_mode;
  float     clock_mute;
  float     paint_x;
  float     paint_y;
  float     paint_radius;
  float     paint_grains;
  float     rest_angle_mult;
  float     protease_power;
  float     lysis_yield;
  float     protease_direct;
  float     joint_load;
  float     swim_grip;
  float     swim_memory;
  float     mouth_leak;
  float     leak_base;
  float     skin_uptake;
  float     death_metab;
  float     salvage;
  float     bond_matter_share;
  float     brownian_rot;
  uint32_t  transport_every;
  float     signal_crosstalk;
  float     flow_mass;
  float     chemo_take;
  float     vent_cycle_period;
  float     vent_cycle_amp;
  float     sediment_cohesion;
  float     sediment_compaction;
  float     rock_crumble;
  float     lysis_matter;
  uint32_t  scramble_conduction;
  uint32_t  scramble_angles;
  uint32_t  scramble_response;
  float     scramble_amount;
  float     pairing_energy_half;
  float     pairing_min_energy;
  float     uv_mutation;
  float     heat_mutation;
  float     birth_crowding;
  float     photo_damage;
  float     naked_decay;
  float     store_loss;
} ribo_sim_params;

// World dimensions and multigrid constants.  The reference fixes a square
// GRID_SIZE / FLUID_SIZE at shader-compile time (src/shaders.rs:134-156,
// src/params.rs:1006-1034) and the multigrid constants as Rust consts
// (src/world/mod.rs:196-202); here they are runtime values.  grid_w/grid_h
// may differ (rectangular worlds); grid_w/fluid_w must equal grid_h/fluid_h
// and both must be integers >= 1.  Zero multigrid fields take the reference
// values MG_PRE=2, MG_POST=2, MG_COARSE=30, MG_MIN_SIZE=8.
typedef struct ribo_world ribo_world;

typedef struct ribo_world_cfg {
  uint32_t grid_w, grid_h;        // environment grid (GRID_SIZE)
  uint32_t fluid_w, fluid_h;      // fluid grid (FLUID_SIZE)
  uint32_t world_units_per_cell;  // 30 in WorldConfig::DEFAULT / TEST
  uint32_t mg_min_size;           // coarsest multigrid side (MG_MIN_SIZE)
  uint32_t mg_pre, mg_post;       // red-black sweeps before / after the coarse correction
  uint32_t mg_coarse;             // red-black sweeps on the coarsest level
  uint32_t precision_mode;        // RIBO_PRECISION_*
  uint32_t device;                // CUDA device ordinal the world lives on
  uint32_t no_graphs;             // 1 = never replay step sequences from CUDA graphs
  uint32_t mg_cluster;            // CTAs per cluster of the small multigrid levels' V-cycle launch:
                                  // 0 automatic (16, else 8, else none), 1 none (a launch per level
                                  // and the single-CTA coarse kernel), 8 or 16 that size where the
                                  // device can run it (else none); the same bits every way
  uint32_t reserved[3];
} ribo_world_cfg;

enum {
  RIBO_PRECISION_F32 = 0,    // the reference's arithmetic (bit-exact with the oracle)
  RIBO_PRECISION_MIXED = 1,  // fp16-storage fine-level smoothing, fp32 defect correction, fp64 coarse solve
};

// Host-side world settings that are not GPU parameters: the hot-path subset
// of the reference's `WorldSettings` (src/world/mod.rs:94-134).
typedef struct ribo_world_settings {
  uint32_t fluid_enabled;  // run the fluid block
  uint32_t fluid_substep;  // fluid every N steps with dt*N (clamped to 1..4)
  uint32_t multigrid;      // 1 = multigrid pressure, 0 = Jacobi
  uint32_t mg_cycles;      // V-cycles per fluid step (>= 1)
  uint32_t jacobi_iters;   // Jacobi iterations (rounded to even, 2..128)
  uint32_t ledger_each_step;  // 1 = run ledger_reduce after every step (read with ribo_world_step_ledgers)
  uint32_t mg_unfused;        // 1 = one dispatch per half-sweep (the reference's recording); 0 = fused kernels (same bits)
  uint32_t transport_simple;  // 1 = one thread per cell for the transport scatter; 0 = mover-parallel tiles (same bits)
  // Mixed-precision pressure solve (precision_mode = RIBO_PRECISION_MIXED;
  // zero fields take the defaults in brackets):
  float mixed_tol;            // relative residual ||rhs - L p|| / ||rhs|| to reach [1e-5]
  float mixed_inner_tol;      // residual reduction of one inner conjugate-gradient solve [1e-3]
  uint32_t mixed_max_outer;   // defect-correction steps at most [4]
  uint32_t mixed_max_inner;   // conjugate-gradient iterations per step at most [64]
  float mixed_alpha;          // over-relaxation of the V-cycle's coarse correction [1.8]
  // UV light (shaders/world/light.wgsl, src/world/mod.rs:1505-1524):
  uint32_t light_mode;           // 0 = the LIGHT field is a frozen input [default]; 1 = the reference's light
                                 // block runs before the fluid block of every step
  uint32_t light_rows_per_step;  // light_mode 1: rows the light propagates per step (at most 16); 0 = a full
                                 // sweep every light_interval steps [1]
  uint32_t light_interval;       // steps between full sweeps when light_rows_per_step = 0 [10]
  // Terrain grains (shaders/world/terrain.wgsl:135-460, src/world/mod.rs:1497-1504):
  uint32_t terrain_mode;  // 0 = GAMMA is a frozen input [default]; 1 = the reference's terrain block (two
                          // relax passes, grain_fall when sediment_settle > 0, the slope) opens every step
                          // and the wall mask is rebuilt at every fluid step.  Single worlds with the
                          // f32 pressure solve only (batches and mixed precision reject it).
} ribo_world_settings;

// Device fields a caller can upload / read.  Sizes in bytes, for a world with
// C = grid_w*grid_h env cells, F = fluid_w*fluid_h fluid cells and
// L = (grid_w/2)*(grid_h/2) light cells.
typedef enum ribo_field {
  RIBO_FIELD_CHEM = 0,           // C*16: 4 u32 per cell (A,U,G,C), low 16 bits activated, high 16 spent
  RIBO_FIELD_GAMMA = 1,          // C*4:  grains per cell (>= 3 rock)
  RIBO_FIELD_LIGHT = 2,          // 2*L*4: UV light, two bands (frozen input)
  RIBO_FIELD_SLOPE = 3,          // C*8:  terrain slope (derived from GAMMA on upload)
  RIBO_FIELD_VELOCITY = 4,       // F*8:  velocity_a (final velocity of a step)
  RIBO_FIELD_PRESSURE = 5,       // F*4:  pressure_a (warm start of the next solve)
  RIBO_FIELD_TEMP = 6,           // F*4:  temperature (temp_in)
  RIBO_FIELD_REDOX = 7,          // F*4:  vent reductant (redox_in)
  RIBO_FIELD_HEAT = 8,           // F*8:  vent heat / chemistry source per fluid cell
  RIBO_FIELD_VEL_SMOOTH = 9,     // F*8:  5-point smoothed final velocity
  RIBO_FIELD_SOLID_MASK = 10,    // F*4:  1 = wall (derived from GAMMA)
  RIBO_FIELD_DIVERGENCE = 11,    // F*4:  last divergence
  RIBO_FIELD_FORCE_VECTORS = 12, // F*8:  fixed-point (x256) force accumulators (agent pushes)
  RIBO_FIELD_REDOX_EATEN = 13,   // F*4:  fixed-point reductant consumed by agents
  RIBO_FIELD_NET_FLUX = 14,      // (fluid_h+fluid_w)*4: row means of v_y then column means of v_x
  RIBO_FIELD_SHADE = 15,         // 2*L*4: agent shade per light cell (fixed point, 100 = one)
  RIBO_FIELD_PRESSURE_LO = 16,   // F*4:  mixed precision only: pressure = PRESSURE + PRESSURE_LO (read-only)
  RIBO_FIELD_COUNT = 17,
} ribo_field;

// Last error text of the calling thread ("" if none).
const char* ribo_last_error(void);

// The reference defaults of SimParams (src/params.rs:553-690) and
// WorldSettings (src/world/mod.rs:117-134).
void ribo_sim_params_default(ribo_sim_params* out);
void ribo_world_settings_default(ribo_world_settings* out);

// World::new (src/world/mod.rs:416): allocates every device buffer of the
// world step, zeroed.  Fails with RIBO_INVALID_ARG on bad sizes and RIBO_OOM
// when device memory runs out.
ribo_status ribo_world_create(const ribo_world_cfg* cfg, ribo_world** out);
void ribo_world_destroy(ribo_world* w);

// Device bytes ribo_world_create allocates for `cfg` (no counterpart in the
// reference; admission control of ribo_server uses it), and the bytes a
// created world holds.  No GPU needed for the first.
ribo_status ribo_world_footprint(const ribo_world_cfg* cfg, uint64_t* bytes);
ribo_status ribo_world_memory(const ribo_world* w, uint64_t* bytes);

ribo_status ribo_world_set_settings(ribo_world* w, const ribo_world_settings* s);
ribo_status ribo_world_get_settings(const ribo_world* w, ribo_world_settings* out);

// queue.write_buffer on a world buffer (seed_matter, src/world/mod.rs:969-988):
// copies `bytes` (must equal the field size) from host memory.  Uploading
// GAMMA recomputes the slope and the fluid wall mask.
ribo_status ribo_world_upload(ribo_world* w, ribo_field field, const void* host, size_t bytes);

// World::encode_paint (src/world/mod.rs:1220-1241) with paint_terrain
// (shaders/world/terrain.wgsl:385-413): `grains` (at most 6) grains in every
// cell whose centre lies in the disc (centre and radius in cells), the
// monomers that no longer fit evicted to a neighbour with room, in the
// order of the terrain block (all stores, then the eviction loops by
// 3 x 3 class of the cell).  The slope and wall mask are re-derived and the
// next light block sweeps.
ribo_status ribo_world_paint_terrain(ribo_world* w, float cx, float cy, float radius, uint32_t grains);

// read_cells_blocking / read_f32_blocking (src/world/mod.rs:1801-1809):
// waits for the world's stream, then copies the field to host memory.
ribo_status ribo_world_read(ribo_world* w, ribo_field field, void* host, size_t bytes);

// The device address and size of a field (for zero-copy callers on the same
// device).  The pointer stays valid until ribo_world_destroy.
ribo_status ribo_world_device_ptr(ribo_world* w, ribo_field field, void** dptr, size_t* bytes);

// Records `n` steps (1..64) with explicit per-step parameters, asynchronously
// on the world's stream: the dispatch sequence of World::encode_steps
// (src/world/mod.rs:1487-1601) for the fluid and transport blocks.  The fluid
// block runs when settings.fluid_enabled and epoch % fluid_substep == 0; the
// transport block when epoch % transport_every == 0.
ribo_status ribo_world_step(ribo_world* w, const ribo_sim_params* per_step, uint32_t n);

// World::encode_steps (src/world/mod.rs:1406-1632): derives the per-step
// copies from `params` (epoch + i, fluid_dt = dt * substep, fluid_enabled from
// the settings, sun_now / sun_slope from the day cycle), records them, and
// advances params->epoch by `steps` (at most 64 per call, as MAX_STEPS_PER_FRAME).
ribo_status ribo_world_encode_steps(ribo_world* w, ribo_sim_params* params, uint32_t steps);

// The per-step copies World::encode_steps would write for `steps` steps
// starting at base->epoch (out must hold `steps` entries).
ribo_status ribo_derive_step_params(const ribo_sim_params* base, const ribo_world_settings* settings,
                                    uint32_t steps, ribo_sim_params* out);

// ledger_blocking (src/world/mod.rs:1834-1839, shaders/world/ledger.wgsl):
// exact per-channel sums [activated A U G C, spent A U G C, held A U G C]
// (held is 0: no agents on this path).  Waits for the world's stream.
ribo_status ribo_world_ledger(ribo_world* w, uint32_t out[12]);

// Asynchronous ledger (encode_ledger_readback + ledger_after_submit /
// poll_ledger, src/world/mod.rs:1758-1799): request records the reduction
// and its copy to pinned host memory on the world's stream, behind the work
// recorded so far, and returns at once (a request while one is pending does
// nothing); poll never waits: *ready = 1 and the ledger in `out` once the
// readback has arrived (the readback is then over), else *ready = 0.
ribo_status ribo_world_request_ledger(ribo_world* w);
ribo_status ribo_world_poll_ledger(ribo_world* w, uint32_t out[12], uint32_t* ready);

// With settings.ledger_each_step, the ledger of the state after each step of
// the last ribo_world_step / encode_steps call (12 words per step, `n` steps
// of that call).  Waits for the world's stream.
ribo_status ribo_world_step_ledgers(ribo_world* w, uint32_t* out, uint32_t n);

// Records timing mark `slot` (0..7) on the world's stream, and the device
// time between two recorded marks in ms (waits for the second).
ribo_status ribo_world_mark(ribo_world* w, uint32_t slot);
ribo_status ribo_world_elapsed_ms(ribo_world* w, uint32_t slot_a, uint32_t slot_b, float* ms);

// Waits until all work recorded on the world's stream has finished.
// Kernels do not trap: a wait that gave up (a TMA that never completed)
// sets a bit in the world's status word, which this call reads and clears,
// returning RIBO_TIMEOUT (the last steps' results are then invalid).
ribo_status ribo_world_sync(ribo_world* w);

// Diagnostics (no counterpart in the reference).  ribo_world_raise_status
// ORs `bits` into the world's status word on its stream, as a kernel whose
// wait gave up would: the next ribo_world_sync reports RIBO_TIMEOUT (host
// side of the error path, testable without a GPU fault).
// ribo_selftest_bounded_wait runs one CTA on `device` that waits, at most
// `polls` polls, on an mbarrier phase that nothing completes, the form every
// TMA wait of the library takes; it stores the status bits the kernel
// recorded (RIBO_ERR_TIMEOUT = 1 expected) in *status_bits and returns
// RIBO_OK when the context is still usable afterwards.
ribo_status ribo_world_raise_status(ribo_world* w, uint32_t bits);
ribo_status ribo_selftest_bounded_wait(uint32_t device, uint32_t polls, uint32_t* status_bits);

// Device time of the last ribo_world_step / encode_steps call, in ms (CUDA
// events on the world's stream; waits for it).
ribo_status ribo_world_last_step_ms(ribo_world* w, float* ms);

// Per-kernel GPU timing, the counterpart of World::enable_kernel_timing /
// read_kernel_timing (src/world/mod.rs:1056-1098): when enabled, every
// kernel of the following ribo_world_step / encode_steps call is bracketed
// by CUDA events on the world's stream.  read_kernel_timing waits for the
// stream and returns one entry per kernel name, summed over that call:
// launches, milliseconds and the algorithmic bytes (compulsory reads +
// writes) those launches move.
typedef struct ribo_kernel_timing {
  char name[40];
  uint32_t launches;
  float ms;
  double bytes;
} ribo_kernel_timing;
ribo_status ribo_world_enable_kernel_timing(ribo_world* w, int enable);
ribo_status ribo_world_read_kernel_timing(ribo_world* w, ribo_kernel_timing* out, uint32_t cap, uint32_t* count);

// Number of kernels this library has launched in this process so far.
uint64_t ribo_kernel_launch_count(void);

// Mixed-precision worlds: statistics of the last pressure solve -- outer
// defect-correction steps, conjugate-gradient iterations in total, and the
// relative residual ||rhs - L(p_hi + p_lo)|| / ||rhs|| of the pressure it
// left (evaluated on the device in FP32-pair arithmetic).  Waits.  No
// counterpart in the reference.
ribo_status ribo_world_solve_info(ribo_world* w, uint32_t* outer, uint32_t* inner, double* rel_residual);

// ---- Batches: many worlds advanced together ---------------------------------
// No single counterpart in the reference, whose World::encode_steps
// (src/world/mod.rs:1406-1632) advances one world per call; a batch runs that
// same dispatch sequence for all of its member worlds in lock step.  Every
// pass of a step is one launch over the tiles of all members (worlds of
// different sizes and shapes); the multigrid V-cycle is one launch per level
// index plus one coarse launch with a CTA per world; repeated step sequences
// replay from one CUDA graph.  Each member's results are the same bits as
// when it is stepped alone with the same parameters.  Members whose schedule
// differs in a step (fluid substep parity, transport_every, settings) are
// grouped and each group gets its own launches.  While a world is a member,
// all of its work -- its own ribo_world_* calls included -- runs in order on
// the batch's stream.  Members must live on the batch's device; a world
// belongs to at most one batch.
typedef struct ribo_batch ribo_batch;
ribo_status ribo_batch_create(uint32_t device, ribo_batch** out);
// Releases the members (it does not destroy them) and frees the batch.
void ribo_batch_destroy(ribo_batch* b);
ribo_status ribo_batch_add(ribo_batch* b, ribo_world* w);
ribo_status ribo_batch_remove(ribo_batch* b, ribo_world* w);
uint32_t ribo_batch_size(const ribo_batch* b);
// Records `n` steps (1..64) of every member, asynchronously on the batch's
// stream.  per_step[k * n + i] holds the parameters of step i of the k-th
// member (membership order: the order of ribo_batch_add, less removals).
ribo_status ribo_batch_step(ribo_batch* b, const ribo_sim_params* per_step, uint32_t n);
// As ribo_batch_step, but member k runs only the first member_steps[k] (<= n)
// of its n entries; the others leave it untouched.
ribo_status ribo_batch_step_ragged(ribo_batch* b, const ribo_sim_params* per_step, uint32_t n,
                                   const uint32_t* member_steps);
// ribo_world_encode_steps for every member: params[k] is the k-th member's
// SimParams; the per-step copies are derived from it with that member's
// settings, and params[k].epoch advances by `n`.
ribo_status ribo_batch_encode_steps(ribo_batch* b, ribo_sim_params* params, uint32_t n);
// Ledgers after each step of the last ribo_batch_step / encode_steps call:
// out[(k * n + i) * 12 + c] for member k, step i (members whose settings
// have ledger_each_step; other members' entries are zero).  Waits.
ribo_status ribo_batch_step_ledgers(ribo_batch* b, uint32_t* out, uint32_t n);
// Waits for the batch's stream and checks every member's kernel status.
ribo_status ribo_batch_sync(ribo_batch* b);
// Timing marks on the batch's stream, as ribo_world_mark / elapsed_ms.
ribo_status ribo_batch_mark(ribo_batch* b, uint32_t slot);
ribo_status ribo_batch_elapsed_ms(ribo_batch* b, uint32_t slot_a, uint32_t slot_b, float* ms);
// Tile-shape autotuner of the batched multigrid kernels: for every fine
// level index it times the candidate tile shapes (by level size, 64x32
// everywhere, 32x16 everywhere) on the members' current state with CUDA
// events and keeps the fastest.  Tile shapes never change results (the
// fused smoothers are bit-identical to one dispatch per half-sweep).
// modes_out (optional, 8 entries) receives the choice per level index:
// 0 = by level size, 1 = 64x32, 2 = 32x16.
ribo_status ribo_batch_autotune(ribo_batch* b, uint32_t* modes_out);
// Sets the tile shape per fine level index explicitly (modes as above; level
// indices past n use 0).
ribo_status ribo_batch_set_tile_modes(ribo_batch* b, const uint32_t* modes, uint32_t n);
// Per-kernel timing of the next ribo_batch_step calls (as for a world).
ribo_status ribo_batch_enable_kernel_timing(ribo_batch* b, int enable);
ribo_status ribo_batch_read_kernel_timing(ribo_batch* b, ribo_kernel_timing* out, uint32_t cap, uint32_t* count);

// ---- Serving: world-step jobs with continuous batching ----------------------
// No counterpart in the reference.  A server keeps a FIFO of submitted jobs
// (a world, its settings and SimParams, a step count, its initial fields)
// and a batch of resident worlds.  Each iteration (1) retires the jobs that
// have run all their steps -- reads their results into the caller's
// buffers, frees their worlds --, (2) admits queued jobs in arrival order
// while their device footprint fits the HBM budget (and the resident
// count stays under max_active), creating and uploading their worlds, and
// (3) advances every resident job by up to max_chunk_steps steps in one
// ragged batched call (a job never runs past its step count).  Jobs that
// arrive while others run join at the next iteration: their work overlaps
// with the others' in the same launches.  A job's results are the same bits
// as when its world is stepped alone with ribo_world_encode_steps.
typedef struct ribo_server ribo_server;

typedef struct ribo_server_cfg {
  uint32_t device;
  uint32_t max_chunk_steps;   // steps per iteration (1..64)
  uint32_t max_active;        // resident jobs at most (0 = limited by the budget only)
  uint32_t reserved0;
  uint64_t hbm_budget_bytes;  // device bytes the resident worlds may hold (ribo_world_footprint)
  uint64_t reserved[2];
} ribo_server_cfg;

typedef struct ribo_job {
  ribo_world_cfg world;
  ribo_world_settings settings;
  ribo_sim_params params;  // the base SimParams; per-step copies as ribo_world_encode_steps derives them
  uint32_t steps;          // steps to run (>= 1)
  uint32_t reserved0;
  uint64_t user_tag;
  // Initial fields (host memory, ribo_world_upload sizes; null = zero),
  // copied by ribo_server_submit.  GAMMA is uploaded first.
  const void* inputs[RIBO_FIELD_COUNT];
  // Result fields: host buffers of ribo_world_read sizes, filled when the job
  // retires (null = not read).  They must stay valid until then.
  void* outputs[RIBO_FIELD_COUNT];
} ribo_job;

typedef struct ribo_job_result {
  uint64_t id;
  uint64_t user_tag;
  int32_t status;          // ribo_status of the job
  uint32_t steps;
  uint32_t ledger[12];     // ledger of the final state
  uint64_t device_bytes;   // footprint the job held while resident
  double t_submit_ms;      // host clock, ms since the server was created
  double t_admit_ms;
  double t_done_ms;        // when the iteration that retired it observed its last step done
} ribo_job_result;

typedef struct ribo_server_stats {
  uint64_t submitted, admitted, completed, pending, active;
  uint64_t bytes_in_use;   // footprint of the resident worlds
  uint64_t world_steps;    // job steps run so far
  uint64_t iterations;
  double gpu_ms;           // device time of the batched calls so far
} ribo_server_stats;

ribo_status ribo_server_create(const ribo_server_cfg* cfg, ribo_server** out);
// Destroys the server and every world it holds; results not yet taken are lost.
void ribo_server_destroy(ribo_server* s);
// Queues a job; its id is written to *id.  RIBO_OVER_BUDGET when the job's
// footprint alone exceeds the budget, RIBO_INVALID_ARG on a bad job.
ribo_status ribo_server_submit(ribo_server* s, const ribo_job* job, uint64_t* id);
// One iteration (retire, admit, advance); *active = resident jobs after it.
ribo_status ribo_server_iterate(ribo_server* s, uint32_t* active);
// Iterates until no job is queued or resident.
ribo_status ribo_server_drain(ribo_server* s);
// Moves up to `cap` finished results to `out` (oldest first); *n = moved.
ribo_status ribo_server_results(ribo_server* s, ribo_job_result* out, uint32_t cap, uint32_t* n);
ribo_status ribo_server_get_stats(const ribo_server* s, ribo_server_stats* out);
// Per-iteration records since the last call (oldest first, at most cap):
// device ms of the iteration's batched call, its steps and resident jobs.
ribo_status ribo_server_iterations(ribo_server* s, float* ms, uint32_t* steps, uint32_t* active, uint32_t cap,
                                   uint32_t* n);

// Allocation-free multigrid pressure solve.  No counterpart in the reference:
// it exists for callers that cannot allocate device memory while they run
// (a host that reserves its whole device budget at start-up and forbids
// later allocations, or a frame loop that cannot absorb the synchronisation
// cudaMalloc/cudaFree may cause).  It performs the world step's pressure
// solve -- the same multigrid V-cycles, bit for bit -- on caller-owned
// device buffers of fluid_w x fluid_h cells: divergence (f32), solid mask
// (u32, 1 = wall) and pressure (f32, warm start in, result out).  The
// multigrid hierarchy lives in a fixed ~6.2 MB array inside the library
// that every GPU loading the library holds until the process exits; grids
// above 512 x 512 cells are rejected with RIBO_INVALID_ARG.  It calls no
// allocation routine.  The call is asynchronous on `cuda_stream` (0 = the
// legacy default stream) on the calling thread's current device.  Its first
// call on a device looks up the array's device address (once per device);
// make that first call before any stream capture.  All calls share the one
// array, so calls whose work overlaps on the GPU (other streams, other host
// threads) race and must be serialised by the caller.  Zero multigrid
// arguments take the reference values (8, 2, 2, 30, 1).
ribo_status ribo_pressure_solve_noalloc(uint32_t fluid_w, uint32_t fluid_h, const float* d_divergence,
                                        const uint32_t* d_solid_mask, float* d_pressure, uint32_t mg_min_size,
                                        uint32_t mg_pre, uint32_t mg_post, uint32_t mg_coarse, uint32_t mg_cycles,
                                        void* cuda_stream);

// Scene files: World::save_scene / Scene::read + World::load_scene
// (src/world/snapshot.rs:274-368, 145-167, 372-553) for the world blocks of
// this path.  The file is the reference's `.ribo` container ("RIBOSCN1", JSON
// header, LZ4 blocks): the header's cfg, params (SimParams by field name) and
// settings, the blocks chem, gamma, velocity, pressure, temperature and
// redox, zero agents (empty agent blocks, so the reference can load the
// file into a world of the same size), and this path's frozen inputs (vent
// heat, light, shade) as extra blocks the reference ignores.  save waits for
// the world's stream and writes `path` through a temporary file.  load
// accepts the reference's scenes: the sizes must match this world's
// (RIBO_INVALID_ARG otherwise), unknown parameter names are ignored and
// missing ones take the defaults (ribo_sim_params_default); it uploads the
// blocks (gamma first: slope and wall mask are rebuilt), sets the world's
// settings from the header, fills `params` (may be null) and leaves the
// fields the file lacks (e.g. light and heat of a reference scene) as they
// were.
ribo_status ribo_world_save_scene(ribo_world* w, const char* path, const ribo_sim_params* params);
ribo_status ribo_world_load_scene(ribo_world* w, const char* path, ribo_sim_params* params);

// SimParams field `i` (0..115) by the reference's name (src/params.rs:71-81,
// the names of to_named / set_named), or NULL past the last.
const char* ribo_sim_param_name(uint32_t i);

// The LZ4 block coder of the scene files (published LZ4 block format, the
// blocks lz4_flex's compress_prepend_size writes after its 4-byte length).
// compress writes at most ribo_lz4_compress_bound(n) bytes; decompress
// fails with RIBO_INVALID_ARG on malformed input or a short output buffer.
size_t ribo_lz4_compress_bound(size_t n);
ribo_status ribo_lz4_compress(const void* src, size_t n, void* dst, size_t cap, size_t* written);
ribo_status ribo_lz4_decompress(const void* src, size_t n, void* dst, size_t cap, size_t* written);

#ifdef __cplusplus
}  // extern "C"
#endif
