// Host side of the world step: buffer ownership, the per-step dispatch order
// and the C ABI declared in include/ribo_world.h.
//
// Restates the GPU half of the reference's `World` (src/world/mod.rs):
// World::new allocates the buffers (:416-932), encode_steps records the
// fluid and transport blocks of every step (:1406-1632) and ledger_blocking /
// read_*_blocking read results back (:1801-1839).  Ping-pong buffers that the
// reference copies back every step (temperature, redox, chem_next) are
// swapped by pointer instead.
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <string>
#include <vector>

#include "../../include/ribo_world.h"
#include "ribo_dev.cuh"
#include "ribo_launch.h"
#include "ribo_world_impl.h"

namespace ribo {

thread_local std::string g_last_error;

ribo_status set_error(ribo_status st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return st;
}

ribo_status cuda_status(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return RIBO_OK;
  cudaGetLastError();  // clear sticky-free errors
  if (e == cudaErrorMemoryAllocation) return set_error(RIBO_OOM, "%s: out of device memory", what);
  return set_error(RIBO_CUDA_ERROR, "%s: %s", what, cudaGetErrorString(e));
}

#define RB_TRY(expr, what)                               \
  do {                                                   \
    ribo_status _st = cuda_status((expr), (what));       \
    if (_st != RIBO_OK) return _st;                      \
  } while (0)

static const uint32_t MAX_STEPS = 64;

// ---- per-launch instrumentation (RB_LAUNCH) ----
static std::atomic<uint64_t> g_launches{0};
static thread_local KTimer* g_active_timer = nullptr;

void ktime_begin(const char* label, double bytes, cudaStream_t s) {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  KTimer* t = g_active_timer;
  if (!t) return;
  KTimer::Rec r{label, bytes, t->event(), t->event()};
  cudaEventRecord(r.a, s);
  t->recs.push_back(r);
}

void ktime_end(cudaStream_t s) {
  KTimer* t = g_active_timer;
  if (!t || t->recs.empty()) return;
  cudaEventRecord(t->recs.back().b, s);
}

uint64_t ktime_launch_count() { return g_launches.load(std::memory_order_relaxed); }
void ktime_set_active(KTimer* t) {
  if (t) {
    t->recs.clear();
    t->used = 0;
  }
  g_active_timer = t;
}
void ktime_add_launches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

cudaEvent_t KTimer::event() {
  if (used == pool.size()) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    pool.push_back(e);
  }
  return pool[used++];
}

KTimer::~KTimer() {
  for (cudaEvent_t e : pool) cudaEventDestroy(e);
}

size_t World::field_bytes(ribo_field f) const { return field_bytes_of(cfg, f); }

size_t field_bytes_of(const ribo_world_cfg& c, ribo_field f) {
  const size_t C = (size_t)c.grid_w * c.grid_h, F = (size_t)c.fluid_w * c.fluid_h;
  const size_t L = (size_t)(c.grid_w / 2) * (c.grid_h / 2);
  const size_t fw = c.fluid_w, fh = c.fluid_h;
  switch (f) {
    case RIBO_FIELD_CHEM: return C * 16;
    case RIBO_FIELD_GAMMA: return C * 4;
    case RIBO_FIELD_LIGHT: return 2 * L * 4;
    case RIBO_FIELD_SLOPE: return C * 8;
    case RIBO_FIELD_VELOCITY: return F * 8;
    case RIBO_FIELD_PRESSURE: return F * 4;
    case RIBO_FIELD_TEMP: return F * 4;
    case RIBO_FIELD_REDOX: return F * 4;
    case RIBO_FIELD_HEAT: return F * 8;
    case RIBO_FIELD_VEL_SMOOTH: return F * 8;
    case RIBO_FIELD_SOLID_MASK: return F * 4;
    case RIBO_FIELD_DIVERGENCE: return F * 4;
    case RIBO_FIELD_FORCE_VECTORS: return F * 8;
    case RIBO_FIELD_REDOX_EATEN: return F * 4;
    case RIBO_FIELD_NET_FLUX: return (fw + fh) * 4;
    case RIBO_FIELD_SHADE: return 2 * L * 4;
    case RIBO_FIELD_PRESSURE_LO: return F * 4;
    default: return 0;
  }
}

void* World::field_ptr(ribo_field f) {
  switch (f) {
    case RIBO_FIELD_CHEM: return chem_cur;
    case RIBO_FIELD_GAMMA: return gamma;
    case RIBO_FIELD_LIGHT: return light;
    case RIBO_FIELD_SLOPE: return slope;
    case RIBO_FIELD_VELOCITY: return va;
    case RIBO_FIELD_PRESSURE: return pa;
    case RIBO_FIELD_TEMP: return temp_cur;
    case RIBO_FIELD_REDOX: return redox_cur;
    case RIBO_FIELD_HEAT: return heat;
    case RIBO_FIELD_VEL_SMOOTH: return vsmooth;
    case RIBO_FIELD_SOLID_MASK: return nullptr;  // stored as bytes; converted on read
    case RIBO_FIELD_DIVERGENCE: return div;
    case RIBO_FIELD_FORCE_VECTORS: return force_vec;
    case RIBO_FIELD_REDOX_EATEN: return redox_eaten;
    case RIBO_FIELD_NET_FLUX: return net_flux;
    case RIBO_FIELD_SHADE: return shade;
    case RIBO_FIELD_PRESSURE_LO: return mixed_pressure_lo(*this);
    default: return nullptr;
  }
}

Dev World::dev() const {
  Dev d{};  // every byte set: batches key their tables on Dev records
  d.gw = gw;
  d.gh = gh;
  d.fw = fw;
  d.fh = fh;
  d.lw = gw / 2;
  d.lh = gh / 2;
  d.rx = gw / fw;
  d.ry = gh / fh;
  d.sx = (float)gw / (float)fw;
  d.sy = (float)gh / (float)fh;
  d.sim_w = (float)(gw * cfg.world_units_per_cell);
  d.sim_h = (float)(gh * cfg.world_units_per_cell);
  d.cell_w = (float)cfg.world_units_per_cell;
  d.wpf_x = d.sim_w / (float)fw;
  d.wpf_y = d.sim_h / (float)fh;
  d.chem = chem_cur;
  d.chem_next = chem_nxt;
  d.gamma = gamma;
  d.light = light;
  d.light_next = light_next;
  d.shade = shade;
  d.slope = slope;
  d.agg_nb = agg_nb;
  d.mask = mask;
  d.normal = normal;
  d.curl = curl;
  d.va = va;
  d.vb = vb;
  d.vsmooth = vsmooth;
  d.pa = pa;
  d.pb = pb;
  d.div = div;
  d.temp_in = temp_cur;
  d.temp_out = temp_nxt;
  d.redox_in = redox_cur;
  d.redox_out = redox_nxt;
  d.redox_eaten = redox_eaten;
  d.force_vec = force_vec;
  d.forces = forces;
  d.heat = heat;
  d.net_flux = net_flux;
  d.ledger = ledger;
  d.fluid0 = (mg.fluid && !levels.empty()) ? mg.fluid + levels[0].off : nullptr;
  d.status = status;
  d.tmap = tmaps;
  return d;
}

// World buffers come from the device's stream-ordered pool: creating and
// destroying worlds (a server admits and retires them continuously) then
// neither synchronises the device nor returns memory to the driver.
ribo_status World::alloc(void** p, size_t bytes, const char* what) {
  cudaError_t e = cudaMallocAsync(p, bytes, own_stream);
  if (e != cudaSuccess) return cuda_status(e, what);
  allocs.push_back(*p);
  device_bytes += bytes;
  e = cudaMemsetAsync(*p, 0, bytes, own_stream);
  return cuda_status(e, what);
}

static void keep_pool_memory(int dev) {
  static DeviceOnce once;
  if (!once.pending(dev & 63)) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  cudaGetLastError();
  once.done(dev & 63);
}

// Multigrid levels (src/world/mod.rs:637-671): halve while both sides are
// above the minimum and even; eps = MG_EPS * 2^l.  Returns the elements of
// the level arrays (64-element aligned level bases).
static size_t build_levels(int fw, int fh, uint32_t min_size, std::vector<MgLevel>& levels) {
  levels.clear();
  int nx = fw, ny = fh, l = 0;
  size_t off = 0;
  for (;;) {
    levels.push_back(MgLevel{nx, ny, off, (float)1e-4 * (float)(1u << l)});
    off += ((size_t)nx * ny + 63) & ~(size_t)63;
    if ((uint32_t)nx > min_size && (uint32_t)ny > min_size && nx % 2 == 0 && ny % 2 == 0) {
      nx /= 2;
      ny /= 2;
      l++;
    } else {
      break;
    }
  }
  return off;
}

// Device bytes World::init allocates for `c` (the sum of its buffers).
size_t world_footprint(const ribo_world_cfg& c) {
  const size_t C = (size_t)c.grid_w * c.grid_h, F = (size_t)c.fluid_w * c.fluid_h;
  const size_t L = (size_t)(c.grid_w / 2) * (c.grid_h / 2);
  std::vector<MgLevel> lv;
  const size_t M = build_levels((int)c.fluid_w, (int)c.fluid_h, c.mg_min_size ? c.mg_min_size : 8, lv);
  size_t b = 0;
  b += C * (16 + 16 + 4 + 8 + 4);                                 // chem a/b, gamma, slope, agg_nb
  b += 2 * C + terrain_list_entries((int)c.grid_w, (int)c.grid_h) * 4 + 64;  // terrain codes, arrivals, lists, counts
  b += 2 * L * 4 * 3;                                             // light, light_next, shade
  b += F * (1 + 8 + 4 + 8 * 3 + 4 * 3 + 4 * 5 + 8 * 3 + 4 + 4);  // mask..heat, mask32, p_tmp
  b += ((size_t)c.fluid_w + c.fluid_h) * 4 + 12 * 4 * 2 + MAX_STEPS * 12 * 4 + 16;
  b += M * (4 + 4 + 1 + 4 + 1);                                   // mg p, rhs, fluid, p2, code
  b += 2 * MAX_STEPS * sizeof(ribo_sim_params);
  b += STENCIL_TMAP_BYTES_HOST;                                   // TMA descriptor of the stencil passes
  if (c.precision_mode == RIBO_PRECISION_MIXED) b += mixed_footprint(c, lv);
  return b;
}

ribo_status World::init(const ribo_world_cfg& c) {
  cfg = c;
  if (!cfg.world_units_per_cell) cfg.world_units_per_cell = 30;
  if (!cfg.mg_min_size) cfg.mg_min_size = 8;
  if (!cfg.mg_pre) cfg.mg_pre = 2;
  if (!cfg.mg_post) cfg.mg_post = 2;
  if (!cfg.mg_coarse) cfg.mg_coarse = 30;
  gw = (int)cfg.grid_w;
  gh = (int)cfg.grid_h;
  fw = (int)cfg.fluid_w;
  fh = (int)cfg.fluid_h;
  ribo_world_settings_default(&st);
  RB_TRY(bind(), "device");
  keep_pool_memory((int)cfg.device);
  RB_TRY(cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking), "stream");
  stream = own_stream;
  size_t C = cells(), F = fcells(), L = lcells();
  ribo_status r;
#define RB_ALLOC(ptr, bytes)                                              \
  if ((r = alloc((void**)&(ptr), (bytes), #ptr)) != RIBO_OK) return r;
  RB_ALLOC(chem_a, C * 16);
  RB_ALLOC(chem_b, C * 16);
  RB_ALLOC(gamma, C * 4);
  RB_ALLOC(light, 2 * L * 4);
  RB_ALLOC(shade, 2 * L * 4);
  RB_ALLOC(light_next, 2 * L * 4);
  RB_ALLOC(slope, C * 8);
  RB_ALLOC(agg_nb, C * 4);
  RB_ALLOC(terrain_code, C);
  RB_ALLOC(terrain_arrivals, C);
  RB_ALLOC(terrain_list, terrain_list_entries(gw, gh) * 4);
  RB_ALLOC(terrain_count, 64);
  RB_ALLOC(mask, F);
  RB_ALLOC(normal, F * 8);
  RB_ALLOC(curl, F * 4);
  RB_ALLOC(va, F * 8);
  RB_ALLOC(vb, F * 8);
  RB_ALLOC(vsmooth, F * 8);
  RB_ALLOC(pa, F * 4);
  RB_ALLOC(pb, F * 4);
  RB_ALLOC(div, F * 4);
  RB_ALLOC(temp_a, F * 4);
  RB_ALLOC(temp_b, F * 4);
  RB_ALLOC(redox_a, F * 4);
  RB_ALLOC(redox_b, F * 4);
  RB_ALLOC(redox_eaten, F * 4);
  RB_ALLOC(force_vec, F * 8);
  RB_ALLOC(forces, F * 8);
  RB_ALLOC(heat, F * 8);
  RB_ALLOC(net_flux, ((size_t)fw + fh) * 4);
  RB_ALLOC(ledger, 12 * 4);
  RB_ALLOC(ledger_async, 12 * 4);
  RB_ALLOC(step_ledgers, MAX_STEPS * 12 * 4);
  RB_ALLOC(mask32, F * 4);
  chem_cur = chem_a;
  chem_nxt = chem_b;
  temp_cur = temp_a;
  temp_nxt = temp_b;
  redox_cur = redox_a;
  redox_nxt = redox_b;

  mg_total = build_levels(fw, fh, cfg.mg_min_size, levels);
  RB_ALLOC(mg.p, mg_total * 4);
  RB_ALLOC(mg.rhs, mg_total * 4);
  RB_ALLOC(mg.fluid, mg_total);
  RB_ALLOC(mg.p_tmp, F * 4);
  RB_ALLOC(mg.p2, mg_total * 4);
  RB_ALLOC(mg.code, mg_total);
  RB_ALLOC(status, 16);
  {
    void* maps = nullptr;
    RB_ALLOC(maps, STENCIL_TMAP_BYTES_HOST);
    const StencilFields f{forces, fw, fh};
    if (stencil_tensor_maps(maps, f, own_stream)) tmaps = maps;
  }
  RB_ALLOC(d_params, 2 * MAX_STEPS * sizeof(ribo_sim_params));
#undef RB_ALLOC
  RB_TRY(cudaMallocHost((void**)&h_params, 2 * MAX_STEPS * sizeof(ribo_sim_params) + 12 * 4), "pinned params");
  ledger_host = reinterpret_cast<uint32_t*>(h_params + 2 * MAX_STEPS);
  for (int k = 0; k < 2; k++) RB_TRY(cudaEventCreateWithFlags(&param_ev[k], cudaEventDisableTiming), "event");
  RB_TRY(cudaEventCreate(&t0), "event");
  RB_TRY(cudaEventCreate(&t1), "event");
  for (int k = 0; k < 8; k++) RB_TRY(cudaEventCreate(&marks[k]), "event");
  RB_TRY(cudaEventCreateWithFlags(&ledger_ev, cudaEventDisableTiming), "event");
  if (cfg.precision_mode == RIBO_PRECISION_MIXED) {
    const MgConfig c{(int)cfg.mg_pre, (int)cfg.mg_post, (int)cfg.mg_coarse, 1};
    if (!multigrid_fused_ok(levels.data(), (int)levels.size(), c))
      return set_error(RIBO_INVALID_ARG, "mixed precision needs 1 <= mg_pre, mg_post <= 7 and a coarse level of <= 4096 cells");
    if ((r = mixed_init(*this)) != RIBO_OK) return r;
  }
  // gamma = 0 at creation: derive slope and mask once.
  Dev d = dev();
  launch_slope(d, (float)cfg.world_units_per_cell, stream);
  launch_solid_mask(target_one(d, nullptr), stream);
  launch_mg_codes(levels.data(), (int)levels.size(), mg, stream);
  RB_TRY(cudaGetLastError(), "init kernels");
  RB_TRY(cudaStreamSynchronize(stream), "init");
  return mixed_setup(*this);
}

World::~World() {
  if (stream) cudaStreamSynchronize(stream);
  mixed_free(*this);
  for (GraphEntry& g : graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  for (void* p : allocs) cudaFreeAsync(p, own_stream);
  if (own_stream) cudaStreamSynchronize(own_stream);
  if (h_params) cudaFreeHost(h_params);
  for (int k = 0; k < 2; k++)
    if (param_ev[k]) cudaEventDestroy(param_ev[k]);
  if (t0) cudaEventDestroy(t0);
  if (t1) cudaEventDestroy(t1);
  for (int k = 0; k < 8; k++)
    if (marks[k]) cudaEventDestroy(marks[k]);
  if (ledger_ev) cudaEventDestroy(ledger_ev);
  if (own_stream) cudaStreamDestroy(own_stream);
}

cudaError_t World::bind() const { return cudaSetDevice((int)cfg.device); }

ribo_status World::upload(ribo_field f, const void* host, size_t bytes) {
  size_t need = field_bytes(f);
  if (!need) return set_error(RIBO_INVALID_ARG, "unknown field %d", (int)f);
  if (bytes != need) return set_error(RIBO_INVALID_ARG, "field %d: %zu bytes given, %zu expected", (int)f, bytes, need);
  if (!host) return set_error(RIBO_INVALID_ARG, "null host pointer");
  RB_TRY(bind(), "device");
  if (f == RIBO_FIELD_SOLID_MASK || f == RIBO_FIELD_SLOPE || f == RIBO_FIELD_NET_FLUX || f == RIBO_FIELD_VEL_SMOOTH ||
      f == RIBO_FIELD_PRESSURE_LO)
    return set_error(RIBO_INVALID_ARG, "field %d is derived and read-only", (int)f);
  RB_TRY(cudaMemcpyAsync(field_ptr(f), host, bytes, cudaMemcpyHostToDevice, stream), "upload");
  if (f == RIBO_FIELD_GAMMA) {
    ribo_status r = terrain_changed();
    if (r != RIBO_OK) return r;
  }
  RB_TRY(cudaStreamSynchronize(stream), "upload");
  return RIBO_OK;
}

ribo_status World::terrain_changed() {
  Dev d = dev();
  launch_slope(d, (float)cfg.world_units_per_cell, stream);
  launch_solid_mask(target_one(d, nullptr), stream);
  launch_mg_codes(levels.data(), (int)levels.size(), mg, stream);
  RB_TRY(cudaGetLastError(), "slope/mask");
  ribo_status ms = mixed_setup(*this);
  if (ms != RIBO_OK) return ms;
  light_dirty = true;  // the terrain changed: the next light block sweeps
  return RIBO_OK;
}

// World::encode_paint (src/world/mod.rs:1220-1241).
ribo_status World::paint_terrain(float cx, float cy, float radius, uint32_t grains) {
  RB_TRY(bind(), "device");
  launch_paint(dev(), terrain_bufs(), cx, cy, radius, grains, stream);
  RB_TRY(cudaGetLastError(), "paint");
  ribo_status r = terrain_changed();
  if (r != RIBO_OK) return r;
  RB_TRY(cudaStreamSynchronize(stream), "paint");
  return check_status();
}

namespace {
__global__ void k_mask_to_u32(const uint8_t* m, uint32_t* out, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = m[i];
}
}  // namespace

ribo_status World::read(ribo_field f, void* host, size_t bytes) {
  size_t need = field_bytes(f);
  if (!need) return set_error(RIBO_INVALID_ARG, "unknown field %d", (int)f);
  if (bytes != need) return set_error(RIBO_INVALID_ARG, "field %d: %zu bytes given, %zu expected", (int)f, bytes, need);
  if (!host) return set_error(RIBO_INVALID_ARG, "null host pointer");
  RB_TRY(bind(), "device");
  const void* src = field_ptr(f);
  if (!src && f != RIBO_FIELD_SOLID_MASK) return set_error(RIBO_INVALID_ARG, "field %d does not exist in this world", (int)f);
  if (f == RIBO_FIELD_SOLID_MASK) {
    size_t n = fcells();
    k_mask_to_u32<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(mask, mask32, n);
    RB_TRY(cudaGetLastError(), "mask read");
    src = mask32;
  }
  RB_TRY(cudaMemcpyAsync(host, src, bytes, cudaMemcpyDeviceToHost, stream), "read");
  RB_TRY(cudaStreamSynchronize(stream), "read");
  {
    ribo_status s = check_status();
    if (s != RIBO_OK) return s;
  }
  return RIBO_OK;
}

// One pressure solve, result in pressure_a (src/world/mod.rs:1545-1581).
void World::pressure_solve(const Dev& d) {
  if (mixed) {
    ribo_status s = mixed_solve(*this);
    if (s != RIBO_OK && solve_error == RIBO_OK) solve_error = s;
    return;
  }
  if (st.multigrid) {
    MgConfig c{(int)cfg.mg_pre, (int)cfg.mg_post, (int)cfg.mg_coarse, (int)(st.mg_cycles < 1 ? 1 : st.mg_cycles),
               (int)cfg.mg_cluster};
    if (!st.mg_unfused && multigrid_fused_ok(levels.data(), (int)levels.size(), c))
      launch_multigrid_fused(d, levels.data(), (int)levels.size(), mg, c, stream);
    else
      launch_multigrid(d, levels.data(), (int)levels.size(), mg, c, stream);
  } else {
    uint32_t it = st.jacobi_iters < 2 ? 2 : (st.jacobi_iters > 128 ? 128 : st.jacobi_iters);
    it = (it + 1u) & ~1u;
    launch_jacobi(d, (int)it, stream);
  }
}

// src/world/mod.rs:1506: a full sweep when the light is dirty or, without
// propagation, every light_interval steps.
bool World::light_sweeps(const ribo_sim_params& hp, bool dirty) const {
  const uint32_t interval = st.light_interval < 1 ? 1 : st.light_interval;
  return dirty || (st.light_rows_per_step == 0 && hp.epoch % interval == 0u);
}

// The terrain, light, fluid and transport blocks of one step
// (src/world/mod.rs:1497-1601).
void World::record_step(const ribo_sim_params& hp, const ribo_sim_params* P, uint32_t i) {
  if (st.terrain_mode) {
    const Dev d = dev();
    const TerrainBufs tb = terrain_bufs();
    launch_relax(d, P, tb, 0u, stream);
    launch_relax(d, P, tb, 1u, stream);
    if (hp.sediment_settle > 0.0f) launch_grain_fall(d, P, tb, stream);
    launch_slope(d, (float)cfg.world_units_per_cell, stream);
  }
  if (st.light_mode) {
    const Target t = target_one(dev(), P);
    if (light_sweeps(hp, light_dirty)) {
      light_dirty = false;
      launch_light_transmit(t, stream);
      launch_light_sweep(dev(), P, stream);
    } else {
      const uint32_t rows = st.light_rows_per_step > 16 ? 16 : st.light_rows_per_step;
      for (uint32_t r = 0; r < rows; r++) {
        launch_light_propagate(t, stream);
        launch_light_commit(t, stream);
      }
    }
  }
  uint32_t substep = st.fluid_substep < 1 ? 1 : (st.fluid_substep > 4 ? 4 : st.fluid_substep);
  if (st.fluid_enabled && hp.epoch % substep == 0u) {
    if (st.terrain_mode) {
      launch_solid_mask(target_one(dev(), P), stream);  // build_solid_mask
      launch_mg_codes(levels.data(), (int)levels.size(), mg, stream);
    }
    launch_temperature(target_one(dev(), P), stream);  // temp_in -> temp_out
    std::swap(temp_cur, temp_nxt);                     // copy_temperature
    std::swap(redox_cur, redox_nxt);
    const Target t = target_one(dev(), P);
    launch_forces(t, stream);                // buoyancy + gather_forces + clear_force_vectors
    launch_add_forces(t, A_TO_B, stream);
    launch_diffuse(t, B_TO_A, stream);
    launch_advect(t, A_TO_B, stream);
    launch_vorticity(t, B_TO_A, stream);
    launch_divergence(t, A_TO_B, stream);    // reads velocity_a
    pressure_solve(t.one);
    launch_subtract_gradient(t, A_TO_B, stream);
    launch_net_flux(t, B_TO_A, stream);      // reads velocity_b
    launch_boundaries(t, B_TO_A, stream);    // final velocity in velocity_a
    launch_smooth(t, A_TO_B, stream);        // reads velocity_a
    launch_thermal(t, stream);
  }
  uint32_t te = hp.transport_every < 1 ? 1 : hp.transport_every;
  if (hp.epoch % te == 0u) {
    const Target t = target_one(dev(), P);
    if (hp.aggregation > 0.0f) launch_agg(t, stream);
    launch_scatter(t, st.transport_simple != 0, stream);
    std::swap(chem_cur, chem_nxt);  // transport_commit
    cudaMemsetAsync(chem_nxt, 0, cells() * 16, stream);
  }
  if (st.ledger_each_step) {
    uint32_t* out = step_ledgers + (size_t)i * 12;
    cudaMemsetAsync(out, 0, 12 * sizeof(uint32_t), stream);
    launch_ledger(target_one(dev(), nullptr), out, stream);
  }
}

ribo_status World::step(const ribo_sim_params* per_step, uint32_t n) {
  if (n == 0) return RIBO_OK;
  if (!per_step) return set_error(RIBO_INVALID_ARG, "null params");
  if (n > MAX_STEPS) return set_error(RIBO_INVALID_ARG, "%u steps per call (at most %u)", n, MAX_STEPS);
  if (st.terrain_mode && mixed)
    return set_error(RIBO_INVALID_ARG, "mixed precision takes a frozen terrain (terrain_mode 0): its solver setup "
                                       "follows the wall mask of the uploaded gamma");
  RB_TRY(bind(), "device");
  // src/world/mod.rs:1414-1421: turning the fluid off clears it once.
  if (!st.fluid_enabled && fluid_was_on) {
    RB_TRY(cudaMemsetAsync(va, 0, fcells() * 8, stream), "clear");
    RB_TRY(cudaMemsetAsync(temp_cur, 0, fcells() * 4, stream), "clear");
    RB_TRY(cudaMemsetAsync(redox_cur, 0, fcells() * 4, stream), "clear");
  }
  fluid_was_on = st.fluid_enabled != 0;
  int slot = param_slot;
  param_slot ^= 1;
  RB_TRY(cudaEventSynchronize(param_ev[slot]), "param slot");
  ribo_sim_params* hs = h_params + slot * MAX_STEPS;
  ribo_sim_params* ds = d_params + slot * MAX_STEPS;
  memcpy(hs, per_step, n * sizeof(ribo_sim_params));
  RB_TRY(cudaEventRecord(t0, stream), "event");
  RB_TRY(cudaMemcpyAsync(ds, hs, n * sizeof(ribo_sim_params), cudaMemcpyHostToDevice, stream), "params");
  RB_TRY(cudaEventRecord(param_ev[slot], stream), "event");
  if (timing) {
    ktime_set_active(&timer);
    for (uint32_t i = 0; i < n; i++) record_step(per_step[i], ds + i, i);
    ktime_set_active(nullptr);
  } else {
    ribo_status s = record_steps_graphed(per_step, ds, n, slot);
    if (s != RIBO_OK) return s;
  }
  last_steps = n;
  if (solve_error != RIBO_OK) {
    ribo_status s = solve_error;
    solve_error = RIBO_OK;
    return s;
  }
  RB_TRY(cudaGetLastError(), "step launch");
  RB_TRY(cudaEventRecord(t1, stream), "event");
  return RIBO_OK;
}

// Repeated step sequences replay from CUDA graphs.  The kernels of a call
// depend only on the per-step schedule (which blocks run), the settings,
// the parameter slot and the ping-pong state of chem / temperature / redox,
// so those form the key; a sequence is captured the second time its key is
// seen and replayed afterwards, with the host ping-pong state moved to the
// state the capture left.
std::string World::graph_key(const ribo_sim_params* per_step, uint32_t n, int slot) const {
  std::string k;
  k.reserve(64 + n);
  auto put = [&](const void* p, size_t b) { k.append(reinterpret_cast<const char*>(p), b); };
  put(&n, 4);
  put(&slot, 4);
  put(&st, sizeof st);
  put(&chem_cur, sizeof(void*));
  put(&temp_cur, sizeof(void*));
  put(&redox_cur, sizeof(void*));
  uint32_t substep = st.fluid_substep < 1 ? 1 : (st.fluid_substep > 4 ? 4 : st.fluid_substep);
  bool dirty = light_dirty;
  for (uint32_t i = 0; i < n; i++) {
    const ribo_sim_params& p = per_step[i];
    uint32_t te = p.transport_every < 1 ? 1 : p.transport_every;
    const bool sweep = st.light_mode && light_sweeps(p, dirty);
    if (sweep) dirty = false;
    char c = (char)((st.fluid_enabled && p.epoch % substep == 0u ? 1 : 0) | (p.epoch % te == 0u ? 2 : 0) |
                    (p.aggregation > 0.0f ? 4 : 0) | (sweep ? 8 : 0) |
                    (st.terrain_mode && p.sediment_settle > 0.0f ? 16 : 0));
    k.push_back(c);
  }
  return k;
}

ribo_status World::record_steps_graphed(const ribo_sim_params* per_step, const ribo_sim_params* ds, uint32_t n, int slot) {
  if (cfg.no_graphs) {
    for (uint32_t i = 0; i < n; i++) record_step(per_step[i], ds + i, i);
    return RIBO_OK;
  }
  std::string key = graph_key(per_step, n, slot);
  for (GraphEntry& g : graphs) {
    if (g.key != key) continue;
    RB_TRY(cudaGraphLaunch(g.exec, stream), "graph launch");
    chem_cur = g.chem_end;
    chem_nxt = g.chem_end == chem_a ? chem_b : chem_a;
    temp_cur = g.temp_end;
    temp_nxt = g.temp_end == temp_a ? temp_b : temp_a;
    redox_cur = g.redox_end;
    redox_nxt = g.redox_end == redox_a ? redox_b : redox_a;
    for (uint32_t i = 0; i < n && st.light_mode; i++)
      if (light_sweeps(per_step[i], light_dirty)) light_dirty = false;
    ktime_add_launches(g.kernels);
    g.uses++;
    return RIBO_OK;
  }
  bool seen = false;
  for (const std::string& s : seen_keys) seen = seen || s == key;
  if (!seen) {
    if (seen_keys.size() >= 16) seen_keys.erase(seen_keys.begin());
    seen_keys.push_back(key);
    for (uint32_t i = 0; i < n; i++) record_step(per_step[i], ds + i, i);
    return RIBO_OK;
  }
  // capture
  uint64_t l0 = ktime_launch_count();
  RB_TRY(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "capture");
  for (uint32_t i = 0; i < n; i++) record_step(per_step[i], ds + i, i);
  cudaGraph_t graph = nullptr;
  RB_TRY(cudaStreamEndCapture(stream, &graph), "capture");
  GraphEntry e;
  e.key = key;
  e.kernels = ktime_launch_count() - l0;
  cudaError_t err = cudaGraphInstantiate(&e.exec, graph, 0);
  cudaGraphDestroy(graph);
  RB_TRY(err, "graph instantiate");
  e.chem_end = chem_cur;
  e.temp_end = temp_cur;
  e.redox_end = redox_cur;
  RB_TRY(cudaGraphLaunch(e.exec, stream), "graph launch");
  if (graphs.size() >= 8) {
    cudaGraphExecDestroy(graphs.front().exec);
    graphs.erase(graphs.begin());
  }
  graphs.push_back(e);
  return RIBO_OK;
}

ribo_status World::read_timing(ribo_kernel_timing* out, uint32_t cap, uint32_t* count) {
  RB_TRY(bind(), "device");
  RB_TRY(cudaStreamSynchronize(stream), "timing");
  return ktimer_read(timer, out, cap, count);
}

ribo_status ktimer_read(const KTimer& timer, ribo_kernel_timing* out, uint32_t cap, uint32_t* count) {
  std::vector<ribo_kernel_timing> agg;
  for (const KTimer::Rec& r : timer.recs) {
    float ms = 0.0f;
    RB_TRY(cudaEventElapsedTime(&ms, r.a, r.b), "elapsed");
    ribo_kernel_timing* e = nullptr;
    for (auto& x : agg)
      if (strncmp(x.name, r.label, sizeof x.name) == 0) e = &x;
    if (!e) {
      ribo_kernel_timing z;
      memset(&z, 0, sizeof z);
      strncpy(z.name, r.label, sizeof z.name - 1);
      agg.push_back(z);
      e = &agg.back();
    }
    e->launches += 1;
    e->ms += ms;
    e->bytes += r.bytes;
  }
  uint32_t n = (uint32_t)agg.size();
  if (count) *count = n;
  for (uint32_t i = 0; i < n && i < cap && out; i++) out[i] = agg[i];
  return RIBO_OK;
}

// Kernel-side failures (a bounded wait that ran out) are reported through
// the status word rather than by trapping; it is read at every host sync.
ribo_status World::check_status() {
  uint32_t h = 0;
  RB_TRY(cudaMemcpyAsync(&h, status, 4, cudaMemcpyDeviceToHost, stream), "status");
  RB_TRY(cudaStreamSynchronize(stream), "status");
  if (h) {
    RB_TRY(cudaMemsetAsync(status, 0, 4, stream), "status");
    if (h & ERR_TIMEOUT)
      return set_error(RIBO_TIMEOUT, "a kernel wait timed out (status 0x%x); results of the last steps are invalid", h);
    return set_error(RIBO_CUDA_ERROR, "a kernel index check failed (status 0x%x); results of the last steps are invalid", h);
  }
  return RIBO_OK;
}

// encode_ledger_readback + ledger_after_submit (src/world/mod.rs:1758-1781):
// the reduction and its copy to pinned memory go on the stream behind the
// work recorded so far; a request while one is pending does nothing.
ribo_status World::ledger_request() {
  if (ledger_pending) return RIBO_OK;
  RB_TRY(bind(), "device");
  RB_TRY(cudaMemsetAsync(ledger_async, 0, 12 * sizeof(uint32_t), stream), "ledger");
  launch_ledger(target_one(dev(), nullptr), ledger_async, stream);
  RB_TRY(cudaGetLastError(), "ledger");
  RB_TRY(cudaMemcpyAsync(ledger_host, ledger_async, 12 * 4, cudaMemcpyDeviceToHost, stream), "ledger");
  RB_TRY(cudaEventRecord(ledger_ev, stream), "ledger");
  ledger_pending = true;
  return RIBO_OK;
}

// poll_ledger (src/world/mod.rs:1783-1799): the ledger once the readback has
// arrived, else nothing; never waits.
ribo_status World::ledger_poll(uint32_t out[12], uint32_t* ready) {
  *ready = 0;
  if (!ledger_pending) return RIBO_OK;
  RB_TRY(bind(), "device");
  const cudaError_t q = cudaEventQuery(ledger_ev);
  if (q == cudaErrorNotReady) return RIBO_OK;
  RB_TRY(q, "ledger");
  ledger_pending = false;
  ribo_status s = check_status();
  if (s != RIBO_OK) return s;
  memcpy(out, ledger_host, 12 * 4);
  *ready = 1;
  return RIBO_OK;
}

ribo_status World::ledger_read(uint32_t out[12]) {
  RB_TRY(bind(), "device");
  RB_TRY(cudaMemsetAsync(ledger, 0, 12 * sizeof(uint32_t), stream), "ledger");
  launch_ledger(target_one(dev(), nullptr), ledger, stream);
  RB_TRY(cudaGetLastError(), "ledger");
  RB_TRY(cudaMemcpyAsync(out, ledger, 12 * 4, cudaMemcpyDeviceToHost, stream), "ledger");
  RB_TRY(cudaStreamSynchronize(stream), "ledger");
  {
    ribo_status s = check_status();
    if (s != RIBO_OK) return s;
  }
  return RIBO_OK;
}

}  // namespace ribo

using ribo::set_error;

// ---------------------------------------------------------------------------
// C ABI

extern "C" {

const char* ribo_last_error(void) { return ribo::g_last_error.c_str(); }

void ribo_sim_params_default(ribo_sim_params* o) {
  if (!o) return;
  memset(o, 0, sizeof *o);
  // src/params.rs:553-690
  o->epoch = 0; o->seed = 1; o->dt = 0.017f; o->diffusion = 12.0f; o->settle = 0.0f;
  o->fluid_dt = (float)(0.017f * 2.0f); o->fluid_decay = 0.99f; o->fluid_vorticity = 7.7f; o->fluid_viscosity = 3.7f;
  o->fumarole_count = 0; o->uv_strength = 3.0f; o->uv_depth = 0.0f; o->fluid_enabled = 1;
  o->fluid_obstacle_strength = 1000.0f; o->slope_steer_rate = 210.0f; o->cohesion = 0.25f; o->spawn_count = 0;
  o->max_agents = 0; o->death_probability = 0.0006f; o->spawn_energy = 5.0f; o->food_power = 6.0f;
  o->maintenance_cost = 0.002f; o->pairing_rate = 3.0f; o->mutation_rate = 0.005f; o->uv_damage = 1.0f;
  o->uptake_rate = 0.0003f; o->brownian = 0.0f; o->phoretic_gain = 0.0f; o->chain_stiffness = 100.0f;
  o->thermal_kt = 0.1f; o->motor_amplitude = 0.4f; o->rft_enabled = 1; o->require_start = 1;
  o->joint_coupling = 0.0f; o->hunger_regulation = 1; o->pairing_cost = 0.1f; o->reactivation_rate = 0.00001f;
  o->swim_gain = 2.0f; o->bioturbation = 0.39f; o->bioturbation_cost = 0.01f; o->monomer_uv_absorb = 0.3f;
  o->sedimentation = 0.0f; o->direct_photoactivation = 0.02f; o->activation_decay = 0.0f; o->monomer_pressure = 0.0f;
  o->agent_fluid_push = 0.001f; o->swim_wobble = 1.0f; o->fluid_swim_only = 0; o->motion_cost = 0.06f;
  o->bond_rate = 0.05f; o->bond_energy_share = 0.1f; o->bond_signal = 0.5f; o->aggregation = 0.03f;
  o->photo_yield = 0.5f; o->heat_kill = 0.27f; o->flow_coupling = 0.9f; o->inertia = 0.0f;
  o->death_energy_cap = 1.0f; o->chemo_yield = 0.9f; o->redox_decay = 0.02f; o->thermal_activation = 0.045f;
  o->denature_temp = 2.0f; o->day_period = 8000.0f; o->sun_slope = 0.0f; o->sun_now = 1.0f;
  o->sun_angle = 80.0f; o->day_fraction = 0.75f; o->metabolic_q10 = 2.0f; o->metabolic_span = 3.0f;
  o->metabolic_ref = 0.0f; o->sun_heat = 1.0f; o->sediment_transport = 1.9f; o->sediment_threshold = 0.5f;
  o->sediment_settle = 0.0f; o->signal_mode = 0.0f; o->clock_mute = 0.0f; o->paint_x = 0.0f;
  o->paint_y = 0.0f; o->paint_radius = 0.0f; o->paint_grains = 0.0f; o->rest_angle_mult = 1.0f;
  o->protease_power = 1.5f; o->lysis_yield = 0.7f; o->protease_direct = 0.5f; o->joint_load = 1.0f;
  o->swim_grip = 10.0f; o->swim_memory = 1.0f; o->mouth_leak = 0.3f; o->leak_base = 0.05f;
  o->skin_uptake = 0.1f; o->death_metab = 0.2f; o->salvage = 0.0f; o->bond_matter_share = 0.1f;
  o->brownian_rot = 0.0f; o->transport_every = 3; o->signal_crosstalk = 0.1f; o->flow_mass = 0.0f;
  o->chemo_take = 0.008f; o->vent_cycle_period = 7000.0f; o->vent_cycle_amp = 0.91f; o->sediment_cohesion = 0.5f;
  o->sediment_compaction = 0.00001f; o->rock_crumble = 0.0001f; o->lysis_matter = 0.5f; o->scramble_conduction = 0;
  o->scramble_angles = 0; o->scramble_response = 0; o->scramble_amount = 1.0f; o->pairing_energy_half = 0.5f;
  o->pairing_min_energy = 0.0f; o->uv_mutation = 0.0f; o->heat_mutation = 0.0f; o->birth_crowding = 80.0f;
  o->photo_damage = 0.005f; o->naked_decay = 0.005f; o->store_loss = 0.0001f;
}

void ribo_world_settings_default(ribo_world_settings* o) {
  if (!o) return;
  memset(o, 0, sizeof *o);
  // src/world/mod.rs:117-134 (hot-path fields)
  o->fluid_enabled = 1;
  o->fluid_substep = 2;
  o->multigrid = 1;
  o->mg_cycles = 1;
  o->jacobi_iters = 128;
  o->mixed_tol = 1e-5f;
  o->mixed_inner_tol = 1e-3f;
  o->mixed_max_outer = 4;
  o->mixed_max_inner = 64;
  o->mixed_alpha = 1.8f;
  o->light_rows_per_step = 1;  // light_mode 0: the light is a frozen input
  o->light_interval = 10;
}

ribo_status ribo_world_solve_info(ribo_world* w, uint32_t* outer, uint32_t* inner, double* rel_residual) {
  if (!w) return set_error(RIBO_INVALID_ARG, "null world");
  ribo_status st = ribo::cuda_status(w->w.bind(), "device");
  if (st != RIBO_OK) return st;
  return ribo::mixed_info(w->w, outer, inner, rel_residual);
}

static ribo_status check_cfg(const ribo_world_cfg* cfg) {
  if (cfg->grid_w < 2 || cfg->grid_h < 2 || cfg->fluid_w < 2 || cfg->fluid_h < 2)
    return set_error(RIBO_INVALID_ARG, "grid and fluid sides must be >= 2");
  if (cfg->grid_w % cfg->fluid_w || cfg->grid_h % cfg->fluid_h || cfg->grid_w / cfg->fluid_w != cfg->grid_h / cfg->fluid_h)
    return set_error(RIBO_INVALID_ARG, "grid/fluid must be the same integer ratio on both axes");
  if (cfg->grid_w % 2 || cfg->grid_h % 2) return set_error(RIBO_INVALID_ARG, "grid sides must be even (light grid is grid/2)");
  if ((uint64_t)cfg->grid_w * cfg->grid_h > (1ull << 28))
    return set_error(RIBO_INVALID_ARG, "grid too large (at most 2^28 cells: chem slot indices are u32)");
  if (cfg->precision_mode > RIBO_PRECISION_MIXED) return set_error(RIBO_INVALID_ARG, "unknown precision mode");
  if (cfg->mg_cluster != 0 && cfg->mg_cluster != 1 && cfg->mg_cluster != 8 && cfg->mg_cluster != 16)
    return set_error(RIBO_INVALID_ARG, "mg_cluster must be 0 (automatic), 1 (none), 8 or 16");
  return RIBO_OK;
}

ribo_status ribo_world_footprint(const ribo_world_cfg* cfg, uint64_t* bytes) {
  if (!cfg || !bytes) return set_error(RIBO_INVALID_ARG, "null argument");
  ribo_status st = check_cfg(cfg);
  if (st != RIBO_OK) return st;
  *bytes = ribo::world_footprint(*cfg);
  return RIBO_OK;
}

ribo_status ribo_world_memory(const ribo_world* w, uint64_t* bytes) {
  if (!w || !bytes) return set_error(RIBO_INVALID_ARG, "null argument");
  *bytes = w->w.device_bytes;
  return RIBO_OK;
}

ribo_status ribo_world_create(const ribo_world_cfg* cfg, ribo_world** out) {
  if (!cfg || !out) return set_error(RIBO_INVALID_ARG, "null argument");
  *out = nullptr;
  ribo_status cst = check_cfg(cfg);
  if (cst != RIBO_OK) return cst;
  ribo_world* w = new (std::nothrow) ribo_world();
  if (!w) return set_error(RIBO_OOM, "host allocation");
  ribo_status st = w->w.init(*cfg);
  if (st != RIBO_OK) {
    delete w;
    return st;
  }
  *out = w;
  return RIBO_OK;
}

void ribo_world_destroy(ribo_world* w) {
  if (w && w->w.batch) ribo_batch_remove(static_cast<ribo_batch*>(w->w.batch), w);
  delete w;
}

ribo_status ribo_world_set_settings(ribo_world* w, const ribo_world_settings* s) {
  if (!w || !s) return set_error(RIBO_INVALID_ARG, "null argument");
  if (s->light_mode && !w->w.st.light_mode) w->w.light_dirty = true;
  w->w.st = *s;
  return RIBO_OK;
}

ribo_status ribo_world_get_settings(const ribo_world* w, ribo_world_settings* out) {
  if (!w || !out) return set_error(RIBO_INVALID_ARG, "null argument");
  *out = w->w.st;
  return RIBO_OK;
}

ribo_status ribo_world_upload(ribo_world* w, ribo_field field, const void* host, size_t bytes) {
  if (!w) return set_error(RIBO_INVALID_ARG, "null world");
  return w->w.upload(field, host, bytes);
}

ribo_status ribo_world_paint_terrain(ribo_world* w, float cx, float cy, float radius, uint32_t grains) {
  if (!w) return set_error(RIBO_INVALID_ARG, "null world");
  return w->w.paint_terrain(cx, cy, radius, grains);
}

ribo_status ribo_world_read(ribo_world* w, ribo_field field, void* host, size_t bytes) {
  if (!w) return set_error(RIBO_INVALID_ARG, "null world");
  return w->w.read(field, host, bytes);
}

ribo_status ribo_world_device_ptr(ribo_world* w, ribo_field field, void** dptr, size_t* bytes) {
  if (!w || !dptr || !bytes) return set_error(RIBO_INVALID_ARG, "null argument");
  size_t n = w->w.field_bytes(field);
  void* p = w->w.field_ptr(field);
  if (!n || !p) return set_error(RIBO_INVALID_ARG, "field %d has no device view", (int)field);
  *dptr = p;
  *bytes = n;
  return RIBO_OK;
}

ribo_status ribo_world_step(ribo_world* w, const ribo_sim_params* per_step, uint32_t n) {
  if (!w) return set_error(RIBO_INVALID_ARG, "null world");
  return w->w.step(per_step, n);
}

// SimParams::day_phase / daylight / sun_slope_at (src/params.rs:497-534).
static void day_phase(const ribo_sim_params* p, uint32_t epoch, bool* day, double* phase) {
  double x = (double)epoch / (double)p->day_period;
  double ph = x - trunc(x);
  double frac = (double)p->day_fraction;
  frac = frac < 0.05 ? 0.05 : (frac > 1.0 ? 1.0 : frac);
  *day = ph < frac;
  *phase = ph / frac;
}
static float sun_daylight(const ribo_sim_params* p, uint32_t epoch) {
  if (p->day_period < 1.0f) return 1.0f;
  bool day;
  double ph;
  day_phase(p, epoch, &day, &ph);
  if (!day) return 0.0f;
  double s = sin(M_PI * ph);
  return (float)(s > 0.0 ? s : 0.0);
}
static float sun_slope_at(const ribo_sim_params* p, uint32_t epoch) {
  if (p->day_period < 1.0f) return 0.0f;
  bool day;
  double ph;
  day_phase(p, epoch, &day, &ph);
  double a = (double)p->sun_angle;
  a = a < 0.0 ? 0.0 : (a > 85.0 ? 85.0 : a);
  double max_angle = a * (M_PI / 180.0);
  if (!day) ph = 1.0;
  double angle = (ph - 0.5) * 2.0 * max_angle;
  return (float)tan(angle);
}

ribo_status ribo_derive_step_params(const ribo_sim_params* base, const ribo_world_settings* s, uint32_t steps,
                                    ribo_sim_params* out) {
  if (!base || !s || (!out && steps)) return set_error(RIBO_INVALID_ARG, "null argument");
  uint32_t substep = s->fluid_substep < 1 ? 1 : (s->fluid_substep > 4 ? 4 : s->fluid_substep);
  ribo_sim_params b = *base;
  b.fluid_dt = b.dt * (float)substep;
  b.fluid_enabled = s->fluid_enabled ? 1u : 0u;
  for (uint32_t i = 0; i < steps; i++) {
    ribo_sim_params p = b;
    p.epoch = b.epoch + i;
    if (i > 0) p.spawn_count = 0;
    p.sun_now = b.uv_strength > 0.0f ? sun_daylight(&b, p.epoch) : 0.0f;
    p.sun_slope = sun_slope_at(&b, p.epoch);
    out[i] = p;
  }
  return RIBO_OK;
}

ribo_status ribo_world_encode_steps(ribo_world* w, ribo_sim_params* params, uint32_t steps) {
  if (!w || !params) return set_error(RIBO_INVALID_ARG, "null argument");
  if (steps > 64) steps = 64;  // MAX_STEPS_PER_FRAME
  if (steps == 0) return RIBO_OK;
  ribo_sim_params buf[64];
  ribo_status st = ribo_derive_step_params(params, &w->w.st, steps, buf);
  if (st != RIBO_OK) return st;
  st = w->w.step(buf, steps);
  if (st != RIBO_OK) return st;
  uint32_t substep = w->w.st.fluid_substep < 1 ? 1 : (w->w.st.fluid_substep > 4 ? 4 : w->w.st.fluid_substep);
  params->fluid_dt = params->dt * (float)substep;
  params->fluid_enabled = w->w.st.fluid_enabled ? 1u : 0u;
  params->epoch += steps;
  return RIBO_OK;
}

ribo_status ribo_world_ledger(ribo_world* w, uint32_t out[12]) {
  if (!w || !out) return set_error(RIBO_INVALID_ARG, "null argument");
  return w->w.ledger_read(out);
}

ribo_status ribo_world_request_ledger(ribo_world* w) {
  if (!w) return set_error(RIBO_INVALID_ARG, "null world");
  return w->w.ledger_request();
}

ribo_status ribo_world_poll_ledger(ribo_world* w, uint32_t out[12], uint32_t* ready) {
  if (!w || !out || !ready) return set_error(RIBO_INVALID_ARG, "null argument");
  return w->w.ledger_poll(out, ready);
}

ribo_status ribo_world_step_ledgers(ribo_world* w, uint32_t* out, uint32_t n) {
  if (!w || (!out && n)) return set_error(RIBO_INVALID_ARG, "null argument");
  if (n > w->w.last_steps) return set_error(RIBO_INVALID_ARG, "last call recorded %u steps", w->w.last_steps);
  if (!w->w.st.ledger_each_step) return set_error(RIBO_INVALID_ARG, "settings.ledger_each_step is off");
  ribo_status st = ribo::cuda_status(w->w.bind(), "device");
  if (st != RIBO_OK) return st;
  st = ribo::cuda_status(cudaMemcpyAsync(out, w->w.step_ledgers, (size_t)n * 48, cudaMemcpyDeviceToHost, w->w.stream), "ledgers");
  if (st != RIBO_OK) return st;
  return ribo::cuda_status(cudaStreamSynchronize(w->w.stream), "ledgers");
}

ribo_status ribo_world_mark(ribo_world* w, uint32_t slot) {
  if (!w || slot >= 8) return set_error(RIBO_INVALID_ARG, "bad mark slot");
  return ribo::cuda_status(cudaEventRecord(w->w.marks[slot], w->w.stream), "mark");
}

ribo_status ribo_world_elapsed_ms(ribo_world* w, uint32_t a, uint32_t b, float* ms) {
  if (!w || a >= 8 || b >= 8 || !ms) return set_error(RIBO_INVALID_ARG, "bad mark slot");
  ribo_status st = ribo::cuda_status(cudaEventSynchronize(w->w.marks[b]), "mark");
  if (st != RIBO_OK) return st;
  return ribo::cuda_status(cudaEventElapsedTime(ms, w->w.marks[a], w->w.marks[b]), "elapsed");
}

ribo_status ribo_world_sync(ribo_world* w) {
  if (!w) return set_error(RIBO_INVALID_ARG, "null world");
  ribo_status st = ribo::cuda_status(cudaStreamSynchronize(w->w.stream), "sync");
  if (st != RIBO_OK) return st;
  return w->w.check_status();
}

ribo_status ribo_world_raise_status(ribo_world* w, uint32_t bits) {
  if (!w) return set_error(RIBO_INVALID_ARG, "null world");
  using ribo::cuda_status;
  RB_TRY(w->w.bind(), "device");
  uint32_t cur = 0;
  RB_TRY(cudaMemcpyAsync(&cur, w->w.status, 4, cudaMemcpyDeviceToHost, w->w.stream), "status");
  RB_TRY(cudaStreamSynchronize(w->w.stream), "status");
  cur |= bits;
  RB_TRY(cudaMemcpyAsync(w->w.status, &cur, 4, cudaMemcpyHostToDevice, w->w.stream), "status");
  RB_TRY(cudaStreamSynchronize(w->w.stream), "status");
  return RIBO_OK;
}

ribo_status ribo_selftest_bounded_wait(uint32_t device, uint32_t polls, uint32_t* status_bits) {
  if (!status_bits) return set_error(RIBO_INVALID_ARG, "null argument");
  *status_bits = 0;
  ribo_status st = ribo::selftest_bounded_wait((int)device, polls, status_bits);
  if (st != RIBO_OK) return st;
  // the context still answers: a trivial synchronous call after the kernel
  return ribo::cuda_status(cudaDeviceSynchronize(), "selftest");
}

ribo_status ribo_world_enable_kernel_timing(ribo_world* w, int enable) {
  if (!w) return set_error(RIBO_INVALID_ARG, "null world");
  w->w.timing = enable != 0;
  return RIBO_OK;
}

ribo_status ribo_world_read_kernel_timing(ribo_world* w, ribo_kernel_timing* out, uint32_t cap, uint32_t* count) {
  if (!w) return set_error(RIBO_INVALID_ARG, "null world");
  return w->w.read_timing(out, cap, count);
}

uint64_t ribo_kernel_launch_count(void) { return ribo::g_launches.load(); }

ribo_status ribo_world_last_step_ms(ribo_world* w, float* ms) {
  if (!w || !ms) return set_error(RIBO_INVALID_ARG, "null argument");
  cudaError_t e = cudaEventSynchronize(w->w.t1);
  if (e != cudaSuccess) return ribo::cuda_status(e, "event");
  return ribo::cuda_status(cudaEventElapsedTime(ms, w->w.t0, w->w.t1), "elapsed");
}

}  // extern "C"
