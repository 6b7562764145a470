// Batches of worlds advanced in lock step (ribo_batch_* of the C ABI), and
// the launch geometry every pass shares with the one-world path.
//
// A batch records the dispatch sequence of World::encode_steps
// (src/world/mod.rs:1487-1601) once for all of its members: each pass is one
// launch whose CTAs are spread over the members' grids through device tables
// (first block and blocks per row of every member, see WorldSet), so a 128^2
// world and a 2048x256 world share every launch while each world's cells see
// exactly the arithmetic of a launch of their own.  Members whose per-step
// schedule or settings differ are split into groups with their own tables.
#include <cuda_runtime.h>
#include <string.h>

#include <map>
#include <string>
#include <vector>

#include "../../include/ribo_world.h"
#include "ribo_dev.cuh"
#include "ribo_launch.h"
#include "ribo_world_impl.h"

namespace ribo {

void geo_blocks(Geo g, const Dev& d, int* nbx, int* nby) {
  const long long cells = (long long)d.gw * d.gh;
  switch (g) {
    case GEO_FLUID:
      *nbx = (d.fw + PASS_BX - 1) / PASS_BX;
      *nby = (d.fh + PASS_BY - 1) / PASS_BY;
      return;
    case GEO_ENV:
      *nbx = (d.gw + PASS_BX - 1) / PASS_BX;
      *nby = (d.gh + PASS_BY - 1) / PASS_BY;
      return;
    case GEO_ENV_LINEAR:
      *nbx = (int)((cells + LINEAR_THREADS - 1) / LINEAR_THREADS);
      *nby = 1;
      return;
    case GEO_SCATTER:
      *nbx = (d.gw + SCATTER_TX - 1) / SCATTER_TX;
      *nby = (d.gh + SCATTER_TY - 1) / SCATTER_TY;
      return;
    case GEO_NET_FLUX:
      *nbx = (d.fh + NET_FLUX_LINES - 1) / NET_FLUX_LINES + (d.fw + NET_FLUX_LINES - 1) / NET_FLUX_LINES;
      *nby = 1;
      return;
    case GEO_LIGHT:
      *nbx = (d.lw + PASS_BX - 1) / PASS_BX;
      *nby = (d.lh + PASS_BY - 1) / PASS_BY;
      return;
    case GEO_FLUID_TALL:
      *nbx = (d.fw + PASS_BX - 1) / PASS_BX;
      *nby = (d.fh + PASS_BY * FLUID_ROWS - 1) / (PASS_BY * FLUID_ROWS);
      return;
    case GEO_ENV_TALL:
      *nbx = (d.gw + PASS_BX - 1) / PASS_BX;
      *nby = (d.gh + PASS_BY * FLUID_ROWS - 1) / (PASS_BY * FLUID_ROWS);
      return;
    case GEO_ENV_LINEAR4:
      *nbx = (int)((cells + 4 * LINEAR_THREADS - 1) / (4 * LINEAR_THREADS));
      *nby = 1;
      return;
    case GEO_LEDGER: {
      long long b = (cells + LEDGER_CELLS_PER_CTA - 1) / LEDGER_CELLS_PER_CTA;
      const long long cap = 8ll * device_sm_count();  // eight CTAs per SM stream the whole grid
      *nbx = (int)(b < 1 ? 1 : (b > cap ? cap : b));
      *nby = 1;
      return;
    }
    default:
      *nbx = *nby = 0;
  }
}

Target target_one(const Dev& d, const ribo_sim_params* P) {
  Target t;
  t.one = d;
  t.P = P;
  t.n = 0;
  t.fcells = (double)d.fw * d.fh;
  t.cells = (double)d.gw * d.gh;
  return t;
}

namespace {

constexpr uint32_t MAX_STEPS = 64;

#define RB_TRY(expr, what)                         \
  do {                                             \
    ribo_status _st = cuda_status((expr), (what)); \
    if (_st != RIBO_OK) return _st;                \
  } while (0)

uint32_t clamp_substep(uint32_t s) { return s < 1 ? 1 : (s > 4 ? 4 : s); }

// Which blocks of the step run for a world: fluid (1), transport (2),
// aggregation counts (4) -- src/world/mod.rs:1527-1601.
uint32_t sched_bits(const World& w, const ribo_sim_params& p) {
  const uint32_t substep = clamp_substep(w.st.fluid_substep);
  const uint32_t te = p.transport_every < 1 ? 1 : p.transport_every;
  return (w.st.fluid_enabled && p.epoch % substep == 0u ? 1u : 0u) | (p.epoch % te == 0u ? 2u : 0u) |
         (p.aggregation > 0.0f ? 4u : 0u);
}

// Settings that must agree for worlds to share launches.
std::string class_key(const World& w, uint32_t sched) {
  std::string k;
  auto put = [&](uint32_t v) { k.append(reinterpret_cast<const char*>(&v), 4); };
  put(sched);
  put(w.st.multigrid);
  put(w.st.mg_unfused);
  put(w.st.mg_cycles < 1 ? 1 : w.st.mg_cycles);
  put(w.st.jacobi_iters);
  put(w.st.ledger_each_step);
  put(w.st.transport_simple);
  put(w.cfg.mg_pre);
  put(w.cfg.mg_post);
  put(w.cfg.mg_coarse);
  put(w.cfg.precision_mode);
  return k;
}

// Worlds that share the launches of a step, with their device tables.
struct Group {
  std::vector<int> members;  // indices into Batch::worlds
  void* blob = nullptr;      // geometry tables
  const int* start[GEO_COUNT] = {};
  const int* nbx[GEO_COUNT] = {};
  int total[GEO_COUNT] = {};
  double fcells = 0.0, cells = 0.0;
  std::map<std::string, Dev*> devs;  // device Dev tables by the members' current records
  MgBatchPlan* mg = nullptr;         // fused V-cycles of the members, or null (per-world solves)
  bool mg_built = false;
  ~Group() {
    if (blob) cudaFree(blob);
    for (auto& e : devs) cudaFree(e.second);
    multigrid_batch_free(mg);
  }
};

// The groups of one step, in launch order, and where their parameters and
// ledgers sit in the call's arrays.
struct StepUse {
  Group* g;
  uint32_t sched;
  size_t slot0;  // first entry of the group in the call's [steps][members] arrays
};

struct BatchGraph {
  std::string key;
  cudaGraphExec_t exec = nullptr;
  std::vector<uint32_t*> chem_end;
  std::vector<float*> temp_end, redox_end;
  uint64_t kernels = 0;
};

}  // namespace

struct Batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<World*> worlds;
  std::map<std::string, Group*> groups;
  std::vector<int> tile_mode;  // per fine level index (autotuned)
  // parameters: 2 slots x 64 steps x members, device + pinned staging
  ribo_sim_params* d_params = nullptr;
  ribo_sim_params* h_params = nullptr;
  size_t param_cap = 0;  // members the buffers hold
  cudaEvent_t param_ev[2] = {nullptr, nullptr};
  int param_slot = 0;
  uint32_t* d_ledgers = nullptr;  // [64][members][12]
  std::vector<std::vector<size_t>> ledger_slot;  // per step of the last call: slot of each member (or SIZE_MAX)
  uint32_t last_steps = 0;
  cudaEvent_t t0 = nullptr, t1 = nullptr, marks[8] = {};
  bool timing = false;
  KTimer timer;
  std::vector<BatchGraph> graphs;
  std::vector<std::string> seen_keys;
  bool table_error = false;
  bool capturing = false;

  ribo_status init(int dev);
  ~Batch();
  cudaError_t bind() const { return cudaSetDevice(device); }
  void clear_tables();
  Group* group(const std::vector<int>& members, const std::string& cls);
  ribo_status build_group(Group* g);
  const Dev* dev_table(Group* g);
  Target target(Group* g, const ribo_sim_params* P);
  void plan_mg(Group* g);
  ribo_status ensure_capacity();
  ribo_status step(const ribo_sim_params* per_step, uint32_t n, const uint32_t* member_steps);
  void record_step(const std::vector<StepUse>& uses, const ribo_sim_params* P0, uint32_t i);
  std::string graph_key(const std::vector<std::vector<StepUse>>& plan, uint32_t n, int slot) const;
  ribo_status record_graphed(const std::vector<std::vector<StepUse>>& plan, const ribo_sim_params* P0, uint32_t n,
                             int slot);
  ribo_status check_status();
  ribo_status autotune(uint32_t* modes_out);
};

ribo_status Batch::init(int dev) {
  device = dev;
  RB_TRY(bind(), "device");
  RB_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "stream");
  for (int k = 0; k < 2; k++) RB_TRY(cudaEventCreateWithFlags(&param_ev[k], cudaEventDisableTiming), "event");
  RB_TRY(cudaEventCreate(&t0), "event");
  RB_TRY(cudaEventCreate(&t1), "event");
  for (int k = 0; k < 8; k++) RB_TRY(cudaEventCreate(&marks[k]), "event");
  return RIBO_OK;
}

Batch::~Batch() {
  bind();
  if (stream) cudaStreamSynchronize(stream);
  for (World* w : worlds) {
    w->stream = w->own_stream;
    w->batch = nullptr;
  }
  clear_tables();
  if (d_params) cudaFree(d_params);
  if (h_params) cudaFreeHost(h_params);
  if (d_ledgers) cudaFree(d_ledgers);
  for (int k = 0; k < 2; k++)
    if (param_ev[k]) cudaEventDestroy(param_ev[k]);
  if (t0) cudaEventDestroy(t0);
  if (t1) cudaEventDestroy(t1);
  for (int k = 0; k < 8; k++)
    if (marks[k]) cudaEventDestroy(marks[k]);
  if (stream) cudaStreamDestroy(stream);
}

// Membership or tile shapes changed: every table and graph is rebuilt on use.
void Batch::clear_tables() {
  if (stream) cudaStreamSynchronize(stream);
  for (BatchGraph& g : graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  graphs.clear();
  seen_keys.clear();
  for (auto& e : groups) delete e.second;
  groups.clear();
}

Group* Batch::group(const std::vector<int>& members, const std::string& cls) {
  std::string key = cls;
  key.append(reinterpret_cast<const char*>(members.data()), members.size() * sizeof(int));
  auto it = groups.find(key);
  if (it != groups.end()) return it->second;
  Group* g = new Group;
  g->members = members;
  if (build_group(g) != RIBO_OK) table_error = true;
  groups[key] = g;
  return g;
}

// Geometry tables of a group: for every launch geometry, the first linear
// block of each member and its blocks per row.
ribo_status Batch::build_group(Group* g) {
  const size_t n = g->members.size();
  std::vector<int> host;
  size_t off_start[GEO_COUNT], off_nbx[GEO_COUNT];
  for (int k = 0; k < GEO_COUNT; k++) {
    std::vector<int> start(1, 0), nb;
    for (int m : g->members) {
      int x = 0, y = 0;
      geo_blocks((Geo)k, worlds[m]->dev(), &x, &y);
      nb.push_back(x);
      start.push_back(start.back() + x * y);
    }
    g->total[k] = start.back();
    off_start[k] = host.size();
    host.insert(host.end(), start.begin(), start.end());
    off_nbx[k] = host.size();
    host.insert(host.end(), nb.begin(), nb.end());
  }
  for (int m : g->members) {
    g->fcells += (double)worlds[m]->fcells();
    g->cells += (double)worlds[m]->cells();
  }
  RB_TRY(cudaMalloc(&g->blob, host.size() * sizeof(int)), "batch tables");
  RB_TRY(cudaMemcpy(g->blob, host.data(), host.size() * sizeof(int), cudaMemcpyHostToDevice), "batch tables");
  const int* base = static_cast<const int*>(g->blob);
  for (int k = 0; k < GEO_COUNT; k++) {
    g->start[k] = base + off_start[k];
    g->nbx[k] = base + off_nbx[k];
  }
  (void)n;
  return RIBO_OK;
}

// The members' current Dev records (ping-pong roles resolved) as a device
// table; one table per distinct state, kept while the group lives (the
// graphs that replay a step reference them).
const Dev* Batch::dev_table(Group* g) {
  std::vector<Dev> v;
  v.reserve(g->members.size());
  for (int m : g->members) v.push_back(worlds[m]->dev());
  std::string key(reinterpret_cast<const char*>(v.data()), v.size() * sizeof(Dev));
  auto it = g->devs.find(key);
  if (it != g->devs.end()) return it->second;
  if (capturing) {  // every state a captured sequence meets was met by its first, uncaptured run
    table_error = true;
    return nullptr;
  }
  Dev* p = nullptr;
  if (cudaMalloc(&p, v.size() * sizeof(Dev)) != cudaSuccess ||
      cudaMemcpy(p, v.data(), v.size() * sizeof(Dev), cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaGetLastError();
    if (p) cudaFree(p);
    table_error = true;
    return nullptr;
  }
  g->devs[key] = p;
  return p;
}

Target Batch::target(Group* g, const ribo_sim_params* P) {
  Target t;
  t.n = (int)g->members.size();
  t.devs = dev_table(g);
  t.P = P;
  for (int k = 0; k < GEO_COUNT; k++) {
    t.start[k] = g->start[k];
    t.nbx[k] = g->nbx[k];
    t.total[k] = t.devs ? g->total[k] : 0;  // no table: launch nothing (the call reports the error)
  }
  t.fcells = g->fcells;
  t.cells = g->cells;
  return t;
}

// The batched V-cycle plan of a group, when every member can use the fused
// multigrid with the same constants (a class key guarantees the latter).
void Batch::plan_mg(Group* g) {
  if (g->mg_built) return;
  g->mg_built = true;
  const World& w0 = *worlds[g->members[0]];
  // mixed-precision members solve one by one (their solver loops on its own
  // convergence test per world)
  if (w0.mixed || !w0.st.multigrid || w0.st.mg_unfused) return;
  const MgConfig c{(int)w0.cfg.mg_pre, (int)w0.cfg.mg_post, (int)w0.cfg.mg_coarse,
                   (int)(w0.st.mg_cycles < 1 ? 1 : w0.st.mg_cycles)};
  std::vector<MgWorld> mw;
  for (int m : g->members) {
    World& w = *worlds[m];
    if (!multigrid_fused_ok(w.levels.data(), (int)w.levels.size(), c)) return;
    mw.push_back(MgWorld{w.dev(), w.levels.data(), (int)w.levels.size(), w.mg});
  }
  if (capturing) {
    table_error = true;
    return;
  }
  g->mg = multigrid_batch_plan(mw.data(), (int)mw.size(), c, tile_mode.data(), (int)tile_mode.size(), stream);
  if (!g->mg) table_error = true;
}

ribo_status Batch::ensure_capacity() {
  const size_t n = worlds.size();
  if (n <= param_cap) return RIBO_OK;
  RB_TRY(cudaStreamSynchronize(stream), "batch");
  if (d_params) cudaFree(d_params);
  if (h_params) cudaFreeHost(h_params);
  if (d_ledgers) cudaFree(d_ledgers);
  d_params = nullptr;
  h_params = nullptr;
  d_ledgers = nullptr;
  param_cap = 0;
  size_t cap = n < 16 ? 16 : n;
  RB_TRY(cudaMalloc((void**)&d_params, 2 * MAX_STEPS * cap * sizeof(ribo_sim_params)), "batch params");
  RB_TRY(cudaMallocHost((void**)&h_params, 2 * MAX_STEPS * cap * sizeof(ribo_sim_params)), "batch params");
  RB_TRY(cudaMalloc((void**)&d_ledgers, MAX_STEPS * cap * 12 * sizeof(uint32_t)), "batch ledgers");
  param_cap = cap;
  // the graphs captured so far point into the old buffers
  for (BatchGraph& g : graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  graphs.clear();
  seen_keys.clear();
  return RIBO_OK;
}

// One step of every group (the fluid and transport blocks of
// src/world/mod.rs:1527-1601 per group, then the ledger).
void Batch::record_step(const std::vector<StepUse>& uses, const ribo_sim_params* P0, uint32_t i) {
  (void)i;
  for (const StepUse& u : uses) {
    Group* g = u.g;
    const ribo_sim_params* P = P0 + u.slot0;
    const World& w0 = *worlds[g->members[0]];
    if (u.sched & 1u) {
      launch_temperature(target(g, P), stream);
      for (int m : g->members) {
        std::swap(worlds[m]->temp_cur, worlds[m]->temp_nxt);
        std::swap(worlds[m]->redox_cur, worlds[m]->redox_nxt);
      }
      const Target t = target(g, P);
      launch_forces(t, stream);
      launch_add_forces(t, A_TO_B, stream);
      launch_diffuse(t, B_TO_A, stream);
      launch_advect(t, A_TO_B, stream);
      launch_vorticity(t, B_TO_A, stream);
      launch_divergence(t, A_TO_B, stream);
      plan_mg(g);
      if (g->mg) {
        launch_multigrid_batch(g->mg, stream);
      } else {
        for (int m : g->members) worlds[m]->pressure_solve(worlds[m]->dev());
      }
      launch_subtract_gradient(t, A_TO_B, stream);
      launch_net_flux(t, B_TO_A, stream);
      launch_boundaries(t, B_TO_A, stream);
      launch_smooth(t, A_TO_B, stream);
      launch_thermal(t, stream);
    }
    if (u.sched & 2u) {
      const Target t = target(g, P);
      if (u.sched & 4u) launch_agg(t, stream);
      launch_scatter(t, w0.st.transport_simple != 0, stream);
      for (int m : g->members) std::swap(worlds[m]->chem_cur, worlds[m]->chem_nxt);  // transport_commit
      launch_zero_next(target(g, P), stream);
    }
    if (w0.st.ledger_each_step) launch_ledger(target(g, P), d_ledgers + u.slot0 * 12, stream);
  }
}

std::string Batch::graph_key(const std::vector<std::vector<StepUse>>& plan, uint32_t n, int slot) const {
  std::string k;
  auto put = [&](const void* p, size_t b) { k.append(reinterpret_cast<const char*>(p), b); };
  put(&n, 4);
  put(&slot, 4);
  for (const World* w : worlds) {
    put(&w, sizeof w);
    put(&w->chem_cur, sizeof(void*));
    put(&w->temp_cur, sizeof(void*));
    put(&w->redox_cur, sizeof(void*));
  }
  for (const auto& uses : plan)
    for (const StepUse& u : uses) {
      put(&u.g, sizeof u.g);
      put(&u.sched, 4);
      put(&u.slot0, sizeof u.slot0);
    }
  return k;
}

ribo_status Batch::record_graphed(const std::vector<std::vector<StepUse>>& plan, const ribo_sim_params* P0, uint32_t n,
                                  int slot) {
  auto record_all = [&]() {
    for (uint32_t i = 0; i < n; i++) record_step(plan[i], P0, i);
  };
  const bool no_graphs = worlds.empty() || worlds[0]->cfg.no_graphs;
  if (no_graphs) {
    record_all();
    return RIBO_OK;
  }
  const std::string key = graph_key(plan, n, slot);
  for (BatchGraph& g : graphs) {
    if (g.key != key) continue;
    RB_TRY(cudaGraphLaunch(g.exec, stream), "graph launch");
    for (size_t k = 0; k < worlds.size(); k++) {
      World& w = *worlds[k];
      w.chem_cur = g.chem_end[k];
      w.chem_nxt = w.chem_cur == w.chem_a ? w.chem_b : w.chem_a;
      w.temp_cur = g.temp_end[k];
      w.temp_nxt = w.temp_cur == w.temp_a ? w.temp_b : w.temp_a;
      w.redox_cur = g.redox_end[k];
      w.redox_nxt = w.redox_cur == w.redox_a ? w.redox_b : w.redox_a;
    }
    ktime_add_launches(g.kernels);
    return RIBO_OK;
  }
  bool seen = false;
  for (const std::string& s : seen_keys) seen = seen || s == key;
  if (!seen) {
    if (seen_keys.size() >= 16) seen_keys.erase(seen_keys.begin());
    seen_keys.push_back(key);
    record_all();
    return RIBO_OK;
  }
  const uint64_t l0 = ktime_launch_count();
  RB_TRY(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "capture");
  capturing = true;
  record_all();
  capturing = false;
  cudaGraph_t graph = nullptr;
  RB_TRY(cudaStreamEndCapture(stream, &graph), "capture");
  BatchGraph e;
  e.key = key;
  e.kernels = ktime_launch_count() - l0;
  cudaError_t err = cudaGraphInstantiate(&e.exec, graph, 0);
  cudaGraphDestroy(graph);
  RB_TRY(err, "graph instantiate");
  for (World* w : worlds) {
    e.chem_end.push_back(w->chem_cur);
    e.temp_end.push_back(w->temp_cur);
    e.redox_end.push_back(w->redox_cur);
  }
  RB_TRY(cudaGraphLaunch(e.exec, stream), "graph launch");
  if (graphs.size() >= 8) {
    cudaGraphExecDestroy(graphs.front().exec);
    graphs.erase(graphs.begin());
  }
  graphs.push_back(std::move(e));
  return RIBO_OK;
}

ribo_status Batch::step(const ribo_sim_params* per_step, uint32_t n, const uint32_t* member_steps) {
  if (n == 0 || worlds.empty()) return RIBO_OK;
  if (!per_step) return set_error(RIBO_INVALID_ARG, "null params");
  if (n > MAX_STEPS) return set_error(RIBO_INVALID_ARG, "%u steps per call (at most %u)", n, MAX_STEPS);
  if (member_steps)
    for (size_t k = 0; k < worlds.size(); k++)
      if (member_steps[k] > n) return set_error(RIBO_INVALID_ARG, "member %zu: %u steps of %u", k, member_steps[k], n);
  for (size_t k = 0; k < worlds.size(); k++)
    if (worlds[k]->st.light_mode)
      return set_error(RIBO_INVALID_ARG, "member %zu: batches take worlds whose light is a frozen input (light_mode 0)", k);
  for (size_t k = 0; k < worlds.size(); k++)
    if (worlds[k]->st.terrain_mode)
      return set_error(RIBO_INVALID_ARG, "member %zu: batches take worlds whose terrain is a frozen input (terrain_mode 0)", k);
  RB_TRY(bind(), "device");
  {
    ribo_status s = ensure_capacity();
    if (s != RIBO_OK) return s;
  }
  const size_t N = worlds.size();
  // src/world/mod.rs:1414-1421: turning the fluid off clears it once.
  for (World* w : worlds) {
    if (!w->st.fluid_enabled && w->fluid_was_on) {
      RB_TRY(cudaMemsetAsync(w->va, 0, w->fcells() * 8, stream), "clear");
      RB_TRY(cudaMemsetAsync(w->temp_cur, 0, w->fcells() * 4, stream), "clear");
      RB_TRY(cudaMemsetAsync(w->redox_cur, 0, w->fcells() * 4, stream), "clear");
    }
    w->fluid_was_on = w->st.fluid_enabled != 0;
  }
  const int slot = param_slot;
  param_slot ^= 1;
  RB_TRY(cudaEventSynchronize(param_ev[slot]), "param slot");
  ribo_sim_params* hs = h_params + (size_t)slot * MAX_STEPS * param_cap;
  ribo_sim_params* ds = d_params + (size_t)slot * MAX_STEPS * param_cap;

  // Group the members of every step; lay the parameters (and ledgers) out
  // as [step][group][member].
  std::vector<std::vector<StepUse>> plan(n);
  ledger_slot.assign(n, std::vector<size_t>(N, SIZE_MAX));
  size_t cursor = 0;
  table_error = false;
  for (uint32_t i = 0; i < n; i++) {
    std::vector<std::string> keys;
    std::vector<std::vector<int>> members;
    std::vector<uint32_t> scheds;
    for (size_t k = 0; k < N; k++) {
      if (member_steps && i >= member_steps[k]) continue;
      const ribo_sim_params& p = per_step[k * n + i];
      const uint32_t sb = sched_bits(*worlds[k], p);
      const std::string ck = class_key(*worlds[k], sb);
      size_t j = 0;
      while (j < keys.size() && keys[j] != ck) j++;
      if (j == keys.size()) {
        keys.push_back(ck);
        members.emplace_back();
        scheds.push_back(sb);
      }
      members[j].push_back((int)k);
    }
    for (size_t j = 0; j < keys.size(); j++) {
      Group* g = group(members[j], keys[j]);
      plan[i].push_back(StepUse{g, scheds[j], cursor});
      for (int m : members[j]) {
        hs[cursor] = per_step[(size_t)m * n + i];
        if (worlds[m]->st.ledger_each_step) ledger_slot[i][m] = cursor;
        cursor++;
      }
    }
  }
  if (table_error) return set_error(RIBO_OOM, "batch tables: out of device memory");
  RB_TRY(cudaEventRecord(t0, stream), "event");
  RB_TRY(cudaMemcpyAsync(ds, hs, cursor * sizeof(ribo_sim_params), cudaMemcpyHostToDevice, stream), "params");
  RB_TRY(cudaEventRecord(param_ev[slot], stream), "event");
  bool any_ledger = false;
  for (World* w : worlds) any_ledger = any_ledger || w->st.ledger_each_step;
  if (any_ledger) RB_TRY(cudaMemsetAsync(d_ledgers, 0, cursor * 12 * sizeof(uint32_t), stream), "ledgers");
  if (timing) {
    ktime_set_active(&timer);
    for (uint32_t i = 0; i < n; i++) record_step(plan[i], ds, i);
    ktime_set_active(nullptr);
  } else {
    ribo_status s = record_graphed(plan, ds, n, slot);
    if (s != RIBO_OK) return s;
  }
  if (table_error) return set_error(RIBO_OOM, "batch tables: out of device memory");
  last_steps = n;
  for (World* w : worlds) {  // a mixed-precision solve that failed to record
    if (w->solve_error != RIBO_OK) {
      const ribo_status s = w->solve_error;
      for (World* v : worlds) v->solve_error = RIBO_OK;
      return s;
    }
  }
  RB_TRY(cudaGetLastError(), "batch step launch");
  RB_TRY(cudaEventRecord(t1, stream), "event");
  return RIBO_OK;
}

ribo_status Batch::check_status() {
  for (World* w : worlds) {
    ribo_status s = w->check_status();
    if (s != RIBO_OK) return s;
  }
  return RIBO_OK;
}

// Times the tile shapes of the pre-smooth launches per fine level index
// (those launches only write arrays that the next V-cycle rewrites before
// reading them, so timing them leaves the worlds' state as it was).
ribo_status Batch::autotune(uint32_t* modes_out) {
  if (modes_out)
    for (int l = 0; l < 8; l++) modes_out[l] = 0;
  if (worlds.empty()) return RIBO_OK;
  RB_TRY(bind(), "device");
  const World& w0 = *worlds[0];
  const MgConfig c{(int)w0.cfg.mg_pre, (int)w0.cfg.mg_post, (int)w0.cfg.mg_coarse, 1};
  std::vector<MgWorld> mw;
  for (World* w : worlds) {
    if (w->mixed || w->cfg.mg_pre != w0.cfg.mg_pre || w->cfg.mg_post != w0.cfg.mg_post) continue;
    if (!multigrid_fused_ok(w->levels.data(), (int)w->levels.size(), c)) continue;
    mw.push_back(MgWorld{w->dev(), w->levels.data(), (int)w->levels.size(), w->mg});
  }
  if (mw.empty()) return RIBO_OK;
  MgBatchPlan* probe = multigrid_batch_plan(mw.data(), (int)mw.size(), c, nullptr, 0, stream);
  if (!probe) return set_error(RIBO_OOM, "autotune tables");
  const int levels = multigrid_batch_levels(probe);
  multigrid_batch_free(probe);
  std::vector<int> modes(levels > 0 ? levels : 0, 0);
  cudaEvent_t a, b;
  RB_TRY(cudaEventCreate(&a), "event");
  RB_TRY(cudaEventCreate(&b), "event");
  for (int l = 0; l < levels; l++) {
    int best = 0;
    float best_ms = 1e30f;
    for (int m = 0; m < 3; m++) {
      std::vector<int> trial = modes;
      trial[l] = m;
      MgBatchPlan* p = multigrid_batch_plan(mw.data(), (int)mw.size(), c, trial.data(), (int)trial.size(), stream);
      if (!p) {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        return set_error(RIBO_OOM, "autotune tables");
      }
      for (int r = 0; r < 2; r++) launch_multigrid_batch_pre(p, l, stream);
      cudaEventRecord(a, stream);
      for (int r = 0; r < 5; r++) launch_multigrid_batch_pre(p, l, stream);
      cudaEventRecord(b, stream);
      cudaError_t e = cudaEventSynchronize(b);
      float ms = 0.0f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
      multigrid_batch_free(p);
      if (e != cudaSuccess) {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        return cuda_status(e, "autotune");
      }
      if (ms < best_ms) {
        best_ms = ms;
        best = m;
      }
    }
    modes[l] = best;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  tile_mode = modes;
  clear_tables();
  if (modes_out)
    for (int l = 0; l < levels && l < 8; l++) modes_out[l] = (uint32_t)modes[l];
  return check_status();
}

}  // namespace ribo

using ribo::set_error;

// ---------------------------------------------------------------------------
// C ABI

struct ribo_batch {
  ribo::Batch b;
};

extern "C" {

ribo_status ribo_batch_create(uint32_t device, ribo_batch** out) {
  if (!out) return set_error(RIBO_INVALID_ARG, "null argument");
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return set_error(RIBO_CUDA_ERROR, "no CUDA device");
  }
  if ((int)device >= count) return set_error(RIBO_INVALID_ARG, "device %u does not exist", device);
  ribo_batch* b = new (std::nothrow) ribo_batch();
  if (!b) return set_error(RIBO_OOM, "host allocation");
  ribo_status st = b->b.init((int)device);
  if (st != RIBO_OK) {
    delete b;
    return st;
  }
  *out = b;
  return RIBO_OK;
}

void ribo_batch_destroy(ribo_batch* b) { delete b; }

ribo_status ribo_batch_add(ribo_batch* b, ribo_world* w) {
  if (!b || !w) return set_error(RIBO_INVALID_ARG, "null argument");
  ribo::World& wd = w->w;
  if (wd.batch) return set_error(RIBO_INVALID_ARG, "world already belongs to a batch");
  if ((int)wd.cfg.device != b->b.device) return set_error(RIBO_INVALID_ARG, "world lives on another device");
  ribo_status st = ribo::cuda_status(b->b.bind(), "device");
  if (st != RIBO_OK) return st;
  st = ribo::cuda_status(cudaStreamSynchronize(wd.stream), "sync");
  if (st != RIBO_OK) return st;
  b->b.clear_tables();
  wd.stream = b->b.stream;
  wd.batch = b;
  b->b.worlds.push_back(&wd);
  return RIBO_OK;
}

ribo_status ribo_batch_remove(ribo_batch* b, ribo_world* w) {
  if (!b || !w) return set_error(RIBO_INVALID_ARG, "null argument");
  auto& ws = b->b.worlds;
  for (size_t k = 0; k < ws.size(); k++) {
    if (ws[k] != &w->w) continue;
    ribo_status st = ribo::cuda_status(b->b.bind(), "device");
    if (st != RIBO_OK) return st;
    b->b.clear_tables();  // waits for the batch's stream
    w->w.stream = w->w.own_stream;
    w->w.batch = nullptr;
    ws.erase(ws.begin() + (long)k);
    return RIBO_OK;
  }
  return set_error(RIBO_INVALID_ARG, "world is not a member of this batch");
}

uint32_t ribo_batch_size(const ribo_batch* b) { return b ? (uint32_t)b->b.worlds.size() : 0u; }

ribo_status ribo_batch_step(ribo_batch* b, const ribo_sim_params* per_step, uint32_t n) {
  if (!b) return set_error(RIBO_INVALID_ARG, "null batch");
  return b->b.step(per_step, n, nullptr);
}

ribo_status ribo_batch_step_ragged(ribo_batch* b, const ribo_sim_params* per_step, uint32_t n,
                                   const uint32_t* member_steps) {
  if (!b || !member_steps) return set_error(RIBO_INVALID_ARG, "null argument");
  return b->b.step(per_step, n, member_steps);
}

ribo_status ribo_batch_encode_steps(ribo_batch* b, ribo_sim_params* params, uint32_t n) {
  if (!b || !params) return set_error(RIBO_INVALID_ARG, "null argument");
  if (n > 64) n = 64;
  const size_t N = b->b.worlds.size();
  if (n == 0 || N == 0) return RIBO_OK;
  std::vector<ribo_sim_params> buf(N * n);
  for (size_t k = 0; k < N; k++) {
    ribo_status st = ribo_derive_step_params(&params[k], &b->b.worlds[k]->st, n, &buf[k * n]);
    if (st != RIBO_OK) return st;
  }
  ribo_status st = b->b.step(buf.data(), n, nullptr);
  if (st != RIBO_OK) return st;
  for (size_t k = 0; k < N; k++) {
    const ribo_world_settings& s = b->b.worlds[k]->st;
    const uint32_t substep = s.fluid_substep < 1 ? 1 : (s.fluid_substep > 4 ? 4 : s.fluid_substep);
    params[k].fluid_dt = params[k].dt * (float)substep;
    params[k].fluid_enabled = s.fluid_enabled ? 1u : 0u;
    params[k].epoch += n;
  }
  return RIBO_OK;
}

ribo_status ribo_batch_step_ledgers(ribo_batch* b, uint32_t* out, uint32_t n) {
  if (!b || (!out && n)) return set_error(RIBO_INVALID_ARG, "null argument");
  ribo::Batch& B = b->b;
  if (n > B.last_steps) return set_error(RIBO_INVALID_ARG, "last call recorded %u steps", B.last_steps);
  const size_t N = B.worlds.size();
  if (n == 0 || N == 0) return RIBO_OK;
  ribo_status st = ribo::cuda_status(B.bind(), "device");
  if (st != RIBO_OK) return st;
  std::vector<uint32_t> h((size_t)n * N * 12);
  st = ribo::cuda_status(cudaMemcpyAsync(h.data(), B.d_ledgers, h.size() * 4, cudaMemcpyDeviceToHost, B.stream), "ledgers");
  if (st != RIBO_OK) return st;
  st = ribo::cuda_status(cudaStreamSynchronize(B.stream), "ledgers");
  if (st != RIBO_OK) return st;
  for (size_t k = 0; k < N; k++)
    for (uint32_t i = 0; i < n; i++) {
      uint32_t* o = out + ((size_t)k * n + i) * 12;
      const size_t sl = i < B.ledger_slot.size() ? B.ledger_slot[i][k] : SIZE_MAX;
      if (sl == SIZE_MAX) memset(o, 0, 48);
      else memcpy(o, &h[sl * 12], 48);
    }
  return B.check_status();
}

ribo_status ribo_batch_sync(ribo_batch* b) {
  if (!b) return set_error(RIBO_INVALID_ARG, "null batch");
  ribo_status st = ribo::cuda_status(b->b.bind(), "device");
  if (st != RIBO_OK) return st;
  st = ribo::cuda_status(cudaStreamSynchronize(b->b.stream), "sync");
  if (st != RIBO_OK) return st;
  return b->b.check_status();
}

ribo_status ribo_batch_mark(ribo_batch* b, uint32_t slot) {
  if (!b || slot >= 8) return set_error(RIBO_INVALID_ARG, "bad mark slot");
  return ribo::cuda_status(cudaEventRecord(b->b.marks[slot], b->b.stream), "mark");
}

ribo_status ribo_batch_elapsed_ms(ribo_batch* b, uint32_t a, uint32_t c, float* ms) {
  if (!b || a >= 8 || c >= 8 || !ms) return set_error(RIBO_INVALID_ARG, "bad mark slot");
  ribo_status st = ribo::cuda_status(cudaEventSynchronize(b->b.marks[c]), "mark");
  if (st != RIBO_OK) return st;
  return ribo::cuda_status(cudaEventElapsedTime(ms, b->b.marks[a], b->b.marks[c]), "elapsed");
}

ribo_status ribo_batch_autotune(ribo_batch* b, uint32_t* modes_out) {
  if (!b) return set_error(RIBO_INVALID_ARG, "null batch");
  return b->b.autotune(modes_out);
}

ribo_status ribo_batch_set_tile_modes(ribo_batch* b, const uint32_t* modes, uint32_t n) {
  if (!b || (!modes && n)) return set_error(RIBO_INVALID_ARG, "null argument");
  for (uint32_t l = 0; l < n; l++)
    if (modes[l] > 2) return set_error(RIBO_INVALID_ARG, "tile mode %u at level %u (0, 1 or 2)", modes[l], l);
  ribo_status st = ribo::cuda_status(b->b.bind(), "device");
  if (st != RIBO_OK) return st;
  b->b.tile_mode.assign(modes, modes + n);
  b->b.clear_tables();
  return RIBO_OK;
}

ribo_status ribo_batch_enable_kernel_timing(ribo_batch* b, int enable) {
  if (!b) return set_error(RIBO_INVALID_ARG, "null batch");
  b->b.timing = enable != 0;
  return RIBO_OK;
}

ribo_status ribo_batch_read_kernel_timing(ribo_batch* b, ribo_kernel_timing* out, uint32_t cap, uint32_t* count) {
  if (!b) return set_error(RIBO_INVALID_ARG, "null batch");
  ribo_status st = ribo::cuda_status(b->b.bind(), "device");
  if (st != RIBO_OK) return st;
  st = ribo::cuda_status(cudaStreamSynchronize(b->b.stream), "timing");
  if (st != RIBO_OK) return st;
  return ribo::ktimer_read(b->b.timer, out, cap, count);
}

}  // extern "C"
