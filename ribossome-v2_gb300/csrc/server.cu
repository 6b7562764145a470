// World-step serving with continuous batching (ribo_server_* of the C ABI).
//
// The scheduler is a client of the world and batch entry points: each
// resident job owns a ribo_world that is a member of the server's
// ribo_batch, so every iteration advances all resident jobs -- whatever
// their sizes -- in the same launches.  Admission is FIFO against an HBM
// budget counted in world footprints (ribo_world_footprint); worlds come
// from the device's stream-ordered pool, so admitting and retiring jobs
// never synchronises the device beyond the one wait per iteration.
//
// One iteration:
//   1. admit queued jobs that fit: create their worlds and upload their
//      fields on the worlds' own streams while the previous chunk still runs
//      on the batch's stream;
//   2. wait for the previous chunk, record its device time;
//   3. retire the jobs that ran all their steps (ledger, result fields,
//      world freed);
//   4. add the admitted worlds to the batch and launch the next chunk: a
//      ragged batched call in which job k runs min(remaining_k, chunk) steps.
#include <cuda_runtime.h>
#include <string.h>

#include <chrono>
#include <deque>
#include <vector>

#include "../../include/ribo_world.h"
#include "ribo_world_impl.h"

namespace ribo {
namespace {

struct Job {
  uint64_t id = 0;
  ribo_job desc{};
  std::vector<std::vector<unsigned char>> data;  // owned copies of the input fields
  uint64_t footprint = 0;
  double t_submit = 0.0, t_admit = 0.0;
  ribo_world* w = nullptr;
  ribo_sim_params params{};
  uint32_t done = 0;
  uint32_t remaining() const { return desc.steps - done; }
};

bool derived_field(int f) {
  return f == RIBO_FIELD_SLOPE || f == RIBO_FIELD_SOLID_MASK || f == RIBO_FIELD_NET_FLUX || f == RIBO_FIELD_VEL_SMOOTH;
}

}  // namespace

struct Server {
  ribo_server_cfg cfg{};
  ribo_batch* batch = nullptr;
  std::deque<Job*> pending;
  std::vector<Job*> active;    // members of the batch, in membership order
  std::vector<Job*> joining;   // admitted, not yet members
  std::deque<ribo_job_result> results;
  std::vector<float> it_ms;
  std::vector<uint32_t> it_steps, it_active;
  bool chunk_in_flight = false;
  uint32_t chunk_steps = 0, chunk_active = 0;
  uint64_t next_id = 1;
  uint64_t submitted = 0, admitted = 0, completed = 0, world_steps = 0, iterations = 0;
  uint64_t bytes_in_use = 0;
  double gpu_ms = 0.0;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();

  double now_ms() const {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  ~Server();
  ribo_status submit(const ribo_job& j, uint64_t* id);
  ribo_status admit();
  ribo_status finish_chunk();
  ribo_status retire();
  ribo_status launch_chunk();
  ribo_status iterate(uint32_t* active_out);
  void fail(Job* j, ribo_status st);
};

Server::~Server() {
  if (batch) ribo_batch_destroy(batch);  // waits for the batch's stream, releases the members
  for (Job* j : active) {
    ribo_world_destroy(j->w);
    delete j;
  }
  for (Job* j : joining) {
    ribo_world_destroy(j->w);
    delete j;
  }
  for (Job* j : pending) delete j;
}

void Server::fail(Job* j, ribo_status st) {
  ribo_job_result r{};
  r.id = j->id;
  r.user_tag = j->desc.user_tag;
  r.status = (int32_t)st;
  r.steps = j->done;
  r.device_bytes = j->footprint;
  r.t_submit_ms = j->t_submit;
  r.t_admit_ms = j->t_admit;
  r.t_done_ms = now_ms();
  results.push_back(r);
  delete j;
}

ribo_status Server::submit(const ribo_job& jd, uint64_t* id) {
  if (jd.steps == 0) return set_error(RIBO_INVALID_ARG, "job with 0 steps");
  if (jd.world.device != cfg.device) return set_error(RIBO_INVALID_ARG, "job world on device %u, server on %u",
                                                      jd.world.device, cfg.device);
  uint64_t fp = 0;
  ribo_status st = ribo_world_footprint(&jd.world, &fp);
  if (st != RIBO_OK) return st;
  if (fp > cfg.hbm_budget_bytes)
    return set_error(RIBO_OVER_BUDGET, "job needs %llu device bytes, budget %llu", (unsigned long long)fp,
                     (unsigned long long)cfg.hbm_budget_bytes);
  Job* j = new (std::nothrow) Job;
  if (!j) return set_error(RIBO_OOM, "host allocation");
  j->desc = jd;
  j->footprint = fp;
  j->data.resize(RIBO_FIELD_COUNT);
  for (int f = 0; f < RIBO_FIELD_COUNT; f++) {
    const size_t n = field_bytes_of(jd.world, (ribo_field)f);
    if (jd.inputs[f]) {
      if (derived_field(f)) {
        delete j;
        return set_error(RIBO_INVALID_ARG, "field %d is derived and cannot be an input", f);
      }
      j->data[f].assign(static_cast<const unsigned char*>(jd.inputs[f]),
                        static_cast<const unsigned char*>(jd.inputs[f]) + n);
    }
    j->desc.inputs[f] = nullptr;
  }
  j->params = jd.params;
  j->id = next_id++;
  j->t_submit = now_ms();
  pending.push_back(j);
  submitted++;
  if (id) *id = j->id;
  return RIBO_OK;
}

// Creates and seeds the worlds of queued jobs that fit, in arrival order.
ribo_status Server::admit() {
  while (!pending.empty()) {
    const size_t resident = active.size() + joining.size();
    if (cfg.max_active && resident >= cfg.max_active) break;
    Job* j = pending.front();
    if (bytes_in_use + j->footprint > cfg.hbm_budget_bytes) break;
    ribo_world* w = nullptr;
    ribo_status st = ribo_world_create(&j->desc.world, &w);
    if (st == RIBO_OOM && resident > 0) break;  // device memory frees up as jobs retire
    pending.pop_front();
    if (st != RIBO_OK) {
      fail(j, st);
      continue;
    }
    st = ribo_world_set_settings(w, &j->desc.settings);
    const int order[RIBO_FIELD_COUNT] = {RIBO_FIELD_GAMMA, 0, 2, 4, 5, 6, 7, 8, 11, 12, 13, 15, 3, 9, 10, 14};
    for (int k = 0; k < RIBO_FIELD_COUNT && st == RIBO_OK; k++) {
      const int f = order[k];
      if (!j->data[f].empty()) st = ribo_world_upload(w, (ribo_field)f, j->data[f].data(), j->data[f].size());
    }
    if (st != RIBO_OK) {
      ribo_world_destroy(w);
      fail(j, st);
      continue;
    }
    j->data.clear();
    j->data.shrink_to_fit();
    j->w = w;
    j->t_admit = now_ms();
    bytes_in_use += j->footprint;
    joining.push_back(j);
    admitted++;
  }
  return RIBO_OK;
}

// Waits for the chunk in flight and records its device time.
ribo_status Server::finish_chunk() {
  if (!chunk_in_flight) return RIBO_OK;
  chunk_in_flight = false;
  ribo_status st = ribo_batch_sync(batch);
  if (st != RIBO_OK) return st;
  float ms = 0.0f;
  st = ribo_batch_elapsed_ms(batch, 0, 1, &ms);
  if (st != RIBO_OK) return st;
  gpu_ms += ms;
  it_ms.push_back(ms);
  it_steps.push_back(chunk_steps);
  it_active.push_back(chunk_active);
  return RIBO_OK;
}

// Results of the jobs that ran all their steps; their worlds are freed.
ribo_status Server::retire() {
  std::vector<Job*> keep;
  for (Job* j : active) {
    if (j->remaining() > 0) {
      keep.push_back(j);
      continue;
    }
    ribo_job_result r{};
    r.id = j->id;
    r.user_tag = j->desc.user_tag;
    r.steps = j->done;
    r.device_bytes = j->footprint;
    r.t_submit_ms = j->t_submit;
    r.t_admit_ms = j->t_admit;
    r.t_done_ms = now_ms();
    ribo_status st = ribo_batch_remove(batch, j->w);
    if (st == RIBO_OK) st = ribo_world_ledger(j->w, r.ledger);
    for (int f = 0; f < RIBO_FIELD_COUNT && st == RIBO_OK; f++)
      if (j->desc.outputs[f])
        st = ribo_world_read(j->w, (ribo_field)f, j->desc.outputs[f], field_bytes_of(j->desc.world, (ribo_field)f));
    r.status = (int32_t)st;
    ribo_world_destroy(j->w);
    bytes_in_use -= j->footprint;
    results.push_back(r);
    completed++;
    delete j;
  }
  active.swap(keep);
  return RIBO_OK;
}

// Joins the admitted worlds and launches the next ragged chunk.
ribo_status Server::launch_chunk() {
  for (Job* j : joining) {
    ribo_status st = ribo_batch_add(batch, j->w);
    if (st != RIBO_OK) return st;
    active.push_back(j);
  }
  joining.clear();
  if (active.empty()) return RIBO_OK;
  uint32_t chunk = cfg.max_chunk_steps, longest = 0;
  for (Job* j : active) longest = j->remaining() > longest ? j->remaining() : longest;
  const uint32_t n = chunk < longest ? chunk : longest;
  const size_t N = active.size();
  std::vector<ribo_sim_params> buf(N * n);
  std::vector<uint32_t> member_steps(N);
  for (size_t k = 0; k < N; k++) {
    Job* j = active[k];
    const uint32_t m = j->remaining() < n ? j->remaining() : n;
    member_steps[k] = m;
    ribo_status st = ribo_derive_step_params(&j->params, &j->desc.settings, m, &buf[k * n]);
    if (st != RIBO_OK) return st;
    for (uint32_t i = m; i < n; i++) buf[k * n + i] = buf[k * n + (m ? m - 1 : 0)];
  }
  ribo_status st = ribo_batch_mark(batch, 0);
  if (st == RIBO_OK) st = ribo_batch_step_ragged(batch, buf.data(), n, member_steps.data());
  if (st == RIBO_OK) st = ribo_batch_mark(batch, 1);
  if (st != RIBO_OK) return st;
  uint64_t steps = 0;
  for (size_t k = 0; k < N; k++) {
    Job* j = active[k];
    const ribo_world_settings& s = j->desc.settings;
    const uint32_t substep = s.fluid_substep < 1 ? 1 : (s.fluid_substep > 4 ? 4 : s.fluid_substep);
    j->params.fluid_dt = j->params.dt * (float)substep;  // as ribo_world_encode_steps leaves it
    j->params.fluid_enabled = s.fluid_enabled ? 1u : 0u;
    j->params.epoch += member_steps[k];
    j->done += member_steps[k];
    steps += member_steps[k];
  }
  world_steps += steps;
  chunk_in_flight = true;
  chunk_steps = n;
  chunk_active = (uint32_t)N;
  return RIBO_OK;
}

ribo_status Server::iterate(uint32_t* active_out) {
  ribo_status st = admit();
  if (st == RIBO_OK) st = finish_chunk();
  if (st == RIBO_OK) st = retire();
  if (st == RIBO_OK) st = launch_chunk();
  iterations++;
  if (active_out) *active_out = (uint32_t)(active.size() + joining.size());
  return st;
}

}  // namespace ribo

using ribo::set_error;

struct ribo_server {
  ribo::Server s;
};

extern "C" {

ribo_status ribo_server_create(const ribo_server_cfg* cfg, ribo_server** out) {
  if (!cfg || !out) return set_error(RIBO_INVALID_ARG, "null argument");
  *out = nullptr;
  if (cfg->max_chunk_steps < 1 || cfg->max_chunk_steps > 64)
    return set_error(RIBO_INVALID_ARG, "max_chunk_steps %u (1..64)", cfg->max_chunk_steps);
  if (cfg->hbm_budget_bytes == 0) return set_error(RIBO_INVALID_ARG, "zero HBM budget");
  ribo_server* s = new (std::nothrow) ribo_server();
  if (!s) return set_error(RIBO_OOM, "host allocation");
  s->s.cfg = *cfg;
  ribo_status st = ribo_batch_create(cfg->device, &s->s.batch);
  if (st != RIBO_OK) {
    delete s;
    return st;
  }
  *out = s;
  return RIBO_OK;
}

void ribo_server_destroy(ribo_server* s) { delete s; }

ribo_status ribo_server_submit(ribo_server* s, const ribo_job* job, uint64_t* id) {
  if (!s || !job) return set_error(RIBO_INVALID_ARG, "null argument");
  return s->s.submit(*job, id);
}

ribo_status ribo_server_iterate(ribo_server* s, uint32_t* active) {
  if (!s) return set_error(RIBO_INVALID_ARG, "null server");
  return s->s.iterate(active);
}

ribo_status ribo_server_drain(ribo_server* s) {
  if (!s) return set_error(RIBO_INVALID_ARG, "null server");
  ribo::Server& S = s->s;
  for (;;) {
    uint32_t a = 0;
    ribo_status st = S.iterate(&a);
    if (st != RIBO_OK) return st;
    if (a == 0 && S.pending.empty() && !S.chunk_in_flight) return RIBO_OK;
  }
}

ribo_status ribo_server_results(ribo_server* s, ribo_job_result* out, uint32_t cap, uint32_t* n) {
  if (!s || (!out && cap)) return set_error(RIBO_INVALID_ARG, "null argument");
  uint32_t k = 0;
  while (k < cap && !s->s.results.empty()) {
    out[k++] = s->s.results.front();
    s->s.results.pop_front();
  }
  if (n) *n = k;
  return RIBO_OK;
}

ribo_status ribo_server_get_stats(const ribo_server* s, ribo_server_stats* out) {
  if (!s || !out) return set_error(RIBO_INVALID_ARG, "null argument");
  const ribo::Server& S = s->s;
  out->submitted = S.submitted;
  out->admitted = S.admitted;
  out->completed = S.completed;
  out->pending = S.pending.size();
  out->active = S.active.size() + S.joining.size();
  out->bytes_in_use = S.bytes_in_use;
  out->world_steps = S.world_steps;
  out->iterations = S.iterations;
  out->gpu_ms = S.gpu_ms;
  return RIBO_OK;
}

ribo_status ribo_server_iterations(ribo_server* s, float* ms, uint32_t* steps, uint32_t* active, uint32_t cap,
                                   uint32_t* n) {
  if (!s) return set_error(RIBO_INVALID_ARG, "null server");
  ribo::Server& S = s->s;
  const uint32_t k = (uint32_t)(S.it_ms.size() < cap ? S.it_ms.size() : cap);
  for (uint32_t i = 0; i < k; i++) {
    if (ms) ms[i] = S.it_ms[i];
    if (steps) steps[i] = S.it_steps[i];
    if (active) active[i] = S.it_active[i];
  }
  S.it_ms.erase(S.it_ms.begin(), S.it_ms.begin() + k);
  S.it_steps.erase(S.it_steps.begin(), S.it_steps.begin() + k);
  S.it_active.erase(S.it_active.begin(), S.it_active.begin() + k);
  if (n) *n = k;
  return RIBO_OK;
}

}  // extern "C"
