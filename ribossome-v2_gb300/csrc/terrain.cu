// Terrain grains of the world step (shaders/world/terrain.wgsl:36-460,
// dispatch src/world/mod.rs:1497-1504) and the terrain brush
// (World::encode_paint, src/world/mod.rs:1220-1241).
//
// The reference moves grains and evicts monomers with in-place atomics while
// every other cell's thread reads the live counts, so one GPU run of it has
// no single result.  These kernels execute one legal serialization of that
// program, exactly:
//  - a relax pass makes every cell's decision from the grain counts as they
//    stand (k_relax_decide: the reads of every thread before any write),
//    then applies every take and add of a grain (k_relax_apply: the new
//    count of a cell is its count - its own move + the grains it receives),
//    then runs the eviction loops of the destinations in nine classes
//    (x mod 3, y mod 3), the arrivals at one destination by ascending source
//    index (k_terrain_evict);
//  - grain_fall runs the columns in three classes (x mod 3), each column's
//    bottom-up loop whole (k_grain_fall: one warp per column);
//  - the brush stores every painted count, then runs the eviction loops of
//    the painted cells by class.
// Destinations of one class are at least 3 cells apart and an eviction loop
// reads and writes only cells within one cell of its destination (columns
// of one class: within one column), so the cells of a class run in parallel
// with the result of any serial order of them.
#include "ribo_dev.cuh"
#include "ribo_launch.h"

namespace ribo {

namespace {

constexpr int BX = PASS_BX, BY = PASS_BY;
constexpr int EVICT_THREADS = 1024;
constexpr int FALL_THREADS = 256;  // 8 columns per CTA, one warp each
constexpr unsigned FULL = 0xffffffffu;

// terrain.wgsl:6-34, transport.wgsl:41
constexpr uint32_t SANDPILE_DIFF = 3u;
constexpr float GAMMA_RELAX_P = (float)0.12;
constexpr float GAMMA_STRAY_WALK_P = (float)0.05;
constexpr float GAMMA_SEDIMENT_FACTOR = (float)0.5;
constexpr float GAMMA_SETTLE_SPEED = (float)0.5;
constexpr uint32_t GAMMA_ROCK_FULL = 6u;
constexpr float VENT_BLOW = (float)8.0;
constexpr float GAMMA_SHED_P = (float)0.03;
constexpr float GRAIN_ADV_CAP = (float)0.9;

// Move codes: 0 = the cell keeps its grain; 1 + k = its grain goes to the
// k-th of the 8 neighbours in ascending cell index (row-major, centre
// skipped).  The neighbour opposite k is 7 - k.
__constant__ const int NB_DX[8] = {-1, 0, 1, -1, 1, -1, 0, 1};
__constant__ const int NB_DY[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
__device__ __forceinline__ uint32_t move_code(int dx, int dy) {
  const int m = (dy + 1) * 3 + (dx + 1);
  return 1u + (uint32_t)(m < 4 ? m : m - 1);
}

__device__ __forceinline__ uint32_t gsnap(const Dev& d, int x, int y) { return __ldg(d.gamma + (size_t)y * d.gw + x); }
__device__ __forceinline__ bool inside(const Dev& d, int x, int y) { return x >= 0 && y >= 0 && x < d.gw && y < d.gh; }

// transport.wgsl:54-58
__device__ __forceinline__ float parcel_hop_p(const Dev& d, const ribo_sim_params* P, float2 v) {
  const float l1 = rb_abs(v.x) + rb_abs(v.y);
  return rb_clamp(l1 * d.sx * rb_max(P->dt, (float)1e-3), 0.0f, GRAIN_ADV_CAP);
}
// terrain.wgsl:24-28 (velocity_in = velocity_a, the previous step's final velocity)
__device__ __forceinline__ float2 fluid_vel_at_cell(const Dev& d, uint32_t cx, uint32_t cy) {
  const uint32_t fx = umin(cx * (uint32_t)d.fw / (uint32_t)d.gw, (uint32_t)d.fw - 1u);
  const uint32_t fy = umin(cy * (uint32_t)d.fh / (uint32_t)d.gh, (uint32_t)d.fh - 1u);
  return sanitize(d.va[(size_t)fy * d.fw + fx]);
}

// terrain.wgsl:137-159, on the snapshot counts: may one grain pass from
// (xs, ys) holding n grains to (xd, yd) holding c without the sandpile
// undoing it?
__device__ bool compaction_stable(const Dev& d, int xs, int ys, int xd, int yd, uint32_t n, uint32_t c) {
  bool ok = true;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int ox = k == 0 ? 1 : (k == 1 ? -1 : 0), oy = k == 2 ? 1 : (k == 3 ? -1 : 0);
    int qx = xd + ox, qy = yd + oy;
    if (inside(d, qx, qy)) {
      const uint32_t low = (qx == xs && qy == ys) ? n - 1u : gsnap(d, qx, qy);
      if (c + 1u >= low + SANDPILE_DIFF) ok = false;
    }
    qx = xs + ox;
    qy = ys + oy;
    if (inside(d, qx, qy)) {
      const uint32_t high = (qx == xd && qy == yd) ? c + 1u : gsnap(d, qx, qy);
      if (high >= n - 1u + SANDPILE_DIFF) ok = false;
    }
  }
  return ok;
}

// terrain.wgsl:161-318: the move of a cell holding 1..2 loose grains.
__device__ uint32_t loose_decide(const Dev& d, const ribo_sim_params* P, int x, int y, uint32_t n, uint32_t phase) {
  const uint32_t idx = (uint32_t)y * (uint32_t)d.gw + (uint32_t)x;
  uint32_t bonds = 0u, best_c = 0xFFFFu, comp_c = 0u;
  int best_score = -1, em_score = -1;
  uint32_t best = 0u, em = 0u, comp = 0u;  // move codes (0 = stay)
  bool em_found = false;
  const rb_u4 rr = rb_pcg4d(idx, P->epoch, RB_S_RELAX + phase, P->seed);
  uint32_t tie = rr.x;
  const float comp_roll = (float)(rb_hash32(rr.x ^ 0x5bd1e995u) >> 8) * (1.0f / 16777216.0f);
  const bool try_comp = comp_roll < P->sediment_compaction;
  for (int dy = -1; dy <= 1; dy++)
    for (int dx = -1; dx <= 1; dx++) {
      if (dx == 0 && dy == 0) continue;
      const int nx = x + dx, ny = y + dy;
      if (!inside(d, nx, ny)) continue;
      const uint32_t ni = (uint32_t)ny * (uint32_t)d.gw + (uint32_t)nx;
      const uint32_t c = gsnap(d, nx, ny);
      if (c >= 1u) bonds++;
      if (try_comp && c >= 1u && c < GAMMA_ROCK_FULL &&
          (c > comp_c || (c == comp_c && (rb_hash32(tie ^ (ni * 31u)) & 1u) == 1u)) &&
          compaction_stable(d, x, y, nx, ny, n, c)) {
        comp_c = c;
        comp = move_code(dx, dy);
      }
      if (c <= n) {
        int score = 0;
        for (int sy = -1; sy <= 1; sy++)
          for (int sx = -1; sx <= 1; sx++) {
            if (sx == 0 && sy == 0) continue;
            const int qx = nx + sx, qy = ny + sy;
            if (!inside(d, qx, qy) || (qx == x && qy == y)) continue;
            if (gsnap(d, qx, qy) >= 1u) score++;
          }
        tie = rb_hash32(tie ^ ni);
        if (score > best_score || (score == best_score && c < best_c) ||
            (score == best_score && c == best_c && (tie & 1u) == 1u)) {
          best_score = score;
          best_c = c;
          best = move_code(dx, dy);
        }
        if (c == 0u && (score > em_score || (score == em_score && (tie & 2u) == 2u))) {
          em_score = score;
          em = move_code(dx, dy);
          em_found = true;
        }
      }
    }
  // pow(0.25, bonds): 2^(-2 bonds), exact in f32 for bonds <= 8
  const float mob = __int_as_float((127 - 2 * (int)bonds) << 23);
  if (try_comp && bonds >= 3u && comp != 0u && comp_roll < P->sediment_compaction * (float)(bonds - 2u) / 6.0f)
    return comp;
  float2 vs = f2(0.0f, 0.0f);
  if (P->fluid_enabled != 0u) {
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int qx = x + (k == 0 ? 1 : (k == 1 ? -1 : 0)), qy = y + (k == 2 ? 1 : (k == 3 ? -1 : 0));
      if (!inside(d, qx, qy) || gsnap(d, qx, qy) != 0u) continue;
      const float2 v = fluid_vel_at_cell(d, (uint32_t)qx, (uint32_t)qy);
      if (dot2(v, v) > dot2(vs, vs)) vs = v;
    }
  }
  const bool unsupported = y > 0 && gsnap(d, x, y - 1) == 0u;
  float2 v_move = f2(0.0f, 0.0f);
  float p_sed;
  if (unsupported && bonds == 0u) {
    v_move = vs;
    p_sed = parcel_hop_p(d, P, v_move);
  } else {
    const float speed = len2(vs);
    const float crit = rb_max(P->sediment_threshold, 0.0f) * (1.0f + rb_max(P->sediment_cohesion, 0.0f) * (float)bonds);
    const float excess = rb_max(speed - crit, 0.0f);
    if (speed > (float)1e-6) v_move = mul2(vs, excess / rb_max(speed, (float)1e-6));
    p_sed = parcel_hop_p(d, P, v_move) * GAMMA_SEDIMENT_FACTOR * rb_max(P->sediment_transport, 0.0f);
  }
  const uint32_t hfx = umin((uint32_t)x * (uint32_t)d.fw / (uint32_t)d.gw, (uint32_t)d.fw - 1u);
  const uint32_t hfy = umin((uint32_t)y * (uint32_t)d.fh / (uint32_t)d.gh, (uint32_t)d.fh - 1u);
  const float2 vent = d.heat[(size_t)hfy * d.fw + hfx];
  const float blow = VENT_BLOW * rb_max(vent.x, vent.y);
  if (blow > 0.0f) {
    v_move = mul2(f2((rr.y & 1u) == 1u ? (float)0.6 : (float)-0.6, 1.0f), blow);
    p_sed = rb_max(p_sed, parcel_hop_p(d, P, v_move));
  }
  if (bonds >= 4u && p_sed <= 0.0f) return 0u;
  const uint32_t hw = rr.y;
  const float rw = rb_u2f(rr.z), rw2 = rb_u2f(rr.w);
  if (n >= 2u && em_found && rw2 < GAMMA_SHED_P * rb_clamp(P->sediment_settle, 0.0f, 1.0f)) return em;
  if (rw < p_sed) {
    int ddx = 0, ddy = 0;
    const float ax = rb_abs(v_move.x), ay = rb_abs(v_move.y);
    if (rb_u2f(hw) < ax / rb_max(ax + ay, (float)1e-6))
      ddx = v_move.x > 0.0f ? 1 : -1;
    else
      ddy = v_move.y > 0.0f ? 1 : -1;
    if (inside(d, x + ddx, y + ddy) && gsnap(d, x + ddx, y + ddy) <= n) return move_code(ddx, ddy);
    return 0u;
  }
  if (rw < p_sed + GAMMA_STRAY_WALK_P * mob) {
    if (best_score > (int)bonds) return best;
    if (bonds == 0u) {
      // terrain.wgsl:294-303: the walk directions in the reference's order
      const uint32_t k = (hw >> 8) % 8u;
      const int wdx = k == 0u || k == 4u || k == 6u ? 1 : (k == 2u || k == 3u ? 0 : -1);
      const int wdy = k == 2u || k == 4u || k == 5u ? 1 : (k == 0u || k == 1u ? 0 : -1);
      if (inside(d, x + wdx, y + wdy) && gsnap(d, x + wdx, y + wdy) <= n) return move_code(wdx, wdy);
    }
  }
  return 0u;
}

// terrain.wgsl:320-372 (sandpile, n >= 3): a slide towards the lowest of the
// four neighbours when it lies SANDPILE_DIFF or more below.
__device__ uint32_t sandpile_decide(const Dev& d, const ribo_sim_params* P, int x, int y, uint32_t n, uint32_t phase) {
  uint32_t best = 0u, best_c = n;
  if (x > 0) { const uint32_t c = gsnap(d, x - 1, y); if (c < best_c) { best_c = c; best = move_code(-1, 0); } }
  if (x + 1 < d.gw) { const uint32_t c = gsnap(d, x + 1, y); if (c < best_c) { best_c = c; best = move_code(1, 0); } }
  if (y > 0) { const uint32_t c = gsnap(d, x, y - 1); if (c < best_c) { best_c = c; best = move_code(0, -1); } }
  if (y + 1 < d.gh) { const uint32_t c = gsnap(d, x, y + 1); if (c < best_c) { best_c = c; best = move_code(0, 1); } }
  if (best == 0u || n - best_c < SANDPILE_DIFF) return 0u;
  const float p = GAMMA_RELAX_P * rb_max(rb_clamp(P->sediment_settle, 0.0f, 1.0f), rb_clamp(P->rock_crumble, 0.0f, 1.0f));
  const uint32_t idx = (uint32_t)y * (uint32_t)d.gw + (uint32_t)x;
  return rb_u2f(rb_pcg4d(idx, P->epoch, RB_S_SAND + phase, P->seed).x) < p ? best : 0u;
}

// The decision reads of relax_gamma_a / _b (terrain.wgsl:449-459), every
// cell from the counts as they stand.
__global__ void __launch_bounds__(BX * BY) k_relax_decide(const __grid_constant__ Dev d, const ribo_sim_params* P,
                                                          uint8_t* code, uint32_t phase) {
  const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
  if (x >= d.gw || y >= d.gh) return;
  const uint32_t n = gsnap(d, x, y);
  uint32_t c = 0u;
  if (n >= SANDPILE_DIFF)
    c = sandpile_decide(d, P, x, y, n, phase);
  else if (n >= 1u)
    c = loose_decide(d, P, x, y, n, phase);
  code[(size_t)y * d.gw + x] = (uint8_t)c;
}

// Every take and add of a relax pass (gamma_take_one + the atomicAdd of
// gamma_move_one, terrain.wgsl:36-46,79): the new count of each cell, and the
// cells that received a grain appended to the eviction list.
__global__ void __launch_bounds__(BX * BY) k_relax_apply(const __grid_constant__ Dev d, uint32_t* gamma, const uint8_t* code,
                                                         uint32_t* list, uint32_t* count) {
  const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
  const bool valid = x < d.gw && y < d.gh;
  uint32_t in = 0u;
  size_t i = 0;
  if (valid) {
    i = (size_t)y * d.gw + x;
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const int jx = x + NB_DX[k], jy = y + NB_DY[k];
      if (inside(d, jx, jy) && code[(size_t)jy * d.gw + jx] == (uint8_t)(8 - k)) in++;
    }
    const uint32_t out = code[i] != 0 ? 1u : 0u;
    if (in != 0u || out != 0u) gamma[i] = gamma[i] - out + in;
  }
  const bool want = valid && in != 0u;
  const unsigned m = __ballot_sync(FULL, want);
  if (m == 0u) return;
  const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
  uint32_t base = 0u;
  if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(m));
  base = __shfl_sync(FULL, base, leader);
  const uint32_t slot = base + (uint32_t)__popc(m & ((1u << lane) - 1u));
  if (want && slot < (uint32_t)d.gw * (uint32_t)d.gh) list[slot] = (uint32_t)i;  // one entry per cell at most
}

// ---- eviction (terrain.wgsl:48-101): plain loads and stores, the cells are
// this thread's alone while its class runs ----
__device__ __forceinline__ uint32_t total_at(const Dev& d, size_t c) {
  const uint4 v = *reinterpret_cast<const uint4*>(d.chem + c * 4);
  return cell_total4(v);
}
__device__ __forceinline__ uint32_t cap_at(const uint32_t* gamma, size_t c) { return capacity_of(gamma[c]); }

// terrain.wgsl:54-72
__device__ size_t evict_target(const Dev& d, const uint32_t* gamma, size_t src, size_t dst) {
  if (total_at(d, src) < cap_at(gamma, src)) return src;
  const int x = (int)(dst % (size_t)d.gw), y = (int)(dst / (size_t)d.gw);
  const size_t NONE = ~(size_t)0;
  size_t not_rock = gamma[src] < GAMMA_SOLID ? src : NONE;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int qx = x + (k == 0 ? 1 : (k == 1 ? -1 : 0)), qy = y + (k == 2 ? 1 : (k == 3 ? -1 : 0));
    if (!inside(d, qx, qy)) continue;
    const size_t n = (size_t)qy * d.gw + qx;
    if (total_at(d, n) < cap_at(gamma, n)) return n;
    if (not_rock == NONE && gamma[n] < GAMMA_SOLID) not_rock = n;
  }
  return not_rock == NONE ? src : not_rock;
}

// The eviction loop of gamma_move_one (terrain.wgsl:82-100) and of
// paint_terrain (:396-412, src == dst): one monomer per round, a channel's
// spent state before its activated state, channels in order.
__device__ void evict(const Dev& d, const uint32_t* gamma, size_t src, size_t dst) {
  const uint32_t cap = cap_at(gamma, dst);
  for (int guard = 0; guard < 64; guard++) {
    if (total_at(d, dst) <= cap) break;
    const size_t to = evict_target(d, gamma, src, dst);
    if (to == dst) break;
    bool moved = false;
    for (int c = 0; c < 4 && !moved; c++) {
      uint32_t* slot = d.chem + dst * 4 + c;
      const uint32_t v = *slot;
      uint32_t one = 0u;
      if ((v >> 16) != 0u)
        one = CHEM_SPENT_ONE;
      else if ((v & CHEM_STATE_MASK) != 0u)
        one = 1u;
      if (one != 0u) {
        *slot = v - one;
        d.chem[to * 4 + c] += one;
        moved = true;
      }
    }
    if (!moved) break;
  }
}

// The eviction loops of one relax pass (paint = 0: the arrivals at each
// listed destination by ascending source index) or of the brush (paint = 1:
// each painted cell for itself), class by class.  One CTA; the list is
// emptied at the end.
__global__ void __launch_bounds__(EVICT_THREADS) k_terrain_evict(const __grid_constant__ Dev d, const uint32_t* gamma,
                                                                 const uint8_t* code, const uint32_t* list,
                                                                 uint32_t* count, int paint) {
  const uint32_t n = umin(*count, (uint32_t)d.gw * (uint32_t)d.gh);
  for (int cls = 0; cls < 9; cls++) {
    for (uint32_t j = threadIdx.x; j < n; j += EVICT_THREADS) {
      const size_t dst = list[j];
      const int x = (int)(dst % (size_t)d.gw), y = (int)(dst / (size_t)d.gw);
      if (x % 3 + 3 * (y % 3) != cls) continue;
      if (paint) {
        evict(d, gamma, dst, dst);
        continue;
      }
      for (int k = 0; k < 8; k++) {
        const int sx = x + NB_DX[k], sy = y + NB_DY[k];
        if (!inside(d, sx, sy)) continue;
        const size_t src = (size_t)sy * d.gw + sx;
        if (code[src] == (uint8_t)(8 - k)) evict(d, gamma, src, dst);
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *count = 0u;
}

// terrain.wgsl:425-446 (grain_fall), the columns x = 3 col + cls: one warp per
// column walks it bottom-up 32 rows at a time.  Whether a loose cell is
// supported follows from the cells below it (a hole clears support, rock
// restores it, loose grains pass it on), so the warp finds the unsupported
// loose cells of 32 rows with two ballots; lane 0 then moves them down in
// ascending row order, as the reference's single thread does.
__global__ void __launch_bounds__(FALL_THREADS) k_grain_fall(const __grid_constant__ Dev d, const ribo_sim_params* P,
                                                             uint32_t* gamma, int cls) {
  const float w_s = GAMMA_SETTLE_SPEED * rb_max(P->sediment_settle, 0.0f);
  const float rate = parcel_hop_p(d, P, f2(0.0f, w_s));
  if (rate <= 0.0f) return;
  const uint32_t rf = rb_f2u(rate * 65536.0f);
  if (((P->epoch * rf) >> 16) == (((P->epoch + 1u) * rf) >> 16)) return;
  const int lane = threadIdx.x & 31;
  const int x = 3 * (int)((blockIdx.x * FALL_THREADS + threadIdx.x) >> 5) + cls;
  if (x >= d.gw) return;  // whole warps
  bool supported = true;  // the bottom of the world supports
  for (int y0 = 0; y0 < d.gh; y0 += 32) {
    const int y = y0 + lane;
    const bool valid = y < d.gh;
    const uint32_t n = valid ? gamma[(size_t)y * d.gw + x] : 0u;
    const unsigned hole = __ballot_sync(FULL, valid && n == 0u);
    const unsigned rock = __ballot_sync(FULL, valid && n >= GAMMA_SOLID);
    const unsigned setters = hole | rock;
    const unsigned below = setters & ((1u << lane) - 1u);
    const bool sup = below != 0u ? ((rock >> (31 - __clz(below))) & 1u) != 0u : supported;
    unsigned movers = __ballot_sync(FULL, valid && n >= 1u && n < GAMMA_SOLID && !sup);
    if (setters != 0u) supported = ((rock >> (31 - __clz(setters))) & 1u) != 0u;
    while (movers != 0u) {
      const int l = __ffs(movers) - 1;
      movers &= movers - 1u;
      const uint32_t k = __shfl_sync(FULL, n, l);
      if (lane == 0) {
        const size_t idx = (size_t)(y0 + l) * d.gw + x;
        for (uint32_t t = 0; t < k; t++) {
          gamma[idx] -= 1u;
          gamma[idx - d.gw] += 1u;
          evict(d, gamma, idx, idx - d.gw);
        }
      }
      __syncwarp();
    }
  }
}

// paint_terrain (terrain.wgsl:390-395): the stores, and the painted cells
// appended to the eviction list.
__global__ void __launch_bounds__(BX * BY) k_paint(const __grid_constant__ Dev d, uint32_t* gamma, uint32_t* list,
                                                   uint32_t* count, float cx, float cy, float radius, uint32_t want) {
  const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
  bool hit = false;
  size_t i = 0;
  if (x < d.gw && y < d.gh) {
    const float ex = (float)x + 0.5f - cx, ey = (float)y + 0.5f - cy;
    hit = !(ex * ex + ey * ey > radius * radius);
    i = (size_t)y * d.gw + x;
    if (hit) gamma[i] = want;
  }
  const unsigned m = __ballot_sync(FULL, hit);
  if (m == 0u) return;
  const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
  uint32_t base = 0u;
  if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(m));
  base = __shfl_sync(FULL, base, leader);
  const uint32_t slot = base + (uint32_t)__popc(m & ((1u << lane) - 1u));
  if (hit && slot < (uint32_t)d.gw * (uint32_t)d.gh) list[slot] = (uint32_t)i;
}

dim3 env_grid(const Dev& d) { return dim3((unsigned)((d.gw + BX - 1) / BX), (unsigned)((d.gh + BY - 1) / BY)); }

}  // namespace

void launch_relax(const Dev& d, const ribo_sim_params* P, const TerrainBufs& t, uint32_t phase, cudaStream_t s) {
  const double C = (double)d.gw * d.gh;
  RB_LAUNCH(phase ? "relax_b" : "relax_a", 5.0 * C, s,
            k_relax_decide<<<env_grid(d), dim3(BX, BY), 0, s>>>(d, P, t.code, phase));
  RB_LAUNCH("relax_apply", 5.0 * C, s, k_relax_apply<<<env_grid(d), dim3(BX, BY), 0, s>>>(d, t.gamma, t.code, t.list, t.count));
  RB_LAUNCH("terrain_evict", 4.0, s, k_terrain_evict<<<1, EVICT_THREADS, 0, s>>>(d, t.gamma, t.code, t.list, t.count, 0));
}

void launch_grain_fall(const Dev& d, const ribo_sim_params* P, const TerrainBufs& t, cudaStream_t s) {
  for (int cls = 0; cls < 3; cls++) {
    const int cols = (d.gw - cls + 2) / 3;
    const unsigned blocks = (unsigned)((cols * 32 + FALL_THREADS - 1) / FALL_THREADS);
    if (cols <= 0) continue;
    RB_LAUNCH("grain_fall", 4.0 * cols * d.gh, s, k_grain_fall<<<blocks, FALL_THREADS, 0, s>>>(d, P, t.gamma, cls));
  }
}

void launch_paint(const Dev& d, const TerrainBufs& t, float cx, float cy, float radius, uint32_t grains, cudaStream_t s) {
  const uint32_t want = grains < 6u ? grains : 6u;
  RB_LAUNCH("paint_terrain", 4.0 * d.gw * d.gh, s,
            k_paint<<<env_grid(d), dim3(BX, BY), 0, s>>>(d, t.gamma, t.list, t.count, cx, cy, radius, want));
  RB_LAUNCH("terrain_evict", 4.0, s, k_terrain_evict<<<1, EVICT_THREADS, 0, s>>>(d, t.gamma, t.code, t.list, t.count, 1));
}

}  // namespace ribo
