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


__device__ __forceinline__ bool inside(const Dev& d, int x, int y) { return x >= 0 && y >= 0 && x < d.gw && y < d.gh; }
// Entries one class can hold: every cell of the class at most once.
__device__ __forceinline__ uint32_t class_seg(const Dev& d) {
  return (uint32_t)((d.gw + 2) / 3) * (uint32_t)((d.gh + 2) / 3);
}

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

// ---- decisions ----
// A CTA's grain counts with a halo of 2 (every read of a decision lies within
// 2 cells) and, for the cells within 1, the occupied cells of their 3 x 3
// block (cells outside the world count as empty).
constexpr int HX = BX + 4, HY = BY + 4;
constexpr int OX = BX + 2, OY = BY + 2;
struct DecideTile {
  uint32_t g[HY][HX];
  uint8_t box[OY][OX];
};
struct Tile {
  const DecideTile& s;
  int x0, y0;
  __device__ uint32_t g(int x, int y) const { return s.g[y - y0 + 2][x - x0 + 2]; }
  __device__ uint32_t box(int x, int y) const { return s.box[y - y0 + 1][x - x0 + 1]; }
};

// terrain.wgsl:137-159: may one grain pass from (xs, ys) holding n grains to
// (xd, yd) holding c without the sandpile undoing it?
__device__ bool compaction_stable(const Dev& d, const Tile& T, int xs, int ys, int xd, int yd, uint32_t n, uint32_t c) {
  bool ok = true;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int ox = k == 0 ? 1 : (k == 1 ? -1 : 0), oy = k == 2 ? 1 : (k == 3 ? -1 : 0);
    int qx = xd + ox, qy = yd + oy;
    if (inside(d, qx, qy)) {
      const uint32_t low = (qx == xs && qy == ys) ? n - 1u : T.g(qx, qy);
      if (c + 1u >= low + SANDPILE_DIFF) ok = false;
    }
    qx = xs + ox;
    qy = ys + oy;
    if (inside(d, qx, qy)) {
      const uint32_t high = (qx == xd && qy == yd) ? c + 1u : T.g(qx, qy);
      if (high >= n - 1u + SANDPILE_DIFF) ok = false;
    }
  }
  return ok;
}

// terrain.wgsl:161-318: the move of a cell holding 1..2 loose grains.  The
// bond count is the cell's 3 x 3 occupancy less itself, and a neighbour's
// nesting score (the occupied cells around it other than itself and this
// cell) its 3 x 3 occupancy less itself and this cell.
__device__ uint32_t loose_decide(const Dev& d, const ribo_sim_params* P, const Tile& T, int x, int y, uint32_t n,
                                 uint32_t phase) {
  const uint32_t idx = (uint32_t)y * (uint32_t)d.gw + (uint32_t)x;
  const uint32_t bonds = T.box(x, y) - 1u;
  uint32_t best_c = 0xFFFFu, comp_c = 0u;
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
      const uint32_t c = T.g(nx, ny);
      if (try_comp && c >= 1u && c < GAMMA_ROCK_FULL &&
          (c > comp_c || (c == comp_c && (rb_hash32(tie ^ (ni * 31u)) & 1u) == 1u)) &&
          compaction_stable(d, T, x, y, nx, ny, n, c)) {
        comp_c = c;
        comp = move_code(dx, dy);
      }
      if (c <= n) {
        const int score = (int)T.box(nx, ny) - (c >= 1u ? 1 : 0) - 1;
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
      if (!inside(d, qx, qy) || T.g(qx, qy) != 0u) continue;
      const float2 v = fluid_vel_at_cell(d, (uint32_t)qx, (uint32_t)qy);
      if (dot2(v, v) > dot2(vs, vs)) vs = v;
    }
  }
  const bool unsupported = y > 0 && T.g(x, y - 1) == 0u;
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
    if (inside(d, x + ddx, y + ddy) && T.g(x + ddx, y + ddy) <= n) return move_code(ddx, ddy);
    return 0u;
  }
  if (rw < p_sed + GAMMA_STRAY_WALK_P * mob) {
    if (best_score > (int)bonds) return best;
    if (bonds == 0u) {
      // terrain.wgsl:294-303: the walk directions in the reference's order
      const uint32_t k = (hw >> 8) % 8u;
      const int wdx = k == 0u || k == 4u || k == 6u ? 1 : (k == 2u || k == 3u ? 0 : -1);
      const int wdy = k == 2u || k == 4u || k == 5u ? 1 : (k == 0u || k == 1u ? 0 : -1);
      if (inside(d, x + wdx, y + wdy) && T.g(x + wdx, y + wdy) <= n) return move_code(wdx, wdy);
    }
  }
  return 0u;
}

// terrain.wgsl:320-372 (sandpile, n >= 3): a slide towards the lowest of the
// four neighbours when it lies SANDPILE_DIFF or more below.
__device__ uint32_t sandpile_decide(const Dev& d, const ribo_sim_params* P, const Tile& T, int x, int y, uint32_t n,
                                    uint32_t phase) {
  uint32_t best = 0u, best_c = n;
  if (x > 0 && T.g(x - 1, y) < best_c) { best_c = T.g(x - 1, y); best = move_code(-1, 0); }
  if (x + 1 < d.gw && T.g(x + 1, y) < best_c) { best_c = T.g(x + 1, y); best = move_code(1, 0); }
  if (y > 0 && T.g(x, y - 1) < best_c) { best_c = T.g(x, y - 1); best = move_code(0, -1); }
  if (y + 1 < d.gh && T.g(x, y + 1) < best_c) { best_c = T.g(x, y + 1); best = move_code(0, 1); }
  if (best == 0u || n - best_c < SANDPILE_DIFF) return 0u;
  const float p = GAMMA_RELAX_P * rb_max(rb_clamp(P->sediment_settle, 0.0f, 1.0f), rb_clamp(P->rock_crumble, 0.0f, 1.0f));
  const uint32_t idx = (uint32_t)y * (uint32_t)d.gw + (uint32_t)x;
  return rb_u2f(rb_pcg4d(idx, P->epoch, RB_S_SAND + phase, P->seed).x) < p ? best : 0u;
}

// The decision reads of relax_gamma_a / _b (terrain.wgsl:449-459), every
// cell from the counts as they stand.
__global__ void __launch_bounds__(BX * BY) k_relax_decide(const __grid_constant__ Dev d, const ribo_sim_params* P,
                                                          uint8_t* code, uint32_t phase) {
  __shared__ DecideTile S;
  const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY, tid = threadIdx.y * BX + threadIdx.x;
  for (int i = tid; i < HX * HY; i += BX * BY) {
    const int gx = x0 + i % HX - 2, gy = y0 + i / HX - 2;
    S.g[i / HX][i % HX] = inside(d, gx, gy) ? __ldg(d.gamma + (size_t)gy * d.gw + gx) : 0u;
  }
  __syncthreads();
  for (int i = tid; i < OX * OY; i += BX * BY) {
    const int ox = i % OX, oy = i / OX;
    uint32_t occ = 0u;
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++) occ += S.g[oy + a][ox + b] != 0u ? 1u : 0u;
    S.box[oy][ox] = (uint8_t)occ;
  }
  __syncthreads();
  const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
  if (x >= d.gw || y >= d.gh) return;
  const Tile T{S, x0, y0};
  const uint32_t n = T.g(x, y);
  uint32_t c = 0u;
  if (n >= SANDPILE_DIFF)
    c = sandpile_decide(d, P, T, x, y, n, phase);
  else if (n >= 1u)
    c = loose_decide(d, P, T, x, y, n, phase);
  code[(size_t)y * d.gw + x] = (uint8_t)c;
}

// Appends cell i (when `want`) to the list segment of its class.  A warp is
// one row of 32 cells (three classes).
__device__ __forceinline__ void append_by_class(const Dev& d, uint32_t* list, uint32_t* count, bool want, int x, int y,
                                                uint32_t i) {
  const int lane = threadIdx.x & 31;
  const uint32_t seg = class_seg(d);
#pragma unroll
  for (int r = 0; r < 3; r++) {
    const bool mine = want && x % 3 == r;
    const unsigned m = __ballot_sync(FULL, mine);
    if (m == 0u) continue;
    const int leader = __ffs(m) - 1, cls = r + 3 * (y % 3);
    uint32_t base = 0u;
    if (lane == leader) base = atomicAdd(count + cls, (uint32_t)__popc(m));
    base = __shfl_sync(FULL, base, leader);
    const uint32_t slot = base + (uint32_t)__popc(m & ((1u << lane) - 1u));
    if (mine && slot < seg) list[(size_t)cls * seg + slot] = i;
  }
}

// Every take and add of a relax pass (gamma_take_one + the atomicAdd of
// gamma_move_one, terrain.wgsl:36-46,79): the new count of each cell, and the
// cells that received a grain appended to the eviction lists.
__global__ void __launch_bounds__(BX * BY) k_relax_apply(const __grid_constant__ Dev d, uint32_t* gamma, const uint8_t* code,
                                                         uint8_t* arrivals, uint32_t* list, uint32_t* count) {
  const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
  const bool valid = x < d.gw && y < d.gh;
  uint32_t in = 0u, mask = 0u;
  size_t i = 0;
  if (valid) {
    i = (size_t)y * d.gw + x;
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const int jx = x + NB_DX[k], jy = y + NB_DY[k];
      if (inside(d, jx, jy) && code[(size_t)jy * d.gw + jx] == (uint8_t)(8 - k)) {
        in++;
        mask |= 1u << k;
      }
    }
    const uint32_t out = code[i] != 0 ? 1u : 0u;
    if (in != 0u || out != 0u) gamma[i] = gamma[i] - out + in;
    if (in != 0u) arrivals[i] = (uint8_t)mask;
  }
  append_by_class(d, list, count, valid && in != 0u, x, y, (uint32_t)i);
}

// ---- eviction (terrain.wgsl:48-101): plain loads and stores, the cells are
// this thread's alone while its class runs ----
__device__ __forceinline__ uint32_t total_at(const Dev& d, size_t c) {
  const uint4 v = *reinterpret_cast<const uint4*>(d.chem + c * 4);
  return cell_total4(v);
}
__device__ __forceinline__ uint32_t cap_at(const uint32_t* gamma, size_t c) { return capacity_of(gamma[c]); }

// terrain.wgsl:54-72 (evict_target), with the room the target has left
// (0xFFFFFFFF for the fallback, which no later round can change).
__device__ size_t evict_target(const Dev& d, const uint32_t* gamma, size_t src, size_t dst, uint32_t* room) {
  const uint32_t ts = total_at(d, src), cs = cap_at(gamma, src);
  if (ts < cs) {
    *room = cs - ts;
    return src;
  }
  const int x = (int)(dst % (size_t)d.gw), y = (int)(dst / (size_t)d.gw);
  const size_t NONE = ~(size_t)0;
  size_t not_rock = gamma[src] < GAMMA_SOLID ? src : NONE;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int qx = x + (k == 0 ? 1 : (k == 1 ? -1 : 0)), qy = y + (k == 2 ? 1 : (k == 3 ? -1 : 0));
    if (!inside(d, qx, qy)) continue;
    const size_t n = (size_t)qy * d.gw + qx;
    const uint32_t tn = total_at(d, n), cn = cap_at(gamma, n);
    if (tn < cn) {
      *room = cn - tn;
      return n;
    }
    if (not_rock == NONE && gamma[n] < GAMMA_SOLID) not_rock = n;
  }
  *room = 0xFFFFFFFFu;
  return not_rock == NONE ? src : not_rock;
}

// The eviction loop of gamma_move_one (terrain.wgsl:82-100) and of
// paint_terrain (:396-412, src == dst): each round moves one monomer, a
// channel's spent state before its activated state, channels in order, to
// evict_target.  While the target stays the same cell (it has room, and the
// cells before it in evict_target's order stay full) the rounds form a
// segment: m rounds move the first m monomers in that order at once.
__device__ void evict(const Dev& d, const uint32_t* gamma, size_t src, size_t dst) {
  const uint32_t cap = cap_at(gamma, dst);
  uint4* dp = reinterpret_cast<uint4*>(d.chem + dst * 4);
  uint4 dv = *dp;
  uint32_t total = cell_total4(dv), rounds = 64u;
  while (rounds != 0u && total > cap) {
    uint32_t room;
    const size_t to = evict_target(d, gamma, src, dst, &room);
    if (to == dst) break;
    const uint32_t moved = umin(umin(total - cap, rounds), room);
    uint32_t m = moved;
    uint32_t w[4] = {dv.x, dv.y, dv.z, dv.w};
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const uint32_t a = umin(w[c] >> 16, m);
      m -= a;
      const uint32_t b = umin(w[c] & CHEM_STATE_MASK, m);
      m -= b;
      const uint32_t one = (a << 16) + b;
      if (one != 0u) {
        w[c] -= one;
        d.chem[to * 4 + c] += one;
      }
    }
    dv = make_uint4(w[0], w[1], w[2], w[3]);
    *dp = dv;
    total -= moved;
    rounds -= moved;
  }
}

// The eviction loops of one relax pass (paint = 0: the arrivals at each
// listed destination by ascending source index, from the arrival mask the
// apply kernel left) or of the brush (paint = 1: each painted cell for
// itself), class by class.  A destination within its capacity when its turn
// comes ends every one of its loops at the first test, so it is skipped.
// One CTA; the lists are emptied at the end.
__global__ void __launch_bounds__(EVICT_THREADS) k_terrain_evict(const __grid_constant__ Dev d, const uint32_t* gamma,
                                                                 const uint8_t* arrivals, const uint32_t* list,
                                                                 uint32_t* count, int paint) {
  const uint32_t seg = class_seg(d);
  for (int cls = 0; cls < 9; cls++) {
    const uint32_t n = umin(count[cls], seg);
    for (uint32_t j = threadIdx.x; j < n; j += EVICT_THREADS) {
      const size_t dst = list[(size_t)cls * seg + j];
      const uint32_t mask = paint ? 1u : arrivals[dst];
      if (total_at(d, dst) <= cap_at(gamma, dst)) continue;
      if (paint) {
        evict(d, gamma, dst, dst);
        continue;
      }
      const int x = (int)(dst % (size_t)d.gw), y = (int)(dst / (size_t)d.gw);
      for (int k = 0; k < 8; k++)
        if ((mask >> k) & 1u) evict(d, gamma, (size_t)(y + NB_DY[k]) * d.gw + (x + NB_DX[k]), dst);
    }
    __syncthreads();
  }
  if (threadIdx.x < 9) count[threadIdx.x] = 0u;
}

// terrain.wgsl:425-446 (grain_fall), the columns x = 3 col + cls: one warp per
// column walks it bottom-up 32 rows at a time.  Whether a loose cell is
// supported follows from the cells below it (a hole clears support, rock
// restores it, loose grains pass it on), so two ballots find the unsupported
// loose cells of 32 rows.  A falling cell touches only the cells within one
// of its landing cell, so a faller waits for the previous one only when that
// lies fewer than 3 rows below: runs of such fallers move in waves, one lane
// per faller, in ascending row order within a run, as the reference's single
// thread moves them.
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
    const size_t idx = (size_t)y * d.gw + x;
    const uint32_t n = valid ? gamma[idx] : 0u;
    const unsigned hole = __ballot_sync(FULL, valid && n == 0u);
    const unsigned rock = __ballot_sync(FULL, valid && n >= GAMMA_SOLID);
    const unsigned setters = hole | rock;
    const unsigned below = setters & ((1u << lane) - 1u);
    const bool sup = below != 0u ? ((rock >> (31 - __clz(below))) & 1u) != 0u : supported;
    const unsigned movers = __ballot_sync(FULL, valid && n >= 1u && n < GAMMA_SOLID && !sup);
    if (setters != 0u) supported = ((rock >> (31 - __clz(setters))) & 1u) != 0u;
    if (movers == 0u) continue;
    int wave = 0, waves = 0, prev = -8, wprev = 0;
    for (unsigned mm = movers; mm != 0u; mm &= mm - 1u) {
      const int l = __ffs(mm) - 1;
      const int wl = l - prev < 3 ? wprev + 1 : 0;
      if (l == lane) wave = wl;
      waves = wl > waves ? wl : waves;
      prev = l;
      wprev = wl;
    }
    const bool mine = ((movers >> lane) & 1u) != 0u;
    for (int w = 0; w <= waves; w++) {
      if (mine && wave == w)
        for (uint32_t t = 0; t < n; t++) {
          gamma[idx] -= 1u;
          gamma[idx - d.gw] += 1u;
          evict(d, gamma, idx, idx - d.gw);
        }
      __syncwarp();
    }
  }
}

// paint_terrain (terrain.wgsl:390-395): the stores, and the painted cells
// appended to the eviction lists.
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
  append_by_class(d, list, count, hit, x, y, (uint32_t)i);
}

dim3 env_grid(const Dev& d) { return dim3((unsigned)((d.gw + BX - 1) / BX), (unsigned)((d.gh + BY - 1) / BY)); }

}  // namespace

size_t terrain_list_entries(int gw, int gh) { return 9 * (size_t)((gw + 2) / 3) * (size_t)((gh + 2) / 3); }

void launch_relax(const Dev& d, const ribo_sim_params* P, const TerrainBufs& t, uint32_t phase, cudaStream_t s) {
  const double C = (double)d.gw * d.gh;
  RB_LAUNCH(phase ? "relax_b" : "relax_a", 5.0 * C, s,
            k_relax_decide<<<env_grid(d), dim3(BX, BY), 0, s>>>(d, P, t.code, phase));
  RB_LAUNCH("relax_apply", 5.0 * C, s,
            k_relax_apply<<<env_grid(d), dim3(BX, BY), 0, s>>>(d, t.gamma, t.code, t.arrivals, t.list, t.count));
  RB_LAUNCH("terrain_evict", 4.0, s, k_terrain_evict<<<1, EVICT_THREADS, 0, s>>>(d, t.gamma, t.arrivals, t.list, t.count, 0));
}

void launch_grain_fall(const Dev& d, const ribo_sim_params* P, const TerrainBufs& t, cudaStream_t s) {
  for (int cls = 0; cls < 3; cls++) {
    const int cols = (d.gw - cls + 2) / 3;
    if (cols <= 0) continue;
    const unsigned blocks = (unsigned)((cols * 32 + FALL_THREADS - 1) / FALL_THREADS);
    RB_LAUNCH("grain_fall", 4.0 * cols * d.gh, s, k_grain_fall<<<blocks, FALL_THREADS, 0, s>>>(d, P, t.gamma, cls));
  }
}

void launch_paint(const Dev& d, const TerrainBufs& t, float cx, float cy, float radius, uint32_t grains, cudaStream_t s) {
  const uint32_t want = grains < 6u ? grains : 6u;
  RB_LAUNCH("paint_terrain", 4.0 * d.gw * d.gh, s,
            k_paint<<<env_grid(d), dim3(BX, BY), 0, s>>>(d, t.gamma, t.list, t.count, cx, cy, radius, want));
  RB_LAUNCH("terrain_evict", 4.0, s, k_terrain_evict<<<1, EVICT_THREADS, 0, s>>>(d, t.gamma, t.arrivals, t.list, t.count, 1));
}

}  // namespace ribo
