// Monomer transport and reactions, ledger and terrain slope
// (shaders/world/transport.wgsl, ledger.wgsl, terrain.wgsl:104-133).
//
// Transport is a two-phase scatter: every cell reads the state before the
// step (chem) and adds each monomer to exactly one destination word of
// chem_next with integer atomics.  Integer adds commute, so the result is
// independent of thread order and bit-identical to the oracle.
#include "ribo_dev.cuh"
#include "ribo_launch.h"

namespace ribo {

namespace {

constexpr int BX = PASS_BX, BY = PASS_BY;

// terrain.wgsl:104-133 (compute_gamma_slope)
__global__ void k_slope(const __grid_constant__ Dev d, float upc) {
  int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
  if (x >= d.gw || y >= d.gh) return;
  auto h = [&](int ix, int iy) {
    int cx = iclamp(ix, 0, d.gw - 1), cy = iclamp(iy, 0, d.gh - 1);
    return (float)__ldg(d.gamma + (size_t)cy * d.gw + cx) * GAMMA_QUANTUM;
  };
  float l = h(x - 1, y), r = h(x + 1, y), b = h(x, y - 1), t = h(x, y + 1);
  float bl = h(x - 1, y - 1), br = h(x + 1, y - 1), tl = h(x - 1, y + 1), tr = h(x + 1, y + 1);
  const float k = (float)(1.0 / (4.0 * 1.41421356237));
  float dx = (r - l) * 0.5f + (tr + br - tl - bl) * k;
  float dy = (t - b) * 0.5f + (tl + tr - bl - br) * k;
  d.slope[(size_t)y * d.gw + x] = f2(dx / upc, dy / upc);
}

// transport.wgsl:419-438 (thermal activation, in place; one thread per cell)
template <class S>
__global__ void k_thermal(const __grid_constant__ S s) {
  RB_WORLD(s);
  // FLUID_ROWS cells of a column per thread (rows BY apart), their
  // temperatures loaded together
  const uint32_t x = cta.bx * BX + threadIdx.x, y0 = cta.by * (BY * FLUID_ROWS) + threadIdx.y;
  if (x >= (uint32_t)d.gw) return;
  const uint32_t fx = umin((x * (uint32_t)d.fw) / (uint32_t)d.gw, (uint32_t)d.fw - 1u);
  float t_loc[FLUID_ROWS];
#pragma unroll
  for (int r = 0; r < FLUID_ROWS; r++) {
    const uint32_t y = umin(y0 + r * BY, (uint32_t)d.gh - 1u);
    const uint32_t fy = umin((y * (uint32_t)d.fh) / (uint32_t)d.gh, (uint32_t)d.fh - 1u);
    t_loc[r] = __ldg(d.temp_in + (size_t)fy * d.fw + fx);
  }
#pragma unroll
  for (int r = 0; r < FLUID_ROWS; r++) {
    const uint32_t y = y0 + r * BY;
    if (y >= (uint32_t)d.gh) break;
    if (t_loc[r] <= TEMP_ACT_THRESHOLD) continue;
    float p_act = rb_clamp(FUMAROLE_ACT_P * rb_max(P->thermal_activation, 0.0f) * (t_loc[r] - TEMP_ACT_THRESHOLD) / TEMP_ACT_THRESHOLD,
                           0.0f, (float)0.9);
    size_t idx = (size_t)y * d.gw + x;
    uint4 c = reinterpret_cast<uint4*>(d.chem)[idx];
    uint32_t w[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
    for (uint32_t ch = 0; ch < 4; ch++) {
      uint32_t slot = (uint32_t)(idx * 4 + ch);
      if ((w[ch] >> 16) > 0u && rb_u2f(rb_pcg4d(slot, P->epoch, RB_S_THERMAL, P->seed).x) < p_act) w[ch] += 0xFFFF0001u;
    }
    reinterpret_cast<uint4*>(d.chem)[idx] = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

// agg_count + agg_neighbours (transport.wgsl:61-87) in one pass.  The
// scatter reads a cell's neighbour count plus its own activated count
// (transport.wgsl:196-201); integer adds commute, so each cell stores that sum
// directly: the 3 x 3 box of activated counts.  A CTA counts the activated
// monomers of its 32 x 8 tile and one-cell ring into shared memory (cells off
// the grid count 0, as the reference skips them) and sums the boxes there.
template <class S>
__global__ void k_agg(const __grid_constant__ S s) {
  RB_WORLD(s);
  constexpr int W = BX + 2, N = W * (BY + 2), NT = BX * BY;
  static_assert(N <= 2 * NT, "two cells of the tile and ring per thread");
  __shared__ uint32_t act[N];
  const int x0 = (int)cta.bx * BX - 1, y0 = (int)cta.by * BY - 1, tid = threadIdx.y * BX + threadIdx.x;
  uint4 c[2];
  bool in[2];
#pragma unroll
  for (int u = 0; u < 2; u++) {  // both loads before either store
    const int i = tid + u * NT, gx = x0 + i % W, gy = y0 + i / W;
    in[u] = i < N && gx >= 0 && gy >= 0 && gx < d.gw && gy < d.gh;
    c[u] = in[u] ? load_cell(d.chem, (size_t)gy * d.gw + gx) : make_uint4(0u, 0u, 0u, 0u);
  }
#pragma unroll
  for (int u = 0; u < 2; u++) {
    const int i = tid + u * NT;
    if (i < N)
      act[i] = (c[u].x & CHEM_STATE_MASK) + (c[u].y & CHEM_STATE_MASK) + (c[u].z & CHEM_STATE_MASK) +
               (c[u].w & CHEM_STATE_MASK);
  }
  __syncthreads();
  const int x = x0 + 1 + (int)threadIdx.x, y = y0 + 1 + (int)threadIdx.y;
  if (x >= d.gw || y >= d.gh) return;
  const int b = ((int)threadIdx.y + 1) * W + (int)threadIdx.x + 1;
  d.agg_nb[(size_t)y * d.gw + x] = act[b - W - 1] + act[b - W] + act[b - W + 1] + act[b - 1] + act[b] + act[b + 1] +
                                   act[b + W - 1] + act[b + W] + act[b + W + 1];
}

// transport.wgsl:260-273 (fluid_velocity_at_world, reading velocity_a)
__device__ __forceinline__ float2 fluid_velocity_at_world(const Dev& d, float2 pw) {
  float gxf = (float)d.fw, gyf = (float)d.fh;
  float gx = rb_clamp(pw.x / d.sim_w * gxf, 0.5f, gxf - 0.5f) - 0.5f;
  float gy = rb_clamp(pw.y / d.sim_h * gyf, 0.5f, gyf - 0.5f) - 0.5f;
  uint32_t x0 = rb_f2u(rb_floor(gx)), y0 = rb_f2u(rb_floor(gy));
  uint32_t x1 = umin(x0 + 1u, (uint32_t)d.fw - 1u), y1 = umin(y0 + 1u, (uint32_t)d.fh - 1u);
  float tx = rb_fract(gx), ty = rb_fract(gy);
  const float2* v = d.va;
  float2 v0 = mix2(sanitize(v[(size_t)y0 * d.fw + x0]), sanitize(v[(size_t)y0 * d.fw + x1]), tx);
  float2 v1 = mix2(sanitize(v[(size_t)y1 * d.fw + x0]), sanitize(v[(size_t)y1 * d.fw + x1]), tx);
  return mix2(v0, v1, ty);
}

// transport.wgsl:95-117
__device__ __forceinline__ float2 lattice_rand(uint32_t ix, uint32_t iy, const ribo_sim_params* P) {
  rb_u4 r = rb_pcg4d((ix * 73856093u) ^ (iy * 19349663u), P->epoch, RB_S_MOVE + MAX_MOVERS_PER_CH + 1u, P->seed);
  return f2(rb_u2f(r.x), rb_u2f(r.y));
}
__device__ __forceinline__ float2 smooth_start(uint32_t x0, uint32_t y0, const ribo_sim_params* P) {
  rb_u4 j = rb_pcg4d(0x85EBCA6Bu, P->epoch, RB_S_MOVE + MAX_MOVERS_PER_CH + 2u, P->seed);
  uint32_t x = x0 + rb_f2u(rb_u2f(j.x) * (float)SMOOTH_CELL);
  uint32_t y = y0 + rb_f2u(rb_u2f(j.y) * (float)SMOOTH_CELL);
  uint32_t gx = x / SMOOTH_CELL, gy = y / SMOOTH_CELL;
  float tx = rb_smoothstep01(((float)(x % SMOOTH_CELL) + 0.5f) / (float)SMOOTH_CELL);
  float ty = rb_smoothstep01(((float)(y % SMOOTH_CELL) + 0.5f) / (float)SMOOTH_CELL);
  float2 n = mix2(mix2(lattice_rand(gx, gy, P), lattice_rand(gx + 1u, gy, P), tx),
                  mix2(lattice_rand(gx, gy + 1u, P), lattice_rand(gx + 1u, gy + 1u, P), tx), ty);
  rb_u4 gr = rb_pcg4d(0x9E3779B9u, P->epoch, RB_S_MOVE + MAX_MOVERS_PER_CH, P->seed);
  float vx = rb_fract(n.x + rb_u2f(gr.x)), vy = rb_fract(n.y + rb_u2f(gr.y));
  return f2(1.0f - rb_abs(2.0f * vx - 1.0f), 1.0f - rb_abs(2.0f * vy - 1.0f));
}

// transport.wgsl:119-406
template <class S>
__global__ void __launch_bounds__(256) k_scatter(const __grid_constant__ S s) {
  RB_WORLD(s);
  uint32_t x = cta.bx * BX + threadIdx.x, y = cta.by * BY + threadIdx.y;
  const uint32_t G = d.gw, GH = d.gh;
  if (x >= G || y >= GH) return;
  size_t idx = (size_t)y * G + x;
  uint4 cw = load_cell(d.chem, idx);
  uint32_t src_total = cell_total4(cw);
  if (src_total == 0u) return;
  uint32_t g_src = __ldg(d.gamma + idx);
  float2 v = f2(0.0f, 0.0f);
  if (P->fluid_enabled != 0u && g_src < GAMMA_SOLID) {
    float2 c = mul2(f2((float)x + 0.5f, (float)y + 0.5f), d.cell_w);
    float2 v0 = fluid_velocity_at_world(d, c);
    float h = rb_max(P->dt, 0.0f);
    float2 c2 = f2(c.x + v0.x * d.wpf_x * h * 0.5f, c.y + v0.y * d.wpf_y * h * 0.5f);
    v = fluid_velocity_at_world(d, c2);
  }
  if (v.x != 0.0f || v.y != 0.0f) {
    bool rock_r = x + 1u < G && __ldg(d.gamma + idx + 1) >= GAMMA_SOLID;
    bool rock_l = x > 0u && __ldg(d.gamma + idx - 1) >= GAMMA_SOLID;
    bool rock_u = y + 1u < GH && __ldg(d.gamma + idx + G) >= GAMMA_SOLID;
    bool rock_d = y > 0u && __ldg(d.gamma + idx - G) >= GAMMA_SOLID;
    if ((v.x > 0.0f && rock_r) || (v.x < 0.0f && rock_l)) v.x = 0.0f;
    else if ((v.x > 0.0f && rock_l) || (v.x < 0.0f && rock_r)) v.x *= 0.5f;
    if ((v.y > 0.0f && rock_u) || (v.y < 0.0f && rock_d)) v.y = 0.0f;
    else if ((v.y > 0.0f && rock_d) || (v.y < 0.0f && rock_u)) v.y *= 0.5f;
  }
  const float tn = (float)(P->transport_every > 1u ? P->transport_every : 1u);
  const float dtp = rb_max(P->dt, 0.0f);
  float2 disp = f2(v.x * d.sx * dtp * tn, v.y * d.sy * dtp * tn);
  float agitation = rb_clamp(len2(v) / DIFF_AGITATION_SPEED, 0.0f, 1.0f);
  float p_diff = rb_clamp(DIFF_HOP_P * rb_mix(DIFF_HOP_FLOOR, 1.0f, agitation) * rb_max(P->diffusion, 0.0f) * tn, 0.0f, 0.5f);
  if (g_src > 0u) p_diff = rb_min(DIFF_HOP_P * BURIED_DIFF_FACTOR / (1.0f + GAMMA_POROSITY_K * (float)g_src) * tn, 0.5f);
  const uint32_t cap_self = capacity_of(g_src);
  if (src_total > cap_self) p_diff = rb_min(CHEM_SQUEEZE_P * tn, 0.5f);
  float p_settle = 0.0f;
  if (g_src == 0u) p_settle = rb_min(MONOMER_SETTLE_P * rb_max(P->settle, 0.0f) * tn, 0.5f);
  const int base_x = rb_floor_i(disp.x) - 1, base_y = rb_floor_i(disp.y) - 1;

  float press[4] = {1.0f, 1.0f, 1.0f, 1.0f};
  float max_drop = 0.0f;
  if (P->monomer_pressure > 0.0f) {
    float f_self = (float)src_total / (float)(cap_self > 1u ? cap_self : 1u);
    long nb[4] = {1, -1, (long)G, -(long)G};
    bool inside[4] = {x + 1u < G, x > 0u, y + 1u < GH, y > 0u};
#pragma unroll
    for (int k = 0; k < 4; k++) {
      if (!inside[k]) continue;
      size_t n = (size_t)((long)idx + nb[k]);
      uint32_t cap_n = capacity_of(__ldg(d.gamma + n));
      if (cap_n == 0u) continue;
      float f_n = (float)cell_total4(load_cell(d.chem, n)) / (float)cap_n;
      press[k] = rb_max((float)0.05, 1.0f + P->monomer_pressure * (f_self - f_n));
      max_drop = rb_max(max_drop, f_self - f_n);
    }
  }
  p_diff = rb_clamp(p_diff + PRESSURE_HOP_P * P->monomer_pressure * max_drop * tn, 0.0f, 0.5f);
  // uv_light_at_cell (light.wgsl:46-50)
  const float light_t = d.light[(size_t)(umin(y, GH - 1u) / LIGHT_DIV) * d.lw + umin(x, G - 1u) / LIGHT_DIV];

  float p_bound = 0.0f;
  float accept[4] = {1.0f, 1.0f, 1.0f, 1.0f};
  float accept_spent[4] = {1.0f, 1.0f, 1.0f, 1.0f};
  if (P->aggregation > 0.0f && src_total <= cap_self) {
    float e[5];
    e[0] = (float)d.agg_nb[idx];  // neighbours + own activated counts
    e[1] = x + 1u < G ? (float)d.agg_nb[idx + 1] : 0.0f;
    e[2] = x > 0u ? (float)d.agg_nb[idx - 1] : 0.0f;
    e[3] = y + 1u < GH ? (float)d.agg_nb[idx + G] : 0.0f;
    e[4] = y > 0u ? (float)d.agg_nb[idx - G] : 0.0f;
    uint32_t fx = umin((x * (uint32_t)d.fw) / G, (uint32_t)d.fw - 1u);
    uint32_t fy = umin((y * (uint32_t)d.fh) / GH, (uint32_t)d.fh - 1u);
    float t_rel = 1.0f + rb_max(d.temp_in[(size_t)fy * d.fw + fx], 0.0f) / TEMP_ACT_THRESHOLD;
    float room = rb_clamp(5.0f * (1.0f - (float)src_total / (float)(cap_self > 1u ? cap_self : 1u)), 0.0f, 1.0f);
    float k_e = P->aggregation * room / t_rel;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      float drop = e[0] - e[k + 1];
      if (drop > 0.0f) accept[k] = rb_exp(-k_e * drop);
      float rise = e[k + 1] - e[0];
      if (rise > 0.0f) accept_spent[k] = rb_exp(-k_e * rise);
    }
    p_bound = 1.0f - rb_exp(-k_e * rb_min(rb_max(e[0] - 1.0f, 0.0f), 48.0f));
  }

  const float2 bound_start = p_bound > 0.0f ? smooth_start(x, y, P) : f2(0.0f, 0.0f);
  const bool disperse = g_src > 0u && (disp.x != 0.0f || disp.y != 0.0f);
  const float disp_len = disperse ? len2(disp) : 0.0f;
  uint32_t words[4] = {cw.x, cw.y, cw.z, cw.w};
  for (uint32_t ch = 0; ch < 4; ch++) {
    const uint32_t slot = (uint32_t)(idx * 4 + ch);
    const uint32_t v_ch = words[ch];
    uint32_t act_n = v_ch & CHEM_STATE_MASK;
    uint32_t spent_n = v_ch >> 16;
    if (act_n + spent_n == 0u) continue;
    if (spent_n > 0u) {
      float sens = 1.0f + CHEM_SENSITIZE * (float)umin(act_n, 8u);
      float exp_act = (float)umin(spent_n, 8u) * tn *
                      (LIGHT_ACT_P * rb_max(P->uv_strength, 0.0f) * rb_max(P->direct_photoactivation, 0.0f) * light_t * sens +
                       rb_max(P->reactivation_rate, 0.0f));
      uint32_t na = rb_f2u(rb_floor(exp_act));
      float frac = exp_act - (float)na;
      if (frac > 0.0f && rb_u2f(rb_pcg4d(slot, P->epoch, RB_S_PHOTO, P->seed).x) < frac) na += 1u;
      na = umin(na, umin(spent_n, 8u));
      act_n += na;
      spent_n -= na;
    }
    if (act_n > 0u) {
      float shield = 1.0f / (1.0f + CHEM_SHIELD * (float)(umin(act_n, 8u) - 1u));
      float exp_dec = (float)umin(act_n, 8u) * rb_max(P->activation_decay, 0.0f) * shield * tn;
      if (exp_dec > 0.0f && rb_u2f(rb_pcg4d(slot, P->epoch, RB_S_DECAY, P->seed).x) < exp_dec) {
        act_n -= 1u;
        spent_n += 1u;
      }
    }
    float coh[4] = {1.0f, 1.0f, 1.0f, 1.0f};
    if (act_n > 0u && P->cohesion > 0.0f) {
      if (x + 1u < G) coh[0] = 1.0f + P->cohesion * (float)umin(__ldg(d.chem + (idx + 1) * 4 + ch) & CHEM_STATE_MASK, 8u);
      if (x > 0u) coh[1] = 1.0f + P->cohesion * (float)umin(__ldg(d.chem + (idx - 1) * 4 + ch) & CHEM_STATE_MASK, 8u);
      if (y + 1u < GH) coh[2] = 1.0f + P->cohesion * (float)umin(__ldg(d.chem + (idx + G) * 4 + ch) & CHEM_STATE_MASK, 8u);
      if (y > 0u) coh[3] = 1.0f + P->cohesion * (float)umin(__ldg(d.chem + (idx - G) * 4 + ch) & CHEM_STATE_MASK, 8u);
    }
    uint32_t bins[16];
#pragma unroll
    for (int b = 0; b < 16; b++) bins[b] = 0u;
    uint32_t stay = 0;
    const uint32_t n = act_n + spent_n;
    const uint32_t movers = umin(n, MAX_MOVERS_PER_CH);
    const uint32_t act_stay = act_n - umin(act_n, movers);
    stay += act_stay + (n - movers - act_stay) * CHEM_SPENT_ONE;
    for (uint32_t k = 0; k < movers; k++) {
      const bool is_act = k < act_n;
      const uint32_t unit = is_act ? 1u : CHEM_SPENT_ONE;
      rb_u4 ru = rb_pcg4d(slot, P->epoch, RB_S_MOVE + k, P->seed);
      float rfx = rb_u2f(ru.x), rfy = rb_u2f(ru.y), rfz = rb_u2f(ru.z), rfw = rb_u2f(ru.w);
      bool bound = is_act && p_bound > 0.0f && rb_fract(rfz * (float)7.31 + rfw * (float)3.17) < p_bound;
      float px = (bound ? bound_start.x : rfx) + disp.x;
      float py = (bound ? bound_start.y : rfy) + disp.y;
      if (disperse) {
        rb_u4 rj = rb_pcg4d(slot, P->epoch, RB_S_DISPERSE + k, P->seed);
        float jx = (rb_u2f(rj.x) * 2.0f - 1.0f) * disp_len * RUBBLE_DISPERSION;
        float jy = (rb_u2f(rj.y) * 2.0f - 1.0f) * disp_len * RUBBLE_DISPERSION;
        px += rb_clamp(jx, (float)-0.9, (float)0.9);
        py += rb_clamp(jy, (float)-0.9, (float)0.9);
      }
      if (rfz < p_diff) {
        float w0 = press[0], w1 = press[1], w2 = press[2], w3 = press[3];
        if (is_act) {
          w0 *= coh[0];
          w1 *= coh[1];
          w2 *= coh[2];
          w3 *= coh[3];
        }
        float u = rfw * (w0 + w1 + w2 + w3);
        uint32_t dd;
        if (u < w0) dd = 0u;
        else if ((u -= w0) < w1) dd = 1u;
        else if ((u -= w1) < w2) dd = 2u;
        else dd = 3u;
        float acc_d = is_act ? accept[dd] : accept_spent[dd];
        bool stay_put = rb_fract(rfw * (float)13.73 + rfx * (float)5.31) >= acc_d;
        if (!stay_put) {
          if (dd == 0u) px += 1.0f;
          else if (dd == 1u) px -= 1.0f;
          else if (dd == 2u) py += 1.0f;
          else py -= 1.0f;
        }
      } else if (rfz < p_diff + p_settle) {
        py -= 1.0f;
      }
      int offx = rb_floor_i(px) - base_x, offy = rb_floor_i(py) - base_y;
      uint32_t bi = (uint32_t)iclamp(offy, 0, 3) * 4u + (uint32_t)iclamp(offx, 0, 3);
      bins[bi] += unit;
    }
#pragma unroll
    for (uint32_t b = 0; b < 16; b++) {
      uint32_t cnt = bins[b];
      if (cnt == 0u) continue;
      int tx = iclamp((int)x + base_x + (int)(b & 3u), 0, (int)G - 1);
      int ty = iclamp((int)y + base_y + (int)(b >> 2), 0, (int)GH - 1);
      size_t t_idx = (size_t)ty * G + tx;
      bool blocked = false;
      if (t_idx != idx) {
        uint32_t g_tgt = __ldg(d.gamma + t_idx);
        if (g_tgt >= GAMMA_SOLID) blocked = g_src < GAMMA_SOLID;
        else if (cell_total4(load_cell(d.chem, t_idx)) > capacity_of(g_tgt)) blocked = true;
      }
      if (blocked) stay += cnt;
      else atomicAdd(d.chem_next + t_idx * 4 + ch, cnt);
    }
    if (stay > 0u) atomicAdd(d.chem_next + slot, stay);
  }
}

// ---------------------------------------------------------------------------
// Mover-parallel scatter (same results as k_scatter, bit for bit).
//
// A CTA owns a 32x8 tile of cells; warp w owns row w (lane = cell).
//  A. Each lane runs the per-cell part of transport_scatter (velocity, hop
//     probabilities, osmotic pressure, Kawasaki acceptance, local reactions)
//     and leaves its results in shared memory -- including, for each of the
//     16 cells of its destination window, the accumulator slot a monomer
//     landing there ends up in: blocking by rock or by a full cell depends
//     only on the destination, so it is resolved here once per cell instead
//     of once per monomer.
//  B. The warp's movers (all cells x channels, ~1000) are split into 32
//     equal contiguous ranges, one per lane, so every lane does the same
//     number of mover iterations whatever the per-cell counts are; each
//     mover adds its unit to its slot of a shared accumulator covering the
//     tile and a 2-cell ring (destinations beyond the ring, only with
//     displacements of more than a cell, go straight to global atomics).
//  C. The accumulator is added to chem_next with one atomic per non-zero
//     word.
namespace st {
constexpr int TX = SCATTER_TX, TY = SCATTER_TY, NT = TX * TY;
constexpr int HALO = 2, AW = TX + 2 * HALO, AH = TY + 2 * HALO, AC = AW * AH;
constexpr uint16_t FAR = 0xFFFFu;  // destination outside the accumulator

// The movers of a warp are its non-empty (cell, channel) segments in order,
// listed with a record each: the hash head (x1) of the cell-channel slot and
// a packed word -- bits 0-14 the segment's first mover in the warp's order,
// 15-19 the cell's lane, 20-21 the channel, 22-30 the activated count after
// the local reactions capped at MAX_MOVERS_PER_CH (a mover index k is below
// it, so k < act reads the same).
constexpr uint32_t SEG_START_BITS = 15, SEG_LANE_SHIFT = 15, SEG_CH_SHIFT = 20, SEG_ACT_SHIFT = 22;
static_assert(TX * 4 * MAX_MOVERS_PER_CH <= (1u << SEG_START_BITS), "warp mover positions must fit the start field");
static_assert(MAX_MOVERS_PER_CH < 512u, "the activated count must fit 9 bits");
constexpr int NSEG = 4 * TX;            // segments of a warp at most
constexpr int SSTART = NSEG + TX + 1;   // start table: a step looks up to 32 entries past the current one
constexpr uint16_t NO_START = 0xFFFFu;  // past the listed segments (above every mover position)
// Movers that hop (diffusion, squeeze) or come from a dispersing rubble cell
// take the general path: the main loop queues them (HQ entries per warp)
// and runs the queue densely, so the rarely taken branch is not a step of
// the whole warp in most iterations.
constexpr int HQ = 64;
// The mover loop compares the top 24 bits of a draw with integer
// thresholds: rb_u2f(z) < p exactly when (z >> 8) < ceil(p * 2^24), for p
// in [0, 1] (rb_u2f is (z >> 8) * 2^-24, and scaling by 2^24 is exact; a NaN
// or negative p gives 0, below every draw, as the float test is false).
__device__ __forceinline__ uint32_t u24_threshold(float p) { return rb_f2u(ceilf(p * 16777216.0f)); }
constexpr uint32_t ALWAYS = 1u << 24;  // a threshold every draw is below

struct Smem {
  // per cell (index = warp * 32 + lane)
  float4 mv0[NT];                  // displacement x, y; bound start x, y
  uint4 thr[NT];                   // p_bound (float bits); general-path, hop and settle thresholds
  float dlen[NT];                  // dispersion length, or -1 where the cell does not disperse
  int2 base[NT];                   // window origin: floor(displacement) - 1 per axis
  float4 press[NT];                // osmotic hop weights (+x, -x, +y, -y)
  float acc[8][NT];                // Kawasaki acceptance per direction: activated 0-3, spent 4-7
  // per channel: the activated counts m of the four neighbours, 4 bits each
  // (capped at 8; 15 off the grid), which select the cohesion factor
  // cohf[m] = 1 + cohesion * m of an activated monomer's hop weights (cohf
  // is 1 for m = 15 and wherever cohesion is off)
  uint16_t nbw[4][NT];
  uint16_t slot[16][NT];           // accumulator slot of each window bin (blocking resolved), or FAR
  uint2 rec[TY][NSEG];             // per warp: segment records (above)
  uint16_t sstart[TY][SSTART];     // per warp: first mover of each listed segment, then NO_START
  uint16_t hq[TY][HQ];             // per warp: queued general-path movers, segment << 8 | mover index
  uint32_t accum[4][AC];           // tile + ring destination sums [channel][cell] (lanes on
                                   // neighbouring cells hit neighbouring banks)
  uint8_t rock[AC];                // destination is rock
  uint8_t blk[AC];                 // bit 0: blocks a monomer from a non-rock cell, bit 1: from a rock cell
  float cohf[16];                  // 1 + cohesion * m for m = 0..8 (1 where cohesion is off)
  float exp_dec[8];                // expected decays for min(act, 8) = 1..8
  float2 lattice[4][4];            // smooth_start lattice values of this tile
  float2 jit, glob;                // smooth_start per-step jitter and offset
};

// rb_pcg4d(a, b, c, d) split at the first word that varies inside a mover
// loop: `head` carries the part fixed by (a, b, d), `draw` finishes the hash
// for c.  Same integer operations in the same order, so the same bits.
struct PcgHead {
  uint32_t x1, y0, w0;
};
__device__ __forceinline__ PcgHead pcg_head(uint32_t a, uint32_t b, uint32_t dd) {
  PcgHead h;
  h.y0 = b * 1664525u + 1013904223u;
  h.w0 = dd * 1664525u + 1013904223u;
  h.x1 = (a * 1664525u + 1013904223u) + h.y0 * h.w0;
  return h;
}
// z0 = c * 1664525 + 1013904223 (the caller steps it by 1664525 per c)
__device__ __forceinline__ rb_u4 pcg_draw(const PcgHead& h, uint32_t z0) {
  uint32_t x = h.x1;
  uint32_t y = h.y0 + z0 * x;
  uint32_t z = z0 + x * y;
  uint32_t w = h.w0 + y * z;
  x ^= x >> 16;
  y ^= y >> 16;
  z ^= z >> 16;
  w ^= w >> 16;
  x += y * w;
  y += z * x;
  z += x * y;
  w += y * z;
  rb_u4 r = {x, y, z, w};
  return r;
}
constexpr uint32_t pcg_z0(uint32_t c) { return c * 1664525u + 1013904223u; }
}  // namespace st

template <class Sel>
__global__ void __launch_bounds__(st::NT, 4) k_scatter_tiled(const __grid_constant__ Sel s) {
  RB_WORLD(s);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  st::Smem& S = *reinterpret_cast<st::Smem*>(smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int X0 = cta.bx * st::TX, Y0 = cta.by * st::TY;
  const uint32_t G = d.gw, GH = d.gh;

  // ---- zero the accumulator, load the blocking flags of tile + ring ----
  for (int e = tid; e < st::AC; e += st::NT) {
    S.accum[0][e] = S.accum[1][e] = S.accum[2][e] = S.accum[3][e] = 0u;
    int gx = X0 - st::HALO + e % st::AW, gy = Y0 - st::HALO + e / st::AW;
    uint8_t rock = 0, full = 0;
    if (gx >= 0 && gy >= 0 && gx < (int)G && gy < (int)GH) {
      size_t t = (size_t)gy * G + gx;
      uint32_t g = __ldg(d.gamma + t);
      rock = g >= GAMMA_SOLID;
      full = cell_total4(load_cell(d.chem, t)) > capacity_of(g);
    }
    S.rock[e] = rock;
    // rock blocks monomers from non-rock cells; a full cell blocks everyone
    // else (transport.wgsl:364-401)
    S.blk[e] = (uint8_t)((rock || full ? 1u : 0u) | (!rock && full ? 2u : 0u));
  }
  // smooth_start (transport.wgsl:95-117): the per-step jitter and offset and
  // the lattice values this tile can touch are computed once per CTA.
  if (tid == 0) {
    rb_u4 j = rb_pcg4d(0x85EBCA6Bu, P->epoch, RB_S_MOVE + MAX_MOVERS_PER_CH + 2u, P->seed);
    S.jit = f2(rb_u2f(j.x), rb_u2f(j.y));
    rb_u4 g = rb_pcg4d(0x9E3779B9u, P->epoch, RB_S_MOVE + MAX_MOVERS_PER_CH, P->seed);
    S.glob = f2(rb_u2f(g.x), rb_u2f(g.y));
  }
  __syncthreads();
  const uint32_t jx = rb_f2u(S.jit.x * (float)SMOOTH_CELL), jy = rb_f2u(S.jit.y * (float)SMOOTH_CELL);
  const uint32_t lgx0 = ((uint32_t)X0 + jx) / SMOOTH_CELL, lgy0 = ((uint32_t)Y0 + jy) / SMOOTH_CELL;
  if (tid < 16) {
    uint32_t ix = lgx0 + (tid & 3), iy = lgy0 + (tid >> 2);
    rb_u4 r = rb_pcg4d((ix * 73856093u) ^ (iy * 19349663u), P->epoch, RB_S_MOVE + MAX_MOVERS_PER_CH + 1u, P->seed);
    S.lattice[tid >> 2][tid & 3] = f2(rb_u2f(r.x), rb_u2f(r.y));
  } else if (tid >= 32 && tid < 48) {
    const int m = tid - 32;
    S.cohf[m] = P->cohesion > 0.0f && m <= 8 ? 1.0f + P->cohesion * (float)m : 1.0f;
  } else if (tid >= 64 && tid < 72) {
    // expected decays of a channel with min(act, 8) = m activated monomers
    // (transport.wgsl:281-287): the step's constants, the same operations
    const uint32_t m = (uint32_t)(tid - 63);
    const float shield = 1.0f / (1.0f + CHEM_SHIELD * (float)(m - 1u));
    S.exp_dec[m - 1] = (float)m * rb_max(P->activation_decay, 0.0f) * shield *
                       (float)(P->transport_every > 1u ? P->transport_every : 1u);
  }
  __syncthreads();

  // ---- A. per-cell part (transport.wgsl:120-304) ----
  const uint32_t x = X0 + lane, y = Y0 + warp;
  const int sax = lane + st::HALO, say = warp + st::HALO;  // own accumulator cell
  const bool in_grid = x < G && y < GH;
  const size_t idx = (size_t)y * G + x;
  const uint4 cw = in_grid ? load_cell(d.chem, idx) : make_uint4(0u, 0u, 0u, 0u);
  // Movers per channel: min(act + spent, MAX_MOVERS_PER_CH), which the local
  // reactions leave unchanged, so the warp places its segments first: the
  // cell's first listed segment and the movers of the warp before the cell.
  uint32_t seg_pos, mover_pos, total, nseg;
  {
    const uint32_t m0 = umin(word_total(cw.x), MAX_MOVERS_PER_CH), m1 = umin(word_total(cw.y), MAX_MOVERS_PER_CH);
    const uint32_t m2 = umin(word_total(cw.z), MAX_MOVERS_PER_CH), m3 = umin(word_total(cw.w), MAX_MOVERS_PER_CH);
    const uint32_t cell_sum = m0 + m1 + m2 + m3;
    const uint32_t nz = (m0 > 0u ? 1u : 0u) + (m1 > 0u ? 1u : 0u) + (m2 > 0u ? 1u : 0u) + (m3 > 0u ? 1u : 0u);
    uint32_t incl = cell_sum, incl_nz = nz;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
      const uint32_t tn = __shfl_up_sync(0xffffffffu, incl_nz, o);
      if (lane >= o) {
        incl += t;
        incl_nz += tn;
      }
    }
    total = __shfl_sync(0xffffffffu, incl, 31);
    nseg = __shfl_sync(0xffffffffu, incl_nz, 31);
    seg_pos = incl_nz - nz;
    mover_pos = incl - cell_sum;
  }
  // the start table past the listed segments
  for (int i = (int)nseg + lane; i < st::SSTART; i += 32) S.sstart[warp][i] = st::NO_START;
  if (in_grid) {
    const uint32_t src_total = cell_total4(cw);
    if (src_total != 0u) {
      const uint32_t g_src = __ldg(d.gamma + idx);
      float2 v = f2(0.0f, 0.0f);
      if (P->fluid_enabled != 0u && g_src < GAMMA_SOLID) {
        float2 c = mul2(f2((float)x + 0.5f, (float)y + 0.5f), d.cell_w);
        // On a world whose fluid grid is its environment grid, with power-of-
        // two sides and sim sizes below 2^23, the first sample point lands
        // exactly on the cell's own centre: ((x + 0.5) w) / (G w) is the exact
        // (x + 0.5) / G, times G is x + 0.5, so the bilinear weights are 0 and
        // the sample is the cell's own (sanitised) velocity, up to the sign of
        // a zero component -- which cannot change c + v0 * wpf * h / 2 below
        // (c > 0).  One load instead of the four-point sample.
        const bool centred = d.gw == d.fw && d.gh == d.fh && (d.gw & (d.gw - 1)) == 0 && (d.gh & (d.gh - 1)) == 0 &&
                             d.sim_w < 8388608.0f && d.sim_h < 8388608.0f;
        float2 v0 = centred ? sanitize(d.va[idx]) : fluid_velocity_at_world(d, c);
        float h = rb_max(P->dt, 0.0f);
        float2 c2 = f2(c.x + v0.x * d.wpf_x * h * 0.5f, c.y + v0.y * d.wpf_y * h * 0.5f);
        v = fluid_velocity_at_world(d, c2);
      }
      if (v.x != 0.0f || v.y != 0.0f) {
        bool rock_r = x + 1u < G && S.rock[say * st::AW + sax + 1];
        bool rock_l = x > 0u && S.rock[say * st::AW + sax - 1];
        bool rock_u = y + 1u < GH && S.rock[(say + 1) * st::AW + sax];
        bool rock_d = y > 0u && S.rock[(say - 1) * st::AW + sax];
        if ((v.x > 0.0f && rock_r) || (v.x < 0.0f && rock_l)) v.x = 0.0f;
        else if ((v.x > 0.0f && rock_l) || (v.x < 0.0f && rock_r)) v.x *= 0.5f;
        if ((v.y > 0.0f && rock_u) || (v.y < 0.0f && rock_d)) v.y = 0.0f;
        else if ((v.y > 0.0f && rock_d) || (v.y < 0.0f && rock_u)) v.y *= 0.5f;
      }
      const float tn = (float)(P->transport_every > 1u ? P->transport_every : 1u);
      const float dtp = rb_max(P->dt, 0.0f);
      float2 disp = f2(v.x * d.sx * dtp * tn, v.y * d.sy * dtp * tn);
      float agitation = rb_clamp(len2(v) / DIFF_AGITATION_SPEED, 0.0f, 1.0f);
      float p_diff = rb_clamp(DIFF_HOP_P * rb_mix(DIFF_HOP_FLOOR, 1.0f, agitation) * rb_max(P->diffusion, 0.0f) * tn, 0.0f, 0.5f);
      if (g_src > 0u) p_diff = rb_min(DIFF_HOP_P * BURIED_DIFF_FACTOR / (1.0f + GAMMA_POROSITY_K * (float)g_src) * tn, 0.5f);
      const uint32_t cap_self = capacity_of(g_src);
      if (src_total > cap_self) p_diff = rb_min(CHEM_SQUEEZE_P * tn, 0.5f);
      float p_settle = 0.0f;
      if (g_src == 0u) p_settle = rb_min(MONOMER_SETTLE_P * rb_max(P->settle, 0.0f) * tn, 0.5f);
      float press[4] = {1.0f, 1.0f, 1.0f, 1.0f};
      float max_drop = 0.0f;
      // neighbour counts for the cohesion factors, 4 bits per direction and
      // channel (transport.wgsl:298-304 reads the same words per monomer);
      // 15 marks a neighbour off the grid, whose factor is 1
      uint32_t nbm[4] = {0u, 0u, 0u, 0u};
      const bool use_press = P->monomer_pressure > 0.0f, use_coh = P->cohesion > 0.0f;
      if (use_press || use_coh) {
        const float f_self = (float)src_total / (float)(cap_self > 1u ? cap_self : 1u);
        const long nb[4] = {1, -1, (long)G, -(long)G};
        const bool inside[4] = {x + 1u < G, x > 0u, y + 1u < GH, y > 0u};
#pragma unroll
        for (int k = 0; k < 4; k++) {
          if (!inside[k]) {
            nbm[0] |= 15u << (4 * k);
            nbm[1] |= 15u << (4 * k);
            nbm[2] |= 15u << (4 * k);
            nbm[3] |= 15u << (4 * k);
            continue;
          }
          const size_t n = (size_t)((long)idx + nb[k]);
          const uint4 wn = load_cell(d.chem, n);
          if (use_coh) {
            nbm[0] |= umin(wn.x & CHEM_STATE_MASK, 8u) << (4 * k);
            nbm[1] |= umin(wn.y & CHEM_STATE_MASK, 8u) << (4 * k);
            nbm[2] |= umin(wn.z & CHEM_STATE_MASK, 8u) << (4 * k);
            nbm[3] |= umin(wn.w & CHEM_STATE_MASK, 8u) << (4 * k);
          }
          if (!use_press) continue;
          const uint32_t cap_n = capacity_of(__ldg(d.gamma + n));
          if (cap_n == 0u) continue;
          const float f_n = (float)cell_total4(wn) / (float)cap_n;
          press[k] = rb_max((float)0.05, 1.0f + P->monomer_pressure * (f_self - f_n));
          max_drop = rb_max(max_drop, f_self - f_n);
        }
      }
      p_diff = rb_clamp(p_diff + PRESSURE_HOP_P * P->monomer_pressure * max_drop * tn, 0.0f, 0.5f);
      const float light_t = d.light[(size_t)(umin(y, GH - 1u) / LIGHT_DIV) * d.lw + umin(x, G - 1u) / LIGHT_DIV];
      float p_bound = 0.0f;
      float acc[4] = {1.0f, 1.0f, 1.0f, 1.0f}, accs[4] = {1.0f, 1.0f, 1.0f, 1.0f};
      if (P->aggregation > 0.0f && src_total <= cap_self) {
        float e[5];
        e[0] = (float)d.agg_nb[idx];  // neighbours + own activated counts
        e[1] = x + 1u < G ? (float)d.agg_nb[idx + 1] : 0.0f;
        e[2] = x > 0u ? (float)d.agg_nb[idx - 1] : 0.0f;
        e[3] = y + 1u < GH ? (float)d.agg_nb[idx + G] : 0.0f;
        e[4] = y > 0u ? (float)d.agg_nb[idx - G] : 0.0f;
        uint32_t fx = umin((x * (uint32_t)d.fw) / G, (uint32_t)d.fw - 1u);
        uint32_t fy = umin((y * (uint32_t)d.fh) / GH, (uint32_t)d.fh - 1u);
        float t_rel = 1.0f + rb_max(d.temp_in[(size_t)fy * d.fw + fx], 0.0f) / TEMP_ACT_THRESHOLD;
        float room = rb_clamp(5.0f * (1.0f - (float)src_total / (float)(cap_self > 1u ? cap_self : 1u)), 0.0f, 1.0f);
        float k_e = P->aggregation * room / t_rel;
        // drop = e0 - ek and rise = ek - e0 are exact negatives of each
        // other, so at most one is positive and it equals |e0 - ek|: one
        // exponential per direction gives both acceptances, the same four
        // calls on every lane instead of a divergent pair per direction.
#pragma unroll
        for (int k = 0; k < 4; k++) {
          const float drop = e[0] - e[k + 1];
          const float a = rb_exp(-k_e * rb_abs(drop));
          if (drop > 0.0f) acc[k] = a;
          else if (drop < 0.0f) accs[k] = a;
        }
        p_bound = 1.0f - rb_exp(-k_e * rb_min(rb_max(e[0] - 1.0f, 0.0f), 48.0f));
      }
      float2 bound_start = f2(0.0f, 0.0f);
      if (p_bound > 0.0f) {  // smooth_start(x, y) from the tile's lattice
        const uint32_t sx = x + jx, sy = y + jy;
        const uint32_t lx = sx / SMOOTH_CELL - lgx0, ly = sy / SMOOTH_CELL - lgy0;
        float tx = rb_smoothstep01(((float)(sx % SMOOTH_CELL) + 0.5f) / (float)SMOOTH_CELL);
        float ty = rb_smoothstep01(((float)(sy % SMOOTH_CELL) + 0.5f) / (float)SMOOTH_CELL);
        float2 n = mix2(mix2(S.lattice[ly][lx], S.lattice[ly][lx + 1], tx), mix2(S.lattice[ly + 1][lx], S.lattice[ly + 1][lx + 1], tx), ty);
        float vx = rb_fract(n.x + S.glob.x), vy = rb_fract(n.y + S.glob.y);
        bound_start = f2(1.0f - rb_abs(2.0f * vx - 1.0f), 1.0f - rb_abs(2.0f * vy - 1.0f));
      }
      const bool disperse = g_src > 0u && (disp.x != 0.0f || disp.y != 0.0f);
      const int basex = rb_floor_i(disp.x) - 1, basey = rb_floor_i(disp.y) - 1;
      S.mv0[tid] = make_float4(disp.x, disp.y, bound_start.x, bound_start.y);
      S.base[tid] = make_int2(basex, basey);
      {
        // A dispersing cell sends every mover down the general path, and so
        // does a displacement of 2^22 cells or more.  Below that, for a start
        // s in [0, 1]: d <= fl(s + d) <= fl(d + 1) <= floor(d) + 2 (an
        // integer, representable), so a main-path mover's window offset
        // floor(fl(s + d)) - floor(d) + 1 is 1, 2 or 3 per axis -- 3 when d is
        // just below an integer and s + d rounds up to the next one -- and 0
        // to 2 in y after settling: its bin is below 16 and needs no clamp.
        const bool general_only = disperse || !(rb_abs(disp.x) < 4194304.0f && rb_abs(disp.y) < 4194304.0f);
        const uint32_t t_hop = st::u24_threshold(p_diff);
        S.thr[tid] = make_uint4(__float_as_uint(p_bound), general_only ? st::ALWAYS : t_hop, t_hop,
                                st::u24_threshold(p_diff + p_settle));
      }
      S.dlen[tid] = disperse ? len2(disp) : -1.0f;
      S.press[tid] = make_float4(press[0], press[1], press[2], press[3]);
#pragma unroll
      for (int k = 0; k < 4; k++) {
        S.acc[k][tid] = acc[k];
        S.acc[4 + k][tid] = accs[k];
      }
      // destination slot of every window bin (transport.wgsl:364-401); the
      // window's columns and rows are clamped and located once
      {
        const uint16_t own = (uint16_t)(say * st::AW + sax);
        const uint32_t src_bit = g_src >= GAMMA_SOLID ? 1u : 0u;
        int txs[4], axs[4];
#pragma unroll
        for (int o = 0; o < 4; o++) {
          txs[o] = iclamp((int)x + basex + o, 0, (int)G - 1);
          axs[o] = txs[o] - (X0 - st::HALO);
        }
        for (int oy = 0; oy < 4; oy++) {
          const int ty = iclamp((int)y + basey + oy, 0, (int)GH - 1), ay = ty - (Y0 - st::HALO);
          const bool near_y = ay >= 0 && ay < st::AH;
#pragma unroll
          for (int ox = 0; ox < 4; ox++) {
            const int ax = axs[ox];
            uint16_t sl;
            if (txs[ox] == (int)x && ty == (int)y) {
              sl = own;
            } else if (near_y && ax >= 0 && ax < st::AW) {
              const int cell = ay * st::AW + ax;
              sl = (S.blk[cell] >> src_bit) & 1u ? own : (uint16_t)cell;
            } else {
              const size_t t = (size_t)ty * G + txs[ox];
              const uint32_t g_t = __ldg(d.gamma + t);
              const bool rock = g_t >= GAMMA_SOLID;
              const bool full = cell_total4(load_cell(d.chem, t)) > capacity_of(g_t);
              const bool blocked = rock ? (g_src < GAMMA_SOLID) : full;
              sl = blocked ? own : st::FAR;
            }
            S.slot[oy * 4 + ox][tid] = sl;
          }
        }
      }
      // local reactions per channel (transport.wgsl:262-294)
      const uint32_t words[4] = {cw.x, cw.y, cw.z, cw.w};
      const float light_term = LIGHT_ACT_P * rb_max(P->uv_strength, 0.0f) * rb_max(P->direct_photoactivation, 0.0f) * light_t;
#pragma unroll
      for (uint32_t ch = 0; ch < 4; ch++) {
        const uint32_t slot = (uint32_t)(idx * 4 + ch);
        uint32_t act_n = words[ch] & CHEM_STATE_MASK;
        uint32_t spent_n = words[ch] >> 16;
        if (act_n + spent_n == 0u) continue;
        // rb_pcg4d(slot, epoch, RB_S_PHOTO / RB_S_DECAY, seed), sharing the slot's head
        const st::PcgHead rh = st::pcg_head(slot, P->epoch, P->seed);
        if (spent_n > 0u) {
          float sens = 1.0f + CHEM_SENSITIZE * (float)umin(act_n, 8u);
          float exp_act = (float)umin(spent_n, 8u) * tn * (light_term * sens + rb_max(P->reactivation_rate, 0.0f));
          uint32_t na = rb_f2u(rb_floor(exp_act));
          float frac = exp_act - (float)na;
          if (frac > 0.0f && rb_u2f(st::pcg_draw(rh, st::pcg_z0(RB_S_PHOTO)).x) < frac) na += 1u;
          na = umin(na, umin(spent_n, 8u));
          act_n += na;
          spent_n -= na;
        }
        if (act_n > 0u) {
          const float exp_dec = S.exp_dec[umin(act_n, 8u) - 1u];
          if (exp_dec > 0.0f && rb_u2f(st::pcg_draw(rh, st::pcg_z0(RB_S_DECAY)).x) < exp_dec) {
            act_n -= 1u;
            spent_n += 1u;
          }
        }
        const uint32_t n = act_n + spent_n;
        const uint32_t movers = umin(n, MAX_MOVERS_PER_CH);
        const uint32_t act_stay = act_n - umin(act_n, movers);
        const uint32_t stay = act_stay + (n - movers - act_stay) * CHEM_SPENT_ONE;
        if (stay) atomicAdd(&S.accum[ch][say * st::AW + sax], stay);
        S.nbw[ch][tid] = (uint16_t)nbm[ch];
        S.rec[warp][seg_pos] = make_uint2(rh.x1, mover_pos | (uint32_t)lane << st::SEG_LANE_SHIFT |
                                                     ch << st::SEG_CH_SHIFT |
                                                     umin(act_n, MAX_MOVERS_PER_CH) << st::SEG_ACT_SHIFT);
        S.sstart[warp][seg_pos] = (uint16_t)mover_pos;
        seg_pos++;
        mover_pos += movers;
      }
    }
  }

  // ---- B. movers: the warp takes 32 consecutive movers per step ----
  // Lane l of a step takes mover jb + l of the warp's order.  Its segment is
  // the one holding mover jb plus the segments that start in (jb, jb + l]:
  // the lanes read the next 32 segment starts (segments are not empty, so at
  // most 32 of them start in a window of 32 movers) and mark those inside
  // the window.  Every lane runs the same instructions; the movers that
  // hop or disperse are queued and run together at the end of the warp's
  // movers, or when the queue fills.
  __syncthreads();
  {
    const uint2* rec = S.rec[warp];
    const uint16_t* sstart = S.sstart[warp];
    uint16_t* hq = S.hq[warp];
    const st::PcgHead ph0 = st::pcg_head(0u, P->epoch, P->seed);  // y0, w0 of every move draw of the step
    const int cy = Y0 + warp;
    const uint32_t lt_mask = (1u << lane) - 1u, le_mask = 0xFFFFFFFFu >> (31 - lane);
    constexpr uint32_t Z_DISPERSE = st::pcg_z0(RB_S_DISPERSE) - st::pcg_z0(RB_S_MOVE);
    constexpr uint32_t START_MASK = (1u << st::SEG_START_BITS) - 1u;

    // the general path of mover k of segment s (transport.wgsl:306-406):
    // bound or uniform start, displacement, rubble dispersion, the
    // diffusion / squeeze hop with osmotic and cohesion weights and Kawasaki
    // acceptance, settling; then the window bin and its accumulator slot, or
    // a global atomic beyond the ring
    auto general = [&](uint32_t q) {
      const uint32_t s = q >> 8, k = q & 255u;
      const uint2 r = rec[s];
      const int ct = warp * 32 + (int)((r.y >> st::SEG_LANE_SHIFT) & 31u), ch = (int)((r.y >> st::SEG_CH_SHIFT) & 3u);
      const bool is_act = k < (r.y >> st::SEG_ACT_SHIFT);
      const uint32_t unit = is_act ? 1u : CHEM_SPENT_ONE;
      const float4 m0 = S.mv0[ct];
      const uint4 th = S.thr[ct];
      const float dlen = S.dlen[ct];
      st::PcgHead ph = ph0;
      ph.x1 = r.x;
      const uint32_t zk = st::pcg_z0(RB_S_MOVE + k);
      const rb_u4 ru = st::pcg_draw(ph, zk);  // rb_pcg4d(slot, epoch, RB_S_MOVE + k, seed)
      const float rfx = rb_u2f(ru.x), rfy = rb_u2f(ru.y), rfz = rb_u2f(ru.z), rfw = rb_u2f(ru.w);
      const float p_bound = __uint_as_float(th.x);
      const bool bound = is_act && p_bound > 0.0f && rb_fract(rfz * (float)7.31 + rfw * (float)3.17) < p_bound;
      float px = (bound ? m0.z : rfx) + m0.x;
      float py = (bound ? m0.w : rfy) + m0.y;
      if (dlen >= 0.0f) {
        const rb_u4 rj = st::pcg_draw(ph, zk + Z_DISPERSE);  // rb_pcg4d(slot, epoch, RB_S_DISPERSE + k, seed)
        float jxx = (rb_u2f(rj.x) * 2.0f - 1.0f) * dlen * RUBBLE_DISPERSION;
        float jyy = (rb_u2f(rj.y) * 2.0f - 1.0f) * dlen * RUBBLE_DISPERSION;
        px += rb_clamp(jxx, (float)-0.9, (float)0.9);
        py += rb_clamp(jyy, (float)-0.9, (float)0.9);
      }
      const uint32_t z24 = ru.z >> 8;
      if (z24 < th.z) {  // rfz < p_diff
        // hop weights: osmotic pressure times, for an activated monomer, the
        // cohesion factors (transport.wgsl:298-304)
        const float4 pr = S.press[ct];
        const uint32_t mw = is_act ? (uint32_t)S.nbw[ch][ct] : 0xFFFFu;
        const float w0 = pr.x * S.cohf[mw & 15u], w1 = pr.y * S.cohf[(mw >> 4) & 15u];
        const float w2 = pr.z * S.cohf[(mw >> 8) & 15u], w3 = pr.w * S.cohf[mw >> 12];
        float u = rfw * (w0 + w1 + w2 + w3);
        uint32_t dd;
        if (u < w0) dd = 0u;
        else if ((u -= w0) < w1) dd = 1u;
        else if ((u -= w1) < w2) dd = 2u;
        else dd = 3u;
        const float acc_d = S.acc[(is_act ? 0u : 4u) + dd][ct];
        const bool stay_put = rb_fract(rfw * (float)13.73 + rfx * (float)5.31) >= acc_d;
        if (!stay_put) {
          if (dd == 0u) px += 1.0f;
          else if (dd == 1u) px -= 1.0f;
          else if (dd == 2u) py += 1.0f;
          else py -= 1.0f;
        }
      } else if (z24 < th.w) {  // rfz < p_diff + p_settle
        py -= 1.0f;
      }
      const int2 bs = S.base[ct];
      const int offx = rb_floor_i(px) - bs.x, offy = rb_floor_i(py) - bs.y;
      const uint32_t bi = (uint32_t)iclamp(offy, 0, 3) * 4u + (uint32_t)iclamp(offx, 0, 3);
      const uint16_t sl = S.slot[bi][ct];
      if (sl != st::FAR) {
        if (RB_IN(sl, st::AC, d.status)) atomicAdd(&S.accum[ch][sl], unit);
      } else {
        const int tx = iclamp(X0 + (ct & 31) + bs.x + (int)(bi & 3u), 0, (int)G - 1);
        const int ty = iclamp(cy + bs.y + (int)(bi >> 2), 0, (int)GH - 1);
        const size_t t = ((size_t)ty * G + tx) * 4 + ch;
        if (RB_IN(t, (size_t)G * GH * 4, d.status)) atomicAdd(d.chem_next + t, unit);
      }
    };

    uint32_t cur = 0;  // the segment holding mover jb (warp-uniform)
    uint32_t qn = 0;   // queued movers (warp-uniform)
    for (uint32_t jb = 0; jb < total; jb += 32) {
      const uint32_t j = jb + lane;
      const bool valid = j < total;
      // cur <= nseg - 1 <= NSEG - 1, so the entry read is below NSEG + 32 < SSTART
      const uint32_t sc = RB_IN(cur + 1 + lane, st::SSTART, d.status) ? sstart[cur + 1 + lane] : st::NO_START;
      const uint32_t starts = __reduce_or_sync(0xffffffffu, sc < jb + 32u ? 1u << (sc - jb) : 0u);
      const uint32_t s = cur + __popc(starts & le_mask);
      cur += __popc(__ballot_sync(0xffffffffu, sc <= jb + 32u));
      const uint2 r = rec[s];
      const uint32_t k = j - (r.y & START_MASK);
      const int ct = warp * 32 + (int)((r.y >> st::SEG_LANE_SHIFT) & 31u), ch = (int)((r.y >> st::SEG_CH_SHIFT) & 3u);
      const float4 m0 = S.mv0[ct];
      const uint4 th = S.thr[ct];
      st::PcgHead ph = ph0;
      ph.x1 = r.x;
      const rb_u4 ru = st::pcg_draw(ph, st::pcg_z0(RB_S_MOVE + k));  // rb_pcg4d(slot, epoch, RB_S_MOVE + k, seed)
      const uint32_t z24 = ru.z >> 8;
      const bool gen = valid && z24 < th.y;  // hops (rfz < p_diff), or the cell takes the general path only
      const uint32_t gm = __ballot_sync(0xffffffffu, gen);
      if (gen && RB_IN(qn + __popc(gm & lt_mask), st::HQ, d.status)) hq[qn + __popc(gm & lt_mask)] = (uint16_t)(s << 8 | k);
      qn += __popc(gm);
      if (valid && !gen) {
        // no hop, no dispersion: bound or uniform start, displacement, settling
        const bool is_act = k < (r.y >> st::SEG_ACT_SHIFT);
        const uint32_t unit = is_act ? 1u : CHEM_SPENT_ONE;
        const float p_bound = __uint_as_float(th.x);
        const bool bound = is_act && p_bound > 0.0f &&
                           rb_fract(rb_u2f(ru.z) * (float)7.31 + rb_u2f(ru.w) * (float)3.17) < p_bound;
        const float px = (bound ? m0.z : rb_u2f(ru.x)) + m0.x;
        float py = (bound ? m0.w : rb_u2f(ru.y)) + m0.y;
        if (z24 < th.w) py -= 1.0f;  // rfz < p_diff + p_settle (and not below p_diff)
        const int2 bs = S.base[ct];
        const uint32_t bi = (uint32_t)((rb_floor_i(py) - bs.y) * 4 + (rb_floor_i(px) - bs.x));  // in [1, 15]
        if (RB_IN(bi, 16, d.status)) {
          const uint16_t sl = S.slot[bi][ct];
          if (sl != st::FAR) {
            if (RB_IN(sl, st::AC, d.status)) atomicAdd(&S.accum[ch][sl], unit);
          } else {
            const int tx = iclamp(X0 + (ct & 31) + bs.x + (int)(bi & 3u), 0, (int)G - 1);
            const int ty = iclamp(cy + bs.y + (int)(bi >> 2), 0, (int)GH - 1);
            const size_t t = ((size_t)ty * G + tx) * 4 + ch;
            if (RB_IN(t, (size_t)G * GH * 4, d.status)) atomicAdd(d.chem_next + t, unit);
          }
        }
      }
      // the queue holds at most HQ - 32 movers before a step adds up to 32
      if (qn > (uint32_t)(st::HQ - 32) || jb + 32u >= total) {
        __syncwarp();
        for (uint32_t q = lane; q < qn; q += 32) general(hq[q]);
        __syncwarp();
        qn = 0;
      }
    }
  }
  __syncthreads();

  // ---- C. accumulator -> chem_next ----
  for (int e = tid; e < st::AC * 4; e += st::NT) {
    int cell = e >> 2, ch = e & 3;
    uint32_t v = S.accum[ch][cell];
    if (!v) continue;
    int gx = X0 - st::HALO + cell % st::AW, gy = Y0 - st::HALO + cell / st::AW;
    // only in-grid destinations receive monomers (the slots are clamped to the grid)
    if (RB_IN(gx, G, d.status) && RB_IN(gy, GH, d.status)) atomicAdd(d.chem_next + ((size_t)gy * G + gx) * 4 + ch, v);
  }
}

// ledger.wgsl:225-245: per-block sums in registers and warp shuffles, then
// one global atomic add per counter (u32, wrapping like the reference).
template <class S>
__global__ void __launch_bounds__(LINEAR_THREADS) k_ledger(const __grid_constant__ S s) {
  RB_WORLD(s);
  uint32_t* out = out_of(s, cta.w);
  const size_t cells = (size_t)d.gw * d.gh;
  uint32_t a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  const uint4* c4 = reinterpret_cast<const uint4*>(d.chem);
  const size_t stride = (size_t)cta.nbx * LINEAR_THREADS;
  auto add = [&](uint4 c) {
    a[0] += c.x & 0xFFFFu;
    a[1] += c.y & 0xFFFFu;
    a[2] += c.z & 0xFFFFu;
    a[3] += c.w & 0xFFFFu;
    a[4] += c.x >> 16;
    a[5] += c.y >> 16;
    a[6] += c.z >> 16;
    a[7] += c.w >> 16;
  };
  // four strides per round, their loads in flight together (u32 sums: the
  // order of the adds does not change them)
  size_t i = (size_t)cta.bx * LINEAR_THREADS + threadIdx.x;
  for (; i + 3 * stride < cells; i += 4 * stride) {
    const uint4 c0 = __ldg(c4 + i), c1 = __ldg(c4 + i + stride), c2 = __ldg(c4 + i + 2 * stride), c3 = __ldg(c4 + i + 3 * stride);
    add(c0);
    add(c1);
    add(c2);
    add(c3);
  }
  for (; i < cells; i += stride) add(__ldg(c4 + i));
  __shared__ uint32_t red[LINEAR_THREADS / 32][8];
#pragma unroll
  for (int k = 0; k < 8; k++) {
    uint32_t v = a[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < 8) {
    uint32_t v = 0;
    for (int wv = 0; wv < LINEAR_THREADS / 32; wv++) v += red[wv][threadIdx.x];
    if (v) atomicAdd(out + threadIdx.x, v);
  }
}

// chem_next = 0 for the next step's scatter (the batched form of a memset).
template <class S>
__global__ void __launch_bounds__(LINEAR_THREADS) k_zero_next(const __grid_constant__ S s) {
  RB_WORLD(s);
  const size_t i = (size_t)cta.bx * LINEAR_THREADS + threadIdx.x;
  if (i < (size_t)d.gw * d.gh) reinterpret_cast<uint4*>(d.chem_next)[i] = make_uint4(0u, 0u, 0u, 0u);
}

}  // namespace

inline double gc(const Dev& d) { return (double)d.gw * d.gh; }

void launch_slope(const Dev& d, float upc, cudaStream_t s) {
  const dim3 grid((d.gw + BX - 1) / BX, (d.gh + BY - 1) / BY);
  RB_LAUNCH("compute_gamma_slope", 12.0 * gc(d), s, k_slope<<<grid, dim3(BX, BY), 0, s>>>(d, upc));
}
void launch_thermal(const Target& t, cudaStream_t s) {
  RB_PASS("thermal_activation", 4.0 * t.fcells, s, t, GEO_ENV_TALL, dim3(BX, BY), 0, k_thermal, nullptr);
}
void launch_agg(const Target& t, cudaStream_t s) {
  RB_PASS("aggregation_counts", 20.0 * t.cells, s, t, GEO_ENV, dim3(BX, BY), 0, k_agg, nullptr);
}
void launch_scatter(const Target& t, bool simple, cudaStream_t s) {
  const double bytes = 45.0 * t.cells + 12.0 * t.fcells;
  if (simple) {
    RB_PASS("transport_scatter_simple", bytes, s, t, GEO_ENV, dim3(BX, BY), 0, k_scatter, nullptr);
    return;
  }
  static DeviceOnce attr;
  const int dev = DeviceOnce::device();
  if (attr.pending(dev)) {
    cudaFuncSetAttribute(k_scatter_tiled<OneWorld>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(st::Smem));
    cudaFuncSetAttribute(k_scatter_tiled<WorldSet>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(st::Smem));
    attr.done(dev);
  }
  RB_PASS("transport_scatter", bytes, s, t, GEO_SCATTER, dim3(st::NT), sizeof(st::Smem), k_scatter_tiled, nullptr);
}
void launch_zero_next(const Target& t, cudaStream_t s) {
  RB_PASS("zero_chem_next", 16.0 * t.cells, s, t, GEO_ENV_LINEAR, dim3(LINEAR_THREADS), 0, k_zero_next, nullptr);
}
void launch_ledger(const Target& t, uint32_t* out, cudaStream_t s) {
  RB_PASS("ledger_reduce", 16.0 * t.cells, s, t, GEO_LEDGER, dim3(LINEAR_THREADS), 0, k_ledger, out);
}

}  // namespace ribo
