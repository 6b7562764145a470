// CPU ORACLE for the world-step hot path -- test infrastructure only.
//
// This file is a from-scratch C++ restatement of the reference's WGSL world
// passes, used by the test suite (and by bench.py's CPU baseline leg) as the
// checker of the CUDA library.  It is never linked into the product.
//
// Each function cites the WGSL (or Rust) lines it restates, with paths
// relative to the reference project.  Arithmetic is IEEE single precision
// with no contraction (-ffp-contract=off); mix/exp/pow/sin/smoothstep come
// from ribo_fmath.h, the same pinned definitions the CUDA kernels use, so
// bit-exact comparison with the GPU is meaningful.  Constant expressions that
// WGSL evaluates as abstract floats (f64) are written as (float)(double).
//
// Parity pinning: the reference publishes no golden vectors for this path
// (its tests assert invariants only); the oracle is pinned by those
// invariants (exact conservation, determinism, finiteness, net-flux bound)
// and by hand-derived known-answer cases in the test suite.
//
// Threads: OpenMP over rows.  Transport adds into chem_next with relaxed
// atomic integer adds (order-independent), so results do not depend on the
// thread count.
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/ribo_world.h"
#include "../ribossome-v2_gb300/csrc/ribo_fmath.h"

namespace {

struct V2 {
  float x, y;
};
static inline V2 v2(float x, float y) { return V2{x, y}; }
static inline V2 operator+(V2 a, V2 b) { return v2(a.x + b.x, a.y + b.y); }
static inline V2 operator-(V2 a, V2 b) { return v2(a.x - b.x, a.y - b.y); }
static inline V2 operator*(V2 a, float s) { return v2(a.x * s, a.y * s); }
static inline V2 operator*(float s, V2 a) { return v2(s * a.x, s * a.y); }
static inline V2 operator/(V2 a, float s) { return v2(a.x / s, a.y / s); }
static inline float dot(V2 a, V2 b) { return a.x * b.x + a.y * b.y; }
static inline float length(V2 a) { return rb_sqrt(a.x * a.x + a.y * a.y); }
static inline V2 mix2(V2 a, V2 b, float t) { return v2(rb_mix(a.x, b.x, t), rb_mix(a.y, b.y, t)); }

// ---- constants (shaders/world/fluid.wgsl:15-56, transport.wgsl:23-50,
// common/chem.wgsl:118-119, common/terrain.wgsl:214, light.wgsl:18-40) ----
const float MAX_DT = (float)0.07;
const float MAX_FORCE = (float)200000.0;
const float MAX_VEL = (float)2000.0;
const float FORCE_SMOOTH_MIX = (float)0.25;
const float SOLID_PERM_THRESHOLD = (float)0.02;
const float TEMP_HEAT_RATE = (float)0.01;
const float TEMP_COOL_RATE = (float)0.12;
const float TEMP_MAX = (float)12.0;
const float SUN_HEAT_RATE = (float)0.15;
const float SUN_IR = (float)1.2;
const float SUN_IR_DEPTH = (float)0.08;
const float TEMP_BUOYANCY = (float)12.0;
const float TEMP_AMBIENT_SURFACE = (float)0.0;
const float TEMP_AMBIENT_ATTEN = (float)4.0;
const float TEMP_DIFFUSE = (float)0.08;
const float TEMP_ROCK_CONDUCT = (float)4.0;
const float REDOX_RATE = (float)0.01;
const float VENT_WAVES = (float)1.5;
const float REDOX_FP = (float)10000.0;
const float REDOX_MAX = (float)50.0;
const float RUBBLE_DRAG = (float)300.0;
const float FORCE_FP = (float)256.0;
const float DIFF_HOP_P = (float)0.01;
const float DIFF_HOP_FLOOR = (float)0.15;
const float DIFF_AGITATION_SPEED = (float)0.5;
const float BURIED_DIFF_FACTOR = (float)1.0;
const float GAMMA_POROSITY_K = (float)0.3;
const float PRESSURE_HOP_P = (float)0.01;
const float RUBBLE_DISPERSION = (float)1.0;
const float CHEM_SQUEEZE_P = (float)0.25;
const float MONOMER_SETTLE_P = (float)0.002;
const uint32_t MAX_MOVERS_PER_CH = 256u;
const float LIGHT_ACT_P = (float)0.006;
const float CHEM_SENSITIZE = (float)0.5;
const float CHEM_SHIELD = (float)0.5;
const float TEMP_ACT_THRESHOLD = (float)2.0;
const float FUMAROLE_ACT_P = (float)0.15;
const uint32_t SMOOTH_CELL = 16u;
const uint32_t CHEM_STATE_MASK = 0xFFFFu;
const uint32_t CHEM_SPENT_ONE = 0x10000u;
const uint32_t CHEM_CELL_CAP = 48u;
const uint32_t GAMMA_SOLID = 3u;
const float GAMMA_QUANTUM = (float)0.25;
const uint32_t LIGHT_DIV = 2u;
const float UV_SHADOW_ABSORB = (float)0.6;
const float AGENT_UV_ABSORB = (float)0.15;
const float SUN_WATER_ABSORB = (float)0.05;
const int LIGHT_TAPS = 7;
const float SHADE_ONE = (float)100.0;
const float MG_EPS = (float)1e-4;
// terrain grains (shaders/world/terrain.wgsl:6-34, transport.wgsl:41)
const uint32_t SANDPILE_DIFF = 3u;
const float GAMMA_RELAX_P = (float)0.12;
const float GAMMA_STRAY_WALK_P = (float)0.05;
const float GAMMA_SEDIMENT_FACTOR = (float)0.5;
const float GAMMA_SETTLE_SPEED = (float)0.5;
const uint32_t GAMMA_ROCK_FULL = 6u;
const float VENT_BLOW = (float)8.0;
const float GAMMA_SHED_P = (float)0.03;
const float GRAIN_ADV_CAP = (float)0.9;
const size_t NO_CELL = ~(size_t)0;

static inline uint32_t atomic_add_u32(uint32_t* p, uint32_t v) {
  return __atomic_fetch_add(p, v, __ATOMIC_RELAXED);
}

struct Level {
  int nx, ny;
  size_t off;
  float eps;
};

struct Oracle {
  ribo_world_cfg cfg;
  ribo_world_settings st;
  int gw, gh, fw, fh, lw, lh, rx, ry;
  float sim_w, sim_h;
  bool fluid_was_on = true;
  bool light_dirty = true;        // the next light block is a full sweep
  std::vector<float> light_next;  // light_propagate's output
  const ribo_sim_params* P = nullptr;

  std::vector<uint32_t> chem, chem_next, gamma, agg_act, agg_nb, shade, force_vec, redox_eaten, solid_mask;
  std::vector<float> light, pressure_a, pressure_b, div, temp_a, temp_b, redox_a, redox_b, net_flux;
  std::vector<V2> slope, vel_a, vel_b, vel_smooth, fluid_forces, heat;
  std::vector<Level> levels;
  std::vector<float> mg_p, mg_rhs;
  std::vector<uint32_t> mg_fluid;

  size_t cells() const { return (size_t)gw * gh; }
  size_t fcells() const { return (size_t)fw * fh; }
  size_t lcells() const { return (size_t)lw * lh; }

  // ---- terrain / chem helpers (common/terrain.wgsl:216, common/chem.wgsl:121-145) ----
  uint32_t gamma_count(size_t c) const { return gamma[c]; }
  uint32_t chem_act_count(size_t idx, uint32_t ch) const { return chem[idx * 4 + ch] & CHEM_STATE_MASK; }
  uint32_t chem_cell_total(size_t cell) const {
    uint32_t t = 0;
    for (int c = 0; c < 4; c++) {
      uint32_t v = chem[cell * 4 + c];
      t += (v & CHEM_STATE_MASK) + (v >> 16);
    }
    return t;
  }
  uint32_t chem_capacity(size_t cell) const {
    uint32_t g = gamma_count(cell);
    if (g >= GAMMA_SOLID) return 0u;
    return CHEM_CELL_CAP * (GAMMA_SOLID - g) / GAMMA_SOLID;
  }

  size_t fgrid(uint32_t x, uint32_t y) const { return (size_t)y * fw + x; }
  bool is_solid(uint32_t x, uint32_t y) const { return solid_mask[fgrid(x, y)] != 0u; }

  // fluid.wgsl:66-83
  float fluid_dt() const { return rb_clamp(P->fluid_dt, 0.0f, MAX_DT); }
  static bool is_bad(float x) { return (x != x) || (rb_abs(x) > (float)1e20); }
  static V2 sanitize(V2 v) { return (is_bad(v.x) || is_bad(v.y)) ? v2(0.0f, 0.0f) : v; }
  static V2 clamp_len(V2 v, float max_len) {
    float len = length(v);
    if (len > max_len) return v * (max_len / rb_max(len, (float)1e-12));
    return v;
  }
  // fluid.wgsl:62-64
  float temp_ambient_at(uint32_t y) const {
    return TEMP_AMBIENT_SURFACE * rb_exp(-TEMP_AMBIENT_ATTEN * (1.0f - ((float)y + 0.5f) / (float)fh));
  }
  // fluid.wgsl:46-54
  float vent_cycle(uint32_t x) const {
    float m = 1.0f;
    if (P->vent_cycle_amp > 0.0f && P->vent_cycle_period >= 1.0f) {
      uint32_t period = rb_f2u(P->vent_cycle_period);
      float t = (float)(P->epoch % period) / (float)period;
      m = rb_max(1.0f + P->vent_cycle_amp * rb_sin((float)6.2831853 * (t + VENT_WAVES * (float)x / (float)fw)), 0.0f);
    }
    return m;
  }

  // ---- obstacles (fluid.wgsl:87-142) ----
  size_t env_cell_for_fluid(uint32_t x, uint32_t y) const {
    float sx = (float)gw / (float)fw, sy = (float)gh / (float)fh;
    uint32_t gx = rb_f2u(rb_clamp(((float)x + 0.5f) * sx, 0.0f, (float)(gw - 1)));
    uint32_t gy = rb_f2u(rb_clamp(((float)y + 0.5f) * sy, 0.0f, (float)(gh - 1)));
    return (size_t)gy * gw + gx;
  }
  float gamma_solidity_at_fluid_cell(uint32_t x, uint32_t y) const {
    float scx = (float)gw / (float)fw, scy = (float)gh / (float)fh;
    float gx = ((float)x + 0.5f) * scx, gy = ((float)y + 0.5f) * scy;
    float hx = scx * 0.25f, hy = scy * 0.25f;
    uint32_t n_solid = 0;
    for (uint32_t s = 0; s < 4; s++) {
      float ox = (s & 1u) == 1u ? hx : -hx;
      float oy = (s & 2u) == 2u ? hy : -hy;
      uint32_t sx = rb_f2u(rb_clamp(gx + ox, 0.0f, (float)(gw - 1)));
      uint32_t sy = rb_f2u(rb_clamp(gy + oy, 0.0f, (float)(gh - 1)));
      if (gamma_count((size_t)sy * gw + sx) >= GAMMA_SOLID) n_solid++;
    }
    return (float)n_solid * 0.25f;
  }
  float gamma_fill_at_fluid_cell(uint32_t x, uint32_t y) const {
    float scx = (float)gw / (float)fw, scy = (float)gh / (float)fh;
    float gx = ((float)x + 0.5f) * scx, gy = ((float)y + 0.5f) * scy;
    float hx = scx * 0.25f, hy = scy * 0.25f;
    float fill = 0.0f;
    for (uint32_t s = 0; s < 4; s++) {
      float ox = (s & 1u) == 1u ? hx : -hx;
      float oy = (s & 2u) == 2u ? hy : -hy;
      uint32_t sx = rb_f2u(rb_clamp(gx + ox, 0.0f, (float)(gw - 1)));
      uint32_t sy = rb_f2u(rb_clamp(gy + oy, 0.0f, (float)(gh - 1)));
      fill += (float)std::min(gamma_count((size_t)sy * gw + sx), GAMMA_SOLID) / (float)GAMMA_SOLID;
    }
    return fill * 0.25f;
  }
  float permeability(uint32_t x, uint32_t y) const {
    float solidity = gamma_solidity_at_fluid_cell(x, y);
    if (solidity >= 0.5f) return 0.0f;
    return rb_clamp(1.0f - solidity * 2.0f, 0.0f, 1.0f);
  }
  // fluid.wgsl:150-161
  float rubble_drag(uint32_t x, uint32_t y, float dt) const {
    float g = 0.0f;
    for (int dy = 0; dy < ry; dy++)
      for (int dx = 0; dx < rx; dx++) {
        uint32_t c = gamma_count((size_t)(y * ry + dy) * gw + x * rx + dx);
        if (c < GAMMA_SOLID) g += (float)c;
      }
    g = g / ((float)(rx * ry) * (float)GAMMA_SOLID);
    return 1.0f / (1.0f + RUBBLE_DRAG * g * dt);
  }
  // fluid.wgsl:165-178
  V2 slope_steer_velocity(uint32_t x, uint32_t y, V2 v_in, float dt) const {
    V2 s0 = sanitize(slope[env_cell_for_fluid(x, y)]);
    V2 s = v2(-s0.x, -s0.y);
    float v_len = length(v_in), s_len = length(s);
    if (v_len < (float)1e-5 || s_len < (float)1e-5) return v_in;
    V2 v_dir = v_in / v_len, s_dir = s / s_len;
    float misalign = rb_clamp(1.0f - dot(v_dir, s_dir), 0.0f, 2.0f);
    float t = rb_clamp(1.0f - rb_exp(-rb_max(P->slope_steer_rate, 0.0f) * misalign * dt), 0.0f, 1.0f);
    V2 dir_raw = v_dir + (s_dir - v_dir) * t;
    float dir_len = length(dir_raw);
    if (dir_len < (float)1e-5) return v_in;
    return (dir_raw / dir_len) * v_len;
  }

  // fluid.wgsl:191-231 (velocity_in is the buffer bound as input)
  V2 raw_velocity_cell(const V2* vin, uint32_t x, uint32_t y) const {
    if (is_solid(x, y)) return v2(0.0f, 0.0f);
    return sanitize(vin[fgrid(x, y)]);
  }
  V2 solid_normal_from_neighbors(uint32_t x, uint32_t y) const {
    uint32_t xm = x == 0u ? x : x - 1u;
    uint32_t xp = x + 1u >= (uint32_t)fw ? x : x + 1u;
    uint32_t ym = y == 0u ? y : y - 1u;
    uint32_t yp = y + 1u >= (uint32_t)fh ? y : y + 1u;
    bool hx0 = x > 0u, hx1 = x + 1u < (uint32_t)fw, hy0 = y > 0u, hy1 = y + 1u < (uint32_t)fh;
    float s_l = (hx0 && is_solid(xm, y)) ? 1.0f : 0.0f;
    float s_r = (hx1 && is_solid(xp, y)) ? 1.0f : 0.0f;
    float s_b = (hy0 && is_solid(x, ym)) ? 1.0f : 0.0f;
    float s_t = (hy1 && is_solid(x, yp)) ? 1.0f : 0.0f;
    float s_bl = (hx0 && hy0 && is_solid(xm, ym)) ? 1.0f : 0.0f;
    float s_tl = (hx0 && hy1 && is_solid(xm, yp)) ? 1.0f : 0.0f;
    float s_br = (hx1 && hy0 && is_solid(xp, ym)) ? 1.0f : 0.0f;
    float s_tr = (hx1 && hy1 && is_solid(xp, yp)) ? 1.0f : 0.0f;
    const float diag = (float)0.70710678;
    float nx = (s_l - s_r) + diag * ((s_bl + s_tl) - (s_br + s_tr));
    float ny = (s_b - s_t) + diag * ((s_bl + s_br) - (s_tl + s_tr));
    V2 n = v2(nx, ny);
    float n_len = length(n);
    return n_len > (float)1e-6 ? n / n_len : v2(0.0f, 0.0f);
  }
  V2 reflect_if_into_solid(uint32_t x, uint32_t y, V2 v_in) const {
    V2 n = solid_normal_from_neighbors(x, y);
    float d = dot(v_in, n);
    if (length(n) > (float)1e-6 && d < 0.0f) return v_in - n * d;
    return v_in;
  }
  bool is_solid_at_pos(V2 pos) const {
    int ix = rb_f2i(rb_floor(pos.x - 0.5f));
    int iy = rb_f2i(rb_floor(pos.y - 0.5f));
    if (ix < 0 || ix >= fw || iy < 0 || iy >= fh) return true;
    return is_solid((uint32_t)ix, (uint32_t)iy);
  }
  // fluid.wgsl:233-255
  V2 sample_velocity(const V2* vin, V2 pos) const {
    float max_x = (float)fw - 0.5f, max_y = (float)fh - 0.5f;
    if (pos.x < 0.5f || pos.x > max_x || pos.y < 0.5f || pos.y > max_y) return v2(0.0f, 0.0f);
    float x = pos.x - 0.5f, y = pos.y - 0.5f;
    int x0 = rb_f2i(rb_floor(x)), y0 = rb_f2i(rb_floor(y));
    float fx = rb_fract(x), fy = rb_fract(y);
    auto cx = [&](int v) { return (uint32_t)std::min(std::max(v, 0), fw - 1); };
    auto cy = [&](int v) { return (uint32_t)std::min(std::max(v, 0), fh - 1); };
    V2 v0 = mix2(raw_velocity_cell(vin, cx(x0), cy(y0)), raw_velocity_cell(vin, cx(x0 + 1), cy(y0)), fx);
    V2 v1 = mix2(raw_velocity_cell(vin, cx(x0), cy(y0 + 1)), raw_velocity_cell(vin, cx(x0 + 1), cy(y0 + 1)), fx);
    return mix2(v0, v1, fy);
  }
  // fluid.wgsl:260-273
  V2 fluid_velocity_at_world(const V2* vin, V2 pw) const {
    float gxf = (float)fw, gyf = (float)fh;
    float gx = rb_clamp(pw.x / sim_w * gxf, 0.5f, gxf - 0.5f) - 0.5f;
    float gy = rb_clamp(pw.y / sim_h * gyf, 0.5f, gyf - 0.5f) - 0.5f;
    uint32_t x0 = rb_f2u(rb_floor(gx)), y0 = rb_f2u(rb_floor(gy));
    uint32_t x1 = std::min(x0 + 1u, (uint32_t)fw - 1u), y1 = std::min(y0 + 1u, (uint32_t)fh - 1u);
    float tx = rb_fract(gx), ty = rb_fract(gy);
    V2 v0 = mix2(sanitize(vin[fgrid(x0, y0)]), sanitize(vin[fgrid(x1, y0)]), tx);
    V2 v1 = mix2(sanitize(vin[fgrid(x0, y1)]), sanitize(vin[fgrid(x1, y1)]), tx);
    return mix2(v0, v1, ty);
  }

  // ---- light helpers used by the temperature pass (light.wgsl:46-102,182-189) ----
  float light_above(uint32_t x, uint32_t row, uint32_t band) const {
    float sh = -P->sun_slope;
    int base = rb_f2i(rb_floor(sh));
    float f = sh - (float)base;
    float s = 0.0f;
    size_t bo = (size_t)band * lcells() + (size_t)row * lw;
    for (int d = 0; d < LIGHT_TAPS; d++) {
      int x0 = std::min(std::max((int)x + d - LIGHT_TAPS / 2 + base, 0), lw - 1);
      int x1 = std::min(std::max(x0 + 1, 0), lw - 1);
      s += rb_mix(light[bo + x0], light[bo + x1], f);
    }
    float cpos = (float)x + sh;
    float inside = rb_clamp(cpos + 1.0f, 0.0f, 1.0f) * rb_clamp((float)lw - cpos, 0.0f, 1.0f);
    return s / (float)LIGHT_TAPS * inside;
  }
  float light_transmit(uint32_t lx, uint32_t ly, uint32_t band) const {
    float g = 0.0f;
    uint32_t m = 0;
    for (uint32_t dy = 0; dy < LIGHT_DIV; dy++)
      for (uint32_t dx = 0; dx < LIGHT_DIV; dx++) {
        size_t c = (size_t)(ly * LIGHT_DIV + dy) * gw + lx * LIGHT_DIV + dx;
        g += (float)gamma_count(c);
        m += chem_cell_total(c);
      }
    g = g / (float)LIGHT_DIV;
    float dens = (float)m / (float)(LIGHT_DIV * LIGHT_DIV);
    float tau_m = rb_max(P->monomer_uv_absorb, 0.0f) * dens * (float)LIGHT_DIV / (float)gh * (band == 1u ? (float)0.35 : 1.0f);
    float sh = (float)shade[(size_t)band * lcells() + (size_t)ly * lw + lx] / SHADE_ONE;
    return rb_exp(-UV_SHADOW_ABSORB * g - AGENT_UV_ABSORB * sh - tau_m);
  }
  float light_absorbed_at(size_t env) const {
    uint32_t lx = (uint32_t)(env % gw) / LIGHT_DIV;
    uint32_t ly = (uint32_t)(env / gw) / LIGHT_DIV;
    float incoming = P->sun_now;
    if (ly + 1u < (uint32_t)lh) incoming = light_above(lx, ly + 1u, 0u);
    incoming = rb_max(incoming, 0.0f);
    return incoming * ((1.0f - light_transmit(lx, ly, 0u)) + SUN_WATER_ABSORB);
  }
  // ---- the light block (light.wgsl:43-45, 141-177; src/world/mod.rs:1505-1524) ----
  float row_water(uint32_t band) const {
    return rb_exp(-rb_max(P->uv_depth, 0.0f) * (band == 1u ? (float)0.03 : 1.0f) * (float)LIGHT_DIV / (float)gh);
  }
  void light_transmit_pass() {
    const size_t L = lcells();
    std::vector<float> t0(L), t1(L);  // every transmission reads chem, gamma and shade only
    for (int y = 0; y < lh; y++)
      for (int x = 0; x < lw; x++) {
        t0[(size_t)y * lw + x] = light_transmit(x, y, 0u);
        t1[(size_t)y * lw + x] = light_transmit(x, y, 1u);
      }
    std::copy(t0.begin(), t0.end(), light.begin());
    std::copy(t1.begin(), t1.end(), light.begin() + L);
  }
  void compute_uv_light() {
    const size_t L = lcells();
    const uint32_t top = (uint32_t)lh - 1u;
    const float w0 = row_water(0u), w1 = row_water(1u);
    for (int x = 0; x < lw; x++) {
      light[(size_t)top * lw + x] *= w0 * P->sun_now;
      light[L + (size_t)top * lw + x] *= w1 * P->sun_now;
    }
    for (uint32_t t = 1; t < (uint32_t)lh; t++) {
      const uint32_t y = (uint32_t)lh - 1u - t;
      for (int x = 0; x < lw; x++) {
        const float a0 = light_above(x, y + 1u, 0u), a1 = light_above(x, y + 1u, 1u);
        light[(size_t)y * lw + x] *= a0 * w0;
        light[L + (size_t)y * lw + x] *= a1 * w1;
      }
    }
  }
  void light_propagate() {
    const size_t L = lcells();
    for (int y = 0; y < lh; y++)
      for (int x = 0; x < lw; x++)
        for (uint32_t band = 0; band < 2u; band++) {
          float above = P->sun_now;
          if ((uint32_t)y + 1u < (uint32_t)lh) above = light_above(x, y + 1u, band);
          light_next[band * L + (size_t)y * lw + x] = above * row_water(band) * light_transmit(x, y, band);
        }
  }
  void light_commit() { light = light_next; }
  void light_block(uint32_t epoch) {
    const uint32_t interval = std::max(st.light_interval, 1u);
    if (light_dirty || (st.light_rows_per_step == 0u && epoch % interval == 0u)) {
      light_dirty = false;
      light_transmit_pass();
      compute_uv_light();
    } else {
      for (uint32_t r = 0; r < std::min(st.light_rows_per_step, 16u); r++) {
        light_propagate();
        light_commit();
      }
    }
  }

  float uv_light_at_cell(uint32_t x, uint32_t y) const {
    uint32_t lx = std::min(x, (uint32_t)gw - 1u) / LIGHT_DIV;
    uint32_t ly = std::min(y, (uint32_t)gh - 1u) / LIGHT_DIV;
    return light[(size_t)ly * lw + lx];
  }

  // ===================== passes =====================

  // terrain.wgsl:104-133 (compute_gamma_slope)
  void compute_slope() {
    auto h = [&](int ix, int iy) {
      int x = std::min(std::max(ix, 0), gw - 1), y = std::min(std::max(iy, 0), gh - 1);
      return (float)gamma[(size_t)y * gw + x] * GAMMA_QUANTUM;
    };
#pragma omp parallel for schedule(static)
    for (int y = 0; y < gh; y++)
      for (int x = 0; x < gw; x++) {
        float l = h(x - 1, y), r = h(x + 1, y), b = h(x, y - 1), t = h(x, y + 1);
        float bl = h(x - 1, y - 1), br = h(x + 1, y - 1), tl = h(x - 1, y + 1), tr = h(x + 1, y + 1);
        const float k = (float)(1.0 / (4.0 * 1.41421356237));
        float dx = (r - l) * 0.5f + (tr + br - tl - bl) * k;
        float dy = (t - b) * 0.5f + (tl + tr - bl - br) * k;
        float u = (float)cfg.world_units_per_cell;
        slope[(size_t)y * gw + x] = v2(dx / u, dy / u);
      }
  }

  // ---- terrain grains (shaders/world/terrain.wgsl:36-460) ----
  //
  // The reference runs these passes with in-place atomics: every cell's
  // thread reads its neighbours' live grain counts while other threads move
  // grains and evict monomers, so a GPU run has no single result.  The oracle
  // executes ONE legal serialization of that program, the one the CUDA
  // kernels reproduce exactly:
  //  relax pass: every thread's decision reads (all grain counts read
  //    before any move); then every take and add of a grain; then the
  //    eviction loops of the moved grains' destinations, in nine classes
  //    (x mod 3, y mod 3) of the destination, ascending destination index in
  //    a class, the arrivals at one destination by ascending source index;
  //  grain_fall: the columns in three classes (x mod 3), each column's loop
  //    run whole, ascending x in a class;
  //  paint: every store, then the eviction loops in the nine classes.
  // Destinations of one class are >= 3 cells apart and an eviction loop only
  // touches cells within one cell of its destination, so the order inside a
  // class changes nothing: the GPU runs a class in parallel.

  // transport.wgsl:54-58
  float parcel_hop_p(V2 v) const {
    const float env_per_fluid = (float)gw / (float)fw;
    const float l1 = rb_abs(v.x) + rb_abs(v.y);
    return rb_clamp(l1 * env_per_fluid * rb_max(P->dt, (float)1e-3), 0.0f, GRAIN_ADV_CAP);
  }
  // terrain.wgsl:24-28
  V2 fluid_vel_at_cell(uint32_t cx, uint32_t cy) const {
    uint32_t fx = std::min(cx * (uint32_t)fw / (uint32_t)gw, (uint32_t)fw - 1u);
    uint32_t fy = std::min(cy * (uint32_t)fh / (uint32_t)gh, (uint32_t)fh - 1u);
    return sanitize(vel_a[fgrid(fx, fy)]);
  }
  // terrain.wgsl:54-72
  size_t evict_target(size_t src, size_t dst) const {
    if (chem_cell_total(src) < chem_capacity(src)) return src;
    const int x = (int)(dst % gw), y = (int)(dst / gw);
    const int nx[4] = {x + 1, x - 1, x, x}, ny[4] = {y, y, y + 1, y - 1};
    size_t not_rock = gamma_count(src) < GAMMA_SOLID ? src : NO_CELL;
    for (int k = 0; k < 4; k++) {
      if (nx[k] < 0 || ny[k] < 0 || nx[k] >= gw || ny[k] >= gh) continue;
      size_t n = (size_t)ny[k] * gw + nx[k];
      if (chem_cell_total(n) < chem_capacity(n)) return n;
      if (not_rock == NO_CELL && gamma_count(n) < GAMMA_SOLID) not_rock = n;
    }
    return not_rock == NO_CELL ? src : not_rock;
  }
  // The eviction loop of gamma_move_one (terrain.wgsl:82-100) and of
  // paint_terrain (:396-412, src == dst): one monomer per round, the spent
  // state of a channel before its activated state, channels in order.
  void evict(size_t src, size_t dst) {
    const uint32_t cap = chem_capacity(dst);
    for (int guard = 0; guard < 64; guard++) {
      if (chem_cell_total(dst) <= cap) break;
      const size_t to = evict_target(src, dst);
      if (to == dst) break;
      bool moved = false;
      for (int c = 0; c < 4 && !moved; c++) {
        uint32_t& v = chem[dst * 4 + c];
        if ((v >> 16) != 0u) {
          v -= CHEM_SPENT_ONE;
          chem[to * 4 + c] += CHEM_SPENT_ONE;
          moved = true;
        } else if ((v & CHEM_STATE_MASK) != 0u) {
          v -= 1u;
          chem[to * 4 + c] += 1u;
          moved = true;
        }
      }
      if (!moved) break;
    }
  }
  // terrain.wgsl:137-159
  bool compaction_stable(size_t src, size_t dst, uint32_t n, uint32_t c) const {
    const int dx4[4] = {1, -1, 0, 0}, dy4[4] = {0, 0, 1, -1};
    const int xd = (int)(dst % gw), yd = (int)(dst / gw), xs = (int)(src % gw), ys = (int)(src / gw);
    bool ok = true;
    for (int k = 0; k < 4; k++) {
      int qx = xd + dx4[k], qy = yd + dy4[k];
      if (qx >= 0 && qy >= 0 && qx < gw && qy < gh) {
        size_t qi = (size_t)qy * gw + qx;
        uint32_t low = qi == src ? n - 1u : gamma_count(qi);
        if (c + 1u >= low + SANDPILE_DIFF) ok = false;
      }
      qx = xs + dx4[k];
      qy = ys + dy4[k];
      if (qx >= 0 && qy >= 0 && qx < gw && qy < gh) {
        size_t qi = (size_t)qy * gw + qx;
        uint32_t high = qi == dst ? c + 1u : gamma_count(qi);
        if (high >= n - 1u + SANDPILE_DIFF) ok = false;
      }
    }
    return ok;
  }
  // terrain.wgsl:161-372 (relax_gamma_pass), the decision of one cell from
  // the grain counts as they are: the destination of its grain, or idx.
  size_t relax_decide(size_t idx, uint32_t phase) const {
    const int x = (int)(idx % gw), y = (int)(idx / gw);
    const uint32_t n = gamma_count(idx);
    if (n == 0u) return idx;
    if (n < SANDPILE_DIFF) {
      // loose grains
      uint32_t bonds = 0u, best_c = 0xFFFFu, comp_c = 0u;
      int best_score = -1, em_score = -1;
      size_t best = idx, em = idx, comp = idx;
      bool em_found = false;
      const rb_u4 rr = rb_pcg4d((uint32_t)idx, P->epoch, RB_S_RELAX + phase, P->seed);
      uint32_t tie = rr.x;
      const float comp_roll = (float)(rb_hash32(rr.x ^ 0x5bd1e995u) >> 8) * (1.0f / 16777216.0f);
      const bool try_comp = comp_roll < P->sediment_compaction;
      for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++) {
          if (dx == 0 && dy == 0) continue;
          const int nx = x + dx, ny = y + dy;
          if (nx < 0 || ny < 0 || nx >= gw || ny >= gh) continue;
          const size_t ni = (size_t)ny * gw + nx;
          const uint32_t c = gamma_count(ni);
          if (c >= 1u) bonds++;
          if (try_comp && c >= 1u && c < GAMMA_ROCK_FULL &&
              (c > comp_c || (c == comp_c && (rb_hash32(tie ^ ((uint32_t)ni * 31u)) & 1u) == 1u)) &&
              compaction_stable(idx, ni, n, c)) {
            comp_c = c;
            comp = ni;
          }
          if (c <= n) {
            int score = 0;
            for (int sy = -1; sy <= 1; sy++)
              for (int sx = -1; sx <= 1; sx++) {
                if (sx == 0 && sy == 0) continue;
                const int qx = nx + sx, qy = ny + sy;
                if (qx < 0 || qy < 0 || qx >= gw || qy >= gh) continue;
                const size_t qi = (size_t)qy * gw + qx;
                if (qi == idx) continue;
                if (gamma_count(qi) >= 1u) score++;
              }
            tie = rb_hash32(tie ^ (uint32_t)ni);
            if (score > best_score || (score == best_score && c < best_c) ||
                (score == best_score && c == best_c && (tie & 1u) == 1u)) {
              best_score = score;
              best_c = c;
              best = ni;
            }
            if (c == 0u && (score > em_score || (score == em_score && (tie & 2u) == 2u))) {
              em_score = score;
              em = ni;
              em_found = true;
            }
          }
        }
      // pow(0.25, bonds): 2^(-2 bonds) is exact in f32 for bonds <= 8
      const float mob = ldexpf(1.0f, -2 * (int)bonds);
      if (try_comp && bonds >= 3u && comp != idx &&
          comp_roll < P->sediment_compaction * (float)(bonds - 2u) / 6.0f)
        return comp;
      V2 vs = v2(0.0f, 0.0f);
      if (P->fluid_enabled != 0u) {
        const int dx4[4] = {1, -1, 0, 0}, dy4[4] = {0, 0, 1, -1};
        for (int k = 0; k < 4; k++) {
          const int qx = x + dx4[k], qy = y + dy4[k];
          if (qx < 0 || qy < 0 || qx >= gw || qy >= gh) continue;
          if (gamma_count((size_t)qy * gw + qx) != 0u) continue;
          const V2 v = fluid_vel_at_cell((uint32_t)qx, (uint32_t)qy);
          if (dot(v, v) > dot(vs, vs)) vs = v;
        }
      }
      const bool unsupported = y > 0 && gamma_count(idx - gw) == 0u;
      V2 v_move = v2(0.0f, 0.0f);
      float p_sed = 0.0f;
      if (unsupported && bonds == 0u) {
        v_move = vs;
        p_sed = parcel_hop_p(v_move);
      } else {
        const float speed = length(vs);
        const float crit = rb_max(P->sediment_threshold, 0.0f) * (1.0f + rb_max(P->sediment_cohesion, 0.0f) * (float)bonds);
        const float excess = rb_max(speed - crit, 0.0f);
        v_move = speed > (float)1e-6 ? vs * (excess / rb_max(speed, (float)1e-6)) : v2(0.0f, 0.0f);
        p_sed = parcel_hop_p(v_move) * GAMMA_SEDIMENT_FACTOR * rb_max(P->sediment_transport, 0.0f);
      }
      const uint32_t hfx = std::min((uint32_t)x * (uint32_t)fw / (uint32_t)gw, (uint32_t)fw - 1u);
      const uint32_t hfy = std::min((uint32_t)y * (uint32_t)fh / (uint32_t)gh, (uint32_t)fh - 1u);
      const V2 vent = heat[fgrid(hfx, hfy)];
      const float blow = VENT_BLOW * rb_max(vent.x, vent.y);
      if (blow > 0.0f) {
        v_move = v2((rr.y & 1u) == 1u ? (float)0.6 : (float)-0.6, 1.0f) * blow;
        p_sed = rb_max(p_sed, parcel_hop_p(v_move));
      }
      if (bonds >= 4u && p_sed <= 0.0f) return idx;
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
        const int wx = x + ddx, wy = y + ddy;
        if (wx >= 0 && wy >= 0 && wx < gw && wy < gh) {
          const size_t wi = (size_t)wy * gw + wx;
          if (gamma_count(wi) <= n) return wi;
        }
        return idx;
      }
      if (rw < p_sed + GAMMA_STRAY_WALK_P * mob) {
        if (best_score > (int)bonds) return best;
        if (bonds == 0u) {
          static const int wdx[8] = {1, -1, 0, 0, 1, -1, 1, -1}, wdy[8] = {0, 0, 1, -1, 1, 1, -1, -1};
          const uint32_t k = (hw >> 8) % 8u;
          const int wx = x + wdx[k], wy = y + wdy[k];
          if (wx >= 0 && wy >= 0 && wx < gw && wy < gh) {
            const size_t wi = (size_t)wy * gw + wx;
            if (gamma_count(wi) <= n) return wi;
          }
        }
      }
      return idx;
    }
    // sandpile: slide towards the lowest of the four neighbours
    size_t best = idx;
    uint32_t best_c = n;
    if (x > 0 && gamma_count(idx - 1) < best_c) { best_c = gamma_count(idx - 1); best = idx - 1; }
    if (x + 1 < gw && gamma_count(idx + 1) < best_c) { best_c = gamma_count(idx + 1); best = idx + 1; }
    if (y > 0 && gamma_count(idx - gw) < best_c) { best_c = gamma_count(idx - gw); best = idx - gw; }
    if (y + 1 < gh && gamma_count(idx + gw) < best_c) { best_c = gamma_count(idx + gw); best = idx + gw; }
    if (best == idx || n - best_c < SANDPILE_DIFF) return idx;
    const float p = GAMMA_RELAX_P * rb_max(rb_clamp(P->sediment_settle, 0.0f, 1.0f), rb_clamp(P->rock_crumble, 0.0f, 1.0f));
    if (rb_u2f(rb_pcg4d((uint32_t)idx, P->epoch, RB_S_SAND + phase, P->seed).x) < p) return best;
    return idx;
  }
  static int cell_class(int x, int y) { return x % 3 + 3 * (y % 3); }
  // relax_gamma_a / relax_gamma_b (terrain.wgsl:449-459) in the order above
  void relax_pass(uint32_t phase) {
    const size_t C = cells();
    std::vector<size_t> dest(C);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)C; i++) dest[i] = relax_decide((size_t)i, phase);
    std::vector<uint8_t> arrived(C, 0);
    for (size_t i = 0; i < C; i++)
      if (dest[i] != i) {
        gamma[i] -= 1u;
        gamma[dest[i]] += 1u;
        arrived[dest[i]] = 1;
      }
    for (int cls = 0; cls < 9; cls++)
      for (int y = cls / 3; y < gh; y += 3)
        for (int x = cls % 3; x < gw; x += 3) {
          const size_t dst = (size_t)y * gw + x;
          if (!arrived[dst]) continue;
          for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++) {
              const int sx = x + dx, sy = y + dy;
              if ((dx == 0 && dy == 0) || sx < 0 || sy < 0 || sx >= gw || sy >= gh) continue;
              const size_t src = (size_t)sy * gw + sx;
              if (dest[src] == dst) evict(src, dst);
            }
        }
  }
  // terrain.wgsl:425-446 (grain_fall)
  void grain_fall() {
    const float w_s = GAMMA_SETTLE_SPEED * rb_max(P->sediment_settle, 0.0f);
    const float rate = parcel_hop_p(v2(0.0f, w_s));
    if (rate <= 0.0f) return;
    const uint32_t rf = rb_f2u(rate * 65536.0f);
    if (((P->epoch * rf) >> 16) == (((P->epoch + 1u) * rf) >> 16)) return;
    for (int cls = 0; cls < 3; cls++)
      for (int x = cls; x < gw; x += 3) {
        bool supported = true;
        for (int y = 0; y < gh; y++) {
          const size_t idx = (size_t)y * gw + x;
          const uint32_t n = gamma_count(idx);
          if (n == 0u) {
            supported = false;
            continue;
          }
          if (n >= GAMMA_SOLID) {
            supported = true;
            continue;
          }
          if (supported) continue;
          for (uint32_t k = 0; k < n; k++) {
            gamma[idx] -= 1u;
            gamma[idx - gw] += 1u;
            evict(idx, idx - gw);
          }
        }
      }
  }
  // World::encode_paint (src/world/mod.rs:1220-1241), paint_terrain (terrain.wgsl:390-413)
  void paint(float cx, float cy, float radius, uint32_t grains) {
    const uint32_t want = std::min(grains, 6u);
    std::vector<uint8_t> painted(cells(), 0);
    for (int y = 0; y < gh; y++)
      for (int x = 0; x < gw; x++) {
        const float ex = (float)x + 0.5f - cx, ey = (float)y + 0.5f - cy;
        if (ex * ex + ey * ey > radius * radius) continue;
        gamma[(size_t)y * gw + x] = want;
        painted[(size_t)y * gw + x] = 1;
      }
    for (int cls = 0; cls < 9; cls++)
      for (int y = cls / 3; y < gh; y += 3)
        for (int x = cls % 3; x < gw; x += 3) {
          const size_t i = (size_t)y * gw + x;
          if (painted[i]) evict(i, i);
        }
    compute_slope();
    build_solid_mask();
    light_dirty = true;
  }
  // src/world/mod.rs:1497-1504: relax a, relax b, grain_fall when grains
  // settle, then the slope
  void terrain_block() {
    relax_pass(0u);
    relax_pass(1u);
    if (P->sediment_settle > 0.0f) grain_fall();
    compute_slope();
  }

  // fluid.wgsl:185-189
  void build_solid_mask() {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < fh; y++)
      for (int x = 0; x < fw; x++) solid_mask[fgrid(x, y)] = permeability(x, y) < SOLID_PERM_THRESHOLD ? 1u : 0u;
  }

  // fluid.wgsl:300-363 (temp_in/redox_in -> temp_out/redox_out; velocity_in = a)
  void update_temperature() {
    const float dt = fluid_dt();
    const V2* vin = vel_a.data();
    const bool sun = rb_max(P->sun_heat, 0.0f) > 0.0f;  // the sun term is exactly 0 otherwise
#pragma omp parallel for schedule(static)
    for (int yi = 0; yi < fh; yi++)
      for (int xi = 0; xi < fw; xi++) {
        uint32_t x = xi, y = yi;
        size_t idx = fgrid(x, y);
        V2 vel = raw_velocity_cell(vin, x, y);
        V2 src = v2((float)x + 0.5f, (float)y + 0.5f) - vel * dt;
        float sxf = rb_clamp(src.x - 0.5f, 0.0f, (float)(fw - 1));
        float syf = rb_clamp(src.y - 0.5f, 0.0f, (float)(fh - 1));
        uint32_t x0 = rb_f2u(rb_floor(sxf)), y0 = rb_f2u(rb_floor(syf));
        uint32_t x1 = std::min(x0 + 1u, (uint32_t)fw - 1u), y1 = std::min(y0 + 1u, (uint32_t)fh - 1u);
        float fx = rb_fract(sxf), fy = rb_fract(syf);
        const float* T = temp_a.data();
        float t = rb_mix(rb_mix(T[fgrid(x0, y0)], T[fgrid(x1, y0)], fx), rb_mix(T[fgrid(x0, y1)], T[fgrid(x1, y1)], fx), fy);
        uint32_t xl = (uint32_t)std::max((int)x - 1, 0), xr = std::min(x + 1u, (uint32_t)fw - 1u);
        uint32_t yb = (uint32_t)std::max((int)y - 1, 0), yt = std::min(y + 1u, (uint32_t)fh - 1u);
        float tl = T[fgrid(xl, y)], tr = T[fgrid(xr, y)], tb = T[fgrid(x, yb)], tt = T[fgrid(x, yt)];
        float fill = gamma_fill_at_fluid_cell(x, y);
        t = rb_mix(t, (tl + tr + tb + tt) * 0.25f, TEMP_DIFFUSE * rb_mix(1.0f, TEMP_ROCK_CONDUCT, fill));
        float vc = vent_cycle(x);
        t += heat[idx].x * vc * TEMP_HEAT_RATE * dt;
        if (sun) {
          size_t env = env_cell_for_fluid(x, y);
          float depth = 1.0f - ((float)y + 0.5f) / (float)fh;
          float ir = P->sun_now * SUN_IR * rb_exp(-depth / SUN_IR_DEPTH);
          t += rb_max(P->sun_heat, 0.0f) * SUN_HEAT_RATE * (light_absorbed_at(env) + ir) * dt;
        }
        float amb = temp_ambient_at(y);
        t = amb + (t - amb) * rb_exp(-TEMP_COOL_RATE * (1.0f - fill) * dt);
        temp_b[idx] = rb_clamp(t, 0.0f, TEMP_MAX);

        const float* R = redox_a.data();
        float r = rb_mix(rb_mix(R[fgrid(x0, y0)], R[fgrid(x1, y0)], fx), rb_mix(R[fgrid(x0, y1)], R[fgrid(x1, y1)], fx), fy);
        float rl = R[fgrid(xl, y)], rr = R[fgrid(xr, y)], rb = R[fgrid(x, yb)], rt = R[fgrid(x, yt)];
        r = rb_mix(r, (rl + rr + rb + rt) * 0.25f, TEMP_DIFFUSE);
        r += heat[idx].y * vc * REDOX_RATE * dt;
        r = rb_max(r - (float)redox_eaten[idx] / REDOX_FP, 0.0f);
        r *= rb_exp(-rb_max(P->redox_decay, 0.0f) * dt);
        redox_b[idx] = rb_clamp(r, 0.0f, REDOX_MAX);
      }
  }

  // fluid.wgsl:365-372
  void copy_temperature() {
    temp_a = temp_b;
    redox_a = redox_b;
    std::fill(redox_eaten.begin(), redox_eaten.end(), 0u);
  }

  // fluid.wgsl:280-296, 376-398
  void atomic_add_force(size_t i, float v) {
    int32_t q = rb_f2i(rb_rint(rb_clamp(v, (float)-1.0e5, (float)1.0e5) * FORCE_FP));
    if (q != 0) force_vec[i] += (uint32_t)q;
  }
  void buoyancy() {
#pragma omp parallel for schedule(static)
    for (int y = 1; y < fh - 1; y++)
      for (int x = 1; x < fw - 1; x++) {
        size_t idx = fgrid(x, y);
        float dev = temp_a[idx] - temp_ambient_at(y);
        if (rb_abs(dev) <= (float)1e-3) continue;
        uint32_t time_bucket = P->epoch / 16u;
        float r = rb_u2f(rb_pcg4d((uint32_t)idx, time_bucket, RB_S_BUOYANCY, P->seed).x);
        float side = (r * 2.0f - 1.0f) * 0.25f * rb_abs(dev) / rb_max(rb_abs(dev), 1.0f);
        V2 f = v2(side * TEMP_BUOYANCY * rb_abs(dev), TEMP_BUOYANCY * dev);
        atomic_add_force(idx * 2, f.x);
        atomic_add_force(idx * 2 + 1, f.y);
      }
  }
  void gather_forces() {
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)fcells(); i++) {
      V2 f = v2((float)(int32_t)force_vec[i * 2] / FORCE_FP, (float)(int32_t)force_vec[i * 2 + 1] / FORCE_FP);
      fluid_forces[i] = clamp_len(sanitize(f), MAX_FORCE);
    }
  }
  void clear_force_vectors() { std::fill(force_vec.begin(), force_vec.end(), 0u); }
  void clear_forces() { std::fill(fluid_forces.begin(), fluid_forces.end(), v2(0.0f, 0.0f)); }

  // fluid.wgsl:410-432
  void add_forces(const V2* vin, V2* vout) {
    const float dt = fluid_dt();
#pragma omp parallel for schedule(static)
    for (int yi = 0; yi < fh; yi++)
      for (int xi = 0; xi < fw; xi++) {
        uint32_t x = xi, y = yi;
        size_t idx = fgrid(x, y);
        if (is_solid(x, y)) {
          vout[idx] = v2(0.0f, 0.0f);
          continue;
        }
        uint32_t xm = x > 0u ? x - 1u : x, xp = x + 1u < (uint32_t)fw ? x + 1u : x;
        uint32_t ym = y > 0u ? y - 1u : y, yp = y + 1u < (uint32_t)fh ? y + 1u : y;
        auto F = [&](uint32_t a, uint32_t b) { return sanitize(fluid_forces[fgrid(a, b)]); };
        V2 f_c = F(x, y);
        V2 f_avg = (4.0f * (F(xm, y) + F(xp, y) + F(x, ym) + F(x, yp)) + (F(xm, ym) + F(xp, ym) + F(xm, yp) + F(xp, yp)) +
                    20.0f * f_c) *
                   (float)(1.0 / 36.0);
        V2 f_user = clamp_len(mix2(f_c, f_avg, FORCE_SMOOTH_MIX), MAX_FORCE);
        V2 v = sanitize(sanitize(vin[idx]) + f_user * dt);
        v = slope_steer_velocity(x, y, v, dt);
        v = v * rubble_drag(x, y, dt);
        v = reflect_if_into_solid(x, y, v);
        vout[idx] = clamp_len(v, MAX_VEL);
      }
  }

  // fluid.wgsl:435-456
  void diffuse_velocity(const V2* vin, V2* vout) {
#pragma omp parallel for schedule(static)
    for (int yi = 0; yi < fh; yi++)
      for (int xi = 0; xi < fw; xi++) {
        uint32_t x = xi, y = yi;
        size_t idx = fgrid(x, y);
        if (is_solid(x, y)) {
          vout[idx] = v2(0.0f, 0.0f);
          continue;
        }
        if (x == 0u || x == (uint32_t)fw - 1u || y == 0u || y == (uint32_t)fh - 1u) {
          vout[idx] = vin[idx];
          continue;
        }
        V2 v_c = raw_velocity_cell(vin, x, y);
        V2 axis_sum = raw_velocity_cell(vin, x - 1, y) + raw_velocity_cell(vin, x + 1, y) + raw_velocity_cell(vin, x, y - 1) +
                      raw_velocity_cell(vin, x, y + 1);
        V2 diag_sum = raw_velocity_cell(vin, x - 1, y - 1) + raw_velocity_cell(vin, x + 1, y - 1) +
                      raw_velocity_cell(vin, x - 1, y + 1) + raw_velocity_cell(vin, x + 1, y + 1);
        V2 lap = (4.0f * axis_sum + diag_sum - 20.0f * v_c) * (float)(1.0 / 6.0);
        float a = rb_max(P->fluid_viscosity, 0.0f) * fluid_dt();
        V2 v = sanitize(v_c + a * lap);
        v = reflect_if_into_solid(x, y, v);
        vout[idx] = clamp_len(v, MAX_VEL);
      }
  }

  // fluid.wgsl:458-477
  void advect_velocity(const V2* vin, V2* vout) {
    const float dt = fluid_dt();
    const float decay_factor = rb_pow(rb_clamp(P->fluid_decay, 0.0f, 1.0f), dt * 60.0f);
#pragma omp parallel for schedule(static)
    for (int yi = 0; yi < fh; yi++)
      for (int xi = 0; xi < fw; xi++) {
        uint32_t x = xi, y = yi;
        size_t idx = fgrid(x, y);
        if (is_solid(x, y)) {
          vout[idx] = v2(0.0f, 0.0f);
          continue;
        }
        V2 pos = v2((float)x + 0.5f, (float)y + 0.5f);
        V2 vel = reflect_if_into_solid(x, y, clamp_len(raw_velocity_cell(vin, x, y), MAX_VEL));
        V2 trace_pos = pos - vel * dt;
        if (is_solid_at_pos(trace_pos)) trace_pos = pos - reflect_if_into_solid(x, y, vel) * dt;
        V2 out_v = sanitize(sample_velocity(vin, trace_pos) * decay_factor);
        out_v = reflect_if_into_solid(x, y, out_v);
        vout[idx] = clamp_len(out_v, MAX_VEL);
      }
  }

  // fluid.wgsl:479-518
  float curl_at(const V2* vin, uint32_t x, uint32_t y) const {
    uint32_t xm = (uint32_t)std::min(std::max((int)x - 1, 0), fw - 1);
    uint32_t xp = (uint32_t)std::min(std::max((int)x + 1, 0), fw - 1);
    uint32_t ym = (uint32_t)std::min(std::max((int)y - 1, 0), fh - 1);
    uint32_t yp = (uint32_t)std::min(std::max((int)y + 1, 0), fh - 1);
    V2 v_l = reflect_if_into_solid(xm, y, raw_velocity_cell(vin, xm, y));
    V2 v_r = reflect_if_into_solid(xp, y, raw_velocity_cell(vin, xp, y));
    V2 v_b = reflect_if_into_solid(x, ym, raw_velocity_cell(vin, x, ym));
    V2 v_t = reflect_if_into_solid(x, yp, raw_velocity_cell(vin, x, yp));
    return 0.5f * (v_r.y - v_l.y) - 0.5f * (v_t.x - v_b.x);
  }
  void vorticity_confinement(const V2* vin, V2* vout) {
    const float epsilon = rb_clamp(P->fluid_vorticity, 0.0f, 10.0f);
#pragma omp parallel for schedule(static)
    for (int yi = 0; yi < fh; yi++)
      for (int xi = 0; xi < fw; xi++) {
        uint32_t x = xi, y = yi;
        size_t idx = fgrid(x, y);
        if (is_solid(x, y)) {
          vout[idx] = v2(0.0f, 0.0f);
          continue;
        }
        const uint32_t border = 2u;
        if (x < border || x >= (uint32_t)fw - border || y < border || y >= (uint32_t)fh - border || epsilon < (float)1e-6) {
          vout[idx] = vin[idx];
          continue;
        }
        float w = curl_at(vin, x, y);
        if (rb_abs(w) < (float)5e-4) {
          vout[idx] = vin[idx];
          continue;
        }
        V2 grad = v2(rb_abs(curl_at(vin, x + 1, y)) - rb_abs(curl_at(vin, x - 1, y)),
                     rb_abs(curl_at(vin, x, y + 1)) - rb_abs(curl_at(vin, x, y - 1))) *
                  0.5f;
        V2 n = grad / rb_max(length(grad), (float)1e-5);
        V2 f = v2(n.y, -n.x) * (w * epsilon);
        V2 dv = clamp_len(f * fluid_dt(), 2.0f);
        V2 v = sanitize(vin[idx] + dv);
        v = reflect_if_into_solid(x, y, v);
        vout[idx] = clamp_len(v, MAX_VEL);
      }
  }

  // fluid.wgsl:520-551
  V2 div_neighbor(const V2* vin, V2 v_c, int nx, int ny, bool axis_x) const {
    bool outside = nx < 0 || ny < 0 || nx >= fw || ny >= fh;
    if (outside || is_solid((uint32_t)nx, (uint32_t)ny)) return axis_x ? v2(-v_c.x, v_c.y) : v2(v_c.x, -v_c.y);
    return raw_velocity_cell(vin, nx, ny);
  }
  void compute_divergence(const V2* vin) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < fh; y++)
      for (int x = 0; x < fw; x++) {
        size_t idx = fgrid(x, y);
        if (is_solid(x, y)) {
          div[idx] = 0.0f;
          continue;
        }
        V2 v_c = raw_velocity_cell(vin, x, y);
        V2 v_l = div_neighbor(vin, v_c, x - 1, y, true);
        V2 v_r = div_neighbor(vin, v_c, x + 1, y, true);
        V2 v_b = div_neighbor(vin, v_c, x, y - 1, false);
        V2 v_t = div_neighbor(vin, v_c, x, y + 1, false);
        div[idx] = 0.5f * ((v_r.x - v_l.x) + (v_t.y - v_b.y));
      }
  }

  // ---- multigrid (shaders/world/multigrid.wgsl; levels src/world/mod.rs:637-671) ----
  void setup_levels() {
    levels.clear();
    uint32_t mn = cfg.mg_min_size;
    int nx = fw, ny = fh;
    size_t off = 0;
    int l = 0;
    for (;;) {
      levels.push_back(Level{nx, ny, off, MG_EPS * (float)(1u << l)});
      off += (size_t)nx * ny;
      if ((uint32_t)nx > mn && (uint32_t)ny > mn && nx % 2 == 0 && ny % 2 == 0) {
        nx /= 2;
        ny /= 2;
        l++;
      } else {
        break;
      }
    }
    mg_p.assign(off, 0.0f);
    mg_rhs.assign(off, 0.0f);
    mg_fluid.assign(off, 0u);
  }
  bool mg_is_fluid(const Level& L, int x, int y) const {
    if (x < 0 || y < 0 || x >= L.nx || y >= L.ny) return false;
    return mg_fluid[L.off + (size_t)y * L.nx + x] != 0u;
  }
  V2 mg_neighbors(const Level& L, int x, int y) const {
    float s = 0.0f, k = 0.0f;
    const float* p = mg_p.data() + L.off;
    if (mg_is_fluid(L, x - 1, y)) { s += p[(size_t)y * L.nx + x - 1]; k += 1.0f; }
    if (mg_is_fluid(L, x + 1, y)) { s += p[(size_t)y * L.nx + x + 1]; k += 1.0f; }
    if (mg_is_fluid(L, x, y - 1)) { s += p[(size_t)(y - 1) * L.nx + x]; k += 1.0f; }
    if (mg_is_fluid(L, x, y + 1)) { s += p[(size_t)(y + 1) * L.nx + x]; k += 1.0f; }
    return v2(s, k);
  }
  void mg_init() {
    const Level& L = levels[0];
#pragma omp parallel for schedule(static)
    for (int y = 0; y < L.ny; y++)
      for (int x = 0; x < L.nx; x++) {
        size_t i = L.off + (size_t)y * L.nx + x, f = fgrid(x, y);
        bool fluid = !is_solid(x, y);
        mg_fluid[i] = fluid ? 1u : 0u;
        mg_rhs[i] = fluid ? div[f] : 0.0f;
        mg_p[i] = fluid ? pressure_a[f] : 0.0f;
      }
  }
  void mg_smooth(int l, uint32_t color) {
    const Level& L = levels[l];
#pragma omp parallel for schedule(static)
    for (int y = 0; y < L.ny; y++)
      for (int x = 0; x < L.nx; x++) {
        if ((((uint32_t)x + (uint32_t)y) & 1u) != color) continue;
        size_t i = L.off + (size_t)y * L.nx + x;
        if (mg_fluid[i] == 0u) continue;
        V2 nb = mg_neighbors(L, x, y);
        mg_p[i] = (nb.x - mg_rhs[i]) / (nb.y + L.eps);
      }
  }
  void mg_restrict(int l) {
    const Level& L = levels[l];
    const Level& C = levels[l + 1];
#pragma omp parallel for schedule(static)
    for (int cy = 0; cy < C.ny; cy++)
      for (int cx = 0; cx < C.nx; cx++) {
        float sum = 0.0f;
        uint32_t nf = 0;
        for (uint32_t c = 0; c < 4; c++) {
          int fx = cx * 2 + (int)(c & 1u), fy = cy * 2 + (int)(c >> 1);
          size_t i = L.off + (size_t)fy * L.nx + fx;
          if (mg_fluid[i] == 0u) continue;
          V2 nb = mg_neighbors(L, fx, fy);
          sum += mg_rhs[i] - (nb.x - (nb.y + L.eps) * mg_p[i]);
          nf++;
        }
        size_t ci = C.off + (size_t)cy * C.nx + cx;
        mg_fluid[ci] = nf > 0u ? 1u : 0u;
        mg_rhs[ci] = nf > 0u ? 2.0f * sum / (float)std::max(nf, 1u) : 0.0f;
        mg_p[ci] = 0.0f;
      }
  }
  void mg_prolong(int l) {
    const Level& L = levels[l];
    const Level& C = levels[l + 1];
#pragma omp parallel for schedule(static)
    for (int y = 0; y < L.ny; y++)
      for (int x = 0; x < L.nx; x++) {
        size_t i = L.off + (size_t)y * L.nx + x;
        if (mg_fluid[i] == 0u) continue;
        mg_p[i] += mg_p[C.off + (size_t)(y / 2) * C.nx + x / 2];
      }
  }
  void mg_finish() {
    const Level& L = levels[0];
    for (int y = 0; y < L.ny; y++)
      for (int x = 0; x < L.nx; x++) pressure_a[fgrid(x, y)] = mg_p[L.off + (size_t)y * L.nx + x];
  }
  // src/world/mod.rs:1545-1577
  void multigrid_solve() {
    int nl = (int)levels.size();
    mg_init();
    uint32_t cycles = std::max(st.mg_cycles, 1u);
    for (uint32_t c = 0; c < cycles; c++) {
      for (int l = 0; l < nl - 1; l++) {
        for (uint32_t k = 0; k < cfg.mg_pre; k++) {
          mg_smooth(l, 0);
          mg_smooth(l, 1);
        }
        mg_restrict(l);
      }
      for (uint32_t k = 0; k < cfg.mg_coarse; k++) {
        mg_smooth(nl - 1, 0);
        mg_smooth(nl - 1, 1);
      }
      for (int l = nl - 2; l >= 0; l--) {
        mg_prolong(l);
        for (uint32_t k = 0; k < cfg.mg_post; k++) {
          mg_smooth(l, 0);
          mg_smooth(l, 1);
        }
      }
    }
    mg_finish();
  }

  // fluid.wgsl:553-608 (one Jacobi sweep pin -> pout)
  void jacobi_sweep(const float* pin, float* pout) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < fh; y++)
      for (int x = 0; x < fw; x++) {
        size_t idx = fgrid(x, y);
        auto load = [&](int gx, int gy, float* p, bool* s) {
          if (gx >= 0 && gy >= 0 && gx < fw && gy < fh) {
            *p = pin[fgrid(gx, gy)];
            *s = is_solid(gx, gy);
          } else {
            *p = 0.0f;
            *s = true;
          }
        };
        float p_c, p_l, p_r, p_b, p_t;
        bool s_c, s_l, s_r, s_b, s_t;
        load(x, y, &p_c, &s_c);
        if (s_c) {
          pout[idx] = 0.0f;
          continue;
        }
        load(x - 1, y, &p_l, &s_l);
        load(x + 1, y, &p_r, &s_r);
        load(x, y - 1, &p_b, &s_b);
        load(x, y + 1, &p_t, &s_t);
        if (s_l) p_l = p_c;
        if (s_r) p_r = p_c;
        if (s_b) p_b = p_c;
        if (s_t) p_t = p_c;
        float d = div[idx];
        if (is_bad(d) || is_bad(p_c)) {
          pout[idx] = 0.0f;
          continue;
        }
        float p_new = (p_l + p_r + p_b + p_t - d) * 0.25f;
        pout[idx] = is_bad(p_new) ? 0.0f : p_new;
      }
  }
  // src/world/mod.rs:1449,1578-1581
  void jacobi_solve() {
    uint32_t it = (std::min(std::max(st.jacobi_iters, 2u), 128u) + 1u) & ~1u;
    for (uint32_t k = 0; k < it; k++) {
      if (k % 2 == 0) jacobi_sweep(pressure_a.data(), pressure_b.data());
      else jacobi_sweep(pressure_b.data(), pressure_a.data());
    }
  }

  // fluid.wgsl:610-630
  void subtract_gradient(const V2* vin, V2* vout) {
    const float* p = pressure_a.data();
#pragma omp parallel for schedule(static)
    for (int yi = 0; yi < fh; yi++)
      for (int xi = 0; xi < fw; xi++) {
        uint32_t x = xi, y = yi;
        size_t idx = fgrid(x, y);
        if (is_solid(x, y)) {
          vout[idx] = v2(0.0f, 0.0f);
          continue;
        }
        float p_c = p[idx];
        float p_l = p_c, p_r = p_c, p_b = p_c, p_t = p_c;
        if (x > 0u && !is_solid(x - 1, y)) p_l = p[fgrid(x - 1, y)];
        if (x + 1u < (uint32_t)fw && !is_solid(x + 1, y)) p_r = p[fgrid(x + 1, y)];
        if (y > 0u && !is_solid(x, y - 1)) p_b = p[fgrid(x, y - 1)];
        if (y + 1u < (uint32_t)fh && !is_solid(x, y + 1)) p_t = p[fgrid(x, y + 1)];
        V2 grad = v2(p_r - p_l, p_t - p_b) * 0.5f;
        V2 v = sanitize(vin[idx]) - grad;
        v = reflect_if_into_solid(x, y, v);
        vout[idx] = clamp_len(sanitize(v), MAX_VEL);
      }
  }

  // fluid.wgsl:640-657 (rows: i < fh; columns: fh + x)
  void compute_net_flux(const V2* vin) {
    int nrows = fh, ncols = fw;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nrows + ncols; i++) {
      bool row = i < nrows;
      int j = row ? i : i - nrows;
      int len = row ? fw : fh;
      float sum = 0.0f, n = 0.0f;
      for (int k = 0; k < len; k++) {
        int x = row ? k : j, y = row ? j : k;
        if (is_solid(x, y)) continue;
        V2 v = sanitize(vin[fgrid(x, y)]);
        sum += row ? v.y : v.x;
        n += 1.0f;
      }
      net_flux[i] = n > 0.0f ? sum / n : 0.0f;
    }
  }
  // fluid.wgsl:663-677
  void enforce_boundaries(const V2* vin, V2* vout) {
#pragma omp parallel for schedule(static)
    for (int yi = 0; yi < fh; yi++)
      for (int xi = 0; xi < fw; xi++) {
        uint32_t x = xi, y = yi;
        size_t idx = fgrid(x, y);
        if (is_solid(x, y)) {
          vout[idx] = v2(0.0f, 0.0f);
          continue;
        }
        V2 v = sanitize(vin[idx]);
        v = v - v2(net_flux[fh + x], net_flux[y]);
        if (x == 0u || x == (uint32_t)fw - 1u) v.x = 0.0f;
        if (y == 0u || y == (uint32_t)fh - 1u) v.y = 0.0f;
        v = reflect_if_into_solid(x, y, v);
        vout[idx] = clamp_len(sanitize(v), MAX_VEL);
      }
  }
  // fluid.wgsl:680-693
  void smooth_velocity(const V2* vin) {
#pragma omp parallel for schedule(static)
    for (int yi = 0; yi < fh; yi++)
      for (int xi = 0; xi < fw; xi++) {
        uint32_t x = xi, y = yi;
        uint32_t xm = x > 0u ? x - 1u : x, xp = std::min(x + 1u, (uint32_t)fw - 1u);
        uint32_t ym = y > 0u ? y - 1u : y, yp = std::min(y + 1u, (uint32_t)fh - 1u);
        V2 v = sanitize(vin[fgrid(x, y)]) + sanitize(vin[fgrid(xm, y)]) + sanitize(vin[fgrid(xp, y)]) +
               sanitize(vin[fgrid(x, ym)]) + sanitize(vin[fgrid(x, yp)]);
        vel_smooth[fgrid(x, y)] = v * 0.2f;
      }
  }

  // transport.wgsl:419-438 (in place; chem_activate_one = chem.wgsl:170-172)
  void thermal_activation() {
#pragma omp parallel for schedule(static)
    for (int yi = 0; yi < gh; yi++)
      for (int xi = 0; xi < gw; xi++) {
        uint32_t x = xi, y = yi;
        uint32_t fx = std::min((x * (uint32_t)fw) / (uint32_t)gw, (uint32_t)fw - 1u);
        uint32_t fy = std::min((y * (uint32_t)fh) / (uint32_t)gh, (uint32_t)fh - 1u);
        float t_loc = temp_a[fgrid(fx, fy)];
        if (t_loc <= TEMP_ACT_THRESHOLD) continue;
        float p_act = rb_clamp(FUMAROLE_ACT_P * rb_max(P->thermal_activation, 0.0f) * (t_loc - TEMP_ACT_THRESHOLD) / TEMP_ACT_THRESHOLD,
                               0.0f, (float)0.9);
        size_t idx = (size_t)y * gw + x;
        for (uint32_t ch = 0; ch < 4; ch++) {
          size_t slot = idx * 4 + ch;
          if ((chem[slot] >> 16) > 0u) {
            if (rb_u2f(rb_pcg4d((uint32_t)slot, P->epoch, RB_S_THERMAL, P->seed).x) < p_act) {
              chem[slot] += 0xFFFF0001u;
            }
          }
        }
      }
  }

  // transport.wgsl:61-87
  void agg_count() {
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)cells(); i++) {
      uint32_t c = 0;
      for (uint32_t ch = 0; ch < 4; ch++) c += chem_act_count(i, ch);
      agg_act[i] = c;
    }
  }
  void agg_neighbours() {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < gh; y++)
      for (int x = 0; x < gw; x++) {
        uint32_t sum = 0;
        for (int dy = -1; dy <= 1; dy++)
          for (int dx = -1; dx <= 1; dx++) {
            if (dx == 0 && dy == 0) continue;
            int nx = x + dx, ny = y + dy;
            if (nx < 0 || ny < 0 || nx >= gw || ny >= gh) continue;
            sum += agg_act[(size_t)ny * gw + nx];
          }
        agg_nb[(size_t)y * gw + x] = sum;
      }
  }

  // transport.wgsl:95-117
  V2 lattice_rand(uint32_t ix, uint32_t iy) const {
    rb_u4 r = rb_pcg4d((ix * 73856093u) ^ (iy * 19349663u), P->epoch, RB_S_MOVE + MAX_MOVERS_PER_CH + 1u, P->seed);
    return v2(rb_u2f(r.x), rb_u2f(r.y));
  }
  V2 smooth_start(uint32_t x0, uint32_t y0) const {
    rb_u4 j = rb_pcg4d(0x85EBCA6Bu, P->epoch, RB_S_MOVE + MAX_MOVERS_PER_CH + 2u, P->seed);
    V2 jit = v2(rb_u2f(j.x), rb_u2f(j.y));
    uint32_t x = x0 + rb_f2u(jit.x * (float)SMOOTH_CELL);
    uint32_t y = y0 + rb_f2u(jit.y * (float)SMOOTH_CELL);
    uint32_t gx = x / SMOOTH_CELL, gy = y / SMOOTH_CELL;
    float tx = rb_smoothstep01(((float)(x % SMOOTH_CELL) + 0.5f) / (float)SMOOTH_CELL);
    float ty = rb_smoothstep01(((float)(y % SMOOTH_CELL) + 0.5f) / (float)SMOOTH_CELL);
    V2 n = mix2(mix2(lattice_rand(gx, gy), lattice_rand(gx + 1u, gy), tx),
                mix2(lattice_rand(gx, gy + 1u), lattice_rand(gx + 1u, gy + 1u), tx), ty);
    rb_u4 gr = rb_pcg4d(0x9E3779B9u, P->epoch, RB_S_MOVE + MAX_MOVERS_PER_CH, P->seed);
    V2 g = v2(rb_u2f(gr.x), rb_u2f(gr.y));
    V2 v = v2(rb_fract(n.x + g.x), rb_fract(n.y + g.y));
    return v2(1.0f - rb_abs(2.0f * v.x - 1.0f), 1.0f - rb_abs(2.0f * v.y - 1.0f));
  }

  // transport.wgsl:119-406
  void transport_scatter() {
    const float cell_w = (float)cfg.world_units_per_cell;
    const float wpf_x = sim_w / (float)fw, wpf_y = sim_h / (float)fh;
    const float rgx = (float)gw / (float)fw, rgy = (float)gh / (float)fh;
    const uint32_t G = gw;
    const V2* vin = vel_a.data();
#pragma omp parallel for schedule(dynamic, 4)
    for (int yi = 0; yi < gh; yi++)
      for (int xi = 0; xi < gw; xi++) {
        uint32_t x = xi, y = yi;
        size_t idx = (size_t)y * gw + x;
        uint32_t src_total = chem_cell_total(idx);
        if (src_total == 0u) continue;
        uint32_t g_src = gamma_count(idx);
        V2 v = v2(0.0f, 0.0f);
        if (P->fluid_enabled != 0u && g_src < GAMMA_SOLID) {
          V2 c = v2((float)x + 0.5f, (float)y + 0.5f) * cell_w;
          V2 v0 = fluid_velocity_at_world(vin, c);
          float h = rb_max(P->dt, 0.0f);
          V2 c2 = v2(c.x + v0.x * wpf_x * h * 0.5f, c.y + v0.y * wpf_y * h * 0.5f);
          v = fluid_velocity_at_world(vin, c2);
        }
        if (v.x != 0.0f || v.y != 0.0f) {
          bool rock_r = x + 1u < G && gamma_count(idx + 1) >= GAMMA_SOLID;
          bool rock_l = x > 0u && gamma_count(idx - 1) >= GAMMA_SOLID;
          bool rock_u = y + 1u < (uint32_t)gh && gamma_count(idx + G) >= GAMMA_SOLID;
          bool rock_d = y > 0u && gamma_count(idx - G) >= GAMMA_SOLID;
          if ((v.x > 0.0f && rock_r) || (v.x < 0.0f && rock_l)) v.x = 0.0f;
          else if ((v.x > 0.0f && rock_l) || (v.x < 0.0f && rock_r)) v.x *= 0.5f;
          if ((v.y > 0.0f && rock_u) || (v.y < 0.0f && rock_d)) v.y = 0.0f;
          else if ((v.y > 0.0f && rock_d) || (v.y < 0.0f && rock_u)) v.y *= 0.5f;
        }
        const float tn = (float)std::max(P->transport_every, 1u);
        const float dtp = rb_max(P->dt, 0.0f);
        V2 disp = v2(v.x * rgx * dtp * tn, v.y * rgy * dtp * tn);
        float agitation = rb_clamp(length(v) / DIFF_AGITATION_SPEED, 0.0f, 1.0f);
        float p_diff = rb_clamp(DIFF_HOP_P * rb_mix(DIFF_HOP_FLOOR, 1.0f, agitation) * rb_max(P->diffusion, 0.0f) * tn, 0.0f, 0.5f);
        if (g_src > 0u) p_diff = rb_min(DIFF_HOP_P * BURIED_DIFF_FACTOR / (1.0f + GAMMA_POROSITY_K * (float)g_src) * tn, 0.5f);
        uint32_t cap_self = chem_capacity(idx);
        if (src_total > cap_self) p_diff = rb_min(CHEM_SQUEEZE_P * tn, 0.5f);
        float p_settle = 0.0f;
        if (g_src == 0u) p_settle = rb_min(MONOMER_SETTLE_P * rb_max(P->settle, 0.0f) * tn, 0.5f);
        int base_x = rb_f2i(rb_floor(disp.x)) - 1, base_y = rb_f2i(rb_floor(disp.y)) - 1;

        float press[4] = {1.0f, 1.0f, 1.0f, 1.0f};
        float max_drop = 0.0f;
        if (P->monomer_pressure > 0.0f) {
          float f_self = (float)src_total / (float)std::max(cap_self, 1u);
          long nb[4] = {1, -1, (long)G, -(long)G};
          bool inside[4] = {x + 1u < G, x > 0u, y + 1u < (uint32_t)gh, y > 0u};
          for (int d = 0; d < 4; d++) {
            if (!inside[d]) continue;
            size_t n = (size_t)((long)idx + nb[d]);
            uint32_t cap_n = chem_capacity(n);
            if (cap_n == 0u) continue;
            float f_n = (float)chem_cell_total(n) / (float)cap_n;
            press[d] = rb_max((float)0.05, 1.0f + P->monomer_pressure * (f_self - f_n));
            max_drop = rb_max(max_drop, f_self - f_n);
          }
        }
        p_diff = rb_clamp(p_diff + PRESSURE_HOP_P * P->monomer_pressure * max_drop * tn, 0.0f, 0.5f);
        float light_t = uv_light_at_cell(x, y);

        float p_bound = 0.0f;
        float accept[4] = {1.0f, 1.0f, 1.0f, 1.0f};
        float accept_spent[4] = {1.0f, 1.0f, 1.0f, 1.0f};
        if (P->aggregation > 0.0f && src_total <= cap_self) {
          float e[5] = {(float)(agg_nb[idx] + agg_act[idx]), 0.0f, 0.0f, 0.0f, 0.0f};
          if (x + 1u < G) e[1] = (float)(agg_nb[idx + 1] + agg_act[idx + 1]);
          if (x > 0u) e[2] = (float)(agg_nb[idx - 1] + agg_act[idx - 1]);
          if (y + 1u < (uint32_t)gh) e[3] = (float)(agg_nb[idx + G] + agg_act[idx + G]);
          if (y > 0u) e[4] = (float)(agg_nb[idx - G] + agg_act[idx - G]);
          uint32_t fx = std::min((x * (uint32_t)fw) / G, (uint32_t)fw - 1u);
          uint32_t fy = std::min((y * (uint32_t)fh) / (uint32_t)gh, (uint32_t)fh - 1u);
          float t_rel = 1.0f + rb_max(temp_a[fgrid(fx, fy)], 0.0f) / TEMP_ACT_THRESHOLD;
          float room = rb_clamp(5.0f * (1.0f - (float)src_total / (float)std::max(cap_self, 1u)), 0.0f, 1.0f);
          float k_e = P->aggregation * room / t_rel;
          for (int d = 0; d < 4; d++) {
            float drop = e[0] - e[d + 1];
            if (drop > 0.0f) accept[d] = rb_exp(-k_e * drop);
            float rise = e[d + 1] - e[0];
            if (rise > 0.0f) accept_spent[d] = rb_exp(-k_e * rise);
          }
          p_bound = 1.0f - rb_exp(-k_e * rb_min(rb_max(e[0] - 1.0f, 0.0f), 48.0f));
        }

        V2 bound_start = v2(0.0f, 0.0f);
        bool have_bound_start = false;
        for (uint32_t ch = 0; ch < 4; ch++) {
          size_t slot = idx * 4 + ch;
          uint32_t v_ch = chem[slot];
          uint32_t act_n = v_ch & CHEM_STATE_MASK;
          uint32_t spent_n = v_ch >> 16;
          if (act_n + spent_n == 0u) continue;
          if (spent_n > 0u) {
            float sens = 1.0f + CHEM_SENSITIZE * (float)std::min(act_n, 8u);
            float exp_act = (float)std::min(spent_n, 8u) * tn *
                            (LIGHT_ACT_P * rb_max(P->uv_strength, 0.0f) * rb_max(P->direct_photoactivation, 0.0f) * light_t * sens +
                             rb_max(P->reactivation_rate, 0.0f));
            uint32_t na = rb_f2u(rb_floor(exp_act));
            float frac = exp_act - (float)na;
            if (frac > 0.0f && rb_u2f(rb_pcg4d((uint32_t)slot, P->epoch, RB_S_PHOTO, P->seed).x) < frac) na += 1u;
            na = std::min(na, std::min(spent_n, 8u));
            act_n += na;
            spent_n -= na;
          }
          if (act_n > 0u) {
            float shield = 1.0f / (1.0f + CHEM_SHIELD * (float)(std::min(act_n, 8u) - 1u));
            float exp_dec = (float)std::min(act_n, 8u) * rb_max(P->activation_decay, 0.0f) * shield * tn;
            if (exp_dec > 0.0f && rb_u2f(rb_pcg4d((uint32_t)slot, P->epoch, RB_S_DECAY, P->seed).x) < exp_dec) {
              act_n -= 1u;
              spent_n += 1u;
            }
          }
          float coh[4] = {1.0f, 1.0f, 1.0f, 1.0f};
          if (act_n > 0u && P->cohesion > 0.0f) {
            if (x + 1u < G) coh[0] = 1.0f + P->cohesion * (float)std::min(chem_act_count(idx + 1, ch), 8u);
            if (x > 0u) coh[1] = 1.0f + P->cohesion * (float)std::min(chem_act_count(idx - 1, ch), 8u);
            if (y + 1u < (uint32_t)gh) coh[2] = 1.0f + P->cohesion * (float)std::min(chem_act_count(idx + G, ch), 8u);
            if (y > 0u) coh[3] = 1.0f + P->cohesion * (float)std::min(chem_act_count(idx - G, ch), 8u);
          }
          uint32_t bins[16] = {0};
          uint32_t stay = 0;
          uint32_t n = act_n + spent_n;
          uint32_t movers = std::min(n, MAX_MOVERS_PER_CH);
          uint32_t act_stay = act_n - std::min(act_n, movers);
          stay += act_stay + (n - movers - act_stay) * CHEM_SPENT_ONE;
          if (!have_bound_start) {
            bound_start = smooth_start(x, y);
            have_bound_start = true;
          }
          for (uint32_t k = 0; k < movers; k++) {
            uint32_t unit = k < act_n ? 1u : CHEM_SPENT_ONE;
            rb_u4 ru = rb_pcg4d((uint32_t)slot, P->epoch, RB_S_MOVE + k, P->seed);
            float rfx = rb_u2f(ru.x), rfy = rb_u2f(ru.y), rfz = rb_u2f(ru.z), rfw = rb_u2f(ru.w);
            bool bound = k < act_n && p_bound > 0.0f && rb_fract(rfz * (float)7.31 + rfw * (float)3.17) < p_bound;
            V2 p = (bound ? bound_start : v2(rfx, rfy)) + disp;
            if (g_src > 0u && (disp.x != 0.0f || disp.y != 0.0f)) {
              rb_u4 rj = rb_pcg4d((uint32_t)slot, P->epoch, RB_S_DISPERSE + k, P->seed);
              float ld = length(disp);
              V2 jitter = v2((rb_u2f(rj.x) * 2.0f - 1.0f) * ld * RUBBLE_DISPERSION,
                             (rb_u2f(rj.y) * 2.0f - 1.0f) * ld * RUBBLE_DISPERSION);
              p = p + v2(rb_clamp(jitter.x, (float)-0.9, (float)0.9), rb_clamp(jitter.y, (float)-0.9, (float)0.9));
            }
            float r = rfz;
            if (r < p_diff) {
              float w[4] = {press[0], press[1], press[2], press[3]};
              if (k < act_n)
                for (int cd = 0; cd < 4; cd++) w[cd] *= coh[cd];
              float u = rfw * (w[0] + w[1] + w[2] + w[3]);
              uint32_t d = 3u;
              for (uint32_t cd = 0; cd < 4; cd++) {
                if (u < w[cd]) {
                  d = cd;
                  break;
                }
                u -= w[cd];
              }
              float acc_d = k < act_n ? accept[d] : accept_spent[d];
              bool stay_put = rb_fract(rfw * (float)13.73 + rfx * (float)5.31) >= acc_d;
              if (!stay_put) {
                if (d == 0u) p.x += 1.0f;
                else if (d == 1u) p.x -= 1.0f;
                else if (d == 2u) p.y += 1.0f;
                else p.y -= 1.0f;
              }
            } else if (r < p_diff + p_settle) {
              p.y -= 1.0f;
            }
            int offx = rb_f2i(rb_floor(p.x)) - base_x, offy = rb_f2i(rb_floor(p.y)) - base_y;
            uint32_t bi = (uint32_t)std::min(std::max(offy, 0), 3) * 4u + (uint32_t)std::min(std::max(offx, 0), 3);
            bins[bi] += unit;
          }
          for (uint32_t b = 0; b < 16; b++) {
            uint32_t cnt = bins[b];
            if (cnt == 0u) continue;
            int tx = std::min(std::max((int)x + base_x + (int)(b & 3u), 0), gw - 1);
            int ty = std::min(std::max((int)y + base_y + (int)(b >> 2), 0), gh - 1);
            size_t t_idx = (size_t)ty * gw + tx;
            bool blocked = false;
            if (t_idx != idx) {
              uint32_t g_tgt = gamma_count(t_idx);
              if (g_tgt >= GAMMA_SOLID) blocked = g_src < GAMMA_SOLID;
              else if (chem_cell_total(t_idx) > chem_capacity(t_idx)) blocked = true;
            }
            if (blocked) stay += cnt;
            else atomic_add_u32(&chem_next[t_idx * 4 + ch], cnt);
          }
          if (stay > 0u) atomic_add_u32(&chem_next[slot], stay);
        }
      }
  }
  // transport.wgsl:409-415
  void transport_commit() {
    chem.swap(chem_next);
    std::fill(chem_next.begin(), chem_next.end(), 0u);
  }

  // ledger.wgsl:225-245
  void ledger(uint32_t out[12]) const {
    uint64_t s[8] = {0};
#pragma omp parallel
    {
      uint64_t loc[8] = {0};
#pragma omp for schedule(static) nowait
      for (long i = 0; i < (long)cells(); i++)
        for (int ch = 0; ch < 4; ch++) {
          uint32_t v = chem[i * 4 + ch];
          loc[ch] += v & CHEM_STATE_MASK;
          loc[4 + ch] += v >> 16;
        }
#pragma omp critical
      for (int k = 0; k < 8; k++) s[k] += loc[k];
    }
    for (int k = 0; k < 8; k++) out[k] = (uint32_t)s[k];  // u32 atomics wrap in the reference
    for (int k = 8; k < 12; k++) out[k] = 0u;
  }

  // src/world/mod.rs:1416-1421, 1487-1601 (fluid and transport blocks of one step)
  void step(const ribo_sim_params* p) {
    P = p;
    uint32_t epoch = p->epoch;
    uint32_t substep = std::min(std::max(st.fluid_substep, 1u), 4u);
    if (st.terrain_mode) terrain_block();
    if (st.light_mode) light_block(epoch);
    if (st.fluid_enabled && epoch % substep == 0u) {
      build_solid_mask();
      update_temperature();
      copy_temperature();
      buoyancy();
      gather_forces();
      clear_force_vectors();
      add_forces(vel_a.data(), vel_b.data());
      clear_forces();
      diffuse_velocity(vel_b.data(), vel_a.data());
      advect_velocity(vel_a.data(), vel_b.data());
      vorticity_confinement(vel_b.data(), vel_a.data());
      compute_divergence(vel_a.data());
      if (st.multigrid) multigrid_solve();
      else jacobi_solve();
      subtract_gradient(vel_a.data(), vel_b.data());
      compute_net_flux(vel_b.data());
      enforce_boundaries(vel_b.data(), vel_a.data());
      smooth_velocity(vel_a.data());
      thermal_activation();
    }
    if (epoch % std::max(p->transport_every, 1u) == 0u) {
      if (p->aggregation > 0.0f) {
        agg_count();
        agg_neighbours();
      }
      transport_scatter();
      transport_commit();
    }
  }

  void* field_ptr(int f, size_t* bytes) {
    switch (f) {
      case RIBO_FIELD_CHEM: *bytes = chem.size() * 4; return chem.data();
      case RIBO_FIELD_GAMMA: *bytes = gamma.size() * 4; return gamma.data();
      case RIBO_FIELD_LIGHT: *bytes = light.size() * 4; return light.data();
      case RIBO_FIELD_SLOPE: *bytes = slope.size() * 8; return slope.data();
      case RIBO_FIELD_VELOCITY: *bytes = vel_a.size() * 8; return vel_a.data();
      case RIBO_FIELD_PRESSURE: *bytes = pressure_a.size() * 4; return pressure_a.data();
      case RIBO_FIELD_TEMP: *bytes = temp_a.size() * 4; return temp_a.data();
      case RIBO_FIELD_REDOX: *bytes = redox_a.size() * 4; return redox_a.data();
      case RIBO_FIELD_HEAT: *bytes = heat.size() * 8; return heat.data();
      case RIBO_FIELD_VEL_SMOOTH: *bytes = vel_smooth.size() * 8; return vel_smooth.data();
      case RIBO_FIELD_SOLID_MASK: *bytes = solid_mask.size() * 4; return solid_mask.data();
      case RIBO_FIELD_DIVERGENCE: *bytes = div.size() * 4; return div.data();
      case RIBO_FIELD_FORCE_VECTORS: *bytes = force_vec.size() * 4; return force_vec.data();
      case RIBO_FIELD_REDOX_EATEN: *bytes = redox_eaten.size() * 4; return redox_eaten.data();
      case RIBO_FIELD_NET_FLUX: *bytes = net_flux.size() * 4; return net_flux.data();
      case RIBO_FIELD_SHADE: *bytes = shade.size() * 4; return shade.data();
    }
    *bytes = 0;
    return nullptr;
  }
};

}  // namespace

extern "C" {

typedef struct Oracle orc_world;

void* orc_create(const ribo_world_cfg* cfg) {
  Oracle* o = new Oracle();
  o->cfg = *cfg;
  if (!o->cfg.world_units_per_cell) o->cfg.world_units_per_cell = 30;
  if (!o->cfg.mg_min_size) o->cfg.mg_min_size = 8;
  if (!o->cfg.mg_pre) o->cfg.mg_pre = 2;
  if (!o->cfg.mg_post) o->cfg.mg_post = 2;
  if (!o->cfg.mg_coarse) o->cfg.mg_coarse = 30;
  o->st = ribo_world_settings{1, 2, 1, 1, 128, 0, 0, 0};
  o->gw = cfg->grid_w;
  o->gh = cfg->grid_h;
  o->fw = cfg->fluid_w;
  o->fh = cfg->fluid_h;
  o->lw = o->gw / 2;
  o->lh = o->gh / 2;
  o->rx = o->gw / o->fw;
  o->ry = o->gh / o->fh;
  o->sim_w = (float)(o->gw * o->cfg.world_units_per_cell);
  o->sim_h = (float)(o->gh * o->cfg.world_units_per_cell);
  size_t C = o->cells(), F = o->fcells(), L = o->lcells();
  o->chem.assign(C * 4, 0);
  o->chem_next.assign(C * 4, 0);
  o->gamma.assign(C, 0);
  o->agg_act.assign(C, 0);
  o->agg_nb.assign(C, 0);
  o->shade.assign(2 * L, 0);
  o->force_vec.assign(F * 2, 0);
  o->redox_eaten.assign(F, 0);
  o->solid_mask.assign(F, 0);
  o->light.assign(2 * L, 0.0f);
  o->light_next.assign(2 * L, 0.0f);
  o->pressure_a.assign(F, 0.0f);
  o->pressure_b.assign(F, 0.0f);
  o->div.assign(F, 0.0f);
  o->temp_a.assign(F, 0.0f);
  o->temp_b.assign(F, 0.0f);
  o->redox_a.assign(F, 0.0f);
  o->redox_b.assign(F, 0.0f);
  o->net_flux.assign((size_t)o->fw + o->fh, 0.0f);
  o->slope.assign(C, V2{0, 0});
  o->vel_a.assign(F, V2{0, 0});
  o->vel_b.assign(F, V2{0, 0});
  o->vel_smooth.assign(F, V2{0, 0});
  o->fluid_forces.assign(F, V2{0, 0});
  o->heat.assign(F, V2{0, 0});
  o->setup_levels();
  return o;
}

void orc_destroy(void* w) { delete (Oracle*)w; }

void orc_set_settings(void* w, const ribo_world_settings* s) {
  Oracle* o = (Oracle*)w;
  if (s->light_mode && !o->st.light_mode) o->light_dirty = true;
  o->st = *s;
}

int orc_upload(void* w, int field, const void* host, size_t bytes) {
  Oracle* o = (Oracle*)w;
  size_t n = 0;
  void* p = o->field_ptr(field, &n);
  if (!p || n != bytes) return 1;
  memcpy(p, host, bytes);
  if (field == RIBO_FIELD_GAMMA) {
    // The slope and wall mask are functions of gamma alone; the step also
    // rebuilds the mask at every fluid step, as the reference does.
    o->compute_slope();
    o->build_solid_mask();
    o->light_dirty = true;
  }
  return 0;
}

int orc_read(void* w, int field, void* host, size_t bytes) {
  Oracle* o = (Oracle*)w;
  size_t n = 0;
  void* p = o->field_ptr(field, &n);
  if (!p || n != bytes) return 1;
  memcpy(host, p, bytes);
  return 0;
}

// Steps with explicit per-step params (same contract as ribo_world_step).
void orc_step(void* w, const ribo_sim_params* per_step, uint32_t n) {
  Oracle* o = (Oracle*)w;
  if (!o->st.fluid_enabled && o->fluid_was_on) {
    std::fill(o->vel_a.begin(), o->vel_a.end(), V2{0, 0});
    std::fill(o->temp_a.begin(), o->temp_a.end(), 0.0f);
    std::fill(o->redox_a.begin(), o->redox_a.end(), 0.0f);
  }
  o->fluid_was_on = o->st.fluid_enabled != 0;
  for (uint32_t i = 0; i < n; i++) o->step(&per_step[i]);
}

void orc_ledger(void* w, uint32_t out[12]) { ((Oracle*)w)->ledger(out); }

int orc_num_levels(void* w) { return (int)((Oracle*)w)->levels.size(); }

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

int orc_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// Single passes, for unit tests of individual kernels.  `which`:
// 0 mask, 1 temperature(+copy), 2 forces(buoyancy, gather, clear), 3 add_forces a->b,
// 4 diffuse b->a, 5 advect a->b, 6 vorticity b->a, 7 divergence(a), 8 pressure solve,
// 9 subtract_gradient a->b, 10 net_flux(b), 11 boundaries b->a, 12 smooth(a),
// 13 thermal, 14 agg_count+agg_neighbours, 15 transport scatter+commit,
// 16 relax pass a, 17 relax pass b, 18 grain_fall.
void orc_pass(void* w, const ribo_sim_params* p, int which) {
  Oracle* o = (Oracle*)w;
  o->P = p;
  switch (which) {
    case 0: o->build_solid_mask(); break;
    case 1: o->update_temperature(); o->copy_temperature(); break;
    case 2: o->buoyancy(); o->gather_forces(); o->clear_force_vectors(); break;
    case 3: o->add_forces(o->vel_a.data(), o->vel_b.data()); o->clear_forces(); break;
    case 4: o->diffuse_velocity(o->vel_b.data(), o->vel_a.data()); break;
    case 5: o->advect_velocity(o->vel_a.data(), o->vel_b.data()); break;
    case 6: o->vorticity_confinement(o->vel_b.data(), o->vel_a.data()); break;
    case 7: o->compute_divergence(o->vel_a.data()); break;
    case 8: if (o->st.multigrid) o->multigrid_solve(); else o->jacobi_solve(); break;
    case 9: o->subtract_gradient(o->vel_a.data(), o->vel_b.data()); break;
    case 10: o->compute_net_flux(o->vel_b.data()); break;
    case 11: o->enforce_boundaries(o->vel_b.data(), o->vel_a.data()); break;
    case 12: o->smooth_velocity(o->vel_a.data()); break;
    case 13: o->thermal_activation(); break;
    case 14: o->agg_count(); o->agg_neighbours(); break;
    case 15: o->transport_scatter(); o->transport_commit(); break;
    case 16: o->relax_pass(0u); break;
    case 17: o->relax_pass(1u); break;
    case 18: o->grain_fall(); break;
  }
}

// World::encode_paint: `grains` grains in every cell of the disc (centre and
// radius in cells), the monomers that no longer fit evicted.
void orc_paint(void* w, float cx, float cy, float radius, uint32_t grains) {
  ((Oracle*)w)->paint(cx, cy, radius, grains);
}

// Reads velocity_b (the intermediate velocity buffer) for per-pass tests.
int orc_read_vel_b(void* w, void* host, size_t bytes) {
  Oracle* o = (Oracle*)w;
  if (bytes != o->vel_b.size() * 8) return 1;
  memcpy(host, o->vel_b.data(), bytes);
  return 0;
}
int orc_write_vel_b(void* w, const void* host, size_t bytes) {
  Oracle* o = (Oracle*)w;
  if (bytes != o->vel_b.size() * 8) return 1;
  memcpy(o->vel_b.data(), host, bytes);
  return 0;
}

// Pinned math, exported so the CPU tests can bound its error against libm.
float orc_exp(float x) { return rb_exp(x); }
float orc_log(float x) { return rb_log(x); }
float orc_pow(float x, float y) { return rb_pow(x, y); }
float orc_sin(float x) { return rb_sin(x); }
void orc_pcg4d(uint32_t a, uint32_t b, uint32_t c, uint32_t d, uint32_t out[4]) {
  rb_u4 r = rb_pcg4d(a, b, c, d);
  out[0] = r.x;
  out[1] = r.y;
  out[2] = r.z;
  out[3] = r.w;
}

}  // extern "C"
