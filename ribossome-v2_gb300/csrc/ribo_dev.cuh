// Device-side world description and the helper functions the world-step
// kernels share.  Every helper restates a WGSL helper of the reference
// (paths relative to the reference project); float arithmetic follows the
// pinned semantics of ribo_fmath.h (the library is compiled with
// -fmad=false, IEEE division and square root).
#pragma once
#include <cstdio>  // device printf of the bounds-checked build
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/ribo_world.h"
#include "ribo_fmath.h"

namespace ribo {

// ---- constants (shaders/world/fluid.wgsl:15-56, transport.wgsl:23-50,
// common/chem.wgsl:118-119, common/terrain.wgsl:214, light.wgsl:18-40).
// Literals that WGSL evaluates as abstract floats are rounded from double.
constexpr float MAX_DT = (float)0.07;
constexpr float MAX_FORCE = (float)200000.0;
constexpr float MAX_VEL = (float)2000.0;
constexpr float FORCE_SMOOTH_MIX = (float)0.25;
constexpr float SOLID_PERM_THRESHOLD = (float)0.02;
constexpr float TEMP_HEAT_RATE = (float)0.01;
constexpr float TEMP_COOL_RATE = (float)0.12;
constexpr float TEMP_MAX = (float)12.0;
constexpr float SUN_HEAT_RATE = (float)0.15;
constexpr float SUN_IR = (float)1.2;
constexpr float SUN_IR_DEPTH = (float)0.08;
constexpr float TEMP_BUOYANCY = (float)12.0;
constexpr float TEMP_AMBIENT_SURFACE = (float)0.0;
constexpr float TEMP_AMBIENT_ATTEN = (float)4.0;
constexpr float TEMP_DIFFUSE = (float)0.08;
constexpr float TEMP_ROCK_CONDUCT = (float)4.0;
constexpr float REDOX_RATE = (float)0.01;
constexpr float VENT_WAVES = (float)1.5;
constexpr float REDOX_FP = (float)10000.0;
constexpr float REDOX_MAX = (float)50.0;
constexpr float RUBBLE_DRAG = (float)300.0;
constexpr float FORCE_FP = (float)256.0;
constexpr float DIFF_HOP_P = (float)0.01;
constexpr float DIFF_HOP_FLOOR = (float)0.15;
constexpr float DIFF_AGITATION_SPEED = (float)0.5;
constexpr float BURIED_DIFF_FACTOR = (float)1.0;
constexpr float GAMMA_POROSITY_K = (float)0.3;
constexpr float PRESSURE_HOP_P = (float)0.01;
constexpr float RUBBLE_DISPERSION = (float)1.0;
constexpr float CHEM_SQUEEZE_P = (float)0.25;
constexpr float MONOMER_SETTLE_P = (float)0.002;
constexpr uint32_t MAX_MOVERS_PER_CH = 256u;
constexpr float LIGHT_ACT_P = (float)0.006;
constexpr float CHEM_SENSITIZE = (float)0.5;
constexpr float CHEM_SHIELD = (float)0.5;
constexpr float TEMP_ACT_THRESHOLD = (float)2.0;
constexpr float FUMAROLE_ACT_P = (float)0.15;
constexpr uint32_t SMOOTH_CELL = 16u;
constexpr uint32_t CHEM_STATE_MASK = 0xFFFFu;
constexpr uint32_t CHEM_SPENT_ONE = 0x10000u;
constexpr uint32_t CHEM_CELL_CAP = 48u;
constexpr uint32_t GAMMA_SOLID = 3u;
constexpr float GAMMA_QUANTUM = (float)0.25;
constexpr uint32_t LIGHT_DIV = 2u;
constexpr float UV_SHADOW_ABSORB = (float)0.6;
constexpr float AGENT_UV_ABSORB = (float)0.15;
constexpr float SUN_WATER_ABSORB = (float)0.05;
constexpr int LIGHT_TAPS = 7;
constexpr float SHADE_ONE = (float)100.0;

// One world as the kernels see it.  Built on the host for every launch, so
// ping-pong roles are resolved there.
struct Dev {
  // dimensions
  int gw, gh;    // environment grid
  int fw, fh;    // fluid grid
  int lw, lh;    // light grid (grid / LIGHT_DIV)
  int rx, ry;    // integer grid/fluid ratio (GRID_SIZE / FLUID_SIZE)
  float sx, sy;  // f32(GRID) / f32(FLUID)
  float sim_w, sim_h, cell_w;
  float wpf_x, wpf_y;  // SIM_SIZE / f32(FLUID_SIZE)
  int pad0;            // explicit, zero: Dev records are compared byte for byte (batch tables)
  // environment-resolution buffers
  uint32_t* chem;       // chem_grid (state before the step)
  uint32_t* chem_next;  // transport destination (zero between steps)
  const uint32_t* gamma;
  const float* light;
  float* light_next;  // light_propagate's output (the light block; the light field itself is written through light)
  const uint32_t* shade;
  float2* slope;
  uint32_t* agg_nb;   // 3 x 3 box sums of the activated counts (aggregation)
  // fluid-resolution buffers
  uint8_t* mask;    // 1 = wall
  float2* normal;   // outward wall normal of each fluid cell (from the mask)
  float* curl;      // curl of the velocity entering the confinement pass
  float2* va;     // velocity_a
  float2* vb;     // velocity_b
  float2* vsmooth;
  float* pa;  // pressure_a
  float* pb;  // pressure_b (Jacobi ping-pong)
  float* div;
  float* temp_in;
  float* temp_out;
  float* redox_in;
  float* redox_out;
  uint32_t* redox_eaten;
  uint32_t* force_vec;
  float2* forces;
  const float2* heat;
  float* net_flux;
  uint32_t* ledger;   // 12 words
  uint8_t* fluid0;    // level-0 water flags of the multigrid (1 = water), rebuilt with the mask
  uint32_t* status;   // error bits written by kernels instead of trapping (RIBO_ERR_*)
  const void* tmap;   // TMA descriptors of the stencil passes' tiles (csrc/ribo_tma.cuh), or null
};
static_assert(sizeof(Dev) == 16 * 4 + 30 * sizeof(void*), "Dev has no padding bytes: every byte is a member");

__device__ __forceinline__ float2 f2(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return f2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return f2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 mul2(float2 a, float s) { return f2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 smul2(float s, float2 a) { return f2(s * a.x, s * a.y); }
__device__ __forceinline__ float2 div2(float2 a, float s) { return f2(a.x / s, a.y / s); }
__device__ __forceinline__ float dot2(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }
__device__ __forceinline__ float len2(float2 a) { return rb_sqrt(a.x * a.x + a.y * a.y); }
__device__ __forceinline__ float2 mix2(float2 a, float2 b, float t) { return f2(rb_mix(a.x, b.x, t), rb_mix(a.y, b.y, t)); }
__device__ __forceinline__ int imin(int a, int b) { return a < b ? a : b; }
__device__ __forceinline__ int imax(int a, int b) { return a > b ? a : b; }
__device__ __forceinline__ int iclamp(int v, int lo, int hi) { return imin(imax(v, lo), hi); }
__device__ __forceinline__ uint32_t umin(uint32_t a, uint32_t b) { return a < b ? a : b; }

// fluid.wgsl:70-83
__device__ __forceinline__ bool is_bad(float x) { return (x != x) || (rb_abs(x) > (float)1e20); }
__device__ __forceinline__ float2 sanitize(float2 v) { return (is_bad(v.x) || is_bad(v.y)) ? f2(0.0f, 0.0f) : v; }
__device__ __forceinline__ float2 clamp_len(float2 v, float max_len) {
  float len = len2(v);
  if (len > max_len) return mul2(v, max_len / rb_max(len, (float)1e-12));
  return v;
}
// fluid.wgsl:66-68
__device__ __forceinline__ float fluid_dt(const ribo_sim_params* P) { return rb_clamp(P->fluid_dt, 0.0f, MAX_DT); }

// common/chem.wgsl:129-145
__device__ __forceinline__ uint32_t word_total(uint32_t v) { return (v & CHEM_STATE_MASK) + (v >> 16); }
__device__ __forceinline__ uint32_t cell_total4(uint4 c) {
  return word_total(c.x) + word_total(c.y) + word_total(c.z) + word_total(c.w);
}
__device__ __forceinline__ uint32_t capacity_of(uint32_t g) {
  return g >= GAMMA_SOLID ? 0u : CHEM_CELL_CAP * (GAMMA_SOLID - g) / GAMMA_SOLID;
}
__device__ __forceinline__ uint4 load_cell(const uint32_t* chem, size_t idx) {
  return __ldg(reinterpret_cast<const uint4*>(chem) + idx);
}

// fluid.wgsl:62-64.  With the surface temperature 0 the product is +0 for
// every cell (the exponential is finite and positive), so it is not evaluated.
__device__ __forceinline__ float temp_ambient_at(const Dev& d, uint32_t y) {
  if (TEMP_AMBIENT_SURFACE == 0.0f) return 0.0f;
  return TEMP_AMBIENT_SURFACE * rb_exp(-TEMP_AMBIENT_ATTEN * (1.0f - ((float)y + 0.5f) / (float)d.fh));
}
// fluid.wgsl:46-54
__device__ __forceinline__ float vent_cycle(const Dev& d, const ribo_sim_params* P, uint32_t x) {
  float m = 1.0f;
  if (P->vent_cycle_amp > 0.0f && P->vent_cycle_period >= 1.0f) {
    uint32_t period = rb_f2u(P->vent_cycle_period);
    float t = (float)(P->epoch % period) / (float)period;
    m = rb_max(1.0f + P->vent_cycle_amp * rb_sin((float)6.2831853 * (t + VENT_WAVES * (float)x / (float)d.fw)), 0.0f);
  }
  return m;
}

__device__ __forceinline__ bool is_solid(const Dev& d, int x, int y) { return d.mask[(size_t)y * d.fw + x] != 0; }

// fluid.wgsl:87-92
__device__ __forceinline__ size_t env_cell_for_fluid(const Dev& d, uint32_t x, uint32_t y) {
  uint32_t gx = rb_f2u(rb_clamp(((float)x + 0.5f) * d.sx, 0.0f, (float)(d.gw - 1)));
  uint32_t gy = rb_f2u(rb_clamp(((float)y + 0.5f) * d.sy, 0.0f, (float)(d.gh - 1)));
  return (size_t)gy * d.gw + gx;
}
// min(g, GAMMA_SOLID) / GAMMA_SOLID for g = 0..GAMMA_SOLID: the quotients the
// fill sum adds, divided once at compile time (IEEE division either way).
__constant__ const float FILL_TERM[4] = {0.0f / (float)GAMMA_SOLID, 1.0f / (float)GAMMA_SOLID,
                                         2.0f / (float)GAMMA_SOLID, 3.0f / (float)GAMMA_SOLID};
static_assert(GAMMA_SOLID == 3u, "FILL_TERM lists the quotients for GAMMA_SOLID = 3");
// fluid.wgsl:114-128
__device__ __forceinline__ float gamma_fill_at_fluid_cell(const Dev& d, uint32_t x, uint32_t y) {
  float gx = ((float)x + 0.5f) * d.sx, gy = ((float)y + 0.5f) * d.sy;
  float hx = d.sx * 0.25f, hy = d.sy * 0.25f;
  float fill = 0.0f;
#pragma unroll
  for (uint32_t s = 0; s < 4; s++) {
    float ox = (s & 1u) == 1u ? hx : -hx;
    float oy = (s & 2u) == 2u ? hy : -hy;
    uint32_t sx = rb_f2u(rb_clamp(gx + ox, 0.0f, (float)(d.gw - 1)));
    uint32_t sy = rb_f2u(rb_clamp(gy + oy, 0.0f, (float)(d.gh - 1)));
    fill += FILL_TERM[umin(__ldg(d.gamma + (size_t)sy * d.gw + sx), GAMMA_SOLID)];
  }
  return fill * 0.25f;
}

// fluid.wgsl:196-224.  n = outward wall normal from the 8 neighbours.
__device__ __forceinline__ float2 solid_normal(const Dev& d, uint32_t x, uint32_t y) {
  uint32_t xm = x == 0u ? x : x - 1u;
  uint32_t xp = x + 1u >= (uint32_t)d.fw ? x : x + 1u;
  uint32_t ym = y == 0u ? y : y - 1u;
  uint32_t yp = y + 1u >= (uint32_t)d.fh ? y : y + 1u;
  bool hx0 = x > 0u, hx1 = x + 1u < (uint32_t)d.fw, hy0 = y > 0u, hy1 = y + 1u < (uint32_t)d.fh;
  float s_l = (hx0 && is_solid(d, xm, y)) ? 1.0f : 0.0f;
  float s_r = (hx1 && is_solid(d, xp, y)) ? 1.0f : 0.0f;
  float s_b = (hy0 && is_solid(d, x, ym)) ? 1.0f : 0.0f;
  float s_t = (hy1 && is_solid(d, x, yp)) ? 1.0f : 0.0f;
  float s_bl = (hx0 && hy0 && is_solid(d, xm, ym)) ? 1.0f : 0.0f;
  float s_tl = (hx0 && hy1 && is_solid(d, xm, yp)) ? 1.0f : 0.0f;
  float s_br = (hx1 && hy0 && is_solid(d, xp, ym)) ? 1.0f : 0.0f;
  float s_tr = (hx1 && hy1 && is_solid(d, xp, yp)) ? 1.0f : 0.0f;
  const float diag = (float)0.70710678;
  float nx = (s_l - s_r) + diag * ((s_bl + s_tl) - (s_br + s_tr));
  float ny = (s_b - s_t) + diag * ((s_bl + s_br) - (s_tl + s_tr));
  float2 n = f2(nx, ny);
  float n_len = len2(n);
  return n_len > (float)1e-6 ? div2(n, n_len) : f2(0.0f, 0.0f);
}
__device__ __forceinline__ float2 reflect_n(float2 n, float2 v_in) {
  float dd = dot2(v_in, n);
  if (len2(n) > (float)1e-6 && dd < 0.0f) return sub2(v_in, mul2(n, dd));
  return v_in;
}
// The wall normal depends on the mask alone, so it is computed once per
// mask build (k_wall_normals) and read here: same function, same bits.  A
// stored normal is either exactly (0, 0) or of length about 1 (solid_normal
// divides by a length above 1e-6), so reflect_n's "length > 1e-6" is
// "not (0, 0)" for it.
__device__ __forceinline__ float2 reflect_stored(float2 n, float2 v) {
  if (n.x == 0.0f && n.y == 0.0f) return v;
  const float dd = dot2(v, n);
  return dd < 0.0f ? sub2(v, mul2(n, dd)) : v;
}
__device__ __forceinline__ float2 reflect_if_into_solid(const Dev& d, uint32_t x, uint32_t y, float2 v) {
  return reflect_stored(d.normal[(size_t)y * d.fw + x], v);
}
// fluid.wgsl:191-194 on an arbitrary input buffer
// Both loads are issued unconditionally (the cell is in the grid), so they
// overlap instead of the velocity load waiting on the mask.
__device__ __forceinline__ float2 raw_velocity_cell(const Dev& d, const float2* vin, uint32_t x, uint32_t y) {
  const size_t i = (size_t)y * d.fw + x;
  const uint8_t solid = d.mask[i];
  const float2 v = vin[i];
  return solid ? f2(0.0f, 0.0f) : sanitize(v);
}

// ---- light helpers used by the temperature pass (light.wgsl:46-102,182-189) ----
__device__ __forceinline__ float light_above(const Dev& d, const ribo_sim_params* P, uint32_t x, uint32_t row, uint32_t band) {
  float sh = -P->sun_slope;
  int base = rb_floor_i(sh);
  float f = sh - (float)base;
  float s = 0.0f;
  size_t bo = (size_t)band * d.lw * d.lh + (size_t)row * d.lw;
  for (int k = 0; k < LIGHT_TAPS; k++) {
    int x0 = iclamp((int)x + k - LIGHT_TAPS / 2 + base, 0, d.lw - 1);
    int x1 = iclamp(x0 + 1, 0, d.lw - 1);
    s += rb_mix(d.light[bo + x0], d.light[bo + x1], f);
  }
  float cpos = (float)x + sh;
  float inside = rb_clamp(cpos + 1.0f, 0.0f, 1.0f) * rb_clamp((float)d.lw - cpos, 0.0f, 1.0f);
  return s / (float)LIGHT_TAPS * inside;
}
__device__ __forceinline__ float light_transmit(const Dev& d, const ribo_sim_params* P, uint32_t lx, uint32_t ly, uint32_t band) {
  float g = 0.0f;
  uint32_t m = 0;
  for (uint32_t dy = 0; dy < LIGHT_DIV; dy++)
    for (uint32_t dx = 0; dx < LIGHT_DIV; dx++) {
      size_t c = (size_t)(ly * LIGHT_DIV + dy) * d.gw + lx * LIGHT_DIV + dx;
      g += (float)d.gamma[c];
      m += cell_total4(load_cell(d.chem, c));
    }
  g = g / (float)LIGHT_DIV;
  float dens = (float)m / (float)(LIGHT_DIV * LIGHT_DIV);
  float tau_m = rb_max(P->monomer_uv_absorb, 0.0f) * dens * (float)LIGHT_DIV / (float)d.gh * (band == 1u ? (float)0.35 : 1.0f);
  float shd = (float)d.shade[(size_t)band * d.lw * d.lh + (size_t)ly * d.lw + lx] / SHADE_ONE;
  return rb_exp(-UV_SHADOW_ABSORB * g - AGENT_UV_ABSORB * shd - tau_m);
}
__device__ __forceinline__ float light_absorbed_at(const Dev& d, const ribo_sim_params* P, size_t env) {
  uint32_t lx = (uint32_t)(env % d.gw) / LIGHT_DIV;
  uint32_t ly = (uint32_t)(env / d.gw) / LIGHT_DIV;
  float incoming = P->sun_now;
  if (ly + 1u < (uint32_t)d.lh) incoming = light_above(d, P, lx, ly + 1u, 0u);
  incoming = rb_max(incoming, 0.0f);
  return incoming * ((1.0f - light_transmit(d, P, lx, ly, 0u)) + SUN_WATER_ABSORB);
}

// Status words written by kernels instead of trapping.
enum : uint32_t { ERR_NONE = 0, ERR_TIMEOUT = 1, ERR_BOUNDS = 2 };

// Index checks of the bounds-checked build (-DRB_BOUNDS_CHECK): RB_IN(i, n)
// is true when 0 <= i < n; otherwise it records ERR_BOUNDS in the world's
// status word and is false, and the caller skips the access.  In the normal
// build it is always true and costs nothing.
#ifdef RB_BOUNDS_CHECK
// The first failure of a launch sequence also prints its source line, index
// and bound (device printf, flushed at the next host synchronisation).
__device__ __forceinline__ bool rb_in_bounds(long long i, long long n, uint32_t* status, int line) {
  if (i >= 0 && i < n) return true;
  if (status) {
    atomicOr(status, ERR_BOUNDS);
    if (atomicCAS(status + 1, 0u, (uint32_t)line) == 0u)
      printf("index check failed at line %d: %lld not in [0, %lld)\n", line, i, n);
  }
  return false;
}
#define RB_IN(i, n, status) ::ribo::rb_in_bounds((long long)(i), (long long)(n), (status), __LINE__)
#else
#define RB_IN(i, n, status) true
#endif

// ---- Where a CTA works ------------------------------------------------------
// Block shapes of the passes, shared by the kernels and by the host code that
// sizes batched launches.
constexpr int PASS_BX = 32, PASS_BY = 8;        // per-cell passes: 32x8 cells per CTA
constexpr int FLUID_ROWS = 4;                   // streaming fluid passes: rows of cells per thread
constexpr int SCATTER_TX = 32, SCATTER_TY = 8;  // transport scatter tile
constexpr int NET_FLUX_LINES = 32;              // rows or columns per net-flux CTA
constexpr int LINEAR_THREADS = 256;             // 1-D passes over the environment cells
constexpr int LEDGER_CELLS_PER_CTA = 16 * LINEAR_THREADS;

// A pass over one world takes the world by value (kernel parameter space).
// A pass over a batch of worlds takes device tables: the worlds' Dev records
// and, for the block shape of that pass, the first linear block of every
// world and its blocks per row; a CTA finds its world by binary search over
// the block starts (six probes for 64 worlds) and works on one block of that
// world's grid, so every world gets exactly the CTAs a launch of its own
// would have.
struct OneWorld {
  Dev d;
  const ribo_sim_params* P;  // this step's parameters
  uint32_t* out;             // pass-specific output (12 ledger words), or null
};
struct WorldSet {
  const Dev* devs;           // [n]
  const int* start;          // [n + 1] first linear block of each world
  const int* nbx;            // [n] blocks per row of each world
  const ribo_sim_params* P;  // [n] this step's parameters of each world
  uint32_t* out;             // [n][12] pass-specific output, or null
  int n;
};
struct Cta {
  uint32_t bx, by;  // block coordinates in the world's grid
  uint32_t nbx;     // blocks per row of the world's grid
  int w;            // index of the world in the batch (0 for one world)
};

__device__ __forceinline__ Cta locate(const OneWorld& s, Dev& d, const ribo_sim_params*& P) {
  d = s.d;
  P = s.P;
  return Cta{blockIdx.x, blockIdx.y, gridDim.x, 0};
}
__device__ __forceinline__ int batch_member(const int* __restrict__ start, int n) {
  const int b = (int)blockIdx.x;
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(start + mid) <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}
__device__ __forceinline__ Cta locate(const WorldSet& s, Dev& d, const ribo_sim_params*& P) {
  const int w = batch_member(s.start, s.n);
  d = s.devs[w];
  P = s.P + w;
  const int r = (int)blockIdx.x - __ldg(s.start + w), nb = __ldg(s.nbx + w);
  return Cta{(uint32_t)(r % nb), (uint32_t)(r / nb), (uint32_t)nb, w};
}
__device__ __forceinline__ uint32_t* out_of(const OneWorld& s, int) { return s.out; }
__device__ __forceinline__ uint32_t* out_of(const WorldSet& s, int w) { return s.out ? s.out + (size_t)w * 12 : nullptr; }

// Opens a pass kernel: the world `d`, its step parameters `P` and the CTA's
// block coordinates `cta`.
#define RB_WORLD(sel)                  \
  Dev d;                               \
  const ribo_sim_params* P;            \
  const Cta cta = locate((sel), d, P); \
  (void)P;                             \
  (void)cta

}  // namespace ribo
