// Fluid passes of the world step (stable fluids at fluid resolution).
// Each kernel restates one WGSL entry point of shaders/world/fluid.wgsl,
// one thread per fluid cell, with the same float operation order.
#include <mutex>

#include "ribo_dev.cuh"
#include "ribo_launch.h"
#include "ribo_tma.cuh"
#include "ribo_world_impl.h"

namespace ribo {

namespace {

constexpr int BX = PASS_BX, BY = PASS_BY;

// fluid.wgsl:95-109,138-142,185-189
template <class S>
__global__ void k_solid_mask(const __grid_constant__ S s) {
  RB_WORLD(s);
  uint32_t x = cta.bx * BX + threadIdx.x, y = cta.by * BY + threadIdx.y;
  if (x >= (uint32_t)d.fw || y >= (uint32_t)d.fh) return;
  float gx = ((float)x + 0.5f) * d.sx, gy = ((float)y + 0.5f) * d.sy;
  float hx = d.sx * 0.25f, hy = d.sy * 0.25f;
  uint32_t n_solid = 0;
#pragma unroll
  for (uint32_t s = 0; s < 4; s++) {
    float ox = (s & 1u) == 1u ? hx : -hx;
    float oy = (s & 2u) == 2u ? hy : -hy;
    uint32_t sx = rb_f2u(rb_clamp(gx + ox, 0.0f, (float)(d.gw - 1)));
    uint32_t sy = rb_f2u(rb_clamp(gy + oy, 0.0f, (float)(d.gh - 1)));
    if (__ldg(d.gamma + (size_t)sy * d.gw + sx) >= GAMMA_SOLID) n_solid++;
  }
  float solidity = (float)n_solid * 0.25f;
  float perm = solidity >= 0.5f ? 0.0f : rb_clamp(1.0f - solidity * 2.0f, 0.0f, 1.0f);
  const bool solid = perm < SOLID_PERM_THRESHOLD;
  d.mask[(size_t)y * d.fw + x] = solid ? 1 : 0;
  if (d.fluid0) d.fluid0[(size_t)y * d.fw + x] = solid ? 0 : 1;  // multigrid level-0 water flags (mg_init)
}

// fluid.wgsl:196-216, evaluated once per mask build for every fluid cell.
template <class S>
__global__ void k_wall_normals(const __grid_constant__ S s) {
  RB_WORLD(s);
  uint32_t x = cta.bx * BX + threadIdx.x, y = cta.by * BY + threadIdx.y;
  if (x >= (uint32_t)d.fw || y >= (uint32_t)d.fh) return;
  d.normal[(size_t)y * d.fw + x] = solid_normal(d, x, y);
}

// fluid.wgsl:300-372 (update_temperature; copy_temperature becomes a
// pointer swap on the host, and the redox_eaten reset happens here after
// its single read).
template <class S>
__global__ void k_temperature(const __grid_constant__ S s) {
  RB_WORLD(s);
  uint32_t x = cta.bx * BX + threadIdx.x, y = cta.by * BY + threadIdx.y;
  if (x >= (uint32_t)d.fw || y >= (uint32_t)d.fh) return;
  const int fw = d.fw, fh = d.fh;
  size_t idx = (size_t)y * fw + x;
  const float dt = fluid_dt(P);
  const float* __restrict__ T = d.temp_in;   // temp_out and redox_out are the other buffers
  const float* __restrict__ R = d.redox_in;
  // the loads that do not depend on the velocity go out with it; only the
  // two bilinear gathers wait for it
  const uint8_t solid = __ldg(d.mask + idx);
  const float2 v_raw = __ldg(d.va + idx);
  uint32_t xl = x > 0u ? x - 1u : 0u, xr = umin(x + 1u, (uint32_t)fw - 1u);
  uint32_t yb = y > 0u ? y - 1u : 0u, yt = umin(y + 1u, (uint32_t)fh - 1u);
  const float tl = __ldg(T + (size_t)y * fw + xl), tr = __ldg(T + (size_t)y * fw + xr);
  const float tb = __ldg(T + (size_t)yb * fw + x), tt = __ldg(T + (size_t)yt * fw + x);
  const float rl = __ldg(R + (size_t)y * fw + xl), rr = __ldg(R + (size_t)y * fw + xr);
  const float rbt = __ldg(R + (size_t)yb * fw + x), rt = __ldg(R + (size_t)yt * fw + x);
  const float2 h = __ldg(d.heat + idx);
  const uint32_t eaten = d.redox_eaten[idx];
  const float fill = gamma_fill_at_fluid_cell(d, x, y);
  float2 vel = solid ? f2(0.0f, 0.0f) : sanitize(v_raw);  // raw_velocity_cell
  float srcx = ((float)x + 0.5f) - vel.x * dt;
  float srcy = ((float)y + 0.5f) - vel.y * dt;
  float sxf = rb_clamp(srcx - 0.5f, 0.0f, (float)(fw - 1));
  float syf = rb_clamp(srcy - 0.5f, 0.0f, (float)(fh - 1));
  uint32_t x0 = rb_f2u(rb_floor(sxf)), y0 = rb_f2u(rb_floor(syf));
  uint32_t x1 = umin(x0 + 1u, (uint32_t)fw - 1u), y1 = umin(y0 + 1u, (uint32_t)fh - 1u);
  float fx = rb_fract(sxf), fy = rb_fract(syf);
  const float t00 = __ldg(T + (size_t)y0 * fw + x0), t01 = __ldg(T + (size_t)y0 * fw + x1);
  const float t10 = __ldg(T + (size_t)y1 * fw + x0), t11 = __ldg(T + (size_t)y1 * fw + x1);
  const float r00 = __ldg(R + (size_t)y0 * fw + x0), r01 = __ldg(R + (size_t)y0 * fw + x1);
  const float r10 = __ldg(R + (size_t)y1 * fw + x0), r11 = __ldg(R + (size_t)y1 * fw + x1);
  float t = rb_mix(rb_mix(t00, t01, fx), rb_mix(t10, t11, fx), fy);
  t = rb_mix(t, (tl + tr + tb + tt) * 0.25f, TEMP_DIFFUSE * rb_mix(1.0f, TEMP_ROCK_CONDUCT, fill));
  // The vent cycle only scales vent heat.  It is finite and >= +0 for a
  // finite amplitude, so with no heat here both products are zeros of the
  // heat's signs whatever its value, and the sine is not evaluated.
  const float vc = (h.x != 0.0f || h.y != 0.0f || !(P->vent_cycle_amp <= 3.0e38f)) ? vent_cycle(d, P, x) : 1.0f;
  t += h.x * vc * TEMP_HEAT_RATE * dt;
  if (rb_max(P->sun_heat, 0.0f) > 0.0f) {  // otherwise the sun term is exactly 0
    size_t env = env_cell_for_fluid(d, x, y);
    float depth = 1.0f - ((float)y + 0.5f) / (float)fh;
    float ir = P->sun_now * SUN_IR * rb_exp(-depth / SUN_IR_DEPTH);
    t += rb_max(P->sun_heat, 0.0f) * SUN_HEAT_RATE * (light_absorbed_at(d, P, env) + ir) * dt;
  }
  float amb = temp_ambient_at(d, y);
  // dt is finite in [0, MAX_DT] and fill in [0, 1], so the cooling factor is
  // finite; with the ambient +0 a zero temperature stays +0 without it.
  if (TEMP_AMBIENT_SURFACE == 0.0f && t == 0.0f) t = 0.0f;
  else t = amb + (t - amb) * rb_exp(-TEMP_COOL_RATE * (1.0f - fill) * dt);
  d.temp_out[idx] = rb_clamp(t, 0.0f, TEMP_MAX);

  float r = rb_mix(rb_mix(r00, r01, fx), rb_mix(r10, r11, fx), fy);
  r = rb_mix(r, (rl + rr + rbt + rt) * 0.25f, TEMP_DIFFUSE);
  r += h.y * vc * REDOX_RATE * dt;
  r = rb_max(r - (float)eaten / REDOX_FP, 0.0f);
  // a zero times a finite factor in [0, 1] keeps its sign: skip the exponential
  const float decay_arg = -rb_max(P->redox_decay, 0.0f) * dt;
  if (r != 0.0f || !(decay_arg <= 0.0f)) r *= rb_exp(decay_arg);
  d.redox_out[idx] = rb_clamp(r, 0.0f, REDOX_MAX);
  d.redox_eaten[idx] = 0u;
}

// fluid.wgsl:280-296,376-404: buoyancy adds into the fixed-point force
// accumulators (each interior cell writes only its own slots, so the add
// needs no atomics), gather_forces converts and clamps them, and
// clear_force_vectors zeroes them -- all in one pass.
__device__ __forceinline__ uint32_t quant_force(float v) {
  int32_t q = rb_f2i(rb_rint(rb_clamp(v, (float)-1.0e5, (float)1.0e5) * FORCE_FP));
  return (uint32_t)q;
}
template <class S>
__global__ void k_forces(const __grid_constant__ S s) {
  RB_WORLD(s);
  const uint32_t x = cta.bx * BX + threadIdx.x, y0 = cta.by * (BY * FLUID_ROWS) + threadIdx.y;
  if (x >= (uint32_t)d.fw) return;
  // FLUID_ROWS cells of the column, every load first (see k_smooth)
  uint2 fv[FLUID_ROWS];
  float tc[FLUID_ROWS];
#pragma unroll
  for (int r = 0; r < FLUID_ROWS; r++) {
    const uint32_t y = umin(y0 + r * BY, (uint32_t)d.fh - 1u);
    const size_t idx = (size_t)y * d.fw + x;
    fv[r] = reinterpret_cast<const uint2*>(d.force_vec)[idx];
    tc[r] = d.temp_in[idx];
  }
#pragma unroll
  for (int r = 0; r < FLUID_ROWS; r++) {
    const uint32_t y = y0 + r * BY;
    if (y >= (uint32_t)d.fh) break;
    const size_t idx = (size_t)y * d.fw + x;
    uint2 v = fv[r];
    if (!(x == 0u || y == 0u || x >= (uint32_t)d.fw - 1u || y >= (uint32_t)d.fh - 1u)) {
      float dev = tc[r] - temp_ambient_at(d, y);
      if (!(rb_abs(dev) <= (float)1e-3)) {
        uint32_t time_bucket = P->epoch / 16u;
        float rr = rb_u2f(rb_pcg4d((uint32_t)idx, time_bucket, RB_S_BUOYANCY, P->seed).x);
        float side = (rr * 2.0f - 1.0f) * 0.25f * rb_abs(dev) / rb_max(rb_abs(dev), 1.0f);
        v.x += quant_force(side * TEMP_BUOYANCY * rb_abs(dev));
        v.y += quant_force(TEMP_BUOYANCY * dev);
      }
    }
    float2 f = f2((float)(int32_t)v.x / FORCE_FP, (float)(int32_t)v.y / FORCE_FP);
    d.forces[idx] = clamp_len(sanitize(f), MAX_FORCE);
    reinterpret_cast<uint2*>(d.force_vec)[idx] = make_uint2(0u, 0u);
  }
}

// fluid.wgsl:150-161
__device__ __forceinline__ float rubble_drag(const Dev& d, uint32_t x, uint32_t y, float dt) {
  float g = 0.0f;
  for (int dy = 0; dy < d.ry; dy++)
    for (int dx = 0; dx < d.rx; dx++) {
      uint32_t c = __ldg(d.gamma + (size_t)(y * d.ry + dy) * d.gw + x * d.rx + dx);
      if (c < GAMMA_SOLID) g += (float)c;
    }
  if (g == 0.0f) return 1.0f;  // 1 / (1 + 0): no rubble under the cell
  g = g / ((float)(d.rx * d.ry) * (float)GAMMA_SOLID);
  return 1.0f / (1.0f + RUBBLE_DRAG * g * dt);
}
// fluid.wgsl:165-178
__device__ __forceinline__ float2 slope_steer(const Dev& d, const ribo_sim_params* P, uint32_t x, uint32_t y, float2 v_in, float dt) {
  float2 s0 = sanitize(d.slope[env_cell_for_fluid(d, x, y)]);
  if (s0.x == 0.0f && s0.y == 0.0f) return v_in;  // s_len = 0 < 1e-5
  float2 s = f2(-s0.x, -s0.y);
  float v_len = len2(v_in), s_len = len2(s);
  if (v_len < (float)1e-5 || s_len < (float)1e-5) return v_in;
  float2 v_dir = div2(v_in, v_len), s_dir = div2(s, s_len);
  float misalign = rb_clamp(1.0f - dot2(v_dir, s_dir), 0.0f, 2.0f);
  float t = rb_clamp(1.0f - rb_exp(-rb_max(P->slope_steer_rate, 0.0f) * misalign * dt), 0.0f, 1.0f);
  float2 dir_raw = add2(v_dir, mul2(sub2(s_dir, v_dir), t));
  float dir_len = len2(dir_raw);
  if (dir_len < (float)1e-5) return v_in;
  return mul2(div2(dir_raw, dir_len), v_len);
}

// fluid.wgsl:410-432 (add_forces; clear_forces is dropped: gather
// overwrites every fluid_forces entry before the next read)
// The gathered forces of the tile and its ring are staged in shared memory
// (a TMA box), so the 3 x 3 average reads them there.
template <class S>
__global__ void k_add_forces(const __grid_constant__ S s, int dir) {
  RB_WORLD(s);
  __shared__ __align__(128) uint2 FB[ST_BOX];
  __shared__ uint64_t bar;
  const int x0 = (int)(cta.bx * BX), y0 = (int)(cta.by * BY);
  {
    const int map[1] = {SM_FORCES};
    const uint2* const src[1] = {reinterpret_cast<const uint2*>(d.forces)};
    uint2* const box[1] = {FB};
    if (!stage_stencil<1>(d.tmap, map, src, box, x0, y0, d.fw, d.fh, &bar, d.status)) return;
  }
  const float2* __restrict__ vin = dir ? d.vb : d.va;
  float2* __restrict__ vout = dir ? d.va : d.vb;
  uint32_t x = x0 + threadIdx.x, y = y0 + threadIdx.y;
  if (x >= (uint32_t)d.fw || y >= (uint32_t)d.fh) return;
  const int fw = d.fw;
  size_t idx = (size_t)y * fw + x;
  // every load issued before any selection (the wall test included)
  const uint8_t mc = __ldg(d.mask + idx);
  const float2 vc = __ldg(vin + idx), n = __ldg(d.normal + idx);
  const float dt = fluid_dt(P);
  uint32_t xm = x > 0u ? x - 1u : x, xp = x + 1u < (uint32_t)fw ? x + 1u : x;
  uint32_t ym = y > 0u ? y - 1u : y, yp = y + 1u < (uint32_t)d.fh ? y + 1u : y;
  const float2* Ff = reinterpret_cast<const float2*>(FB);
  auto F = [&](uint32_t a, uint32_t b) { return sanitize(Ff[st_at(x0, y0, (int)a, (int)b)]); };
  float2 f_c = F(x, y);
  float2 axis = add2(add2(add2(F(xm, y), F(xp, y)), F(x, ym)), F(x, yp));
  float2 diag = add2(add2(add2(F(xm, ym), F(xp, ym)), F(xm, yp)), F(xp, yp));
  float2 f_avg = mul2(add2(add2(smul2(4.0f, axis), diag), smul2(20.0f, f_c)), (float)(1.0 / 36.0));
  float2 f_user = clamp_len(mix2(f_c, f_avg, FORCE_SMOOTH_MIX), MAX_FORCE);
  float2 v = sanitize(add2(sanitize(vc), mul2(f_user, dt)));
  v = slope_steer(d, P, x, y, v, dt);
  const float drag = rubble_drag(d, x, y, dt);
  if (drag != 1.0f) v = mul2(v, drag);  // v * 1 is v
  v = reflect_stored(n, v);
  vout[idx] = mc ? f2(0.0f, 0.0f) : clamp_len(v, MAX_VEL);
}

// fluid.wgsl:435-456
template <class S>
__global__ void k_diffuse(const __grid_constant__ S s, int dir) {
  RB_WORLD(s);
  const float2* __restrict__ vin = dir ? d.vb : d.va;
  float2* __restrict__ vout = dir ? d.va : d.vb;
  uint32_t x = cta.bx * BX + threadIdx.x, y = cta.by * BY + threadIdx.y;
  if (x >= (uint32_t)d.fw || y >= (uint32_t)d.fh) return;
  const size_t fw = (size_t)d.fw, idx = (size_t)y * fw + x;
  const bool border = x == 0u || x == (uint32_t)d.fw - 1u || y == 0u || y == (uint32_t)d.fh - 1u;
  // the 3 x 3 block (clamped at the border, where the result is the copy)
  const size_t cl = x > 0u ? 1 : 0, cr = x + 1u < (uint32_t)d.fw ? 1 : 0;
  const size_t rb = y > 0u ? fw : 0, rt = y + 1u < (uint32_t)d.fh ? fw : 0;
  const size_t at[9] = {idx, idx - cl, idx + cr, idx - rb, idx + rt, idx - rb - cl, idx - rb + cr, idx + rt - cl, idx + rt + cr};
  uint8_t m[9];
  float2 v[9];
#pragma unroll
  for (int k = 0; k < 9; k++) {
    m[k] = __ldg(d.mask + at[k]);
    v[k] = __ldg(vin + at[k]);
  }
  const float2 n = __ldg(d.normal + idx);
  float2 r[9];  // raw_velocity_cell
#pragma unroll
  for (int k = 0; k < 9; k++) r[k] = m[k] ? f2(0.0f, 0.0f) : sanitize(v[k]);
  const float2 v_c = r[0];
  const float2 axis_sum = add2(add2(add2(r[1], r[2]), r[3]), r[4]);
  const float2 diag_sum = add2(add2(add2(r[5], r[6]), r[7]), r[8]);
  const float2 lap = mul2(sub2(add2(smul2(4.0f, axis_sum), diag_sum), smul2(20.0f, v_c)), (float)(1.0 / 6.0));
  const float a = rb_max(P->fluid_viscosity, 0.0f) * fluid_dt(P);
  float2 vv = sanitize(add2(v_c, smul2(a, lap)));
  vv = reflect_stored(n, vv);
  vout[idx] = m[0] ? f2(0.0f, 0.0f) : (border ? v[0] : clamp_len(vv, MAX_VEL));
}

// fluid.wgsl:226-255
__device__ __forceinline__ bool is_solid_at_pos(const Dev& d, float2 pos) {
  int ix = rb_floor_i(pos.x - 0.5f);
  int iy = rb_floor_i(pos.y - 0.5f);
  if (ix < 0 || ix >= d.fw || iy < 0 || iy >= d.fh) return true;
  return is_solid(d, ix, iy);
}
__device__ __forceinline__ float2 sample_velocity(const Dev& d, const float2* vin, float2 pos) {
  float max_x = (float)d.fw - 0.5f, max_y = (float)d.fh - 0.5f;
  if (pos.x < 0.5f || pos.x > max_x || pos.y < 0.5f || pos.y > max_y) return f2(0.0f, 0.0f);
  float x = pos.x - 0.5f, y = pos.y - 0.5f;
  int x0 = rb_floor_i(x), y0 = rb_floor_i(y);
  float fx = rb_fract(x), fy = rb_fract(y);
  uint32_t cx0 = iclamp(x0, 0, d.fw - 1), cx1 = iclamp(x0 + 1, 0, d.fw - 1);
  uint32_t cy0 = iclamp(y0, 0, d.fh - 1), cy1 = iclamp(y0 + 1, 0, d.fh - 1);
  float2 v0 = mix2(raw_velocity_cell(d, vin, cx0, cy0), raw_velocity_cell(d, vin, cx1, cy0), fx);
  float2 v1 = mix2(raw_velocity_cell(d, vin, cx0, cy1), raw_velocity_cell(d, vin, cx1, cy1), fx);
  return mix2(v0, v1, fy);
}
// fluid.wgsl:458-477
template <class S>
__global__ void k_advect(const __grid_constant__ S s, int dir) {
  RB_WORLD(s);
  const float2* __restrict__ vin = dir ? d.vb : d.va;
  float2* __restrict__ vout = dir ? d.va : d.vb;
  // the step's decay factor, one evaluation per CTA (every thread would
  // compute the same value)
  __shared__ float decay_shared;
  if (threadIdx.x == 0 && threadIdx.y == 0) decay_shared = rb_pow(rb_clamp(P->fluid_decay, 0.0f, 1.0f), fluid_dt(P) * 60.0f);
  __syncthreads();
  uint32_t x = cta.bx * BX + threadIdx.x, y = cta.by * BY + threadIdx.y;
  if (x >= (uint32_t)d.fw || y >= (uint32_t)d.fh) return;
  size_t idx = (size_t)y * d.fw + x;
  // the cell's own loads together, the wall test at the end
  const uint8_t mc = __ldg(d.mask + idx);
  const float2 vc = __ldg(vin + idx), n = __ldg(d.normal + idx);
  const float dt = fluid_dt(P);
  const float decay_factor = decay_shared;
  float2 pos = f2((float)x + 0.5f, (float)y + 0.5f);
  float2 vel = reflect_stored(n, clamp_len(sanitize(vc), MAX_VEL));  // raw_velocity_cell of a water cell
  float2 trace_pos = sub2(pos, mul2(vel, dt));
  if (is_solid_at_pos(d, trace_pos)) trace_pos = sub2(pos, mul2(reflect_stored(n, vel), dt));
  float2 out_v = sanitize(mul2(sample_velocity(d, vin, trace_pos), decay_factor));
  out_v = reflect_stored(n, out_v);
  vout[idx] = mc ? f2(0.0f, 0.0f) : clamp_len(out_v, MAX_VEL);
}

// fluid.wgsl:479-518
// curl_at for every fluid cell (input of the confinement pass).  Each
// neighbour term reflect_if_into_solid(raw_velocity_cell(n)) is a function
// of the neighbour alone: the CTA computes it once for its tile and the
// 1-cell ring (coordinates clamped to the grid as curl_at clamps them, so a
// clamped neighbour is the cell itself) and reads the four terms from there.
template <class S>
__global__ void k_curl(const __grid_constant__ S s, int dir) {
  RB_WORLD(s);
  const float2* __restrict__ vin = dir ? d.vb : d.va;
  __shared__ float2 u[BY + 2][BX + 2];
  const int x0 = cta.bx * BX, y0 = cta.by * BY, tid = threadIdx.y * BX + threadIdx.x;
  for (int i = tid; i < (BX + 2) * (BY + 2); i += BX * BY) {
    const int tx = i % (BX + 2), ty = i / (BX + 2);
    const size_t n = (size_t)iclamp(y0 + ty - 1, 0, d.fh - 1) * d.fw + iclamp(x0 + tx - 1, 0, d.fw - 1);
    const uint8_t m = __ldg(d.mask + n);
    const float2 v = __ldg(vin + n), wn = __ldg(d.normal + n);
    u[ty][tx] = reflect_stored(wn, m ? f2(0.0f, 0.0f) : sanitize(v));
  }
  __syncthreads();
  const uint32_t x = x0 + threadIdx.x, y = y0 + threadIdx.y;
  if (x >= (uint32_t)d.fw || y >= (uint32_t)d.fh) return;
  const int tx = threadIdx.x + 1, ty = threadIdx.y + 1;
  const float2 v_l = u[ty][tx - 1], v_r = u[ty][tx + 1], v_b = u[ty - 1][tx], v_t = u[ty + 1][tx];
  d.curl[(size_t)y * d.fw + x] = 0.5f * (v_r.y - v_l.y) - 0.5f * (v_t.x - v_b.x);
}
template <class S>
__global__ void k_vorticity(const __grid_constant__ S s, int dir) {
  RB_WORLD(s);
  const float2* __restrict__ vin = dir ? d.vb : d.va;
  float2* __restrict__ vout = dir ? d.va : d.vb;
  uint32_t x = cta.bx * BX + threadIdx.x, y = cta.by * BY + threadIdx.y;
  if (x >= (uint32_t)d.fw || y >= (uint32_t)d.fh) return;
  const size_t fw = (size_t)d.fw, idx = (size_t)y * fw + x;
  const float epsilon = rb_clamp(P->fluid_vorticity, 0.0f, 10.0f);
  const uint32_t border = 2u;
  const bool copy = x < border || x >= (uint32_t)d.fw - border || y < border || y >= (uint32_t)d.fh - border ||
                    epsilon < (float)1e-6;
  // curl_at of this cell and its 4 neighbours, precomputed once per cell by
  // k_curl (the same function of the same inputs, so the same bits); the
  // neighbour addresses are clamped where the cell is copied anyway
  const size_t il = x > 0u ? idx - 1 : idx, ir = x + 1u < (uint32_t)d.fw ? idx + 1 : idx;
  const size_t ib = y > 0u ? idx - fw : idx, it = y + 1u < (uint32_t)d.fh ? idx + fw : idx;
  const float* __restrict__ cu = d.curl;
  const uint8_t mc = __ldg(d.mask + idx);
  const float w = __ldg(cu + idx), cl = __ldg(cu + il), cr = __ldg(cu + ir), cb = __ldg(cu + ib), ct = __ldg(cu + it);
  const float2 vc = __ldg(vin + idx), n_wall = __ldg(d.normal + idx);
  float2 grad = mul2(f2(rb_abs(cr) - rb_abs(cl), rb_abs(ct) - rb_abs(cb)), 0.5f);
  float2 n = div2(grad, rb_max(len2(grad), (float)1e-5));
  float2 f = mul2(f2(n.y, -n.x), w * epsilon);
  float2 dv = clamp_len(mul2(f, fluid_dt(P)), 2.0f);
  float2 v = sanitize(add2(vc, dv));
  v = reflect_stored(n_wall, v);
  vout[idx] = mc ? f2(0.0f, 0.0f) : ((copy || rb_abs(w) < (float)5e-4) ? vc : clamp_len(v, MAX_VEL));
}

// fluid.wgsl:520-551
// The stencil passes below issue every global load of a cell first (border
// neighbours clamped to the cell itself, so every address is in the grid)
// and select afterwards: one load latency per cell instead of a chain of
// mask -> neighbour mask -> value.  A wall cell's value is computed and
// discarded; a water cell's is the same expression as the branching form.
template <class S>
__global__ void k_divergence(const __grid_constant__ S s, int dir) {
  RB_WORLD(s);
  const float2* __restrict__ vin = dir ? d.vb : d.va;
  int x = cta.bx * BX + threadIdx.x, y = cta.by * BY + threadIdx.y;
  if (x >= d.fw || y >= d.fh) return;
  const size_t fw = (size_t)d.fw, idx = (size_t)y * fw + x;
  const bool hl = x > 0, hr = x + 1 < d.fw, hb = y > 0, ht = y + 1 < d.fh;
  const size_t il = hl ? idx - 1 : idx, ir = hr ? idx + 1 : idx, ib = hb ? idx - fw : idx, it = ht ? idx + fw : idx;
  const uint8_t mc = __ldg(d.mask + idx), ml = __ldg(d.mask + il), mr = __ldg(d.mask + ir);
  const uint8_t mb = __ldg(d.mask + ib), mt = __ldg(d.mask + it);
  const float2 vc = __ldg(vin + idx), vl = __ldg(vin + il), vr = __ldg(vin + ir), vb = __ldg(vin + ib), vt = __ldg(vin + it);
  // div_neighbor: the border or a wall mirrors the cell's own velocity
  const float2 v_c = sanitize(vc);
  const float2 v_l = (!hl || ml) ? f2(-v_c.x, v_c.y) : sanitize(vl);
  const float2 v_r = (!hr || mr) ? f2(-v_c.x, v_c.y) : sanitize(vr);
  const float2 v_b = (!hb || mb) ? f2(v_c.x, -v_c.y) : sanitize(vb);
  const float2 v_t = (!ht || mt) ? f2(v_c.x, -v_c.y) : sanitize(vt);
  d.div[idx] = mc ? 0.0f : 0.5f * ((v_r.x - v_l.x) + (v_t.y - v_b.y));
}

// fluid.wgsl:610-630
template <class S>
__global__ void k_subtract_gradient(const __grid_constant__ S s, int dir) {
  RB_WORLD(s);
  const float2* __restrict__ vin = dir ? d.vb : d.va;
  float2* __restrict__ vout = dir ? d.va : d.vb;
  uint32_t x = cta.bx * BX + threadIdx.x, y = cta.by * BY + threadIdx.y;
  if (x >= (uint32_t)d.fw || y >= (uint32_t)d.fh) return;
  const size_t fw = (size_t)d.fw, idx = (size_t)y * fw + x;
  const bool hl = x > 0u, hr = x + 1u < (uint32_t)d.fw, hb = y > 0u, ht = y + 1u < (uint32_t)d.fh;
  const size_t il = hl ? idx - 1 : idx, ir = hr ? idx + 1 : idx, ib = hb ? idx - fw : idx, it = ht ? idx + fw : idx;
  const float* __restrict__ p = d.pa;
  const uint8_t mc = __ldg(d.mask + idx), ml = __ldg(d.mask + il), mr = __ldg(d.mask + ir);
  const uint8_t mb = __ldg(d.mask + ib), mt = __ldg(d.mask + it);
  const float p_c = __ldg(p + idx), pl = __ldg(p + il), pr = __ldg(p + ir), pb = __ldg(p + ib), pt = __ldg(p + it);
  const float2 vc = __ldg(vin + idx), n = __ldg(d.normal + idx);
  // a wall or the border neighbour takes the cell's own pressure
  const float p_l = (hl && !ml) ? pl : p_c, p_r = (hr && !mr) ? pr : p_c;
  const float p_b = (hb && !mb) ? pb : p_c, p_t = (ht && !mt) ? pt : p_c;
  float2 grad = mul2(f2(p_r - p_l, p_t - p_b), 0.5f);
  float2 v = sub2(sanitize(vc), grad);
  v = reflect_stored(n, v);
  vout[idx] = mc ? f2(0.0f, 0.0f) : clamp_len(sanitize(v), MAX_VEL);
}

// fluid.wgsl:640-657.  The reference sums each row (column) serially in
// f32; the order of those adds fixes the rounding, so each line is summed
// by one lane in index order.  A block owns 32 lines: its warps 1..15 stream
// chunks of NF_C elements of those lines into a double-buffered shared
// tile, while warp 0 (lane = line) runs the 32 serial add chains over the
// previous chunk (the double buffer lives in dynamic shared memory).  A
// chunk is NF_C units of one coalesced warp load (32
// cells of a row, or one position of the 32 columns); a loader warp issues
// all its units' loads before storing any, so a chunk costs about one load
// latency.  Wall cells are stored as +0.0: the running sum starts at +0.0
// and never becomes -0.0 in round-to-nearest, so adding +0.0 leaves it
// unchanged, and the chain needs no branch; the water cells are counted
// separately (the reference's n, an exact integer in f32).  Row blocks and
// column blocks share one launch.
constexpr int NF_L = NET_FLUX_LINES, NF_C = 256, NF_THREADS = 512;
constexpr size_t NF_SMEM = (size_t)2 * NF_L * (NF_C + 1) * sizeof(float);
constexpr int NF_LOADERS = NF_THREADS / 32 - 1, NF_UPW = (NF_C + NF_LOADERS - 1) / NF_LOADERS;
static_assert(NF_L == 32 && NF_C % 32 == 0, "a unit is one warp load");
template <class S>
__global__ void __launch_bounds__(NF_THREADS) k_net_flux(const __grid_constant__ S s, int dir) {
  RB_WORLD(s);
  const float2* __restrict__ vin = dir ? d.vb : d.va;
  const uint8_t* __restrict__ mask = d.mask;
  const int row_blocks = (d.fh + NF_L - 1) / NF_L;
  extern __shared__ float nf_smem[];
  float(*val)[NF_L][NF_C + 1] = reinterpret_cast<float(*)[NF_L][NF_C + 1]>(nf_smem);
  __shared__ uint32_t wet_cells[NF_L];
  const bool rows = (int)cta.bx < row_blocks;
  const int line0 = (rows ? (int)cta.bx : (int)cta.bx - row_blocks) * NF_L;
  const int nlines = rows ? d.fh : d.fw;
  const int len = rows ? d.fw : d.fh;
  const int nchunks = (len + NF_C - 1) / NF_C;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x < NF_L) wet_cells[threadIdx.x] = 0u;
  uint32_t my_wet = 0;  // column blocks: water cells of line `lane` seen by this loader

  // unit u of a row block: line u / (NF_C / 32), cells 32 (u % (NF_C / 32)) + lane
  // of the chunk; of a column block: position u of line `lane`
  auto load = [&](int c, int b, int lw) {
    const int k0 = c * NF_C;
    float2 sv[NF_UPW];
    uint8_t wall[NF_UPW];
    bool in[NF_UPW];
#pragma unroll
    for (int q = 0; q < NF_UPW; q++) {  // loads only, all in flight together
      const int u = lw + NF_LOADERS * q;
      const int l = rows ? u / (NF_C / 32) : lane, k = rows ? (u % (NF_C / 32)) * 32 + lane : u;
      const int line = line0 + l, pos = k0 + k;
      in[q] = u < NF_C && line < nlines && pos < len;
      const size_t i = in[q] ? (rows ? (size_t)line * d.fw + pos : (size_t)pos * d.fw + line) : 0;
      sv[q] = __ldg(vin + i);
      wall[q] = __ldg(mask + i);
    }
#pragma unroll
    for (int q = 0; q < NF_UPW; q++) {
      const int u = lw + NF_LOADERS * q;
      if (u >= NF_C) continue;  // uniform over the warp
      const int l = rows ? u / (NF_C / 32) : lane, k = rows ? (u % (NF_C / 32)) * 32 + lane : u;
      const bool wet_q = in[q] && !wall[q];
      const float2 s2 = sanitize(sv[q]);
      val[b][l][k] = wet_q ? (rows ? s2.y : s2.x) : 0.0f;
      if (rows) {
        const uint32_t m = __ballot_sync(0xffffffffu, wet_q);
        if (lane == 0 && m) atomicAdd(&wet_cells[l], (uint32_t)__popc(m));
      } else {
        my_wet += wet_q ? 1u : 0u;
      }
    }
  };

  __syncthreads();
  if (warp > 0) load(0, 0, warp - 1);
  __syncthreads();
  float sum = 0.0f;
  for (int c = 0; c < nchunks; c++) {
    const int b = c & 1;
    if (warp == 0) {
#pragma unroll 16
      for (int k = 0; k < NF_C; k++) sum += val[b][lane][k];
    } else if (c + 1 < nchunks) {
      load(c + 1, b ^ 1, warp - 1);
    }
    __syncthreads();
  }
  if (!rows && warp > 0 && my_wet) atomicAdd(&wet_cells[lane], my_wet);
  __syncthreads();
  const float n = (float)wet_cells[lane];
  if (warp == 0 && line0 + lane < nlines) d.net_flux[(rows ? 0 : d.fh) + line0 + lane] = n > 0.0f ? sum / n : 0.0f;
}

// fluid.wgsl:663-677
template <class S>
__global__ void k_boundaries(const __grid_constant__ S s, int dir) {
  RB_WORLD(s);
  const float2* __restrict__ vin = dir ? d.vb : d.va;
  float2* __restrict__ vout = dir ? d.va : d.vb;
  const uint32_t x = cta.bx * BX + threadIdx.x, y0 = cta.by * (BY * FLUID_ROWS) + threadIdx.y;
  if (x >= (uint32_t)d.fw) return;
  const float fx = __ldg(d.net_flux + d.fh + x);
  uint8_t mc[FLUID_ROWS];
  float2 vc[FLUID_ROWS], n[FLUID_ROWS];
  float fy[FLUID_ROWS];
#pragma unroll
  for (int r = 0; r < FLUID_ROWS; r++) {
    const uint32_t y = umin(y0 + r * BY, (uint32_t)d.fh - 1u);
    const size_t idx = (size_t)y * d.fw + x;
    mc[r] = __ldg(d.mask + idx);
    vc[r] = __ldg(vin + idx);
    n[r] = __ldg(d.normal + idx);
    fy[r] = __ldg(d.net_flux + y);
  }
#pragma unroll
  for (int r = 0; r < FLUID_ROWS; r++) {
    const uint32_t y = y0 + r * BY;
    if (y >= (uint32_t)d.fh) break;
    float2 v = sanitize(vc[r]);
    v = sub2(v, f2(fx, fy[r]));
    if (x == 0u || x == (uint32_t)d.fw - 1u) v.x = 0.0f;
    if (y == 0u || y == (uint32_t)d.fh - 1u) v.y = 0.0f;
    v = reflect_stored(n[r], v);
    vout[(size_t)y * d.fw + x] = mc[r] ? f2(0.0f, 0.0f) : clamp_len(sanitize(v), MAX_VEL);
  }
}

// fluid.wgsl:680-693
// The streaming passes below take FLUID_ROWS cells of a column per thread
// (rows BY apart) and load all of them before computing any: four cells'
// loads in flight per thread instead of one.  Rows past the grid load the
// last row and store nothing.
template <class S>
__global__ void k_smooth(const __grid_constant__ S s, int dir) {
  RB_WORLD(s);
  const float2* __restrict__ vin = dir ? d.vb : d.va;
  const uint32_t x = cta.bx * BX + threadIdx.x, y0 = cta.by * (BY * FLUID_ROWS) + threadIdx.y;
  if (x >= (uint32_t)d.fw) return;
  const int fw = d.fw;
  const uint32_t xm = x > 0u ? x - 1u : x, xp = umin(x + 1u, (uint32_t)fw - 1u);
  float2 v[FLUID_ROWS][5];
#pragma unroll
  for (int r = 0; r < FLUID_ROWS; r++) {
    const uint32_t y = umin(y0 + r * BY, (uint32_t)d.fh - 1u);
    const uint32_t ym = y > 0u ? y - 1u : y, yp = umin(y + 1u, (uint32_t)d.fh - 1u);
    v[r][0] = __ldg(vin + (size_t)y * fw + x);
    v[r][1] = __ldg(vin + (size_t)y * fw + xm);
    v[r][2] = __ldg(vin + (size_t)y * fw + xp);
    v[r][3] = __ldg(vin + (size_t)ym * fw + x);
    v[r][4] = __ldg(vin + (size_t)yp * fw + x);
  }
#pragma unroll
  for (int r = 0; r < FLUID_ROWS; r++) {
    const uint32_t y = y0 + r * BY;
    if (y >= (uint32_t)d.fh) break;
    const float2 a = add2(add2(add2(add2(sanitize(v[r][0]), sanitize(v[r][1])), sanitize(v[r][2])), sanitize(v[r][3])),
                          sanitize(v[r][4]));
    d.vsmooth[(size_t)y * fw + x] = mul2(a, 0.2f);
  }
}

// One CTA that waits on an mbarrier phase nothing completes (one arrival
// expected, with 16 bytes of transactions that no copy delivers): the wait
// gives up after `polls` polls and records a timeout, as a kernel's bounded
// wait on a bulk copy would.
__global__ void k_selftest_bounded_wait(uint32_t polls, uint32_t* status) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_arrive_expect(&bar, 16u);
  }
  __syncthreads();
  const bool late = !mbar_wait(&bar, 0u, polls);
  if (__syncthreads_or(late) && threadIdx.x == 0) atomicOr(status, ERR_TIMEOUT);
}

}  // namespace

ribo_status selftest_bounded_wait(int device, uint32_t polls, uint32_t* bits) {
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_status(e, "device");
  uint32_t* d_status = nullptr;
  e = cudaMalloc((void**)&d_status, 4);
  if (e != cudaSuccess) return cuda_status(e, "selftest");
  e = cudaMemset(d_status, 0, 4);
  if (e == cudaSuccess) {
    k_selftest_bounded_wait<<<1, 32>>>(polls, d_status);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(bits, d_status, 4, cudaMemcpyDeviceToHost);
  cudaFree(d_status);
  return cuda_status(e, "selftest");
}

// One descriptor per staged 8-byte field: dimensions (fw, fh), row pitch
// fw * 8 bytes, the ST_BW x ST_BH box, zero fill outside the field.  The pitch
// must be a multiple of 16 bytes (fw even), the fields 16-byte aligned and the
// descriptors' home 64-byte aligned; otherwise the passes use plain loads.
bool stencil_tensor_maps(void* dst, const StencilFields& f, cudaStream_t s) {
  using Encode = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*,
                              const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                              CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  static Encode encode = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      encode = reinterpret_cast<Encode>(fn);
    cudaGetLastError();
  });
  if (!encode || f.fw % 2 != 0 || f.fw < 1 || f.fh < 1 || (reinterpret_cast<uintptr_t>(dst) & 63u)) return false;
  const void* fields[SM_COUNT] = {f.forces};
  static_assert(STENCIL_TMAP_BYTES == SM_COUNT * sizeof(CUtensorMap) && STENCIL_TMAP_BYTES == STENCIL_TMAP_BYTES_HOST,
                "one descriptor per field");
  CUtensorMap maps[SM_COUNT];
  const cuuint64_t dims[2] = {(cuuint64_t)f.fw, (cuuint64_t)f.fh};
  const cuuint64_t pitch[1] = {(cuuint64_t)f.fw * 8u};
  const cuuint32_t box[2] = {(cuuint32_t)ST_BW, (cuuint32_t)ST_BH};
  const cuuint32_t unit[2] = {1u, 1u};
  for (int k = 0; k < SM_COUNT; k++) {
    if (reinterpret_cast<uintptr_t>(fields[k]) & 15u) return false;
    if (encode(&maps[k], CU_TENSOR_MAP_DATA_TYPE_INT64, 2, const_cast<void*>(fields[k]), dims, pitch, box, unit,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return false;
  }
  // pageable source: the call returns once the descriptors are staged
  if (cudaMemcpyAsync(dst, maps, sizeof maps, cudaMemcpyHostToDevice, s) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return true;
}

void launch_solid_mask(const Target& t, cudaStream_t s) {
  const dim3 blk(BX, BY);
  RB_PASS("build_solid_mask", 4.0 * t.cells + t.fcells, s, t, GEO_FLUID, blk, 0, k_solid_mask, nullptr);
  RB_PASS("wall_normals", 9.0 * t.fcells, s, t, GEO_FLUID, blk, 0, k_wall_normals, nullptr);
}
void launch_temperature(const Target& t, cudaStream_t s) {
  RB_PASS("update_temperature", 41.0 * t.fcells + 4.0 * t.cells, s, t, GEO_FLUID, dim3(BX, BY), 0, k_temperature, nullptr);
}
void launch_forces(const Target& t, cudaStream_t s) {
  RB_PASS("forces", 28.0 * t.fcells, s, t, GEO_FLUID_TALL, dim3(BX, BY), 0, k_forces, nullptr);
}
void launch_add_forces(const Target& t, int dir, cudaStream_t s) {
  RB_PASS("add_forces", 33.0 * t.fcells + 4.0 * t.cells, s, t, GEO_FLUID, dim3(BX, BY), 0, k_add_forces, nullptr, dir);
}
void launch_diffuse(const Target& t, int dir, cudaStream_t s) {
  RB_PASS("diffuse_velocity", 17.0 * t.fcells, s, t, GEO_FLUID, dim3(BX, BY), 0, k_diffuse, nullptr, dir);
}
void launch_advect(const Target& t, int dir, cudaStream_t s) {
  RB_PASS("advect_velocity", 17.0 * t.fcells, s, t, GEO_FLUID, dim3(BX, BY), 0, k_advect, nullptr, dir);
}
void launch_vorticity(const Target& t, int dir, cudaStream_t s) {
  RB_PASS("curl", 12.0 * t.fcells, s, t, GEO_FLUID, dim3(BX, BY), 0, k_curl, nullptr, dir);
  RB_PASS("vorticity", 21.0 * t.fcells, s, t, GEO_FLUID, dim3(BX, BY), 0, k_vorticity, nullptr, dir);
}
void launch_divergence(const Target& t, int dir, cudaStream_t s) {
  RB_PASS("divergence", 13.0 * t.fcells, s, t, GEO_FLUID, dim3(BX, BY), 0, k_divergence, nullptr, dir);
}
void launch_subtract_gradient(const Target& t, int dir, cudaStream_t s) {
  RB_PASS("subtract_gradient", 21.0 * t.fcells, s, t, GEO_FLUID, dim3(BX, BY), 0, k_subtract_gradient, nullptr, dir);
}
void launch_net_flux(const Target& t, int dir, cudaStream_t s) {
  static DeviceOnce attr;  // the double buffer is above the 48 KB default
  const int dev = DeviceOnce::device();
  if (attr.pending(dev)) {
    cudaFuncSetAttribute(k_net_flux<OneWorld>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)NF_SMEM);
    cudaFuncSetAttribute(k_net_flux<WorldSet>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)NF_SMEM);
    attr.done(dev);
  }
  RB_PASS("net_flux", 18.0 * t.fcells, s, t, GEO_NET_FLUX, dim3(NF_THREADS), NF_SMEM, k_net_flux, nullptr, dir);
}
void launch_boundaries(const Target& t, int dir, cudaStream_t s) {
  RB_PASS("enforce_boundaries", 17.0 * t.fcells, s, t, GEO_FLUID_TALL, dim3(BX, BY), 0, k_boundaries, nullptr, dir);
}
void launch_smooth(const Target& t, int dir, cudaStream_t s) {
  RB_PASS("smooth_velocity", 16.0 * t.fcells, s, t, GEO_FLUID_TALL, dim3(BX, BY), 0, k_smooth, nullptr, dir);
}

}  // namespace ribo
