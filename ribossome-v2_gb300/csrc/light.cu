// UV light block of the world step (shaders/world/light.wgsl:104-180,
// dispatch src/world/mod.rs:1505-1524): the transmission pre-pass and the
// full top-to-bottom sweep, and the parallel propagation of one row per
// launch with its commit.  Two bands (index + band * light cells).  Light
// cells are LIGHT_DIV x LIGHT_DIV environment cells; rows run along y, the
// sun at the top (y = lh - 1).
//
// The agent shade is this path's input (the SHADE field): the reference's
// clear_shade + agents_shade pair rebuilds it from the agents every step,
// which are not on this path.
#include "ribo_dev.cuh"
#include "ribo_launch.h"

namespace ribo {

namespace {

constexpr int BX = PASS_BX, BY = PASS_BY;
constexpr int SWEEP_THREADS = 1024;

// light.wgsl:43-45 (row_water_of): attenuation by the water of one light row
__device__ __forceinline__ float row_water(const Dev& d, const ribo_sim_params* P, uint32_t band) {
  return rb_exp(-rb_max(P->uv_depth, 0.0f) * (band == 1u ? (float)0.03 : 1.0f) * (float)LIGHT_DIV / (float)d.gh);
}

// light.wgsl:141-149 (light_transmit_pass): the transmission of every light
// cell into the light field, both bands.
template <class S>
__global__ void k_light_transmit(const __grid_constant__ S s) {
  RB_WORLD(s);
  const uint32_t x = cta.bx * BX + threadIdx.x, y = cta.by * BY + threadIdx.y;
  if (x >= (uint32_t)d.lw || y >= (uint32_t)d.lh) return;
  const size_t L = (size_t)d.lw * d.lh, i = (size_t)y * d.lw + x;
  float* light = const_cast<float*>(d.light);
  light[i] = light_transmit(d, P, x, y, 0u);
  light[L + i] = light_transmit(d, P, x, y, 1u);
}

// light.wgsl:151-176 (compute_uv_light): one CTA sweeps the rows from the
// top down, each row multiplied in place by the mean of the row above (the
// row's final values) and the water of a row; the top row takes the sun.
__global__ void __launch_bounds__(SWEEP_THREADS) k_light_sweep(const __grid_constant__ Dev d, const ribo_sim_params* P) {
  const size_t L = (size_t)d.lw * d.lh;
  float* light = const_cast<float*>(d.light);
  const float water0 = row_water(d, P, 0u), water1 = row_water(d, P, 1u);
  const uint32_t top = (uint32_t)d.lh - 1u;
  for (uint32_t x = threadIdx.x; x < (uint32_t)d.lw; x += SWEEP_THREADS) {
    light[(size_t)top * d.lw + x] *= water0 * P->sun_now;
    light[L + (size_t)top * d.lw + x] *= water1 * P->sun_now;
  }
  __syncthreads();
  for (uint32_t t = 1; t < (uint32_t)d.lh; t++) {
    const uint32_t y = (uint32_t)d.lh - 1u - t;
    for (uint32_t x = threadIdx.x; x < (uint32_t)d.lw; x += SWEEP_THREADS) {
      const float a0 = light_above(d, P, x, y + 1u, 0u), a1 = light_above(d, P, x, y + 1u, 1u);
      light[(size_t)y * d.lw + x] *= a0 * water0;
      light[L + (size_t)y * d.lw + x] *= a1 * water1;
    }
    __syncthreads();
  }
}

// light.wgsl:159-170 (light_propagate): each cell's new light from the row
// above of the previous step, the water and its own transmission.
template <class S>
__global__ void k_light_propagate(const __grid_constant__ S s) {
  RB_WORLD(s);
  const uint32_t x = cta.bx * BX + threadIdx.x, y = cta.by * BY + threadIdx.y;
  if (x >= (uint32_t)d.lw || y >= (uint32_t)d.lh) return;
  const size_t L = (size_t)d.lw * d.lh, i = (size_t)y * d.lw + x;
  for (uint32_t band = 0; band < 2u; band++) {
    float above = P->sun_now;
    if (y + 1u < (uint32_t)d.lh) above = light_above(d, P, x, y + 1u, band);
    d.light_next[band * L + i] = above * row_water(d, P, band) * light_transmit(d, P, x, y, band);
  }
}

// light.wgsl:172-177 (light_commit)
template <class S>
__global__ void k_light_commit(const __grid_constant__ S s) {
  RB_WORLD(s);
  const uint32_t x = cta.bx * BX + threadIdx.x, y = cta.by * BY + threadIdx.y;
  if (x >= (uint32_t)d.lw || y >= (uint32_t)d.lh) return;
  const size_t L = (size_t)d.lw * d.lh, i = (size_t)y * d.lw + x;
  float* light = const_cast<float*>(d.light);
  light[i] = d.light_next[i];
  light[L + i] = d.light_next[L + i];
}

}  // namespace

// Byte models per light cell (both bands): the transmission reads the
// LIGHT_DIV^2 chem words and gamma counts under the cell and its shade;
// the propagation also reads 7 taps of the row above; the commit copies.
void launch_light_transmit(const Target& t, cudaStream_t s) {
  const double lc = t.cells / (LIGHT_DIV * LIGHT_DIV);
  RB_PASS("light_transmit", lc * (LIGHT_DIV * LIGHT_DIV * 20.0 + 16.0), s, t, GEO_LIGHT, dim3(BX, BY), 0,
          k_light_transmit, nullptr);
}
void launch_light_sweep(const Dev& d, const ribo_sim_params* P, cudaStream_t s) {
  const double lc = (double)d.lw * d.lh;
  RB_LAUNCH("uv_light", lc * 24.0, s, k_light_sweep<<<1, SWEEP_THREADS, 0, s>>>(d, P));
}
void launch_light_propagate(const Target& t, cudaStream_t s) {
  const double lc = t.cells / (LIGHT_DIV * LIGHT_DIV);
  RB_PASS("light_propagate", lc * (LIGHT_DIV * LIGHT_DIV * 20.0 + 32.0), s, t, GEO_LIGHT, dim3(BX, BY), 0,
          k_light_propagate, nullptr);
}
void launch_light_commit(const Target& t, cudaStream_t s) {
  const double lc = t.cells / (LIGHT_DIV * LIGHT_DIV);
  RB_PASS("light_commit", lc * 16.0, s, t, GEO_LIGHT, dim3(BX, BY), 0, k_light_commit, nullptr);
}

}  // namespace ribo
