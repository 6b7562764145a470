// Pressure Poisson solve: cell-centred geometric multigrid with red-black
// Gauss-Seidel smoothing (shaders/world/multigrid.wgsl, schedule
// src/world/mod.rs:1545-1577) and the Jacobi alternative
// (shaders/world/fluid.wgsl:553-608, src/world/mod.rs:1578-1581).
//
// Red-black sweeps update one colour from the other colour only, so every
// fused or tiled variant below produces the same bits as one dispatch per
// half-sweep.
#include "ribo_dev.cuh"
#include "ribo_launch.h"

namespace ribo {

namespace {

constexpr int BX = 32, BY = 8;
inline dim3 grid2(int w, int h) { return dim3((w + BX - 1) / BX, (h + BY - 1) / BY); }

struct Lv {
  int nx, ny;
  float* p;
  float* rhs;
  uint8_t* fl;
  float eps;
};
inline Lv lv(const MgLevel& L, const MgBufs& b) { return Lv{L.nx, L.ny, b.p + L.off, b.rhs + L.off, b.fluid + L.off, L.eps}; }

// multigrid.wgsl:29-45: sum of the water neighbours and their count
__device__ __forceinline__ void neighbors(const Lv& L, int x, int y, float& s, float& k) {
  s = 0.0f;
  k = 0.0f;
  size_t i = (size_t)y * L.nx + x;
  if (x > 0 && L.fl[i - 1]) { s += L.p[i - 1]; k += 1.0f; }
  if (x + 1 < L.nx && L.fl[i + 1]) { s += L.p[i + 1]; k += 1.0f; }
  if (y > 0 && L.fl[i - L.nx]) { s += L.p[i - L.nx]; k += 1.0f; }
  if (y + 1 < L.ny && L.fl[i + L.nx]) { s += L.p[i + L.nx]; k += 1.0f; }
}

// multigrid.wgsl:49-58
__global__ void k_mg_init(const __grid_constant__ Dev d, Lv L) {
  int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
  if (x >= L.nx || y >= L.ny) return;
  size_t i = (size_t)y * L.nx + x, f = (size_t)y * d.fw + x;
  bool fluid = !is_solid(d, x, y);
  L.fl[i] = fluid ? 1 : 0;
  L.rhs[i] = fluid ? d.div[f] : 0.0f;
  L.p[i] = fluid ? d.pa[f] : 0.0f;
}

// multigrid.wgsl:60-77
__global__ void k_mg_smooth(Lv L, uint32_t color) {
  int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
  if (x >= L.nx || y >= L.ny) return;
  if ((((uint32_t)x + (uint32_t)y) & 1u) != color) return;
  size_t i = (size_t)y * L.nx + x;
  if (!L.fl[i]) return;
  float s, k;
  neighbors(L, x, y, s, k);
  L.p[i] = (s - L.rhs[i]) / (k + L.eps);
}

// multigrid.wgsl:82-105
__global__ void k_mg_restrict(Lv L, Lv C) {
  int cx = blockIdx.x * BX + threadIdx.x, cy = blockIdx.y * BY + threadIdx.y;
  if (cx >= C.nx || cy >= C.ny) return;
  float sum = 0.0f;
  uint32_t nf = 0;
#pragma unroll
  for (uint32_t c = 0; c < 4; c++) {
    int fx = cx * 2 + (int)(c & 1u), fy = cy * 2 + (int)(c >> 1);
    size_t i = (size_t)fy * L.nx + fx;
    if (!L.fl[i]) continue;
    float s, k;
    neighbors(L, fx, fy, s, k);
    sum += L.rhs[i] - (s - (k + L.eps) * L.p[i]);
    nf++;
  }
  size_t ci = (size_t)cy * C.nx + cx;
  C.fl[ci] = nf > 0u ? 1 : 0;
  C.rhs[ci] = nf > 0u ? 2.0f * sum / (float)(nf > 1u ? nf : 1u) : 0.0f;
  C.p[ci] = 0.0f;
}

// multigrid.wgsl:108-114
__global__ void k_mg_prolong(Lv L, Lv C) {
  int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
  if (x >= L.nx || y >= L.ny) return;
  size_t i = (size_t)y * L.nx + x;
  if (!L.fl[i]) return;
  L.p[i] += C.p[(size_t)(y / 2) * C.nx + x / 2];
}

// multigrid.wgsl:117-121
__global__ void k_mg_finish(const __grid_constant__ Dev d, Lv L) {
  int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
  if (x >= L.nx || y >= L.ny) return;
  d.pa[(size_t)y * d.fw + x] = L.p[(size_t)y * L.nx + x];
}

// fluid.wgsl:553-608: one Jacobi sweep pin -> pout; cells outside the grid
// count as walls (p = 0, solid), wall neighbours mirror p_c.
__global__ void k_jacobi(const __grid_constant__ Dev d, const float* __restrict__ pin, float* __restrict__ pout) {
  int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
  if (x >= d.fw || y >= d.fh) return;
  size_t idx = (size_t)y * d.fw + x;
  if (is_solid(d, x, y)) {
    pout[idx] = 0.0f;
    return;
  }
  float p_c = pin[idx];
  float p_l = (x > 0 && !is_solid(d, x - 1, y)) ? pin[idx - 1] : p_c;
  float p_r = (x + 1 < d.fw && !is_solid(d, x + 1, y)) ? pin[idx + 1] : p_c;
  float p_b = (y > 0 && !is_solid(d, x, y - 1)) ? pin[idx - d.fw] : p_c;
  float p_t = (y + 1 < d.fh && !is_solid(d, x, y + 1)) ? pin[idx + d.fw] : p_c;
  float dv = d.div[idx];
  if (is_bad(dv) || is_bad(p_c)) {
    pout[idx] = 0.0f;
    return;
  }
  float p_new = (p_l + p_r + p_b + p_t - dv) * 0.25f;
  pout[idx] = is_bad(p_new) ? 0.0f : p_new;
}

}  // namespace

inline double cells(const Lv& L) { return (double)L.nx * L.ny; }

void launch_multigrid(const Dev& d, const MgLevel* levels, int nl, const MgBufs& b, const MgConfig& c, cudaStream_t s) {
  const dim3 blk(BX, BY);
  Lv L0 = lv(levels[0], b);
  RB_LAUNCH("mg_init", 18.0 * cells(L0), s, k_mg_init<<<grid2(L0.nx, L0.ny), blk, 0, s>>>(d, L0));
  int cycles = c.cycles < 1 ? 1 : c.cycles;
  auto sweep = [&](const Lv& L) {
    RB_LAUNCH("mg_smooth", 9.0 * cells(L), s, k_mg_smooth<<<grid2(L.nx, L.ny), blk, 0, s>>>(L, 0u));
    RB_LAUNCH("mg_smooth", 9.0 * cells(L), s, k_mg_smooth<<<grid2(L.nx, L.ny), blk, 0, s>>>(L, 1u));
  };
  for (int cy = 0; cy < cycles; cy++) {
    for (int l = 0; l < nl - 1; l++) {
      Lv L = lv(levels[l], b);
      for (int k = 0; k < c.pre; k++) sweep(L);
      Lv C = lv(levels[l + 1], b);
      RB_LAUNCH("mg_restrict", 9.0 * cells(L) + 9.0 * cells(C), s, k_mg_restrict<<<grid2(C.nx, C.ny), blk, 0, s>>>(L, C));
    }
    Lv Lc = lv(levels[nl - 1], b);
    for (int k = 0; k < c.coarse; k++) sweep(Lc);
    for (int l = nl - 2; l >= 0; l--) {
      Lv L = lv(levels[l], b), C = lv(levels[l + 1], b);
      RB_LAUNCH("mg_prolong", 9.0 * cells(L) + 4.0 * cells(C), s, k_mg_prolong<<<grid2(L.nx, L.ny), blk, 0, s>>>(L, C));
      for (int k = 0; k < c.post; k++) sweep(L);
    }
  }
  RB_LAUNCH("mg_finish", 8.0 * cells(L0), s, k_mg_finish<<<grid2(L0.nx, L0.ny), blk, 0, s>>>(d, L0));
}

void launch_jacobi(const Dev& d, int iters, cudaStream_t s) {
  const dim3 blk(BX, BY);
  double b = 13.0 * (double)d.fw * d.fh;
  for (int k = 0; k < iters; k++) {
    if (k % 2 == 0) RB_LAUNCH("jacobi_pressure", b, s, k_jacobi<<<grid2(d.fw, d.fh), blk, 0, s>>>(d, d.pa, d.pb));
    else RB_LAUNCH("jacobi_pressure", b, s, k_jacobi<<<grid2(d.fw, d.fh), blk, 0, s>>>(d, d.pb, d.pa));
  }
}

}  // namespace ribo
