// Mixed-precision pressure solve (ribo_world_cfg.precision_mode =
// RIBO_PRECISION_MIXED): the world step's pressure Poisson problem solved to
// a relative residual tolerance instead of a fixed number of V-cycles.
//
// The problem is the reference's level-0 operator (shaders/world/
// multigrid.wgsl:29-77) written exactly: for every water cell,
//     (L p)_i = sum over water neighbours j of (p_j - p_i) - eps0 * p_i,
// eps0 = 1e-4 (the f32 value), and L p = rhs with rhs = the divergence.
//
// * Outer loop (defect correction): the solution is kept as an unevaluated
//   pair of FP32 numbers (pressure_a = hi, a second buffer = lo); the
//   residual rhs - L(hi + lo) is evaluated with error-free FP32
//   transformations (Knuth's TwoSum, Dekker's FastTwoSum, the FMA two-product),
//   which resolves it to ~2^-44 where a single FP32 vector stalls at ~1e-5
//   relative residual on 256^2 and above.
// * Inner loop: flexible conjugate gradients in FP32 on L e = r
//   (Polak-Ribiere beta, which tolerates the preconditioner's FP16 rounding),
//   preconditioned by a symmetric V-cycle: FP16 storage of the smoothing
//   arrays on levels 0-3, FP32 below, an exact FP64 solve on the coarsest
//   level (dense inverse), and FP64 mean removal: every connected water
//   region is a pure-Neumann-like problem whose constant vector is an exact
//   eigenvector of L (eigenvalue -eps0), so the preconditioner removes the
//   residual's mean per region before the V-cycle and adds the exact
//   constant correction -mean/eps0 after it.
// * Both loops run on the device as CUDA graph WHILE nodes; their bodies'
//   last kernels decide whether to iterate again, with hard caps on the
//   iteration counts.  No host synchronisation happens inside a solve.
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stddef.h>
#include <string.h>

#include <vector>

#include "ribo_dev.cuh"
#include "ribo_launch.h"
#include "ribo_world_impl.h"

namespace ribo {

namespace {

constexpr int BX = PASS_BX, BY = PASS_BY, NT = BX * BY;
constexpr int COMP_CAP = 65536;        // water components tracked (later ones share the last slot)
constexpr int COARSEST_CAP = 1024;     // cells of the coarsest level (dense FP64 inverse)
constexpr int HALF_LEVELS = 4;         // fine levels 0..3 store FP16

// ---- FP32 pair ("double-float") arithmetic -------------------------------
struct df32 {
  float hi, lo;
};
// Knuth's TwoSum: s + e == a + b exactly.
__device__ __forceinline__ df32 two_sum(float a, float b) {
  const float s = a + b;
  const float bp = s - a;
  const float e = (a - (s - bp)) + (b - bp);
  return df32{s, e};
}
// Dekker's FastTwoSum (|a| >= |b|).
__device__ __forceinline__ df32 fast_two_sum(float a, float b) {
  const float s = a + b;
  return df32{s, b - (s - a)};
}
__device__ __forceinline__ df32 df_add(df32 a, df32 b) {
  df32 s = two_sum(a.hi, b.hi);
  const df32 t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = fast_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df32 df_neg(df32 a) { return df32{-a.hi, -a.lo}; }
// (hi + lo) * b with the FMA two-product of hi * b.
__device__ __forceinline__ df32 df_mul_f(df32 a, float b) {
  const float p = a.hi * b;
  float e = __fmaf_rn(a.hi, b, -p);
  e += a.lo * b;
  return fast_two_sum(p, e);
}

// ---- solver state --------------------------------------------------------
struct MpCtl {
  unsigned int done;  // blocks finished in the current reduction kernel
  int outer, inner, total_inner;
  int converged, inner_done;
  int max_outer, max_inner;
  int ncomp;
  int big;            // the largest water component
  float tol2, itol2;  // squared relative tolerances
  float rz, alpha, beta;
  float scale[2];     // V-cycle input scale and its inverse
  float r0n2;         // ||r||^2 at the start of the outer iteration
  float itarget2;     // squared residual reduction the inner solve stops at
  float nwater;
  double bn2;         // ||rhs||^2
  double rho;         // relative residual of the last outer evaluation
};

struct MpArgs {
  int fw, fh;
  float eps0;
  float* hi;  // pressure_a
  float* lo;
  const float* rhs;     // divergence
  const uint8_t* fl;    // level-0 water flags
  const int* label;     // component per cell (-1: wall)
  float *r, *e, *d, *q, *z;
  float* part;          // per-block partial sums [blocks][2]
  double* part_c;       // per-block sum over the block's dominant component
  int* part_dom;        // per-block dominant component (-1: none)
  MpCtl* ctl;
  double* comp_sum_r;
  double* comp_sum_z;
  double* comp_mean;
  float* comp_mean_f;   // FP32 copies for the per-cell passes
  float* comp_shift;    // per component: mean of z + mean of r / eps0
  const double* comp_size;
};

// The per-cell kernels of the CG run one thread per RR cells of a column:
// a block covers BX x (BY * RR) cells, which keeps the number of blocks (and
// of partial sums the last block gathers) small.
constexpr int RR = 8;

struct Cell {
  int x, y;
  size_t i;
  bool in, water;
};
__device__ __forceinline__ Cell cell_at(const MpArgs& a, int k) {
  Cell c;
  c.x = blockIdx.x * BX + threadIdx.x;
  c.y = (blockIdx.y * RR + k) * BY + threadIdx.y;
  c.in = c.x < a.fw && c.y < a.fh;
  c.i = c.in ? (size_t)c.y * a.fw + c.x : 0;
  c.water = c.in && a.fl[c.i] != 0;
  return c;
}
// position of cell k of this thread inside the block's region (row-major)
__device__ __forceinline__ int cell_pos(int k) { return ((k * BY + (int)threadIdx.y) * BX) + (int)threadIdx.x; }
// Cell k's index without its flag (0 outside the grid, a valid address):
// the vector kernels below load a group of RG cells' inputs before they
// compute or store any, since their stores would otherwise order every
// later load behind them (the buffers do not alias, but are not declared so).
constexpr int RG = 4;
static_assert(RR % RG == 0, "cells split into whole groups");
__device__ __forceinline__ size_t cell_idx(const MpArgs& a, int k, bool& in) {
  const int x = blockIdx.x * BX + threadIdx.x, y = (blockIdx.y * RR + k) * BY + threadIdx.y;
  in = x < a.fw && y < a.fh;
  return in ? (size_t)y * a.fw + x : 0;
}

// Block sums of two values written to the per-block partials; returns true in
// every thread of the block that finished last (its partials are visible).
__device__ __forceinline__ bool block_partials(const MpArgs& a, float v0, float v1) {
  __shared__ float s0[NT / 32], s1[NT / 32];
  __shared__ bool last;
  const int tid = threadIdx.y * BX + threadIdx.x;
  for (int o = 16; o > 0; o >>= 1) {
    v0 += __shfl_down_sync(0xffffffffu, v0, o);
    v1 += __shfl_down_sync(0xffffffffu, v1, o);
  }
  if ((tid & 31) == 0) {
    s0[tid >> 5] = v0;
    s1[tid >> 5] = v1;
  }
  __syncthreads();
  if (tid == 0) {
    float t0 = 0.0f, t1 = 0.0f;
    for (int w = 0; w < NT / 32; w++) {
      t0 += s0[w];
      t1 += s1[w];
    }
    const unsigned b = blockIdx.y * gridDim.x + blockIdx.x;
    a.part[2 * b] = t0;
    a.part[2 * b + 1] = t1;
    __threadfence();
    const unsigned n = gridDim.x * gridDim.y;
    last = atomicAdd(&a.ctl->done, 1u) == n - 1;
  }
  __syncthreads();
  return last;
}

// In the last block: the totals of the partials, summed in a fixed order
// (deterministic), returned in every thread.
__device__ __forceinline__ void total_partials(const MpArgs& a, float& t0, float& t1) {
  __shared__ float s0[NT], s1[NT];
  __threadfence();
  const int tid = threadIdx.y * BX + threadIdx.x;
  const unsigned n = gridDim.x * gridDim.y;
  float v0 = 0.0f, v1 = 0.0f;
  const float2* part = reinterpret_cast<const float2*>(a.part);
#pragma unroll 8
  for (unsigned b = tid; b < n; b += NT) {
    const float2 pv = __ldcg(part + b);  // L2: the other blocks' partials
    v0 += pv.x;
    v1 += pv.y;
  }
  s0[tid] = v0;
  s1[tid] = v1;
  __syncthreads();
  for (int o = NT / 2; o > 0; o >>= 1) {
    if (tid < o) {
      s0[tid] += s0[tid + o];
      s1[tid] += s1[tid + o];
    }
    __syncthreads();
  }
  t0 = s0[0];
  t1 = s1[0];
  __syncthreads();
}

// Per-component FP64 sums of a per-cell value.  The block's dominant
// component is that of its first water cell (smallest position; key =
// position << 16 | component, components below 2^16); the block sums its
// cells of that component and records the partial with the component, and
// cells of other components (rare: the block straddles a rock wall) add
// directly.  The last block gathers the partials (comp_gather), so no address
// receives an atomic from every block.
__device__ __forceinline__ int block_dom(int key) {
  __shared__ int best;
  if (threadIdx.x == 0 && threadIdx.y == 0) best = 0x7fffffff;
  __syncthreads();
  if (key != 0x7fffffff) atomicMin(&best, key);
  __syncthreads();
  const int b = best;
  return b == 0x7fffffff ? -1 : (b & 0xffff);
}
__device__ __forceinline__ void comp_record(const MpArgs& a, double* sums, int dom, const float* v, const int* lab) {
  __shared__ double sh[NT / 32];
  const int tid = threadIdx.y * BX + threadIdx.x;
  float own = 0.0f;
#pragma unroll
  for (int k = 0; k < RR; k++) {
    if (lab[k] < 0) continue;
    if (lab[k] == dom) own += v[k];
    else atomicAdd(sums + lab[k], (double)v[k]);
  }
  double dv = (double)own;
  for (int o = 16; o > 0; o >>= 1) dv += __shfl_down_sync(0xffffffffu, dv, o);
  if ((tid & 31) == 0) sh[tid >> 5] = dv;
  __syncthreads();
  if (tid == 0) {
    double t = 0.0;
    for (int w = 0; w < NT / 32; w++) t += sh[w];
    const unsigned b = blockIdx.y * gridDim.x + blockIdx.x;
    a.part_c[b] = t;
    a.part_dom[b] = dom;
  }
  __threadfence();  // partials and direct adds land before this block counts itself done
}

// In the last block: every block's partial added to its component's sum --
// the largest component's in a fixed order (deterministic), the others
// (few) with atomics -- complete and visible when this returns.
__device__ __forceinline__ void comp_gather(const MpArgs& a, double* sums, unsigned nblocks) {
  __shared__ double sh[NT];
  const int tid = threadIdx.y * BX + threadIdx.x;
  const int big = a.ctl->big;
  double acc = 0.0;
#pragma unroll 8
  for (unsigned b = tid; b < nblocks; b += NT) {
    const int d = __ldcg(a.part_dom + b);
    const double v = __ldcg(a.part_c + b);
    if (d == big) acc += v;
    else if (d >= 0) atomicAdd(sums + d, v);
  }
  sh[tid] = acc;
  __syncthreads();
  for (int o = NT / 2; o > 0; o >>= 1) {
    if (tid < o) sh[tid] += sh[tid + o];
    __syncthreads();
  }
  if (tid == 0 && big >= 0) sums[big] += sh[0];
  __threadfence();
  __syncthreads();
}

// In the last block: component means of the residual (FP64) and the power-of-
// two scale that brings its RMS to ~1 for the FP16 levels.
__device__ __forceinline__ void finish_residual_stats(const MpArgs& a, float rn2) {
  const int tid = threadIdx.y * BX + threadIdx.x;
  MpCtl* ctl = a.ctl;
  const int nc = ctl->ncomp;
  comp_gather(a, a.comp_sum_r, gridDim.x * gridDim.y);
  for (int c = tid; c < nc; c += NT) {
    const double m = a.comp_size[c] > 0.0 ? __ldcg(a.comp_sum_r + c) / a.comp_size[c] : 0.0;
    a.comp_mean[c] = m;
    a.comp_mean_f[c] = (float)m;
    a.comp_sum_r[c] = 0.0;
  }
  if (tid == 0) {
    const float rms = ctl->nwater > 0.0f ? sqrtf(rn2 / ctl->nwater) : 0.0f;
    float sc = 1.0f;
    if (rms > 0.0f && rms == rms) {
      int ex = 0;
      frexpf(rms, &ex);
      sc = ldexpf(1.0f, -ex);
    }
    ctl->scale[0] = sc;
    ctl->scale[1] = 1.0f / sc;
  }
}

// `graph` = 1 when the kernel runs inside the solve's graph (it then sets the
// loop conditions); 0 when the host drives the loops.
__global__ void k_mp_begin(MpArgs a, int max_outer, int max_inner, float tol, float itol,
                           cudaGraphConditionalHandle h_outer, int graph) {
  MpCtl* ctl = a.ctl;
  for (int c = threadIdx.x; c < ctl->ncomp; c += blockDim.x) {
    a.comp_sum_r[c] = 0.0;
    a.comp_sum_z[c] = 0.0;
  }
  if (threadIdx.x == 0) {
    ctl->done = 0;
    ctl->outer = ctl->inner = ctl->total_inner = 0;
    ctl->converged = ctl->inner_done = 0;
    ctl->max_outer = max_outer;
    ctl->max_inner = max_inner;
    ctl->tol2 = tol * tol;
    ctl->itol2 = itol * itol;
    ctl->bn2 = 0.0;
    ctl->rho = 0.0;
    if (graph) cudaGraphSetConditional(h_outer, 1u);
  }
}

// Outer residual r = rhs - L(hi + lo) in FP32-pair arithmetic; the CG
// starts from e = 0 on it.  The last block decides both loops.
__global__ void __launch_bounds__(NT) k_mp_residual(MpArgs a, cudaGraphConditionalHandle h_outer,
                                                    cudaGraphConditionalHandle h_inner, int final_pass, int graph) {
  float rf[RR];
  int lab[RR];
  float rn2 = 0.0f, bn2 = 0.0f;
  int key = 0x7fffffff;
  const int x = blockIdx.x * BX + threadIdx.x;
#pragma unroll
  for (int g = 0; g < RR; g += RG) {
    bool in[RG], inn[RG][4];
    uint8_t wf[RG], fn[RG][4];
    float phi[RG], plo[RG], nhi[RG][4], nlo[RG][4], bv[RG];
    int lb[RG];
#pragma unroll
    for (int k = 0; k < RG; k++) {
      const size_t i = cell_idx(a, g + k, in[k]);
      const int y = (blockIdx.y * RR + g + k) * BY + threadIdx.y;
      // left, right, below, above (multigrid.wgsl:34-45 order), clamped to the cell off the grid
      inn[k][0] = x > 0;
      inn[k][1] = x + 1 < a.fw;
      inn[k][2] = y > 0;
      inn[k][3] = y + 1 < a.fh;
      const size_t nb[4] = {inn[k][0] ? i - 1 : i, inn[k][1] ? i + 1 : i, inn[k][2] ? i - a.fw : i, inn[k][3] ? i + a.fw : i};
      wf[k] = in[k] ? a.fl[i] : 0;
      phi[k] = a.hi[i];
      plo[k] = a.lo[i];
      bv[k] = a.rhs[i];
      lb[k] = a.label[i];
#pragma unroll
      for (int n = 0; n < 4; n++) {
        fn[k][n] = a.fl[nb[n]];
        nhi[k][n] = a.hi[nb[n]];
        nlo[k][n] = a.lo[nb[n]];
      }
    }
#pragma unroll
    for (int k = 0; k < RG; k++) {
      bool inb;
      const size_t i = cell_idx(a, g + k, inb);
      rf[g + k] = 0.0f;
      lab[g + k] = -1;
      if (wf[k]) {
        const df32 pi = df32{phi[k], plo[k]};
        df32 sum = df32{0.0f, 0.0f};
#pragma unroll
        for (int n = 0; n < 4; n++) {
          if (!inn[k][n] || !fn[k][n]) continue;
          sum = df_add(sum, df_add(df32{nhi[k][n], nlo[k][n]}, df_neg(pi)));
        }
        const df32 lp = df_add(sum, df_neg(df_mul_f(pi, a.eps0)));
        const float b = bv[k];
        const df32 res = df_add(df32{b, 0.0f}, df_neg(lp));
        rf[g + k] = res.hi + res.lo;
        rn2 += rf[g + k] * rf[g + k];
        bn2 += b * b;
        lab[g + k] = lb[k];
        if (key == 0x7fffffff) key = (cell_pos(g + k) << 16) | lab[g + k];
      }
      if (in[k]) {
        a.r[i] = rf[g + k];
        a.e[i] = 0.0f;
      }
    }
  }
  if (!final_pass) comp_record(a, a.comp_sum_r, block_dom(key), rf, lab);
  if (!block_partials(a, rn2, bn2)) return;
  float trn2, tbn2;
  total_partials(a, trn2, tbn2);
  MpCtl* ctl = a.ctl;
  const int tid = threadIdx.y * BX + threadIdx.x;
  if (final_pass) {
    if (tid == 0) {
      ctl->rho = ctl->bn2 > 0.0 ? sqrt((double)trn2 / ctl->bn2) : 0.0;
      ctl->done = 0;
    }
    return;
  }
  finish_residual_stats(a, trn2);
  if (tid == 0) {
    if (ctl->outer == 0) ctl->bn2 = (double)tbn2;
    const double rho2 = ctl->bn2 > 0.0 ? (double)trn2 / ctl->bn2 : 0.0;
    ctl->rho = sqrt(rho2);
    const bool conv = rho2 <= (double)ctl->tol2 || !(rho2 == rho2);
    ctl->converged = conv ? 1 : 0;
    ctl->inner = 0;
    ctl->inner_done = conv ? 1 : 0;
    ctl->r0n2 = trn2;
    // the inner solve stops at mixed_inner_tol, or as soon as the outer
    // residual would be half the tolerance if it is closer than that
    const double need = rho2 > 0.0 ? 0.25 * (double)ctl->tol2 / rho2 : 1.0;
    ctl->itarget2 = (float)(need > (double)ctl->itol2 ? (need < 1.0 ? need : 1.0) : (double)ctl->itol2);
    ctl->outer += 1;
    ctl->done = 0;
    if (graph) {
      cudaGraphSetConditional(h_inner, conv ? 0u : 1u);
      cudaGraphSetConditional(h_outer, (!conv && ctl->outer < ctl->max_outer) ? 1u : 0u);
    }
  }
}

// z <- z - (mean of z over its component) - comp_mean / eps0 (the shift
// k_mp_zshift formed), then the dot products z.r and z.q of the flexible CG.
__global__ void __launch_bounds__(NT) k_mp_dots(MpArgs a) {
  float zr = 0.0f, zq = 0.0f;
#pragma unroll
  for (int g = 0; g < RR; g += RG) {
    bool in[RG];
    uint8_t wf[RG];
    float zv[RG], rv[RG], qv[RG], sh[RG];
    int lb[RG];
#pragma unroll
    for (int k = 0; k < RG; k++) {
      const size_t i = cell_idx(a, g + k, in[k]);
      wf[k] = in[k] ? a.fl[i] : 0;
      zv[k] = a.z[i];
      rv[k] = a.r[i];
      qv[k] = a.q[i];
      lb[k] = a.label[i];
    }
#pragma unroll
    for (int k = 0; k < RG; k++) sh[k] = wf[k] ? a.comp_shift[lb[k]] : 0.0f;
#pragma unroll
    for (int k = 0; k < RG; k++) {
      bool inb;
      const size_t i = cell_idx(a, g + k, inb);
      if (wf[k]) {
        const float zc = zv[k] - sh[k];
        a.z[i] = zc;
        zr += zc * rv[k];
        zq += zc * qv[k];
      } else if (in[k]) {
        a.z[i] = 0.0f;
      }
    }
  }
  if (!block_partials(a, zr, zq)) return;
  float tzr, tzq;
  total_partials(a, tzr, tzq);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    MpCtl* ctl = a.ctl;
    ctl->beta = (ctl->inner == 0 || ctl->rz == 0.0f) ? 0.0f : -ctl->alpha * tzq / ctl->rz;
    ctl->rz = tzr;
    ctl->done = 0;
  }
}

// After the V-cycle (one block): gathers the per-tile sums of z the level-0
// post kernel recorded, and forms each component's shift = mean of z + mean
// of the residual / eps0 in FP64 (the mean removal), which the next kernel
// subtracts in FP32.
__global__ void __launch_bounds__(NT) k_mp_zshift(MpArgs a, unsigned ntiles) {
  comp_gather(a, a.comp_sum_z, ntiles);
  const int tid = threadIdx.y * BX + threadIdx.x;
  const int nc = a.ctl->ncomp;
  for (int c = tid; c < nc; c += NT) {
    const double zm = a.comp_size[c] > 0.0 ? __ldcg(a.comp_sum_z + c) / a.comp_size[c] : 0.0;
    a.comp_shift[c] = (float)(zm + a.comp_mean[c] / (double)a.eps0);
    a.comp_sum_z[c] = 0.0;
  }
}

__global__ void __launch_bounds__(NT) k_mp_direction(MpArgs a) {
  const float beta = a.ctl->beta;
  const bool first = a.ctl->inner == 0;  // d starts as z (whatever d held before)
#pragma unroll
  for (int g = 0; g < RR; g += RG) {
    bool in[RG];
    uint8_t wf[RG];
    float zv[RG], dv[RG];
#pragma unroll
    for (int k = 0; k < RG; k++) {
      const size_t i = cell_idx(a, g + k, in[k]);
      wf[k] = in[k] ? a.fl[i] : 0;
      zv[k] = a.z[i];
      dv[k] = a.d[i];
    }
#pragma unroll
    for (int k = 0; k < RG; k++) {
      bool inb;
      const size_t i = cell_idx(a, g + k, inb);
      if (in[k]) a.d[i] = wf[k] ? (first ? zv[k] : zv[k] + beta * dv[k]) : 0.0f;
    }
  }
}

// q = L d in FP32 (differences first, so a constant d gives -eps0 * d
// exactly), and d.q; alpha = z.r / d.q.
__global__ void __launch_bounds__(NT) k_mp_matvec(MpArgs a) {
  float dq = 0.0f;
  const int x = blockIdx.x * BX + threadIdx.x;
#pragma unroll
  for (int g = 0; g < RR; g += RG) {
    bool in[RG];
    uint8_t wf[RG], fn[RG][4];
    float dc[RG], dn[RG][4];
#pragma unroll
    for (int k = 0; k < RG; k++) {
      const size_t i = cell_idx(a, g + k, in[k]);
      const int y = (blockIdx.y * RR + g + k) * BY + threadIdx.y;
      // left, right, below, above (clamped to the cell itself off the grid)
      const size_t nb[4] = {x > 0 ? i - 1 : i, x + 1 < a.fw ? i + 1 : i, y > 0 ? i - a.fw : i, y + 1 < a.fh ? i + a.fw : i};
      wf[k] = in[k] ? a.fl[i] : 0;
      dc[k] = a.d[i];
#pragma unroll
      for (int n = 0; n < 4; n++) {
        fn[k][n] = a.fl[nb[n]];
        dn[k][n] = a.d[nb[n]];
      }
    }
#pragma unroll
    for (int k = 0; k < RG; k++) {
      bool inb;
      const size_t i = cell_idx(a, g + k, inb);
      const int y = (blockIdx.y * RR + g + k) * BY + threadIdx.y;
      if (wf[k]) {
        const float di = dc[k];
        float sum = 0.0f;
        if (x > 0 && fn[k][0]) sum += dn[k][0] - di;
        if (x + 1 < a.fw && fn[k][1]) sum += dn[k][1] - di;
        if (y > 0 && fn[k][2]) sum += dn[k][2] - di;
        if (y + 1 < a.fh && fn[k][3]) sum += dn[k][3] - di;
        const float q = sum - a.eps0 * di;
        a.q[i] = q;
        dq += di * q;
      } else if (in[k]) {
        a.q[i] = 0.0f;
      }
    }
  }
  if (!block_partials(a, dq, 0.0f)) return;
  float tdq, unused;
  total_partials(a, tdq, unused);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    MpCtl* ctl = a.ctl;
    ctl->alpha = tdq != 0.0f ? ctl->rz / tdq : 0.0f;
    ctl->done = 0;
  }
}

// e += alpha d, r -= alpha q; the last block tests the inner tolerance,
// prepares the next preconditioner input and sets the inner loop condition.
__global__ void __launch_bounds__(NT) k_mp_axpy(MpArgs a, cudaGraphConditionalHandle h_inner, int graph) {
  const float alpha = a.ctl->alpha;
  float rn[RR];
  int lab[RR];
  float rn2 = 0.0f;
  int key = 0x7fffffff;
#pragma unroll
  for (int g = 0; g < RR; g += RG) {
    uint8_t wf[RG];
    float ev[RG], dv[RG], rv[RG], qv[RG];
    int lb[RG];
#pragma unroll
    for (int k = 0; k < RG; k++) {
      bool in;
      const size_t i = cell_idx(a, g + k, in);
      wf[k] = in ? a.fl[i] : 0;
      ev[k] = a.e[i];
      dv[k] = a.d[i];
      rv[k] = a.r[i];
      qv[k] = a.q[i];
      lb[k] = a.label[i];
    }
#pragma unroll
    for (int k = 0; k < RG; k++) {
      bool in;
      const size_t i = cell_idx(a, g + k, in);
      rn[g + k] = 0.0f;
      lab[g + k] = -1;
      if (wf[k]) {
        a.e[i] = ev[k] + alpha * dv[k];
        rn[g + k] = rv[k] - alpha * qv[k];
        a.r[i] = rn[g + k];
        rn2 += rn[g + k] * rn[g + k];
        lab[g + k] = lb[k];
        if (key == 0x7fffffff) key = (cell_pos(g + k) << 16) | lb[k];
      }
    }
  }
  comp_record(a, a.comp_sum_r, block_dom(key), rn, lab);
  if (!block_partials(a, rn2, 0.0f)) return;
  float trn2, unused;
  total_partials(a, trn2, unused);
  finish_residual_stats(a, trn2);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    MpCtl* ctl = a.ctl;
    ctl->inner += 1;
    ctl->total_inner += 1;
    const bool done = trn2 <= ctl->itarget2 * ctl->r0n2 || !(trn2 == trn2);
    ctl->inner_done = done ? 1 : 0;
    ctl->done = 0;
    if (graph) cudaGraphSetConditional(h_inner, (!done && ctl->inner < ctl->max_inner) ? 1u : 0u);
  }
}

// (hi, lo) += e; walls hold 0 (as the f32 multigrid leaves them).
__global__ void __launch_bounds__(NT) k_mp_update(MpArgs a) {
#pragma unroll
  for (int k = 0; k < RR; k++) {
    const Cell c = cell_at(a, k);
    if (!c.in) continue;
    if (!c.water) {
      a.hi[c.i] = 0.0f;
      a.lo[c.i] = 0.0f;
      continue;
    }
    const df32 p = df_add(df32{a.hi[c.i], a.lo[c.i]}, df32{a.e[c.i], 0.0f});
    a.hi[c.i] = p.hi;
    a.lo[c.i] = p.lo;
  }
}

}  // namespace

// Buffers and graphs of one world's mixed-precision solver.
struct MixedSolver {
  float* lo = nullptr;
  float *r = nullptr, *e = nullptr, *d = nullptr, *q = nullptr, *z = nullptr;
  float* part = nullptr;
  int* label = nullptr;
  MpCtl* ctl = nullptr;
  double *comp_sum_r = nullptr, *comp_sum_z = nullptr, *comp_mean = nullptr, *comp_size = nullptr;
  float *comp_mean_f = nullptr, *comp_shift = nullptr;
  double* part_c = nullptr;
  int* part_dom = nullptr;
  double* inv = nullptr;
  int coarsest_cells = 0;
  MpHierarchy h{};
  cudaStream_t cap[3] = {nullptr, nullptr, nullptr};
  cudaGraphExec_t standalone = nullptr;
  ribo_world_settings built_for{};
  int ncomp = 0;
};

namespace {

int half_levels(const World& w) {
  const int k = multigrid_first_coarse_level(w.levels.data(), (int)w.levels.size());
  return k < HALF_LEVELS ? k : HALF_LEVELS;
}

// Entries of part_c / part_dom: written per residual block by the CG
// kernels and per level-0 tile by the V-cycle.
size_t part_entries(const ribo_world_cfg& c, const std::vector<MgLevel>& levels) {
  const size_t blocks = ((size_t)(c.fluid_w + BX - 1) / BX) * ((c.fluid_h + BY - 1) / BY);
  const MgConfig mc{(int)c.mg_pre, (int)c.mg_post, (int)c.mg_coarse, 1};
  const size_t tiles = mixed_vcycle_tiles(levels.data(), (int)levels.size(), mc);
  return blocks > tiles ? blocks : tiles;
}

MpArgs mp_args(const World& w, const MixedSolver& m) {
  MpArgs a{};
  a.fw = w.fw;
  a.fh = w.fh;
  a.eps0 = (float)1e-4;
  a.hi = w.pa;
  a.lo = m.lo;
  a.rhs = w.div;
  a.fl = w.mg.fluid + w.levels[0].off;
  a.label = m.label;
  a.r = m.r;
  a.e = m.e;
  a.d = m.d;
  a.q = m.q;
  a.z = m.z;
  a.part = m.part;
  a.ctl = m.ctl;
  a.comp_sum_r = m.comp_sum_r;
  a.comp_sum_z = m.comp_sum_z;
  a.comp_mean = m.comp_mean;
  a.comp_size = m.comp_size;
  a.comp_mean_f = m.comp_mean_f;
  a.comp_shift = m.comp_shift;
  a.part_c = m.part_c;
  a.part_dom = m.part_dom;
  return a;
}

float setting_or(float v, float dflt) { return v > 0.0f ? v : dflt; }
int setting_or(uint32_t v, int dflt) { return v > 0 ? (int)v : dflt; }

#define RB_CK(expr)                       \
  do {                                    \
    cudaError_t _e = (expr);              \
    if (_e != cudaSuccess) return _e;     \
  } while (0)

// Adds the solve to the graph that stream `s` is capturing: a WHILE node for
// the outer loop whose body holds the residual, a WHILE node for the inner
// loop and the update.
cudaError_t capture_solve(World& w, MixedSolver& m, cudaStream_t s) {
  const MpArgs a = mp_args(w, m);
  const dim3 grid((w.fw + BX - 1) / BX, (w.fh + BY * RR - 1) / (BY * RR)), blk(BX, BY);
  const ribo_world_settings& st = w.st;
  cudaStreamCaptureStatus cs;
  unsigned long long id = 0;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  const cudaGraphEdgeData* ed = nullptr;
  size_t nd = 0;
  RB_CK(cudaStreamGetCaptureInfo(s, &cs, &id, &g, &deps, &ed, &nd));
  if (cs != cudaStreamCaptureStatusActive) return cudaErrorIllegalState;
  // Each handle belongs to the graph that contains its WHILE node; neither has
  // a default value: a kernel sets it before its node runs (k_mp_begin for the
  // outer loop, k_mp_residual for the inner one), and the bodies' last kernels
  // stop the loops once converged or at the iteration caps.
  cudaGraphConditionalHandle ho, hi;
  RB_CK(cudaGraphConditionalHandleCreate(&ho, g, 0, 0));
  k_mp_begin<<<1, 256, 0, s>>>(a, setting_or(st.mixed_max_outer, 4), setting_or(st.mixed_max_inner, 64),
                               setting_or(st.mixed_tol, 1e-5f), setting_or(st.mixed_inner_tol, 1e-3f), ho, 1);
  RB_CK(cudaGetLastError());
  RB_CK(cudaStreamGetCaptureInfo(s, &cs, &id, &g, &deps, &ed, &nd));
  cudaGraphNodeParams po = {};
  po.type = cudaGraphNodeTypeConditional;
  po.conditional.handle = ho;
  po.conditional.type = cudaGraphCondTypeWhile;
  po.conditional.size = 1;
  cudaGraphNode_t no;
  RB_CK(cudaGraphAddNode(&no, g, deps, ed, nd, &po));
  cudaGraph_t body_o = po.conditional.phGraph_out[0];
  RB_CK(cudaStreamUpdateCaptureDependencies(s, &no, nullptr, 1, cudaStreamSetCaptureDependencies));

  RB_CK(cudaGraphConditionalHandleCreate(&hi, body_o, 0, 0));

  // outer body: residual, inner loop, update
  cudaStream_t so = m.cap[1];
  RB_CK(cudaStreamBeginCaptureToGraph(so, body_o, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  k_mp_residual<<<grid, blk, 0, so>>>(a, ho, hi, 0, 1);
  cudaGraph_t gb = nullptr;
  RB_CK(cudaStreamGetCaptureInfo(so, &cs, &id, &gb, &deps, &ed, &nd));
  cudaGraphNodeParams pi = {};
  pi.type = cudaGraphNodeTypeConditional;
  pi.conditional.handle = hi;
  pi.conditional.type = cudaGraphCondTypeWhile;
  pi.conditional.size = 1;
  cudaGraphNode_t ni;
  RB_CK(cudaGraphAddNode(&ni, gb, deps, ed, nd, &pi));
  cudaGraph_t body_i = pi.conditional.phGraph_out[0];
  RB_CK(cudaStreamUpdateCaptureDependencies(so, &ni, nullptr, 1, cudaStreamSetCaptureDependencies));
  k_mp_update<<<grid, blk, 0, so>>>(a);
  cudaGraph_t tmp = nullptr;
  RB_CK(cudaStreamEndCapture(so, &tmp));

  // inner body: one flexible-CG iteration
  cudaStream_t si = m.cap[2];
  RB_CK(cudaStreamBeginCaptureToGraph(si, body_i, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  MpHierarchy h = m.h;
  h.alpha = setting_or(st.mixed_alpha, 1.8f);
  h.pre = (int)w.cfg.mg_pre;
  h.post = (int)w.cfg.mg_post;
  const int tiles = launch_mixed_vcycle(w.dev(), w.levels.data(), (int)w.levels.size(), w.mg, h, si);
  k_mp_zshift<<<1, blk, 0, si>>>(a, (unsigned)tiles);
  k_mp_dots<<<grid, blk, 0, si>>>(a);
  k_mp_direction<<<grid, blk, 0, si>>>(a);
  k_mp_matvec<<<grid, blk, 0, si>>>(a);
  k_mp_axpy<<<grid, blk, 0, si>>>(a, hi, 1);
  RB_CK(cudaStreamEndCapture(si, &tmp));

  k_mp_residual<<<grid, blk, 0, s>>>(a, ho, hi, 1, 1);  // residual of the result
  return cudaGetLastError();
}

// The same solve with the loops driven from the host (one wait per
// iteration to read the loop state): every kernel is launched on its own,
// so kernel timing and profilers see each of them.
cudaError_t direct_solve(World& w, MixedSolver& m) {
  const MpArgs a = mp_args(w, m);
  cudaStream_t s = w.stream;
  const dim3 grid((w.fw + BX - 1) / BX, (w.fh + BY * RR - 1) / (BY * RR)), blk(BX, BY);
  const ribo_world_settings& st = w.st;
  const int max_outer = setting_or(st.mixed_max_outer, 4), max_inner = setting_or(st.mixed_max_inner, 64);
  const double F = (double)w.fcells();
  MpHierarchy h = m.h;
  h.alpha = setting_or(st.mixed_alpha, 1.8f);
  h.pre = (int)w.cfg.mg_pre;
  h.post = (int)w.cfg.mg_post;
  cudaGraphConditionalHandle none = 0;
  RB_LAUNCH("mp_begin", 0.0, s,
            k_mp_begin<<<1, 256, 0, s>>>(a, max_outer, max_inner, setting_or(st.mixed_tol, 1e-5f),
                                         setting_or(st.mixed_inner_tol, 1e-3f), none, 0));
  MpCtl c{};
  auto read_ctl = [&]() {
    cudaError_t e = cudaMemcpyAsync(&c, m.ctl, sizeof c, cudaMemcpyDeviceToHost, s);
    return e == cudaSuccess ? cudaStreamSynchronize(s) : e;
  };
  for (int o = 0; o < max_outer; o++) {
    RB_LAUNCH("mp_residual", 25.0 * F, s, k_mp_residual<<<grid, blk, 0, s>>>(a, none, none, 0, 0));
    RB_CK(read_ctl());
    if (c.converged) break;
    for (int i = 0; i < max_inner; i++) {
      const int tiles = launch_mixed_vcycle(w.dev(), w.levels.data(), (int)w.levels.size(), w.mg, h, s);
      RB_LAUNCH("mp_zshift", 0.0, s, k_mp_zshift<<<1, blk, 0, s>>>(a, (unsigned)tiles));
      RB_LAUNCH("mp_dots", 17.0 * F, s, k_mp_dots<<<grid, blk, 0, s>>>(a));
      RB_LAUNCH("mp_direction", 13.0 * F, s, k_mp_direction<<<grid, blk, 0, s>>>(a));
      RB_LAUNCH("mp_matvec", 9.0 * F, s, k_mp_matvec<<<grid, blk, 0, s>>>(a));
      RB_LAUNCH("mp_axpy", 29.0 * F, s, k_mp_axpy<<<grid, blk, 0, s>>>(a, none, 0));
      RB_CK(read_ctl());
      if (c.inner_done) break;
    }
    RB_LAUNCH("mp_update", 21.0 * F, s, k_mp_update<<<grid, blk, 0, s>>>(a));
  }
  RB_LAUNCH("mp_residual", 25.0 * F, s, k_mp_residual<<<grid, blk, 0, s>>>(a, none, none, 1, 0));
  return cudaGetLastError();
}

}  // namespace

// Allocates the solver's buffers (World::init of a mixed-precision world).
ribo_status mixed_init(World& w) {
  const int nl = (int)w.levels.size();
  const int k = multigrid_first_coarse_level(w.levels.data(), nl);
  const MgLevel& last = w.levels[nl - 1];
  if (k == 0)
    return set_error(RIBO_INVALID_ARG, "mixed precision needs a fluid grid above %d cells", 4096);
  if ((long)last.nx * last.ny > COARSEST_CAP)
    return set_error(RIBO_INVALID_ARG, "mixed precision: coarsest level %dx%d above %d cells (raise mg_min_size)", last.nx,
                     last.ny, COARSEST_CAP);
  MixedSolver* m = new (std::nothrow) MixedSolver;
  if (!m) return set_error(RIBO_OOM, "host allocation");
  w.mixed = m;
  const size_t F = w.fcells();
  const size_t blocks = ((size_t)(w.fw + BX - 1) / BX) * ((w.fh + BY - 1) / BY);
  ribo_status r;
#define MP_ALLOC(ptr, bytes) \
  if ((r = w.alloc((void**)&(ptr), (bytes), #ptr)) != RIBO_OK) return r;
  MP_ALLOC(m->lo, F * 4);
  MP_ALLOC(m->r, F * 4);
  MP_ALLOC(m->e, F * 4);
  MP_ALLOC(m->d, F * 4);
  MP_ALLOC(m->q, F * 4);
  MP_ALLOC(m->z, F * 4);
  MP_ALLOC(m->label, F * 4);
  MP_ALLOC(m->part, blocks * 2 * 4);
  MP_ALLOC(m->ctl, sizeof(MpCtl));
  MP_ALLOC(m->comp_sum_r, COMP_CAP * 8);
  MP_ALLOC(m->comp_sum_z, COMP_CAP * 8);
  MP_ALLOC(m->comp_mean, COMP_CAP * 8);
  MP_ALLOC(m->comp_size, COMP_CAP * 8);
  MP_ALLOC(m->comp_mean_f, COMP_CAP * 4);
  MP_ALLOC(m->comp_shift, COMP_CAP * 4);
  const size_t tiles = part_entries(w.cfg, w.levels);
  MP_ALLOC(m->part_c, tiles * 8);
  MP_ALLOC(m->part_dom, tiles * 4);
  m->coarsest_cells = last.nx * last.ny;
  MP_ALLOC(m->inv, (size_t)m->coarsest_cells * m->coarsest_cells * 8);
  const int nh = half_levels(w);
  m->h.nhalf = nh;
  for (int l = 0; l < k; l++) {
    const size_t n = (size_t)w.levels[l].nx * w.levels[l].ny;
    const size_t es = l < nh ? 2 : 4;
    MP_ALLOC(m->h.fine[l].ef, n * es);
    if (l > 0) {
      MP_ALLOC(m->h.fine[l].rhs, n * es);
      MP_ALLOC(m->h.fine[l].E, n * 4);
    }
  }
#undef MP_ALLOC
  m->h.r = m->r;
  m->h.label = m->label;
  m->h.comp_mean = m->comp_mean_f;
  m->h.part_c = m->part_c;
  m->h.part_dom = m->part_dom;
  m->h.scale = reinterpret_cast<const float*>(reinterpret_cast<const char*>(m->ctl) + offsetof(MpCtl, scale));
  m->h.z = m->z;
  m->h.comp_sum_z = m->comp_sum_z;
  m->h.coarse_inv = m->inv;
  for (int i = 0; i < 3; i++)
    if (cudaStreamCreateWithFlags(&m->cap[i], cudaStreamNonBlocking) != cudaSuccess)
      return cuda_status(cudaGetLastError(), "stream");
  multigrid_prepare_mixed();
  return RIBO_OK;
}

// Device bytes mixed_init adds for a world with these levels.
size_t mixed_footprint(const ribo_world_cfg& c, const std::vector<MgLevel>& levels) {
  const size_t F = (size_t)c.fluid_w * c.fluid_h;
  const size_t blocks = ((size_t)(c.fluid_w + BX - 1) / BX) * ((c.fluid_h + BY - 1) / BY);
  const int nl = (int)levels.size();
  const int k = multigrid_first_coarse_level(levels.data(), nl);
  const size_t nc = (size_t)levels[nl - 1].nx * levels[nl - 1].ny;
  size_t b = F * 4 * 7 + blocks * 8 + part_entries(c, levels) * (8 + 4) + sizeof(MpCtl) + (size_t)COMP_CAP * (8 * 4 + 4 * 2) +
             nc * nc * 8;
  const int nh = k < HALF_LEVELS ? k : HALF_LEVELS;
  for (int l = 0; l < k; l++) {
    const size_t n = (size_t)levels[l].nx * levels[l].ny, es = l < nh ? 2 : 4;
    b += n * es + (l > 0 ? n * es + n * 4 : 0);
  }
  return b;
}

void mixed_free(World& w) {
  MixedSolver* m = w.mixed;
  if (!m) return;
  if (m->standalone) cudaGraphExecDestroy(m->standalone);
  for (int i = 0; i < 3; i++)
    if (m->cap[i]) cudaStreamDestroy(m->cap[i]);
  delete m;
  w.mixed = nullptr;
}

// Dense inverse by Gauss-Jordan elimination with partial pivoting (FP64).
static bool invert(std::vector<double>& a, int n, std::vector<double>& inv) {
  inv.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; i++) inv[(size_t)i * n + i] = 1.0;
  for (int col = 0; col < n; col++) {
    int piv = col;
    for (int r = col + 1; r < n; r++)
      if (fabs(a[(size_t)r * n + col]) > fabs(a[(size_t)piv * n + col])) piv = r;
    if (a[(size_t)piv * n + col] == 0.0) return false;
    if (piv != col)
      for (int j = 0; j < n; j++) {
        std::swap(a[(size_t)piv * n + j], a[(size_t)col * n + j]);
        std::swap(inv[(size_t)piv * n + j], inv[(size_t)col * n + j]);
      }
    const double p = a[(size_t)col * n + col];
    for (int j = 0; j < n; j++) {
      a[(size_t)col * n + j] /= p;
      inv[(size_t)col * n + j] /= p;
    }
    for (int r = 0; r < n; r++) {
      if (r == col) continue;
      const double f = a[(size_t)r * n + col];
      if (f == 0.0) continue;
      for (int j = 0; j < n; j++) {
        a[(size_t)r * n + j] -= f * a[(size_t)col * n + j];
        inv[(size_t)r * n + j] -= f * inv[(size_t)col * n + j];
      }
    }
  }
  return true;
}

// After every wall-mask build: water components (labels, sizes), the water
// flags of every level (any water child), and the dense inverse of the
// coarsest level's operator.  Runs on the host from the mask read back.
ribo_status mixed_setup(World& w) {
  MixedSolver* m = w.mixed;
  if (!m) return RIBO_OK;
  const int fw = w.fw, fh = w.fh;
  const size_t F = w.fcells();
  std::vector<uint8_t> mask(F);
  cudaError_t e = cudaMemcpyAsync(mask.data(), w.mask, F, cudaMemcpyDeviceToHost, w.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(w.stream);
  if (e != cudaSuccess) return cuda_status(e, "mixed setup");
  // 4-connected water components (breadth-first)
  std::vector<int> label(F, -1);
  std::vector<double> size(COMP_CAP, 0.0);
  std::vector<int> queue;
  queue.reserve(F);
  int ncomp = 0;
  for (size_t s = 0; s < F; s++) {
    if (mask[s] || label[s] >= 0) continue;
    const int id = ncomp < COMP_CAP ? ncomp : COMP_CAP - 1;
    ncomp++;
    queue.clear();
    queue.push_back((int)s);
    label[s] = id;
    for (size_t qi = 0; qi < queue.size(); qi++) {
      const int i = queue[qi], x = i % fw, y = i / fw;
      size[id] += 1.0;
      const int nb[4] = {x > 0 ? i - 1 : -1, x + 1 < fw ? i + 1 : -1, y > 0 ? i - fw : -1, y + 1 < fh ? i + fw : -1};
      for (int j : nb)
        if (j >= 0 && !mask[j] && label[j] < 0) {
          label[j] = id;
          queue.push_back(j);
        }
    }
  }
  if (ncomp > COMP_CAP) ncomp = COMP_CAP;
  m->ncomp = ncomp;
  // level water flags
  const int nl = (int)w.levels.size();
  std::vector<std::vector<uint8_t>> fl(nl);
  fl[0].resize(F);
  for (size_t i = 0; i < F; i++) fl[0][i] = mask[i] ? 0 : 1;
  for (int l = 1; l < nl; l++) {
    const int nx = w.levels[l].nx, ny = w.levels[l].ny, px = w.levels[l - 1].nx;
    fl[l].assign((size_t)nx * ny, 0);
    for (int y = 0; y < ny; y++)
      for (int x = 0; x < nx; x++) {
        const size_t c0 = (size_t)(2 * y) * px + 2 * x;
        fl[l][(size_t)y * nx + x] = (fl[l - 1][c0] | fl[l - 1][c0 + 1] | fl[l - 1][c0 + px] | fl[l - 1][c0 + px + 1]) ? 1 : 0;
      }
  }
  // coarsest operator: sum over water neighbours - (k + eps) on water cells, identity on the others
  const MgLevel& cl = w.levels[nl - 1];
  const int n = cl.nx * cl.ny;
  std::vector<double> A((size_t)n * n, 0.0), inv;
  const std::vector<uint8_t>& cf = fl[nl - 1];
  for (int y = 0; y < cl.ny; y++)
    for (int x = 0; x < cl.nx; x++) {
      const int i = y * cl.nx + x;
      if (!cf[i]) {
        A[(size_t)i * n + i] = 1.0;
        continue;
      }
      int k = 0;
      const int nb[4] = {x > 0 ? i - 1 : -1, x + 1 < cl.nx ? i + 1 : -1, y > 0 ? i - cl.nx : -1,
                         y + 1 < cl.ny ? i + cl.nx : -1};
      for (int j : nb)
        if (j >= 0 && cf[j]) {
          A[(size_t)i * n + j] = 1.0;
          k++;
        }
      A[(size_t)i * n + i] = -((double)k + (double)cl.eps);
    }
  if (!invert(A, n, inv)) return set_error(RIBO_CUDA_ERROR, "mixed setup: singular coarsest operator");
  // upload
  e = cudaMemcpyAsync(m->label, label.data(), F * 4, cudaMemcpyHostToDevice, w.stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->comp_size, size.data(), COMP_CAP * 8, cudaMemcpyHostToDevice, w.stream);
  for (int l = 1; l < nl && e == cudaSuccess; l++)
    e = cudaMemcpyAsync(w.mg.fluid + w.levels[l].off, fl[l].data(), fl[l].size(), cudaMemcpyHostToDevice, w.stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->inv, inv.data(), inv.size() * 8, cudaMemcpyHostToDevice, w.stream);
  MpCtl ctl{};
  ctl.ncomp = ncomp;
  double nwater = 0.0;
  for (int c = 0; c < ncomp; c++) nwater += size[c];
  ctl.nwater = (float)nwater;
  ctl.big = -1;
  for (int c = 0; c < ncomp; c++)
    if (ctl.big < 0 || size[c] > size[ctl.big]) ctl.big = c;
  ctl.scale[0] = ctl.scale[1] = 1.0f;
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->ctl, &ctl, sizeof ctl, cudaMemcpyHostToDevice, w.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(w.stream);
  return cuda_status(e, "mixed setup");
}

// The pressure solve of one step, on the world's stream.  Inside a step
// capture the solve's loops become nodes of the captured graph; otherwise a
// standalone graph of the solve (built once per settings) is launched.
ribo_status mixed_solve(World& w) {
  MixedSolver* m = w.mixed;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(w.stream, &cs);
  if (e != cudaSuccess) return cuda_status(e, "mixed solve");
  if (cs == cudaStreamCaptureStatusActive) {
    e = capture_solve(w, *m, w.stream);
    return cuda_status(e, "mixed solve capture");
  }
  if (w.cfg.no_graphs || w.timing) return cuda_status(direct_solve(w, *m), "mixed solve");
  if (m->standalone && memcmp(&m->built_for, &w.st, sizeof w.st) != 0) {
    cudaGraphExecDestroy(m->standalone);
    m->standalone = nullptr;
  }
  if (!m->standalone) {
    cudaGraph_t g = nullptr;
    e = cudaStreamBeginCapture(m->cap[0], cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      cudaError_t ce = capture_solve(w, *m, m->cap[0]);
      e = cudaStreamEndCapture(m->cap[0], &g);
      if (ce != cudaSuccess) e = ce;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&m->standalone, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_status(e, "mixed solve graph");
    m->built_for = w.st;
  }
  RB_LAUNCH("mixed_pressure_solve", 0.0, w.stream, e = cudaGraphLaunch(m->standalone, w.stream));
  return cuda_status(e, "mixed solve launch");
}

ribo_status mixed_info(World& w, uint32_t* outer, uint32_t* inner, double* rho) {
  if (!w.mixed) return set_error(RIBO_INVALID_ARG, "the world is not in mixed-precision mode");
  MpCtl c{};
  cudaError_t e = cudaMemcpyAsync(&c, w.mixed->ctl, sizeof c, cudaMemcpyDeviceToHost, w.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(w.stream);
  if (e != cudaSuccess) return cuda_status(e, "mixed info");
  if (outer) *outer = (uint32_t)c.outer;
  if (inner) *inner = (uint32_t)c.total_inner;
  if (rho) *rho = c.rho;
  return RIBO_OK;
}

float* mixed_pressure_lo(World& w) { return w.mixed ? w.mixed->lo : nullptr; }

}  // namespace ribo
