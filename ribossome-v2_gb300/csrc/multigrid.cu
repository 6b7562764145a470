// Pressure Poisson solve: cell-centred geometric multigrid with red-black
// Gauss-Seidel smoothing (shaders/world/multigrid.wgsl, schedule
// src/world/mod.rs:1545-1577) and the Jacobi alternative
// (shaders/world/fluid.wgsl:553-608, src/world/mod.rs:1578-1581).
//
// Red-black sweeps update one colour from the other colour only, so every
// fused or tiled variant below produces the same bits as one dispatch per
// half-sweep.
#include <cuda_fp16.h>
#include <string.h>

#include <type_traits>
#include <vector>

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

// ---------------------------------------------------------------------------
// One dispatch per half-sweep / restrict / prolong, as the reference records
// them (src/world/mod.rs:1545-1577).

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

// Neighbour codes of level L (0: not water, else 1 + the water neighbours
// inside the level, multigrid.wgsl:29-45) and, when C is given, the water
// flags of the next coarser level: a coarse cell is water when any of its four
// children is (the restriction's nf > 0, multigrid.wgsl:82-105).  The flags
// follow the wall mask alone, so they and the codes are built once per mask.
__global__ void k_mg_codes(Lv L, uint8_t* __restrict__ code, uint8_t* __restrict__ cfl, int cnx, int cny) {
  int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
  if (x >= L.nx || y >= L.ny) return;
  const size_t i = (size_t)y * L.nx + x;
  const uint8_t* fl = L.fl;
  uint8_t k = 0;
  if (fl[i])
    k = (uint8_t)(1 + (x > 0 && fl[i - 1]) + (x + 1 < L.nx && fl[i + 1]) + (y > 0 && fl[i - L.nx]) +
                  (y + 1 < L.ny && fl[i + L.nx]));
  code[i] = k;
  if (cfl && !(x & 1) && !(y & 1) && x / 2 < cnx && y / 2 < cny)
    cfl[(size_t)(y / 2) * cnx + x / 2] = (fl[i] | fl[i + 1] | fl[i + L.nx] | fl[i + L.nx + 1]) ? 1 : 0;
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

// ---------------------------------------------------------------------------
// Fused V-cycle.
//
// Fine levels: one kernel does "pre-smooth nu sweeps + residual + restrict"
// and one does "prolong + post-smooth nu sweeps", each on a tile held in
// shared memory with a halo of H = 2nu+1 (resp. 2nu) cells: the box.  After
// half-sweep s the cells at distance > s from the edge of the box hold
// exactly the values a dispatch per half-sweep would give, whatever the cells
// nearer the edge hold, so after 2nu half-sweeps the tile and its one-cell
// ring are exact.  Every half-sweep therefore updates all cells at distance
// >= 1 (the extra updates near the edge are wasted but keep every lane of a
// warp on a full row).
//
// The box has a fixed shape per kernel (RbBox: W = 2 QW + 2 columns by
// RH = ROWS + 2 rows), and the tile is what the halo leaves inside it:
// TW = W - 2H by TH = RH - 2H.  Cells are stored by colour -- colour c of row
// j is plane c, row j, index q = i >> 1, the two colours alternating along a
// row -- so the cells one half-sweep updates and the other-colour neighbours
// they read are contiguous, and a warp's shared-memory accesses are
// conflict-free.  A neighbour code per cell (0: no update; else 1 + the
// number of water neighbours) replaces the four flag tests: a non-water
// cell's p is +0.0 and stays so, and adding +0.0 to the running neighbour
// sum (which starts at +0.0 and never becomes -0.0 in round-to-nearest)
// leaves it unchanged, so the sum of all four neighbours is the sum of the
// water ones, bit for bit.  Cells outside the level load as not water, p = 0.
//
// Coarse levels (at most MG_SMEM_CELLS cells on the top one): one CTA runs
// the whole remaining V-cycle in shared memory.
//
// Level 0 reads pressure_a (masked), the divergence and the level-0 water
// flags (the negated wall mask, rebuilt with it) directly -- mg_init -- and
// the last post kernel writes pressure_a (mg_finish).  A coarse level's p
// starts every cycle at 0 (mg_restrict zeroes it), so the pre kernels of
// levels >= 1 do not load it.
constexpr int MG_SMEM_CELLS = 4096;
constexpr int COARSE_THREADS = 1024;

template <int QW_, int ROWS_>
struct RbBox {
  static constexpr int QW = QW_, ROWS = ROWS_;
  static constexpr int W = 2 * QW + 2, RH = ROWS + 2;  // box columns and rows
  static constexpr int QS = QW + 1;                    // cells of one colour in a box row
  // stride of a colour plane: its RH x QS cells, padded to 16 words past a
  // multiple of 32 so that lanes alternating between the planes (natural
  // order loads and stores) hit distinct banks
  static constexpr int PL = RH * QS + ((16 - (RH * QS) % 32) + 32) % 32;
  static constexpr int RPW = 32 / QW;                  // box rows a warp sweeps at once
  static constexpr int STEPS = ROWS / (RPW * BY);      // sweep steps of a warp per half-sweep
  static_assert(QW == 16 || QW == 32, "a box row is swept by a warp or a half-warp");
  static_assert(ROWS % (RPW * BY) == 0, "box rows split evenly over the warps");
  // p and rhs (float, both colours), neighbour codes (both colours), water
  // flags (natural order, used to build the codes)
  static constexpr size_t SMEM = (size_t)2 * PL * 4 * 2 + (size_t)2 * PL + (size_t)RH * W;
  static constexpr size_t SMEM_CODED = (size_t)2 * PL * 4 * 2 + (size_t)2 * PL;  // no flag array (codes loaded)
  __host__ __device__ static constexpr int tile_w(int H) { return W - 2 * H; }
  __host__ __device__ static constexpr int tile_h(int H) { return RH - 2 * H; }
  __host__ __device__ static constexpr bool fits(int H) { return tile_w(H) >= 2 && tile_h(H) >= 2; }
};
using BoxBig = RbBox<32, 48>;    // 66 x 50 box: a 52 x 36 tile with 3 + 3 sweeps
using BoxSmall = RbBox<16, 32>;  // 34 x 34 box: a 20 x 20 tile with 3 + 3 sweeps

template <class B>
struct RbSmem {
  float* P;    // [2][RH][QS]
  float* R;    // [2][RH][QS]
  uint8_t* K;  // [2][RH][QS]
  uint8_t* F;  // [RH][W]
  int par;     // colour of box cell (0, 0)
  __device__ __forceinline__ RbSmem(unsigned char* raw, int par_)
      : P(reinterpret_cast<float*>(raw)),
        R(P + 2 * B::PL),
        K(reinterpret_cast<uint8_t*>(R + 2 * B::PL)),
        F(K + 2 * B::PL),
        par(par_) {}
  __device__ __forceinline__ int at(int j, int i) const { return ((i + j + par) & 1) * B::PL + j * B::QS + (i >> 1); }
};

// Sum of the four neighbours of box cell (j, i) (split index a), in the order
// of multigrid.wgsl:34-45: left, right, below, above.
template <class B>
__device__ __forceinline__ float rb_nb_sum(const RbSmem<B>& S, int j, int i, int a) {
  const int o = i & 1;
  const int b = a + (((i + j + S.par) & 1) ? -B::PL : B::PL);  // same (row, q) in the other colour
  float s = 0.0f;
  s += S.P[b - 1 + o];
  s += S.P[b + o];
  s += S.P[b - B::QS];
  s += S.P[b + B::QS];
  return s;
}

// Fills the box from the level: `cell(in, gi, gx, gy, f, r, p)` gives the
// water flag, rhs and initial p of a cell (gi = its index, 0 outside the
// level); then builds the neighbour codes.  Loads are issued for every cell
// (index 0 outside the level) so they overlap.
// With CODED the cell's byte is its neighbour code (precomputed per level,
// 0: not water): the box edge is forced to 0 (never updated) and no code
// pass runs.
template <class B, bool CODED = false, class Fn>
__device__ __forceinline__ void rb_load(const RbSmem<B>& S, int X0, int Y0, int nx, int ny, Fn&& cell) {
  const int tid = threadIdx.y * BX + threadIdx.x;
  constexpr int N = B::W * B::RH, NT = BX * BY, IT = (N + NT - 1) / NT, BATCH = 4;
#pragma unroll
  for (int it0 = 0; it0 < IT; it0 += BATCH) {
    uint8_t f[BATCH];
    float r[BATCH], p[BATCH];
#pragma unroll
    for (int u = 0; u < BATCH; u++) {  // a batch's loads are all issued before its stores
      const int e = tid + (it0 + u) * NT;
      const int j = e / B::W, i = e - j * B::W;
      const int gx = X0 + i, gy = Y0 + j;
      const bool in = it0 + u < IT && e < N && gx >= 0 && gy >= 0 && gx < nx && gy < ny;
      const size_t gi = in ? (size_t)gy * nx + gx : 0;
      cell(in, gi, gx, gy, f[u], r[u], p[u]);
    }
#pragma unroll
    for (int u = 0; u < BATCH; u++) {
      const int e = tid + (it0 + u) * NT;
      if (it0 + u >= IT || e >= N) continue;
      const int j = e / B::W, i = e - j * B::W;
      const int a = S.at(j, i);
      if constexpr (CODED) S.K[a] = (i == 0 || j == 0 || i == B::W - 1 || j == B::RH - 1) ? 0 : f[u];
      else S.F[e] = f[u];
      S.P[a] = f[u] ? p[u] : 0.0f;
      S.R[a] = f[u] ? r[u] : 0.0f;
    }
  }
  __syncthreads();
  if constexpr (!CODED) {
    for (int e = tid; e < B::W * B::RH; e += BX * BY) {
      const int j = e / B::W, i = e - j * B::W;
      uint8_t k = 0;
      if (i > 0 && j > 0 && i < B::W - 1 && j < B::RH - 1 && S.F[e])
        k = (uint8_t)(1 + S.F[e - 1] + S.F[e + 1] + S.F[e - B::W] + S.F[e + B::W]);
      S.K[S.at(j, i)] = k;
    }
    __syncthreads();
  }
}

// nsweeps half-sweeps over the cells at distance >= 1 from the box edge;
// half-sweep s updates colour (s & 1) ^ c0 (red first for c0 = 0), with the
// update of multigrid.wgsl:60-77.
template <class B>
__device__ __forceinline__ void rb_sweeps(int nsweeps, int c0, float eps, const RbSmem<B>& S) {
  const int sub = B::RPW == 1 ? 0 : (int)threadIdx.x / B::QW, ql = (int)threadIdx.x % B::QW;
  for (int s = 0; s < nsweeps; s++) {
    const int c = (s & 1) ^ c0;
    float* Pc = S.P + c * B::PL;
    const float* Po = S.P + (c ^ 1) * B::PL;
    const float* Rc = S.R + c * B::PL;
    const uint8_t* Kc = S.K + c * B::PL;
#pragma unroll
    for (int it = 0; it < B::STEPS; it++) {
      const int j = 1 + (it * BY + (int)threadIdx.y) * B::RPW + sub;
      const int o = (c + S.par + j) & 1;  // column parity of colour c in row j
      const int a = j * B::QS + ql + 1 - o;  // column 2q + o, in [1, W - 2]
      const uint8_t kk = Kc[a];
      if (kk) {
        float sum = 0.0f;
        sum += Po[a - 1 + o];
        sum += Po[a + o];
        sum += Po[a - B::QS];
        sum += Po[a + B::QS];
        Pc[a] = (sum - Rc[a]) / ((float)(kk - 1) + eps);
      }
    }
    __syncthreads();
  }
}

// Residual r - (s - (k + eps) p) of water cell (j, i) (multigrid.wgsl:82-105).
template <class B>
__device__ __forceinline__ bool rb_residual(const RbSmem<B>& S, int j, int i, float eps, float& res) {
  const int a = S.at(j, i);
  const uint8_t kk = S.K[a];
  if (!kk) return false;
  const float s = rb_nb_sum<B>(S, j, i, a);
  res = S.R[a] - (s - ((float)(kk - 1) + eps) * S.P[a]);
  return true;
}

// One fine level of one world in a fused pre- or post-smooth launch.
struct MgPass {
  Lv L, C;               // the level and the next coarser one
  const float* p_src;    // p loaded with the box (pre on level 0: pressure_a; post: pre-smoothed p)
  const float* r_src;    // right-hand side of the level
  const uint8_t* f_src;  // water flags of the level
  float* p_out;          // smoothed p of the level
  const uint8_t* k_src;  // neighbour codes of the level (null: built from the flags)
};
// A launch over one world's level, or over the same level index of a batch
// of worlds (the CTA finds its world as the per-cell passes do).
struct MgOne {
  MgPass e;
};
struct MgSet {
  const MgPass* e;
  const int* start;  // [n + 1]
  const int* nbx;    // [n]
  int n;
};
__device__ __forceinline__ void mg_locate(const MgOne& s, MgPass& e, int& tx, int& ty) {
  e = s.e;
  tx = (int)blockIdx.x;
  ty = (int)blockIdx.y;
}
__device__ __forceinline__ void mg_locate(const MgSet& s, MgPass& e, int& tx, int& ty) {
  const int w = batch_member(s.start, s.n);
  e = s.e[w];
  const int r = (int)blockIdx.x - __ldg(s.start + w), nb = __ldg(s.nbx + w);
  tx = r % nb;
  ty = r / nb;
}

// Stores the tile (box cells H.., H..) of p to a level array.
template <class B, class St>
__device__ __forceinline__ void rb_store_tile(const RbSmem<B>& S, int H, int x0, int y0, int nx, int ny, St&& put) {
  const int TW = B::tile_w(H), TH = B::tile_h(H);
  for (int y = threadIdx.y; y < TH; y += BY)
    for (int x = threadIdx.x; x < TW; x += BX) {
      const int gx = x0 + x, gy = y0 + y;
      if (gx < nx && gy < ny) put((size_t)gy * nx + gx, S.P[S.at(H + y, H + x)]);
    }
}

// Pre-smooth (nu sweeps) + residual + restrict (multigrid.wgsl:60-105).
// Coded boxes need no flag array: seven fit in an SM's shared memory, and a
// single world's kernels fit seven CTAs' registers (32 per thread) without
// spilling in the sweeps; the batched kernels (member lookup) are held to six.
template <class S>
constexpr int mg_min_blocks(bool coded) { return coded ? (std::is_same<S, MgOne>::value ? 7 : 6) : 1; }

template <class B, bool TOP, class S, bool CODED>
__global__ void __launch_bounds__(BX* BY, mg_min_blocks<S>(CODED)) k_mg_pre(const __grid_constant__ S s, int nu) {
  MgPass e;
  int tile_x, tile_y;
  mg_locate(s, e, tile_x, tile_y);
  const Lv& L = e.L;
  const Lv& C = e.C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int H = 2 * nu + 1, TW = B::tile_w(H), TH = B::tile_h(H);
  const int x0 = tile_x * TW, y0 = tile_y * TH;
  const RbSmem<B> Sm(smem_raw, (x0 + y0) & 1);  // box cell (0, 0) is (x0 - H, y0 - H)
  const float* __restrict__ p_src = e.p_src;
  const float* __restrict__ r_src = e.r_src;
  const uint8_t* __restrict__ f_src = e.f_src;
  const uint8_t* __restrict__ k_src = e.k_src;
  auto cell = [&](const uint8_t* __restrict__ src) {
    return [&, src](bool in, size_t gi, int, int, uint8_t& f, float& r, float& p) {
      f = in ? src[gi] : 0;
      r = r_src[gi];
      p = TOP ? p_src[gi] : 0.0f;  // mg_init: p = water ? pressure_a : 0 (levels >= 1 start at 0)
    };
  };
  rb_load<B, CODED>(Sm, x0 - H, y0 - H, L.nx, L.ny, cell(CODED ? k_src : f_src));
  rb_sweeps<B>(2 * nu, 0, L.eps, Sm);
  float* __restrict__ p_out = e.p_out;
  rb_store_tile<B>(Sm, H, x0, y0, L.nx, L.ny, [&](size_t i, float v) { p_out[i] = v; });
  // residual of the 4 children of each coarse cell of the tile, x2 average
  for (int cj = threadIdx.y; cj < TH / 2; cj += BY)
    for (int ci = threadIdx.x; ci < TW / 2; ci += BX) {
      const int cgx = tile_x * (TW / 2) + ci, cgy = tile_y * (TH / 2) + cj;
      if (cgx >= C.nx || cgy >= C.ny) continue;
      float sum = 0.0f;
      uint32_t nf = 0;
#pragma unroll
      for (uint32_t q = 0; q < 4; q++) {
        float res;
        if (!rb_residual<B>(Sm, H + 2 * cj + (int)(q >> 1), H + 2 * ci + (int)(q & 1u), L.eps, res)) continue;
        sum += res;
        nf++;
      }
      const size_t ci_g = (size_t)cgy * C.nx + cgx;
      C.fl[ci_g] = nf > 0u ? 1 : 0;
      C.rhs[ci_g] = nf > 0u ? 2.0f * sum / (float)(nf > 1u ? nf : 1u) : 0.0f;
    }
}

// Prolong (add the coarse correction to water cells) + post-smooth nu sweeps
// (multigrid.wgsl:108-114, 60-77).
template <class B, class S, bool CODED>
__global__ void __launch_bounds__(BX* BY, mg_min_blocks<S>(CODED)) k_mg_post(const __grid_constant__ S s, int nu) {
  MgPass e;
  int tile_x, tile_y;
  mg_locate(s, e, tile_x, tile_y);
  const Lv& L = e.L;
  const Lv& C = e.C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int H = 2 * nu, TW = B::tile_w(H), TH = B::tile_h(H);
  const int x0 = tile_x * TW, y0 = tile_y * TH;
  const RbSmem<B> Sm(smem_raw, (x0 + y0) & 1);
  const float* __restrict__ p_src = e.p_src;
  const float* __restrict__ r_src = e.r_src;
  const uint8_t* __restrict__ f_src = e.f_src;
  const float* __restrict__ cp = C.p;
  const int cnx = C.nx;
  const uint8_t* __restrict__ k_src = e.k_src;
  auto cell = [&](const uint8_t* __restrict__ src) {
    return [&, src](bool in, size_t gi, int gx, int gy, uint8_t& f, float& r, float& p) {
      f = in ? src[gi] : 0;
      r = r_src[gi];
      p = p_src[gi] + cp[in ? (size_t)(gy / 2) * cnx + gx / 2 : 0];
    };
  };
  rb_load<B, CODED>(Sm, x0 - H, y0 - H, L.nx, L.ny, cell(CODED ? k_src : f_src));
  rb_sweeps<B>(2 * nu, 0, L.eps, Sm);
  float* __restrict__ p_out = e.p_out;
  rb_store_tile<B>(Sm, H, x0, y0, L.nx, L.ny, [&](size_t i, float v) { p_out[i] = v; });
}

// The V-cycle below (and including) level `top`, in one CTA.
struct CoarseSet {
  int n;  // levels in the set (top .. coarsest)
  int nx[16], ny[16];
  float eps[16];
  int off[16];  // first cell of each level's padded colour planes in shared memory
  int total;    // cells of all levels' planes
  const float* rhs_top;
  const uint8_t* fl_top;
  float* p_out;  // level `top` result
};
// The coarse V-cycle of one world: its levels from the first one that fits
// in shared memory down, and, when that is level 0 (top), the world's own
// pressure_a, divergence and wall mask.
struct CoarsePass {
  CoarseSet cs;
  const uint8_t* mask;
  const float* div;
  float* pa;
  int fw;
  int top;
  // Mixed-precision preconditioner form (null inv: the reference's V-cycle):
  // restriction 1/2 * sum over water children, the coarse correction
  // prolonged times `alpha`, post-smoothing colours reversed (the V-cycle is
  // then a symmetric operator), and the coarsest level solved exactly in
  // FP64 with its dense inverse `inv` (row-major, cells x cells).
  const double* inv;
  float alpha;
};
struct CoarseOne {
  CoarsePass e;
};
struct CoarseMany {
  const CoarsePass* e;  // [n], one CTA each
  int n;
};
__device__ __forceinline__ const CoarsePass& coarse_of(const CoarseOne& s) { return s.e; }
__device__ __forceinline__ const CoarsePass& coarse_of(const CoarseMany& s) { return s.e[blockIdx.x]; }

// A coarse level in shared memory: the level plus a ring of non-water cells,
// (nx + 2) x (ny + 2), stored by colour like the fine boxes (plane
// (i + j) & 1, row j, index i >> 1 in padded coordinates), with the same
// neighbour codes, so its sweeps read contiguous, conflict-free words and
// need no flag tests or bounds checks.
__host__ __device__ constexpr int coarse_qs(int nx) { return (nx + 3) / 2; }
__host__ __device__ constexpr int coarse_cells(int nx, int ny) { return 2 * (ny + 2) * coarse_qs(nx); }
struct CLv {
  int nx, ny, qs, pl;
  float eps;
  float* P;
  float* R;
  uint8_t* K;
  uint8_t* F;
  __device__ __forceinline__ int at(int y, int x) const {  // level cell (x, y)
    const int j = y + 1, i = x + 1;
    return ((i + j) & 1) * pl + j * qs + (i >> 1);
  }
};
__device__ __forceinline__ CLv coarse_level(const CoarseSet& cs, unsigned char* smem, int l) {
  CLv L;
  L.nx = cs.nx[l];
  L.ny = cs.ny[l];
  L.qs = coarse_qs(L.nx);
  L.pl = (L.ny + 2) * L.qs;
  L.eps = cs.eps[l];
  float* base = reinterpret_cast<float*>(smem);
  L.P = base + cs.off[l];
  L.R = base + cs.total + cs.off[l];
  L.K = reinterpret_cast<uint8_t*>(base + 2 * cs.total) + cs.off[l];
  L.F = L.K + cs.total;
  return L;
}
// Neighbour codes from the water flags (F) of a level.
__device__ __forceinline__ void coarse_codes(const CLv& L) {
  for (int e = threadIdx.x; e < L.nx * L.ny; e += COARSE_THREADS) {
    const int y = e / L.nx, x = e - y * L.nx;
    const int a = L.at(y, x);
    uint8_t k = 0;
    if (L.F[a]) {
      const int o = (x + 1) & 1, b = a + (((x + y) & 1) ? -L.pl : L.pl);
      k = (uint8_t)(1 + L.F[b - 1 + o] + L.F[b + o] + L.F[b - L.qs] + L.F[b + L.qs]);
    }
    L.K[a] = k;
  }
}
// One colour of a red-black sweep (multigrid.wgsl:60-77): warps take rows,
// lanes the colour's cells of the row.
__device__ __forceinline__ void coarse_sweep(const CLv& L, int c) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float* Pc = L.P + c * L.pl;
  const float* Po = L.P + (c ^ 1) * L.pl;
  const float* Rc = L.R + c * L.pl;
  const uint8_t* Kc = L.K + c * L.pl;
  for (int j = 1 + warp; j <= L.ny; j += COARSE_THREADS / 32) {
    const int o = (c + j) & 1;  // padded column parity of colour c in row j
    for (int q = lane + 1 - o; 2 * q + o <= L.nx; q += 32) {
      const int a = j * L.qs + q;
      const uint8_t kk = Kc[a];
      if (!kk) continue;
      float sum = 0.0f;
      sum += Po[a - 1 + o];
      sum += Po[a + o];
      sum += Po[a - L.qs];
      sum += Po[a + L.qs];
      Pc[a] = (sum - Rc[a]) / ((float)(kk - 1) + L.eps);
    }
  }
  __syncthreads();
}
// Residual of level cell (x, y) if it is water (multigrid.wgsl:82-105).
__device__ __forceinline__ bool coarse_residual(const CLv& L, int y, int x, float& res) {
  const int a = L.at(y, x);
  const uint8_t kk = L.K[a];
  if (!kk) return false;
  const int o = (x + 1) & 1, b = a + (((x + y) & 1) ? -L.pl : L.pl);
  float s = 0.0f;
  s += L.P[b - 1 + o];
  s += L.P[b + o];
  s += L.P[b - L.qs];
  s += L.P[b + L.qs];
  res = L.R[a] - (s - ((float)(kk - 1) + L.eps) * L.P[a]);
  return true;
}

// The downward half of a coarse set's V-cycle: pre-smooth and restrict from
// the top level (in shared memory, codes built) to the coarsest.
template <bool MP>
__device__ __forceinline__ void coarse_down(const CoarsePass& e, unsigned char* smem, int nu_pre) {
  const CoarseSet& cs = e.cs;
  for (int l = 0; l + 1 < cs.n; l++) {
    const CLv L = coarse_level(cs, smem, l), C = coarse_level(cs, smem, l + 1);
    for (int k = 0; k < nu_pre; k++) {
      coarse_sweep(L, 0);
      coarse_sweep(L, 1);
    }
    for (int ci = threadIdx.x; ci < C.nx * C.ny; ci += COARSE_THREADS) {
      const int cy = ci / C.nx, cx = ci - cy * C.nx;
      float sum = 0.0f;
      uint32_t nf = 0;
      for (uint32_t q = 0; q < 4; q++) {
        float res;
        if (!coarse_residual(L, cy * 2 + (int)(q >> 1), cx * 2 + (int)(q & 1u), res)) continue;
        sum += res;
        nf++;
      }
      const int a = C.at(cy, cx);
      C.F[a] = nf > 0u ? 1 : 0;
      if (MP) C.R[a] = nf > 0u ? 0.5f * sum : 0.0f;
      else C.R[a] = nf > 0u ? 2.0f * sum / (float)(nf > 1u ? nf : 1u) : 0.0f;
      C.P[a] = 0.0f;
    }
    __syncthreads();
    coarse_codes(C);
    __syncthreads();
  }
}

// The upward half: prolong the coarser level's correction and post-smooth,
// up to the top level, whose p is left in shared memory.
template <bool MP>
__device__ __forceinline__ void coarse_up(const CoarsePass& e, unsigned char* smem, int nu_post) {
  const CoarseSet& cs = e.cs;
  for (int l = cs.n - 2; l >= 0; l--) {
    const CLv L = coarse_level(cs, smem, l), C = coarse_level(cs, smem, l + 1);
    for (int idx = threadIdx.x; idx < L.nx * L.ny; idx += COARSE_THREADS) {
      const int y = idx / L.nx, x = idx - y * L.nx;
      const int a = L.at(y, x);
      if (!L.K[a]) continue;
      const float pc = C.P[C.at(y / 2, x / 2)];
      L.P[a] += MP ? e.alpha * pc : pc;
    }
    __syncthreads();
    const int c0 = MP ? 1 : 0;
    for (int k = 0; k < nu_post; k++) {
      coarse_sweep(L, c0);
      coarse_sweep(L, c0 ^ 1);
    }
  }
}

// Rows [i0, i1) of the exact FP64 coarsest solve: p_i = sum_j inv[i][j] rhs_j
// (the inverse indexes the level's cells in row-major order), one warp per
// row, stored at the cell's place in `P` (L's p plane, in this CTA or, through
// distributed shared memory, in another one).
__device__ __forceinline__ void coarsest_dense_rows(const CoarsePass& e, const CLv& L, const float* rn, float* P, int i0,
                                                    int i1) {
  const int nc = L.nx * L.ny;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = i0 + warp; i < i1; i += COARSE_THREADS / 32) {
    const double* row = e.inv + (size_t)i * nc;
    double acc = 0.0;
    for (int j = lane; j < nc; j += 32) acc += row[j] * (double)rn[j];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) P[L.at(i / L.nx, i % L.nx)] = (float)acc;
  }
}

// The V-cycle of a coarse set whose top level (flags, rhs, p) is in shared
// memory with its codes built: down to the coarsest level, its solve (the
// reference's sweeps, or in the mixed-precision form the exact FP64 solve
// with the dense inverse), and back up; the top level's p is left in shared
// memory.
template <bool MP>
__device__ __forceinline__ void coarse_cycle(const CoarsePass& e, unsigned char* smem, int nu_pre, int nu_post,
                                             int coarse) {
  const CoarseSet& cs = e.cs;
  coarse_down<MP>(e, smem, nu_pre);
  {
    const CLv L = coarse_level(cs, smem, cs.n - 1);
    if (MP) {
      const int nc = L.nx * L.ny;
      float* rn = reinterpret_cast<float*>(smem + (size_t)10 * cs.total);
      for (int i = threadIdx.x; i < nc; i += COARSE_THREADS) rn[i] = L.R[L.at(i / L.nx, i % L.nx)];
      __syncthreads();
      coarsest_dense_rows(e, L, rn, L.P, 0, nc);
      __syncthreads();
    } else {
      for (int k = 0; k < coarse; k++) {
        coarse_sweep(L, 0);
        coarse_sweep(L, 1);
      }
    }
  }
  coarse_up<MP>(e, smem, nu_post);
}

// Clears a coarse set's planes (rings and rows outside stay non-water, p =
// rhs = 0), loads its top level (the world's own pressure_a, divergence and
// wall mask when the top is level 0) and builds the top level's codes.
__device__ __forceinline__ void coarse_load_top(const CoarsePass& e, unsigned char* smem) {
  const CoarseSet& cs = e.cs;
  const bool TOP = e.top != 0;
  {
    float* f = reinterpret_cast<float*>(smem);
    for (int i = threadIdx.x; i < 2 * cs.total; i += COARSE_THREADS) f[i] = 0.0f;
    uint8_t* b = reinterpret_cast<uint8_t*>(f + 2 * cs.total);
    for (int i = threadIdx.x; i < 2 * cs.total; i += COARSE_THREADS) b[i] = 0;
  }
  __syncthreads();
  const CLv L = coarse_level(cs, smem, 0);
  for (int idx = threadIdx.x; idx < L.nx * L.ny; idx += COARSE_THREADS) {
    const int y = idx / L.nx, x = idx - y * L.nx;
    uint8_t f;
    float r, p = 0.0f;
    if (TOP) {
      const size_t gi = (size_t)y * e.fw + x;
      f = e.mask[gi] ? 0 : 1;
      r = e.div[gi];
      p = f ? e.pa[gi] : 0.0f;
    } else {
      f = cs.fl_top[idx];
      r = cs.rhs_top[idx];
    }
    const int a = L.at(y, x);
    L.F[a] = f;
    L.P[a] = f ? p : 0.0f;
    L.R[a] = f ? r : 0.0f;
  }
  __syncthreads();
  coarse_codes(L);
  __syncthreads();
}

// Stores the top level's p (to pressure_a when the top is level 0).
__device__ __forceinline__ void coarse_store_top(const CoarsePass& e, unsigned char* smem) {
  const CoarseSet& cs = e.cs;
  const CLv L = coarse_level(cs, smem, 0);
  for (int idx = threadIdx.x; idx < L.nx * L.ny; idx += COARSE_THREADS) {
    const int y = idx / L.nx, x = idx - y * L.nx;
    const float v = L.P[L.at(y, x)];
    if (e.top) e.pa[(size_t)y * e.fw + x] = v;
    else cs.p_out[idx] = v;
  }
}

template <class S, bool MP = false>
__global__ void __launch_bounds__(COARSE_THREADS) k_mg_coarse(const __grid_constant__ S s, int nu_pre, int nu_post, int coarse) {
  const CoarsePass& e = coarse_of(s);
  extern __shared__ __align__(16) unsigned char smem[];
  coarse_load_top(e, smem);
  coarse_cycle<MP>(e, smem, nu_pre, nu_post, coarse);
  coarse_store_top(e, smem);
}

// ---------------------------------------------------------------------------
// Cluster V-cycle of the latency-bound levels.
//
// The small fine levels (the slab levels: at most SLAB_MAX_CELLS owned cells
// per CTA) and the coarsest level run in ONE launch per V-cycle, on a
// thread-block cluster of NC CTAs of COARSE_THREADS threads.  CTA r owns rows
// [r R_l, (r + 1) R_l) of slab level l, with R_l = 2 R_{l+1} (even), so the
// children of a coarse row are rows of the same CTA: restriction stays inside
// the CTA.  A CTA holds its rows in a window with G = 2 nu + 1 ghost rows on
// each side, stored like the coarse levels (colour planes, a non-water column
// on each side, neighbour codes); the window's first and last rows are never
// updated.  This is the fine kernels' box argument along y: after s
// half-sweeps the rows at distance >= s from the window edge hold exactly
// what one dispatch per half-sweep gives, so after 2 nu half-sweeps the owned
// rows and their one-row ring are exact, and a level is swept with block
// barriers only.  Owners push what other windows need through distributed
// shared memory (remote stores, made visible by the next cluster barrier):
// the right-hand sides and water flags of the rows they restrict, their
// pre-smoothed p, and the rows of their post-smoothed p that the finer
// level's windows prolong from (into a per-level staging area of natural-
// order rows).  The coarsest slab level restricts into CTA 0's copy of the
// coarsest level, which CTA 0 solves alone (the coarse kernel's code) while
// the other CTAs wait at the next cluster barrier.  Cluster barriers are
// hardware barriers: every CTA executes the same sequence of them, and no
// thread spins on memory.
constexpr int MG_MAX_SLAB_LEVELS = 8;
constexpr int SLAB_MAX_CELLS = 1024;  // owned cells per CTA of a slab level (more: issue-bound on NC SMs)
struct SlabLv {
  int nx, ny;
  int R;       // rows owned per CTA
  int wr;      // window rows: R + 2 G
  int qs, pl;  // cells per colour row, cells per colour plane (wr * qs)
  int off;     // first cell of the window's planes
  int so;      // first float of the staging area (coarse correction rows)
  int srows;   // staging rows: R / 2 + G + 1
  int cnx;     // width of the next coarser level (staging row length)
  float eps;
};
struct ClusterPass {
  int nslab;  // slab levels, finest first (levels m .. g - 1)
  SlabLv w[MG_MAX_SLAB_LEVELS];
  int G;      // ghost rows on each side
  int par;    // colour of window cell (row 0, padded column 0), the same in every CTA
  int nc;     // CTAs of the cluster
  CoarsePass co;  // the coarsest level (g = nl - 1); co.cs.total = cells of every plane
  // level m's inputs and output: levels >= 1 read rhs and flags and write p;
  // level 0 reads the wall mask, divergence and pressure_a and writes pressure_a
  const float* rhs_top;
  const uint8_t* fl_top;
  float* p_out;
  uint32_t* status;  // index checks of the bounds-checked build
};

__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory"); }
__device__ __forceinline__ void cluster_sync() {
  cluster_arrive();
  cluster_wait();
}
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;\n" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_size() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;\n" : "=r"(r));
  return r;
}
// The address of `p` (this CTA's shared memory) in CTA `rank` of the cluster.
template <class T>
__device__ __forceinline__ T* cta_map(T* p, uint32_t rank) {
  uint64_t r;
  asm volatile("mapa.u64 %0, %1, %2;\n" : "=l"(r) : "l"(reinterpret_cast<uint64_t>(p)), "r"(rank));
  return reinterpret_cast<T*>(r);
}
__device__ __forceinline__ int floor_half(int v) { return v >= 0 ? v / 2 : -((1 - v) / 2); }

// A slab level's window in shared memory (P, R: float; K, F: byte arrays of
// `total` cells each, like the coarse levels') and its staging area.
struct Win {
  SlabLv L;
  int par;
  float* P;
  float* R;
  uint8_t* K;
  uint8_t* F;
  float* S;
  __device__ __forceinline__ Win(const SlabLv& l, int par_, unsigned char* smem, int total) : L(l), par(par_) {
    float* base = reinterpret_cast<float*>(smem);
    P = base + l.off;
    R = base + total + l.off;
    uint8_t* bytes = reinterpret_cast<uint8_t*>(base + 2 * total);  // K and F arrays, then the staging floats
    K = bytes + l.off;
    F = K + total;
    S = reinterpret_cast<float*>(bytes + 2 * total) + l.so;
  }
  // window row wy, padded column i (level column i - 1)
  __device__ __forceinline__ int at(int wy, int i) const { return ((i + wy + par) & 1) * L.pl + wy * L.qs + (i >> 1); }
};

__device__ __forceinline__ void win_codes(const Win& W) {
  const SlabLv& L = W.L;
  for (int e = threadIdx.x; e < L.wr * L.nx; e += COARSE_THREADS) {
    const int wy = e / L.nx, i = e - wy * L.nx + 1;
    const int a = W.at(wy, i);
    uint8_t k = 0;
    if (wy > 0 && wy < L.wr - 1 && W.F[a]) {
      const int o = i & 1, b = a + (((i + wy + W.par) & 1) ? -L.pl : L.pl);
      k = (uint8_t)(1 + W.F[b - 1 + o] + W.F[b + o] + W.F[b - L.qs] + W.F[b + L.qs]);
    }
    W.K[a] = k;
  }
}

// One colour of a red-black sweep over window rows lo..hi (multigrid.wgsl:60-77).
__device__ __forceinline__ void win_sweep(const Win& W, int lo, int hi, int c) {
  const SlabLv& L = W.L;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float* Pc = W.P + c * L.pl;
  const float* Po = W.P + (c ^ 1) * L.pl;
  const float* Rc = W.R + c * L.pl;
  const uint8_t* Kc = W.K + c * L.pl;
  for (int j = lo + warp; j <= hi; j += COARSE_THREADS / 32) {
    const int o = (c + j + W.par) & 1;  // padded column parity of colour c in window row j
    for (int q = lane + 1 - o; 2 * q + o <= L.nx; q += 32) {
      const int a = j * L.qs + q;
      const uint8_t kk = Kc[a];
      if (!kk) continue;
      float sum = 0.0f;
      sum += Po[a - 1 + o];
      sum += Po[a + o];
      sum += Po[a - L.qs];
      sum += Po[a + L.qs];
      Pc[a] = (sum - Rc[a]) / ((float)(kk - 1) + L.eps);
    }
  }
  __syncthreads();
}

// Residual of window cell (wy, i) if it is updated (multigrid.wgsl:82-105).
__device__ __forceinline__ bool win_residual(const Win& W, int wy, int i, float& res) {
  const SlabLv& L = W.L;
  const int a = W.at(wy, i);
  const uint8_t kk = W.K[a];
  if (!kk) return false;
  const int o = i & 1, b = a + (((i + wy + W.par) & 1) ? -L.pl : L.pl);
  float s = 0.0f;
  s += W.P[b - 1 + o];
  s += W.P[b + o];
  s += W.P[b - L.qs];
  s += W.P[b + L.qs];
  res = W.R[a] - (s - ((float)(kk - 1) + L.eps) * W.P[a]);
  return true;
}

// Pushes this CTA's owned rows of `a1` (and of `a2`, an array of the same
// layout, when given: window arrays of floats or bytes, both colour planes)
// into the windows of the other CTAs that hold them as ghost rows.  Each
// thread takes an owned element and stores it to those CTAs: CTA rr's window
// holds rows [rr R - G, rr R + R + G).
template <class T1, class T2>
__device__ __forceinline__ void win_push_owned(const Win& W, T1* a1, T2* a2, int G, int nc, uint32_t rank,
                                               uint32_t* status) {
  const SlabLv& L = W.L;
  const int r0 = (int)rank * L.R;
  const int y1 = r0 + L.R < L.ny ? r0 + L.R : L.ny;
  const int n = (y1 - r0) * 2 * L.qs;
  for (int e = threadIdx.x; e < n; e += COARSE_THREADS) {
    const int q = e % L.qs, t = e / L.qs, plane = t & 1, y = r0 + (t >> 1);
    const int a = plane * L.pl + (y - r0 + G) * L.qs + q;
    const T1 v1 = a1[a];
    const T2 v2 = a2 ? a2[a] : T2(0);
    int rlo = y - G - L.R + 1;
    rlo = rlo <= 0 ? 0 : (rlo + L.R - 1) / L.R;
    int rhi = (y + G) / L.R;
    if (rhi > nc - 1) rhi = nc - 1;
    for (int rr = rlo; rr <= rhi; rr++) {
      if (rr == (int)rank) continue;
      const int d = a + (r0 - rr * L.R) * L.qs;
      if (!RB_IN(d, 2 * L.pl, status)) continue;
      *cta_map(a1 + d, (uint32_t)rr) = v1;
      if (a2) *cta_map(a2 + d, (uint32_t)rr) = v2;
    }
  }
}

// Pushes rows [c0, c1) of a coarse level's p (read by `get(cy, cx)`) into the
// staging areas of slab level W (the next finer one) of the CTAs whose
// windows prolong from them: CTA rr's window rows [rr R - G, rr R + R + G)
// read coarse rows floor(y / 2), staged from row floor((rr R - G) / 2) on.
template <class Get>
__device__ __forceinline__ void stage_push(const Win& W, int c0, int c1, int G, int nc, uint32_t* status, Get&& get) {
  const SlabLv& L = W.L;
  const int n = (c1 - c0) * L.cnx;
  for (int e = threadIdx.x; e < n; e += COARSE_THREADS) {
    const int cy = c0 + e / L.cnx, cx = e % L.cnx;
    const float v = get(cy, cx);
    int rlo = 2 * cy - L.R - G + 1;
    rlo = rlo <= 0 ? 0 : (rlo + L.R - 1) / L.R;
    int rhi = (2 * cy + 1 + G) / L.R;
    if (rhi > nc - 1) rhi = nc - 1;
    for (int rr = rlo; rr <= rhi; rr++) {
      const int row = cy - floor_half(rr * L.R - G);
      if (row < 0 || row >= L.srows) continue;
      const int si = row * L.cnx + cx;
      if (RB_IN(si, L.srows * L.cnx, status)) *cta_map(W.S + si, (uint32_t)rr) = v;
    }
  }
}

__global__ void __launch_bounds__(COARSE_THREADS, 1)
    k_mg_cluster(const __grid_constant__ ClusterPass cp, int nu_pre, int nu_post, int coarse) {
  extern __shared__ __align__(16) unsigned char smem[];
  const uint32_t rank = cluster_rank();
  const CoarsePass& e = cp.co;
  const CoarseSet& cs = e.cs;
  const int total = cs.total, G = cp.G, nc = cp.nc;
  // every cell starts as non-water, p = rhs = 0 (rings, rows outside the level)
  {
    float4* f = reinterpret_cast<float4*>(smem);
    const int n16 = (10 * total + 15) / 16;
    for (int i = threadIdx.x; i < n16; i += COARSE_THREADS) f[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  }
  __syncthreads();
  cluster_arrive();  // every CTA has started and cleared its memory (waited for before the first remote access)
  // the top slab level: the whole window from global memory
  {
    const Win W(cp.w[0], cp.par, smem, total);
    const SlabLv& L = W.L;
    const int r0 = (int)rank * L.R, n = L.wr * L.nx;
    const bool TOP = e.top != 0;
    constexpr int BATCH = 4;
    for (int e0 = threadIdx.x; e0 < n; e0 += BATCH * COARSE_THREADS) {
      uint8_t f[BATCH];
      float r[BATCH], p[BATCH];
#pragma unroll
      for (int u = 0; u < BATCH; u++) {  // a batch's loads are all issued before its stores
        const int el = e0 + u * COARSE_THREADS;
        const int wy = el / L.nx, x = el - wy * L.nx, y = r0 - G + wy;
        const bool in = el < n && y >= 0 && y < L.ny;
        const size_t gi = in ? (size_t)y * (TOP ? e.fw : L.nx) + x : 0;
        if (TOP) {
          f[u] = in && !e.mask[gi] ? 1 : 0;
          r[u] = e.div[gi];
          p[u] = e.pa[gi];
        } else {
          f[u] = in ? cp.fl_top[gi] : 0;
          r[u] = cp.rhs_top[gi];
          p[u] = 0.0f;
        }
      }
#pragma unroll
      for (int u = 0; u < BATCH; u++) {
        const int el = e0 + u * COARSE_THREADS;
        if (el >= n) continue;
        const int wy = el / L.nx, i = el - wy * L.nx + 1;
        const int a = W.at(wy, i);
        W.F[a] = f[u];
        W.P[a] = f[u] ? p[u] : 0.0f;
        W.R[a] = f[u] ? r[u] : 0.0f;
      }
    }
    __syncthreads();
  }
  // pre-smooth, residual and restriction down the slab levels
  for (int s = 0; s < cp.nslab; s++) {
    const Win W(cp.w[s], cp.par, smem, total);
    const SlabLv& L = W.L;
    const int r0 = (int)rank * L.R;
    win_codes(W);
    __syncthreads();
    const int lo = max(1, G - r0), hi = min(L.wr - 2, G - r0 + L.ny - 1);
    for (int k = 0; k < nu_pre; k++) {
      win_sweep(W, lo, hi, 0);
      win_sweep(W, lo, hi, 1);
    }
    // restriction of the owned rows into the next slab level's owned rows
    // (local, then pushed to the windows that hold them as ghost rows) or
    // into CTA 0's coarsest level (remote)
    const bool last = s + 1 == cp.nslab;
    const CLv T = coarse_level(cs, smem, 0);
    const int cnx = last ? cs.nx[0] : cp.w[s + 1].nx, cny = last ? cs.ny[0] : cp.w[s + 1].ny, cR = L.R / 2;
    const Win C(cp.w[last ? s : s + 1], cp.par, smem, total);
    float* tP = cta_map(T.P, 0u);
    float* tR = cta_map(T.R, 0u);
    uint8_t* tF = cta_map(T.F, 0u);
    if (s == 0) cluster_wait();
    const int c0 = (int)rank * cR;
    for (int ce = threadIdx.x; ce < cR * cnx; ce += COARSE_THREADS) {
      const int cyl = ce / cnx, cx = ce - cyl * cnx, cy = c0 + cyl;
      if (cy >= cny) continue;
      float sum = 0.0f;
      uint32_t nf = 0;
      for (uint32_t q = 0; q < 4; q++) {
        float res;
        const int fy = cy * 2 + (int)(q >> 1), fx = cx * 2 + (int)(q & 1u);
        if (!win_residual(W, fy - r0 + G, fx + 1, res)) continue;
        sum += res;
        nf++;
      }
      const uint8_t fl = nf > 0u ? 1 : 0;
      const float rh = nf > 0u ? 2.0f * sum / (float)(nf > 1u ? nf : 1u) : 0.0f;
      if (last) {
        const int a = T.at(cy, cx);
        tF[a] = fl;
        tR[a] = rh;
        tP[a] = 0.0f;
      } else {
        const int a = C.at(cyl + G, cx + 1);
        C.F[a] = fl;
        C.R[a] = rh;
      }
    }
    if (!last) {
      __syncthreads();
      win_push_owned(C, C.R, C.F, G, nc, rank, cp.status);
    }
    cluster_sync();  // the next level's windows (or the coarsest level) are complete everywhere
  }
  // every CTA's windows are pre-smoothed: push the owned p to the windows
  // that hold it as ghost rows (nobody writes a window's p until the next
  // barrier); CTA 0 solves the coarsest level and stages it for the
  // coarsest slab level
  for (int s = 0; s < cp.nslab; s++) {
    const Win W(cp.w[s], cp.par, smem, total);
    win_push_owned(W, W.P, (uint8_t*)nullptr, G, nc, rank, cp.status);
  }
  if (rank == 0) {
    const CLv T = coarse_level(cs, smem, 0);
    coarse_codes(T);
    __syncthreads();
    coarse_cycle<false>(e, smem, nu_pre, nu_post, coarse);
    const Win W(cp.w[cp.nslab - 1], cp.par, smem, total);
    stage_push(W, 0, T.ny, G, nc, cp.status, [&](int cy, int cx) { return T.P[T.at(cy, cx)]; });
  }
  cluster_sync();  // ghost p and the coarse correction have arrived
  // prolongation (from the staged coarse rows) and post-smooth up the slab levels
  for (int s = cp.nslab - 1; s >= 0; s--) {
    const Win W(cp.w[s], cp.par, smem, total);
    const SlabLv& L = W.L;
    const int r0 = (int)rank * L.R, sb = floor_half(r0 - G);
    for (int el = threadIdx.x; el < L.wr * L.nx; el += COARSE_THREADS) {
      const int wy = el / L.nx, x = el - wy * L.nx, y = r0 - G + wy;
      if (y < 0 || y >= L.ny) continue;
      const int a = W.at(wy, x + 1);
      if (!W.F[a]) continue;
      const int si = (floor_half(y) - sb) * L.cnx + x / 2;
      if (RB_IN(si, L.srows * L.cnx, cp.status)) W.P[a] += W.S[si];
    }
    __syncthreads();
    const int lo = max(1, G - r0), hi = min(L.wr - 2, G - r0 + L.ny - 1);
    for (int k = 0; k < nu_post; k++) {
      win_sweep(W, lo, hi, 0);
      win_sweep(W, lo, hi, 1);
    }
    if (s > 0) {
      // the owned rows are final: stage them for the next finer level
      const Win F(cp.w[s - 1], cp.par, smem, total);
      int c1 = r0 + L.R;
      if (c1 > L.ny) c1 = L.ny;
      stage_push(F, r0, c1, G, nc, cp.status, [&](int cy, int cx) { return W.P[W.at(cy - r0 + G, cx + 1)]; });
      cluster_sync();
    }
  }
  // the top slab level's owned rows leave for the next finer level (or pressure_a)
  {
    const Win W(cp.w[0], cp.par, smem, total);
    const SlabLv& L = W.L;
    const int r0 = (int)rank * L.R;
    const bool TOP = e.top != 0;
    for (int el = threadIdx.x; el < L.R * L.nx; el += COARSE_THREADS) {
      const int yl = el / L.nx, x = el - yl * L.nx, y = r0 + yl;
      if (y >= L.ny) continue;
      const float v = W.P[W.at(yl + G, x + 1)];
      if (TOP) e.pa[(size_t)y * e.fw + x] = v;
      else cp.p_out[(size_t)y * L.nx + x] = v;
    }
  }
}

// The mixed-precision preconditioner's coarse V-cycle with its exact FP64
// coarsest solve spread over a thread-block cluster: CTA 0 runs the levels
// (down, then up, as k_mg_coarse does); for the solve every CTA takes a share
// of the rows of the dense inverse, multiplies them with the coarsest
// right-hand side (copied from CTA 0 through distributed shared memory) in
// the same order as one CTA would, and stores its part of the solution into
// CTA 0's plane.  The FP64 products and the inverse's loads then run on NC
// SMs instead of one.
__global__ void __launch_bounds__(COARSE_THREADS, 1)
    k_mp_coarse_cluster(const __grid_constant__ CoarseOne s, int nu_pre, int nu_post) {
  const CoarsePass& e = s.e;
  const CoarseSet& cs = e.cs;
  extern __shared__ __align__(16) unsigned char smem[];
  const uint32_t rank = cluster_rank(), ncta = cluster_size();
  const CLv L = coarse_level(cs, smem, cs.n - 1);
  const int nc = L.nx * L.ny;
  float* rn = reinterpret_cast<float*>(smem + (size_t)10 * cs.total);
  if (rank == 0) {
    coarse_load_top(e, smem);
    coarse_down<true>(e, smem, nu_pre);
    for (int i = threadIdx.x; i < nc; i += COARSE_THREADS) rn[i] = L.R[L.at(i / L.nx, i % L.nx)];
  }
  cluster_sync();  // the coarsest right-hand side is ready (and every CTA has started)
  if (rank != 0) {
    const float* r0 = cta_map(rn, 0u);
    for (int i = threadIdx.x; i < nc; i += COARSE_THREADS) rn[i] = r0[i];
    __syncthreads();
  }
  const int per = (nc + (int)ncta - 1) / (int)ncta;
  const int i0 = min(nc, (int)rank * per), i1 = min(nc, i0 + per);
  coarsest_dense_rows(e, L, rn, cta_map(L.P, 0u), i0, i1);
  cluster_sync();  // the solution is complete in CTA 0; no CTA reads another after this
  if (rank == 0) {
    coarse_up<true>(e, smem, nu_post);
    coarse_store_top(e, smem);
  }
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

void launch_mg_codes(const MgLevel* levels, int nl, const MgBufs& b, cudaStream_t s) {
  if (!b.code) return;
  const dim3 blk(BX, BY);
  for (int l = 0; l < nl; l++) {
    const Lv L = lv(levels[l], b);
    const bool down = l + 1 < nl;
    uint8_t* cfl = down ? b.fluid + levels[l + 1].off : nullptr;
    const int cnx = down ? levels[l + 1].nx : 0, cny = down ? levels[l + 1].ny : 0;
    RB_LAUNCH("mg_codes", 2.0 * cells(L), s,
              k_mg_codes<<<grid2(L.nx, L.ny), blk, 0, s>>>(L, b.code + levels[l].off, cfl, cnx, cny));
  }
}

void launch_jacobi(const Dev& d, int iters, cudaStream_t s) {
  const dim3 blk(BX, BY);
  double b = 13.0 * (double)d.fw * d.fh;
  for (int k = 0; k < iters; k++) {
    if (k % 2 == 0) RB_LAUNCH("jacobi_pressure", b, s, k_jacobi<<<grid2(d.fw, d.fh), blk, 0, s>>>(d, d.pa, d.pb));
    else RB_LAUNCH("jacobi_pressure", b, s, k_jacobi<<<grid2(d.fw, d.fh), blk, 0, s>>>(d, d.pb, d.pa));
  }
}

static const char* const PRE_NAMES[8] = {"mg_pre_restrict_L0", "mg_pre_restrict_L1", "mg_pre_restrict_L2",
                                         "mg_pre_restrict_L3", "mg_pre_restrict_L4", "mg_pre_restrict_L5",
                                         "mg_pre_restrict_L6", "mg_pre_restrict_L7+"};
static const char* const POST_NAMES[8] = {"mg_prolong_post_L0", "mg_prolong_post_L1", "mg_prolong_post_L2",
                                          "mg_prolong_post_L3", "mg_prolong_post_L4", "mg_prolong_post_L5",
                                          "mg_prolong_post_L6", "mg_prolong_post_L7+"};

// Box of a fine level: the 66 x 50 box where it gives at least three tiles
// per SM of the device, the 34 x 34 box on the smaller levels, whose kernels are
// bound by the latency of one tile rather than by bandwidth (measured on the
// 2048^2 levels: 1024^2 is faster with the big box, 512^2 with the small).
static bool small_tiles(const MgLevel& L, const MgConfig& c) {
  const int H = 2 * c.pre + 1, tw = BoxBig::tile_w(H), th = BoxBig::tile_h(H);
  const long big = (long)((L.nx + tw - 1) / tw) * ((L.ny + th - 1) / th);
  return big < 3l * device_sm_count();
}

// Tiles of a fine level's pre (halo 2 pre + 1) or post (halo 2 post) pass.
struct TileGrid {
  int nbx, nby;
};
template <class B>
static TileGrid tile_grid(const MgLevel& L, int H) {
  const int tw = B::tile_w(H), th = B::tile_h(H);
  return TileGrid{(L.nx + tw - 1) / tw, (L.ny + th - 1) / th};
}
static TileGrid tile_grid(const MgLevel& L, bool small, int H) {
  return small ? tile_grid<BoxSmall>(L, H) : tile_grid<BoxBig>(L, H);
}

int multigrid_first_coarse_level(const MgLevel* levels, int nl) {
  int k = 0;
  while (k < nl && (size_t)levels[k].nx * levels[k].ny > (size_t)MG_SMEM_CELLS) k++;
  return k;
}

// Shared memory of the coarse kernel: the padded colour planes of every
// coarse level (p, rhs: 4 bytes; codes, flags: 1 byte) and a row-major copy
// of the coarsest rhs for the FP64 dense solve.
static size_t coarse_smem_bytes(const MgLevel* levels, int nl) {
  const int k = multigrid_first_coarse_level(levels, nl);
  size_t cells = 0;
  for (int l = k; l < nl; l++) cells += (size_t)coarse_cells(levels[l].nx, levels[l].ny);
  return cells * 10 + (size_t)levels[nl - 1].nx * levels[nl - 1].ny * 4;
}
constexpr size_t COARSE_SMEM_MAX = 200 * 1024;

bool multigrid_fused_ok(const MgLevel* levels, int nl, const MgConfig& c) {
  if (c.pre < 1 || c.post < 1 || !BoxSmall::fits(2 * c.pre + 1) || !BoxSmall::fits(2 * c.post) || nl > 16) return false;
  return multigrid_first_coarse_level(levels, nl) < nl && coarse_smem_bytes(levels, nl) <= COARSE_SMEM_MAX;
}

static void set_smem_attrs() {
  static DeviceOnce attr;
  const int dev = DeviceOnce::device();
  if (!attr.pending(dev)) return;
  const int mx = (int)COARSE_SMEM_MAX;
  cudaFuncSetAttribute(k_mg_coarse<CoarseOne>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  cudaFuncSetAttribute(k_mg_coarse<CoarseMany>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  cudaFuncSetAttribute(k_mg_coarse<CoarseOne, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  attr.done(dev);
}

// The pre- and post-smooth passes of fine level l.  Level 0 reads
// pressure_a (masked) and the divergence directly and its post pass writes
// pressure_a; the pre-smoothed p goes to p_tmp (level 0) or p2.
static MgPass pre_pass(const Dev& d, const MgLevel* levels, int l, const MgBufs& b) {
  const Lv L = lv(levels[l], b), C = lv(levels[l + 1], b);
  return MgPass{L, C, l == 0 ? d.pa : nullptr, l == 0 ? d.div : L.rhs, L.fl, l == 0 ? b.p_tmp : b.p2 + levels[l].off,
                b.code ? b.code + levels[l].off : nullptr};
}
static MgPass post_pass(const Dev& d, const MgLevel* levels, int l, const MgBufs& b) {
  const Lv L = lv(levels[l], b), C = lv(levels[l + 1], b);
  return MgPass{L, C, l == 0 ? b.p_tmp : b.p2 + levels[l].off, l == 0 ? d.div : L.rhs, L.fl, l == 0 ? d.pa : L.p,
                b.code ? b.code + levels[l].off : nullptr};
}
static double pre_bytes(const MgLevel* levels, int l) {
  return (l == 0 ? 13.0 : 9.0) * (double)levels[l].nx * levels[l].ny + 5.0 * (double)levels[l + 1].nx * levels[l + 1].ny;
}
static double post_bytes(const MgLevel* levels, int l) {
  return 13.0 * (double)levels[l].nx * levels[l].ny + 4.0 * (double)levels[l + 1].nx * levels[l + 1].ny;
}

// The coarse V-cycle of one world (levels from the first one that fits in
// shared memory down) and its shared-memory size.
static CoarsePass coarse_pass(const Dev& d, const MgLevel* levels, int nl, const MgBufs& b, size_t* smem, double* bytes) {
  const int k = multigrid_first_coarse_level(levels, nl);
  CoarsePass e{};
  CoarseSet& cs = e.cs;
  cs.n = nl - k;
  int off = 0;
  for (int l = k; l < nl; l++) {
    cs.nx[l - k] = levels[l].nx;
    cs.ny[l - k] = levels[l].ny;
    cs.eps[l - k] = levels[l].eps;
    cs.off[l - k] = off;
    off += coarse_cells(levels[l].nx, levels[l].ny);
  }
  cs.total = off;
  cs.rhs_top = b.rhs + levels[k].off;
  cs.fl_top = b.fluid + levels[k].off;
  cs.p_out = b.p + levels[k].off;
  e.mask = d.mask;
  e.div = d.div;
  e.pa = d.pa;
  e.fw = d.fw;
  e.top = k == 0 ? 1 : 0;
  *smem = coarse_smem_bytes(levels, nl);
  *bytes = 13.0 * levels[k].nx * levels[k].ny;
  return e;
}

template <class B>
static void launch_pre(const Dev& d, const MgLevel* levels, int l, const MgBufs& b, const MgConfig& c, cudaStream_t s) {
  const MgOne one{pre_pass(d, levels, l, b)};
  const TileGrid t = tile_grid<B>(levels[l], 2 * c.pre + 1);
  const dim3 grid(t.nbx, t.nby), blk(BX, BY);
  const char* name = PRE_NAMES[l < 7 ? l : 7];
  const double bytes = pre_bytes(levels, l);
  if (b.code) {
    if (l == 0) RB_LAUNCH(name, bytes, s, k_mg_pre<B, true, MgOne, true><<<grid, blk, B::SMEM_CODED, s>>>(one, c.pre));
    else RB_LAUNCH(name, bytes, s, k_mg_pre<B, false, MgOne, true><<<grid, blk, B::SMEM_CODED, s>>>(one, c.pre));
  } else {
    if (l == 0) RB_LAUNCH(name, bytes, s, k_mg_pre<B, true, MgOne, false><<<grid, blk, B::SMEM, s>>>(one, c.pre));
    else RB_LAUNCH(name, bytes, s, k_mg_pre<B, false, MgOne, false><<<grid, blk, B::SMEM, s>>>(one, c.pre));
  }
}

template <class B>
static void launch_post(const Dev& d, const MgLevel* levels, int l, const MgBufs& b, const MgConfig& c, cudaStream_t s) {
  const MgOne one{post_pass(d, levels, l, b)};
  const TileGrid t = tile_grid<B>(levels[l], 2 * c.post);
  const dim3 grid(t.nbx, t.nby), blk(BX, BY);
  const double bytes = post_bytes(levels, l);
  const char* name = POST_NAMES[l < 7 ? l : 7];
  if (b.code) RB_LAUNCH(name, bytes, s, k_mg_post<B, MgOne, true><<<grid, blk, B::SMEM_CODED, s>>>(one, c.post));
  else RB_LAUNCH(name, bytes, s, k_mg_post<B, MgOne, false><<<grid, blk, B::SMEM, s>>>(one, c.post));
}

// CTAs per cluster that k_mg_cluster can run with on this device at the
// largest opt-in shared memory (16, else 8; 0: no cluster launch).  Queried
// once per device outside stream capture; a call during capture before the
// first query answers 0 (the launch-per-level path, same results).
static int cluster_ctas(cudaStream_t s) {
  static std::atomic<int> cache[64];
  const int dev = DeviceOnce::device();
  const int v = cache[dev].load(std::memory_order_acquire);
  if (v != 0) return v < 0 ? 0 : v;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    return 0;
  }
  int smax = 0, found = -1;
  if (cudaDeviceGetAttribute(&smax, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) == cudaSuccess && smax > 0 &&
      cudaFuncSetAttribute(k_mg_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, smax) == cudaSuccess &&
      cudaFuncSetAttribute(k_mg_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
    for (int nc : {16, 8}) {
      cudaLaunchConfig_t cfg = {};
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = (unsigned)nc;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.gridDim = dim3((unsigned)nc);
      cfg.blockDim = dim3(COARSE_THREADS);
      cfg.dynamicSmemBytes = (size_t)smax;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int n = 0;
      if (cudaOccupancyMaxActiveClusters(&n, k_mg_cluster, &cfg) == cudaSuccess && n >= 1) {
        found = nc;
        break;
      }
    }
  }
  cudaGetLastError();
  cache[dev].store(found, std::memory_order_release);
  return found < 0 ? 0 : found;
}

static int smem_optin() {
  static std::atomic<int> cache[64];
  const int dev = DeviceOnce::device();
  int v = cache[dev].load(std::memory_order_relaxed);
  if (v <= 0) {
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess || v <= 0) {
      cudaGetLastError();
      return 0;
    }
    cache[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}

// The cluster V-cycle's arguments for a world: the coarsest level g and the
// slab levels m .. g - 1 above it with at most SLAB_MAX_CELLS owned cells per
// CTA, as far up as their windows fit in one CTA's shared memory.  False
// when no slab level qualifies.
static bool cluster_pass(const Dev& d, const MgLevel* levels, int nl, const MgBufs& b, const MgConfig& c, int nc,
                         size_t smax, ClusterPass* out, int* m_out, size_t* smem_out) {
  const int g = nl - 1;
  if (nc <= 0 || g < 1 || multigrid_first_coarse_level(levels, nl) >= nl) return false;
  const int G = 2 * (c.pre > c.post ? c.pre : c.post) + 1;
  const int Rk = (levels[g].ny + nc - 1) / nc;
  const size_t coarse = (size_t)coarse_cells(levels[g].nx, levels[g].ny);
  size_t win = 0, stage = 0;
  int m = g;
  while (m > 0 && g - (m - 1) <= MG_MAX_SLAB_LEVELS) {
    const MgLevel& L = levels[m - 1];
    const long R = (long)Rk << (g - (m - 1));
    if (R * L.nx > SLAB_MAX_CELLS) break;
    const size_t cells = (size_t)2 * (size_t)(R + 2 * G) * (size_t)coarse_qs(L.nx);
    const size_t st = (size_t)(R / 2 + G + 1) * (size_t)levels[m].nx;
    if (10 * (win + cells + coarse) + 4 * (stage + st) + 16 > smax) break;
    win += cells;
    stage += st;
    m--;
  }
  if (m == g) return false;
  ClusterPass& cp = *out;
  cp = ClusterPass{};
  cp.nslab = g - m;
  cp.G = G;
  cp.par = (G + 1) & 1;
  cp.nc = nc;
  int off = 0, so = 0;
  for (int l = m; l < g; l++) {
    SlabLv& w = cp.w[l - m];
    w.nx = levels[l].nx;
    w.ny = levels[l].ny;
    w.R = Rk << (g - l);
    w.wr = w.R + 2 * G;
    w.qs = coarse_qs(w.nx);
    w.pl = w.wr * w.qs;
    w.off = off;
    w.so = so;
    w.srows = w.R / 2 + G + 1;
    w.cnx = levels[l + 1].nx;
    w.eps = levels[l].eps;
    off += 2 * w.pl;
    so += w.srows * w.cnx;
  }
  CoarseSet& cs = cp.co.cs;
  cs.n = 1;
  cs.nx[0] = levels[g].nx;
  cs.ny[0] = levels[g].ny;
  cs.eps[0] = levels[g].eps;
  cs.off[0] = off;
  off += coarse_cells(levels[g].nx, levels[g].ny);
  cs.total = off;
  cp.co.mask = d.mask;
  cp.co.div = d.div;
  cp.co.pa = d.pa;
  cp.co.fw = d.fw;
  cp.co.top = m == 0 ? 1 : 0;
  cp.rhs_top = b.rhs + levels[m].off;
  cp.fl_top = b.fluid + levels[m].off;
  cp.p_out = b.p + levels[m].off;
  cp.status = d.status;
  *m_out = m;
  *smem_out = ((size_t)10 * off + (size_t)4 * so + 15) & ~(size_t)15;
  return true;
}

void launch_multigrid_fused(const Dev& d, const MgLevel* levels, int nl, const MgBufs& b, const MgConfig& c, cudaStream_t s) {
  set_smem_attrs();
  const int cycles = c.cycles < 1 ? 1 : c.cycles;
  {
    const int avail = cluster_ctas(s);
    const int nc = c.cluster == 0 ? avail : (c.cluster == 1 || c.cluster > avail ? 0 : c.cluster);
    ClusterPass cp;
    int m = 0;
    size_t smem = 0;
    if (cluster_pass(d, levels, nl, b, c, nc, (size_t)smem_optin(), &cp, &m, &smem)) {
      cudaLaunchConfig_t cfg = {};
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = (unsigned)nc;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.gridDim = dim3((unsigned)nc);
      cfg.blockDim = dim3(COARSE_THREADS);
      cfg.dynamicSmemBytes = smem;
      cfg.stream = s;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      const double bytes = (m == 0 ? 13.0 : 9.0) * (double)levels[m].nx * levels[m].ny;
      for (int cy = 0; cy < cycles; cy++) {
        for (int l = 0; l < m; l++) {
          if (small_tiles(levels[l], c)) launch_pre<BoxSmall>(d, levels, l, b, c, s);
          else launch_pre<BoxBig>(d, levels, l, b, c, s);
        }
        RB_LAUNCH("mg_cluster_vcycle", bytes, s, cudaLaunchKernelEx(&cfg, k_mg_cluster, cp, c.pre, c.post, c.coarse));
        for (int l = m - 1; l >= 0; l--) {
          if (small_tiles(levels[l], c)) launch_post<BoxSmall>(d, levels, l, b, c, s);
          else launch_post<BoxBig>(d, levels, l, b, c, s);
        }
      }
      return;
    }
  }
  const int k = multigrid_first_coarse_level(levels, nl);
  size_t coarse_smem = 0;
  double coarse_bytes = 0.0;
  const CoarseOne co{coarse_pass(d, levels, nl, b, &coarse_smem, &coarse_bytes)};
  for (int cy = 0; cy < cycles; cy++) {
    for (int l = 0; l < k; l++) {
      if (small_tiles(levels[l], c)) launch_pre<BoxSmall>(d, levels, l, b, c, s);
      else launch_pre<BoxBig>(d, levels, l, b, c, s);
    }
    RB_LAUNCH("mg_coarse_vcycle", coarse_bytes, s,
              k_mg_coarse<CoarseOne><<<1, COARSE_THREADS, coarse_smem, s>>>(co, c.pre, c.post, c.coarse));
    for (int l = k - 1; l >= 0; l--) {
      if (small_tiles(levels[l], c)) launch_post<BoxSmall>(d, levels, l, b, c, s);
      else launch_post<BoxBig>(d, levels, l, b, c, s);
    }
  }
}

// ---------------------------------------------------------------------------
// Batched V-cycles.  Worlds of different sizes have different numbers of
// fine levels; every launch covers one fine level index (and one tile
// shape) of the worlds that have it, in V order: pre-smooth level 0, 1, ...,
// the coarse solves (one CTA per world), post-smooth ..., 1, 0.  Each world
// sees its own kernels in its own order, so its results are the same bits
// as when it is stepped alone.

struct MgBatchPlan {
  // One fine level index and box shape over the worlds that have it; the
  // pre and post passes tile the level differently (their halos differ).
  struct Group {
    int level;   // fine level index
    bool small;  // BoxSmall (else BoxBig)
    bool coded;  // every member loads precomputed neighbour codes (no flag array in the box)
    int n;
    const MgPass* pre;  // device [n]
    const MgPass* post;
    int total_pre, total_post;
    const int* start_pre;  // device [n + 1]: first CTA of each world
    const int* start_post;
    const int* nbx_pre;    // device [n]: tiles per row of each world
    const int* nbx_post;
    double bytes_pre, bytes_post;
  };
  MgConfig c{};
  std::vector<Group> groups;
  int levels = 0;
  int n = 0;
  const CoarsePass* coarse = nullptr;
  size_t coarse_smem = 0;
  double coarse_bytes = 0.0;
  void* blob = nullptr;
};

MgBatchPlan* multigrid_batch_plan(const MgWorld* ws, int n, const MgConfig& c, const int* tile_mode, int nmodes,
                                  cudaStream_t s) {
  MgBatchPlan* plan = new MgBatchPlan;
  plan->c = c;
  plan->n = n;
  std::vector<unsigned char> host;
  auto put = [&](const void* p, size_t bytes) {
    size_t off = (host.size() + 63) & ~(size_t)63;
    host.resize(off + bytes);
    if (bytes) memcpy(host.data() + off, p, bytes);
    return off;
  };
  struct Offs {
    size_t pre, post, start_pre, start_post, nbx_pre, nbx_post;
  };
  std::vector<Offs> offs;
  for (int w = 0; w < n; w++) {
    int k = multigrid_first_coarse_level(ws[w].levels, ws[w].nlevels);
    if (k > plan->levels) plan->levels = k;
  }
  for (int l = 0; l < plan->levels; l++) {
    for (int small = 0; small < 2; small++) {
      std::vector<MgPass> pre, post;
      std::vector<int> start_pre(1, 0), start_post(1, 0), nbx_pre, nbx_post;
      double bpre = 0.0, bpost = 0.0;
      bool coded = true;
      for (int w = 0; w < n; w++) {
        const MgWorld& W = ws[w];
        if (l >= multigrid_first_coarse_level(W.levels, W.nlevels)) continue;
        const int mode = l < nmodes ? tile_mode[l] : 0;
        const bool sm = mode == 1 ? false : (mode == 2 ? true : small_tiles(W.levels[l], c));
        if (sm != (small != 0)) continue;
        const TileGrid tp = tile_grid(W.levels[l], sm, 2 * c.pre + 1), tq = tile_grid(W.levels[l], sm, 2 * c.post);
        pre.push_back(pre_pass(W.d, W.levels, l, W.b));
        post.push_back(post_pass(W.d, W.levels, l, W.b));
        coded = coded && W.b.code != nullptr;
        nbx_pre.push_back(tp.nbx);
        nbx_post.push_back(tq.nbx);
        start_pre.push_back(start_pre.back() + tp.nbx * tp.nby);
        start_post.push_back(start_post.back() + tq.nbx * tq.nby);
        bpre += pre_bytes(W.levels, l);
        bpost += post_bytes(W.levels, l);
      }
      if (pre.empty()) continue;
      MgBatchPlan::Group g{};
      g.level = l;
      g.small = small != 0;
      g.coded = coded;
      g.n = (int)pre.size();
      g.total_pre = start_pre.back();
      g.total_post = start_post.back();
      g.bytes_pre = bpre;
      g.bytes_post = bpost;
      plan->groups.push_back(g);
      offs.push_back(Offs{put(pre.data(), pre.size() * sizeof(MgPass)), put(post.data(), post.size() * sizeof(MgPass)),
                          put(start_pre.data(), start_pre.size() * sizeof(int)),
                          put(start_post.data(), start_post.size() * sizeof(int)),
                          put(nbx_pre.data(), nbx_pre.size() * sizeof(int)),
                          put(nbx_post.data(), nbx_post.size() * sizeof(int))});
    }
  }
  std::vector<CoarsePass> co;
  for (int w = 0; w < n; w++) {
    size_t sm = 0;
    double by = 0.0;
    co.push_back(coarse_pass(ws[w].d, ws[w].levels, ws[w].nlevels, ws[w].b, &sm, &by));
    if (sm > plan->coarse_smem) plan->coarse_smem = sm;
    plan->coarse_bytes += by;
  }
  const size_t co_off = put(co.data(), co.size() * sizeof(CoarsePass));
  if (cudaMalloc(&plan->blob, host.size()) != cudaSuccess) {
    cudaGetLastError();
    delete plan;
    return nullptr;
  }
  if (cudaMemcpyAsync(plan->blob, host.data(), host.size(), cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(plan->blob);
    delete plan;
    return nullptr;
  }
  unsigned char* base = static_cast<unsigned char*>(plan->blob);
  for (size_t i = 0; i < plan->groups.size(); i++) {
    MgBatchPlan::Group& g = plan->groups[i];
    g.pre = reinterpret_cast<const MgPass*>(base + offs[i].pre);
    g.post = reinterpret_cast<const MgPass*>(base + offs[i].post);
    g.start_pre = reinterpret_cast<const int*>(base + offs[i].start_pre);
    g.start_post = reinterpret_cast<const int*>(base + offs[i].start_post);
    g.nbx_pre = reinterpret_cast<const int*>(base + offs[i].nbx_pre);
    g.nbx_post = reinterpret_cast<const int*>(base + offs[i].nbx_post);
  }
  plan->coarse = reinterpret_cast<const CoarsePass*>(base + co_off);
  return plan;
}

void multigrid_batch_free(MgBatchPlan* plan) {
  if (!plan) return;
  if (plan->blob) cudaFree(plan->blob);
  delete plan;
}

int multigrid_batch_levels(const MgBatchPlan* plan) { return plan ? plan->levels : 0; }

template <class B>
static void launch_group_pre_b(const MgBatchPlan::Group& g, const MgConfig& c, cudaStream_t s) {
  const MgSet set{g.pre, g.start_pre, g.nbx_pre, g.n};
  const char* name = PRE_NAMES[g.level < 7 ? g.level : 7];
  const dim3 blk(BX, BY);
  if (g.coded) {
    if (g.level == 0)
      RB_LAUNCH(name, g.bytes_pre, s, k_mg_pre<B, true, MgSet, true><<<g.total_pre, blk, B::SMEM_CODED, s>>>(set, c.pre));
    else
      RB_LAUNCH(name, g.bytes_pre, s, k_mg_pre<B, false, MgSet, true><<<g.total_pre, blk, B::SMEM_CODED, s>>>(set, c.pre));
  } else {
    if (g.level == 0)
      RB_LAUNCH(name, g.bytes_pre, s, k_mg_pre<B, true, MgSet, false><<<g.total_pre, blk, B::SMEM, s>>>(set, c.pre));
    else
      RB_LAUNCH(name, g.bytes_pre, s, k_mg_pre<B, false, MgSet, false><<<g.total_pre, blk, B::SMEM, s>>>(set, c.pre));
  }
}
static void launch_group_pre(const MgBatchPlan::Group& g, const MgConfig& c, cudaStream_t s) {
  if (g.small) launch_group_pre_b<BoxSmall>(g, c, s);
  else launch_group_pre_b<BoxBig>(g, c, s);
}

template <class B>
static void launch_group_post_b(const MgBatchPlan::Group& g, const MgConfig& c, cudaStream_t s) {
  const MgSet set{g.post, g.start_post, g.nbx_post, g.n};
  const char* name = POST_NAMES[g.level < 7 ? g.level : 7];
  if (g.coded)
    RB_LAUNCH(name, g.bytes_post, s, k_mg_post<B, MgSet, true><<<g.total_post, dim3(BX, BY), B::SMEM_CODED, s>>>(set, c.post));
  else
    RB_LAUNCH(name, g.bytes_post, s, k_mg_post<B, MgSet, false><<<g.total_post, dim3(BX, BY), B::SMEM, s>>>(set, c.post));
}
static void launch_group_post(const MgBatchPlan::Group& g, const MgConfig& c, cudaStream_t s) {
  if (g.small) launch_group_post_b<BoxSmall>(g, c, s);
  else launch_group_post_b<BoxBig>(g, c, s);
}

void launch_multigrid_batch(const MgBatchPlan* plan, cudaStream_t s) {
  set_smem_attrs();
  const MgConfig& c = plan->c;
  const int cycles = c.cycles < 1 ? 1 : c.cycles;
  for (int cy = 0; cy < cycles; cy++) {
    for (int l = 0; l < plan->levels; l++)
      for (const MgBatchPlan::Group& g : plan->groups)
        if (g.level == l) launch_group_pre(g, c, s);
    RB_LAUNCH("mg_coarse_vcycle", plan->coarse_bytes, s,
              k_mg_coarse<CoarseMany><<<plan->n, COARSE_THREADS, plan->coarse_smem, s>>>(CoarseMany{plan->coarse, plan->n},
                                                                                         c.pre, c.post, c.coarse));
    for (int l = plan->levels - 1; l >= 0; l--)
      for (const MgBatchPlan::Group& g : plan->groups)
        if (g.level == l) launch_group_post(g, c, s);
  }
}

void launch_multigrid_batch_pre(const MgBatchPlan* plan, int level, cudaStream_t s) {
  set_smem_attrs();
  for (const MgBatchPlan::Group& g : plan->groups)
    if (g.level == level) launch_group_pre(g, plan->c, s);
}

// ---------------------------------------------------------------------------
// Mixed-precision preconditioner V-cycle (the solver around it is in
// mixed.cu).
//
// It approximates L e = r for the scaled, component-mean-free residual r of
// the flexible CG.  A fine level keeps two arrays of type T (FP16 on the
// first levels, FP32 below): its right-hand side and its pre-smoothed
// correction e_f.  Post-smoothing adds the coarse level's total correction
// (FP32, times alpha) to e_f in shared memory and sweeps in FP32, so the
// large smooth part of a correction is never rounded to FP16; a level's
// total correction leaves as FP32 (levels >= 1) or, on level 0, as the
// unscaled output z with its per-component sums (FP64).  Restriction is
// 1/2 * sum over the water children (the transpose of the piecewise-constant
// prolongation up to the factor that keeps R L P the coarse operator), and
// post-smoothing runs the colours in reverse order, so the V-cycle is a
// symmetric operator.  Every level loads with plain loads.
namespace {

struct MpLevelArgs {
  int nx, ny;
  float eps;
  const uint8_t* code;  // neighbour codes of the level (0: not water)
  const void* rhs;    // right-hand side (type T); level 0: the CG residual (float)
  void* ef;           // pre-smoothed correction (type T)
  int cnx, cny;
  void* crhs;         // coarse right-hand side (pre output)
  const float* cE;    // coarse total correction (post input)
  float* E;           // total correction of the level (post output, levels >= 1)
  float alpha;
  // level 0
  const int* label;          // water component of each cell (-1: wall)
  const float* comp_mean;    // mean of the CG residual per component
  const float* scale;        // [0] scale applied to the residual, [1] its inverse
  float* z;                  // V-cycle output, unscaled
  double* comp_sum_z;        // per-component sums of z (cells outside a tile's dominant component)
  double* part_c;            // per tile: sum of z over the tile's dominant component
  int* part_dom;             // per tile: that component (-1: none)
};

__device__ __forceinline__ float mp_ld(const float* p, size_t i) { return p[i]; }
__device__ __forceinline__ float mp_ld(const __half* p, size_t i) { return __half2float(p[i]); }
__device__ __forceinline__ void mp_st(float* p, size_t i, float v) { p[i] = v; }
__device__ __forceinline__ void mp_st(__half* p, size_t i, float v) { p[i] = __float2half_rn(v); }

// The right-hand side of a level's cell: level 0 the CG residual minus its
// component's mean, times the FP16 scale; below, the stored restriction.
template <bool TOP, class T>
__device__ __forceinline__ float mp_rhs(const MpLevelArgs& a, size_t gi, float sc) {
  if (TOP) {
    const float rr = static_cast<const float*>(a.rhs)[gi];
    const int lab = a.label[gi];
    return (rr - a.comp_mean[lab < 0 ? 0 : lab]) * sc;
  }
  return mp_ld(static_cast<const T*>(a.rhs), gi);
}

// Pre-smooth from zero + residual + restriction (1/2 * sum over water children).
template <class B, bool TOP, class T, class CT>
__global__ void __launch_bounds__(BX* BY) k_mp_pre(const __grid_constant__ MpLevelArgs a, int nu) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int H = 2 * nu + 1, TW = B::tile_w(H), TH = B::tile_h(H);
  const int x0 = blockIdx.x * TW, y0 = blockIdx.y * TH;
  const RbSmem<B> Sm(smem_raw, (x0 + y0) & 1);
  const float sc = TOP ? a.scale[0] : 1.0f;
  rb_load<B, true>(Sm, x0 - H, y0 - H, a.nx, a.ny, [&](bool in, size_t gi, int, int, uint8_t& f, float& r, float& p) {
    f = in ? a.code[gi] : 0;
    r = mp_rhs<TOP, T>(a, gi, sc);
    p = 0.0f;
  });
  rb_sweeps<B>(2 * nu, 0, a.eps, Sm);
  T* ef = static_cast<T*>(a.ef);
  rb_store_tile<B>(Sm, H, x0, y0, a.nx, a.ny, [&](size_t i, float v) { mp_st(ef, i, v); });
  CT* crhs = static_cast<CT*>(a.crhs);
  for (int cj = threadIdx.y; cj < TH / 2; cj += BY)
    for (int ci = threadIdx.x; ci < TW / 2; ci += BX) {
      const int cgx = blockIdx.x * (TW / 2) + ci, cgy = blockIdx.y * (TH / 2) + cj;
      if (cgx >= a.cnx || cgy >= a.cny) continue;
      float sum = 0.0f;
      uint32_t nf = 0;
#pragma unroll
      for (uint32_t q = 0; q < 4; q++) {
        float res;
        if (!rb_residual<B>(Sm, H + 2 * cj + (int)(q >> 1), H + 2 * ci + (int)(q & 1u), a.eps, res)) continue;
        sum += res;
        nf++;
      }
      mp_st(crhs, (size_t)cgy * a.cnx + cgx, nf > 0u ? 0.5f * sum : 0.0f);
    }
}

// Prolong (alpha * coarse total) + post-smooth (colours reversed).
template <class B, bool TOP, class T>
__global__ void __launch_bounds__(BX* BY) k_mp_post(const __grid_constant__ MpLevelArgs a, int nu) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double zsh[BX * BY / 32];
  __shared__ int dom;
  const int H = 2 * nu, TW = B::tile_w(H), TH = B::tile_h(H);
  const int x0 = blockIdx.x * TW, y0 = blockIdx.y * TH;
  const RbSmem<B> Sm(smem_raw, (x0 + y0) & 1);
  const float sc = TOP ? a.scale[0] : 1.0f;
  rb_load<B, true>(Sm, x0 - H, y0 - H, a.nx, a.ny, [&](bool in, size_t gi, int gx, int gy, uint8_t& f, float& r, float& p) {
    f = in ? a.code[gi] : 0;
    r = mp_rhs<TOP, T>(a, gi, sc);
    const size_t ci = in ? (size_t)(gy / 2) * a.cnx + gx / 2 : 0;
    p = mp_ld(static_cast<const T*>(a.ef), gi) + a.alpha * a.cE[ci];
  });
  rb_sweeps<B>(2 * nu, 1, a.eps, Sm);
  if (!TOP) {
    float* E = a.E;
    rb_store_tile<B>(Sm, H, x0, y0, a.nx, a.ny, [&](size_t i, float v) { E[i] = v; });
    return;
  }
  // the tile's dominant component: that of its first water cell in row-major order
  const int tid = threadIdx.y * BX + threadIdx.x;
  if (tid == 0) dom = 0x7fffffff;
  __syncthreads();
  {
    int first = 0x7fffffff;
    for (int j = threadIdx.y; j < TH; j += BY)
      for (int i = threadIdx.x; i < TW; i += BX) {
        const int gx = x0 + i, gy = y0 + j;
        if (gx < a.nx && gy < a.ny && a.label[(size_t)gy * a.nx + gx] >= 0) first = min(first, j * TW + i);
      }
    for (int o = 16; o > 0; o >>= 1) first = min(first, __shfl_xor_sync(0xffffffffu, first, o));
    if ((tid & 31) == 0 && first != 0x7fffffff) atomicMin(&dom, first);
  }
  __syncthreads();
  if (tid == 0) dom = dom == 0x7fffffff ? -1 : a.label[(size_t)(y0 + dom / TW) * a.nx + x0 + dom % TW];
  __syncthreads();
  const float inv = a.scale[1];
  float own = 0.0f;
  for (int j = threadIdx.y; j < TH; j += BY)
    for (int i = threadIdx.x; i < TW; i += BX) {
      const int gx = x0 + i, gy = y0 + j;
      if (gx >= a.nx || gy >= a.ny) continue;
      const size_t gi = (size_t)gy * a.nx + gx;
      const int lab = a.label[gi];
      const float z = lab >= 0 ? Sm.P[Sm.at(H + j, H + i)] * inv : 0.0f;
      a.z[gi] = z;
      if (lab >= 0) {
        if (lab == dom) own += z;
        else atomicAdd(a.comp_sum_z + lab, (double)z);
      }
    }
  // the tile's partial for its dominant component (FP64 above the thread level)
  double t = (double)own;
  for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  if ((tid & 31) == 0) zsh[tid >> 5] = t;
  __syncthreads();
  if (tid == 0) {
    double s = 0.0;
    for (int w = 0; w < BX * BY / 32; w++) s += zsh[w];
    const unsigned b = blockIdx.y * gridDim.x + blockIdx.x;
    a.part_c[b] = s;
    a.part_dom[b] = dom;
  }
}

const char* const MP_PRE_NAMES[8] = {"mp_pre_L0", "mp_pre_L1", "mp_pre_L2", "mp_pre_L3",
                                     "mp_pre_L4", "mp_pre_L5", "mp_pre_L6", "mp_pre_L7+"};
const char* const MP_POST_NAMES[8] = {"mp_post_L0", "mp_post_L1", "mp_post_L2", "mp_post_L3",
                                      "mp_post_L4", "mp_post_L5", "mp_post_L6", "mp_post_L7+"};

// Algorithmic bytes: level 0 reads the CG residual (4), the component label
// (4) and the water flag (1); levels >= 1 their rhs (2 or 4) and flag; the
// correction is written (2 or 4), the coarse rhs written (a quarter size);
// post reads e_f, rhs, flag and a quarter-size coarse total and writes the
// total (z and its label read on level 0).
template <class B>
void mp_launch_pre(const MpLevelArgs& a, const MgLevel& L, int l, bool top, bool half, bool chalf, int nu, cudaStream_t s) {
  const TileGrid t = tile_grid<B>(L, 2 * nu + 1);
  const dim3 grid(t.nbx, t.nby), blk(BX, BY);
  const size_t sm = B::SMEM_CODED;
  const double es = half ? 2.0 : 4.0, n = (double)a.nx * a.ny;
  const double bytes = n * ((top ? 9.0 : es + 1.0) + es + (chalf ? 2.0 : 4.0) / 4.0);
  const char* name = MP_PRE_NAMES[l < 7 ? l : 7];
  if (top && half && chalf) RB_LAUNCH(name, bytes, s, k_mp_pre<B, true, __half, __half><<<grid, blk, sm, s>>>(a, nu));
  else if (top && half) RB_LAUNCH(name, bytes, s, k_mp_pre<B, true, __half, float><<<grid, blk, sm, s>>>(a, nu));
  else if (top) RB_LAUNCH(name, bytes, s, k_mp_pre<B, true, float, float><<<grid, blk, sm, s>>>(a, nu));
  else if (half && chalf) RB_LAUNCH(name, bytes, s, k_mp_pre<B, false, __half, __half><<<grid, blk, sm, s>>>(a, nu));
  else if (half) RB_LAUNCH(name, bytes, s, k_mp_pre<B, false, __half, float><<<grid, blk, sm, s>>>(a, nu));
  else RB_LAUNCH(name, bytes, s, k_mp_pre<B, false, float, float><<<grid, blk, sm, s>>>(a, nu));
}

template <class B>
void mp_launch_post(const MpLevelArgs& a, const MgLevel& L, int l, bool top, bool half, int nu, cudaStream_t s) {
  const TileGrid t = tile_grid<B>(L, 2 * nu);
  const dim3 grid(t.nbx, t.nby), blk(BX, BY);
  const size_t sm = B::SMEM_CODED;
  const double es = half ? 2.0 : 4.0, n = (double)a.nx * a.ny;
  const double bytes = n * (es + (top ? 9.0 : es + 1.0) + 1.0 + (top ? 8.0 : 4.0));
  const char* name = MP_POST_NAMES[l < 7 ? l : 7];
  if (top && half) RB_LAUNCH(name, bytes, s, k_mp_post<B, true, __half><<<grid, blk, sm, s>>>(a, nu));
  else if (top) RB_LAUNCH(name, bytes, s, k_mp_post<B, true, float><<<grid, blk, sm, s>>>(a, nu));
  else if (half) RB_LAUNCH(name, bytes, s, k_mp_post<B, false, __half><<<grid, blk, sm, s>>>(a, nu));
  else RB_LAUNCH(name, bytes, s, k_mp_post<B, false, float><<<grid, blk, sm, s>>>(a, nu));
}

}  // namespace

// CTAs per cluster for k_mp_coarse_cluster on this device (16, else 8; 0: one
// CTA), queried when a mixed-precision world is created (outside capture).
static std::atomic<int> g_mp_cluster[64];
void multigrid_prepare_mixed() {
  set_smem_attrs();
  const int dev = DeviceOnce::device();
  if (g_mp_cluster[dev].load(std::memory_order_acquire) != 0) return;
  int found = -1;
  if (cudaFuncSetAttribute(k_mp_coarse_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)COARSE_SMEM_MAX) ==
          cudaSuccess &&
      cudaFuncSetAttribute(k_mp_coarse_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
    for (int nc : {16, 8}) {
      cudaLaunchConfig_t cfg = {};
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = (unsigned)nc;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.gridDim = dim3((unsigned)nc);
      cfg.blockDim = dim3(COARSE_THREADS);
      cfg.dynamicSmemBytes = COARSE_SMEM_MAX;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int n = 0;
      if (cudaOccupancyMaxActiveClusters(&n, k_mp_coarse_cluster, &cfg) == cudaSuccess && n >= 1) {
        found = nc;
        break;
      }
    }
  }
  cudaGetLastError();
  g_mp_cluster[dev].store(found, std::memory_order_release);
}

size_t mixed_vcycle_tiles(const MgLevel* levels, int nl, const MgConfig& c) {
  (void)nl;
  const TileGrid t = tile_grid(levels[0], small_tiles(levels[0], c), 2 * c.post);
  return (size_t)t.nbx * t.nby;
}

int launch_mixed_vcycle(const Dev& d, const MgLevel* levels, int nl, const MgBufs& b, const MpHierarchy& h,
                        cudaStream_t s) {
  multigrid_prepare_mixed();
  const int k = multigrid_first_coarse_level(levels, nl);
  const MgConfig c{h.pre, h.post, 0, 1};
  auto args = [&](int l) {
    MpLevelArgs a{};
    a.nx = levels[l].nx;
    a.ny = levels[l].ny;
    a.eps = levels[l].eps;
    a.code = b.code + levels[l].off;
    a.rhs = l == 0 ? static_cast<const void*>(h.r) : h.fine[l].rhs;
    a.ef = h.fine[l].ef;
    a.cnx = levels[l + 1].nx;
    a.cny = levels[l + 1].ny;
    a.crhs = l + 1 < k ? h.fine[l + 1].rhs : static_cast<void*>(b.rhs + levels[k].off);
    a.cE = l + 1 < k ? h.fine[l + 1].E : b.p + levels[k].off;
    a.E = h.fine[l].E;
    a.alpha = h.alpha;
    a.label = h.label;
    a.comp_mean = h.comp_mean;
    a.scale = h.scale;
    a.z = h.z;
    a.comp_sum_z = h.comp_sum_z;
    a.part_c = h.part_c;
    a.part_dom = h.part_dom;
    return a;
  };
  for (int l = 0; l < k; l++) {
    const MpLevelArgs a = args(l);
    const bool half = l < h.nhalf, chalf = l + 1 < k && l + 1 < h.nhalf;
    if (small_tiles(levels[l], c)) mp_launch_pre<BoxSmall>(a, levels[l], l, l == 0, half, chalf, h.pre, s);
    else mp_launch_pre<BoxBig>(a, levels[l], l, l == 0, half, chalf, h.pre, s);
  }
  size_t coarse_smem = 0;
  double coarse_bytes = 0.0;
  CoarseOne co{coarse_pass(d, levels, nl, b, &coarse_smem, &coarse_bytes)};
  co.e.inv = h.coarse_inv;
  co.e.alpha = h.alpha;
  const int ncl = g_mp_cluster[DeviceOnce::device()].load(std::memory_order_acquire);
  if (ncl > 0) {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)ncl;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)ncl);
    cfg.blockDim = dim3(COARSE_THREADS);
    cfg.dynamicSmemBytes = coarse_smem;
    cfg.stream = s;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    RB_LAUNCH("mp_coarse_vcycle", coarse_bytes, s, cudaLaunchKernelEx(&cfg, k_mp_coarse_cluster, co, h.pre, h.post));
  } else {
    RB_LAUNCH("mp_coarse_vcycle", coarse_bytes, s,
              k_mg_coarse<CoarseOne, true><<<1, COARSE_THREADS, coarse_smem, s>>>(co, h.pre, h.post, 0));
  }
  for (int l = k - 1; l >= 0; l--) {
    const MpLevelArgs a = args(l);
    const bool half = l < h.nhalf;
    if (small_tiles(levels[l], c)) mp_launch_post<BoxSmall>(a, levels[l], l, l == 0, half, h.post, s);
    else mp_launch_post<BoxBig>(a, levels[l], l, l == 0, half, h.post, s);
  }
  return (int)mixed_vcycle_tiles(levels, nl, c);
}

}  // namespace ribo
