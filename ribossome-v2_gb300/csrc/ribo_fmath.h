// Pinned float semantics shared by the CUDA kernels and the CPU oracle.
//
// WGSL leaves the exact results of exp/pow/sin, of mix() and of fused
// multiply-adds to the backend, so the reference's own bits differ between
// wgpu backends.  This header fixes one definition of each of those
// operations.  Every function here is plain IEEE-754 single-precision
// arithmetic (no FMA contraction: kernels are compiled with -fmad=false and
// the oracle with -ffp-contract=off), so a CUDA kernel and the oracle that
// both call it produce identical bits on x86-64 and aarch64 hosts and on the
// GPU.
//
// Transcendentals follow published methods, written from the mathematics:
//  * exp:  Cody & Waite additive range reduction x = k*ln2 + r with ln2
//          split in a 16-bit head and a tail, then the degree-7 Taylor
//          polynomial of e^r on |r| <= ln2/2 in Horner form, then an exact
//          scale by 2^k built from the exponent bits.
//  * log:  x = m*2^e with m in [sqrt(1/2), sqrt(2)), then
//          log(m) = 2*atanh(s), s = (m-1)/(m+1), by its odd power series.
//  * sin:  Cody & Waite reduction by pi/2 split in three parts, then the
//          Taylor polynomials of sin and cos on |r| <= pi/4 and quadrant
//          selection.
// They are accurate to a few ulp over the ranges the world step uses (the
// CPU test suite bounds the error against double-precision libm).
#pragma once
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define RB_HD __host__ __device__ __forceinline__
#else
#define RB_HD static inline
#endif

RB_HD float rb_bits_to_f32(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}

RB_HD uint32_t rb_f32_to_bits(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
#endif
}

// Ordered comparisons, so that -0/+0 and NaN give the same bits everywhere
// (the hardware min/max instructions differ on signed zeros).
RB_HD float rb_min(float a, float b) { return (a < b) ? a : b; }
RB_HD float rb_max(float a, float b) { return (a > b) ? a : b; }
RB_HD float rb_clamp(float x, float lo, float hi) { return rb_min(rb_max(x, lo), hi); }
RB_HD float rb_abs(float x) { return rb_bits_to_f32(rb_f32_to_bits(x) & 0x7fffffffu); }

RB_HD float rb_floor(float x) {
#if defined(__CUDA_ARCH__)
  return floorf(x);
#else
  return __builtin_floorf(x);
#endif
}

// Round half to even (WGSL round()).
RB_HD float rb_rint(float x) {
#if defined(__CUDA_ARCH__)
  return rintf(x);
#else
  return __builtin_rintf(x);
#endif
}

RB_HD float rb_sqrt(float x) {
#if defined(__CUDA_ARCH__)
  return __fsqrt_rn(x);
#else
  return __builtin_sqrtf(x);
#endif
}

RB_HD float rb_fract(float x) { return x - rb_floor(x); }

// mix(a, b, t) = a*(1-t) + b*t, each product and sum rounded separately.
RB_HD float rb_mix(float a, float b, float t) { return a * (1.0f - t) + b * t; }

// smoothstep(0, 1, x) = t*t*(3 - 2t), t = clamp(x, 0, 1).
RB_HD float rb_smoothstep01(float x) {
  float t = rb_clamp(x, 0.0f, 1.0f);
  return t * t * (3.0f - 2.0f * t);
}

// Saturating float -> integer conversions (WGSL semantics: NaN -> 0,
// out-of-range values clamp to the nearest representable integer).  The
// GPU's conversion instructions saturate and map NaN to 0 by definition,
// so device code uses them directly; host code spells the same rule out.
RB_HD int32_t rb_f2i(float x) {
#if defined(__CUDA_ARCH__)
  return __float2int_rz(x);
#else
  if (!(x == x)) return 0;
  if (x >= 2147483648.0f) return 2147483647;
  if (x <= -2147483648.0f) return (int32_t)0x80000000u;
  return (int32_t)x;
#endif
}

RB_HD uint32_t rb_f2u(float x) {
#if defined(__CUDA_ARCH__)
  return __float2uint_rz(x);
#else
  if (!(x > 0.0f)) return 0u;  // negatives, -0 and NaN
  if (x >= 4294967296.0f) return 0xffffffffu;
  return (uint32_t)x;
#endif
}

// i32(floor(x)) with the saturating conversion above (one rounding-mode
// conversion instruction on the GPU).
RB_HD int32_t rb_floor_i(float x) {
#if defined(__CUDA_ARCH__)
  return __float2int_rd(x);
#else
  return rb_f2i(rb_floor(x));
#endif
}

// 2^k * p for k in [-252, 254] with at most one rounding.
RB_HD float rb_scale2(float p, int k) {
  if (k > 127) {
    p = p * rb_bits_to_f32(0x7f000000u);  // 2^127
    k -= 127;
    if (k > 127) k = 127;
  } else if (k < -126) {
    p = p * rb_bits_to_f32(0x00800000u);  // 2^-126
    k += 126;
    if (k < -126) k = -126;
  }
  return p * rb_bits_to_f32((uint32_t)(k + 127) << 23);
}

#define RB_LN2_HI 0.693145751953125f        // 0x3f317200: 16 significant bits
#define RB_LN2_LO 1.428606765330187e-06f    // ln2 - RB_LN2_HI
#define RB_LOG2E 1.4426950216293335f

RB_HD float rb_exp(float x) {
  if (!(x == x)) return x;
  if (x > 88.72283935546875f) return rb_bits_to_f32(0x7f800000u);
  if (x < -103.97208404541016f) return 0.0f;
  float kf = rb_rint(x * RB_LOG2E);
  float r = (x - kf * RB_LN2_HI) - kf * RB_LN2_LO;
  // e^r = 1 + r + r^2/2! + ... + r^7/7!
  float p = 1.0f / 5040.0f;
  p = p * r + 1.0f / 720.0f;
  p = p * r + 1.0f / 120.0f;
  p = p * r + 1.0f / 24.0f;
  p = p * r + 1.0f / 6.0f;
  p = p * r + 0.5f;
  p = p * r + 1.0f;
  p = p * r + 1.0f;
  return rb_scale2(p, (int)kf);
}

// Natural logarithm for x > 0 (0 -> -inf, negative/NaN -> NaN).
RB_HD float rb_log(float x) {
  if (!(x > 0.0f)) return (x == 0.0f) ? rb_bits_to_f32(0xff800000u) : rb_bits_to_f32(0x7fc00000u);
  if (x == rb_bits_to_f32(0x7f800000u)) return x;
  int e = 0;
  if (x < 1.17549435e-38f) {  // subnormal: normalise first
    x = x * 16777216.0f;
    e = -24;
  }
  uint32_t u = rb_f32_to_bits(x);
  e += (int)((u >> 23) & 0xffu) - 127;
  float m = rb_bits_to_f32((u & 0x007fffffu) | 0x3f800000u);  // [1, 2)
  if (m > 1.41421353816986083984375f) {
    m = m * 0.5f;
    e += 1;
  }
  float s = (m - 1.0f) / (m + 1.0f);
  float s2 = s * s;
  // atanh(s) = s + s^3/3 + s^5/5 + s^7/7 + s^9/9 + s^11/11
  float q = 1.0f / 11.0f;
  q = q * s2 + 1.0f / 9.0f;
  q = q * s2 + 1.0f / 7.0f;
  q = q * s2 + 1.0f / 5.0f;
  q = q * s2 + 1.0f / 3.0f;
  float lm = 2.0f * s + 2.0f * s * s2 * q;
  float ef = (float)e;
  return (ef * RB_LN2_HI + lm) + ef * RB_LN2_LO;
}

// pow(x, y) for x >= 0, as exp(y * ln x).
RB_HD float rb_pow(float x, float y) {
  if (y == 0.0f) return 1.0f;
  if (x == 1.0f) return 1.0f;
  if (x == 0.0f) return (y > 0.0f) ? 0.0f : rb_bits_to_f32(0x7f800000u);
  if (!(x > 0.0f)) return rb_bits_to_f32(0x7fc00000u);
  return rb_exp(y * rb_log(x));
}

#define RB_PIO2_1 1.5703125f
#define RB_PIO2_2 0.0004837512969970703f
#define RB_PIO2_3 7.549790126404332e-08f
#define RB_2OPI 0.6366197466850281f

// sin(x) for |x| < 2^15 (the world step calls it with |x| < 20).
RB_HD float rb_sin(float x) {
  if (!(x == x)) return x;
  float kf = rb_rint(x * RB_2OPI);
  float r = ((x - kf * RB_PIO2_1) - kf * RB_PIO2_2) - kf * RB_PIO2_3;
  int q = ((int)kf) & 3;
  float r2 = r * r;
  // sin r = r - r^3/3! + r^5/5! - r^7/7! + r^9/9!
  float ps = 1.0f / 362880.0f;
  ps = ps * r2 - 1.0f / 5040.0f;
  ps = ps * r2 + 1.0f / 120.0f;
  ps = ps * r2 - 1.0f / 6.0f;
  float sn = r + r * r2 * ps;
  // cos r = 1 - r^2/2! + r^4/4! - r^6/6! + r^8/8! - r^10/10!
  float pc = -1.0f / 3628800.0f;
  pc = pc * r2 + 1.0f / 40320.0f;
  pc = pc * r2 - 1.0f / 720.0f;
  pc = pc * r2 + 1.0f / 24.0f;
  pc = pc * r2 - 0.5f;
  float cs = 1.0f + r2 * pc;
  float v = (q & 1) ? cs : sn;
  return (q & 2) ? -v : v;
}

// ---------------------------------------------------------------------------
// Counter-based RNG: PCG4D hash (Jarzynski & Olano, "Hash Functions for GPU
// Rendering", JCGT 2020), keyed by (key, epoch, stream, seed).
typedef struct {
  uint32_t x, y, z, w;
} rb_u4;

RB_HD rb_u4 rb_pcg4d(uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  uint32_t x = a * 1664525u + 1013904223u;
  uint32_t y = b * 1664525u + 1013904223u;
  uint32_t z = c * 1664525u + 1013904223u;
  uint32_t w = d * 1664525u + 1013904223u;
  x += y * w;
  y += z * x;
  z += x * y;
  w += y * z;
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

// 24-bit uniform float in [0, 1) from a 32-bit word.
RB_HD float rb_u2f(uint32_t u) { return (float)(u >> 8) * (1.0f / 16777216.0f); }

// RNG stream bases (sub-indices are added to them; blocks of 2^16 do not overlap).
#define RB_S_PHOTO 1u
#define RB_S_DECAY 2u
#define RB_S_THERMAL 3u
#define RB_S_BUOYANCY 4u
#define RB_S_RELAX 16u  // + relax phase (0, 1)
#define RB_S_SAND 32u   // + relax phase (0, 1)
#define RB_S_MOVE (1u << 16)
#define RB_S_DISPERSE (6u << 16)

// Integer mixer of tie-breaks (not a random stream): shift-xor-multiply with
// the "lowbias32" constants of C. Wellons' hash-prospector, as the
// reference's hash() (shaders/common/rng.wgsl:46-50).
RB_HD uint32_t rb_hash32(uint32_t v) {
  uint32_t x = v;
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}
