// om_math.h -- oracle definition of the WGSL built-ins used by Pike's passes.
//
// TEST INFRASTRUCTURE ONLY.  This header belongs to the CPU oracle: only the
// tests, the smoke check and bench.py's CPU-baseline leg may use it.
//
// The reference runs its shaders on whatever WebGPU implementation the
// browser ships; WGSL leaves sin/cos/atan2/acos/pow/exp2/log2 accuracy,
// dot-product summation order and FMA contraction to the implementation, so
// its outputs are not pinned by any test of the reference (it has none).
// This file *defines* those built-ins for parity purposes:
//   * IEEE-754 binary32 arithmetic, round-to-nearest-even, no FMA contraction
//     (compile with -ffp-contract=off), correctly rounded division and sqrt,
//     denormals preserved;
//   * dot/cross/mat*vec summed left to right;
//   * min/max follow IEEE-754 minNum/maxNum (a NaN operand yields the other
//     operand; equal operands yield the second);
//   * sin/cos: Cody-Waite reduction by pi/2 with a three-part constant, then
//     the Taylor series of sin (to x^9) and cos (to x^10) on [-pi/4, pi/4];
//   * atan2: octant reduction to t in [0,1], t > tan(pi/8) shifted by
//     atan(t) = pi/4 + atan((t-1)/(t+1)), Taylor series of atan to z^21;
//   * acos(x) = atan2(sqrt((1-x)(1+x)), x);
//   * exp2: x = k + f, |f| <= 1/2, 2^f = sum (ln2)^n f^n / n! to n = 8,
//     scaled by exact powers of two (two steps so subnormals round once);
//   * log2: x = 2^e m with m in [sqrt(1/2), sqrt(2)], s = (m-1)/(m+1),
//     log2 m = (2/ln2) atanh(s), atanh by its Taylor series to s^13;
//   * pow(x, y) = exp2(y * log2(x))   (the WGSL definition of pow).
// Every coefficient is a Taylor coefficient (1/n!, 1/(2n+1), (ln2)^n/n!) or a
// rounding of pi/2, 2/pi, 2/ln2, tan(pi/8), sqrt(2), rounded to binary32 and
// written as an exact hexadecimal literal.  The device code implements the
// same definition independently (pike_gb300/csrc/pk_math.cuh); GPU tests check
// the two bit for bit over large input sweeps.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace om {

static inline uint32_t f2u(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
static inline float u2f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
static inline bool isnan_(float x) { return x != x; }

// IEEE minNum/maxNum; for equal operands (e.g. -0 and +0) returns b.
static inline float fmin_(float a, float b) { if (isnan_(a)) return b; if (isnan_(b)) return a; return a < b ? a : b; }
static inline float fmax_(float a, float b) { if (isnan_(a)) return b; if (isnan_(b)) return a; return a > b ? a : b; }
static inline float clamp_(float x, float lo, float hi) { return fmin_(fmax_(x, lo), hi); }

// WGSL f32 -> i32: truncate toward zero, saturate, NaN -> 0.
static inline int32_t f2i(float x) {
  if (isnan_(x)) return 0;
  if (x >= 2147483520.0f) return 2147483647;
  if (x <= -2147483648.0f) return (int32_t)0x80000000u;
  return (int32_t)x;
}

// 2^n as a float for n in [-126, 127].
static inline float pow2i(int n) { return u2f((uint32_t)(n + 127) << 23); }

static const float PIO2_1 = 0x1.92p+0f;
static const float PIO2_2 = 0x1.fb6p-12f;
static const float PIO2_3 = -0x1.777a5cp-25f;
static const float TWO_OVER_PI = 0x1.45f306p-1f;
static const float S1 = -0x1.555556p-3f, S2 = 0x1.111112p-7f, S3 = -0x1.a01a02p-13f, S4 = 0x1.71de3ap-19f;
static const float C1 = -0x1.0p-1f, C2 = 0x1.555556p-5f, C3 = -0x1.6c16c2p-10f, C4 = 0x1.a01a02p-16f, C5 = -0x1.27e4fcp-22f;

static inline float sin_poly(float r) {
  float s = r * r;
  float p = S4;
  p = S3 + s * p;
  p = S2 + s * p;
  p = S1 + s * p;
  return r + (r * s) * p;
}
static inline float cos_poly(float r) {
  float s = r * r;
  float p = C5;
  p = C4 + s * p;
  p = C3 + s * p;
  p = C2 + s * p;
  p = C1 + s * p;
  return 1.0f + s * p;
}
// Reduce x to r in about [-pi/4, pi/4] and quadrant q in {0,1,2,3}.
static inline float reduce_pio2(float x, int* q) {
  float k = std::floor(x * TWO_OVER_PI + 0.5f);
  float r = x - k * PIO2_1;
  r = r - k * PIO2_2;
  r = r - k * PIO2_3;
  float k4 = k - 4.0f * std::floor(k * 0.25f);
  *q = (int)k4;
  return r;
}
static inline float sin_(float x) {
  if (!(std::fabs(x) < 1.0e30f)) return x - x;  // NaN for NaN/inf
  int q; float r = reduce_pio2(x, &q);
  switch (q) {
    case 0: return sin_poly(r);
    case 1: return cos_poly(r);
    case 2: return -sin_poly(r);
    default: return -cos_poly(r);
  }
}
static inline float cos_(float x) {
  if (!(std::fabs(x) < 1.0e30f)) return x - x;
  int q; float r = reduce_pio2(x, &q);
  switch (q) {
    case 0: return cos_poly(r);
    case 1: return -sin_poly(r);
    case 2: return -cos_poly(r);
    default: return sin_poly(r);
  }
}
static inline float tan_(float x) { return sin_(x) / cos_(x); }

static const float PI_F = 0x1.921fb6p+1f, PIO2_F = 0x1.921fb6p+0f, PIO4_F = 0x1.921fb6p-1f;
static const float TAN_PI_8 = 0x1.a8279ap-2f;
static const float A1 = -0x1.555556p-2f, A2 = 0x1.99999ap-3f, A3 = -0x1.24924ap-3f, A4 = 0x1.c71c72p-4f,
                   A5 = -0x1.745d18p-4f, A6 = 0x1.3b13b2p-4f, A7 = -0x1.111112p-4f, A8 = 0x1.e1e1e2p-5f,
                   A9 = -0x1.af286cp-5f, A10 = 0x1.861862p-5f;

// atan(t) for t in [0, 1].
static inline float atan01(float t) {
  float base = 0.0f;
  float z = t;
  if (t > TAN_PI_8) { z = (t - 1.0f) / (t + 1.0f); base = PIO4_F; }
  float z2 = z * z;
  float p = A10;
  p = A9 + z2 * p;
  p = A8 + z2 * p;
  p = A7 + z2 * p;
  p = A6 + z2 * p;
  p = A5 + z2 * p;
  p = A4 + z2 * p;
  p = A3 + z2 * p;
  p = A2 + z2 * p;
  p = A1 + z2 * p;
  return base + (z + (z * z2) * p);
}
static inline float atan2_(float y, float x) {
  if (isnan_(x) || isnan_(y)) return x + y;
  float ax = std::fabs(x), ay = std::fabs(y);
  float a;
  if (ax == 0.0f && ay == 0.0f) {
    a = 0.0f;
  } else if (std::isinf(ax) && std::isinf(ay)) {
    a = PIO4_F;
  } else if (ay > ax) {
    a = PIO2_F - atan01(ax / ay);
  } else {
    a = atan01(ay / ax);
  }
  if (std::signbit(x)) a = PI_F - a;
  return std::copysign(a, y);
}
static inline float acos_(float x) { return atan2_(std::sqrt((1.0f - x) * (1.0f + x)), x); }

static const float E1 = 0x1.62e43p-1f, E2 = 0x1.ebfbep-3f, E3 = 0x1.c6b08ep-5f, E4 = 0x1.3b2ab6p-7f,
                   E5 = 0x1.5d87fep-10f, E6 = 0x1.430912p-13f, E7 = 0x1.ffcbfcp-17f, E8 = 0x1.62c022p-20f;
static inline float exp2_(float x) {
  if (isnan_(x)) return x;
  if (x >= 128.0f) return INFINITY;
  if (x < -150.0f) return 0.0f;
  float k = std::floor(x + 0.5f);
  float f = x - k;
  float p = E8;
  p = E7 + f * p;
  p = E6 + f * p;
  p = E5 + f * p;
  p = E4 + f * p;
  p = E3 + f * p;
  p = E2 + f * p;
  p = E1 + f * p;
  float r = 1.0f + f * p;
  int ki = (int)k;
  if (ki > 64) { r = r * pow2i(64); ki -= 64; }
  if (ki < -64) { r = r * pow2i(-64); ki += 64; }
  return r * pow2i(ki);
}

static const float L1 = 0x1.555556p-2f, L2 = 0x1.99999ap-3f, L3 = 0x1.24924ap-3f, L4 = 0x1.c71c72p-4f,
                   L5 = 0x1.745d18p-4f, L6 = 0x1.3b13b2p-4f;
static const float TWO_OVER_LN2 = 0x1.715476p+1f;
static const float SQRT2_F = 0x1.6a09e6p+0f;
static inline float log2_(float x) {
  if (isnan_(x) || x < 0.0f) return NAN;
  if (x == 0.0f) return -INFINITY;
  if (std::isinf(x)) return INFINITY;
  int e = 0;
  if (x < 0x1.0p-126f) { x = x * 0x1.0p+23f; e = -23; }
  uint32_t b = f2u(x);
  e += (int)((b >> 23) & 0xffu) - 127;
  float m = u2f((b & 0x7fffffu) | 0x3f800000u);
  if (m > SQRT2_F) { m = m * 0.5f; e += 1; }
  float s = (m - 1.0f) / (m + 1.0f);
  float s2 = s * s;
  float p = L6;
  p = L5 + s2 * p;
  p = L4 + s2 * p;
  p = L3 + s2 * p;
  p = L2 + s2 * p;
  p = L1 + s2 * p;
  float t = s + (s * s2) * p;
  return (float)e + t * TWO_OVER_LN2;
}
static inline float pow_(float x, float y) { return exp2_(y * log2_(x)); }

// ---- WGSL packing built-ins (WGSL spec, "Data packing/unpacking") --------
static inline float unorm16(uint32_t v) { return (float)v / 65535.0f; }
static inline float snorm16(int32_t v) { return fmax_((float)v / 32767.0f, -1.0f); }
static inline float snorm8(int32_t v) { return fmax_((float)v / 127.0f, -1.0f); }
static inline void unpack2x16unorm(uint32_t w, float* a, float* b) { *a = unorm16(w & 0xffffu); *b = unorm16(w >> 16); }
static inline void unpack2x16snorm(uint32_t w, float* a, float* b) {
  *a = snorm16((int16_t)(uint16_t)(w & 0xffffu));
  *b = snorm16((int16_t)(uint16_t)(w >> 16));
}
static inline void unpack4x8snorm3(uint32_t w, float* a, float* b, float* c) {
  *a = snorm8((int8_t)(uint8_t)(w & 0xffu));
  *b = snorm8((int8_t)(uint8_t)((w >> 8) & 0xffu));
  *c = snorm8((int8_t)(uint8_t)((w >> 16) & 0xffu));
}
// pack2x16unorm: floor(0.5 + 65535 * min(1, max(0, e))).
static inline uint32_t pack_unorm16(float e) { return (uint32_t)std::floor(0.5f + 65535.0f * fmin_(1.0f, fmax_(0.0f, e))); }
static inline uint32_t pack2x16unorm(float a, float b) { return pack_unorm16(a) | (pack_unorm16(b) << 16); }

// ---- vec3 in WGSL evaluation order --------------------------------------
struct V3 { float x, y, z; };
static inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
static inline V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 mul(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline V3 scale(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline V3 neg(V3 a) { return v3(-a.x, -a.y, -a.z); }
static inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 cross(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline float length(V3 a) { return std::sqrt(dot(a, a)); }
static inline V3 normalize(V3 a) { float l = length(a); return v3(a.x / l, a.y / l, a.z / l); }
// mat3x3(c0, c1, c2) * v
static inline V3 matvec(V3 c0, V3 c1, V3 c2, V3 v) { return add(add(scale(c0, v.x), scale(c1, v.y)), scale(c2, v.z)); }
// v * mat3x3(c0, c1, c2)
static inline V3 vecmat(V3 v, V3 c0, V3 c1, V3 c2) { return v3(dot(v, c0), dot(v, c1), dot(v, c2)); }
static inline float mix1(float a, float b, float t) { return a * (1.0f - t) + b * t; }
static inline V3 reflect(V3 e1, V3 e2) { return sub(e1, scale(e2, 2.0f * dot(e2, e1))); }
static inline float inverse_sqrt(float x) { return 1.0f / std::sqrt(x); }

}  // namespace om
