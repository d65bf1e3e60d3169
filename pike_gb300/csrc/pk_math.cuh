// pk_math.cuh -- device definition of the WGSL built-ins Pike's passes use.
//
// WGSL leaves the accuracy of sin/cos/atan2/acos/pow/exp2/log2, the summation
// order of dot products and FMA contraction to the implementation.  This
// library pins them so that every pass is reproducible bit for bit:
//   * binary32, round-to-nearest-even, no contraction (the library is built
//     with -fmad=false -prec-div=true -prec-sqrt=true -ftz=false);
//   * dot/cross/mat*vec summed left to right;
//   * min/max are IEEE minNum/maxNum; equal operands give the second one;
//   * sin/cos: Cody-Waite reduction by pi/2 (three-part constant), Taylor
//     polynomials of sin to r^9 and cos to r^10 on [-pi/4, pi/4];
//   * atan2: octant reduction to t in [0,1]; t > tan(pi/8) uses
//     atan(t) = pi/4 + atan((t-1)/(t+1)); Taylor polynomial of atan to z^21;
//   * acos(x) = atan2(sqrt((1-x)(1+x)), x);
//   * exp2: x = k + f with |f| <= 1/2, 2^f by its Taylor series in f
//     (coefficients (ln 2)^n / n!, n <= 8), scaled by exact powers of two;
//   * log2: x = 2^e m, m in [sqrt(1/2), sqrt(2)], s = (m-1)/(m+1),
//     log2 m = (2/ln 2) atanh(s) with the Taylor series of atanh to s^13;
//   * pow(x, y) = exp2(y log2 x), as WGSL defines pow.
// Coefficients are Taylor coefficients rounded to binary32 (hex literals).
#pragma once
#include <cstdint>

namespace pk {

__device__ __forceinline__ float fmin_(float a, float b) { return (a != a) ? b : ((b != b) ? a : (a < b ? a : b)); }
__device__ __forceinline__ float fmax_(float a, float b) { return (a != a) ? b : ((b != b) ? a : (a > b ? a : b)); }
__device__ __forceinline__ float clamp_(float x, float lo, float hi) { return fmin_(fmax_(x, lo), hi); }

// WGSL f32 -> i32: truncate, saturate, NaN -> 0.
__device__ __forceinline__ int f2i(float x) {
  if (x != x) return 0;
  if (x >= 2147483520.0f) return 2147483647;
  if (x <= -2147483648.0f) return (int)0x80000000u;
  return (int)x;
}
__device__ __forceinline__ float pow2i(int n) { return __uint_as_float((uint32_t)(n + 127) << 23); }

namespace c {
constexpr float PIO2_1 = 0x1.92p+0f, PIO2_2 = 0x1.fb6p-12f, PIO2_3 = -0x1.777a5cp-25f;
constexpr float TWO_OVER_PI = 0x1.45f306p-1f;
constexpr float S1 = -0x1.555556p-3f, S2 = 0x1.111112p-7f, S3 = -0x1.a01a02p-13f, S4 = 0x1.71de3ap-19f;
constexpr float C1 = -0x1.0p-1f, C2 = 0x1.555556p-5f, C3 = -0x1.6c16c2p-10f, C4 = 0x1.a01a02p-16f,
                C5 = -0x1.27e4fcp-22f;
constexpr float PI = 0x1.921fb6p+1f, PIO2 = 0x1.921fb6p+0f, PIO4 = 0x1.921fb6p-1f;
constexpr float TAN_PI_8 = 0x1.a8279ap-2f;
constexpr float A1 = -0x1.555556p-2f, A2 = 0x1.99999ap-3f, A3 = -0x1.24924ap-3f, A4 = 0x1.c71c72p-4f,
                A5 = -0x1.745d18p-4f, A6 = 0x1.3b13b2p-4f, A7 = -0x1.111112p-4f, A8 = 0x1.e1e1e2p-5f,
                A9 = -0x1.af286cp-5f, A10 = 0x1.861862p-5f;
constexpr float E1 = 0x1.62e43p-1f, E2 = 0x1.ebfbep-3f, E3 = 0x1.c6b08ep-5f, E4 = 0x1.3b2ab6p-7f,
                E5 = 0x1.5d87fep-10f, E6 = 0x1.430912p-13f, E7 = 0x1.ffcbfcp-17f, E8 = 0x1.62c022p-20f;
constexpr float L1 = 0x1.555556p-2f, L2 = 0x1.99999ap-3f, L3 = 0x1.24924ap-3f, L4 = 0x1.c71c72p-4f,
                L5 = 0x1.745d18p-4f, L6 = 0x1.3b13b2p-4f;
constexpr float TWO_OVER_LN2 = 0x1.715476p+1f, SQRT2 = 0x1.6a09e6p+0f;
constexpr float TAU = 6.283185307179586f, INV_PI = 0.3183098861837907f;
}  // namespace c

__device__ __forceinline__ float sin_poly(float r) {
  const float s = r * r;
  float p = c::S4;
  p = c::S3 + s * p;
  p = c::S2 + s * p;
  p = c::S1 + s * p;
  return r + (r * s) * p;
}
__device__ __forceinline__ float cos_poly(float r) {
  const float s = r * r;
  float p = c::C5;
  p = c::C4 + s * p;
  p = c::C3 + s * p;
  p = c::C2 + s * p;
  p = c::C1 + s * p;
  return 1.0f + s * p;
}
__device__ __forceinline__ float reduce_pio2(float x, int& q) {
  const float k = floorf(x * c::TWO_OVER_PI + 0.5f);
  float r = x - k * c::PIO2_1;
  r = r - k * c::PIO2_2;
  r = r - k * c::PIO2_3;
  q = (int)(k - 4.0f * floorf(k * 0.25f));
  return r;
}
// sin_, cos_ and atan2_ are called, not inlined: shading uses them at a dozen
// sites, and one copy each keeps the batch megakernel's code within the
// instruction cache (948 vs 1057 ms on the 64-request batch, the drop-in
// frame rate unchanged).
static __device__ __noinline__ float sin_(float x) {
  if (!(fabsf(x) < 1.0e30f)) return x - x;
  int q;
  const float r = reduce_pio2(x, q);
  const float v = (q & 1) ? cos_poly(r) : sin_poly(r);
  return (q & 2) ? -v : v;
}
static __device__ __noinline__ float cos_(float x) {
  if (!(fabsf(x) < 1.0e30f)) return x - x;
  int q;
  const float r = reduce_pio2(x, q);
  const float v = (q & 1) ? sin_poly(r) : cos_poly(r);
  return ((q + 1) & 2) ? -v : v;
}
__device__ __forceinline__ float tan_(float x) { return sin_(x) / cos_(x); }

__device__ __forceinline__ float atan01(float t) {
  float base = 0.0f, z = t;
  if (t > c::TAN_PI_8) {
    z = (t - 1.0f) / (t + 1.0f);
    base = c::PIO4;
  }
  const float z2 = z * z;
  float p = c::A10;
  p = c::A9 + z2 * p;
  p = c::A8 + z2 * p;
  p = c::A7 + z2 * p;
  p = c::A6 + z2 * p;
  p = c::A5 + z2 * p;
  p = c::A4 + z2 * p;
  p = c::A3 + z2 * p;
  p = c::A2 + z2 * p;
  p = c::A1 + z2 * p;
  return base + (z + (z * z2) * p);
}
static __device__ __noinline__ float atan2_(float y, float x) {
  if (x != x || y != y) return x + y;
  const float ax = fabsf(x), ay = fabsf(y);
  float a;
  if (ax == 0.0f && ay == 0.0f) a = 0.0f;
  else if (isinf(ax) && isinf(ay)) a = c::PIO4;
  else if (ay > ax) a = c::PIO2 - atan01(ax / ay);
  else a = atan01(ay / ax);
  if (signbit(x)) a = c::PI - a;
  return copysignf(a, y);
}
__device__ __forceinline__ float acos_(float x) { return atan2_(sqrtf((1.0f - x) * (1.0f + x)), x); }

__device__ __forceinline__ float exp2_(float x) {
  if (x != x) return x;
  if (x >= 128.0f) return __int_as_float(0x7f800000);
  if (x < -150.0f) return 0.0f;
  const float k = floorf(x + 0.5f);
  const float f = x - k;
  float p = c::E8;
  p = c::E7 + f * p;
  p = c::E6 + f * p;
  p = c::E5 + f * p;
  p = c::E4 + f * p;
  p = c::E3 + f * p;
  p = c::E2 + f * p;
  p = c::E1 + f * p;
  float r = 1.0f + f * p;
  int ki = (int)k;
  if (ki > 64) { r = r * pow2i(64); ki -= 64; }
  if (ki < -64) { r = r * pow2i(-64); ki += 64; }
  return r * pow2i(ki);
}
__device__ __forceinline__ float log2_(float x) {
  if (x != x || x < 0.0f) return __int_as_float(0x7fc00000);
  if (x == 0.0f) return __int_as_float(0xff800000);
  if (isinf(x)) return x;
  int e = 0;
  if (x < 0x1.0p-126f) { x = x * 0x1.0p+23f; e = -23; }
  const uint32_t b = __float_as_uint(x);
  e += (int)((b >> 23) & 0xffu) - 127;
  float m = __uint_as_float((b & 0x7fffffu) | 0x3f800000u);
  if (m > c::SQRT2) { m = m * 0.5f; e += 1; }
  const float s = (m - 1.0f) / (m + 1.0f);
  const float s2 = s * s;
  float p = c::L6;
  p = c::L5 + s2 * p;
  p = c::L4 + s2 * p;
  p = c::L3 + s2 * p;
  p = c::L2 + s2 * p;
  p = c::L1 + s2 * p;
  const float t = s + (s * s2) * p;
  return (float)e + t * c::TWO_OVER_LN2;
}
__device__ __forceinline__ float pow_(float x, float y) { return exp2_(y * log2_(x)); }

// ---- WGSL data packing ---------------------------------------------------
// v / d for an integer-valued v by a constant d: the product with r = RN(1/d)
// corrected by one FMA with the exact residual v - q0 d.  For the domains
// used below (v in [-128, 127] by 127, [0, 255] by 255, [0, 65535] by 65535,
// [-32768, 32767] by 32767) this equals the IEEE quotient for every input
// (the GPU tests check each domain exhaustively); it replaces an IEEE division
// (a longer inline sequence with a slow-path call) at some 45 sites per hit.
__device__ __forceinline__ float qdiv(float v, float d, float r) {
  const float q0 = __fmul_rn(v, r);
  return __fmaf_rn(__fmaf_rn(-q0, d, v), r, q0);
}
__device__ __forceinline__ float unorm16(uint32_t v) { return qdiv((float)v, 65535.0f, 0x1.0001p-16f); }
__device__ __forceinline__ float snorm16(int v) { return fmax_(qdiv((float)v, 32767.0f, 0x1.0002p-15f), -1.0f); }
__device__ __forceinline__ float snorm8(int v) { return fmax_(qdiv((float)v, 127.0f, 0x1.020408p-7f), -1.0f); }
__device__ __forceinline__ float unorm8(uint32_t v) { return qdiv((float)v, 255.0f, 0x1.010102p-8f); }
__device__ __forceinline__ uint32_t pack_unorm16(float e) {
  return (uint32_t)floorf(0.5f + 65535.0f * fmin_(1.0f, fmax_(0.0f, e)));
}

// ---- vec3 in WGSL evaluation order ---------------------------------------
struct V3 { float x, y, z; };
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 mul(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ V3 scale(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V3 neg(V3 a) { return v3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
// Called, not inlined (an IEEE square root and three IEEE quotients at a
// dozen shading sites), for the same instruction-cache reason as sin_.
static __device__ __noinline__ V3 normalize(V3 a) {
  const float l = sqrtf(dot(a, a));
  return v3(a.x / l, a.y / l, a.z / l);
}
__device__ __forceinline__ V3 matvec(V3 c0, V3 c1, V3 c2, V3 v) {
  return add(add(scale(c0, v.x), scale(c1, v.y)), scale(c2, v.z));
}
__device__ __forceinline__ V3 vecmat(V3 v, V3 c0, V3 c1, V3 c2) { return v3(dot(v, c0), dot(v, c1), dot(v, c2)); }
__device__ __forceinline__ float mix1(float a, float b, float t) { return a * (1.0f - t) + b * t; }
__device__ __forceinline__ V3 reflect(V3 e1, V3 e2) { return sub(e1, scale(e2, 2.0f * dot(e2, e1))); }

// Jarzynski & Olano PCG-style hash used by camera.wgsl and shade_hit.wgsl.
struct Hash {
  uint32_t seed;
  __device__ __forceinline__ uint32_t next() {
    const uint32_t state = seed;
    seed = seed * 747796405u + 2891336453u;
    const uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
  }
  __device__ __forceinline__ float rand() { return (float)next() / 4294967296.0f; }
};

}  // namespace pk
