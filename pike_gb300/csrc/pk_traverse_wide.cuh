// pk_traverse_wide.cuh -- form (1)'s traversal pieces: the compressed 8-wide
// node test (pk_wide.h) and the watertight triangle test shared by the 8-wide
// traversal and the FP32 binary reference (PK_TRACE_EXACT).
//
// Closest hit is the minimum of (t, slot) over every triangle the watertight
// test accepts, any hit is "some triangle accepted": boxes enclose their
// triangles with a margin and are tested with a relative slack, so the result
// does not depend on the traversal order, and both traversals (and the
// oracle's brute force) return the same bits.
#pragma once
#include "pk_internal.cuh"

namespace pk {

constexpr float WIDE_SLACK = 0x1p-16f;

// Three-input minimum and maximum (sm_100 and later).
__device__ __forceinline__ float max3f(float a, float b, float c) {
  float d;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
  float d;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}

// 1/d clamped to +-1e30, so that axis-parallel rays (d = +-0) keep finite slab
// terms (an infinite inverse would turn q * 2^e * inv + (p - o) * inv into inf - inf).
__device__ __forceinline__ float wide_inverse(float d) { return fminf(fmaxf(1.0f / d, -1e30f), 1e30f); }

// Per-ray set-up of the watertight test (Woop, Benthin & Wald, "Watertight
// Ray/Triangle Intersection", JCGT 2(1), 2013): kz = the axis of largest
// |d| (first of equals), kx, ky the next two cyclically (swapped when
// d[kz] < 0, which keeps the winding), shear S = (d[kx]/d[kz], d[ky]/d[kz],
// 1/d[kz]).  The origin is stored permuted.
struct WtRay {
  int kx, ky, kz;
  float sx, sy, sz;
  float ox, oy, oz;  // origin[kx], origin[ky], origin[kz]
};
__device__ __forceinline__ float sel3(float x, float y, float z, int k) { return k == 0 ? x : (k == 1 ? y : z); }
__device__ __forceinline__ WtRay wt_setup(float ox, float oy, float oz, float dx, float dy, float dz) {
  WtRay w;
  const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
  int kz = 0;
  float m = ax;
  if (ay > m) { kz = 1; m = ay; }
  if (az > m) kz = 2;
  int kx = kz == 2 ? 0 : kz + 1;
  int ky = kx == 2 ? 0 : kx + 1;
  const float dkz = sel3(dx, dy, dz, kz);
  if (dkz < 0.0f) { const int t = kx; kx = ky; ky = t; }
  w.kx = kx; w.ky = ky; w.kz = kz;
  w.sx = sel3(dx, dy, dz, kx) / dkz;
  w.sy = sel3(dx, dy, dz, ky) / dkz;
  w.sz = 1.0f / dkz;
  w.ox = sel3(ox, oy, oz, kx);
  w.oy = sel3(ox, oy, oz, ky);
  w.oz = sel3(ox, oy, oz, kz);
  return w;
}

// The watertight test on one triangle record {v0.xyz, v1.x}{v1.yz, v2.xy}
// {v2.z, slot, -, -}: false when rejected; otherwise t = T/det (accepted when
// t > eps, eps = the pass's EPSILON: 1e-8 closest, 1e-7 any hit) and the
// barycentrics of v1 and v2 (u = V/det, v = W/det, the reference's (u, v)).
// An edge function that is exactly zero is recomputed in double from the
// exact products, as in the paper, so rays through shared edges and vertices
// hit at least one of the triangles.
__device__ __forceinline__ bool wt_test(const float4* __restrict__ tris, uint32_t rec, const WtRay& r, float eps,
                                        float& t, float& u, float& v, uint32_t& slot) {
  const float4* tp = tris + 3 * (size_t)rec;
  const float4 P = __ldg(tp), Q = __ldg(tp + 1), R = __ldg(tp + 2);
  // A = v0 - o, B = v1 - o, C = v2 - o in the permuted frame
  const float Akx = sel3(P.x, P.y, P.z, r.kx) - r.ox, Aky = sel3(P.x, P.y, P.z, r.ky) - r.oy,
              Akz = sel3(P.x, P.y, P.z, r.kz) - r.oz;
  const float Bkx = sel3(P.w, Q.x, Q.y, r.kx) - r.ox, Bky = sel3(P.w, Q.x, Q.y, r.ky) - r.oy,
              Bkz = sel3(P.w, Q.x, Q.y, r.kz) - r.oz;
  const float Ckx = sel3(Q.z, Q.w, R.x, r.kx) - r.ox, Cky = sel3(Q.z, Q.w, R.x, r.ky) - r.oy,
              Ckz = sel3(Q.z, Q.w, R.x, r.kz) - r.oz;
  const float Ax = Akx - r.sx * Akz, Ay = Aky - r.sy * Akz;
  const float Bx = Bkx - r.sx * Bkz, By = Bky - r.sy * Bkz;
  const float Cx = Ckx - r.sx * Ckz, Cy = Cky - r.sy * Ckz;
  float U = Cx * By - Cy * Bx;
  float V = Ax * Cy - Ay * Cx;
  float W = Bx * Ay - By * Ax;
  if (U == 0.0f || V == 0.0f || W == 0.0f) {
    U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
    V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
    W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
  }
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
  const float det = U + V + W;
  if (det == 0.0f) return false;
  const float Az = r.sz * Akz, Bz = r.sz * Bkz, Cz = r.sz * Ckz;
  const float T = U * Az + V * Bz + W * Cz;
  t = T / det;
  if (!(t > eps)) return false;
  u = V / det;
  v = W / det;
  slot = __float_as_uint(R.y);
  return true;
}

// Byte k of `word` as a float.  (Building the float 2^23 + byte by a byte
// permute and subtracting 2^23, instead of the conversion instruction, was
// measured no faster: 2966-2990 against 2980-2984 Mrays/s.)
__device__ __forceinline__ float byte_float(uint32_t word, int k) { return (float)((word >> (8 * k)) & 0xffu); }

// Child test of one compressed wide node (pk_wide.h).  Returns the node's
// internal-child hit mask, with the child of slot s at bit (s ^ oct) (the
// visiting order of the ray's octant), and the triangle-record hit mask
// relative to tri_base; child_base, tri_base and imask are read from the
// node.  The decode is folded into the slab test: t = q * (2^e * inv) +
// (p - o) * inv, one FMA per plane, near and far planes chosen per axis
// from the sign of inv; relative to the exact planes p + 2^e q this moves a
// plane by a few ulps of |p - o|, well inside the 2^-18 margin the builder
// adds around every box.  `cull`: the current best hit.
__device__ __forceinline__ void cw_node(const float4* __restrict__ nodes, uint32_t node, float ox, float oy,
                                        float oz, float ix, float iy, float iz, uint32_t oct, float cull,
                                        uint32_t& child_base, uint32_t& tri_base, uint32_t& imask,
                                        uint32_t& inner_hits, uint32_t& tri_hits) {
  const float4* r = nodes + 5 * (size_t)node;
  const float4 h = __ldg(r);
  const uint4 b = __ldg(reinterpret_cast<const uint4*>(r) + 1);
  const uint4 q0 = __ldg(reinterpret_cast<const uint4*>(r) + 2);
  const uint4 q1 = __ldg(reinterpret_cast<const uint4*>(r) + 3);
  const uint4 q2 = __ldg(reinterpret_cast<const uint4*>(r) + 4);
  const uint32_t packed = __float_as_uint(h.w);
  const float sx = __uint_as_float((packed & 0xffu) << 23);
  const float sy = __uint_as_float(((packed >> 8) & 0xffu) << 23);
  const float sz = __uint_as_float(((packed >> 16) & 0xffu) << 23);
  imask = packed >> 24;
  child_base = b.x;
  tri_base = b.y;
  const float ax = (h.x - ox) * ix, ay = (h.y - oy) * iy, az = (h.z - oz) * iz;
  const float bx = sx * ix, by = sy * iy, bz = sz * iz;
  // byte planes: x lo (q0.x q0.y) hi (q1.z q1.w); y lo (q0.z q0.w) hi (q2.x q2.y); z lo (q1.x q1.y) hi (q2.z q2.w)
  const bool px = ix >= 0.0f, py = iy >= 0.0f, pz = iz >= 0.0f;
  const uint32_t nx0 = px ? q0.x : q1.z, nx1 = px ? q0.y : q1.w, fx0 = px ? q1.z : q0.x, fx1 = px ? q1.w : q0.y;
  const uint32_t ny0 = py ? q0.z : q2.x, ny1 = py ? q0.w : q2.y, fy0 = py ? q2.x : q0.z, fy1 = py ? q2.y : q0.w;
  const uint32_t nz0 = pz ? q1.x : q2.z, nz1 = pz ? q1.y : q2.w, fz0 = pz ? q2.z : q1.x, fz1 = pz ? q2.w : q1.y;
  const float cull_s = cull + cull * WIDE_SLACK;
  inner_hits = 0u;
  tri_hits = 0u;
  // The slot hit mask first, from three-input min/max and one comparison:
  // max(tmin, 0) <= min(tmax_s, cull_s) is tmin <= tmax_s && tmax_s >= 0 &&
  // tmin <= cull_s, since cull_s > 0.  Empty slots need no test of their
  // own: they are neither internal nor own triangles (meta 0).  Against
  // per-child tests with the masks built inside the loop: 1080p frame
  // 3348-3352 against 3292-3301 Mrays/s, closest-hit launch 0.376 against
  // 0.385 ms.
  uint32_t hb = 0u;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const int kb = k & 3;
    const float tnx = __fmaf_rn(byte_float(k < 4 ? nx0 : nx1, kb), bx, ax);
    const float tny = __fmaf_rn(byte_float(k < 4 ? ny0 : ny1, kb), by, ay);
    const float tnz = __fmaf_rn(byte_float(k < 4 ? nz0 : nz1, kb), bz, az);
    const float tfx = __fmaf_rn(byte_float(k < 4 ? fx0 : fx1, kb), bx, ax);
    const float tfy = __fmaf_rn(byte_float(k < 4 ? fy0 : fy1, kb), by, ay);
    const float tfz = __fmaf_rn(byte_float(k < 4 ? fz0 : fz1, kb), bz, az);
    const float tmax = min3f(tfx, tfy, tfz);
    const float hi = fminf(__fmaf_rn(fabsf(tmax), WIDE_SLACK, tmax), cull_s);
    if (fmaxf(max3f(tnx, tny, tnz), 0.0f) <= hi) hb |= 1u << k;
  }
  // internal children: slot k -> visiting position k ^ oct
  uint32_t x = hb & imask;
  if (oct & 1u) x = ((x & 0x55u) << 1) | ((x >> 1) & 0x55u);
  if (oct & 2u) x = ((x & 0x33u) << 2) | ((x >> 2) & 0x33u);
  if (oct & 4u) x = ((x & 0x0fu) << 4) | ((x >> 4) & 0x0fu);
  inner_hits = x;
  uint32_t leaves = hb & ~imask;
  while (leaves) {
    const uint32_t k = (uint32_t)__ffs(leaves) - 1u;
    leaves &= leaves - 1u;
    const uint32_t meta = ((k < 4u ? b.z : b.w) >> (8u * (k & 3u))) & 0xffu;
    tri_hits |= (meta >> 5) << (meta & 31u);
  }
}

}  // namespace pk
