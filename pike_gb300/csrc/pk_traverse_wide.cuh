// pk_traverse_wide.cuh -- traversal of the 8-wide compressed BVH (pk_wide.h).
//
// Closest hit is the minimum of (t, triangle slot) over every triangle the
// reference's Moller-Trumbore test accepts (trace.wgsl:97-114, same
// arithmetic, so t, u and v are bit-identical to the binary traversal's for
// the same triangle).  Child boxes enclose their triangles with a margin and
// are tested with a relative slack, so the result does not depend on the
// traversal order; ties on t go to the lower slot.
#pragma once
#include "pk_internal.cuh"

namespace pk {

constexpr int WIDE_STACK_SMEM = 24;   // per-thread entries (code + entry distance) in shared memory
constexpr int WIDE_STACK_LOCAL = 72;  // overflow entries in local memory
constexpr float WIDE_SLACK = 0x1p-16f;

__device__ __forceinline__ uint32_t qbyte(uint32_t lo4, uint32_t hi4, int k) {
  return ((k < 4 ? lo4 : hi4) >> (8 * (k & 3))) & 0xffu;
}

// Entry distances of the eight children of wide node `node` (+inf when the
// slot is empty, missed, or starts beyond `cull`) and their codes.  The
// decode is folded into the slab test: t = q * (2^e * inv) + (p - o) * inv,
// one FMA per bound, with the near and far byte planes chosen per axis from
// the sign of inv.  Relative to the exact planes p + 2^e q this moves each
// plane by a few ulps of |p - o|, well inside the 2^-18 margin the builder
// adds around every box; `ix, iy, iz` must be finite (see wide_inverse).
__device__ __forceinline__ void wide_children(const float4* __restrict__ W, int node, float ox, float oy, float oz,
                                              float ix, float iy, float iz, float cull, float (&d)[8], int (&c)[8]) {
  const float4* r = W + 6 * (size_t)node;
  const float4 h = __ldg(r);
  const int4 c0 = __ldg(reinterpret_cast<const int4*>(r) + 1);
  const int4 c1 = __ldg(reinterpret_cast<const int4*>(r) + 2);
  const uint4 q0 = __ldg(reinterpret_cast<const uint4*>(r) + 3);
  const uint4 q1 = __ldg(reinterpret_cast<const uint4*>(r) + 4);
  const uint4 q2 = __ldg(reinterpret_cast<const uint4*>(r) + 5);
  const uint32_t packed = __float_as_uint(h.w);
  const float sx = __uint_as_float((packed & 0xffu) << 23);
  const float sy = __uint_as_float(((packed >> 8) & 0xffu) << 23);
  const float sz = __uint_as_float(((packed >> 16) & 0xffu) << 23);
  const uint32_t valid = packed >> 24;
  c[0] = c0.x; c[1] = c0.y; c[2] = c0.z; c[3] = c0.w;
  c[4] = c1.x; c[5] = c1.y; c[6] = c1.z; c[7] = c1.w;
  const float ax = (h.x - ox) * ix, ay = (h.y - oy) * iy, az = (h.z - oz) * iz;
  const float bx = sx * ix, by = sy * iy, bz = sz * iz;
  // byte planes: x lo (q0.x q0.y) hi (q1.z q1.w); y lo (q0.z q0.w) hi (q2.x q2.y); z lo (q1.x q1.y) hi (q2.z q2.w)
  const bool px = ix >= 0.0f, py = iy >= 0.0f, pz = iz >= 0.0f;
  const uint32_t nx0 = px ? q0.x : q1.z, nx1 = px ? q0.y : q1.w, fx0 = px ? q1.z : q0.x, fx1 = px ? q1.w : q0.y;
  const uint32_t ny0 = py ? q0.z : q2.x, ny1 = py ? q0.w : q2.y, fy0 = py ? q2.x : q0.z, fy1 = py ? q2.y : q0.w;
  const uint32_t nz0 = pz ? q1.x : q2.z, nz1 = pz ? q1.y : q2.w, fz0 = pz ? q2.z : q1.x, fz1 = pz ? q2.w : q1.y;
  const float cull_s = cull + cull * WIDE_SLACK;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const float tnx = __fmaf_rn((float)qbyte(nx0, nx1, k), bx, ax);
    const float tny = __fmaf_rn((float)qbyte(ny0, ny1, k), by, ay);
    const float tnz = __fmaf_rn((float)qbyte(nz0, nz1, k), bz, az);
    const float tfx = __fmaf_rn((float)qbyte(fx0, fx1, k), bx, ax);
    const float tfy = __fmaf_rn((float)qbyte(fy0, fy1, k), by, ay);
    const float tfz = __fmaf_rn((float)qbyte(fz0, fz1, k), bz, az);
    const float tmin = fmaxf(fmaxf(tnx, tny), tnz);
    const float tmax = fminf(fminf(tfx, tfy), tfz);
    const float tmax_s = tmax + fabsf(tmax) * WIDE_SLACK;
    const bool hit = ((valid >> k) & 1u) && tmin <= tmax_s && tmax_s >= 0.0f && tmin <= cull_s;
    d[k] = hit ? tmin : __int_as_float(0x7f800000);
  }
}

// 1/d clamped to +-1e30, so that axis-parallel rays (d = +-0) keep finite slab
// terms (an infinite inverse would turn q * 2^e * inv + (p - o) * inv into inf - inf).
__device__ __forceinline__ float wide_inverse(float d) { return fminf(fmaxf(1.0f / d, -1e30f), 1e30f); }

// trace.wgsl:97-114 on one traversal-format triangle record; returns false
// when the test rejects.  eps is EPSILON of the pass (1e-8 closest, 1e-7 any).
__device__ __forceinline__ bool tri_test(const float4* __restrict__ tris, int slot, float ox, float oy, float oz,
                                         float dx, float dy, float dz, float eps, float& res, float& u, float& v) {
  const float4* tp = tris + 3 * (size_t)slot;
  const float4 A = __ldg(tp), B = __ldg(tp + 1), Cc = __ldg(tp + 2);
  const float e1x = A.w, e1y = B.x, e1z = B.y, e2x = B.z, e2y = B.w, e2z = Cc.x;
  const float px = dy * e2z - dz * e2y, py = dz * e2x - dx * e2z, pz = dx * e2y - dy * e2x;
  const float det = e1x * px + e1y * py + e1z * pz;
  if (fabsf(det) < eps) return false;
  const float inv_det = 1.0f / det;
  const float tx = ox - A.x, ty = oy - A.y, tz = oz - A.z;
  u = (tx * px + ty * py + tz * pz) * inv_det;
  if (u < 0.0f || u > 1.0f) return false;
  const float qx = ty * e1z - tz * e1y, qy = tz * e1x - tx * e1z, qz = tx * e1y - ty * e1x;
  v = (dx * qx + dy * qy + dz * qz) * inv_det;
  if (v < 0.0f || u + v > 1.0f) return false;
  const float dist = (e2x * qx + e2y * qy + e2z * qz) * inv_det;
  res = dist > eps ? dist : 100000.0f;
  return true;
}

}  // namespace pk
