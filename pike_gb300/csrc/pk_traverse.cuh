// pk_traverse.cuh -- binary-BVH traversal of trace.wgsl / trace_shadow.wgsl
// on the traversal-format BVH (see SceneDev in pk_internal.cuh).
#pragma once
#include "pk_internal.cuh"

namespace pk {

constexpr float MAX_T = 100000.0f;

// =====================================================================
// trace.wgsl:83-189 / trace_shadow.wgsl:82-190: BVH traversal.
// =====================================================================
__device__ __forceinline__ float box_hit(float xa, float xb, float ya, float yb, float za, float zb, float ox,
                                         float oy, float oz, float ix, float iy, float iz) {
  // t1 uses the x_range.x bounds (quantised max), t2 the x_range.y bounds (min).
  const float t1x = (xa - ox) * ix, t2x = (xb - ox) * ix;
  const float t1y = (ya - oy) * iy, t2y = (yb - oy) * iy;
  const float t1z = (za - oz) * iz, t2z = (zb - oz) * iz;
  // fminf/fmaxf agree with minNum/maxNum except for the sign of a zero
  // result, which only ever feeds comparisons here.  (Three-input min/max
  // for the outer reductions measured no faster: 3709-3748 against
  // 3740-3745 Mrays/s.)
  const float tmax = fminf(fminf(fmaxf(t1x, t2x), fmaxf(t1y, t2y)), fmaxf(t1z, t2z));
  const float tmin = fmaxf(fmaxf(fminf(t1x, t2x), fminf(t1y, t2y)), fminf(t1z, t2z));
  return (tmax >= tmin && tmax > 0.0f) ? tmin : MAX_T;
}

// unpack2x16snorm component: max(s / 32767, -1).  For integer s in
// [-32768, 32767] the product with RN(1/32767) corrected by two FMAs equals the
// IEEE quotient for every input (the tests check all 65536), so this is the
// same value the reference decode and the 64-byte records hold.
__device__ __forceinline__ float snorm16_decode(int s) {
  const float sf = (float)s;
  const float r = 0x1.0002p-15f;
  const float q0 = sf * r;
  const float e = __fmaf_rn(-q0, 32767.0f, sf);
  return fmax_(__fmaf_rn(e, r, q0), -1.0f);
}
__device__ __forceinline__ float snorm_lo(int m) { return snorm16_decode((int)(int16_t)(uint16_t)((uint32_t)m & 0xffffu)); }
__device__ __forceinline__ float snorm_hi(int m) { return snorm16_decode((int)(int16_t)(uint16_t)((uint32_t)m >> 16)); }

// One inner-node step: both children's entry distances and child codes.
// 32-byte records keep the reference's snorm16 boxes {Lx, Ly, Lz, Rx}{Ry, Rz,
// codeL, codeR}; 64-byte records (the default: fewer instructions per step,
// which matters more than bytes here) hold the same boxes decoded.
// (Prefetching both children's records into L1 while the boxes are tested
// measured far slower at 1080p: 3188-3197 Mrays/s against 3738-3746, and
// 2766-2769 with the leaves' first triangle too.)
__device__ __forceinline__ void inner_children(const SceneDev& sc, int cur, float ox, float oy, float oz, float ix,
                                               float iy, float iz, float& lh, float& rh, int& cl, int& cr);

// trace.wgsl:97-114: Moller-Trumbore on one leaf-ordered triangle record
// {v0.xyz, e1.x}{e1.yz, e2.xy}{e2.z}.  Returns false where the reference
// `continue`s (parallel ray, u or v outside the triangle); otherwise res = the
// distance when it exceeds eps, else MAX_T.
__device__ __forceinline__ bool mt_test(const SceneDev& sc, int idx, float ox, float oy, float oz, float dx,
                                        float dy, float dz, float eps, float& res, float& u, float& v) {
  const float4* tp = sc.tris + 3 * (size_t)idx;
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
  res = dist > eps ? dist : MAX_T;
  return true;
}

constexpr int TRACE_THREADS = 128;
constexpr int STACK_SMEM = 32;   // per-thread entries kept in shared memory
// (traverse_rt keeps the remaining 64 - SSTACK entries in local memory)

__device__ __forceinline__ void inner_children(const SceneDev& sc, int cur, float ox, float oy, float oz, float ix,
                                               float iy, float iz, float& lh, float& rh, int& cl, int& cr) {
  if (sc.inner32) {
    const int4* rec = sc.inner32 + 2 * (size_t)cur;
    const int4 q0 = __ldg(rec), q1 = __ldg(rec + 1);
    lh = box_hit(snorm_lo(q0.x), snorm_hi(q0.x), snorm_lo(q0.y), snorm_hi(q0.y), snorm_lo(q0.z), snorm_hi(q0.z), ox,
                 oy, oz, ix, iy, iz);
    rh = box_hit(snorm_lo(q0.w), snorm_hi(q0.w), snorm_lo(q1.x), snorm_hi(q1.x), snorm_lo(q1.y), snorm_hi(q1.y), ox,
                 oy, oz, ix, iy, iz);
    cl = q1.z;
    cr = q1.w;
  } else {
    const float4* rec = sc.inner + 4 * (size_t)cur;
    const float4 a = __ldg(rec), b = __ldg(rec + 1), c4 = __ldg(rec + 2);
    const int4 ch = __ldg(reinterpret_cast<const int4*>(rec) + 3);
    lh = box_hit(a.x, a.y, a.z, a.w, b.x, b.y, ox, oy, oz, ix, iy, iz);
    rh = box_hit(b.z, b.w, c4.x, c4.y, c4.z, c4.w, ox, oy, oz, ix, iy, iz);
    cl = ch.x;
    cr = ch.y;
  }
}

// Leaf-loop unroll of this shared traversal: kept off, the code size costs
// the megakernels that inline it (unrolled by 4: 64-request batch 530 against
// 440 ms, form (3) forward 691-693 against 796-799 Mrays/s, adjoint 563
// against 690-692).
#ifndef PK_RT_LEAF_UNROLL
#define PK_RT_LEAF_UNROLL 0
#endif
constexpr int RT_LEAF_UNROLL = PK_RT_LEAF_UNROLL;

// BLOCK threads per block share `sstack` (SSTACK entries per thread in shared
// memory, 64 - SSTACK more in local memory).  ANY: any hit (trace_shadow.wgsl)
// rather than closest hit; a constant at every inlined call site, a run-time
// value where one out-of-line copy serves both.
template <bool COUNT, int BLOCK, int SSTACK>
__device__ __forceinline__ void traverse_rt(const bool ANY, const SceneDev& sc, float ox, float oy, float oz,
                                            float dx, float dy, float dz, float& best_t, int& best_i,
                                            uint32_t& best_b, int (*sstack)[BLOCK], uint32_t* err,
                                            uint32_t& nfetch, uint32_t& ntest) {
  const float eps = ANY ? 1e-7f : 1e-8f;
  const float ix = 1.0f / dx, iy = 1.0f / dy, iz = 1.0f / dz;
  constexpr int LOCAL = 64 - SSTACK;  // 64 entries in all
  int lstack[LOCAL];
  const int tid = threadIdx.x;
  int sp = 0;
  int cur = sc.root;
  best_t = MAX_T;
  best_i = -1;
  best_b = 0u;
  for (;;) {
    if (cur >= 0) {
      if (COUNT) nfetch += 3;
      float lh, rh;
      int cl, cr;
      inner_children(sc, cur, ox, oy, oz, ix, iy, iz, lh, rh, cl, cr);
      const bool lok = lh < best_t, rok = rh < best_t;
      if (lok && rok) {
        int nearc, farc;
        if (lh > rh) { nearc = cr; farc = cl; } else { nearc = cl; farc = cr; }
        if (sp < SSTACK) sstack[sp][tid] = farc;
        else if (sp < SSTACK + LOCAL) lstack[sp - SSTACK] = farc;
        else { atomicOr(err, ERR_STACK); break; }
        ++sp;
        cur = nearc;
        continue;
      }
      if (lok) { cur = cl; continue; }
      if (rok) { cur = cr; continue; }
    } else {
      if (COUNT) nfetch += 1;
      const uint32_t word = (uint32_t)cur & 0x7fffffffu;
      const int size = (int)(word >> 24);
      const int base = (int)(word & 0x00ffffffu);
#if PK_RT_LEAF_UNROLL
#pragma unroll RT_LEAF_UNROLL
#endif
      for (int i = 0; i < size; i++) {
        if (COUNT) ntest += 1;
        float res, u, v;
        if (!mt_test(sc, base + i, ox, oy, oz, dx, dy, dz, eps, res, u, v)) continue;
        if (res < best_t) {
          best_t = res;
          best_i = base + i;
          best_b = pack_unorm16(u) | (pack_unorm16(v) << 16);
        }
      }
      if (ANY && best_i != -1) break;
    }
    if (sp == 0) break;
    --sp;
    cur = sp < SSTACK ? sstack[sp][tid] : lstack[sp - SSTACK];
  }
}
template <bool ANY, bool COUNT, int BLOCK = TRACE_THREADS, int SSTACK = STACK_SMEM>
__device__ __forceinline__ void traverse(const SceneDev& sc, float ox, float oy, float oz, float dx, float dy,
                                         float dz, float& best_t, int& best_i, uint32_t& best_b,
                                         int (*sstack)[BLOCK], uint32_t* err, uint32_t& nfetch,
                                         uint32_t& ntest) {
  traverse_rt<COUNT, BLOCK, SSTACK>(ANY, sc, ox, oy, oz, dx, dy, dz, best_t, best_i, best_b, sstack, err, nfetch,
                                    ntest);
}

}  // namespace pk
