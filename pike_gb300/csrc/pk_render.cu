// pk_render.cu -- the per-frame passes of Pike's wavefront path tracer on sm_103a.
//
// Each kernel follows one WGSL entry point of the reference (cited per kernel)
// and reproduces its results bit for bit under the arithmetic definition in
// pk_math.cuh.  Queue slots are assigned by stable (order-preserving)
// compaction, i.e. in increasing source slot, the order the reference's
// atomic appends take when invocations run serially.
#include <cuda_runtime.h>

#include <algorithm>

#include "pk_internal.cuh"
#include "pk_render.h"
#include "pk_shade.cuh"
#include "pk_traverse.cuh"
#include "pk_traverse_wide.cuh"

namespace pk {

// offset >= 0 replaces the camera's invocationOffset (tick()'s batch j passes
// j * BATCH_SIZE, pike.js:146).
__global__ void __launch_bounds__(128) k_camera(const CamState* __restrict__ camp, Counters* __restrict__ ctr,
                                                RayQ R, uint32_t n_threads, uint32_t capacity, int64_t offset) {
  const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= n_threads) return;
  const CamState cam = *camp;
  const uint32_t W = cam.dims_mask >> 16, H = cam.dims_mask & 0xffffu;
  const uint32_t idx = gid + (offset >= 0 ? (uint32_t)offset : cam.invocation_offset);
  const uint32_t px = idx % W, py = idx / W;
  if (px >= W || py >= H) return;
  V3 org, dir;
  camera_ray(cam, px, py, W, H, ctr->samples, org, dir);
  if (gid < capacity) {
    R.o[gid] = make_float4(org.x, org.y, org.z, 0.0f);
    R.d[gid] = make_float4(dir.x, dir.y, dir.z, 0.0f);
    R.t[gid] = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(idx));
  } else {
    atomicOr(&ctr->err, ERR_QUEUE);
  }
  atomicAdd(&ctr->num_rays, 1u);
}

__device__ __forceinline__ void add_color(float4* color, uint32_t npix, uint32_t idx, float r, float g, float b,
                                          float a, uint32_t* err) {
  if (idx >= npix) { atomicOr(err, ERR_PIXEL); return; }
  float4 c = color[idx];
  c.x = c.x + r; c.y = c.y + g; c.z = c.z + b; c.w = c.w + a;
  color[idx] = c;
}

// shade_miss.wgsl:45-57 for a ray that left the scene inside a traversal
// kernel: add its contribution now, or (closest hit, `defer`) park it in the
// ray's hit record {r, g, b, pixel} for the compaction of this trace to add
// once the previous bounce's shadow rays are done with the pixel.
template <bool ANY>
__device__ __forceinline__ void fused_miss(float4* color, uint32_t npix, uint4* hrec, uint32_t j, uint32_t idx,
                                           float r, float g, float b, int defer, uint32_t* err) {
  if (!ANY && defer) hrec[j] = make_uint4(__float_as_uint(r), __float_as_uint(g), __float_as_uint(b), idx);
  else add_color(color, npix, idx, r, g, b, 1.0f, err);
}

// trace.wgsl:191-213 main (closest hit) and trace_shadow.wgsl:192-207 main (any
// hit).  Warps claim 32 consecutive queue slots at a time; the outcome bit of
// every slot goes to flags[slot / 32].  FUSED: a ray that reaches the
// environment adds its shade_miss.wgsl contribution directly (the miss queue
// is not materialised); otherwise the compaction kernel builds the miss queue.
template <bool ANY, bool FUSED, bool COUNT>
__global__ void __launch_bounds__(TRACE_THREADS) k_trace(SceneDev sc, EnvDev env, Counters* __restrict__ ctr,
                                                          const uint32_t* __restrict__ countp, RayQ R,
                                                          uint4* __restrict__ hrec, uint32_t* __restrict__ flags,
                                                          float4* __restrict__ color, uint32_t npix,
                                                          uint32_t* __restrict__ ticket) {
  __shared__ int sstack[STACK_SMEM][TRACE_THREADS];
  const uint32_t n = *countp;
  const int lane = threadIdx.x & 31;
  const float theta = ctr->env_theta;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    atomicAdd(&ctr->rays_traced, (unsigned long long)n);
    if (COUNT) atomicAdd(&ctr->stat[ANY ? 5 : 4], (unsigned long long)n);
  }
  uint32_t nhit = 0;
  uint32_t nfetch = 0, ntest = 0;
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(ticket, 32u);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= n) break;
    const uint32_t j = base + lane;
    bool hit = false;
    if (j < n) {
      const float4 o = R.o[j], d = R.d[j];
      float bt;
      int bi;
      uint32_t bb;
      traverse<ANY, COUNT>(sc, o.x, o.y, o.z, d.x, d.y, d.z, bt, bi, bb, sstack, &ctr->err, nfetch, ntest);
      hit = bi != -1;
      if (hit && !ANY) hrec[j] = make_uint4(__float_as_uint(bt), (uint32_t)bi, bb, 0u);
      if (!hit && FUSED) {
        const float4 tp = R.t[j];
        const V3 e = env_color(env, theta, v3(d.x, d.y, d.z));
        add_color(color, npix, __float_as_uint(tp.w) & 0x0fffffffu, e.x * tp.x, e.y * tp.y, e.z * tp.z, 1.0f,
                  &ctr->err);
      }
    }
    const uint32_t m = __ballot_sync(0xffffffffu, hit);
    if (lane == 0) flags[base >> 5] = m;
    if (COUNT && lane == 0) nhit += (uint32_t)__popc(m);
  }
  if (COUNT) {
    atomicAdd(&ctr->stat[ANY ? 2 : 0], (unsigned long long)nfetch);
    atomicAdd(&ctr->stat[ANY ? 3 : 1], (unsigned long long)ntest);
    if (lane == 0) atomicAdd(&ctr->stat[ANY ? 7 : 6], (unsigned long long)nhit);
  }
}

// Persistent variant of the same two entry points.  Each lane owns one ray at a
// time; when at least REFILL_MIN lanes of a warp are idle (or no lane has work)
// they claim new queue slots together with one atomic, so a warp no longer
// waits for the slowest of a fixed group of 32 rays.  The loop is split into an
// inner-node loop and a leaf loop (while-while).  There is no speculation: a
// leaf is intersected as soon as the ray reaches it, so each ray visits the
// same nodes in the same order as trace.wgsl's loop and gets the same hit.
// Hit bits are set with atomicOr in a flag array zeroed before the launch.
#ifndef PK_REFILL_MIN
#define PK_REFILL_MIN 16
#endif
constexpr int REFILL_MIN = PK_REFILL_MIN;

// Traversal stack entries per lane kept in shared memory (the rest of the 64
// in local memory).  Shared memory and L1 share one array per SM, so the
// shared stack of 10 resident blocks (DYN_SMEM * 128 * 4 bytes each) is taken
// from the cache that serves the node records.
// (1080p: 32 entries 3425-3457 Mrays/s, 24: 3447-3449, 16: 3532-3562, 12:
// 3541-3546, 8: 3552-3572, 4: 3511-3523).  The driver's own carveout for the
// resulting shared memory was kept: asking for 25% gave 3547-3556, 50%
// 3495-3514, and 0% (all L1) cut the resident blocks: 975.
// (with the concurrent-work grids: 4 entries 3826-3867, 8 3905-3971, 12
// 3870-3980, 16 3908-3972 in paired runs: 8 kept)
#ifndef PK_DYN_SMEM
#define PK_DYN_SMEM 8
#endif
constexpr int DYN_SMEM = PK_DYN_SMEM;
constexpr int DYN_LOCAL = 64 - DYN_SMEM;

// Any-hit rays report only whether some triangle is hit, and the set of leaves
// a ray can reach (every box on the path from the root hit) does not depend
// on the visiting order, so the any-hit kernel could postpone leaves (Aila &
// Laine, "Understanding the Efficiency of Ray Traversal on GPUs", HPG 2009,
// speculative while-while): a lane that reaches a leaf keeps it and goes on
// popping inner nodes until every active lane of the warp holds a leaf.
// Closest-hit rays cannot: trace.wgsl culls a child box against the best
// distance found so far and its snorm16 boxes are truncated inward, so a hit
// can lie outside its leaf's box, and testing a leaf later changes which boxes
// are culled and so, on rare rays, the hit.  Measured on the 1080p benchmark
// (paired runs, same call), postponing was slower: 2971-2976 Mrays/s against
// 3000-3002 without (the any-hit share of the frame rose from 0.288 to 0.304:
// with about 2 leaves per shadow ray the extra inner steps cost more than the
// coherent leaf tests save), and it was removed.  So was a bound on the
// leaves a lane tests before the warp meets again (no gain).
// Inner-node steps a lane takes before the warp meets again at the top of the
// loop (0: until it reaches a leaf).  Lanes whose rays need many steps no
// longer hold the warp while the others wait in the leaf loop or idle for a
// refill.  Measured at 1080p, Mrays/s: unbounded 3137-3140; 1 step
// 2749-2754, 2: 3082, 3: 3171-3190, 4: 3288-3342, 6: 3281-3294, 8:
// 3365-3418, 12: 3345-3349, 16: 3248-3267, 24: 3165-3167.  PK_ANY_BUDGET
// is the any-hit kernel's (default: the same; 0, 4, 12 and 16 measured within
// the noise of 8: 3702-3745 Mrays/s).  Measured again with the concurrent-work
// grids: 8 3899-3928, 6 3736-3752, 12 3877-3885; refill threshold 16
// 3899-3928, 8 3898-3933, 12 3903-3962, 20 3868-3880.
#ifndef PK_INNER_BUDGET
#define PK_INNER_BUDGET 8
#endif
#ifndef PK_ANY_BUDGET
#define PK_ANY_BUDGET PK_INNER_BUDGET
#endif
constexpr int INNER_BUDGET = PK_INNER_BUDGET;
// Unroll of the leaf loop (the compiler then issues the next triangle's loads
// early).  1080p, three paired runs: unrolled by 4 3753-3769 Mrays/s and a
// 0.357-0.359 ms closest-hit launch, not unrolled 3727-3747 and 0.364-0.366
// ms, by 2 3726-3734, by 8 3663-3673.
#ifndef PK_LEAF_UNROLL
#define PK_LEAF_UNROLL 4
#endif
constexpr int LEAF_UNROLL = PK_LEAF_UNROLL;

constexpr int ANY_BUDGET = PK_ANY_BUDGET;

// Box test of the exact binary records: like box_hit, with the far distance
// widened by WIDE_SLACK (relative) so that rounding never drops a box.
__device__ __forceinline__ float box_hit_exact(float xa, float xb, float ya, float yb, float za, float zb, float ox,
                                               float oy, float oz, float ix, float iy, float iz) {
  const float t1x = (xa - ox) * ix, t2x = (xb - ox) * ix;
  const float t1y = (ya - oy) * iy, t2y = (yb - oy) * iy;
  const float t1z = (za - oz) * iz, t2z = (zb - oz) * iz;
  const float tmax = fminf(fminf(fmaxf(t1x, t2x), fmaxf(t1y, t2y)), fmaxf(t1z, t2z));
  const float tmin = fmaxf(fmaxf(fminf(t1x, t2x), fminf(t1y, t2y)), fminf(t1z, t2z));
  const float tmax_s = tmax + fabsf(tmax) * WIDE_SLACK;
  return (tmax_s >= tmin && tmax_s >= 0.0f) ? tmin : MAX_T;
}
__device__ __forceinline__ void inner_children_exact(const SceneDev& sc, int cur, float ox, float oy, float oz,
                                                     float ix, float iy, float iz, float& lh, float& rh, int& cl,
                                                     int& cr) {
  const float4* rec = sc.inner + 4 * (size_t)cur;
  const float4 a = __ldg(rec), b = __ldg(rec + 1), c4 = __ldg(rec + 2);
  const int4 ch = __ldg(reinterpret_cast<const int4*>(rec) + 3);
  lh = box_hit_exact(a.x, a.y, a.z, a.w, b.x, b.y, ox, oy, oz, ix, iy, iz);
  rh = box_hit_exact(b.z, b.w, c4.x, c4.y, c4.z, c4.w, ox, oy, oz, ix, iy, iz);
  cl = ch.x;
  cr = ch.y;
}

// 10 resident blocks per SM (<= 48 registers): with several frames in
// flight this beats the unconstrained 55 registers (2607-2611 vs 2579-2581
// Mrays/s at 1080p, paired runs) and 12 blocks (2494).
// (9 blocks 3721-3728 Mrays/s, 11: 3669-3700, 10: 3738-3762)
#ifndef PK_DYN_MINBLOCKS
#define PK_DYN_MINBLOCKS 10
#endif
template <bool ANY, bool FUSED, bool COUNT, bool EXACT>
__global__ void __launch_bounds__(TRACE_THREADS, PK_DYN_MINBLOCKS) k_trace_dyn(SceneDev sc, EnvDev env, Counters* __restrict__ ctr,
                                                              const uint32_t* __restrict__ countp, RayQ R,
                                                              uint4* __restrict__ hrec, uint32_t* __restrict__ flags,
                                                              float4* __restrict__ color, uint32_t npix,
                                                              uint32_t* __restrict__ ticket, int defer) {
  __shared__ int sstack[DYN_SMEM][TRACE_THREADS];
  int lstack[DYN_LOCAL];
  const uint32_t n = *countp;
  const int lane = threadIdx.x & 31;
  const int tid = threadIdx.x;
  const uint32_t ltmask = (1u << lane) - 1u;
  const float theta = ctr->env_theta;
  const float eps = ANY ? 1e-7f : 1e-8f;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    atomicAdd(&ctr->rays_traced, (unsigned long long)n);
    if (COUNT) atomicAdd(&ctr->stat[ANY ? 5 : 4], (unsigned long long)n);
  }
  uint32_t nfetch = 0, ntest = 0, nhit = 0;
  uint32_t j = 0;
  bool have = false, exhausted = false;
  float ox = 0.f, oy = 0.f, oz = 0.f, dx = 0.f, dy = 0.f, dz = 0.f, ix = 0.f, iy = 0.f, iz = 0.f;
  WtRay wr{};  // EXACT: the watertight test's per-ray set-up
  float best_t = MAX_T;
  int best_i = -1;
  uint32_t best_b = 0u;
  int sp = 0, cur = 0;
  for (;;) {
    const uint32_t idle = __ballot_sync(0xffffffffu, !have && !exhausted);
    const uint32_t busy = __ballot_sync(0xffffffffu, have);
    if (idle && (__popc(idle) >= REFILL_MIN || busy == 0u)) {
      const int leader = __ffs(idle) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(ticket, (uint32_t)__popc(idle));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (!have && !exhausted) {
        j = base + (uint32_t)__popc(idle & ltmask);
        if (j < n) {
          const float4 o = __ldcs(R.o + j), d = __ldcs(R.d + j);  // read once
          ox = o.x; oy = o.y; oz = o.z;
          dx = d.x; dy = d.y; dz = d.z;
          if (EXACT) {
            ix = wide_inverse(dx); iy = wide_inverse(dy); iz = wide_inverse(dz);
            wr = wt_setup(ox, oy, oz, dx, dy, dz);
          } else {
            ix = 1.0f / dx; iy = 1.0f / dy; iz = 1.0f / dz;
          }
          best_t = MAX_T; best_i = -1; best_b = 0u;
          sp = 0;
          cur = sc.root;
          have = true;
        } else {
          exhausted = true;
        }
      }
    }
    if (!__any_sync(0xffffffffu, have)) break;
    if (!have) continue;
    bool fin = false;
    // inner nodes (at most INNER_BUDGET steps before the warp meets again at
    // the top of the loop, when the budget is not 0)
    constexpr int BUDGET = ANY ? ANY_BUDGET : INNER_BUDGET;
    int budget = BUDGET;
    while (cur >= 0 && (BUDGET == 0 || budget-- > 0)) {
      if (COUNT) nfetch += 3;
      float lh, rh;
      int cl, cr;
      bool lok, rok;
      if (EXACT) {
        inner_children_exact(sc, cur, ox, oy, oz, ix, iy, iz, lh, rh, cl, cr);
        const float lim = best_t + best_t * WIDE_SLACK;
        lok = lh < MAX_T && lh <= lim;
        rok = rh < MAX_T && rh <= lim;
      } else {
        inner_children(sc, cur, ox, oy, oz, ix, iy, iz, lh, rh, cl, cr);
        lok = lh < best_t;
        rok = rh < best_t;
      }
      if (lok && rok) {
        int nearc, farc;
        if (lh > rh) { nearc = cr; farc = cl; } else { nearc = cl; farc = cr; }
        if (sp < DYN_SMEM) sstack[sp][tid] = farc;
        else if (sp < DYN_SMEM + DYN_LOCAL) lstack[sp - DYN_SMEM] = farc;
        else { atomicOr(&ctr->err, ERR_STACK); fin = true; break; }
        ++sp;
        cur = nearc;
        continue;
      }
      if (lok) { cur = cl; continue; }
      if (rok) { cur = cr; continue; }
      if (sp == 0) { fin = true; break; }
      --sp;
      cur = sp < DYN_SMEM ? sstack[sp][tid] : lstack[sp - DYN_SMEM];
    }
    // leaves
    while (!fin && cur < 0) {
      if (COUNT) nfetch += 1;
      const uint32_t word = (uint32_t)cur & 0x7fffffffu;
      const int size = (int)(word >> 24);
      const int base = (int)(word & 0x00ffffffu);
#if PK_LEAF_UNROLL
#pragma unroll LEAF_UNROLL
#endif
      for (int i = 0; i < size; i++) {
        if (COUNT) ntest += 1;
        if (EXACT) {  // the watertight test of form (1), min (t, slot)
          float t, u, v;
          uint32_t slot;
          if (wt_test(sc.wtris, (uint32_t)(base + i), wr, eps, t, u, v, slot) &&
              (t < best_t || (t == best_t && (int)slot < best_i))) {
            best_t = t;
            best_i = (int)slot;
            best_b = pack_unorm16(u) | (pack_unorm16(v) << 16);
          }
          if (ANY && !COUNT && best_i != -1) break;
          continue;
        }
        float res, u, v;
        if (!mt_test(sc, base + i, ox, oy, oz, dx, dy, dz, eps, res, u, v)) continue;
        if (res < best_t) {
          best_t = res;
          best_i = base + i;
          best_b = pack_unorm16(u) | (pack_unorm16(v) << 16);
        }
        // any hit only reports whether some triangle is hit: stop at the first
        // (the counting variant tests the whole leaf, as trace_shadow.wgsl does)
        if (ANY && !COUNT && best_i != -1) break;
      }
      if (ANY && best_i != -1) { fin = true; break; }
      if (sp == 0) { fin = true; break; }
      --sp;
      cur = sp < DYN_SMEM ? sstack[sp][tid] : lstack[sp - DYN_SMEM];
    }
    if (fin) {
      const bool hit = best_i != -1;
      if (hit) {
        if (!ANY) __stcs(hrec + j, make_uint4(__float_as_uint(best_t), (uint32_t)best_i, best_b, 0u));
        if (!(ANY && FUSED)) atomicOr(flags + (j >> 5), 1u << (j & 31u));
        if (COUNT) nhit += 1;
      } else if (FUSED) {
        const float4 tpv = __ldcs(R.t + j);
        const V3 e = env_color(env, theta, v3(dx, dy, dz));
        fused_miss<ANY>(color, npix, hrec, j, __float_as_uint(tpv.w) & 0x0fffffffu, e.x * tpv.x, e.y * tpv.y,
                        e.z * tpv.z, defer, &ctr->err);
      }
      have = false;
    }
  }
  if (COUNT) {
    atomicAdd(&ctr->stat[ANY ? 2 : 0], (unsigned long long)nfetch);
    atomicAdd(&ctr->stat[ANY ? 3 : 1], (unsigned long long)ntest);
    atomicAdd(&ctr->stat[ANY ? 7 : 6], (unsigned long long)nhit);
  }
}

// =====================================================================
// Persistent traversal of the compressed 8-wide BVH (pk_wide.h), after
// Ylitie, Karras & Laine (HPG 2017): the stack holds groups, not nodes.  A
// node group {child_base, hits << 24 | imask} stands for the hit internal
// children of one node, visited in the ray's octant order (lowest bit
// first); a triangle group {tri_base, triangle bits} for its hit leaf
// triangles.  Each step visits one child of the current node group (pushing
// the rest of the group) and then tests the triangle group in hand.  Ylitie
// et al.'s triangle postponing (while fewer than p lanes of the warp have
// triangles and this lane still has nodes to visit, push the triangle group
// and test it later) cost more than it saved on the 1080p benchmark (p = 4:
// 2669 Mrays/s, p = 8: 2569, without: 2939) and was removed.  Lanes take new rays as
// in k_trace_dyn.  Unlike the binary traversal, letting a lane visit several
// nodes in a row before the warp meets again did not pay (1080p: one visit
// 3102-3108 Mrays/s, up to two 2893-2900, up to four 1753-1767), and the
// refill threshold of the binary traversal (16 idle lanes) is also best here
// (1080p: 4 lanes 3275-3285, 8: 3305-3312, 16: 3357-3360, 24: 3315).
// Prefetching the next node's record into L1 before the triangle tests
// measured slightly slower (3320-3334 against 3347), and so did unrolling the
// triangle loop (by 2: 3308-3326, by 4: 3171-3193, against 3347-3355).
// Closest hit = min (t, slot) over accepted triangles, any hit = the first
// accepted triangle: the answer does not depend on the visiting order.
// =====================================================================
// (1080p, wide traversal: 16 entries 3118-3137 Mrays/s, 8: 3155-3168, 4:
// 3156-3172; with the concurrent-work grids 16: 3377-3394, 8: 3400-3412, 4:
// 3432-3451)
#ifndef PK_CW_SMEM
#define PK_CW_SMEM 4
#endif
constexpr int CW_STACK_SMEM = PK_CW_SMEM;       // group entries per thread in shared memory
constexpr int CW_STACK_LOCAL = 32 - PK_CW_SMEM;  // overflow entries in local memory

__device__ __forceinline__ bool cw_push(uint2 (*sstack)[TRACE_THREADS], uint2* lstack, int tid, int& sp, uint2 g) {
  if (sp < CW_STACK_SMEM) sstack[sp][tid] = g;
  else if (sp < CW_STACK_SMEM + CW_STACK_LOCAL) lstack[sp - CW_STACK_SMEM] = g;
  else return false;
  ++sp;
  return true;
}
__device__ __forceinline__ uint2 cw_pop(uint2 (*sstack)[TRACE_THREADS], const uint2* lstack, int tid, int& sp) {
  --sp;
  return sp < CW_STACK_SMEM ? sstack[sp][tid] : lstack[sp - CW_STACK_SMEM];
}

// 8 resident blocks per SM (64 registers): 2982 Mrays/s on the 1080p
// benchmark against 2945 at 10 blocks and 2744 at 12 (same call).
#ifndef PK_CW_MINBLOCKS
#define PK_CW_MINBLOCKS 8
#endif
template <bool ANY, bool FUSED, bool COUNT>
__global__ void __launch_bounds__(TRACE_THREADS, PK_CW_MINBLOCKS) k_trace_cw(SceneDev sc, EnvDev env, Counters* __restrict__ ctr,
                                                             const uint32_t* __restrict__ countp, RayQ R,
                                                             uint4* __restrict__ hrec, uint32_t* __restrict__ flags,
                                                             float4* __restrict__ color, uint32_t npix,
                                                             uint32_t* __restrict__ ticket, int defer) {
  __shared__ uint2 sstack[CW_STACK_SMEM][TRACE_THREADS];
  uint2 lstack[CW_STACK_LOCAL];
  const uint32_t n = *countp;
  const int lane = threadIdx.x & 31;
  const int tid = threadIdx.x;
  const uint32_t ltmask = (1u << lane) - 1u;
  const float theta = ctr->env_theta;
  const float eps = ANY ? 1e-7f : 1e-8f;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    atomicAdd(&ctr->rays_traced, (unsigned long long)n);
    if (COUNT) atomicAdd(&ctr->stat[ANY ? 5 : 4], (unsigned long long)n);
  }
  uint32_t nfetch = 0, ntest = 0, nhit = 0;
  uint32_t j = 0;
  bool have = false, exhausted = false;
  float ox = 0.f, oy = 0.f, oz = 0.f, ix = 0.f, iy = 0.f, iz = 0.f;
  WtRay wr{};
  uint32_t oct = 0;
  float best_t = MAX_T;
  int best_i = -1;
  uint32_t best_b = 0u;
  int sp = 0;
  uint2 G = make_uint2(0u, 0u), T = make_uint2(0u, 0u);
  for (;;) {
    const uint32_t idle = __ballot_sync(0xffffffffu, !have && !exhausted);
    const uint32_t busy = __ballot_sync(0xffffffffu, have);
    if (idle && (__popc(idle) >= REFILL_MIN || busy == 0u)) {
      const int leader = __ffs(idle) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(ticket, (uint32_t)__popc(idle));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (!have && !exhausted) {
        j = base + (uint32_t)__popc(idle & ltmask);
        if (j < n) {
          const float4 o = __ldcs(R.o + j), d = __ldcs(R.d + j);  // read once
          ox = o.x; oy = o.y; oz = o.z;
          ix = wide_inverse(d.x); iy = wide_inverse(d.y); iz = wide_inverse(d.z);
          oct = (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
          wr = wt_setup(o.x, o.y, o.z, d.x, d.y, d.z);
          best_t = MAX_T; best_i = -1; best_b = 0u;
          sp = 0;
          G = make_uint2(0u, (1u << (24u + oct)) | 1u);  // the root: slot 0 of a one-child group
          T = make_uint2(0u, 0u);
          have = true;
        } else {
          exhausted = true;
        }
      }
    }
    if (!__any_sync(0xffffffffu, have)) break;
    if (!have) continue;
    bool fin = false;
    if (G.y > 0x00ffffffu) {  // visit the nearest remaining child of the node group
      const uint32_t bit = (uint32_t)__ffs(G.y >> 24) - 1u;
      const uint32_t slot = bit ^ oct;
      const uint32_t node = G.x + (uint32_t)__popc(G.y & ((1u << slot) - 1u) & 0xffu);
      G.y &= ~(1u << (24u + bit));
      if (G.y > 0x00ffffffu && !cw_push(sstack, lstack, tid, sp, G)) {
        atomicOr(&ctr->err, ERR_STACK);
        fin = true;
      }
      if (COUNT) nfetch += 1;
      uint32_t cb, tb, im, ih, th;
      cw_node(sc.wide, node, ox, oy, oz, ix, iy, iz, oct, best_t, cb, tb, im, ih, th);
      G = ih ? make_uint2(cb, (ih << 24) | im) : make_uint2(0u, 0u);
      T = make_uint2(tb, th);
    }
    while (!fin && T.y != 0u) {
      const uint32_t i = (uint32_t)__ffs(T.y) - 1u;
      T.y &= T.y - 1u;
      if (COUNT) ntest += 1;
      float t, u, v;
      uint32_t slot;
      if (wt_test(sc.wtris, T.x + i, wr, eps, t, u, v, slot) &&
          (t < best_t || (t == best_t && (int)slot < best_i))) {
        best_t = t;
        best_i = (int)slot;
        best_b = pack_unorm16(u) | (pack_unorm16(v) << 16);
        if (ANY && !COUNT) fin = true;  // any hit: the first is enough
      }
    }
    if (!fin) {
      if (ANY && best_i != -1) fin = true;
      else if (G.y <= 0x00ffffffu) {
        if (sp == 0) fin = true;
        else G = cw_pop(sstack, lstack, tid, sp);
      }
    }
    if (fin) {
      const bool hit = best_i != -1;
      if (hit) {
        if (!ANY) __stcs(hrec + j, make_uint4(__float_as_uint(best_t), (uint32_t)best_i, best_b, 0u));
        if (!(ANY && FUSED)) atomicOr(flags + (j >> 5), 1u << (j & 31u));
        if (COUNT) nhit += 1;
      } else if (FUSED) {
        const float4 tpv = __ldcs(R.t + j), d = __ldcs(R.d + j);
        const V3 e = env_color(env, theta, v3(d.x, d.y, d.z));
        fused_miss<ANY>(color, npix, hrec, j, __float_as_uint(tpv.w) & 0x0fffffffu, e.x * tpv.x, e.y * tpv.y,
                        e.z * tpv.z, defer, &ctr->err);
      }
      have = false;
    }
  }
  if (COUNT) {
    atomicAdd(&ctr->stat[ANY ? 2 : 0], (unsigned long long)nfetch);
    atomicAdd(&ctr->stat[ANY ? 3 : 1], (unsigned long long)ntest);
    atomicAdd(&ctr->stat[ANY ? 7 : 6], (unsigned long long)nhit);
  }
}

// =====================================================================
// Stable compaction of trace / shadow outcomes.
//   MODE 0: closest-hit flags -> hit list (+ miss queue when MISSQ; + the
//           contributions of misses parked in miss_rec when given)
//   MODE 1: any-hit flags     -> unoccluded shadow rays appended to the miss queue
// =====================================================================
// (1080p: 256 threads 3734-3748 Mrays/s, 512: 3738-3760, 1024: 3698-3711)
#ifndef PK_COMPACT_THREADS
#define PK_COMPACT_THREADS 256
#endif
constexpr int COMPACT_THREADS = PK_COMPACT_THREADS;
// The compaction and shade kernels take their tile's prefix with a whole warp
// (lookback2_warp) rather than one thread (lookback2): 3137-3140 against
// 3020-3026 Mrays/s at 1080p when it was introduced.

template <int MODE, bool MISSQ>
__global__ void __launch_bounds__(COMPACT_THREADS) k_compact(Counters* __restrict__ ctr,
                                                              const uint32_t* __restrict__ flags,
                                                              uint32_t* __restrict__ hit_list, RayQ src, RayQ M,
                                                              uint32_t miss_capacity, uint32_t* __restrict__ ticket,
                                                              unsigned long long* __restrict__ tiles,
                                                              const uint4* __restrict__ miss_rec,
                                                              float4* __restrict__ color, uint32_t npix) {
  __shared__ uint32_t s_tile;
  __shared__ uint32_t s_warp[COMPACT_THREADS / 32 + 1][2];
  __shared__ unsigned long long s_excl;
  const uint32_t n = MODE == 0 ? ctr->num_rays : ctr->num_shadow;
  const uint32_t miss_base = MODE == 0 ? 0u : ctr->num_misses;
  const uint32_t nwords = (n + 31) >> 5;
  const uint32_t ntiles = (nwords + COMPACT_THREADS - 1) / COMPACT_THREADS;
  if (ntiles == 0) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      if (MODE == 0) { ctr->num_hits = 0; if (MISSQ) ctr->num_misses = 0; }
    }
    return;
  }
  for (;;) {
    if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= ntiles) break;
    const uint32_t w = tile * COMPACT_THREADS + threadIdx.x;
    uint32_t valid = 0u, hm = 0u;
    if (w < nwords) {
      valid = (w == nwords - 1 && (n & 31u)) ? ((1u << (n & 31u)) - 1u) : 0xffffffffu;
      hm = flags[w] & valid;
    }
    const uint32_t mm = valid & ~hm;
    // MODE 0 counts hits (a) and misses (b); MODE 1 counts unoccluded rays (b).
    const uint32_t ca = MODE == 0 ? (uint32_t)__popc(hm) : 0u;
    const uint32_t cb = (MODE == 1 || MISSQ) ? (uint32_t)__popc(mm) : 0u;
    uint32_t ea, eb, ta, tb;
    block_scan2<COMPACT_THREADS / 32>(ca, cb, ea, eb, ta, tb, s_warp);
    if (threadIdx.x < 32) {
      const unsigned long long e = lookback2_warp(tiles, tile, pack2(ta, tb), &ctr->err);
      if (threadIdx.x == 0) s_excl = e;
    }
    __syncthreads();
    const uint32_t pa = unpack_a(s_excl) + ea;
    uint32_t pb = unpack_b(s_excl) + eb;
    if (MODE == 0) {
      uint32_t bits = hm, k = pa;
      while (bits) {
        const int b = __ffs(bits) - 1;
        bits &= bits - 1u;
        hit_list[k++] = w * 32u + (uint32_t)b;
      }
    }
    if (MODE == 0 && !MISSQ && miss_rec) {  // misses parked by a deferring closest-hit trace
      uint32_t bits = mm;
      while (bits) {
        const int b = __ffs(bits) - 1;
        bits &= bits - 1u;
        const uint4 m = miss_rec[w * 32u + (uint32_t)b];
        add_color(color, npix, m.w, __uint_as_float(m.x), __uint_as_float(m.y), __uint_as_float(m.z), 1.0f,
                  &ctr->err);
      }
    }
    if (MODE == 1 || MISSQ) {
      uint32_t bits = mm, k = miss_base + pb;
      while (bits) {
        const int b = __ffs(bits) - 1;
        bits &= bits - 1u;
        const uint32_t j = w * 32u + (uint32_t)b;
        if (k < miss_capacity) {
          M.o[k] = src.o[j];
          M.d[k] = src.d[j];
          M.t[k] = src.t[j];
        } else {
          atomicOr(&ctr->err, ERR_QUEUE);
        }
        ++k;
      }
    }
    if (tile == ntiles - 1 && threadIdx.x == 0) {
      const uint32_t tot_a = unpack_a(s_excl) + ta, tot_b = unpack_b(s_excl) + tb;
      if (MODE == 0) {
        ctr->num_hits = tot_a;
        if (MISSQ) ctr->num_misses = tot_b;
      } else {
        ctr->num_misses = miss_base + tot_b;
      }
    }
    __syncthreads();
  }
}

// k_shade: shade_hit.wgsl main (:407-483).  Tiles of SHADE_THREADS hits are
// claimed in order; bounce and shadow rays are written at their stable ranks
// found by a block scan plus decoupled look-back, so slot order equals the
// serial order of the reference.  Occupancy is held at 1536 threads per SM
// (<= 40 registers): more shading warps in flight to cover the attribute,
// texel and env gathers; some registers spill to L1.  Block size at that
// occupancy, 1080p frame, two runs each in one call: 64 threads x 24 blocks
// 3334-3337 Mrays/s, 128 x 12 3519-3526, 256 x 6 3690-3692, 512 x 3
// 3706-3718, 1024 x 1 3514-3551; fewer resident threads at 256 (5 blocks
// 3665-3676, 4 blocks 3638-3639).  Larger tiles mean fewer look-back steps
// per hit (with the concurrent-work grids, 256 x 6 measured 3606-3661
// against 3871-3970 for 512 x 3).  One warp per 32-hit tile with its own look-back and no block
// barrier (bit-identical queues) measured slower again with the warp-wide
// look-back: 3405-3415 against 3718-3759.
#ifndef PK_SHADE_THREADS
#define PK_SHADE_THREADS 512
#endif
constexpr int SHADE_THREADS = PK_SHADE_THREADS;

// shade_hit.wgsl:407-483 for one hit: the hit record of slot `r` (its
// position in the hit list, which seeds the RNG) on ray (o4, d4, t4).
// Returns whether the surface emits (emission contribution in em); eb/es with
// the bounce and shadow rays as in the reference.
__device__ __forceinline__ bool shade_one(const SceneDev& sc, const EnvDev& env, float theta, int32_t samples,
                                          uint32_t r, float4 o4, float4 d4, float4 t4, uint4 hr, V3& em, bool& eb,
                                          float4& bo, float4& bd, float4& bt, bool& es, float4& so, float4& sd,
                                          float4& st) {
  bool emitted = false;
  em = v3(0.0f, 0.0f, 0.0f);
  const V3 ro = v3(o4.x, o4.y, o4.z), rd = v3(d4.x, d4.y, d4.z);
  const float ht = __uint_as_float(hr.x);
  const uint32_t mask = __float_as_uint(t4.w);
  const uint32_t color_idx = mask & 0x0fffffffu;
  const uint32_t ray_type = mask & 0xf0000000u;
  Hash h;
  h.seed = (r * 1973u + color_idx * 9277u + (uint32_t)samples * 26699u) | 1u;
  h.seed = h.next();
  const SI si = surface(sc, ro, rd, ht, (int)hr.y, hr.z);
  if (h.rand() > si.opacity) {
    const V3 ao = add(ro, scale(rd, ht + SHADE_EPS * 40.0f));
    eb = true;
    bo = make_float4(ao.x, ao.y, ao.z, 0.0f);
    bd = d4;
    bt = t4;
  } else if (dot(si.emission, v3(1.0f, 1.0f, 1.0f)) > 0.0f) {
    const float att = fmax_(dot(si.n, matvec(si.b1, si.b2, si.n, si.wo)), 0.0f);
    em = v3(50.0f * si.emission.x * t4.x * att, 50.0f * si.emission.y * t4.y * att,
            50.0f * si.emission.z * t4.z * att);
    emitted = true;
  } else if (ray_type != 0x10000000u) {
    const V3 m = sample_ggx(h, si);
    const float f = mix1(schlick(fmax_(dot(si.wo, m), 0.0f), 1.5f), 1.0f, si.metallic);
    Sample bs;
    V3 bsdf;
    if (h.rand() > f) {
      const float lr = sqrtf(h.rand());
      const float lphi = c::TAU * h.rand();
      const float x = lr * cos_(lphi);
      const float y = lr * sin_(lphi);
      const float z = sqrtf(fmax_(0.0f, 1.0f - x * x - y * y));
      bs.wi = v3(x, y, z);
      bs.pdf = lambert_pdf(bs.wi);
      bsdf = eval_lambert(si, bs);
    } else {
      bs.wi = reflect(neg(si.wo), m);
      bs.pdf = specular_pdf(si, m);
      bsdf = eval_specular(si, bs);
    }
    if (bs.wi.z > 0.0f) {
      const V3 dir = matvec(si.b1, si.b2, si.n, bs.wi);
      const float weight = env.enabled ? power_heuristic(bs.pdf, env_pdf_dir(env, theta, dir)) : 1.0f;
      eb = true;
      bo = make_float4(si.origin.x, si.origin.y, si.origin.z, 0.0f);
      bd = make_float4(dir.x, dir.y, dir.z, 0.0f);
      bt = make_float4(bsdf.x * t4.x * weight, bsdf.y * t4.y * weight, bsdf.z * t4.z * weight, t4.w);
    }
    if (env.enabled) {
      const Sample es_ = sample_env(env, theta, h, si);
      if (dot(es_.wi, m) > 0.0f && es_.wi.z > 0.0f) {
        // createMaterialSampleRay (:339-348)
        const float lw = power_heuristic(es_.pdf, lambert_pdf(es_.wi));
        const V3 el = eval_lambert(si, es_);
        V3 scv = scale(v3((1.0f - f) * el.x, (1.0f - f) * el.y, (1.0f - f) * el.z), lw);
        const V3 hv = normalize(add(si.wo, es_.wi));
        const float sw = power_heuristic(es_.pdf, specular_pdf(si, hv));
        const V3 ev = eval_specular(si, es_);
        scv = add(scv, scale(v3(f * ev.x, f * ev.y, f * ev.z), sw));
        const V3 sdir = matvec(si.b1, si.b2, si.n, es_.wi);
        es = true;
        so = make_float4(si.origin.x, si.origin.y, si.origin.z, 0.0f);
        sd = make_float4(sdir.x, sdir.y, sdir.z, 0.0f);
        st = make_float4(scv.x * t4.x, scv.y * t4.y, scv.z * t4.z, t4.w);
      }
    }
  }
  return emitted;
}

// Resident blocks per SM (at 128 threads, warp-wide look-back, 1080p: 10
// blocks 3342-3359 Mrays/s, 12: 3394-3396, 14: 3392-3407, 16: 3384-3392).
#ifndef PK_SHADE_BLOCKS
#define PK_SHADE_BLOCKS (1536 / SHADE_THREADS)
#endif
__global__ void __launch_bounds__(SHADE_THREADS, PK_SHADE_BLOCKS) k_shade(SceneDev sc, EnvDev env, Counters* __restrict__ ctr,
                                                          const uint32_t* __restrict__ hit_list,
                                                          const uint4* __restrict__ hrec, RayQ Rin, RayQ Rout,
                                                          RayQ S, uint32_t capacity, float4* __restrict__ color,
                                                          uint32_t npix, uint32_t* __restrict__ ticket,
                                                          unsigned long long* __restrict__ tiles) {
  __shared__ uint32_t s_tile;
  __shared__ uint32_t s_warp[SHADE_THREADS / 32 + 1][2];
  __shared__ unsigned long long s_excl;
  const uint32_t nh = ctr->num_hits;
  const int32_t samples = ctr->samples;
  const float theta = ctr->env_theta;
  const uint32_t ntiles = (nh + SHADE_THREADS - 1) / SHADE_THREADS;
  if (ntiles == 0) {
    if (blockIdx.x == 0 && threadIdx.x == 0) { ctr->num_rays = 0; ctr->num_shadow = 0; }
    return;
  }
  for (;;) {
    if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= ntiles) break;
    const uint32_t r = tile * SHADE_THREADS + threadIdx.x;
    bool eb = false, es = false;
    float4 bo, bd, bt, so, sd, st;
    uint32_t j = 0;
    uint4 hr = make_uint4(0u, 0u, 0u, 0u);
    bool valid = r < nh;
    if (valid) {  // hit list, hit records and rays are read once: streaming loads
      j = __ldcs(hit_list + r);
      if (j < capacity) hr = __ldcs(hrec + j);
      if (j >= capacity || hr.y >= sc.n_tris) { atomicOr(&ctr->err, ERR_QUEUE); valid = false; }
    }
    if (valid) {
      const float4 o4 = __ldcs(Rin.o + j), d4 = __ldcs(Rin.d + j), t4 = __ldcs(Rin.t + j);
      V3 em;
      if (shade_one(sc, env, theta, samples, r, o4, d4, t4, hr, em, eb, bo, bd, bt, es, so, sd, st))
        add_color(color, npix, __float_as_uint(t4.w) & 0x0fffffffu, em.x, em.y, em.z, 1.0f, &ctr->err);
    }
    uint32_t ea, es2, ta, tb;
    block_scan2<SHADE_THREADS / 32>(eb ? 1u : 0u, es ? 1u : 0u, ea, es2, ta, tb, s_warp);
    if (threadIdx.x < 32) {
      const unsigned long long e = lookback2_warp(tiles, tile, pack2(ta, tb), &ctr->err);
      if (threadIdx.x == 0) s_excl = e;
    }
    __syncthreads();
    const uint32_t pb = unpack_a(s_excl) + ea, ps = unpack_b(s_excl) + es2;
    if (eb) {
      if (pb < capacity) {  // read once by the next traversal: streaming stores
        __stcs(Rout.o + pb, bo);
        __stcs(Rout.d + pb, bd);
        __stcs(Rout.t + pb, bt);
      }
      else atomicOr(&ctr->err, ERR_QUEUE);
    }
    if (es) {
      if (ps < capacity) {
        __stcs(S.o + ps, so);
        __stcs(S.d + ps, sd);
        __stcs(S.t + ps, st);
      }
      else atomicOr(&ctr->err, ERR_QUEUE);
    }
    if (tile == ntiles - 1 && threadIdx.x == 0) {
      ctr->num_rays = unpack_a(s_excl) + ta;
      ctr->num_shadow = unpack_b(s_excl) + tb;
    }
    __syncthreads();
  }
}

// shade_miss.wgsl:45-57 over the materialised miss queue.
__global__ void __launch_bounds__(128) k_shade_miss(EnvDev env, Counters* __restrict__ ctr, RayQ M,
                                                    float4* __restrict__ color, uint32_t npix) {
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= ctr->num_misses) return;
  const float4 d = M.d[tid], tp = M.t[tid];
  const V3 e = env_color(env, ctr->env_theta, v3(d.x, d.y, d.z));
  add_color(color, npix, __float_as_uint(tp.w) & 0x0fffffffu, e.x * tp.x, e.y * tp.y, e.z * tp.z, 1.0f, &ctr->err);
}

// accumulate.wgsl:20-34 (pixels x < W only; the reference's `>` bound lets
// invocation x == W alias pixel (0, y+1) in a race, which is not reproduced).
__global__ void __launch_bounds__(256) k_accumulate(const Counters* __restrict__ ctr, const float4* __restrict__ color,
                                                    float4* __restrict__ accum, uint32_t npix) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npix) return;
  const float s = (float)ctr->samples, s1 = (float)(ctr->samples + 1);
  const float4 c = color[i];
  float4 a = accum[i];
  a.x = (fmax_(c.x, 0.0f) + a.x * s) / s1;
  a.y = (fmax_(c.y, 0.0f) + a.y * s) / s1;
  a.z = (fmax_(c.z, 0.0f) + a.z * s) / s1;
  a.w = 1.0f;
  accum[i] = a;
}

// Compensated accumulation (precision form, not the reference's running
// mean): Kahan sums of max(c, 0) per pixel; the accumulation buffer receives
// sum / (n + 1) so postprocess and readback see the same mean.
__global__ void __launch_bounds__(256) k_accumulate_kahan(const Counters* __restrict__ ctr,
                                                          const float4* __restrict__ color, float4* __restrict__ sum,
                                                          float4* __restrict__ comp, float4* __restrict__ accum,
                                                          uint32_t npix) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npix) return;
  const int32_t n = ctr->samples;
  const float4 c = color[i];
  float4 sv = n == 0 ? make_float4(0.f, 0.f, 0.f, 0.f) : sum[i];
  float4 cv = n == 0 ? make_float4(0.f, 0.f, 0.f, 0.f) : comp[i];
  const float in[3] = {fmax_(c.x, 0.0f), fmax_(c.y, 0.0f), fmax_(c.z, 0.0f)};
  float* sp = &sv.x;
  float* cp = &cv.x;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const float y = in[k] - cp[k];
    const float t = sp[k] + y;
    cp[k] = (t - sp[k]) - y;
    sp[k] = t;
  }
  sum[i] = sv;
  comp[i] = cv;
  const float s1 = (float)(n + 1);
  accum[i] = make_float4(sv.x / s1, sv.y / s1, sv.z / s1, 1.0f);
}

// postprocess.wgsl:36-99 frag_main as a compute kernel writing a headless buffer.
__device__ __forceinline__ float rrt(float v) {
  const float a = v * (v + 0.0245786f) - 0.000090537f;
  const float b = v * (0.983729f * v + 0.4329510f) + 0.238081f;
  return a / b;
}
__global__ void __launch_bounds__(256) k_postprocess(const float4* __restrict__ accum, float4* __restrict__ out,
                                                     uchar4* __restrict__ out8, uint32_t npix, float exposure,
                                                     float saturation) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npix) return;
  const float4 a4 = accum[i];
  V3 cc = scale(v3(a4.x, a4.y, a4.z), exposure);
  V3 o = vecmat(cc, v3(0.59719f, 0.35458f, 0.04823f), v3(0.07600f, 0.90834f, 0.01566f), v3(0.02840f, 0.13383f, 0.83777f));
  o = v3(rrt(o.x), rrt(o.y), rrt(o.z));
  o = vecmat(o, v3(1.60475f, -0.53108f, -0.07367f), v3(-0.10208f, 1.10813f, -0.00605f), v3(-0.00327f, -0.07276f, 1.07602f));
  o = v3(clamp_(o.x, 0.0f, 1.0f), clamp_(o.y, 0.0f, 1.0f), clamp_(o.z, 0.0f, 1.0f));
  const float oms = 1.0f - saturation;
  const V3 red = add(v3(0.3086f * oms, 0.3086f * oms, 0.3086f * oms), v3(saturation, 0.0f, 0.0f));
  const V3 green = add(v3(0.6094f * oms, 0.6094f * oms, 0.6094f * oms), v3(0.0f, saturation, 0.0f));
  const V3 blue = add(v3(0.0820f * oms, 0.0820f * oms, 0.0820f * oms), v3(0.0f, 0.0f, saturation));
  o = matvec(red, green, blue, o);
  float ch[3] = {o.x, o.y, o.z};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const float cut = ch[k] <= 0.0031308f ? 1.0f : 0.0f;
    const float higher = 1.055f * pow_(ch[k], 1.0f / 2.4f) - 0.055f;
    const float lower = ch[k] * 12.92f;
    ch[k] = higher * (1.0f - cut) + lower * cut;
  }
  out[i] = make_float4(ch[0], ch[1], ch[2], 1.0f);
  uchar4 q;
  q.x = (unsigned char)floorf(clamp_(ch[0], 0.0f, 1.0f) * 255.0f + 0.5f);
  q.y = (unsigned char)floorf(clamp_(ch[1], 0.0f, 1.0f) * 255.0f + 0.5f);
  q.z = (unsigned char)floorf(clamp_(ch[2], 0.0f, 1.0f) * 255.0f + 0.5f);
  q.w = 255;
  out8[i] = q;
}

__global__ void k_end_frame(Counters* ctr) { ctr->samples += 1; }
// The render state a frame starts from (RenderState + CameraPass uniforms).
__global__ void k_set_state(Counters* ctr, CamState* cam, int32_t samples, float theta, CamState cs, int with_cam) {
  ctr->samples = samples;
  ctr->env_theta = theta;
  if (with_cam) *cam = cs;
}

// Elementwise math probes (same numbering as the oracle's or_math).
__global__ void k_math(int fn, const float* __restrict__ x, const float* __restrict__ y, float* __restrict__ out,
                       uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float a = x[i], b = y ? y[i] : 0.0f;
  float r;
  switch (fn) {
    case 0: r = sin_(a); break;
    case 1: r = cos_(a); break;
    case 2: r = tan_(a); break;
    case 3: r = atan2_(a, b); break;
    case 4: r = acos_(a); break;
    case 5: r = exp2_(a); break;
    case 6: r = log2_(a); break;
    case 7: r = pow_(a, b); break;
    case 8: r = snorm16_decode(__float_as_int(a)); break;
    case 9: r = snorm8(__float_as_int(a)); break;     // integer inputs, bit-cast
    case 10: r = unorm8((uint32_t)__float_as_int(a)); break;
    case 11: r = unorm16((uint32_t)__float_as_int(a)); break;
    case 12: r = snorm16(__float_as_int(a)); break;
    default: r = __int_as_float(0x7fc00000);
  }
  out[i] = r;
}

// =====================================================================
// launchers
// =====================================================================
static unsigned grid_for(uint32_t n, unsigned block) { return (unsigned)((n + block - 1) / block); }

uint32_t compact_tiles(uint32_t capacity) { return ((capacity + 31u) / 32u + COMPACT_THREADS - 1) / COMPACT_THREADS; }
uint32_t shade_tiles(uint32_t capacity) { return (capacity + SHADE_THREADS - 1) / SHADE_THREADS; }

// Persistent grids: enough resident blocks to fill every multiprocessor, never
// more blocks than there can be work items.

// =====================================================================
// Form (2): one persistent launch renders many requests (camera, resolution,
// spp, depth, resident scene).  A path is (request, sample, pixel); lanes
// take path ids from a warp-local range that one lane refills with a single
// atomicAdd of chunk * 32 ids, and every lane advances its own path one
// bounce per iteration (trace, shade_hit, the shadow ray, env on a miss), so
// lanes whose paths end early pick up new ones without waiting for the
// warp.  Shading is the drop-in's (shade_one); the slot that seeds its RNG
// is the bounce index, since no hit queue orders the paths here.
// =====================================================================
__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Out-of-line calls for the batch megakernel: inlining both traversals, the
// whole shade_hit body and the camera into one loop overflows the instruction
// cache (ncu: most warps stalled waiting for instructions).  One traversal
// copy serves closest and shadow rays.
template <int BLOCK, int SSTACK>
__device__ __noinline__ void batch_trace(bool any, const SceneDev& sc, float4 o, float4 d, float& t, int& idx,
                                         uint32_t& bary, int (*sstack)[BLOCK], uint32_t* err) {
  uint32_t nf = 0, nt = 0;
  traverse_rt<false, BLOCK, SSTACK>(any, sc, o.x, o.y, o.z, d.x, d.y, d.z, t, idx, bary, sstack, err, nf, nt);
}
__device__ __noinline__ bool batch_shade(const SceneDev& sc, const EnvDev& env, float theta, int32_t samples,
                                         uint32_t r, float4 o4, float4 d4, float4 t4, uint4 hr, V3& em, bool& eb,
                                         float4& bo, float4& bd, float4& bt, bool& es, float4& so, float4& sd,
                                         float4& st) {
  return shade_one(sc, env, theta, samples, r, o4, d4, t4, hr, em, eb, bo, bd, bt, es, so, sd, st);
}
__device__ __noinline__ void batch_camera(const CamState& cam, uint32_t px, uint32_t py, uint32_t W, uint32_t H,
                                          int32_t samples, V3& org, V3& dir) {
  camera_ray(cam, px, py, W, H, samples, org, dir);
}

// 40 resident warps per SM (48 registers, some spilled): the loop stalls
// mostly on instruction fetch and memory latency, and more warps hide both
// (64-request batch with the current shading code: 481 ms at 32 warps, 425 at
// 40, 434 at 48, 489 at 64).
// A lane traces a path's closest-hit ray and then, when shading emitted one,
// its shadow ray within the same step.  (Carrying the shadow ray to the next
// step, so that every lane runs one traversal per step, measured slower:
// 64-request batch 493 against 440 ms.)
template <int BLOCK, int SSTACK>
__global__ void __launch_bounds__(BLOCK, 1280 / BLOCK) k_batch(const BatchScene* __restrict__ scenes, int nscenes,
                                                 const BatchReq* __restrict__ reqs, int nreq,
                                                 unsigned long long total, int chunk,
                                                 unsigned long long* __restrict__ counter,
                                                 const uint32_t* __restrict__ frame, float4* __restrict__ accum,
                                                 unsigned long long n_accum, uint32_t* __restrict__ err,
                                                 unsigned long long* __restrict__ remaining,
                                                 unsigned long long* __restrict__ done_ns) {
  __shared__ int sstack[SSTACK][BLOCK];
  __shared__ unsigned long long s_begin[BATCH_MAX_REQ + 1];
  __shared__ BatchScene s_scene[BATCH_MAX_SCENES];
  for (int i = threadIdx.x; i < nreq; i += BLOCK) s_begin[i] = reqs[i].path_begin;
  if (threadIdx.x == 0) s_begin[nreq] = total;
  for (int i = threadIdx.x; i < nscenes; i += BLOCK) s_scene[i] = scenes[i];
  if (blockIdx.x == 0 && threadIdx.x == 0) done_ns[nreq] = globaltimer_ns();  // launch start
  __syncthreads();
  const uint32_t fr = *frame;
  const int lane = threadIdx.x & 31;
  const uint32_t ltmask = (1u << lane) - 1u;
  unsigned long long wq_next = 0, wq_end = 0;  // warp-uniform
  bool warp_done = false;
  bool have = false;
  int req = 0, bounce = 0;
  uint32_t pix = 0;
  int32_t samples = 0;
  float4 o4 = make_float4(0.f, 0.f, 0.f, 0.f), d4 = o4, t4 = o4;
  for (;;) {
    const uint32_t idle = __ballot_sync(0xffffffffu, !have);
    if (idle && !warp_done) {
      if (wq_next >= wq_end) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(counter, (unsigned long long)chunk * 32ull);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= total) {
          warp_done = true;
        } else {
          wq_next = base;
          wq_end = min(base + (unsigned long long)chunk * 32ull, total);
        }
      }
      if (!warp_done) {
        const unsigned long long avail = wq_end - wq_next;
        const uint32_t rank = __popc(idle & ltmask);
        if (!have && rank < avail) {
          const unsigned long long pid = wq_next + rank;
          int lo = 0, hi = nreq - 1;  // last request with begin <= pid
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s_begin[mid] <= pid) lo = mid; else hi = mid - 1;
          }
          req = lo;
          const BatchReq& q = reqs[req];
          const unsigned long long local = pid - s_begin[req];
          const unsigned long long npix = (unsigned long long)q.W * q.H;
          pix = (uint32_t)(local % npix);
          samples = (int32_t)(fr * q.spp + (uint32_t)(local / npix));
          V3 org, dir;
          batch_camera(q.cam, pix % q.W, pix / q.W, q.W, q.H, samples, org, dir);
          o4 = make_float4(org.x, org.y, org.z, 0.0f);
          d4 = make_float4(dir.x, dir.y, dir.z, 0.0f);
          t4 = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(pix));
          bounce = 0;
          have = true;
        }
        wq_next += min((unsigned long long)__popc(idle), avail);
      }
    }
    if (!__any_sync(0xffffffffu, have)) {
      if (warp_done) break;
      continue;
    }
    bool finished = false;
    if (have) {
      const BatchReq& q = reqs[req];
      const BatchScene& S = s_scene[q.scene];
      const unsigned long long oi = q.out_offset + pix;
      float t;
      int idx;
      uint32_t bary;
      batch_trace<BLOCK, SSTACK>(false, S.sc, o4, d4, t, idx, bary, sstack, err);
      float cr = 0.0f, cg = 0.0f, cb = 0.0f;
      bool next = false;
      if (idx < 0) {
        const V3 e = env_color(S.env, S.theta, v3(d4.x, d4.y, d4.z));
        cr = e.x * t4.x; cg = e.y * t4.y; cb = e.z * t4.z;
      } else {
        bool eb = false, es = false;
        float4 bo, bd, bt, so, sd, st;
        V3 em;
        const uint4 hr = make_uint4(__float_as_uint(t), (uint32_t)idx, bary, 0u);
        if (batch_shade(S.sc, S.env, S.theta, samples, (uint32_t)bounce, o4, d4, t4, hr, em, eb, bo, bd, bt, es, so,
                        sd, st)) {
          cr = em.x; cg = em.y; cb = em.z;
        }
        if (es) {
          float ts;
          int is;
          uint32_t bs;
          batch_trace<BLOCK, SSTACK>(true, S.sc, so, sd, ts, is, bs, sstack, err);
          if (is < 0) {
            const V3 e = env_color(S.env, S.theta, v3(sd.x, sd.y, sd.z));
            cr += e.x * st.x; cg += e.y * st.y; cb += e.z * st.z;
          }
        }
        if (eb && bounce + 1 < (int)q.depth) {
          o4 = bo; d4 = bd; t4 = bt;
          bounce++;
          next = true;
        }
      }
      if (cr != 0.0f || cg != 0.0f || cb != 0.0f) {
        if (oi < n_accum) {
          atomicAdd(&accum[oi].x, cr);
          atomicAdd(&accum[oi].y, cg);
          atomicAdd(&accum[oi].z, cb);
        } else {
          atomicOr(err, ERR_PIXEL);
        }
      }
      finished = !next;
      have = next;
    }
    // per-request completion: one atomic per request per warp step; the lane
    // that retires a request's last path stamps its completion time
    const unsigned peers = __match_any_sync(0xffffffffu, finished ? req : -1);
    if (finished && (int)(threadIdx.x & 31u) == __ffs(peers) - 1) {
      const unsigned long long n = (unsigned long long)__popc(peers);
      if (atomicAdd(&remaining[req], (unsigned long long)(-(long long)n)) == n) done_ns[req] = globaltimer_ns();
    }
  }
}

__global__ void k_batch_next_frame(uint32_t* frame) { *frame += 1u; }

#define PK_BATCH_CONFIGS(X) X(64, 8) X(64, 16) X(64, 32) X(128, 8) X(128, 16) X(128, 32) X(256, 8) X(256, 16) X(256, 32)

bool batch_config_ok(const BatchConfig& c) {
#define PK_B_OK(B, S) if (c.block == B && c.stack == S) return c.chunk >= 1 && c.chunk <= 64;
  PK_BATCH_CONFIGS(PK_B_OK)
#undef PK_B_OK
  return false;
}

int batch_blocks_per_sm(const BatchConfig& c) {
  int n = 0;
#define PK_B_OCC(B, S) \
  if (c.block == B && c.stack == S) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch<B, S>, B, 0);
  PK_BATCH_CONFIGS(PK_B_OCC)
#undef PK_B_OCC
  return n;
}

void launch_batch(cudaStream_t s, const BatchConfig& c, unsigned grid, const BatchScene* scenes, int nscenes,
                  const BatchReq* reqs, int nreq, unsigned long long total, unsigned long long* counter,
                  uint32_t* frame, float4* accum, unsigned long long n_accum, uint32_t* err,
                  unsigned long long* remaining, unsigned long long* done_ns) {
#define PK_B_LAUNCH(B, S)                                                                                          \
  if (c.block == B && c.stack == S) {                                                                              \
    k_batch<B, S><<<grid, B, 0, s>>>(scenes, nscenes, reqs, nreq, total, c.chunk, counter, frame, accum, n_accum, \
                                     err, remaining, done_ns);                                                     \
    return;                                                                                                        \
  }
  PK_BATCH_CONFIGS(PK_B_LAUNCH)
#undef PK_B_LAUNCH
}

void launch_batch_next_frame(cudaStream_t s, uint32_t* frame) { k_batch_next_frame<<<1, 1, 0, s>>>(frame); }

void kernel_grids(int sms, uint32_t capacity, unsigned* trace, unsigned* compact, unsigned* shade,
                  unsigned* trace_wide) {
  int t = 0, c = 0, s = 0, w = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&t, k_trace_dyn<false, true, false, false>, TRACE_THREADS, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&w, k_trace_cw<false, true, false>, TRACE_THREADS, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, k_compact<0, true>, COMPACT_THREADS, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&s, k_shade, SHADE_THREADS, 0);
  const unsigned warps = (capacity + 31u) / 32u;
  *trace = std::max(1u, std::min((unsigned)(sms * std::max(t, 1)), (warps + TRACE_THREADS / 32 - 1) / (TRACE_THREADS / 32)));
  *compact = std::max(1u, std::min((unsigned)(sms * std::max(c, 1)), compact_tiles(capacity)));
  *shade = std::max(1u, std::min((unsigned)(sms * std::max(s, 1)), shade_tiles(capacity)));
  *trace_wide =
      std::max(1u, std::min((unsigned)(sms * std::max(w, 1)), (warps + TRACE_THREADS / 32 - 1) / (TRACE_THREADS / 32)));
}

void launch_camera(const LaunchCtx& L, RayQ R, uint32_t n_threads, int64_t offset) {
  if (n_threads == 0) return;
  k_camera<<<grid_for(n_threads, 128), 128, 0, L.stream>>>(L.cam, L.ctr, R, n_threads, L.capacity, offset);
}

void launch_trace(const LaunchCtx& L, bool any_hit, bool fused, bool count, const uint32_t* countp, RayQ R,
                  uint4* hrec, uint32_t* flags, uint32_t* ticket) {
  const dim3 grid(L.trace_blocks), block(TRACE_THREADS);
  const int defer = (L.defer_miss && fused && !any_hit) ? 1 : 0;
  if (L.trace_mode & TRACE_WIDE) {
    // (concurrent-work grids: 1080p, eight frames in flight, 3399-3423
    // Mrays/s against 3348-3379 with the full grid)
    const dim3 grid(std::max(1u, L.trace_blocks_wide * (any_hit ? L.any_tenths : L.closest_tenths) / 10u));
    const unsigned words = (L.capacity + 31u) / 32u + 1u;
    if (!(any_hit && fused)) cudaMemsetAsync(flags, 0, (size_t)words * 4, L.stream);
#define PK_TRACEW(A, F, C) \
  k_trace_cw<A, F, C><<<grid, block, 0, L.stream>>>(L.scene, L.env, L.ctr, countp, R, hrec, flags, L.color, L.npix, \
                                                      ticket, defer)
    if (!any_hit) {
      if (fused) { if (count) PK_TRACEW(false, true, true); else PK_TRACEW(false, true, false); }
      else { if (count) PK_TRACEW(false, false, true); else PK_TRACEW(false, false, false); }
    } else {
      if (fused) { if (count) PK_TRACEW(true, true, true); else PK_TRACEW(true, true, false); }
      else { if (count) PK_TRACEW(true, false, true); else PK_TRACEW(true, false, false); }
    }
#undef PK_TRACEW
    return;
  }
  if (L.trace_mode & TRACE_PERSISTENT) {
    const dim3 grid(std::max(1u, L.trace_blocks * (any_hit ? L.any_tenths : L.closest_tenths) / 10u));
    const unsigned words = (L.capacity + 31u) / 32u + 1u;
    if (!(any_hit && fused)) cudaMemsetAsync(flags, 0, (size_t)words * 4, L.stream);
#define PK_TRACED(A, F, C)                                                                                         \
  do {                                                                                                             \
    if (L.trace_mode & TRACE_EXACT)                                                                                \
      k_trace_dyn<A, F, C, true><<<grid, block, 0, L.stream>>>(L.scene, L.env, L.ctr, countp, R, hrec, flags,       \
                                                               L.color, L.npix, ticket, defer);                    \
    else                                                                                                           \
      k_trace_dyn<A, F, C, false><<<grid, block, 0, L.stream>>>(L.scene, L.env, L.ctr, countp, R, hrec, flags,      \
                                                                L.color, L.npix, ticket, defer);                   \
  } while (0)
    if (!any_hit) {
      if (fused) { if (count) PK_TRACED(false, true, true); else PK_TRACED(false, true, false); }
      else { if (count) PK_TRACED(false, false, true); else PK_TRACED(false, false, false); }
    } else {
      if (fused) { if (count) PK_TRACED(true, true, true); else PK_TRACED(true, true, false); }
      else { if (count) PK_TRACED(true, false, true); else PK_TRACED(true, false, false); }
    }
#undef PK_TRACED
    return;
  }
#define PK_TRACE(A, F, C) \
  k_trace<A, F, C><<<grid, block, 0, L.stream>>>(L.scene, L.env, L.ctr, countp, R, hrec, flags, L.color, L.npix, ticket)
  if (!any_hit) {
    if (fused) { if (count) PK_TRACE(false, true, true); else PK_TRACE(false, true, false); }
    else { if (count) PK_TRACE(false, false, true); else PK_TRACE(false, false, false); }
  } else {
    if (fused) { if (count) PK_TRACE(true, true, true); else PK_TRACE(true, true, false); }
    else { if (count) PK_TRACE(true, false, true); else PK_TRACE(true, false, false); }
  }
#undef PK_TRACE
}

void launch_compact_trace(const LaunchCtx& L, bool missq, const uint32_t* flags, uint32_t* hit_list, RayQ src,
                          RayQ M, uint32_t* ticket, unsigned long long* tiles, const uint4* miss_rec) {
  const unsigned grid = std::max(1u, L.compact_blocks * L.compact_tenths / 10u);
  if (missq)
    k_compact<0, true><<<grid, COMPACT_THREADS, 0, L.stream>>>(L.ctr, flags, hit_list, src, M, L.miss_capacity,
                                                                ticket, tiles, nullptr, L.color, L.npix);
  else
    k_compact<0, false><<<grid, COMPACT_THREADS, 0, L.stream>>>(L.ctr, flags, hit_list, src, M, L.miss_capacity,
                                                                 ticket, tiles, miss_rec, L.color, L.npix);
}

void launch_compact_shadow(const LaunchCtx& L, const uint32_t* flags, RayQ S, RayQ M, uint32_t* ticket,
                           unsigned long long* tiles) {
  k_compact<1, true><<<L.compact_blocks, COMPACT_THREADS, 0, L.stream>>>(L.ctr, flags, nullptr, S, M,
                                                                           L.miss_capacity, ticket, tiles, nullptr,
                                                                           L.color, L.npix);
}

void launch_shade(const LaunchCtx& L, const uint32_t* hit_list, const uint4* hrec, RayQ Rin, RayQ Rout, RayQ S,
                  uint32_t* ticket, unsigned long long* tiles) {
  k_shade<<<std::max(1u, L.shade_blocks * L.shade_tenths / 10u), SHADE_THREADS, 0, L.stream>>>(L.scene, L.env, L.ctr, hit_list, hrec, Rin, Rout, S,
                                                          L.capacity, L.color, L.npix, ticket, tiles);
}

void launch_shade_miss(const LaunchCtx& L, RayQ M) {
  k_shade_miss<<<grid_for(L.miss_capacity, 128), 128, 0, L.stream>>>(L.env, L.ctr, M, L.color, L.npix);
}

void launch_accumulate(const LaunchCtx& L) {
  if (L.accum_sum)
    k_accumulate_kahan<<<grid_for(L.npix, 256), 256, 0, L.stream>>>(L.ctr, L.color, L.accum_sum, L.accum_comp,
                                                                     L.accum, L.npix);
  else
    k_accumulate<<<grid_for(L.npix, 256), 256, 0, L.stream>>>(L.ctr, L.color, L.accum, L.npix);
}

void launch_postprocess(const LaunchCtx& L, float exposure, float saturation) {
  k_postprocess<<<grid_for(L.npix, 256), 256, 0, L.stream>>>(L.accum, L.display, L.display8, L.npix, exposure,
                                                             saturation);
}

void launch_end_frame(const LaunchCtx& L) { k_end_frame<<<1, 1, 0, L.stream>>>(L.ctr); }
void launch_set_state(cudaStream_t s, Counters* ctr, CamState* cam, int32_t samples, float theta, const CamState& cs,
                      bool with_cam) {
  k_set_state<<<1, 1, 0, s>>>(ctr, cam, samples, theta, cs, with_cam ? 1 : 0);
}

void launch_math(cudaStream_t s, int fn, const float* x, const float* y, float* out, uint32_t n) {
  if (n == 0) return;
  k_math<<<grid_for(n, 256), 256, 0, s>>>(fn, x, y, out, n);
}

}  // namespace pk
