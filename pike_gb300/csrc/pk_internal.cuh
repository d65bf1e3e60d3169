// pk_internal.cuh -- device data layout and shared device helpers of libpike.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "pk_math.cuh"

namespace pk {

// ---- error bits reported through pk_ctx status --------------------------------
enum : uint32_t {
  ERR_STACK = 1u,      // traversal stack overflow (ray result incomplete)
  ERR_LOOKBACK = 2u,   // decoupled look-back gave up waiting (bounded spin)
  ERR_QUEUE = 4u,      // a queue write would exceed its capacity
  ERR_PIXEL = 8u,      // a colour write addressed a pixel outside the image
  ERR_BVH = 16u,       // BVH build: degenerate node / leaf too large
};

// Work-counter slots in Counters::work (reset before each launch that uses them).
enum : int { W_TRACE = 0, W_TILE = 1, W_SHADE = 2, W_AUX = 3 };

// Device-resident RenderState header (camera_pass.js:3-77) plus queue counters.
struct Counters {
  int32_t samples;
  float env_theta;
  uint32_t num_hits, num_misses, num_rays, num_shadow;
  uint32_t err;
  uint32_t pad0;
  uint32_t work[8];
  unsigned long long rays_traced;   // closest-hit + shadow rays, all frames since reset
  unsigned long long trace_launch_rays;
  // traversal counters of the counting kernels: closest {fetch, tests}, shadow
  // {fetch, tests}, rays {closest, shadow}, hits {closest, occluded shadow}
  unsigned long long stat[8];
};

// CameraStateStuct (structs.js:235-249): eye ray, dimsMask = W<<16|H, lens params.
struct CamState {
  float pos[3];
  float dir[3];
  uint32_t dims_mask;
  float fov, focal_depth, aperture, distortion, bokeh;
  uint32_t invocation_offset;
};

// One ray queue in SoA form.  Together the three float4 are the reference's
// 48-byte DeferredRay {origin, dir, throughput}; t.w holds the pixel index bits.
struct RayQ {
  float4* o;
  float4* d;
  float4* t;
};

// Traversal-format BVH (built from the reference's 20-byte nodes without
// changing any box or order): one 64-byte record per inner node holding both
// children's decoded boxes and child codes.  Child code >= 0: inner record
// index; child code < 0: leaf, (code & 0x7fffffff) = reference `triangles`
// word (size << 24 | base).  Triangles are stored leaf-ordered as
// {v0.xyz, e1.x}, {e1.yz, e2.xy}, {e2.z, -, -, -} with e1 = v1 - v0, e2 = v2 - v0.
struct SceneDev {
  const float4* inner;     // 4 float4 per inner record (64-byte format)
  const int4* inner32;     // 2 int4 per inner record (32-byte format); used when not null
  const float4* tris;      // 3 float4 per leaf-ordered triangle
  const int4* tri4;        // leaf-ordered {i0, i1, i2, matId}
  const uint4* attrs;      // per-vertex {tangent, bitangent, normal (snorm8x4), uv (snorm16x2)}
  const int4* mat4;        // per-material atlas layers {diff, metRough, norm, emit}
  const uchar4* layers;    // rgba8 atlas layers, atlas_res x atlas_res each
  int n_layers;
  int atlas_res;
  int root;                // child code of the root
  uint32_t n_tris;         // leaf-ordered triangles
  uint32_t n_verts;        // vertex attributes
  uint32_t n_mats;         // material index entries
  const float4* wide;      // 5 float4 per compressed 8-wide node (pk_wide.h); null unless built
  const float4* wtris;     // form (1) triangle records {v0, v1, v2, slot} (pk_wide.h): the 8-wide
                           // BVH's order (PK_TRACE_WIDE) or the binary leaf order (PK_TRACE_EXACT)
};

struct EnvDev {
  const uchar4* rgbe;      // rgba8 texels, alpha = exponent
  const int2* bins;        // {h0, h1}
  const int2* coords;      // {x, y}, descending radiance
  const float* pdf;        // r32f per texel (the alias table's when `alias` is set)
  int w, h, nb;
  int enabled;             // SAMPLE_ENV_LIGHT
  const uint2* alias;      // PK_ENV_ALIAS: per texel {keep threshold, alias texel}; null: the histogram
};

// ---- decoupled look-back over tiles carrying two 31-bit counts ------------
constexpr unsigned long long TILE_AGG = 1ull << 62;
constexpr unsigned long long TILE_PRE = 2ull << 62;
constexpr unsigned long long TILE_VAL = (1ull << 62) - 1;
constexpr int LOOKBACK_SPIN_LIMIT = 1 << 22;

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long pack2(uint32_t a, uint32_t b) {
  return (unsigned long long)a | ((unsigned long long)b << 31);
}
__device__ __forceinline__ uint32_t unpack_a(unsigned long long v) { return (uint32_t)(v & 0x7fffffffull); }
__device__ __forceinline__ uint32_t unpack_b(unsigned long long v) { return (uint32_t)((v >> 31) & 0x7fffffffull); }

// Exclusive prefix of this tile's two counts over all earlier tiles.  Called by
// one thread.  Tiles are numbered in the order blocks claim them (an atomic
// ticket), so every earlier tile belongs to a block that is already running;
// waits are bounded and report ERR_LOOKBACK instead of hanging.
__device__ __forceinline__ unsigned long long lookback2(unsigned long long* tiles, uint32_t tile,
                                                        unsigned long long agg, uint32_t* err) {
  if (tile == 0) {
    st_release(&tiles[0], TILE_PRE | agg);
    return 0ull;
  }
  st_release(&tiles[tile], TILE_AGG | agg);
  unsigned long long excl = 0;
  int i = (int)tile - 1;
  while (i >= 0) {
    unsigned long long v = ld_acquire(&tiles[i]);
    int spins = 0;
    while ((v & ~TILE_VAL) == 0) {
      if (++spins > LOOKBACK_SPIN_LIMIT) {
        atomicOr(err, ERR_LOOKBACK);
        v = TILE_PRE;
        break;
      }
      __nanosleep(64);
      v = ld_acquire(&tiles[i]);
    }
    excl += v & TILE_VAL;
    if ((v & ~TILE_VAL) == TILE_PRE) break;
    --i;
  }
  st_release(&tiles[tile], TILE_PRE | (excl + agg));
  return excl;
}

// The same prefix computed by one whole warp (every lane calls it; all get
// the result): each round reads a window of 32 earlier tiles at once, waits
// (bounded) until each has published, and sums the aggregates from the tile
// before this one back to the nearest tile holding an inclusive prefix, which
// ends the walk.  A walk over n unfinished predecessors takes n / 32 rounds
// of memory latency instead of n.
__device__ __forceinline__ unsigned long long lookback2_warp(unsigned long long* tiles, uint32_t tile,
                                                             unsigned long long agg, uint32_t* err) {
  const int lane = (int)(threadIdx.x & 31u);
  if (tile == 0) {
    if (lane == 0) st_release(&tiles[0], TILE_PRE | agg);
    return 0ull;
  }
  if (lane == 0) st_release(&tiles[tile], TILE_AGG | agg);
  unsigned long long excl = 0;
  int base = (int)tile - 1;  // the window is tiles base, base - 1, ..., base - 31
  for (;;) {
    const int i = base - lane;
    unsigned long long v = i >= 0 ? ld_acquire(&tiles[i]) : TILE_PRE;  // before tile 0: an empty prefix
    int spins = 0;
    uint32_t pre;
    for (;;) {  // until every tile from this one's predecessor to the nearest prefix has published
      const uint32_t ready = __ballot_sync(0xffffffffu, (v & ~TILE_VAL) != 0);
      pre = __ballot_sync(0xffffffffu, (v & ~TILE_VAL) == TILE_PRE);
      const int last = pre ? __ffs(pre) - 1 : 31;
      const uint32_t need = last == 31 ? 0xffffffffu : ((1u << (last + 1)) - 1u);
      if ((ready & need) == need) break;
      if ((v & ~TILE_VAL) == 0) {
        if (++spins > LOOKBACK_SPIN_LIMIT) {
          atomicOr(err, ERR_LOOKBACK);
          v = TILE_PRE;
        } else {
          __nanosleep(64);
          v = ld_acquire(&tiles[i]);
        }
      }
    }
    const int first = pre ? __ffs(pre) - 1 : 32;  // the nearest inclusive prefix in the window
    unsigned long long c = lane <= first ? (v & TILE_VAL) : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    excl += c;
    if (pre) break;
    base -= 32;
  }
  if (lane == 0) st_release(&tiles[tile], TILE_PRE | (excl + agg));
  return excl;
}

// Block-wide exclusive scan of two per-thread counts (blockDim.x <= 1024,
// multiple of 32).  Returns this thread's exclusive offsets and the block totals.
template <int NWARPS>
__device__ __forceinline__ void block_scan2(uint32_t a, uint32_t b, uint32_t& ea, uint32_t& eb, uint32_t& ta,
                                            uint32_t& tb, uint32_t (*s_warp)[2]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t ia = a, ib = b;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t xa = __shfl_up_sync(0xffffffffu, ia, o);
    uint32_t xb = __shfl_up_sync(0xffffffffu, ib, o);
    if (lane >= o) { ia += xa; ib += xb; }
  }
  if (lane == 31) { s_warp[warp][0] = ia; s_warp[warp][1] = ib; }
  __syncthreads();
  if (warp == 0) {
    uint32_t wa = lane < NWARPS ? s_warp[lane][0] : 0u;
    uint32_t wb = lane < NWARPS ? s_warp[lane][1] : 0u;
    uint32_t sa = wa, sb = wb;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t xa = __shfl_up_sync(0xffffffffu, sa, o);
      uint32_t xb = __shfl_up_sync(0xffffffffu, sb, o);
      if (lane >= o) { sa += xa; sb += xb; }
    }
    if (lane < NWARPS) { s_warp[lane][0] = sa - wa; s_warp[lane][1] = sb - wb; }
    if (lane == NWARPS - 1) { s_warp[NWARPS][0] = sa; s_warp[NWARPS][1] = sb; }
  }
  __syncthreads();
  ea = s_warp[warp][0] + ia - a;
  eb = s_warp[warp][1] + ib - b;
  ta = s_warp[NWARPS][0];
  tb = s_warp[NWARPS][1];
}

}  // namespace pk
