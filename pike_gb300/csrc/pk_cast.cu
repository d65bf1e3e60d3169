// pk_cast.cu -- ray queries against the context's BVH on caller-owned device
// buffers: the GPU counterpart of the reference's CPU Raycaster used for
// autofocus (render/raycaster.js:114-131), with the closest-hit and any-hit
// semantics of trace.wgsl / trace_shadow.wgsl.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "../../include/pike.h"
#include "pk_ctx.h"
#include "pk_internal.cuh"
#include "pk_traverse.cuh"
#include "pk_util.h"

namespace pk {
namespace {

constexpr int CAST_THREADS = TRACE_THREADS;
constexpr int LIST_THREADS = 256;

// Every ray gets a record {t bits, triangle index or 0xffffffff, bary_mask, 0};
// bit j of flags is set when ray j hit.
template <bool ANY>
__global__ void __launch_bounds__(CAST_THREADS) k_cast(SceneDev sc, const float4* __restrict__ o4,
                                                        const float4* __restrict__ d4, uint32_t n,
                                                        uint4* __restrict__ hits4, uint32_t* __restrict__ flags,
                                                        uint32_t* __restrict__ ticket, uint32_t* __restrict__ err) {
  __shared__ int sstack[STACK_SMEM][TRACE_THREADS];
  const int lane = threadIdx.x & 31;
  uint32_t nf = 0, nt = 0;
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(ticket, 32u);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= n) break;
    const uint32_t j = base + lane;
    bool hit = false;
    if (j < n) {
      const float4 o = o4[j], d = d4[j];
      float bt;
      int bi;
      uint32_t bb;
      traverse<ANY, false>(sc, o.x, o.y, o.z, d.x, d.y, d.z, bt, bi, bb, sstack, err, nf, nt);
      hit = bi != -1;
      hits4[j] = make_uint4(__float_as_uint(bt), (uint32_t)bi, bb, 0u);
    }
    const uint32_t m = __ballot_sync(0xffffffffu, hit);
    if (lane == 0) flags[base >> 5] = m;
  }
}

// Stable list of the rays that hit (increasing ray index) and its length.
__global__ void __launch_bounds__(LIST_THREADS) k_hit_list(const uint32_t* __restrict__ flags, uint32_t n,
                                                            uint32_t* __restrict__ list, uint32_t* __restrict__ count,
                                                            uint32_t* __restrict__ ticket,
                                                            unsigned long long* __restrict__ tiles,
                                                            uint32_t* __restrict__ err) {
  __shared__ uint32_t s_tile;
  __shared__ uint32_t s_warp[LIST_THREADS / 32 + 1][2];
  __shared__ unsigned long long s_excl;
  const uint32_t nwords = (n + 31) >> 5;
  const uint32_t ntiles = (nwords + LIST_THREADS - 1) / LIST_THREADS;
  if (ntiles == 0) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *count = 0;
    return;
  }
  for (;;) {
    if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= ntiles) break;
    const uint32_t w = tile * LIST_THREADS + threadIdx.x;
    uint32_t hm = 0u;
    if (w < nwords) {
      const uint32_t valid = (w == nwords - 1 && (n & 31u)) ? ((1u << (n & 31u)) - 1u) : 0xffffffffu;
      hm = flags[w] & valid;
    }
    uint32_t ea, eb, ta, tb;
    block_scan2<LIST_THREADS / 32>((uint32_t)__popc(hm), 0u, ea, eb, ta, tb, s_warp);
    if (threadIdx.x == 0) s_excl = lookback2(tiles, tile, pack2(ta, 0u), err);
    __syncthreads();
    uint32_t k = unpack_a(s_excl) + ea;
    uint32_t bits = hm;
    while (bits) {
      const int b = __ffs(bits) - 1;
      bits &= bits - 1u;
      list[k++] = w * 32u + (uint32_t)b;
    }
    if (tile == ntiles - 1 && threadIdx.x == 0) *count = unpack_a(s_excl) + ta;
    __syncthreads();
  }
}

}  // namespace

// Scratch words the two kernels need for n rays: two tickets, an error word,
// the hit bitmask, and one look-back tile state per LIST_THREADS words.
struct CastScratch {
  uint32_t* tickets;  // [0] trace, [1] list, [2] error flags, [3] unused
  uint32_t* flags;
  unsigned long long* tiles;
};
size_t cast_flag_words(uint32_t n) { return ((size_t)n + 31) / 32; }
size_t cast_tiles(uint32_t n) { return (cast_flag_words(n) + LIST_THREADS - 1) / LIST_THREADS; }

// Enqueue the query on `stream`: zero what must start at zero, then trace and list.
int cast_enqueue(pk_ctx* c, const float4* o4, const float4* d4, uint32_t n, int any_hit, uint4* hits4,
                 uint32_t* hit_index, uint32_t* n_hits, const CastScratch& s, cudaStream_t stream) {
  check(cudaMemsetAsync(s.tickets, 0, 16, stream), "memset");
  if (cast_tiles(n)) check(cudaMemsetAsync(s.tiles, 0, cast_tiles(n) * 8, stream), "memset");
  LaunchCtx L = c->launch();
  L.scene = c->dropin_scene();  // the drop-in's records whatever the trace mode
  const unsigned warps = (unsigned)((n + 31) / 32);
  const unsigned grid = std::max(1u, std::min(L.trace_blocks, (warps + CAST_THREADS / 32 - 1) / (CAST_THREADS / 32)));
  if (n) {
    if (any_hit)
      k_cast<true><<<grid, CAST_THREADS, 0, stream>>>(L.scene, o4, d4, n, hits4, s.flags, s.tickets, s.tickets + 2);
    else
      k_cast<false><<<grid, CAST_THREADS, 0, stream>>>(L.scene, o4, d4, n, hits4, s.flags, s.tickets, s.tickets + 2);
  }
  const unsigned lgrid = (unsigned)std::max<size_t>(1, std::min<size_t>(cast_tiles(n), (size_t)c->sms * 4));
  k_hit_list<<<lgrid, LIST_THREADS, 0, stream>>>(s.flags, n, hit_index, n_hits, s.tickets + 1, s.tiles,
                                                  s.tickets + 2);
  check(cudaGetLastError(), "pk_cast_rays");
  return PK_OK;
}

}  // namespace pk

using namespace pk;

extern "C" int pk_cast_rays(pk_ctx* c, const float* ray_o4, const float* ray_d4, uint32_t n, int any_hit,
                            uint32_t* hits4, uint32_t* hit_index, uint32_t* n_hits) {
  if (!c) return PK_ERR_ARG;
  try {
    check(cudaSetDevice(c->device), "cudaSetDevice");
    if (!c->bvh_ready) { c->err = "pk_cast_rays: no BVH"; return PK_ERR_STATE; }
    if ((n && (!ray_o4 || !ray_d4 || !hits4 || !hit_index)) || !n_hits) { c->err = "pk_cast_rays: null buffer"; return PK_ERR_ARG; }
    if (n > (1u << 30)) { c->err = "pk_cast_rays: too many rays"; return PK_ERR_ARG; }
    DevBuf<uint32_t> tickets(4), flags(std::max<size_t>(cast_flag_words(n), 1));
    DevBuf<unsigned long long> tiles(std::max<size_t>(cast_tiles(n), 1));
    const CastScratch s{tickets.p, flags.p, tiles.p};
    cast_enqueue(c, reinterpret_cast<const float4*>(ray_o4), reinterpret_cast<const float4*>(ray_d4), n, any_hit,
                 reinterpret_cast<uint4*>(hits4), hit_index, n_hits, s, c->stream);
    uint32_t err = 0;
    check(cudaMemcpyAsync(&err, tickets.p + 2, 4, cudaMemcpyDeviceToHost, c->stream), "D2H");
    check(cudaStreamSynchronize(c->stream), "sync");
    if (err) { c->err = "pk_cast_rays: device error flags"; return PK_ERR_DEVICE; }
    return PK_OK;
  } catch (CudaError& e) {
    c->err = e.what();
    return PK_ERR_CUDA;
  }
}

// ---- allocation-free variant -------------------------------------------------
// pk_cast_rays allocates its scratch (work tickets, the per-ray hit bitmask and
// the look-back tile states of the hit list) with cudaMalloc on every call.
// pk_cast_rays_noalloc takes it from the file-scope array below instead, so it
// calls neither cudaMalloc nor cudaFree.  Every GPU that loads the library
// holds one copy of the array until the process exits.
namespace pk {
namespace {

constexpr uint32_t NOALLOC_MAX_RAYS = 1u << 20;                      // rays per call
constexpr size_t NOALLOC_FLAG_WORDS = NOALLOC_MAX_RAYS / 32;          // 32768 u32
constexpr size_t NOALLOC_TILES = (NOALLOC_FLAG_WORDS + LIST_THREADS - 1) / LIST_THREADS;  // 128 u64
constexpr size_t NOALLOC_FLAGS_OFF = 256;
constexpr size_t NOALLOC_TILES_OFF = NOALLOC_FLAGS_OFF + NOALLOC_FLAG_WORDS * 4;
constexpr size_t NOALLOC_BYTES = NOALLOC_TILES_OFF + NOALLOC_TILES * 8;  // 132,352 bytes

static __device__ __align__(256) unsigned char g_cast_scratch[NOALLOC_BYTES];

}  // namespace

// The array's device address on the current device.  In host code the name
// g_cast_scratch is only a host-side stand-in, not a device address, so
// pk_create looks the address up once, with the context's device current, and
// keeps it in the context: it stays valid exactly as long as the context's
// other device memory (a device reset invalidates both; the next pk_create
// looks it up again).
void* noalloc_scratch_address() {
  void* p = nullptr;
  check(cudaGetSymbolAddress(&p, g_cast_scratch), "cudaGetSymbolAddress(g_cast_scratch)");
  return p;
}

}  // namespace pk

extern "C" int pk_cast_rays_noalloc(pk_ctx* c, const float* ray_o4, const float* ray_d4, uint32_t n, int any_hit,
                                    uint32_t* hits4, uint32_t* hit_index, uint32_t* n_hits) {
  if (!c) return PK_ERR_ARG;
  try {
    check(cudaSetDevice(c->device), "cudaSetDevice");
    if (!c->bvh_ready) { c->err = "pk_cast_rays_noalloc: no BVH"; return PK_ERR_STATE; }
    if ((n && (!ray_o4 || !ray_d4 || !hits4 || !hit_index)) || !n_hits) {
      c->err = "pk_cast_rays_noalloc: null buffer";
      return PK_ERR_ARG;
    }
    if (n > NOALLOC_MAX_RAYS) {
      c->err = "pk_cast_rays_noalloc: at most 1048576 rays per call (the size of its static scratch)";
      return PK_ERR_ARG;
    }
    if (!c->cast_scratch) { c->err = "pk_cast_rays_noalloc: scratch address not set up"; return PK_ERR_STATE; }
    unsigned char* base = static_cast<unsigned char*>(c->cast_scratch);
    const CastScratch s{reinterpret_cast<uint32_t*>(base), reinterpret_cast<uint32_t*>(base + NOALLOC_FLAGS_OFF),
                        reinterpret_cast<unsigned long long*>(base + NOALLOC_TILES_OFF)};
    cast_enqueue(c, reinterpret_cast<const float4*>(ray_o4), reinterpret_cast<const float4*>(ray_d4), n, any_hit,
                 reinterpret_cast<uint4*>(hits4), hit_index, n_hits, s, c->stream);
    uint32_t err = 0;
    check(cudaMemcpyAsync(&err, s.tickets + 2, 4, cudaMemcpyDeviceToHost, c->stream), "D2H");
    check(cudaStreamSynchronize(c->stream), "sync");
    if (err) { c->err = "pk_cast_rays_noalloc: device error flags"; return PK_ERR_DEVICE; }
    return PK_OK;
  } catch (CudaError& e) {
    c->err = e.what();
    return PK_ERR_CUDA;
  }
}

// ---- autofocus distance --------------------------------------------------------
// Raycaster.cast (render/raycaster.js:13-131): one ray traversed in double
// precision over the exact (unquantised) node bounds and normalised triangles,
// Möller-Trumbore with epsilon 1e-12, MAX_T = 1e6.  The recursion is kept as
// an explicit stack: closestNode orders the two children by entry distance,
// and each is entered only if its distance is below the closest hit found so
// far when its turn comes.  Math.min / Math.max propagate NaN, so a slab with
// 0 * inf culls the box exactly as the reference does.
namespace pk {
namespace {

__device__ __forceinline__ double jmin(double a, double b) {
  return (a != a || b != b) ? __longlong_as_double(0x7ff8000000000000ll) : (a < b ? a : (b < a ? b : (signbit(a) ? a : b)));
}
__device__ __forceinline__ double jmax(double a, double b) {
  return (a != a || b != b) ? __longlong_as_double(0x7ff8000000000000ll) : (a > b ? a : (b > a ? b : (signbit(a) ? b : a)));
}

struct FocusScene {
  const double* pos3;
  const int32_t* nodes5;
  const double* box6;
  const int4* tri4_leaf;
  double cx, cy, cz, s;
};

__device__ __forceinline__ double focus_box(const FocusScene& f, int node, const double* o, const double* inv) {
  const double* b = f.box6 + 6 * (size_t)node;
  const double c[3] = {f.cx, f.cy, f.cz};
  double t1[3], t2[3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const double mn = (b[a] - c[a]) * f.s, mx = (b[3 + a] - c[a]) * f.s;
    t1[a] = (mn - o[a]) * inv[a];
    t2[a] = (mx - o[a]) * inv[a];
  }
  double tmin = jmin(t1[0], t2[0]), tmax = jmax(t1[0], t2[0]);
  tmin = jmax(tmin, jmin(t1[1], t2[1]));
  tmax = jmin(tmax, jmax(t1[1], t2[1]));
  tmin = jmax(tmin, jmin(t1[2], t2[2]));
  tmax = jmin(tmax, jmax(t1[2], t2[2]));
  return (tmax >= tmin && tmax >= 0.0) ? tmin : 1000000.0;
}

__device__ __forceinline__ double focus_tri(const FocusScene& f, const int4 t4, const double* o, const double* d) {
  const double eps = 0.000000000001;
  double v[3][3];
  const int ids[3] = {t4.x, t4.y, t4.z};
  const double c[3] = {f.cx, f.cy, f.cz};
#pragma unroll
  for (int k = 0; k < 3; k++)
#pragma unroll
    for (int a = 0; a < 3; a++) v[k][a] = (f.pos3[3 * (size_t)ids[k] + a] - c[a]) * f.s;
  double e1[3], e2[3], tv[3];
#pragma unroll
  for (int a = 0; a < 3; a++) { e1[a] = v[1][a] - v[0][a]; e2[a] = v[2][a] - v[0][a]; tv[a] = o[a] - v[0][a]; }
  const double p[3] = {d[1] * e2[2] - d[2] * e2[1], -(d[0] * e2[2] - d[2] * e2[0]), d[0] * e2[1] - d[1] * e2[0]};
  const double det = 0.0 + e1[0] * p[0] + e1[1] * p[1] + e1[2] * p[2];
  if (det > -eps && det < eps) return 1000000.0;
  const double inv = 1.0 / det;
  const double u = (0.0 + tv[0] * p[0] + tv[1] * p[1] + tv[2] * p[2]) * inv;
  if (u < 0.0 || u > 1.0) return 1000000.0;
  const double q[3] = {tv[1] * e1[2] - tv[2] * e1[1], -(tv[0] * e1[2] - tv[2] * e1[0]), tv[0] * e1[1] - tv[1] * e1[0]};
  const double vv = (0.0 + d[0] * q[0] + d[1] * q[1] + d[2] * q[2]) * inv;
  if (vv < 0.0 || u + vv > 1.0) return 1000000.0;
  const double t = (0.0 + e2[0] * q[0] + e2[1] * q[1] + e2[2] * q[2]) * inv;
  return t > eps ? t : 1000000.0;
}

constexpr int FOCUS_STACK = 96;

__global__ void k_focus(FocusScene f, const double* __restrict__ rays6, uint32_t n, double* __restrict__ t_out,
                        uint32_t* __restrict__ err) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const double o[3] = {rays6[6 * r], rays6[6 * r + 1], rays6[6 * r + 2]};
  const double d[3] = {rays6[6 * r + 3], rays6[6 * r + 4], rays6[6 * r + 5]};
  const double inv[3] = {1.0 / d[0], 1.0 / d[1], 1.0 / d[2]};
  int stack_node[FOCUS_STACK];
  double stack_t[FOCUS_STACK];
  int sp = 0;
  double closest = 1000000.0;
  // the root is entered unconditionally (cast -> traverse(root, MAX_T))
  stack_node[sp] = 0;
  stack_t[sp] = -__longlong_as_double(0x7ff0000000000000ll);
  sp++;
  bool first = true;
  while (sp > 0) {
    --sp;
    const int node = stack_node[sp];
    if (!first && !(stack_t[sp] < closest)) continue;
    first = false;
    const int32_t* nd = f.nodes5 + 5 * (size_t)node;
    if (nd[1] > -1) {  // leaf: processLeaf returns the leaf's own minimum
      const int size = nd[1] >> 24, base = nd[1] & 0x00ffffff;
      double res = 1000000.0;
      for (int i = 0; i < size; i++) {
        const double x = focus_tri(f, f.tri4_leaf[base + i], o, d);
        if (x < res) res = x;
      }
      closest = jmin(res, closest);
      continue;
    }
    const int l = nd[0], rr = nd[0] + 1;
    const double tl = focus_box(f, l, o, inv), tr = focus_box(f, rr, o, inv);
    // closestNode: a child whose box is missed is dropped; the nearer one goes first
    const int ln = tl < 1000000.0 ? l : -1, rn = tr < 1000000.0 ? rr : -1;
    int o0, o1;
    double t0, t1;
    if (tl < tr) { o0 = ln; t0 = tl; o1 = rn; t1 = tr; } else { o0 = rn; t0 = tr; o1 = ln; t1 = tl; }
    if (sp + 2 > FOCUS_STACK) { atomicOr(err, 1u); break; }
    if (o1 >= 0) { stack_node[sp] = o1; stack_t[sp] = t1; sp++; }
    if (o0 >= 0) { stack_node[sp] = o0; stack_t[sp] = t0; sp++; }
  }
  t_out[r] = closest;
}

}  // namespace
}  // namespace pk

extern "C" int pk_focus_distance(pk_ctx* c, const double origin[3], const double dir[3], double* t_out,
                                 double* focal_depth_out) {
  if (!c) return PK_ERR_ARG;
  try {
    check(cudaSetDevice(c->device), "cudaSetDevice");
    if (!c->bvh_ready || !c->node_box_d.p || c->norm[3] == 0.0) {
      c->err = "pk_focus_distance: needs a BVH built by pk_bvh_build (its exact node bounds)";
      return PK_ERR_STATE;
    }
    if (!origin || !dir || !t_out) { c->err = "pk_focus_distance: null argument"; return PK_ERR_ARG; }
    const double ray[6] = {origin[0], origin[1], origin[2], dir[0], dir[1], dir[2]};
    DevBuf<double> dray(6), dt(1);
    DevBuf<uint32_t> err(1);
    check(cudaMemsetAsync(err.p, 0, 4, c->stream), "memset");
    check(cudaMemcpyAsync(dray.p, ray, sizeof ray, cudaMemcpyHostToDevice, c->stream), "H2D");
    const FocusScene f{c->pos.p, c->nodes5.p, c->node_box_d.p, reinterpret_cast<const int4*>(c->tri4_leaf.p),
                       c->norm[0], c->norm[1], c->norm[2], c->norm[3]};
    k_focus<<<1, 32, 0, c->stream>>>(f, dray.p, 1, dt.p, err.p);
    check(cudaGetLastError(), "k_focus");
    double t = 0.0;
    uint32_t e = 0;
    check(cudaMemcpyAsync(&t, dt.p, 8, cudaMemcpyDeviceToHost, c->stream), "D2H");
    check(cudaMemcpyAsync(&e, err.p, 4, cudaMemcpyDeviceToHost, c->stream), "D2H");
    check(cudaStreamSynchronize(c->stream), "sync");
    if (e) { c->err = "pk_focus_distance: traversal stack overflow"; return PK_ERR_DEVICE; }
    *t_out = t;
    if (focal_depth_out) *focal_depth_out = 1.0 - 1.0 / t;  // PikeRenderer.focusCamera (pike.js:88-90)
    return PK_OK;
  } catch (CudaError& e) {
    c->err = e.what();
    return PK_ERR_CUDA;
  }
}
