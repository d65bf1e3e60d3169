// pk_bvh.cu -- GPU rebuild of the reference BVH: bvh.js full-sweep object SAH
// (render/bvh.js:12-223, render/primitives.js:3-44), BFS serialisation
// (bvh.js:46-74) and trace_pass.js packing (trace_pass.js:166-170,202-262).
//
// Exactness argument.  Every reference ref list of a node is its triangles
// ordered by (centroid[axis], triangle index): the root lists come from a
// stable sort of triangles in index order, and #splitNode keeps relative
// order.  So each level keeps three arrays A[axis] whose node segments are
// exactly the reference lists.  Box unions are exact (min/max), so segmented
// prefix/suffix scans reproduce every bbFront/bbBack box bit for bit, and the
// surface areas and costs are evaluated with the same double expressions in
// the same order (the library is built without FMA contraction).  The first
// minimum in (axis, index) order is the reference's strict `<` winner.
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "pk_bvh.h"
#include "pk_internal.cuh"
#include "pk_util.h"

namespace pk {
namespace {

struct Box6 {
  double mn[3];
  double mx[3];
};

__device__ __forceinline__ Box6 box_empty() {
  Box6 b;
#pragma unroll
  for (int i = 0; i < 3; i++) { b.mn[i] = __longlong_as_double(0x7ff0000000000000ll); b.mx[i] = -b.mn[i]; }
  return b;
}
__device__ __forceinline__ Box6 box_union(const Box6& a, const Box6& b) {
  Box6 r;
#pragma unroll
  for (int i = 0; i < 3; i++) { r.mn[i] = fmin(a.mn[i], b.mn[i]); r.mx[i] = fmax(a.mx[i], b.mx[i]); }
  return r;
}
// BoundingBox.getSurfaceArea (primitives.js:39-44)
__device__ __forceinline__ double box_sa(const Box6& b) {
  const double xl = fmax(b.mx[0] - b.mn[0], 0.0);
  const double yl = fmax(b.mx[1] - b.mn[1], 0.0);
  const double zl = fmax(b.mx[2] - b.mn[2], 0.0);
  return (xl * yl + xl * zl + yl * zl) * 2.0;
}
__device__ __forceinline__ Box6 shfl_up_box(const Box6& b, int o) {
  Box6 r;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    r.mn[i] = __shfl_up_sync(0xffffffffu, b.mn[i], o);
    r.mx[i] = __shfl_up_sync(0xffffffffu, b.mx[i], o);
  }
  return r;
}
// Segmented-scan operator: (a, then b) = b restarts the segment if it holds a head.
__device__ __forceinline__ void seg_op(const Box6& ab, bool af, const Box6& bb, bool bf, Box6& rb, bool& rf) {
  rb = bf ? bb : box_union(ab, bb);
  rf = af || bf;
}

// ---- per-triangle boxes and sort keys (Node.sortRefs keys) -------------------
__global__ void k_tri_boxes(const double* __restrict__ pos3, const int4* __restrict__ tri4, uint32_t n,
                            Box6* __restrict__ boxes, unsigned long long* __restrict__ keys,
                            uint32_t* __restrict__ vals) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int4 tr = tri4[t];
  const int v[3] = {tr.x, tr.y, tr.z};
  Box6 b = box_empty();
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const double* p = pos3 + 3 * (size_t)v[k];
#pragma unroll
    for (int a = 0; a < 3; a++) { b.mn[a] = fmin(p[a], b.mn[a]); b.mx[a] = fmax(p[a], b.mx[a]); }
  }
  boxes[t] = b;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    double c = (b.mn[a] + b.mx[a]) * 0.5;  // BoundingBox.centroid (primitives.js:32-37)
    if (c == 0.0) c = 0.0;                 // -0 and +0 compare equal in the reference sort
    const unsigned long long u = (unsigned long long)__double_as_longlong(c);
    keys[(size_t)a * n + t] = (u >> 63) ? ~u : (u | 0x8000000000000000ull);
    vals[(size_t)a * n + t] = t;
  }
}

// ---- segmented box scans with decoupled look-back ------------------------------
constexpr int SEG_THREADS = 256;
constexpr int SEG_ITEMS = 4;
constexpr int SEG_TILE = SEG_THREADS * SEG_ITEMS;
constexpr int SEG_WARPS = SEG_THREADS / 32;

struct SegState {
  uint32_t* status;   // 0 none, 1 aggregate, 2 inclusive
  Box6* agg;
  uint32_t* aggflag;
  Box6* incl;
  uint32_t* ticket;
  uint32_t* err;
};

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(uint32_t* p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ Box6 ld_box_cg(const Box6* p) {
  Box6 b;
  const double* d = reinterpret_cast<const double*>(p);
#pragma unroll
  for (int i = 0; i < 3; i++) { b.mn[i] = __ldcg(d + i); b.mx[i] = __ldcg(d + 3 + i); }
  return b;
}

// REV = false: prefix boxes (bbFront), SA written per position, and the node
// box at each segment's last position.  REV = true: suffix boxes (bbBack):
// sa_out[p] = SA of the union of positions p .. segment end.
template <bool REV>
__global__ void __launch_bounds__(SEG_THREADS) k_segscan(const int32_t* __restrict__ A, const int32_t* __restrict__ seg,
                                                         const uint32_t* __restrict__ nstart,
                                                         const uint32_t* __restrict__ ncount,
                                                         const Box6* __restrict__ tri_box, uint32_t n,
                                                         double* __restrict__ sa_out, Box6* __restrict__ seg_box,
                                                         SegState st) {
  __shared__ uint32_t s_tile;
  __shared__ Box6 s_wbox[SEG_WARPS];
  __shared__ uint32_t s_wflag[SEG_WARPS];
  __shared__ Box6 s_carry;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t ntiles = (n + SEG_TILE - 1) / SEG_TILE;
  for (;;) {
    if (threadIdx.x == 0) s_tile = atomicAdd(st.ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= ntiles) break;
    const uint32_t q0 = tile * SEG_TILE + threadIdx.x * SEG_ITEMS;
    Box6 bx[SEG_ITEMS];
    bool hd[SEG_ITEMS];
    Box6 agg = box_empty();
    bool af = false;
#pragma unroll
    for (int k = 0; k < SEG_ITEMS; k++) {
      const uint32_t q = q0 + k;
      hd[k] = false;
      bx[k] = box_empty();
      if (q < n) {
        const uint32_t p = REV ? n - 1 - q : q;
        const int32_t s = seg[p];
        const uint32_t s0 = nstart[s], sc = ncount[s];
        hd[k] = REV ? (p == s0 + sc - 1) : (p == s0);
        bx[k] = tri_box[A[p]];
        Box6 r;
        bool rf;
        seg_op(agg, af, bx[k], hd[k], r, rf);
        agg = r;
        af = rf;
      }
    }
    // warp inclusive segmented scan of thread aggregates
    Box6 inc = agg;
    bool incf = af;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const Box6 ub = shfl_up_box(inc, o);
      const bool uf = __shfl_up_sync(0xffffffffu, incf, o);
      if (lane >= o) {
        Box6 r;
        bool rf;
        seg_op(ub, uf, inc, incf, r, rf);
        inc = r;
        incf = rf;
      }
    }
    if (lane == 31) { s_wbox[warp] = inc; s_wflag[warp] = incf; }
    __syncthreads();
    if (threadIdx.x == 0) {
      // exclusive prefixes of warp totals, then the tile total
      Box6 run = box_empty();
      bool rf = false;
      for (int w = 0; w < SEG_WARPS; w++) {
        const Box6 wb = s_wbox[w];
        const bool wf = s_wflag[w] != 0;
        s_wbox[w] = run;
        s_wflag[w] = rf;
        Box6 r2;
        bool f2;
        seg_op(run, rf, wb, wf, r2, f2);
        run = r2;
        rf = f2;
      }
      // decoupled look-back for the carry into this tile
      if (tile == 0) {
        st.incl[0] = run;
        __threadfence();
        st_release_u32(&st.status[0], 2u);
        s_carry = box_empty();
      } else {
        if (rf) {  // a head inside the tile: successors need nothing before it
          st.incl[tile] = run;
          __threadfence();
          st_release_u32(&st.status[tile], 2u);
        } else {
          st.agg[tile] = run;
          st.aggflag[tile] = 0u;
          __threadfence();
          st_release_u32(&st.status[tile], 1u);
        }
        Box6 carry = box_empty();
        int i = (int)tile - 1;
        while (i >= 0) {
          uint32_t v = ld_acquire_u32(&st.status[i]);
          int spins = 0;
          while (v == 0u) {
            if (++spins > LOOKBACK_SPIN_LIMIT) { atomicOr(st.err, ERR_LOOKBACK); v = 3u; break; }
            __nanosleep(64);
            v = ld_acquire_u32(&st.status[i]);
          }
          if (v == 3u) break;
          if (v == 2u) { carry = box_union(ld_box_cg(&st.incl[i]), carry); break; }
          carry = box_union(ld_box_cg(&st.agg[i]), carry);
          --i;
        }
        if (!rf) {
          st.incl[tile] = box_union(carry, run);
          __threadfence();
          st_release_u32(&st.status[tile], 2u);
        }
        s_carry = carry;
      }
    }
    __syncthreads();
    // this thread's exclusive prefix: carry (no head) then warps before, then lanes before
    Box6 pre;
    bool pf;
    {
      Box6 lb = shfl_up_box(inc, 1);
      bool lf = __shfl_up_sync(0xffffffffu, incf, 1);
      if (lane == 0) { lb = box_empty(); lf = false; }
      Box6 wpre;
      bool wpf;
      seg_op(s_carry, false, s_wbox[warp], s_wflag[warp] != 0, wpre, wpf);
      seg_op(wpre, wpf, lb, lf, pre, pf);
    }
    Box6 run = pre;
#pragma unroll
    for (int k = 0; k < SEG_ITEMS; k++) {
      const uint32_t q = q0 + k;
      if (q >= n) break;
      const uint32_t p = REV ? n - 1 - q : q;
      run = hd[k] ? bx[k] : box_union(run, bx[k]);
      sa_out[p] = box_sa(run);
      if (!REV && seg_box) {
        const int32_t s = seg[p];
        if (p == nstart[s] + ncount[s] - 1) seg_box[s] = run;
      }
    }
    __syncthreads();
  }
}

// ---- costs and the first minimum ------------------------------------------------
__global__ void k_node_sa(const Box6* __restrict__ level_box, uint32_t m, double* __restrict__ psa) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < m) psa[k] = box_sa(level_box[k]);
}

// bvh.js:195-208: cost = TRAVERSAL_COST + (sAf/pSA)(i+1) + (sAb/pSA)(n-1-i)
__global__ void k_cost(const int32_t* __restrict__ seg, const uint32_t* __restrict__ nstart,
                       const uint32_t* __restrict__ ncount, const double* __restrict__ psa,
                       const double* __restrict__ saf, const double* __restrict__ sab, uint32_t n,
                       double* __restrict__ cost_out, unsigned long long* __restrict__ best_cost) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  int k = -1;
  unsigned long long bits = ~0ull;
  if (p < n) {
    k = seg[p];
    const uint32_t i = p - nstart[k];
    const uint32_t cnt = ncount[k];
    const double ps = psa[k];
    const double cost = 0.5 + (saf[p] / ps) * (double)(i + 1) + (sab[p] / ps) * (double)(cnt - 1 - i);
    cost_out[p] = cost;
    if (cost < __longlong_as_double(0x7ff0000000000000ll)) bits = (unsigned long long)__double_as_longlong(cost);
  }
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long ob = __shfl_down_sync(0xffffffffu, bits, o);
    const int ok = __shfl_down_sync(0xffffffffu, k, o);
    if (lane + o < 32 && ok == k && ob < bits) bits = ob;
  }
  const int kp = __shfl_up_sync(0xffffffffu, k, 1);
  const bool head = lane == 0 || kp != k;
  if (p < n && head && bits != ~0ull) atomicMin(best_cost + k, bits);
}

__global__ void k_argmin(const int32_t* __restrict__ seg, const uint32_t* __restrict__ nstart,
                         const uint32_t* __restrict__ ncount, const double* __restrict__ cost, uint32_t n, uint32_t axis,
                         const unsigned long long* __restrict__ best_cost, uint32_t* __restrict__ best_idx) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  int k = -1;
  uint32_t key = ~0u;
  if (p < n) {
    k = seg[p];
    if ((unsigned long long)__double_as_longlong(cost[p]) == best_cost[k]) {
      key = axis * ncount[k] + (p - nstart[k]);
    }
  }
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t ob = __shfl_down_sync(0xffffffffu, key, o);
    const int ok = __shfl_down_sync(0xffffffffu, k, o);
    if (lane + o < 32 && ok == k && ob < key) key = ob;
  }
  const int kp = __shfl_up_sync(0xffffffffu, k, 1);
  const bool head = lane == 0 || kp != k;
  if (p < n && head && key != ~0u) atomicMin(best_idx + k, key);
}

// Node ctor (bvh.js:127-143): leaf iff cost > n; the leaf keeps the best axis' order.
__global__ void k_decide(uint32_t m, const uint32_t* __restrict__ ncount, const uint32_t* __restrict__ nbfs,
                         const unsigned long long* __restrict__ best_cost, const uint32_t* __restrict__ best_idx,
                         const Box6* __restrict__ level_box, Box6* __restrict__ node_box, uint32_t* __restrict__ is_inner,
                         uint32_t* __restrict__ inner_cnt, uint32_t* __restrict__ leaf_cnt, uint32_t* __restrict__ axis_out,
                         uint32_t* __restrict__ nleft, uint32_t* __restrict__ err) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  const uint32_t cnt = ncount[k];
  const unsigned long long bc = best_cost[k];
  node_box[nbfs[k]] = level_box[k];
  uint32_t axis = 0, idx = 0;
  bool leaf;
  if (bc == ~0ull || best_idx[k] == ~0u) {
    atomicOr(err, ERR_BVH);  // no finite split cost: the reference throws here
    leaf = true;
  } else {
    axis = best_idx[k] / cnt;
    idx = best_idx[k] % cnt;
    leaf = __longlong_as_double((long long)bc) > (double)cnt;
  }
  if (leaf && cnt >= 128u) atomicOr(err, ERR_BVH);  // does not fit the packed leaf word
  is_inner[k] = leaf ? 0u : 1u;
  inner_cnt[k] = leaf ? 0u : cnt;
  leaf_cnt[k] = leaf ? cnt : 0u;
  axis_out[k] = axis;
  nleft[k] = idx + 1u;
}

// #splitNode (bvh.js:80-107): mark the left refs along the split axis.
__global__ void k_left_flags(const int32_t* __restrict__ A, const int32_t* __restrict__ seg, uint32_t n, uint32_t axis,
                             const uint32_t* __restrict__ nstart, const uint32_t* __restrict__ is_inner,
                             const uint32_t* __restrict__ split_axis, const uint32_t* __restrict__ nleft,
                             uint8_t* __restrict__ left) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int32_t k = seg[p];
  if (!is_inner[k] || split_axis[k] != axis) return;
  left[A[p]] = (p - nstart[k]) < nleft[k] ? 1 : 0;
}

__global__ void k_flag_vals(const int32_t* __restrict__ A, const int32_t* __restrict__ seg, uint32_t n,
                            const uint32_t* __restrict__ is_inner, const uint8_t* __restrict__ left,
                            uint32_t* __restrict__ f) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  f[p] = is_inner[seg[p]] ? (uint32_t)left[A[p]] : 0u;
}

// Stable partition into the children's segments; leaf refs leave the level and
// are written to the leaf-ordered triangle list in the leaf's axis order.
__global__ void k_scatter(const int32_t* __restrict__ A, const int32_t* __restrict__ seg, uint32_t n, uint32_t axis,
                          const uint32_t* __restrict__ nstart, const uint32_t* __restrict__ ncount,
                          const uint32_t* __restrict__ is_inner, const uint32_t* __restrict__ split_axis,
                          const uint32_t* __restrict__ nleft, const uint32_t* __restrict__ inner_rank,
                          const uint32_t* __restrict__ new_base, const uint32_t* __restrict__ leaf_base,
                          uint32_t leaf_offset, const uint8_t* __restrict__ left, const uint32_t* __restrict__ X,
                          int32_t* __restrict__ A2, int32_t* __restrict__ seg2, int32_t* __restrict__ leaf_ids) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int32_t k = seg[p];
  const uint32_t s0 = nstart[k];
  const uint32_t i = p - s0;
  const int32_t tri = A[p];
  if (!is_inner[k]) {
    if (split_axis[k] == axis) leaf_ids[leaf_offset + leaf_base[k] + i] = tri;
    return;
  }
  const uint32_t nl = nleft[k];
  const bool fl = left[tri] != 0;
  const uint32_t rank_l = X ? X[p] - X[s0] : i;
  const uint32_t np = new_base[k] + (fl ? rank_l : nl + (i - rank_l));
  A2[np] = tri;
  if (seg2) seg2[np] = (int32_t)(2u * inner_rank[k] + (fl ? 0u : 1u));
}

// serializeTree (bvh.js:46-74): children of level node k are the next level's
// nodes 2r and 2r+1 (r = rank of k among inner nodes), i.e. BFS order.
__global__ void k_children(uint32_t m, const uint32_t* __restrict__ nstart, const uint32_t* __restrict__ ncount,
                           const uint32_t* __restrict__ nbfs, const uint32_t* __restrict__ is_inner,
                           const uint32_t* __restrict__ nleft, const uint32_t* __restrict__ inner_rank,
                           const uint32_t* __restrict__ new_base, const uint32_t* __restrict__ leaf_base,
                           uint32_t leaf_offset, uint32_t bfs_next, uint32_t* __restrict__ nstart2,
                           uint32_t* __restrict__ ncount2, uint32_t* __restrict__ nbfs2, int32_t* __restrict__ nodes5,
                           uint32_t* __restrict__ err) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  int32_t* nd = nodes5 + 5 * (size_t)nbfs[k];
  const uint32_t cnt = ncount[k];
  if (is_inner[k]) {
    const uint32_t r = inner_rank[k];
    const uint32_t nl = nleft[k];
    nstart2[2 * r] = new_base[k];
    ncount2[2 * r] = nl;
    nstart2[2 * r + 1] = new_base[k] + nl;
    ncount2[2 * r + 1] = cnt - nl;
    nbfs2[2 * r] = bfs_next + 2 * r;
    nbfs2[2 * r + 1] = bfs_next + 2 * r + 1;
    nd[0] = (int32_t)(bfs_next + 2 * r);
    nd[1] = -1;
  } else {
    const uint32_t base = leaf_offset + leaf_base[k];
    if (base >= (1u << 24)) atomicOr(err, ERR_BVH);
    nd[0] = -1;
    nd[1] = (int32_t)((cnt << 24) | base);  // maskTriIndex (trace_pass.js:166-170)
  }
}

// trace_pass.js:213-218 quantizeVec2ToInt on normalised bounds.
__device__ __forceinline__ int js_toint16(double v) {
  if (!isfinite(v)) return 0;
  double m = fmod(trunc(v), 65536.0);
  if (m < 0.0) m += 65536.0;
  int mi = (int)m;
  if (mi >= 32768) mi -= 65536;
  return mi;
}
__device__ __forceinline__ uint32_t quantize2(double a, double b) {
  const int s0 = js_toint16(a * (a > 0.0 ? 32767.0 : 32768.0));
  const int s1 = js_toint16(b * (b > 0.0 ? 32767.0 : 32768.0));
  return (uint32_t)(uint16_t)s0 | ((uint32_t)(uint16_t)s1 << 16);
}
__global__ void k_quantize_nodes(uint32_t m, const Box6* __restrict__ node_box, double cx, double cy, double cz,
                                 double longest, int32_t* __restrict__ nodes5) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= m) return;
  const Box6 bx = node_box[b];
  const double c[3] = {cx, cy, cz};
  int32_t* nd = nodes5 + 5 * (size_t)b;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const double mn = (bx.mn[a] - c[a]) * (2.0 / longest);
    const double mx = (bx.mx[a] - c[a]) * (2.0 / longest);
    nd[2 + a] = (int32_t)quantize2(mx, mn);
  }
}
__global__ void k_norm_verts(const double* __restrict__ pos3, uint32_t n, double cx, double cy, double cz,
                             double longest, float4* __restrict__ verts4) {
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  const double* p = pos3 + 3 * (size_t)v;
  verts4[v] = make_float4((float)((p[0] - cx) * (2.0 / longest)), (float)((p[1] - cy) * (2.0 / longest)),
                          (float)((p[2] - cz) * (2.0 / longest)), 0.0f);
}
__global__ void k_gather_tris(const int4* __restrict__ tri4, const int32_t* __restrict__ ids, uint32_t n,
                              int4* __restrict__ out) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) out[q] = tri4[ids[q]];
}
__global__ void k_fill_u64(unsigned long long* p, uint32_t n, unsigned long long v) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}
__global__ void k_fill_u32(uint32_t* p, uint32_t n, uint32_t v) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

unsigned blocks(uint32_t n, unsigned t = 256) { return (unsigned)((n + t - 1) / t); }

double js_max(double a, double b) { return (a != a || b != b) ? NAN : (a > b ? a : (b > a ? b : (std::signbit(a) ? b : a))); }

}  // namespace

int build_bvh_sweep(cudaStream_t s, const double* pos3, uint32_t n_verts, const int4* tri4, uint32_t T,
                    BvhOut& out, std::string& why) {
  if (T == 0) { why = "no triangles"; return 1; }
  if (T > (1u << 26)) { why = "too many triangles"; return 1; }
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);

  DevBuf<Box6> tri_box(T);
  DevBuf<unsigned long long> keys(3 * (size_t)T), keys_tmp(T);
  DevBuf<uint32_t> vals(3 * (size_t)T), vals_tmp(T);
  k_tri_boxes<<<blocks(T), 256, 0, s>>>(pos3, tri4, T, tri_box.p, keys.p, vals.p);
  check(cudaGetLastError(), "k_tri_boxes");
  for (int a = 0; a < 3; a++)
    radix_sort_pairs_u64(s, reinterpret_cast<uint64_t*>(keys.p) + (size_t)a * T, vals.p + (size_t)a * T,
                         reinterpret_cast<uint64_t*>(keys_tmp.p), vals_tmp.p, T, 64);
  keys.release();
  keys_tmp.release();
  vals_tmp.release();

  DevBuf<int32_t> A(3 * (size_t)T), A2(3 * (size_t)T), seg(T), seg2(T);
  check(cudaMemcpyAsync(A.p, vals.p, 3 * (size_t)T * 4, cudaMemcpyDeviceToDevice, s), "memcpy");
  vals.release();
  check(cudaMemsetAsync(seg.p, 0, (size_t)T * 4, s), "memset");
  DevBuf<uint32_t> nstart(T), ncount(T), nbfs(T), nstart2(T), ncount2(T), nbfs2(T);
  DevBuf<double> saf(T), sab(T), cost(3 * (size_t)T), psa(T);
  DevBuf<unsigned long long> best_cost(T);
  DevBuf<uint32_t> best_idx(T), is_inner(T), inner_cnt(T), leaf_cnt(T), split_axis(T), nleft(T);
  DevBuf<uint32_t> inner_rank(T), new_base(T), leaf_base(T), X(T), fvals(T), totals(4);
  DevBuf<uint8_t> left(T);
  DevBuf<Box6> level_box(T);
  const uint32_t max_nodes = 2 * T - 1;
  DevBuf<Box6> node_box(max_nodes);
  DevBuf<int32_t> nodes5(5 * (size_t)max_nodes);
  DevBuf<int32_t> leaf_ids(T);
  const uint32_t seg_tiles = (T + SEG_TILE - 1) / SEG_TILE;
  DevBuf<uint32_t> st_status(seg_tiles), st_aggflag(seg_tiles), st_aux(2);
  DevBuf<Box6> st_agg(seg_tiles), st_incl(seg_tiles);
  const SegState st{st_status.p, st_agg.p, st_aggflag.p, st_incl.p, st_aux.p, st_aux.p + 1};
  check(cudaMemsetAsync(st_aux.p, 0, 8, s), "memset");
  DevBuf<uint32_t> derr(1);
  check(cudaMemsetAsync(derr.p, 0, 4, s), "memset");

  const uint32_t zero = 0;
  check(cudaMemcpyAsync(nstart.p, &zero, 4, cudaMemcpyHostToDevice, s), "H2D");
  check(cudaMemcpyAsync(ncount.p, &T, 4, cudaMemcpyHostToDevice, s), "H2D");
  check(cudaMemcpyAsync(nbfs.p, &zero, 4, cudaMemcpyHostToDevice, s), "H2D");

  uint32_t n_active = T, m = 1, bfs_base = 0, leaf_offset = 0, depth = 0;
  const unsigned seg_grid = (unsigned)std::max(1u, std::min<uint32_t>(seg_tiles, (uint32_t)sms * 4u));
  while (m > 0) {
    depth++;
    const uint32_t n = n_active;
    k_fill_u64<<<blocks(m), 256, 0, s>>>(best_cost.p, m, ~0ull);
    k_fill_u32<<<blocks(m), 256, 0, s>>>(best_idx.p, m, ~0u);
    for (uint32_t a = 0; a < 3; a++) {
      const int32_t* Aa = A.p + (size_t)a * T;
      const uint32_t nt = (n + SEG_TILE - 1) / SEG_TILE;
      for (int dir = 0; dir < 2; dir++) {
        check(cudaMemsetAsync(st_status.p, 0, (size_t)nt * 4, s), "memset");
        check(cudaMemsetAsync(st_aux.p, 0, 4, s), "memset");
        if (dir == 0)
          k_segscan<false><<<seg_grid, SEG_THREADS, 0, s>>>(Aa, seg.p, nstart.p, ncount.p, tri_box.p, n, saf.p,
                                                             a == 0 ? level_box.p : nullptr, st);
        else
          k_segscan<true><<<seg_grid, SEG_THREADS, 0, s>>>(Aa, seg.p, nstart.p, ncount.p, tri_box.p, n, sab.p,
                                                            nullptr, st);
      }
      if (a == 0) k_node_sa<<<blocks(m), 256, 0, s>>>(level_box.p, m, psa.p);
      k_cost<<<blocks(n), 256, 0, s>>>(seg.p, nstart.p, ncount.p, psa.p, saf.p, sab.p, n, cost.p + (size_t)a * T,
                                        best_cost.p);
    }
    for (uint32_t a = 0; a < 3; a++)
      k_argmin<<<blocks(n), 256, 0, s>>>(seg.p, nstart.p, ncount.p, cost.p + (size_t)a * T, n, a, best_cost.p,
                                          best_idx.p);
    k_decide<<<blocks(m), 256, 0, s>>>(m, ncount.p, nbfs.p, best_cost.p, best_idx.p, level_box.p, node_box.p,
                                        is_inner.p, inner_cnt.p, leaf_cnt.p, split_axis.p, nleft.p, derr.p);
    check(cudaGetLastError(), "bvh level");
    scan_exclusive_u32(s, is_inner.p, inner_rank.p, m, totals.p + 0);
    scan_exclusive_u32(s, inner_cnt.p, new_base.p, m, totals.p + 1);
    scan_exclusive_u32(s, leaf_cnt.p, leaf_base.p, m, totals.p + 2);
    uint32_t tot[3];
    check(cudaMemcpyAsync(tot, totals.p, 12, cudaMemcpyDeviceToHost, s), "D2H");
    check(cudaStreamSynchronize(s), "sync");
    const uint32_t n_inner = tot[0], n_next = tot[1], n_leaf = tot[2];
    if (n_inner) check(cudaMemsetAsync(left.p, 0, T, s), "memset");
    for (uint32_t a = 0; a < 3 && n_inner; a++)
      k_left_flags<<<blocks(n), 256, 0, s>>>(A.p + (size_t)a * T, seg.p, n, a, nstart.p, is_inner.p, split_axis.p,
                                              nleft.p, left.p);
    for (uint32_t a = 0; a < 3; a++) {
      const int32_t* Aa = A.p + (size_t)a * T;
      if (n_inner) {
        k_flag_vals<<<blocks(n), 256, 0, s>>>(Aa, seg.p, n, is_inner.p, left.p, fvals.p);
        scan_exclusive_u32(s, fvals.p, X.p, n, nullptr);
      }
      k_scatter<<<blocks(n), 256, 0, s>>>(Aa, seg.p, n, a, nstart.p, ncount.p, is_inner.p, split_axis.p, nleft.p,
                                           inner_rank.p, new_base.p, leaf_base.p, leaf_offset, left.p,
                                           n_inner ? X.p : nullptr, A2.p + (size_t)a * T, a == 0 ? seg2.p : nullptr,
                                           leaf_ids.p);
    }
    k_children<<<blocks(m), 256, 0, s>>>(m, nstart.p, ncount.p, nbfs.p, is_inner.p, nleft.p, inner_rank.p,
                                          new_base.p, leaf_base.p, leaf_offset, bfs_base + m, nstart2.p, ncount2.p,
                                          nbfs2.p, nodes5.p, derr.p);
    check(cudaGetLastError(), "bvh partition");
    uint32_t herr = 0, lerr = 0;
    check(cudaMemcpyAsync(&herr, derr.p, 4, cudaMemcpyDeviceToHost, s), "D2H");
    check(cudaMemcpyAsync(&lerr, st_aux.p + 1, 4, cudaMemcpyDeviceToHost, s), "D2H");
    check(cudaStreamSynchronize(s), "sync");
    if (lerr) { why = "segmented scan look-back timed out"; return 1; }
    if (herr) { why = "degenerate node (no finite SAH cost) or a leaf of 128+ triangles"; return 1; }
    leaf_offset += n_leaf;
    bfs_base += m;
    m = 2 * n_inner;
    n_active = n_next;
    std::swap(A.p, A2.p);
    std::swap(seg.p, seg2.p);
    std::swap(nstart.p, nstart2.p);
    std::swap(ncount.p, ncount2.p);
    std::swap(nbfs.p, nbfs2.p);
  }
  const uint32_t n_nodes = bfs_base;
  if (leaf_offset != T) { why = "leaf triangle count mismatch"; return 1; }

  // #makeNormalizer(root.bounds) on the host, in double, JavaScript order
  Box6 root;
  check(cudaMemcpy(&root, node_box.p, sizeof(Box6), cudaMemcpyDeviceToHost), "D2H");
  double span[3], center[3];
  for (int i = 0; i < 3; i++) span[i] = root.mx[i] - root.mn[i];
  const double longest = js_max(js_max(span[0], span[1]), span[2]);
  for (int i = 0; i < 3; i++) center[i] = root.mn[i] + span[i] * 0.5;

  out.nodes5.alloc(5 * (size_t)n_nodes);
  check(cudaMemcpyAsync(out.nodes5.p, nodes5.p, 5 * (size_t)n_nodes * 4, cudaMemcpyDeviceToDevice, s), "memcpy");
  k_quantize_nodes<<<blocks(n_nodes), 256, 0, s>>>(n_nodes, node_box.p, center[0], center[1], center[2], longest,
                                                    out.nodes5.p);
  out.verts4.alloc(n_verts);
  k_norm_verts<<<blocks(n_verts), 256, 0, s>>>(pos3, n_verts, center[0], center[1], center[2], longest, out.verts4.p);
  out.tri4_leaf.alloc(T);
  k_gather_tris<<<blocks(T), 256, 0, s>>>(tri4, leaf_ids.p, T, out.tri4_leaf.p);
  out.node_box.alloc(6 * (size_t)n_nodes);
  check(cudaMemcpyAsync(out.node_box.p, node_box.p, (size_t)n_nodes * sizeof(Box6), cudaMemcpyDeviceToDevice, s),
        "memcpy");
  check(cudaGetLastError(), "bvh pack");
  check(cudaStreamSynchronize(s), "sync");
  out.n_nodes = n_nodes;
  out.n_leaf_tris = T;
  out.depth = depth;
  for (int i = 0; i < 3; i++) out.norm[i] = center[i];
  out.norm[3] = 2.0 / longest;
  return 0;
}


// =====================================================================
// Binned SAH builder (PK_BVH_BINNED): not the reference's topology; a fast
// build for callers that do not need bit parity with bvh.js.
//
// Phase 1, level-synchronous over nodes of more than BIN_SMALL triangles:
// each block bins one tile of one node (16 bins per axis by centroid, counts
// and exact double boxes through order-preserving 64-bit keys in shared
// memory, flushed with global atomics), one warp per node scans the bins for
// the cheapest SAH split, and a stable partition (global scan of the
// left flags) keeps every node's triangles contiguous.  Phase 2: one block
// per remaining node builds its whole subtree in place with the same binned
// SAH, allocating child pairs with an atomic counter (children always get
// larger indices than their parent).  Leaves hold at most BIN_MAX_LEAF
// triangles; a node whose centroids share one bin is split at its middle.
// =====================================================================
namespace {

constexpr int NB = 16;
constexpr uint32_t BIN_SMALL = 1024;
constexpr uint32_t BIN_MAX_LEAF = 8;
constexpr int BIN_TILE = 2048;
constexpr int BIN_THREADS = 256;
constexpr double C_TRAV = 1.0;

__device__ __forceinline__ unsigned long long dkey(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double dval(unsigned long long k) {
  const unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)u);
}

// One bin: count, triangle-box bounds and centroid bounds as 64-bit keys.
struct Bin {
  unsigned long long bmin[3], bmax[3], cmin[3], cmax[3];
  unsigned int n, pad;
};
__device__ __forceinline__ void bin_clear(Bin& b) {
  for (int a = 0; a < 3; a++) { b.bmin[a] = b.cmin[a] = ~0ull; b.bmax[a] = b.cmax[a] = 0ull; }
  b.n = 0;
}
template <bool GLOBAL>
__device__ __forceinline__ void bin_add(Bin& b, const Box6& box, const double* c) {
  atomicAdd(&b.n, 1u);
  for (int a = 0; a < 3; a++) {
    atomicMin(&b.bmin[a], dkey(box.mn[a]));
    atomicMax(&b.bmax[a], dkey(box.mx[a]));
    atomicMin(&b.cmin[a], dkey(c[a]));
    atomicMax(&b.cmax[a], dkey(c[a]));
  }
}
__device__ __forceinline__ void bin_merge_global(Bin& dst, const Bin& src) {
  if (!src.n) return;
  atomicAdd(&dst.n, src.n);
  for (int a = 0; a < 3; a++) {
    atomicMin(&dst.bmin[a], src.bmin[a]);
    atomicMax(&dst.bmax[a], src.bmax[a]);
    atomicMin(&dst.cmin[a], src.cmin[a]);
    atomicMax(&dst.cmax[a], src.cmax[a]);
  }
}

struct NodeInfo {
  uint32_t start, count, node;   // element range in the permutation, node index
  int axis, split;               // chosen split: axis and last left bin (-1: middle split)
  uint32_t nleft;
  double cmin[3], cmax[3];       // centroid bounds of the node
  double lcmin[3], lcmax[3], rcmin[3], rcmax[3];
};

__device__ __forceinline__ int bin_of(double c, double lo, double hi) {
  const double ext = hi - lo;
  if (!(ext > 0.0)) return 0;
  int b = (int)((c - lo) * ((double)NB / ext));
  return b < 0 ? 0 : (b >= NB ? NB - 1 : b);
}

__device__ __forceinline__ void centroid(const Box6& b, double* c) {
  for (int a = 0; a < 3; a++) c[a] = (b.mn[a] + b.mx[a]) * 0.5;
}

__global__ void k_tri_boxes_plain(const double* __restrict__ pos3, const int4* __restrict__ tri4, uint32_t n,
                                  Box6* __restrict__ boxes, uint32_t* __restrict__ ids) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int4 tr = tri4[t];
  const int v[3] = {tr.x, tr.y, tr.z};
  Box6 b = box_empty();
  for (int k = 0; k < 3; k++) {
    const double* p = pos3 + 3 * (size_t)v[k];
    for (int a = 0; a < 3; a++) { b.mn[a] = fmin(p[a], b.mn[a]); b.mx[a] = fmax(p[a], b.mx[a]); }
  }
  boxes[t] = b;
  ids[t] = t;
}

// Root box and centroid bounds (one bin holding everything).
__global__ void k_root_bounds(const Box6* __restrict__ boxes, uint32_t n, Bin* __restrict__ root) {
  __shared__ Bin s;
  if (threadIdx.x == 0) bin_clear(s);
  __syncthreads();
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const Box6 b = boxes[t];
    double c[3];
    centroid(b, c);
    bin_add<false>(s, b, c);
  }
  __syncthreads();
  if (threadIdx.x == 0) bin_merge_global(*root, s);
}

struct Tile {
  uint32_t slot, begin, count;
};

__global__ void __launch_bounds__(BIN_THREADS) k_bin_tiles(const Tile* __restrict__ tiles,
                                                           const NodeInfo* __restrict__ nodes,
                                                           const uint32_t* __restrict__ A,
                                                           const Box6* __restrict__ boxes, Bin* __restrict__ bins) {
  __shared__ Bin s[3 * NB];
  const Tile t = tiles[blockIdx.x];
  const NodeInfo& nd = nodes[t.slot];
  for (int i = threadIdx.x; i < 3 * NB; i += BIN_THREADS) bin_clear(s[i]);
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < t.count; i += BIN_THREADS) {
    const Box6 b = boxes[A[t.begin + i]];
    double c[3];
    centroid(b, c);
    for (int a = 0; a < 3; a++) bin_add<false>(s[a * NB + bin_of(c[a], nd.cmin[a], nd.cmax[a])], b, c);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 3 * NB; i += BIN_THREADS) bin_merge_global(bins[(size_t)t.slot * 3 * NB + i], s[i]);
}

// Best binned SAH split of a node from its 3 x NB bins (one thread).
__device__ void choose_split(const Bin* bins, uint32_t count, int& axis, int& split, uint32_t& nleft, Box6& lb,
                             Box6& rb, double* lcmin, double* lcmax, double* rcmin, double* rcmax) {
  double best = 1e300;
  axis = -1;
  split = -1;
  for (int a = 0; a < 3; a++) {
    // suffix areas and counts
    double rarea[NB];
    uint32_t rcount[NB];
    Box6 acc = box_empty();
    uint32_t n = 0;
    for (int b = NB - 1; b >= 0; b--) {
      const Bin& x = bins[a * NB + b];
      if (x.n) {
        for (int k = 0; k < 3; k++) { acc.mn[k] = fmin(acc.mn[k], dval(x.bmin[k])); acc.mx[k] = fmax(acc.mx[k], dval(x.bmax[k])); }
        n += x.n;
      }
      rarea[b] = n ? box_sa(acc) : 0.0;
      rcount[b] = n;
    }
    acc = box_empty();
    n = 0;
    for (int b = 0; b < NB - 1; b++) {
      const Bin& x = bins[a * NB + b];
      if (x.n) {
        for (int k = 0; k < 3; k++) { acc.mn[k] = fmin(acc.mn[k], dval(x.bmin[k])); acc.mx[k] = fmax(acc.mx[k], dval(x.bmax[k])); }
        n += x.n;
      }
      if (n == 0 || rcount[b + 1] == 0) continue;
      const double cost = box_sa(acc) * n + rarea[b + 1] * rcount[b + 1];
      if (cost < best) { best = cost; axis = a; split = b; nleft = n; }
    }
  }
  if (axis < 0) {  // every centroid in one bin on every axis: split the range in the middle
    nleft = count / 2;
    return;
  }
  lb = box_empty();
  rb = box_empty();
  for (int k = 0; k < 3; k++) { lcmin[k] = rcmin[k] = 1e300; lcmax[k] = rcmax[k] = -1e300; }
  for (int b = 0; b < NB; b++) {
    const Bin& x = bins[axis * NB + b];
    if (!x.n) continue;
    Box6& d = b <= split ? lb : rb;
    double* cmn = b <= split ? lcmin : rcmin;
    double* cmx = b <= split ? lcmax : rcmax;
    for (int k = 0; k < 3; k++) {
      d.mn[k] = fmin(d.mn[k], dval(x.bmin[k]));
      d.mx[k] = fmax(d.mx[k], dval(x.bmax[k]));
      cmn[k] = fmin(cmn[k], dval(x.cmin[k]));
      cmx[k] = fmax(cmx[k], dval(x.cmax[k]));
    }
  }
  (void)best;
}

__global__ void k_choose_large(NodeInfo* __restrict__ nodes, uint32_t m, const Bin* __restrict__ bins,
                               uint32_t child_base, int32_t* __restrict__ nodes5, Box6* __restrict__ node_box) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  NodeInfo& nd = nodes[k];
  Box6 lb, rb;
  choose_split(bins + (size_t)k * 3 * NB, nd.count, nd.axis, nd.split, nd.nleft, lb, rb, nd.lcmin, nd.lcmax,
               nd.rcmin, nd.rcmax);
  const uint32_t c = child_base + 2 * k;
  int32_t* p = nodes5 + 5 * (size_t)nd.node;
  p[0] = (int32_t)c;
  p[1] = -1;
  if (nd.axis >= 0) {
    node_box[c] = lb;
    node_box[c + 1] = rb;
  } else {  // middle split: both halves keep the node's bounds
    node_box[c] = node_box[nd.node];
    node_box[c + 1] = node_box[nd.node];
    for (int a = 0; a < 3; a++) {
      nd.lcmin[a] = nd.rcmin[a] = nd.cmin[a];
      nd.lcmax[a] = nd.rcmax[a] = nd.cmax[a];
    }
  }
}

__global__ void k_left_flags_binned(const Tile* __restrict__ tiles, const NodeInfo* __restrict__ nodes,
                                    const uint32_t* __restrict__ A, const Box6* __restrict__ boxes,
                                    uint32_t* __restrict__ flags) {
  const Tile t = tiles[blockIdx.x];
  const NodeInfo& nd = nodes[t.slot];
  for (uint32_t i = threadIdx.x; i < t.count; i += blockDim.x) {
    const uint32_t pos = t.begin + i;
    bool left;
    if (nd.axis < 0) {
      left = pos - nd.start < nd.nleft;
    } else {
      double c[3];
      centroid(boxes[A[pos]], c);
      left = bin_of(c[nd.axis], nd.cmin[nd.axis], nd.cmax[nd.axis]) <= nd.split;
    }
    flags[pos] = left ? 1u : 0u;
  }
}

// Stable partition of each large node's range; X = exclusive scan of flags over all T.
__global__ void k_partition_binned(const Tile* __restrict__ tiles, const NodeInfo* __restrict__ nodes,
                                   const uint32_t* __restrict__ A, const uint32_t* __restrict__ flags,
                                   const uint32_t* __restrict__ X, uint32_t* __restrict__ A2,
                                   uint32_t* __restrict__ err) {
  const Tile t = tiles[blockIdx.x];
  const NodeInfo& nd = nodes[t.slot];
  const uint32_t x0 = X[nd.start];
  for (uint32_t i = threadIdx.x; i < t.count; i += blockDim.x) {
    const uint32_t pos = t.begin + i;
    const uint32_t before_left = X[pos] - x0;
    const uint32_t np = flags[pos] ? nd.start + before_left : nd.start + nd.nleft + (pos - nd.start - before_left);
    if (np < nd.start + nd.count) A2[np] = A[pos];
    else atomicOr(err, ERR_BVH);
  }
}

// Phase 2: one warp builds the subtree of one node of at most BIN_SMALL
// triangles, depth first, with warp-private bins (no atomics: peers that hit
// the same bin are combined with __match_any_sync / __reduce_*_sync and their
// leader updates the bin), a ballot-based stable partition through a
// warp-private buffer, and exact double node boxes from warp reductions.
struct SmallTask {
  uint32_t start, count, node;
};
constexpr int SMALL_WARPS = 4;
constexpr int SMALL_STACK = 128;

__device__ __forceinline__ uint32_t fkey(float x) {
  const uint32_t u = __float_as_uint(x);
  return (u >> 31) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float fval(uint32_t k) {
  return __uint_as_float((k >> 31) ? (k & 0x7fffffffu) : ~k);
}
struct FBin {
  uint32_t n, mn[3], mx[3];
};

__device__ __forceinline__ double warp_min_d(double v) {
  for (int o = 16; o; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ double warp_max_d(double v) {
  for (int o = 16; o; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__global__ void __launch_bounds__(SMALL_WARPS * 32) k_build_small(const SmallTask* __restrict__ tasks,
                                                                  uint32_t n_tasks, uint32_t* __restrict__ A,
                                                                  const Box6* __restrict__ boxes,
                                                                  int32_t* __restrict__ nodes5,
                                                                  Box6* __restrict__ node_box,
                                                                  uint32_t* __restrict__ node_counter,
                                                                  uint32_t max_nodes, uint32_t* __restrict__ err) {
  __shared__ FBin sbin[SMALL_WARPS][3 * NB];
  __shared__ SmallTask sstack[SMALL_WARPS][SMALL_STACK];
  __shared__ uint32_t stmp[SMALL_WARPS][BIN_SMALL];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t ti = blockIdx.x * SMALL_WARPS + w;
  if (ti >= n_tasks) return;  // whole warps only
  FBin* bins = sbin[w];
  SmallTask* stack = sstack[w];
  uint32_t* tmp = stmp[w];
  int sp = 1;
  if (lane == 0) stack[0] = tasks[ti];
  __syncwarp();
  while (sp > 0) {
    const SmallTask task = stack[sp - 1];
    __syncwarp();
    sp--;
    const uint32_t n = task.count;
    // exact node box (double) and centroid bounds (float)
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    float cmn[3] = {3e38f, 3e38f, 3e38f}, cmx[3] = {-3e38f, -3e38f, -3e38f};
    for (uint32_t i = lane; i < n; i += 32) {
      const Box6 b = boxes[A[task.start + i]];
      for (int a = 0; a < 3; a++) {
        mn[a] = fmin(mn[a], b.mn[a]);
        mx[a] = fmax(mx[a], b.mx[a]);
        const float c = (float)((b.mn[a] + b.mx[a]) * 0.5);
        cmn[a] = fminf(cmn[a], c);
        cmx[a] = fmaxf(cmx[a], c);
      }
    }
    Box6 nb;
    for (int a = 0; a < 3; a++) {
      nb.mn[a] = warp_min_d(mn[a]);
      nb.mx[a] = warp_max_d(mx[a]);
      cmn[a] = fval(__reduce_min_sync(0xffffffffu, fkey(cmn[a])));
      cmx[a] = fval(__reduce_max_sync(0xffffffffu, fkey(cmx[a])));
    }
    if (lane == 0) node_box[task.node] = nb;
    bool leaf = n <= 3;
    int axis = -1, split = -1;
    uint32_t nleft = n / 2;
    if (!leaf) {
      for (int i = lane; i < 3 * NB; i += 32) {
        bins[i].n = 0;
        for (int a = 0; a < 3; a++) { bins[i].mn[a] = ~0u; bins[i].mx[a] = 0u; }
      }
      __syncwarp();
      for (uint32_t base = 0; base < n; base += 32) {
        const uint32_t i = base + lane;
        const bool on = i < n;
        Box6 b = box_empty();
        if (on) b = boxes[A[task.start + i]];
        for (int ax = 0; ax < 3; ax++) {
          float c = 0.0f;
          int bin = -1;
          if (on) {
            c = (float)((b.mn[ax] + b.mx[ax]) * 0.5);
            const float ext = cmx[ax] - cmn[ax];
            bin = ext > 0.0f ? min(NB - 1, max(0, (int)((c - cmn[ax]) * ((float)NB / ext)))) : 0;
          }
          const unsigned peers = __match_any_sync(0xffffffffu, bin);
          const uint32_t cnt = __popc(peers);
          uint32_t kmn[3], kmx[3];
          for (int a = 0; a < 3; a++) {
            kmn[a] = __reduce_min_sync(peers, on ? fkey((float)b.mn[a]) : ~0u);
            kmx[a] = __reduce_max_sync(peers, on ? fkey((float)b.mx[a]) : 0u);
          }
          if (on && lane == __ffs(peers) - 1) {
            FBin& x = bins[ax * NB + bin];
            x.n += cnt;
            for (int a = 0; a < 3; a++) { x.mn[a] = min(x.mn[a], kmn[a]); x.mx[a] = max(x.mx[a], kmx[a]); }
          }
          __syncwarp();
        }
      }
      // every lane evaluates candidate planes (axis, bin) = divmod(l, NB - 1) for
      // l = lane and lane + 32; the warp keeps the cheapest (lowest index on ties)
      double best = 1e300;
      int bl = 1 << 30;
      for (int l = lane; l < 3 * (NB - 1); l += 32) {
        const int ax = l / (NB - 1), sb = l % (NB - 1);
        float lmn[3] = {3e38f, 3e38f, 3e38f}, lmx[3] = {-3e38f, -3e38f, -3e38f};
        float rmn[3] = {3e38f, 3e38f, 3e38f}, rmx[3] = {-3e38f, -3e38f, -3e38f};
        uint32_t lc = 0, rc = 0;
        for (int bi = 0; bi < NB; bi++) {
          const FBin& x = bins[ax * NB + bi];
          if (!x.n) continue;
          float* mnp = bi <= sb ? lmn : rmn;
          float* mxp = bi <= sb ? lmx : rmx;
          for (int a2 = 0; a2 < 3; a2++) { mnp[a2] = fminf(mnp[a2], fval(x.mn[a2])); mxp[a2] = fmaxf(mxp[a2], fval(x.mx[a2])); }
          if (bi <= sb) lc += x.n; else rc += x.n;
        }
        if (!lc || !rc) continue;
        const float lx = lmx[0] - lmn[0], ly = lmx[1] - lmn[1], lz = lmx[2] - lmn[2];
        const float rx = rmx[0] - rmn[0], ry = rmx[1] - rmn[1], rz = rmx[2] - rmn[2];
        const double cost = (double)(lx * ly + ly * lz + lz * lx) * lc + (double)(rx * ry + ry * rz + rz * rx) * rc;
        if (cost < best) { best = cost; bl = l; }
      }
      for (int o = 16; o; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int ol = __shfl_xor_sync(0xffffffffu, bl, o);
        if (ob < best || (ob == best && ol < bl)) { best = ob; bl = ol; }
      }
      if (bl < (1 << 30)) {
        axis = bl / (NB - 1);
        split = bl % (NB - 1);
        uint32_t lc = 0;
        for (int bi = 0; bi <= split; bi++) lc += bins[axis * NB + bi].n;
        nleft = lc;
      } else {
        axis = -1;
        nleft = n / 2;
      }
      if (lane == 0 && n <= BIN_MAX_LEAF) {
        const double ex = nb.mx[0] - nb.mn[0], ey = nb.mx[1] - nb.mn[1], ez = nb.mx[2] - nb.mn[2];
        const double area = ex * ey + ey * ez + ez * ex;
        const double split_cost = axis >= 0 && area > 0.0 ? C_TRAV + best / area : 1e300;
        leaf = !(split_cost < (double)n);
      }
      leaf = __shfl_sync(0xffffffffu, leaf, 0);
      axis = __shfl_sync(0xffffffffu, axis, 0);
      split = __shfl_sync(0xffffffffu, split, 0);
      nleft = __shfl_sync(0xffffffffu, nleft, 0);
    }
    if (leaf) {
      if (lane == 0) {
        int32_t* p = nodes5 + 5 * (size_t)task.node;
        p[0] = -1;
        p[1] = (int32_t)((n << 24) | task.start);
      }
      continue;
    }
    uint32_t c = 0;
    if (lane == 0) c = atomicAdd(node_counter, 2u);
    c = __shfl_sync(0xffffffffu, c, 0);
    if (c + 1 >= max_nodes || sp + 2 > SMALL_STACK) {
      if (lane == 0) {
        atomicOr(err, ERR_BVH);
        int32_t* p = nodes5 + 5 * (size_t)task.node;
        p[0] = -1;
        p[1] = (int32_t)((min(n, 127u) << 24) | task.start);
      }
      continue;
    }
    // stable partition: left elements in order, then right elements in order
    uint32_t lbase = 0, rbase = nleft;
    for (uint32_t base = 0; base < n; base += 32) {
      const uint32_t i = base + lane;
      const bool on = i < n;
      bool left = false;
      uint32_t id = 0;
      if (on) {
        id = A[task.start + i];
        if (axis < 0) {
          left = i < nleft;
        } else {
          const Box6 b = boxes[id];
          const float cc = (float)((b.mn[axis] + b.mx[axis]) * 0.5);
          const float ext = cmx[axis] - cmn[axis];
          const int bin = ext > 0.0f ? min(NB - 1, max(0, (int)((cc - cmn[axis]) * ((float)NB / ext)))) : 0;
          left = bin <= split;
        }
      }
      const unsigned lm = __ballot_sync(0xffffffffu, on && left), rm = __ballot_sync(0xffffffffu, on && !left);
      const uint32_t below = (1u << lane) - 1u;
      if (on) {
        const uint32_t q = left ? lbase + __popc(lm & below) : rbase + __popc(rm & below);
        if (q < n) tmp[q] = id;
        else atomicOr(err, ERR_BVH);
      }
      lbase += __popc(lm);
      rbase += __popc(rm);
    }
    __syncwarp();
    if (lbase != nleft && lane == 0) atomicOr(err, ERR_BVH);
    for (uint32_t i = lane; i < n; i += 32) A[task.start + i] = tmp[i];
    if (lane == 0) {
      int32_t* p = nodes5 + 5 * (size_t)task.node;
      p[0] = (int32_t)c;
      p[1] = -1;
      stack[sp] = SmallTask{task.start + nleft, n - nleft, c + 1};
      stack[sp + 1] = SmallTask{task.start, nleft, c};
    }
    sp += 2;
    __syncwarp();
  }
}

__global__ void k_init_bins(Bin* bins, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) bin_clear(bins[i]);
}

}  // namespace

int build_bvh_binned(cudaStream_t s, const double* pos3, uint32_t n_verts, const int4* tri4, uint32_t T,
                     BvhOut& out, std::string& why) {
  if (T == 0) { why = "no triangles"; return 1; }
  if (T >= (1u << 24)) { why = "too many triangles for the 24-bit leaf base"; return 1; }
  const uint32_t max_nodes = 2 * T;
  DevBuf<Box6> tri_box(T), node_box(max_nodes);
  DevBuf<uint32_t> A(T), A2(T), flags(T), X(T), counter(1), derr(1);
  DevBuf<int32_t> nodes5(5 * (size_t)max_nodes);
  DevBuf<Bin> root_bin(1);
  check(cudaMemsetAsync(derr.p, 0, 4, s), "memset");
  k_tri_boxes_plain<<<blocks(T), 256, 0, s>>>(pos3, tri4, T, tri_box.p, A.p);
  k_init_bins<<<1, 32, 0, s>>>(root_bin.p, 1);
  k_root_bounds<<<std::min<unsigned>(blocks(T), 1024u), 256, 0, s>>>(tri_box.p, T, root_bin.p);
  check(cudaGetLastError(), "binned roots");
  Bin rb;
  check(cudaMemcpyAsync(&rb, root_bin.p, sizeof(Bin), cudaMemcpyDeviceToHost, s), "D2H");
  check(cudaStreamSynchronize(s), "sync");
  auto hval = [](unsigned long long k) {
    const unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    double d;
    std::memcpy(&d, &u, 8);
    return d;
  };
  Box6 root;
  for (int a = 0; a < 3; a++) { root.mn[a] = hval(rb.bmin[a]); root.mx[a] = hval(rb.bmax[a]); }
  check(cudaMemcpyAsync(node_box.p, &root, sizeof(Box6), cudaMemcpyHostToDevice, s), "H2D");

  std::vector<NodeInfo> large;
  std::vector<SmallTask> small;
  uint32_t next = 1;
  {
    NodeInfo r{};
    r.start = 0; r.count = T; r.node = 0;
    for (int a = 0; a < 3; a++) { r.cmin[a] = hval(rb.cmin[a]); r.cmax[a] = hval(rb.cmax[a]); }
    if (T > BIN_SMALL) large.push_back(r);
    else small.push_back(SmallTask{0, T, 0});
  }
  // per-level buffers at their largest: every large node holds more than BIN_SMALL triangles
  const uint32_t m_max = T / BIN_SMALL + 2;
  DevBuf<NodeInfo> d_nodes(m_max);
  DevBuf<Tile> d_tiles(T / BIN_TILE + m_max + 1);
  DevBuf<Bin> bins((size_t)m_max * 3 * NB);
  uint32_t depth = 1;
  while (!large.empty()) {
    depth++;
    const uint32_t m = (uint32_t)large.size();
    std::vector<Tile> tiles;
    for (uint32_t k = 0; k < m; k++)
      for (uint32_t b = 0; b < large[k].count; b += BIN_TILE)
        tiles.push_back(Tile{k, large[k].start + b, std::min<uint32_t>(BIN_TILE, large[k].count - b)});
    if (m > m_max || tiles.size() > d_tiles.n) { why = "internal: level buffers too small"; return 1; }
    check(cudaMemcpyAsync(d_nodes.p, large.data(), m * sizeof(NodeInfo), cudaMemcpyHostToDevice, s), "H2D");
    check(cudaMemcpyAsync(d_tiles.p, tiles.data(), tiles.size() * sizeof(Tile), cudaMemcpyHostToDevice, s), "H2D");
    k_init_bins<<<(unsigned)(((size_t)m * 3 * NB + 255) / 256), 256, 0, s>>>(bins.p, (size_t)m * 3 * NB);
    k_bin_tiles<<<(unsigned)tiles.size(), BIN_THREADS, 0, s>>>(d_tiles.p, d_nodes.p, A.p, tri_box.p, bins.p);
    if (next + 2 * m > max_nodes) { why = "node budget exceeded"; return 1; }
    k_choose_large<<<blocks(m, 64), 64, 0, s>>>(d_nodes.p, m, bins.p, next, nodes5.p, node_box.p);
    check(cudaMemsetAsync(flags.p, 0, (size_t)T * 4, s), "memset");
    k_left_flags_binned<<<(unsigned)tiles.size(), BIN_THREADS, 0, s>>>(d_tiles.p, d_nodes.p, A.p, tri_box.p, flags.p);
    scan_exclusive_u32(s, flags.p, X.p, T, nullptr);
    check(cudaMemcpyAsync(A2.p, A.p, (size_t)T * 4, cudaMemcpyDeviceToDevice, s), "memcpy");
    k_partition_binned<<<(unsigned)tiles.size(), BIN_THREADS, 0, s>>>(d_tiles.p, d_nodes.p, A.p, flags.p, X.p, A2.p,
                                                                      derr.p);
    check(cudaGetLastError(), "binned level");
    std::swap(A.p, A2.p);
    check(cudaMemcpyAsync(large.data(), d_nodes.p, m * sizeof(NodeInfo), cudaMemcpyDeviceToHost, s), "D2H");
    uint32_t lerr = 0;
    check(cudaMemcpyAsync(&lerr, derr.p, 4, cudaMemcpyDeviceToHost, s), "D2H");
    check(cudaStreamSynchronize(s), "sync");
    if (lerr) { why = "binned partition out of range"; return 1; }
    std::vector<NodeInfo> nl;
    for (uint32_t k = 0; k < m; k++) {
      const NodeInfo& p = large[k];
      const uint32_t c = next + 2 * k;
      NodeInfo L{}, R{};
      L.start = p.start; L.count = p.nleft; L.node = c;
      R.start = p.start + p.nleft; R.count = p.count - p.nleft; R.node = c + 1;
      for (int a = 0; a < 3; a++) {
        L.cmin[a] = p.lcmin[a]; L.cmax[a] = p.lcmax[a];
        R.cmin[a] = p.rcmin[a]; R.cmax[a] = p.rcmax[a];
      }
      for (const NodeInfo& q : {L, R}) {
        if (q.count == 0) { why = "empty child"; return 1; }
        if (q.count > BIN_SMALL) nl.push_back(q);
        else small.push_back(SmallTask{q.start, q.count, q.node});
      }
    }
    next += 2 * m;
    large.swap(nl);
  }
  check(cudaMemcpyAsync(counter.p, &next, 4, cudaMemcpyHostToDevice, s), "H2D");
  if (!small.empty()) {
    DevBuf<SmallTask> d_small(small.size());
    check(cudaMemcpyAsync(d_small.p, small.data(), small.size() * sizeof(SmallTask), cudaMemcpyHostToDevice, s), "H2D");
    const unsigned nb = (unsigned)((small.size() + SMALL_WARPS - 1) / SMALL_WARPS);
    k_build_small<<<nb, SMALL_WARPS * 32, 0, s>>>(d_small.p, (uint32_t)small.size(), A.p, tri_box.p, nodes5.p,
                                                 node_box.p, counter.p, max_nodes, derr.p);
    check(cudaGetLastError(), "k_build_small");
  }
  uint32_t n_nodes = 0, herr = 0;
  check(cudaMemcpyAsync(&n_nodes, counter.p, 4, cudaMemcpyDeviceToHost, s), "D2H");
  check(cudaMemcpyAsync(&herr, derr.p, 4, cudaMemcpyDeviceToHost, s), "D2H");
  check(cudaStreamSynchronize(s), "sync");
  if (herr) { why = "binned build ran out of node or stack budget"; return 1; }

  double span[3], center[3];
  for (int i = 0; i < 3; i++) span[i] = root.mx[i] - root.mn[i];
  const double longest = js_max(js_max(span[0], span[1]), span[2]);
  for (int i = 0; i < 3; i++) center[i] = root.mn[i] + span[i] * 0.5;
  out.nodes5.alloc(5 * (size_t)n_nodes);
  check(cudaMemcpyAsync(out.nodes5.p, nodes5.p, 5 * (size_t)n_nodes * 4, cudaMemcpyDeviceToDevice, s), "memcpy");
  k_quantize_nodes<<<blocks(n_nodes), 256, 0, s>>>(n_nodes, node_box.p, center[0], center[1], center[2], longest,
                                                    out.nodes5.p);
  out.verts4.alloc(n_verts);
  k_norm_verts<<<blocks(n_verts), 256, 0, s>>>(pos3, n_verts, center[0], center[1], center[2], longest, out.verts4.p);
  out.tri4_leaf.alloc(T);
  k_gather_tris<<<blocks(T), 256, 0, s>>>(tri4, reinterpret_cast<const int32_t*>(A.p), T, out.tri4_leaf.p);
  out.node_box.alloc(6 * (size_t)n_nodes);
  check(cudaMemcpyAsync(out.node_box.p, node_box.p, (size_t)n_nodes * sizeof(Box6), cudaMemcpyDeviceToDevice, s),
        "memcpy");
  check(cudaGetLastError(), "binned pack");
  check(cudaStreamSynchronize(s), "sync");
  out.n_nodes = n_nodes;
  out.n_leaf_tris = T;
  out.depth = depth;
  for (int i = 0; i < 3; i++) out.norm[i] = center[i];
  out.norm[3] = 2.0 / longest;
  return 0;
}

}  // namespace pk
