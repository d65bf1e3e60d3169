// pk_wide.cu -- form (1)'s structures built on the GPU from the binary BVH
// (record layouts in pk_wide.h): the compressed 8-wide BVH and the FP32
// binary reference's outward-rounded records.
//
// Inputs are the drop-in's device arrays (binary nodes with children after
// their parents, the leaf-ordered triangle indices, normalised vertices).
// Every step works one tree level at a time (the level's node list built top
// down by a prefix sum) with one thread per node, in double precision where
// boxes are formed:
//   1. triangle boxes over the three vertices and the 48-byte triangle
//      records of the binary leaf order (slot = leaf-order index);
//   2. node boxes bottom up (leaf: union of its triangles, inner: union of
//      its children), then widened by a margin of 2^-18 max(1, |x|);
//   3. the SAH-optimal collapse of Ylitie, Karras & Laine ("Efficient
//      Incoherent Ray Traversal on GPUs Through Compressed Wide BVHs", HPG
//      2017, section 3.1), bottom up: for every binary node n and slot budget
//      i (1..8) the cheapest representation of n's subtree as at most i
//      children of a wide node -- one leaf child (at most three triangles),
//      one internal child (a wide node), or (i >= 2) its two children sharing
//      the i slots -- with unit cost per wide-node visit and 0.3 per triangle
//      test, each weighted by the surface area of the box tested;
//   4. top down, wide nodes one level at a time: the children the collapse
//      chose (a binary leaf of more than three triangles is halved,
//      largest area first, as if it were inner), octant slots assigned
//      greedily (the child whose centroid lies furthest against an octant
//      takes that octant's slot), the child boxes quantised outward to 8 bits
//      against an FP32 frame (each bound checked against the device decode),
//      and a prefix sum over the level placing every node's internal
//      children and triangle records after all earlier ones.
// The result is fully determined by the inputs (no atomics decide an order).
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "pk_util.h"
#include "pk_wide.h"

namespace pk {
namespace {

struct BoxD {
  double lo[3], hi[3];
};

__device__ __forceinline__ BoxD box_empty() {
  BoxD b;
  for (int a = 0; a < 3; a++) {
    b.lo[a] = INFINITY;
    b.hi[a] = -INFINITY;
  }
  return b;
}
__device__ __forceinline__ void box_add(BoxD& b, double x, double y, double z) {
  const double v[3] = {x, y, z};
  for (int a = 0; a < 3; a++) {
    b.lo[a] = v[a] < b.lo[a] ? v[a] : b.lo[a];
    b.hi[a] = b.hi[a] < v[a] ? v[a] : b.hi[a];
  }
}
__device__ __forceinline__ void box_add(BoxD& b, const BoxD& o) {
  for (int a = 0; a < 3; a++) {
    b.lo[a] = o.lo[a] < b.lo[a] ? o.lo[a] : b.lo[a];
    b.hi[a] = b.hi[a] < o.hi[a] ? o.hi[a] : b.hi[a];
  }
}
__device__ __forceinline__ bool box_is_empty(const BoxD& b) {
  return !(b.lo[0] <= b.hi[0] && b.lo[1] <= b.hi[1] && b.lo[2] <= b.hi[2]);
}
__device__ __forceinline__ double box_area(const BoxD& b) {
  if (box_is_empty(b)) return 0.0;
  const double x = b.hi[0] - b.lo[0], y = b.hi[1] - b.lo[1], z = b.hi[2] - b.lo[2];
  return x * y + y * z + z * x;
}
__device__ __forceinline__ double box_centre(const BoxD& b, int a) {
  return box_is_empty(b) ? 0.0 : 0.5 * (b.lo[a] + b.hi[a]);
}
constexpr double MARGIN = 0x1p-18;
__device__ __forceinline__ void widen(BoxD& b) {
  for (int a = 0; a < 3; a++) {
    if (!(b.lo[a] <= b.hi[a])) continue;  // empty: never hit
    b.lo[a] -= MARGIN * fmax(1.0, fabs(b.lo[a]));
    b.hi[a] += MARGIN * fmax(1.0, fabs(b.hi[a]));
  }
}
// Largest float not above x / smallest float not below x.
__device__ __forceinline__ float f_down(double x) {
  float f = __double2float_rn(x);
  if ((double)f > x) f = nextafterf(f, -INFINITY);
  return f;
}
__device__ __forceinline__ float f_up(double x) {
  float f = __double2float_rn(x);
  if ((double)f < x) f = nextafterf(f, INFINITY);
  return f;
}
// The traversal's decode of a plane: one exact product (q has 8 bits, s is a
// power of two) and one rounded FP32 add.
__device__ __forceinline__ float decode(float p, float s, int q) {
  const float m = __fmul_rn(s, (float)q);
  return __fadd_rn(p, m);
}

constexpr uint32_t LEAF_MAX = 3;
// Triangle cost relative to a wide-node visit (1080p frame through the wide
// traversal: 0.15 3309 Mrays/s, 0.3 3334-3341, 0.6 3204-3208, 1.0 3201-3205,
// 2.0 3216-3220).
constexpr float COST_NODE = 1.0f, COST_TRI = 0.3f;
constexpr uint8_t OPT_LEAF = 0xf0, OPT_INNER = 0xf1;  // else: split, j slots to the left child
constexpr uint32_t E_VERTEX = 1, E_LEAF = 2, E_ORDER = 4, E_FIT = 8;

// A child candidate of a wide node: a binary inner node (kind 0), a range of
// leaf-ordered triangles (1), or a binary subtree of at most LEAF_MAX
// triangles taken as one leaf child (2).
struct Item {
  uint32_t kind, a, n;
};

// 1. triangle boxes and binary-order triangle records
__global__ void k_tri_data(const int4* __restrict__ tri4, uint32_t n_tris, const float4* __restrict__ verts4,
                           uint32_t n_verts, BoxD* __restrict__ tbox, float* __restrict__ recs, uint32_t* err) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tris) return;
  const int4 tr = tri4[t];
  const int idx[3] = {tr.x, tr.y, tr.z};
  float r[WIDE_TRI_FLOATS];
  for (int k = 0; k < WIDE_TRI_FLOATS; k++) r[k] = 0.0f;
  BoxD b = box_empty();
  for (int k = 0; k < 3; k++) {
    if (idx[k] < 0 || (uint32_t)idx[k] >= n_verts) {
      atomicOr(err, E_VERTEX);
      continue;
    }
    const float4 v = verts4[idx[k]];
    r[3 * k] = v.x;
    r[3 * k + 1] = v.y;
    r[3 * k + 2] = v.z;
    box_add(b, v.x, v.y, v.z);
  }
  r[9] = __uint_as_float(t);
  for (int k = 0; k < WIDE_TRI_FLOATS; k++) recs[(size_t)WIDE_TRI_FLOATS * t + k] = r[k];
  tbox[t] = b;
}

// 2. node boxes of one level (children already done)
__global__ void k_node_boxes(const int32_t* __restrict__ nodes5, const uint32_t* __restrict__ order, uint32_t b,
                             uint32_t e, uint32_t n_tris, const BoxD* __restrict__ tbox, BoxD* __restrict__ nbox,
                             uint32_t* err) {
  const uint32_t k = b + blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= e) return;
  const uint32_t i = order[k];
  const int32_t* nd = nodes5 + 5 * (size_t)i;
  BoxD bx = box_empty();
  if (nd[1] > -1) {
    const uint32_t w = (uint32_t)nd[1];
    const uint32_t size = w >> 24, base = w & 0x00ffffffu;
    if (size >= 128u || (uint64_t)base + size > n_tris) {
      atomicOr(err, E_LEAF);
    } else {
      for (uint32_t k = 0; k < size; k++) box_add(bx, tbox[base + k]);
    }
  } else {
    const uint32_t l = (uint32_t)nd[0];
    bx = nbox[l];
    box_add(bx, nbox[l + 1]);
  }
  nbox[i] = bx;
}
__global__ void k_widen(BoxD* __restrict__ box, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) widen(box[i]);
}

// 3. the collapse's dynamic programme for one level
__global__ void k_collapse(const int32_t* __restrict__ nodes5, const uint32_t* __restrict__ order, uint32_t b,
                           uint32_t e, const BoxD* __restrict__ nbox, float* __restrict__ cost,
                           uint8_t* __restrict__ opt, uint8_t* __restrict__ split, uint32_t* __restrict__ tris) {
  const uint32_t k = b + blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= e) return;
  const uint32_t n = order[k];
  const int32_t* nd = nodes5 + 5 * (size_t)n;
  float* C = cost + 8 * (size_t)n;
  uint8_t* O = opt + 8 * (size_t)n;
  const double area = box_area(nbox[n]);
  const float INF = INFINITY;
  if (nd[1] > -1) {
    const uint32_t t = (uint32_t)nd[1] >> 24;
    tris[n] = t;
    split[n] = 1;
    const float leaf = t <= LEAF_MAX ? __double2float_rn(area * (double)COST_TRI * (double)t) : INF;
    const float per = __fadd_rn(COST_NODE, __fmul_rn(COST_TRI, (float)t));  // in binary32, then times the area
    const float inner = t > LEAF_MAX ? __double2float_rn(area * (double)per) : INF;
    for (int i = 0; i < 8; i++) {
      C[i] = fminf(leaf, inner);
      O[i] = leaf <= inner ? OPT_LEAF : OPT_INNER;
    }
    return;
  }
  const uint32_t l = (uint32_t)nd[0], r = l + 1;
  tris[n] = tris[l] + tris[r];
  const float* Cl = cost + 8 * (size_t)l;
  const float* Cr = cost + 8 * (size_t)r;
  float D[8];
  uint8_t J[8];
  D[0] = INF;
  J[0] = 1;
  for (int i = 2; i <= 8; i++) {  // i slots, j of them to the left
    float best = INF;
    uint8_t bj = 1;
    for (int j = 1; j < i; j++) {
      const float c = __fadd_rn(Cl[j - 1], Cr[i - j - 1]);
      if (c < best) { best = c; bj = (uint8_t)j; }
    }
    D[i - 1] = best;
    J[i - 1] = bj;
  }
  split[n] = J[7];
  const float leaf = tris[n] <= LEAF_MAX ? __double2float_rn(area * (double)COST_TRI * (double)tris[n]) : INF;
  const float inner = __fadd_rn(__double2float_rn(area * (double)COST_NODE), D[7]);
  float c0 = fminf(leaf, inner);
  uint8_t o0 = leaf <= inner ? OPT_LEAF : OPT_INNER;
  C[0] = c0;
  O[0] = o0;
  for (int i = 1; i < 8; i++) {
    if (D[i] < c0) { c0 = D[i]; o0 = J[i]; }
    C[i] = c0;
    O[i] = o0;
  }
}

struct BuildView {
  const int32_t* nodes5;
  const BoxD* tbox;
  const BoxD* nbox;  // widened
  const uint8_t* opt;
  const uint8_t* split;
  const uint32_t* tris;
};

__device__ __forceinline__ bool is_leaf(const BuildView& V, uint32_t n) { return V.nodes5[5 * (size_t)n + 1] > -1; }
__device__ __forceinline__ Item item_of(const BuildView& V, uint32_t node) {
  const int32_t t = V.nodes5[5 * (size_t)node + 1];
  if (t > -1) return Item{1u, (uint32_t)t & 0x00ffffffu, (uint32_t)t >> 24};
  return Item{0u, node, 0u};
}
__device__ __forceinline__ BoxD box_of(const BuildView& V, const Item& it) {
  if (it.kind != 1) return V.nbox[it.a];
  BoxD b = box_empty();
  for (uint32_t k = 0; k < it.n; k++) box_add(b, V.tbox[it.a + k]);
  widen(b);
  return b;
}
__device__ __forceinline__ bool openable(const Item& it) { return it.kind == 0 || (it.kind == 1 && it.n > LEAF_MAX); }

// The leaf-ordered triangles of a leaf child, in order.
__device__ void leaf_tris(const BuildView& V, const Item& it, uint32_t (&out)[LEAF_MAX], uint32_t& count) {
  count = 0;
  if (it.kind == 1) {
    for (uint32_t k = 0; k < it.n && count < LEAF_MAX; k++) out[count++] = it.a + k;
    return;
  }
  uint32_t stack[64];
  int sp = 0;
  stack[sp++] = it.a;
  while (sp) {
    const uint32_t n = stack[--sp];
    const int32_t* nd = V.nodes5 + 5 * (size_t)n;
    if (nd[1] > -1) {
      const uint32_t w = (uint32_t)nd[1];
      for (uint32_t k = 0; k < (w >> 24) && count < LEAF_MAX; k++) out[count++] = (w & 0x00ffffffu) + k;
    } else if (sp + 2 <= 64) {
      stack[sp++] = (uint32_t)nd[0] + 1;
      stack[sp++] = (uint32_t)nd[0];
    }
  }
}

// The children that binary node n's subtree contributes with a budget of i
// slots (the collapse's decisions, left subtree first).
__device__ void collect(const BuildView& V, uint32_t n0, int i0, Item* ch, int& nc) {
  uint32_t sn[16];
  int si[16];
  int sp = 0;
  sn[sp] = n0;
  si[sp++] = i0;
  while (sp && nc < 8) {
    --sp;
    const uint32_t n = sn[sp];
    const int i = si[sp];
    const uint8_t o = V.opt[8 * (size_t)n + (i - 1)];
    if (o == OPT_LEAF) {
      ch[nc++] = is_leaf(V, n) ? item_of(V, n) : Item{2u, n, V.tris[n]};
    } else if (o == OPT_INNER) {
      ch[nc++] = item_of(V, n);
    } else if (sp + 2 <= 16) {
      const uint32_t l = (uint32_t)V.nodes5[5 * (size_t)n];
      sn[sp] = l + 1;
      si[sp++] = i - o;
      sn[sp] = l;
      si[sp++] = o;
    }
  }
}

// Children of the wide node for `it` (at most 8) in slot order (empty slots:
// kind 1, n 0), their boxes and the used slots.
__device__ void children(const BuildView& V, const Item& it, Item (&slot)[8], BoxD (&sbox)[8], bool (&used)[8]) {
  Item ch[8];
  BoxD cb[8];
  int nc = 0;
  if (it.kind == 0) {
    const uint32_t l = (uint32_t)V.nodes5[5 * (size_t)it.a];
    const int j = V.split[it.a];
    collect(V, l, j, ch, nc);
    collect(V, l + 1, 8 - j, ch, nc);
  } else if (openable(it)) {  // a long range: halves, opened largest first
    const uint32_t h = it.n / 2;
    ch[0] = Item{1u, it.a, h};
    ch[1] = Item{1u, it.a + h, it.n - h};
    nc = 2;
    while (nc < 8) {
      int best = -1;
      double best_a = -1.0;
      for (int k = 0; k < nc; k++) {
        if (!openable(ch[k])) continue;
        const double a = box_area(box_of(V, ch[k]));
        if (a > best_a) { best_a = a; best = k; }
      }
      if (best < 0) break;
      const Item o = ch[best];
      for (int k = nc; k > best + 1; k--) ch[k] = ch[k - 1];
      ch[best] = Item{1u, o.a, o.n / 2};
      ch[best + 1] = Item{1u, o.a + o.n / 2, o.n - o.n / 2};
      nc++;
    }
  } else {
    ch[0] = it;
    nc = 1;
  }
  for (int k = 0; k < nc; k++) cb[k] = box_of(V, ch[k]);
  BoxD all = box_empty();
  for (int k = 0; k < nc; k++) box_add(all, cb[k]);
  double cost[8][8];
  for (int k = 0; k < nc; k++) {
    const double dx = box_centre(cb[k], 0) - box_centre(all, 0), dy = box_centre(cb[k], 1) - box_centre(all, 1),
                 dz = box_centre(cb[k], 2) - box_centre(all, 2);
    for (int s = 0; s < 8; s++) cost[k][s] = ((s & 1) ? -dx : dx) + ((s & 2) ? -dy : dy) + ((s & 4) ? -dz : dz);
  }
  bool cdone[8];
  for (int s = 0; s < 8; s++) {
    cdone[s] = false;
    used[s] = false;
  }
  for (int round = 0; round < nc; round++) {
    int bk = -1, bs = -1;
    double bc = INFINITY;
    for (int k = 0; k < nc; k++) {
      if (cdone[k]) continue;
      for (int s = 0; s < 8; s++)
        if (!used[s] && (bk < 0 || cost[k][s] < bc)) {
          bc = cost[k][s];
          bk = k;
          bs = s;
        }
    }
    cdone[bk] = true;
    used[bs] = true;
    slot[bs] = ch[bk];
    sbox[bs] = cb[bk];
  }
  for (int s = 0; s < 8; s++)
    if (!used[s]) slot[s] = Item{1u, 0u, 0u};
}

// 4a. internal children and triangles of every wide node of a level
__global__ void k_wide_count(BuildView V, const Item* __restrict__ items, uint32_t n, uint32_t* __restrict__ n_inner,
                             uint32_t* __restrict__ n_tri) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Item slot[8];
  BoxD sbox[8];
  bool used[8];
  children(V, items[i], slot, sbox, used);
  uint32_t ni = 0, nt = 0;
  for (int s = 0; s < 8; s++) {
    if (!used[s]) continue;
    if (openable(slot[s])) ni++;
    else nt += slot[s].n;
  }
  n_inner[i] = ni;
  n_tri[i] = nt;
}

// ceil(log2(x)) for x > 0, exactly (frexp: x = m 2^k, m in [0.5, 1)).
__device__ __forceinline__ int ceil_log2(double x) {
  int k;
  const double m = frexp(x, &k);
  return m == 0.5 ? k - 1 : k;
}

// 4b. the node records of a level, their triangle records and the next level's items
__global__ void k_wide_write(BuildView V, const Item* __restrict__ items, uint32_t n, uint32_t node_base,
                             const uint32_t* __restrict__ child_off, const uint32_t* __restrict__ tri_off,
                             uint32_t tri_base, const float* __restrict__ brecs, float* __restrict__ nodes_out,
                             float* __restrict__ tris_out, Item* __restrict__ next, uint32_t* err) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Item slot[8];
  BoxD sbox[8];
  bool used[8];
  children(V, items[i], slot, sbox, used);
  const uint32_t child0 = node_base + n + child_off[i];
  const uint32_t tri0 = tri_base + tri_off[i];
  uint8_t q[6][8], meta[8];
  for (int s = 0; s < 8; s++) {
    meta[s] = 0;
    for (int a = 0; a < 6; a++) q[a][s] = 0;
  }
  BoxD all = box_empty();
  for (int s = 0; s < 8; s++)
    if (used[s]) box_add(all, sbox[s]);
  float org[3];
  int ex[3];
  for (int a = 0; a < 3; a++) {
    double lo = all.lo[a], hi = all.hi[a];
    if (!(lo <= hi)) { lo = 0.0; hi = 0.0; }
    org[a] = f_down(lo);
    const double ext = hi - (double)org[a];
    int e2 = ext > 0.0 ? ceil_log2(ext / 255.0) : -100;
    e2 = max(-100, min(e2, 127));
    while (e2 < 127 && (double)decode(org[a], ldexpf(1.0f, e2), 255) < hi) e2++;
    ex[a] = e2;
  }
  uint32_t imask = 0, inner_rank = 0, toff = 0;
  bool fit = true;
  for (int s = 0; s < 8; s++) {
    if (!used[s]) continue;
    const Item& c = slot[s];
    if (openable(c)) {
      imask |= 1u << s;
      meta[s] = (uint8_t)(0x20u | (uint32_t)s);
      next[child0 - node_base - n + inner_rank] = c;
      inner_rank++;
    } else {
      if (c.n == 0) continue;
      uint32_t ids[LEAF_MAX], cnt = 0;
      leaf_tris(V, c, ids, cnt);
      meta[s] = (uint8_t)((((1u << cnt) - 1u) << 5) | toff);
      for (uint32_t k = 0; k < cnt; k++)
        for (int f = 0; f < WIDE_TRI_FLOATS; f++)
          tris_out[(size_t)WIDE_TRI_FLOATS * (tri0 + toff + k) + f] = brecs[(size_t)WIDE_TRI_FLOATS * ids[k] + f];
      toff += cnt;
    }
    const BoxD& cb = sbox[s];
    if (box_is_empty(cb)) continue;  // all-zero planes at the frame origin: no triangles
    for (int a = 0; a < 3; a++) {
      const float sc = ldexpf(1.0f, ex[a]);
      int lo = (int)floor((cb.lo[a] - (double)org[a]) / (double)sc);
      lo = max(0, min(lo, 255));
      while (lo > 0 && (double)decode(org[a], sc, lo) > cb.lo[a]) lo--;
      int hi = (int)ceil((cb.hi[a] - (double)org[a]) / (double)sc);
      hi = max(0, min(hi, 255));
      while (hi < 255 && (double)decode(org[a], sc, hi) < cb.hi[a]) hi++;
      if ((double)decode(org[a], sc, lo) > cb.lo[a] || (double)decode(org[a], sc, hi) < cb.hi[a]) fit = false;
      q[a][s] = (uint8_t)lo;
      q[3 + a][s] = (uint8_t)hi;
    }
  }
  if (!fit) atomicOr(err, E_FIT);
  uint32_t rec[WIDE_NODE_FLOATS];
  rec[0] = __float_as_uint(org[0]);
  rec[1] = __float_as_uint(org[1]);
  rec[2] = __float_as_uint(org[2]);
  rec[3] = (uint32_t)(ex[0] + 127) | ((uint32_t)(ex[1] + 127) << 8) | ((uint32_t)(ex[2] + 127) << 16) | (imask << 24);
  rec[4] = inner_rank ? child0 : 0u;
  rec[5] = tri0;
  auto pack = [](const uint8_t* b) {
    return (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24);
  };
  rec[6] = pack(meta);
  rec[7] = pack(meta + 4);
  // qlo.x qlo.y | qlo.z qhi.x | qhi.y qhi.z
  for (int a = 0; a < 6; a++) {
    rec[8 + 2 * a] = pack(q[a]);
    rec[9 + 2 * a] = pack(q[a] + 4);
  }
  uint32_t* out = reinterpret_cast<uint32_t*>(nodes_out) + (size_t)WIDE_NODE_FLOATS * (node_base + i);
  for (int k = 0; k < WIDE_NODE_FLOATS; k++) out[k] = rec[k];
}

// FP32 binary reference: per inner node its children's widened boxes rounded
// outward ({hi, lo} per axis; an empty child a point at 1e30) and child codes.
__global__ void k_inner_flags(const int32_t* __restrict__ nodes5, uint32_t n, uint32_t* __restrict__ flag) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flag[i] = nodes5[5 * (size_t)i + 1] <= -1 ? 1u : 0u;
}
__device__ __forceinline__ int32_t node_code(const int32_t* nodes5, const uint32_t* rank, uint32_t i) {
  const int32_t t = nodes5[5 * (size_t)i + 1];
  return t > -1 ? (int32_t)(0x80000000u | (uint32_t)t) : (int32_t)rank[i];
}
__device__ __forceinline__ void put_box(float* r, const BoxD& b) {
  for (int a = 0; a < 3; a++) {
    const bool empty = !(b.lo[a] <= b.hi[a]);
    r[2 * a] = empty ? 1e30f : f_up(b.hi[a]);
    r[2 * a + 1] = empty ? 1e30f : f_down(b.lo[a]);
  }
}
__global__ void k_exact_records(const int32_t* __restrict__ nodes5, uint32_t n, const uint32_t* __restrict__ rank,
                                const BoxD* __restrict__ nbox, float* __restrict__ records, int32_t* root_code) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) *root_code = node_code(nodes5, rank, 0);
  if (i >= n || nodes5[5 * (size_t)i + 1] > -1) return;
  const uint32_t l = (uint32_t)nodes5[5 * (size_t)i];
  float r[16];
  put_box(r, nbox[l]);
  put_box(r + 6, nbox[l + 1]);
  r[12] = __int_as_float(node_code(nodes5, rank, l));
  r[13] = __int_as_float(node_code(nodes5, rank, l + 1));
  r[14] = 0.0f;
  r[15] = 0.0f;
  for (int k = 0; k < 16; k++) records[16 * (size_t)rank[i] + k] = r[k];
}

unsigned blocks(uint32_t n, unsigned t = 128) { return (unsigned)std::max<uint32_t>(1u, (n + t - 1) / t); }

uint32_t read_u32(cudaStream_t s, const uint32_t* p) {
  uint32_t v = 0;
  check(cudaMemcpyAsync(&v, p, 4, cudaMemcpyDeviceToHost, s), "D2H");
  check(cudaStreamSynchronize(s), "sync");
  return v;
}

const char* error_text(uint32_t e) {
  if (e & E_VERTEX) return "triangle vertex index out of range";
  if (e & E_LEAF) return "leaf outside the triangle array";
  if (e & E_ORDER) return "malformed binary tree (a child not after its parent, or a node not reached once)";
  if (e & E_FIT) return "child box does not fit its 8-bit frame";
  return "internal error";
}

// Steps 1 and 2, shared by both builds: the levels (node lists), triangle
// boxes and records, widened node boxes.
struct Prepared {
  std::vector<uint32_t> level;  // level d = order[level[d], level[d + 1])
  DevBuf<uint32_t> order;
  DevBuf<BoxD> tbox, nbox;
  DevBuf<float> brecs;
};
int prepare(cudaStream_t s, const int32_t* nodes5, uint32_t n_nodes, const int4* tri4, uint32_t n_tris,
            const float4* verts4, uint32_t n_verts, DevBuf<uint32_t>& err, Prepared& P, std::string& why) {
  P.tbox.alloc(std::max<uint32_t>(n_tris, 1u));
  P.brecs.alloc((size_t)WIDE_TRI_FLOATS * std::max<uint32_t>(n_tris, 1u));
  P.nbox.alloc(n_nodes);
  if (n_tris) k_tri_data<<<blocks(n_tris), 128, 0, s>>>(tri4, n_tris, verts4, n_verts, P.tbox.p, P.brecs.p, err.p);
  if (tree_levels(s, nodes5, n_nodes, P.order, P.level)) { why = error_text(E_ORDER); return 1; }
  if (uint32_t ev = read_u32(s, err.p)) { why = error_text(ev); return 1; }
  for (size_t d = P.level.size() - 1; d-- > 0;)
    k_node_boxes<<<blocks(P.level[d + 1] - P.level[d]), 128, 0, s>>>(nodes5, P.order.p, P.level[d], P.level[d + 1],
                                                                      n_tris, P.tbox.p, P.nbox.p, err.p);
  k_widen<<<blocks(n_nodes), 128, 0, s>>>(P.nbox.p, n_nodes);
  check(cudaGetLastError(), "form (1) boxes");
  if (uint32_t ev = read_u32(s, err.p)) { why = error_text(ev); return 1; }
  return 0;
}

}  // namespace

int build_wide_bvh_gpu(cudaStream_t s, const int32_t* nodes5, uint32_t n_nodes, const int4* tri4, uint32_t n_tris,
                       const float4* verts4, uint32_t n_verts, DevBuf<float4>& nodes_out, DevBuf<float4>& tris_out,
                       uint32_t& n_wide, uint32_t& depth, std::string& why) {
  if (n_nodes == 0) { why = "empty BVH"; return 1; }
  DevBuf<uint32_t> err(1);
  check(cudaMemsetAsync(err.p, 0, 4, s), "memset");
  Prepared P;
  if (prepare(s, nodes5, n_nodes, tri4, n_tris, verts4, n_verts, err, P, why)) return 1;
  DevBuf<float> cost(8 * (size_t)n_nodes);
  DevBuf<uint8_t> opt(8 * (size_t)n_nodes), split(n_nodes);
  DevBuf<uint32_t> ntri(n_nodes);
  for (size_t d = P.level.size() - 1; d-- > 0;)
    k_collapse<<<blocks(P.level[d + 1] - P.level[d]), 128, 0, s>>>(nodes5, P.order.p, P.level[d], P.level[d + 1],
                                                                    P.nbox.p, cost.p, opt.p, split.p, ntri.p);
  check(cudaGetLastError(), "k_collapse");
  const BuildView V{nodes5, P.tbox.p, P.nbox.p, opt.p, split.p, ntri.p};
  // top down; node capacity grows geometrically
  size_t cap = std::max<size_t>(1024, n_nodes / 4);
  DevBuf<float> W((size_t)WIDE_NODE_FLOATS * cap);
  DevBuf<float> T((size_t)WIDE_TRI_FLOATS * std::max<uint32_t>(n_tris, 1u));
  DevBuf<Item> items(1), next;
  Item root;  // item_of(0)
  {
    int32_t nd1 = 0;
    check(cudaMemcpyAsync(&nd1, nodes5 + 1, 4, cudaMemcpyDeviceToHost, s), "D2H");
    check(cudaStreamSynchronize(s), "sync");
    root = nd1 > -1 ? Item{1u, (uint32_t)nd1 & 0x00ffffffu, (uint32_t)nd1 >> 24} : Item{0u, 0u, 0u};
  }
  check(cudaMemcpyAsync(items.p, &root, sizeof(Item), cudaMemcpyHostToDevice, s), "H2D");
  uint32_t n = 1, node_base = 0, tri_base = 0;
  depth = 0;
  DevBuf<uint32_t> n_inner, n_tri, tot(2);
  while (n) {
    depth++;
    n_inner.alloc(n);
    n_tri.alloc(n);
    k_wide_count<<<blocks(n), 128, 0, s>>>(V, items.p, n, n_inner.p, n_tri.p);
    check(cudaGetLastError(), "k_wide_count");
    scan_exclusive_u32(s, n_inner.p, n_inner.p, n, tot.p);
    scan_exclusive_u32(s, n_tri.p, n_tri.p, n, tot.p + 1);
    uint32_t th[2];
    check(cudaMemcpyAsync(th, tot.p, 8, cudaMemcpyDeviceToHost, s), "D2H");
    check(cudaStreamSynchronize(s), "sync");
    if ((uint64_t)tri_base + th[1] > n_tris) { why = "internal: triangle count mismatch"; return 1; }
    if ((size_t)node_base + n > cap) {
      const size_t ncap = std::max((size_t)node_base + n, 2 * cap);
      DevBuf<float> W2((size_t)WIDE_NODE_FLOATS * ncap);
      check(cudaMemcpyAsync(W2.p, W.p, (size_t)WIDE_NODE_FLOATS * 4 * node_base, cudaMemcpyDeviceToDevice, s), "D2D");
      W = std::move(W2);
      cap = ncap;
    }
    next.alloc(std::max<uint32_t>(th[0], 1u));
    k_wide_write<<<blocks(n), 128, 0, s>>>(V, items.p, n, node_base, n_inner.p, n_tri.p, tri_base, P.brecs.p, W.p, T.p,
                                           next.p, err.p);
    check(cudaGetLastError(), "k_wide_write");
    node_base += n;
    tri_base += th[1];
    n = th[0];
    std::swap(items, next);
  }
  if (uint32_t ev = read_u32(s, err.p)) { why = error_text(ev); return 1; }
  if (tri_base != n_tris) { why = "internal: triangle count mismatch"; return 1; }
  nodes_out.alloc(5 * (size_t)node_base);
  check(cudaMemcpyAsync(nodes_out.p, W.p, (size_t)WIDE_NODE_FLOATS * 4 * node_base, cudaMemcpyDeviceToDevice, s),
        "D2D");
  tris_out.alloc(3 * (size_t)std::max<uint32_t>(n_tris, 1u));
  check(cudaMemcpyAsync(tris_out.p, T.p, (size_t)WIDE_TRI_FLOATS * 4 * std::max<uint32_t>(n_tris, 1u),
                        cudaMemcpyDeviceToDevice, s),
        "D2D");
  check(cudaStreamSynchronize(s), "sync");
  n_wide = node_base;
  return 0;
}

int build_exact_binary_gpu(cudaStream_t s, const int32_t* nodes5, uint32_t n_nodes, const int4* tri4,
                           uint32_t n_tris, const float4* verts4, uint32_t n_verts, DevBuf<float4>& records,
                           DevBuf<float4>& tris, int32_t& root_code, std::string& why) {
  if (n_nodes == 0) { why = "empty BVH"; return 1; }
  DevBuf<uint32_t> err(1);
  check(cudaMemsetAsync(err.p, 0, 4, s), "memset");
  Prepared P;
  if (prepare(s, nodes5, n_nodes, tri4, n_tris, verts4, n_verts, err, P, why)) return 1;
  DevBuf<uint32_t> rank(n_nodes), tot(1);
  k_inner_flags<<<blocks(n_nodes), 128, 0, s>>>(nodes5, n_nodes, rank.p);
  scan_exclusive_u32(s, rank.p, rank.p, n_nodes, tot.p);
  const uint32_t n_inner = read_u32(s, tot.p);
  records.alloc(4 * (size_t)std::max<uint32_t>(n_inner, 1u));
  check(cudaMemsetAsync(records.p, 0, records.bytes(), s), "memset");
  DevBuf<int32_t> rc(1);
  k_exact_records<<<blocks(n_nodes), 128, 0, s>>>(nodes5, n_nodes, rank.p, P.nbox.p,
                                                  reinterpret_cast<float*>(records.p), rc.p);
  check(cudaGetLastError(), "k_exact_records");
  tris.alloc(3 * (size_t)std::max<uint32_t>(n_tris, 1u));
  check(cudaMemcpyAsync(tris.p, P.brecs.p, P.brecs.bytes(), cudaMemcpyDeviceToDevice, s), "D2D");
  check(cudaMemcpyAsync(&root_code, rc.p, 4, cudaMemcpyDeviceToHost, s), "D2H");
  check(cudaStreamSynchronize(s), "sync");
  return 0;
}

}  // namespace pk
