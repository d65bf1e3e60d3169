// om_wide.h -- host restatement of form (1)'s builders (the compressed 8-wide
// BVH by the SAH-optimal collapse, and the FP32 binary reference's records);
// the record layouts are those of pike_gb300/csrc/pk_wide.h.
//
// TEST INFRASTRUCTURE ONLY (see om_math.h): the library builds these
// structures on the GPU (pike_gb300/csrc/pk_wide.cu), and the tests require
// its records to equal this restatement's bit for bit.
//
// Collapse: the SAH-optimal collapse of Ylitie et al. (HPG 2017, section
// 3.1; see Collapse below) picks, for every binary node, whether it becomes a
// leaf child, a wide node, or shares its slots between its two children.  A
// leaf child holds at most three triangles; a binary leaf with more is split
// into halves of its triangle range as if it were an inner node.  Children
// are assigned to slots greedily by the octant cost of Ylitie et al. (the
// child whose centroid lies furthest against a direction octant takes that
// octant's slot).  Nodes are built one breadth-first level at a time, each
// level in parallel; a prefix sum over the level gives every node's internal
// children consecutive indices after all earlier nodes.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace om_wide {

constexpr int WIDE_NODE_FLOATS = 20;
constexpr int WIDE_TRI_FLOATS = 12;

struct WideHost {
  std::vector<float> nodes;  // WIDE_NODE_FLOATS per node
  std::vector<float> tris;   // WIDE_TRI_FLOATS per triangle, in the wide BVH's order
  uint32_t n_nodes = 0;
  uint32_t max_depth = 0;
};

}  // namespace om_wide


#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>

namespace om_wide {

namespace detail {

struct DBox {
  double lo[3] = {INFINITY, INFINITY, INFINITY};
  double hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  void add(double x, double y, double z) {
    const double v[3] = {x, y, z};
    for (int a = 0; a < 3; a++) {
      lo[a] = std::min(lo[a], v[a]);
      hi[a] = std::max(hi[a], v[a]);
    }
  }
  void add(const DBox& b) {
    for (int a = 0; a < 3; a++) {
      lo[a] = std::min(lo[a], b.lo[a]);
      hi[a] = std::max(hi[a], b.hi[a]);
    }
  }
  bool empty() const { return !(lo[0] <= hi[0] && lo[1] <= hi[1] && lo[2] <= hi[2]); }
  double area() const {
    if (empty()) return 0.0;
    const double x = hi[0] - lo[0], y = hi[1] - lo[1], z = hi[2] - lo[2];
    return x * y + y * z + z * x;
  }
  double centre(int a) const { return empty() ? 0.0 : 0.5 * (lo[a] + hi[a]); }
};

template <class F>
void parallel_for(size_t n, F fn) {
  const size_t hw = std::max<size_t>(1, std::thread::hardware_concurrency());
  const size_t nt = std::min(hw, std::max<size_t>(1, n / 4096));
  if (nt <= 1) {
    fn(0, n);
    return;
  }
  std::vector<std::thread> th;
  const size_t chunk = (n + nt - 1) / nt;
  for (size_t t = 0; t < nt; t++) {
    const size_t b = t * chunk, e = std::min(n, b + chunk);
    if (b < e) th.emplace_back([=]() { fn(b, e); });
  }
  for (std::thread& x : th) x.join();
}

// Largest float not above x / smallest float not below x.
float f_down(double x) {
  float f = (float)x;
  if ((double)f > x) f = std::nextafter(f, -INFINITY);
  return f;
}
float f_up(double x) {
  float f = (float)x;
  if ((double)f < x) f = std::nextafter(f, INFINITY);
  return f;
}
// The device decode: one exact multiply (q has 8 bits, s is a power of two)
// and one rounded FP32 add.
float decode(float p, float s, int q) {
  const float m = s * (float)q;
  return p + m;
}

constexpr double MARGIN = 0x1p-18;

void widen(DBox& b) {
  for (int a = 0; a < 3; a++) {
    if (!(b.lo[a] <= b.hi[a])) continue;  // empty: never hit
    b.lo[a] -= MARGIN * std::max(1.0, std::fabs(b.lo[a]));
    b.hi[a] += MARGIN * std::max(1.0, std::fabs(b.hi[a]));
  }
}

// Triangle boxes over the three vertices and the 48-byte triangle records of
// the binary leaf order (slot = leaf-order index).
int triangle_data(const int32_t* tri4, uint32_t n_tris, const float* verts4, uint32_t n_verts,
                  std::vector<DBox>& tbox, std::vector<float>& recs, std::string& why) {
  tbox.assign(n_tris, DBox());
  recs.assign((size_t)WIDE_TRI_FLOATS * n_tris, 0.0f);
  std::atomic<bool> bad{false};
  parallel_for(n_tris, [&](size_t b, size_t e) {
    for (size_t t = b; t < e; t++) {
      const int32_t* tr = tri4 + 4 * t;
      float* r = &recs[(size_t)WIDE_TRI_FLOATS * t];
      DBox box;
      for (int k = 0; k < 3; k++) {
        if (tr[k] < 0 || (uint32_t)tr[k] >= n_verts) { bad = true; continue; }
        const float* v = verts4 + 4 * (size_t)tr[k];
        r[3 * k] = v[0];
        r[3 * k + 1] = v[1];
        r[3 * k + 2] = v[2];
        box.add(v[0], v[1], v[2]);
      }
      const uint32_t slot = (uint32_t)t;
      std::memcpy(&r[9], &slot, 4);
      tbox[t] = box;
    }
  });
  if (bad) {
    why = "triangle vertex index out of range";
    return 1;
  }
  return 0;
}

// Bounds of every binary node over its triangles' vertices, widened by MARGIN.
int node_boxes(const int32_t* nodes5, uint32_t n_nodes, uint32_t n_tris, const std::vector<DBox>& tbox,
               std::vector<DBox>& box, std::string& why) {
  box.assign(n_nodes, DBox());
  for (int64_t i = (int64_t)n_nodes - 1; i >= 0; i--) {  // children have larger BFS indices
    const int32_t* nd = nodes5 + 5 * (size_t)i;
    DBox b;
    if (nd[1] > -1) {
      const uint32_t word = (uint32_t)nd[1];
      const uint32_t size = word >> 24, base = word & 0x00ffffffu;
      if (size >= 128u || (uint64_t)base + size > n_tris) {
        why = "leaf outside the triangle array";
        return 1;
      }
      for (uint32_t k = 0; k < size; k++) b.add(tbox[base + k]);
    } else {
      const int32_t l = nd[0];
      if (l <= (int32_t)i || (uint32_t)l + 1 >= n_nodes) {
        why = "child index not after its parent";
        return 1;
      }
      b = box[l];
      b.add(box[l + 1]);
    }
    box[i] = b;
  }
  return 0;
}

// A child candidate of a wide node: a binary inner node (a wide node of its
// own), a range of leaf-ordered triangles (part of a binary leaf), or a binary
// subtree of at most LEAF_MAX triangles taken as one leaf child.
struct Item {
  uint32_t kind;  // 0 binary inner node, 1 triangle range, 2 subtree as one leaf
  uint32_t a;     // node index, or first triangle
  uint32_t n;     // triangle count
};

constexpr uint32_t LEAF_MAX = 3;
// SAH weights of the collapse: one wide-node visit (eight child tests) and
// one triangle test, per unit of surface area of the box tested.
constexpr float COST_NODE = 1.0f, COST_TRI = 0.3f;
constexpr uint8_t OPT_LEAF = 0xf0, OPT_INNER = 0xf1;  // else: split, j slots to the left child

// The SAH-optimal collapse of Ylitie et al. (HPG 2017, section 3.1): for
// every binary node n and slot budget i (1..8), cost[n][i] is the cheapest
// way to represent n's subtree with at most i children of a wide node: one
// leaf child (subtree of at most LEAF_MAX triangles: area * COST_TRI *
// triangles), one internal child (a wide node: area * COST_NODE + the best
// distribution of n's two children over 8 slots), or (i >= 2) its two
// children sharing the i slots.  Computed bottom-up, one binary level at a
// time, each level in parallel.
struct Collapse {
  std::vector<float> cost;     // 8 per node (budgets 1..8)
  std::vector<uint8_t> opt;    // 8 per node
  std::vector<uint8_t> split;  // left child's slots in the node's own 8-slot distribution
  std::vector<uint32_t> tris;  // triangles in the subtree

  void run(const int32_t* nodes5, uint32_t n_nodes, const std::vector<DBox>& nbox) {
    cost.assign(8 * (size_t)n_nodes, 0.0f);
    opt.assign(8 * (size_t)n_nodes, OPT_LEAF);
    split.assign(n_nodes, 1);
    tris.assign(n_nodes, 0);
    std::vector<uint32_t> depth(n_nodes, 0);
    uint32_t maxd = 0;
    for (uint32_t n = 0; n < n_nodes; n++) {
      const int32_t* nd = nodes5 + 5 * (size_t)n;
      if (nd[1] <= -1) depth[nd[0]] = depth[nd[0] + 1] = depth[n] + 1;
      maxd = std::max(maxd, depth[n]);
    }
    std::vector<uint32_t> start(maxd + 2, 0), order(n_nodes);
    for (uint32_t n = 0; n < n_nodes; n++) start[depth[n] + 1]++;
    for (uint32_t d = 0; d <= maxd; d++) start[d + 1] += start[d];
    {
      std::vector<uint32_t> at(start.begin(), start.end() - 1);
      for (uint32_t n = 0; n < n_nodes; n++) order[at[depth[n]]++] = n;
    }
    const float INF = INFINITY;
    for (int64_t d = maxd; d >= 0; d--) {
      const uint32_t b = start[d], e = start[d + 1];
      parallel_for(e - b, [&](size_t lo, size_t hi) {
        for (size_t k = lo; k < hi; k++) {
          const uint32_t n = order[b + k];
          const int32_t* nd = nodes5 + 5 * (size_t)n;
          float* C = &cost[8 * (size_t)n];
          uint8_t* O = &opt[8 * (size_t)n];
          const double area = nbox[n].area();
          if (nd[1] > -1) {
            const uint32_t t = (uint32_t)nd[1] >> 24;
            tris[n] = t;
            const float leaf = t <= LEAF_MAX ? (float)(area * COST_TRI * t) : INF;
            const float inner = t > LEAF_MAX ? (float)(area * (COST_NODE + COST_TRI * t)) : INF;
            for (int i = 0; i < 8; i++) {
              C[i] = std::min(leaf, inner);
              O[i] = leaf <= inner ? OPT_LEAF : OPT_INNER;
            }
            continue;
          }
          const uint32_t l = (uint32_t)nd[0], r = l + 1;
          tris[n] = tris[l] + tris[r];
          const float* Cl = &cost[8 * (size_t)l];
          const float* Cr = &cost[8 * (size_t)r];
          float D[8];
          uint8_t J[8];
          D[0] = INF;
          J[0] = 1;
          for (int i = 2; i <= 8; i++) {  // i slots, j of them to the left
            float best = INF;
            uint8_t bj = 1;
            for (int j = 1; j < i; j++) {
              const float c = Cl[j - 1] + Cr[i - j - 1];
              if (c < best) { best = c; bj = (uint8_t)j; }
            }
            D[i - 1] = best;
            J[i - 1] = bj;
          }
          split[n] = J[7];
          const float leaf = tris[n] <= LEAF_MAX ? (float)(area * COST_TRI * tris[n]) : INF;
          const float inner = (float)(area * COST_NODE) + D[7];
          C[0] = std::min(leaf, inner);
          O[0] = leaf <= inner ? OPT_LEAF : OPT_INNER;
          for (int i = 1; i < 8; i++) {
            C[i] = C[i - 1];
            O[i] = O[i - 1];
            if (D[i] < C[i]) { C[i] = D[i]; O[i] = J[i]; }
          }
        }
      });
    }
  }
};

struct Builder {
  const int32_t* nodes5;
  const std::vector<DBox>& tbox;
  const std::vector<DBox>& nbox;  // widened binary node boxes
  const Collapse& dp;

  bool is_leaf(uint32_t n) const { return nodes5[5 * (size_t)n + 1] > -1; }
  Item item_of(uint32_t node) const {
    const int32_t t = nodes5[5 * (size_t)node + 1];
    if (t > -1) return Item{1u, (uint32_t)t & 0x00ffffffu, (uint32_t)t >> 24};
    return Item{0u, node, 0u};
  }
  DBox box_of(const Item& it) const {
    if (it.kind != 1) return nbox[it.a];
    DBox b;
    for (uint32_t k = 0; k < it.n; k++) b.add(tbox[it.a + k]);
    widen(b);
    return b;
  }
  bool openable(const Item& it) const { return it.kind == 0 || (it.kind == 1 && it.n > LEAF_MAX); }
  // The leaf-ordered triangles of a leaf child, in order.
  void leaf_tris(const Item& it, uint32_t (&out)[LEAF_MAX], uint32_t& count) const {
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
      const int32_t* nd = nodes5 + 5 * (size_t)n;
      if (nd[1] > -1) {
        const uint32_t w = (uint32_t)nd[1];
        for (uint32_t k = 0; k < (w >> 24) && count < LEAF_MAX; k++) out[count++] = (w & 0x00ffffffu) + k;
      } else if (sp + 2 <= 64) {
        stack[sp++] = (uint32_t)nd[0] + 1;
        stack[sp++] = (uint32_t)nd[0];
      }
    }
  }
  // The children that binary node n's subtree contributes with a budget of i slots.
  void collect(uint32_t n, int i, Item* ch, int& nc) const {
    const uint8_t o = dp.opt[8 * (size_t)n + (i - 1)];
    if (o == OPT_LEAF) {
      ch[nc++] = is_leaf(n) ? item_of(n) : Item{2u, n, dp.tris[n]};
    } else if (o == OPT_INNER) {
      ch[nc++] = item_of(n);  // an inner node, or a binary leaf of more than LEAF_MAX triangles (a range)
    } else {
      const uint32_t l = (uint32_t)nodes5[5 * (size_t)n];
      collect(l, o, ch, nc);
      collect(l + 1, i - o, ch, nc);
    }
  }

  // Children of the wide node for `it` (at most 8), in slot order (empty slots
  // have n = 0 and kind 1), and their boxes.
  void children(const Item& it, Item (&slot)[8], DBox (&sbox)[8], bool (&used)[8]) const {
    Item ch[8];
    DBox cb[8];
    int nc = 0;
    if (it.kind == 0) {
      const uint32_t l = (uint32_t)nodes5[5 * (size_t)it.a];
      const int j = dp.split[it.a];
      collect(l, j, ch, nc);
      collect(l + 1, 8 - j, ch, nc);
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
          const double a = box_of(ch[k]).area();
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
    for (int k = 0; k < nc; k++) cb[k] = box_of(ch[k]);
    // octant slots: cost(child, s) = dot(centre offset, sign vector of s);
    // repeatedly take the cheapest free (child, slot) pair
    DBox all;
    for (int k = 0; k < nc; k++) all.add(cb[k]);
    double cost[8][8];
    for (int k = 0; k < nc; k++) {
      const double dx = cb[k].centre(0) - all.centre(0), dy = cb[k].centre(1) - all.centre(1),
                   dz = cb[k].centre(2) - all.centre(2);
      for (int s = 0; s < 8; s++)
        cost[k][s] = ((s & 1) ? -dx : dx) + ((s & 2) ? -dy : dy) + ((s & 4) ? -dz : dz);
    }
    bool cdone[8] = {false, false, false, false, false, false, false, false};
    for (int s = 0; s < 8; s++) used[s] = false;
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
};

}  // namespace detail
using namespace detail;

inline int build_wide_bvh(const int32_t* nodes5, uint32_t n_nodes, const int32_t* tri4, uint32_t n_tris,
                   const float* verts4, uint32_t n_verts, WideHost& out, std::string& why) {
  out = WideHost();
  if (n_nodes == 0) {
    why = "empty BVH";
    return 1;
  }
  std::vector<DBox> tbox, nbox;
  std::vector<float> brecs;
  if (triangle_data(tri4, n_tris, verts4, n_verts, tbox, brecs, why)) return 1;
  if (node_boxes(nodes5, n_nodes, n_tris, tbox, nbox, why)) return 1;
  for (DBox& b : nbox) widen(b);
  Collapse dp;
  dp.run(nodes5, n_nodes, nbox);
  const Builder B{nodes5, tbox, nbox, dp};

  struct Plan {
    Item slot[8];
    DBox sbox[8];
    bool used[8];
    uint32_t n_inner = 0, n_tri = 0;
  };
  std::vector<Item> level{B.item_of(0)};
  uint32_t node_base = 0;  // index of the level's first node
  uint32_t depth = 0;
  std::vector<float>& W = out.nodes;
  std::vector<float>& T = out.tris;
  while (!level.empty()) {
    depth++;
    const size_t n = level.size();
    std::vector<Plan> plan(n);
    parallel_for(n, [&](size_t b, size_t e) {
      for (size_t i = b; i < e; i++) {
        Plan& p = plan[i];
        B.children(level[i], p.slot, p.sbox, p.used);
        for (int s = 0; s < 8; s++) {
          if (!p.used[s]) continue;
          if (B.openable(p.slot[s])) p.n_inner++;
          else p.n_tri += p.slot[s].n;
        }
      }
    });
    // prefix sums: internal children follow the level in order; triangle
    // records follow those of all earlier nodes
    std::vector<uint32_t> child0(n), tri0(n);
    uint32_t next_child = node_base + (uint32_t)n, next_tri = (uint32_t)(T.size() / WIDE_TRI_FLOATS);
    for (size_t i = 0; i < n; i++) {
      child0[i] = next_child;
      tri0[i] = next_tri;
      next_child += plan[i].n_inner;
      next_tri += plan[i].n_tri;
    }
    W.resize((size_t)WIDE_NODE_FLOATS * (node_base + n));
    T.resize((size_t)WIDE_TRI_FLOATS * next_tri);
    std::vector<Item> nxt(next_child - node_base - (uint32_t)n);
    std::atomic<bool> fit{true};
    parallel_for(n, [&](size_t b, size_t e) {
      for (size_t i = b; i < e; i++) {
        const Plan& p = plan[i];
        float rec[WIDE_NODE_FLOATS];
        std::memset(rec, 0, sizeof(rec));
        uint8_t q[6][8], meta[8];
        std::memset(q, 0, sizeof(q));
        std::memset(meta, 0, sizeof(meta));
        DBox all;
        for (int s = 0; s < 8; s++)
          if (p.used[s]) all.add(p.sbox[s]);
        float org[3];
        int ex[3];
        for (int a = 0; a < 3; a++) {
          double lo = all.lo[a], hi = all.hi[a];
          if (!(lo <= hi)) { lo = 0.0; hi = 0.0; }
          org[a] = f_down(lo);
          const double ext = hi - (double)org[a];
          int e2 = -100;  // ceil(log2(ext / 255)), exactly: ext / 255 = m 2^k with m in [0.5, 1)
          if (ext > 0.0) {
            int k;
            const double m = std::frexp(ext / 255.0, &k);
            e2 = m == 0.5 ? k - 1 : k;
          }
          e2 = std::max(-100, std::min(e2, 127));
          while (e2 < 127 && (double)decode(org[a], std::ldexp(1.0f, e2), 255) < hi) e2++;
          ex[a] = e2;
        }
        uint32_t imask = 0, inner_rank = 0, tri_off = 0;
        for (int s = 0; s < 8; s++) {
          if (!p.used[s]) continue;
          const Item& c = p.slot[s];
          if (B.openable(c)) {
            imask |= 1u << s;
            meta[s] = (uint8_t)(0x20u | (uint32_t)s);
            nxt[child0[i] - node_base - n + inner_rank] = c;
            inner_rank++;
          } else {
            if (c.n == 0) continue;
            uint32_t ids[LEAF_MAX], cnt = 0;
            B.leaf_tris(c, ids, cnt);
            meta[s] = (uint8_t)((((1u << cnt) - 1u) << 5) | tri_off);
            for (uint32_t k = 0; k < cnt; k++)
              std::memcpy(&T[(size_t)WIDE_TRI_FLOATS * (tri0[i] + tri_off + k)],
                          &brecs[(size_t)WIDE_TRI_FLOATS * ids[k]], WIDE_TRI_FLOATS * sizeof(float));
            tri_off += cnt;
          }
          const DBox& cb = p.sbox[s];
          if (cb.empty()) continue;  // all-zero planes at the frame origin: hit tests may pass, no triangles
          for (int a = 0; a < 3; a++) {
            const float sc = std::ldexp(1.0f, ex[a]);
            int lo = (int)std::floor((cb.lo[a] - (double)org[a]) / (double)sc);
            lo = std::max(0, std::min(lo, 255));
            while (lo > 0 && (double)decode(org[a], sc, lo) > cb.lo[a]) lo--;
            int hi = (int)std::ceil((cb.hi[a] - (double)org[a]) / (double)sc);
            hi = std::max(0, std::min(hi, 255));
            while (hi < 255 && (double)decode(org[a], sc, hi) < cb.hi[a]) hi++;
            if ((double)decode(org[a], sc, lo) > cb.lo[a] || (double)decode(org[a], sc, hi) < cb.hi[a]) fit = false;
            q[a][s] = (uint8_t)lo;
            q[3 + a][s] = (uint8_t)hi;
          }
        }
        rec[0] = org[0];
        rec[1] = org[1];
        rec[2] = org[2];
        const uint32_t packed = (uint32_t)(ex[0] + 127) | ((uint32_t)(ex[1] + 127) << 8) |
                                ((uint32_t)(ex[2] + 127) << 16) | (imask << 24);
        std::memcpy(&rec[3], &packed, 4);
        const uint32_t bases[2] = {p.n_inner ? child0[i] : 0u, tri0[i]};
        std::memcpy(&rec[4], bases, 8);
        std::memcpy(&rec[6], meta, 8);
        // qlo.x qlo.y | qlo.z qhi.x | qhi.y qhi.z
        std::memcpy(&rec[8], q[0], 8);
        std::memcpy(&rec[10], q[1], 8);
        std::memcpy(&rec[12], q[2], 8);
        std::memcpy(&rec[14], q[3], 8);
        std::memcpy(&rec[16], q[4], 8);
        std::memcpy(&rec[18], q[5], 8);
        std::memcpy(&W[(size_t)WIDE_NODE_FLOATS * (node_base + i)], rec, sizeof(rec));
      }
    });
    if (!fit) {
      why = "child box does not fit its 8-bit frame";
      return 1;
    }
    node_base += (uint32_t)n;
    level.swap(nxt);
  }
  out.n_nodes = node_base;
  out.max_depth = depth;
  if (T.size() != (size_t)WIDE_TRI_FLOATS * n_tris) {
    why = "internal: triangle count mismatch";
    return 1;
  }
  return 0;
}

inline int build_exact_binary(const int32_t* nodes5, uint32_t n_nodes, const int32_t* tri4, uint32_t n_tris,
                       const float* verts4, uint32_t n_verts, std::vector<float>& records,
                       std::vector<float>& tris, int32_t& root_code, std::string& why) {
  if (n_nodes == 0) {
    why = "empty BVH";
    return 1;
  }
  std::vector<DBox> tbox, box;
  if (triangle_data(tri4, n_tris, verts4, n_verts, tbox, tris, why)) return 1;
  if (node_boxes(nodes5, n_nodes, n_tris, tbox, box, why)) return 1;
  for (DBox& b : box) widen(b);
  std::vector<uint32_t> rank(n_nodes);
  uint32_t n_inner = 0;
  for (uint32_t i = 0; i < n_nodes; i++) {
    rank[i] = n_inner;
    if (nodes5[5 * (size_t)i + 1] <= -1) n_inner++;
  }
  auto code = [&](uint32_t i) -> int32_t {
    const int32_t t = nodes5[5 * (size_t)i + 1];
    return t > -1 ? (int32_t)(0x80000000u | (uint32_t)t) : (int32_t)rank[i];
  };
  auto put = [&](float* r, const DBox& b) {  // {hi, lo} per axis, rounded outward
    for (int a = 0; a < 3; a++) {
      const bool empty = !(b.lo[a] <= b.hi[a]);
      // an empty child becomes a point at 1e30: its entry distance exceeds any hit
      r[2 * a] = empty ? 1e30f : f_up(b.hi[a]);
      r[2 * a + 1] = empty ? 1e30f : f_down(b.lo[a]);
    }
  };
  records.assign(16 * (size_t)std::max<uint32_t>(n_inner, 1u), 0.0f);
  for (uint32_t i = 0; i < n_nodes; i++) {
    if (nodes5[5 * (size_t)i + 1] > -1) continue;
    const uint32_t l = (uint32_t)nodes5[5 * (size_t)i];
    float* r = &records[16 * (size_t)rank[i]];
    float lb[6], rb[6];
    put(lb, box[l]);
    put(rb, box[l + 1]);
    std::memcpy(r, lb, 24);
    std::memcpy(r + 6, rb, 24);
    const int32_t c[4] = {code(l), code(l + 1), 0, 0};
    std::memcpy(r + 12, c, 16);
  }
  root_code = code(0);
  return 0;
}

}  // namespace om_wide
