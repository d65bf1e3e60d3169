// pk_wide.cpp -- collapse of the binary BVH into 8-wide nodes with 8-bit
// child boxes (host side; the record layout is described in pk_wide.h).
//
// Collapse: a wide node starts from its binary node's two children and
// repeatedly opens the inner child of largest surface area until it holds
// eight children or only leaves (the greedy collapse of Wald et al.,
// "Getting Rid of Packets", 2008; Ylitie et al., HPG 2017 use the same child
// budget).  Wide nodes are numbered breadth first, so every child index is
// larger than its parent's.
#include "pk_wide.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <deque>

namespace pk {

namespace {

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
  double area() const {
    const double x = hi[0] - lo[0], y = hi[1] - lo[1], z = hi[2] - lo[2];
    return x * y + y * z + z * x;
  }
};

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

// Bounds of every binary node over the triangle records the test reads
// (v0, v0 + e1, v0 + e2), widened by MARGIN * max(1, |x|).
int node_boxes(const int32_t* nodes5, uint32_t n_nodes, const float* tris, uint32_t n_tris, std::vector<DBox>& box,
               std::string& why) {
  // ---- conservative binary node boxes (children have larger BFS indices)
  box.assign(n_nodes, DBox());
  for (int64_t i = (int64_t)n_nodes - 1; i >= 0; i--) {
    const int32_t* nd = nodes5 + 5 * (size_t)i;
    DBox b;
    if (nd[1] > -1) {
      const uint32_t word = (uint32_t)nd[1];
      const uint32_t size = word >> 24, base = word & 0x00ffffffu;
      if (size >= 128u || (uint64_t)base + size > n_tris) {
        why = "leaf outside the triangle array";
        return 1;
      }
      for (uint32_t k = 0; k < size; k++) {
        const float* t = tris + 12 * (size_t)(base + k);
        const double v0[3] = {t[0], t[1], t[2]};
        const double e1[3] = {t[3], t[4], t[5]};
        const double e2[3] = {t[6], t[7], t[8]};
        b.add(v0[0], v0[1], v0[2]);
        b.add(v0[0] + e1[0], v0[1] + e1[1], v0[2] + e1[2]);
        b.add(v0[0] + e2[0], v0[1] + e2[1], v0[2] + e2[2]);
      }
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
  for (DBox& b : box)
    for (int a = 0; a < 3; a++) {
      if (!(b.lo[a] <= b.hi[a])) continue;  // empty leaf: never hit
      b.lo[a] -= MARGIN * std::max(1.0, std::fabs(b.lo[a]));
      b.hi[a] += MARGIN * std::max(1.0, std::fabs(b.hi[a]));
    }
  return 0;
}

}  // namespace

int build_wide_bvh(const int32_t* nodes5, uint32_t n_nodes, const float* tris, uint32_t n_tris, WideHost& out,
                   std::string& why) {
  out = WideHost();
  if (n_nodes == 0) {
    why = "empty BVH";
    return 1;
  }
  std::vector<DBox> box;
  if (node_boxes(nodes5, n_nodes, tris, n_tris, box, why)) return 1;
  auto is_leaf = [&](uint32_t i) { return nodes5[5 * (size_t)i + 1] > -1; };

  // ---- collapse, breadth first
  struct Item {
    uint32_t bin;
    uint32_t depth;
  };
  std::deque<Item> queue;
  queue.push_back({0u, 1u});
  std::vector<float>& W = out.nodes;
  uint32_t next = 1;
  while (!queue.empty()) {
    const Item it = queue.front();
    queue.pop_front();
    out.max_depth = std::max(out.max_depth, it.depth);
    std::vector<uint32_t> ch;
    if (is_leaf(it.bin)) {
      ch.push_back(it.bin);
    } else {
      const uint32_t l = (uint32_t)nodes5[5 * (size_t)it.bin];
      ch.push_back(l);
      ch.push_back(l + 1);
      while (ch.size() < 8) {
        int best = -1;
        double best_a = -1.0;
        for (size_t k = 0; k < ch.size(); k++) {
          if (is_leaf(ch[k])) continue;
          const double a = box[ch[k]].area();
          if (a > best_a) {
            best_a = a;
            best = (int)k;
          }
        }
        if (best < 0) break;
        const uint32_t l2 = (uint32_t)nodes5[5 * (size_t)ch[best]];
        ch[best] = l2;
        ch.insert(ch.begin() + best + 1, l2 + 1);
      }
    }
    // frame: origin rounded down, power-of-two scale so that 255 steps reach
    // the largest child bound
    float rec[24];
    std::memset(rec, 0, sizeof(rec));
    uint8_t q[6][8];
    std::memset(q, 0, sizeof(q));
    int32_t code[8];
    for (int k = 0; k < 8; k++) code[k] = (int32_t)0x80000000u;
    DBox all;
    for (uint32_t c : ch) all.add(box[c]);
    uint32_t valid = 0;
    float p[3];
    int ex[3];
    for (int a = 0; a < 3; a++) {
      if (!(all.lo[a] <= all.hi[a])) { all.lo[a] = 0.0; all.hi[a] = 0.0; }
      p[a] = f_down(all.lo[a]);
      const double ext = all.hi[a] - (double)p[a];
      int e = ext > 0.0 ? (int)std::ceil(std::log2(ext / 255.0)) : -100;
      e = std::max(-100, std::min(e, 127));
      while (e < 127 && (double)decode(p[a], std::ldexp(1.0f, e), 255) < all.hi[a]) e++;
      ex[a] = e;
    }
    for (size_t k = 0; k < ch.size(); k++) {
      const DBox& b = box[ch[k]];
      bool empty = false;
      for (int a = 0; a < 3; a++) empty |= !(b.lo[a] <= b.hi[a]);
      if (is_leaf(ch[k])) {
        const uint32_t word = (uint32_t)nodes5[5 * (size_t)ch[k] + 1];
        if ((word >> 24) == 0u) empty = true;
        code[k] = (int32_t)(0x80000000u | word);
      } else {
        code[k] = (int32_t)next++;
        queue.push_back({ch[k], it.depth + 1});
      }
      if (empty) continue;
      valid |= 1u << k;
      for (int a = 0; a < 3; a++) {
        const float s = std::ldexp(1.0f, ex[a]);
        int lo = (int)std::floor((b.lo[a] - (double)p[a]) / (double)s);
        lo = std::max(0, std::min(lo, 255));
        while (lo > 0 && (double)decode(p[a], s, lo) > b.lo[a]) lo--;
        int hi = (int)std::ceil((b.hi[a] - (double)p[a]) / (double)s);
        hi = std::max(0, std::min(hi, 255));
        while (hi < 255 && (double)decode(p[a], s, hi) < b.hi[a]) hi++;
        if ((double)decode(p[a], s, lo) > b.lo[a] || (double)decode(p[a], s, hi) < b.hi[a]) {
          why = "child box does not fit its 8-bit frame";
          return 1;
        }
        q[a][k] = (uint8_t)lo;
        q[3 + a][k] = (uint8_t)hi;
      }
    }
    rec[0] = p[0];
    rec[1] = p[1];
    rec[2] = p[2];
    const uint32_t packed = (uint32_t)(ex[0] + 127) | ((uint32_t)(ex[1] + 127) << 8) |
                            ((uint32_t)(ex[2] + 127) << 16) | (valid << 24);
    std::memcpy(&rec[3], &packed, 4);
    std::memcpy(&rec[4], code, 32);
    // qlo.x qlo.y | qlo.z qhi.x | qhi.y qhi.z
    std::memcpy(&rec[12], q[0], 8);
    std::memcpy(&rec[14], q[1], 8);
    std::memcpy(&rec[16], q[2], 8);
    std::memcpy(&rec[18], q[3], 8);
    std::memcpy(&rec[20], q[4], 8);
    std::memcpy(&rec[22], q[5], 8);
    W.insert(W.end(), rec, rec + 24);
  }
  out.n_nodes = (uint32_t)(W.size() / 24);
  if (out.n_nodes != next) {
    why = "internal: wide node count mismatch";
    return 1;
  }
  return 0;
}

int build_exact_binary(const int32_t* nodes5, uint32_t n_nodes, const float* tris, uint32_t n_tris,
                       std::vector<float>& records, int32_t& root_code, std::string& why) {
  if (n_nodes == 0) {
    why = "empty BVH";
    return 1;
  }
  std::vector<DBox> box;
  if (node_boxes(nodes5, n_nodes, tris, n_tris, box, why)) return 1;
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

}  // namespace pk
