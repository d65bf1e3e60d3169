// om_build.h -- oracle restatement of Pike's CPU data-build layer.
//
// TEST INFRASTRUCTURE ONLY (see om_math.h).  Parity unpinned: the reference
// ships no tests, fixtures or golden vectors for this path and its own code
// (JavaScript + WGSL on WebGPU) cannot run on this machine, so every golden
// vector is generated from this restatement of the reference source.
//
// Follows, in double precision with JavaScript's evaluation order:
//   render/scene.js:104-118,163-170      attribute quantisation (_quantizeVec3ToInt/_quantizeVec2ToInt)
//   render/util/texture_packer.js:87-136 addColor dedup, 1x1 layers (getResolution with maxRes=1)
//   render/bvh.js:12-107,119-223         full-sweep object SAH, leaf rule, stable partition
//   render/primitives.js:3-44            BoundingBox, centroid, surface area
//   render/bvh.js:46-74 + util/utility.js:45-79  BFS serialisation (FIFO queue)
//   render/passes/trace_pass.js:166-170,202-262  normaliser, quantiser, 20-byte node packing
//   render/env_sampler.js:43-157         env luminance, stable sort, equal-mass bins, pdf
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <deque>
#include <stdexcept>
#include <string>
#include <vector>

namespace om {

// ---- JavaScript number helpers ----------------------------------------
// ToInt16/ToInt8 (ECMAScript 7.1.8/7.1.10): NaN/inf -> 0, truncate, wrap.
static inline int32_t js_toint(double v, int bits) {
  if (!std::isfinite(v)) return 0;
  double t = std::trunc(v);
  double m = std::fmod(t, std::ldexp(1.0, bits));
  if (m < 0) m += std::ldexp(1.0, bits);
  int64_t mi = (int64_t)m;
  if (mi >= (int64_t(1) << (bits - 1))) mi -= (int64_t(1) << bits);
  return (int32_t)mi;
}
// Math.min / Math.max (NaN propagates; -0 < +0).
static inline double js_min(double a, double b) {
  if (a != a || b != b) return NAN;
  if (a < b) return a;
  if (b < a) return b;
  return std::signbit(a) ? a : b;
}
static inline double js_max(double a, double b) {
  if (a != a || b != b) return NAN;
  if (a > b) return a;
  if (b > a) return b;
  return std::signbit(a) ? b : a;
}

// ---- Row S: scene.js _createBuffers attribute quantisation ----------------
// Vec.magnitude = sqrt(((x*x + y*y) + z*z)); Vec.normalize = v * (1/m).
static inline void js_normalize3(const double* v, double* o) {
  double m = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  double s = 1.0 / m;
  o[0] = v[0] * s; o[1] = v[1] * s; o[2] = v[2] * s;
}
// scene.js:104-111
static inline uint32_t quantize_vec3_to_int(const double* v) {
  uint32_t out = 0;
  for (int i = 0; i < 3; i++) {
    int32_t b = js_toint(v[i] * (v[i] > 0 ? 127.0 : 128.0), 8);
    out |= (uint32_t)(uint8_t)b << (8 * i);
  }
  return out;
}
// scene.js:113-118 and trace_pass.js:213-218
static inline uint32_t quantize_vec2_to_int(double a, double b) {
  int32_t s0 = js_toint(a * (a > 0 ? 32767.0 : 32768.0), 16);
  int32_t s1 = js_toint(b * (b > 0 ? 32767.0 : 32768.0), 16);
  return (uint32_t)(uint16_t)s0 | ((uint32_t)(uint16_t)s1 << 16);
}

// One vertex of scene.js:458-470 with a transform {scale, translate}.  The
// bitangent is built from bn/bt4, the normal and signed tangent before the
// prop's rotations (scene.js:160); without rotations they are nrm and tan4.
struct FlatVertex { double pos[3]; uint32_t tangent, bitangent, normal, uv; };
static inline FlatVertex flatten_vertex(const double* pos, const double* nrm, const double* tan4,
                                        const double* uv, double scale_, const double* translate,
                                        const double* bn = nullptr, const double* bt4 = nullptr) {
  if (!bn) bn = nrm;
  if (!bt4) bt4 = tan4;
  FlatVertex fv;
  for (int i = 0; i < 3; i++) fv.pos[i] = pos[i] * scale_ + translate[i];
  double normal[3], tangent[3];
  for (int i = 0; i < 3; i++) normal[i] = nrm[i] * 1.0 + 0.0;
  for (int i = 0; i < 3; i++) tangent[i] = tan4[i] * 1.0 + 0.0;
  // Vec3.cross(normalAt, tangentAt): y = -(a0*b2 - a2*b0)
  double c[3];
  c[0] = bn[1] * bt4[2] - bn[2] * bt4[1];
  c[1] = -(bn[0] * bt4[2] - bn[2] * bt4[0]);
  c[2] = bn[0] * bt4[1] - bn[1] * bt4[0];
  double w = bt4[3];
  double sgn = (w != 0.0 && w == w) ? w : 1.0;  // signedTangent[3] || 1
  for (int i = 0; i < 3; i++) c[i] = c[i] * sgn;
  double bt[3], tn[3], nn[3];
  js_normalize3(c, bt);
  js_normalize3(tangent, tn);
  js_normalize3(normal, nn);
  fv.tangent = quantize_vec3_to_int(tn);
  fv.bitangent = quantize_vec3_to_int(bt);
  fv.normal = quantize_vec3_to_int(nn);
  fv.uv = quantize_vec2_to_int(uv[0], uv[1]);
  return fv;
}

// ---- Row M: material layers (texture_packer.js addColor + getPixels) ------
// A constant colour becomes one 1x1 rgba8 layer drawn by gl.clearColor(r,g,b,1)
// and read back; float->unorm8 is restated as floor(clamp(c,0,1)*255 + 0.5).
static inline uint8_t gl_unorm8(double c) {
  double x = c != c ? 0.0 : std::min(1.0, std::max(0.0, c));
  return (uint8_t)std::floor(x * 255.0 + 0.5);
}
struct MaterialTable {
  std::vector<std::vector<double>> keys;   // addColor keys, in insertion order
  std::vector<uint8_t> layers;             // rgba8 per layer (1x1)
  std::vector<int32_t> index4;             // {diffMap, metRoughMap, normMap, emitMap} per material
  int add_color(const std::vector<double>& color) {
    for (size_t i = 0; i < keys.size(); i++) {
      if (keys[i].size() != color.size()) continue;
      bool eq = true;
      for (size_t k = 0; k < color.size(); k++) if (!(keys[i][k] == color[k])) { eq = false; break; }
      if (eq) return (int)i;
    }
    keys.push_back(color);
    layers.push_back(gl_unorm8(color[0]));
    layers.push_back(gl_unorm8(color[1]));
    layers.push_back(gl_unorm8(color[2]));
    layers.push_back(255);
    return (int)keys.size() - 1;
  }
  // scene.js:43-70 for a material without textures.
  // mat = {base r,g,b,a, roughness, metallic, emissive r,g,b}
  void add_material(const double* m) {
    int d = add_color({m[0], m[1], m[2], m[3]});
    int mr = add_color({0.0, m[4], m[5]});
    int n = add_color({0.5, 0.5, 1.0});
    int e = add_color({m[6], m[7], m[8]});
    index4.push_back(d); index4.push_back(mr); index4.push_back(n); index4.push_back(e);
  }
};

// ---- Row BVH: bvh.js sweep SAH ------------------------------------------
struct Box {
  double mn[3] = {INFINITY, INFINITY, INFINITY};
  double mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  void add_vertex(const double* v) {  // primitives.js:9-14: min = Vec3.min(vert, min)
    for (int i = 0; i < 3; i++) { mn[i] = js_min(v[i], mn[i]); mx[i] = js_max(v[i], mx[i]); }
  }
  void add_box(const Box& b) {        // primitives.js:24-29: min = Vec3.min(min, box.min)
    for (int i = 0; i < 3; i++) { mn[i] = js_min(mn[i], b.mn[i]); mx[i] = js_max(mx[i], b.mx[i]); }
  }
  double centroid(int a) const { return (mn[a] + mx[a]) * 0.5; }
  double area() const {              // primitives.js:39-44
    double xl = js_max(mx[0] - mn[0], 0.0);
    double yl = js_max(mx[1] - mn[1], 0.0);
    double zl = js_max(mx[2] - mn[2], 0.0);
    return (xl * yl + xl * zl + yl * zl) * 2.0;
  }
};

struct BuiltNode {
  Box bounds;
  bool leaf = false;
  int left = -1, right = -1;        // indices into BVHBuild::nodes (build order)
  std::vector<int32_t> leaf_tris;   // triangle ids in split-axis order
};

struct BVHBuild {
  std::vector<BuiltNode> nodes;     // nodes[0] is the root
  std::vector<Box> tri_box;
  int max_depth = 0;
  size_t num_leaf_tris = 0;
  size_t largest_leaf = 0;
};

// bvh.js:170-215 #computeSplit over axes 0,1,2; returns axis=-1 if no cost < inf.
struct Split { int axis = -1; double cost = INFINITY; long index = -1; };
static inline Split compute_split(const std::vector<int32_t>* axis_refs, const std::vector<Box>& tri_box,
                                  double parent_sa, std::vector<double>& af, std::vector<double>& ab) {
  Split s;
  const long n = (long)axis_refs[0].size();
  af.resize(n); ab.resize(n);
  for (int axis = 0; axis < 3; axis++) {
    const std::vector<int32_t>& refs = axis_refs[axis];
    Box f, b;
    for (long i = 0; i < n; i++) {
      f.add_box(tri_box[refs[i]]);
      b.add_box(tri_box[refs[n - 1 - i]]);
      af[i] = f.area();
      ab[i] = b.area();
    }
    for (long i = 0; i < n; i++) {
      double saf = af[i];
      double sab = ab[n - 1 - i];
      double cost = 0.5 + (saf / parent_sa) * (double)(i + 1) + (sab / parent_sa) * (double)(n - 1 - i);
      if (cost < s.cost) { s.cost = cost; s.index = i; s.axis = axis; }
    }
  }
  return s;
}

// bvh.js:12-43 (+ Node ctor :119-144, #splitNode :80-107, #setLeaf :217-223).
static inline BVHBuild build_bvh(const double* pos3, const int32_t* tri4, size_t n_tris) {
  BVHBuild out;
  if (n_tris == 0) throw std::runtime_error("bvh: no triangles");
  out.tri_box.resize(n_tris);
  for (size_t t = 0; t < n_tris; t++) {
    Box b;
    for (int k = 0; k < 3; k++) b.add_vertex(pos3 + 3 * (size_t)tri4[4 * t + k]);
    out.tri_box[t] = b;
  }
  std::vector<int32_t> root_refs[3];
  for (int a = 0; a < 3; a++) {
    root_refs[a].resize(n_tris);
    for (size_t t = 0; t < n_tris; t++) root_refs[a][t] = (int32_t)t;
    // Node.sortRefs: stable sort (TimSort) by centroid[a], comparator <,>,=.
    std::vector<double> key(n_tris);
    for (size_t t = 0; t < n_tris; t++) key[t] = out.tri_box[t].centroid(a);
    std::stable_sort(root_refs[a].begin(), root_refs[a].end(),
                     [&](int32_t x, int32_t y) { return key[x] < key[y]; });
  }
  struct Work { int node; int depth; std::vector<int32_t> refs[3]; };
  std::vector<Work> stack;
  out.nodes.emplace_back();
  stack.emplace_back();
  stack.back().node = 0; stack.back().depth = 1;
  for (int a = 0; a < 3; a++) stack.back().refs[a] = std::move(root_refs[a]);
  std::vector<double> af, ab;
  std::vector<uint8_t> in_left(n_tris, 0);
  while (!stack.empty()) {
    Work w = std::move(stack.back());
    stack.pop_back();
    out.max_depth = std::max(out.max_depth, w.depth);
    BuiltNode nd;
    for (int32_t r : w.refs[0]) nd.bounds.add_box(out.tri_box[r]);
    const double psa = nd.bounds.area();
    Split s = compute_split(w.refs, out.tri_box, psa, af, ab);
    if (s.axis < 0) throw std::runtime_error("bvh: no finite split cost (degenerate node); the reference throws here too");
    const long n = (long)w.refs[0].size();
    if (s.cost > (double)n) {
      nd.leaf = true;
      nd.leaf_tris = std::move(w.refs[s.axis]);
      out.num_leaf_tris += nd.leaf_tris.size();
      out.largest_leaf = std::max(out.largest_leaf, nd.leaf_tris.size());
      out.nodes[w.node] = std::move(nd);
      continue;
    }
    Work L, R;
    const std::vector<int32_t>& sa = w.refs[s.axis];
    L.refs[s.axis].assign(sa.begin(), sa.begin() + s.index + 1);
    R.refs[s.axis].assign(sa.begin() + s.index + 1, sa.end());
    for (int32_t r : L.refs[s.axis]) in_left[r] = 1;
    for (int a = 0; a < 3; a++) {
      if (a == s.axis) continue;
      L.refs[a].reserve(L.refs[s.axis].size());
      R.refs[a].reserve(R.refs[s.axis].size());
      for (int32_t r : w.refs[a]) (in_left[r] ? L.refs[a] : R.refs[a]).push_back(r);
    }
    for (int32_t r : L.refs[s.axis]) in_left[r] = 0;
    int li = (int)out.nodes.size();
    out.nodes.emplace_back();
    int ri = (int)out.nodes.size();
    out.nodes.emplace_back();
    nd.left = li; nd.right = ri;
    out.nodes[w.node] = std::move(nd);
    L.node = li; L.depth = w.depth + 1;
    R.node = ri; R.depth = w.depth + 1;
    stack.push_back(std::move(R));   // left is processed first (depth-first, as createChildNodes)
    stack.push_back(std::move(L));
  }
  return out;
}

// Serialised, GPU-format BVH (trace_pass.js:220-263, structs.js:160-210).
struct PackedBVH {
  std::vector<int32_t> nodes5;    // per node: childBaseIdx, triangles, xMask, yMask, zMask (20 B)
  std::vector<int32_t> tri4;      // leaf-ordered {i0,i1,i2,matId}
  std::vector<float> verts4;      // normalised positions, 16-B stride (xyz, 0)
  double root_min[3], root_max[3];
  double center[3];
  double scale;                   // 2 / longest
};

// bvh.js:46-74 serializeTree + trace_pass.js:230-259.
static inline PackedBVH pack_bvh(const BVHBuild& b, const double* pos3, size_t n_verts, const int32_t* tri4) {
  PackedBVH p;
  // BFS with a FIFO queue; parent.left = i for odd i, parent.right = i for even i.
  struct QE { int node; int parent; };
  std::vector<QE> order;
  order.reserve(b.nodes.size());
  std::deque<QE> q;
  q.push_back({0, -1});
  while (!q.empty()) {
    QE e = q.front(); q.pop_front();
    int parent = (int)order.size();
    order.push_back(e);
    if (!b.nodes[e.node].leaf) {
      q.push_back({b.nodes[e.node].left, parent});
      q.push_back({b.nodes[e.node].right, parent});
    }
  }
  std::vector<int> left_of(order.size(), -1);
  for (size_t i = 0; i < order.size(); i++)
    if (order[i].parent >= 0 && (i % 2) == 1) left_of[order[i].parent] = (int)i;
  // #makeNormalizer(root.bounds)
  const Box& rb = b.nodes[0].bounds;
  double span[3];
  for (int i = 0; i < 3; i++) { p.root_min[i] = rb.mn[i]; p.root_max[i] = rb.mx[i]; span[i] = rb.mx[i] - rb.mn[i]; }
  double longest = js_max(js_max(span[0], span[1]), span[2]);
  for (int i = 0; i < 3; i++) p.center[i] = rb.mn[i] + span[i] * 0.5;
  p.scale = 2.0 / longest;
  auto norm = [&](const double* v, double* o) { for (int i = 0; i < 3; i++) o[i] = (v[i] - p.center[i]) * (2.0 / longest); };
  p.nodes5.resize(order.size() * 5);
  int32_t tri_index = 0;
  for (size_t i = 0; i < order.size(); i++) {
    const BuiltNode& nd = b.nodes[order[i].node];
    double mn[3], mx[3];
    norm(nd.bounds.mn, mn);
    norm(nd.bounds.mx, mx);
    int32_t* o = &p.nodes5[5 * i];
    o[0] = nd.leaf ? -1 : left_of[i];
    // maskTriIndex: (numTris << 24) | index, int32 arithmetic.
    o[1] = nd.leaf ? (int32_t)(((uint32_t)nd.leaf_tris.size() << 24) | (uint32_t)tri_index) : -1;
    o[2] = (int32_t)quantize_vec2_to_int(mx[0], mn[0]);
    o[3] = (int32_t)quantize_vec2_to_int(mx[1], mn[1]);
    o[4] = (int32_t)quantize_vec2_to_int(mx[2], mn[2]);
    if (nd.leaf) {
      tri_index += (int32_t)nd.leaf_tris.size();
      for (int32_t t : nd.leaf_tris) for (int k = 0; k < 4; k++) p.tri4.push_back(tri4[4 * (size_t)t + k]);
    }
  }
  p.verts4.resize(n_verts * 4);
  for (size_t v = 0; v < n_verts; v++) {
    double o[3];
    norm(pos3 + 3 * v, o);
    p.verts4[4 * v + 0] = (float)o[0];
    p.verts4[4 * v + 1] = (float)o[1];
    p.verts4[4 * v + 2] = (float)o[2];
    p.verts4[4 * v + 3] = 0.0f;
  }
  return p;
}

// ---- raycaster.js: the CPU autofocus cast (double precision) -------------------
// Raycaster.cast / traverse / closestNode / rayBoxIntersect / rayTriangleIntersect
// (raycaster.js:13-131) on the built tree with exact double bounds.
struct Raycaster {
  const BVHBuild& b;
  const double* pos3;
  const int32_t* tri4;
  double center[3], s;
  double o[3], d[3];
  static constexpr double MAXT = 1e6;
  void norm(const double* v, double* out) const { for (int i = 0; i < 3; i++) out[i] = (v[i] - center[i]) * s; }
  double box(const Box& bb) const {
    double mn[3], mx[3], inv[3];
    norm(bb.mn, mn);
    norm(bb.mx, mx);
    for (int i = 0; i < 3; i++) inv[i] = 1.0 / d[i];
    const double tx1 = (mn[0] - o[0]) * inv[0], tx2 = (mx[0] - o[0]) * inv[0];
    const double ty1 = (mn[1] - o[1]) * inv[1], ty2 = (mx[1] - o[1]) * inv[1];
    const double tz1 = (mn[2] - o[2]) * inv[2], tz2 = (mx[2] - o[2]) * inv[2];
    double tmin = js_min(tx1, tx2), tmax = js_max(tx1, tx2);
    tmin = js_max(tmin, js_min(ty1, ty2));
    tmax = js_min(tmax, js_max(ty1, ty2));
    tmin = js_max(tmin, js_min(tz1, tz2));
    tmax = js_min(tmax, js_max(tz1, tz2));
    return (tmax >= tmin && tmax >= 0) ? tmin : MAXT;
  }
  double tri(int32_t id) const {
    const double eps = 0.000000000001;
    double v0[3], v1[3], v2[3];
    norm(pos3 + 3 * (size_t)tri4[4 * (size_t)id + 0], v0);
    norm(pos3 + 3 * (size_t)tri4[4 * (size_t)id + 1], v1);
    norm(pos3 + 3 * (size_t)tri4[4 * (size_t)id + 2], v2);
    double e1[3], e2[3], tv[3];
    for (int i = 0; i < 3; i++) { e1[i] = v1[i] - v0[i]; e2[i] = v2[i] - v0[i]; tv[i] = o[i] - v0[i]; }
    // Vec3.cross: y = -(a0*b2 - a2*b0); Vec.dot sums from 0 left to right
    const double p[3] = {d[1] * e2[2] - d[2] * e2[1], -(d[0] * e2[2] - d[2] * e2[0]), d[0] * e2[1] - d[1] * e2[0]};
    const double det = 0.0 + e1[0] * p[0] + e1[1] * p[1] + e1[2] * p[2];
    if (det > -eps && det < eps) return MAXT;
    const double inv = 1.0 / det;
    const double u = (0.0 + tv[0] * p[0] + tv[1] * p[1] + tv[2] * p[2]) * inv;
    if (u < 0 || u > 1) return MAXT;
    const double q[3] = {tv[1] * e1[2] - tv[2] * e1[1], -(tv[0] * e1[2] - tv[2] * e1[0]), tv[0] * e1[1] - tv[1] * e1[0]};
    const double v = (0.0 + d[0] * q[0] + d[1] * q[1] + d[2] * q[2]) * inv;
    if (v < 0 || u + v > 1) return MAXT;
    const double t = (0.0 + e2[0] * q[0] + e2[1] * q[1] + e2[2] * q[2]) * inv;
    return t > eps ? t : MAXT;
  }
  double traverse(int node, double closest) const {
    const BuiltNode& n = b.nodes[node];
    if (n.leaf) {
      double res = MAXT;
      for (int32_t id : n.leaf_tris) { const double x = tri(id); if (x < res) res = x; }
      return res;
    }
    const double tl = box(b.nodes[n.left].bounds), tr = box(b.nodes[n.right].bounds);
    const int l = tl < MAXT ? n.left : -1, r = tr < MAXT ? n.right : -1;
    int ord[2];
    double ot[2];
    if (tl < tr) { ord[0] = l; ot[0] = tl; ord[1] = r; ot[1] = tr; } else { ord[0] = r; ot[0] = tr; ord[1] = l; ot[1] = tl; }
    for (int i = 0; i < 2; i++) {
      if (ord[i] >= 0 && ot[i] < closest) {
        const double res = traverse(ord[i], closest);
        closest = js_min(res, closest);
      }
    }
    return closest;
  }
};

// ---- Row E: env_sampler.js tables ----------------------------------------
struct EnvTables {
  uint32_t w = 0, h = 0;
  std::vector<uint8_t> rgbe;       // rgba8 texels (alpha = shared exponent)
  std::vector<int32_t> bins2;      // {h0, h1}
  std::vector<int32_t> coords2;    // {x, y} in descending-radiance order
  std::vector<float> pdf;          // r32f, texel (x + w*y)
  double total = 0, brightest = 0;
};
// The tables from per-texel radiance in row-major order (_sortPixels: y
// outer, x inner): totalRadiance and brightestTexel accumulated in that order,
// stable descending sort, equal-mass bins, pdf.
static inline void build_env_from_rad(EnvTables& e, const std::vector<double>& rad) {
  const uint32_t w = e.w;
  const size_t N = rad.size();
  for (size_t i = 0; i < N; i++) {
    e.brightest = js_max(rad[i], e.brightest);
    e.total += rad[i];
  }
  std::vector<int32_t> order(N);
  for (size_t i = 0; i < N; i++) order[i] = (int32_t)i;
  // sort((a,b) => b.rad - a.rad): stable, descending.
  std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return rad[b] - rad[a] < 0; });
  double num_bins = js_min(256.0, js_max(32.0, 2.0 * std::ceil(e.total / e.brightest)));
  if (!(num_bins == num_bins)) throw std::runtime_error("env: black environment (the reference throws here too)");
  double bin_size = e.total / num_bins;
  double current = 0;
  for (size_t i = 0; i < N; i++) {
    if (current >= bin_size) {
      int32_t prev = e.bins2.empty() ? 0 : e.bins2.back();
      e.bins2.push_back(prev);
      e.bins2.push_back((int32_t)i);
      current = 0;
    }
    current += rad[order[i]];
  }
  if (e.bins2.empty()) throw std::runtime_error("env: fewer than two bins (the reference throws here too)");
  int32_t last = e.bins2.back();
  e.bins2.push_back(last);
  e.bins2.push_back((int32_t)N);
  e.coords2.resize(2 * N);
  for (size_t i = 0; i < N; i++) {
    e.coords2[2 * i] = order[i] % (int32_t)w;
    e.coords2[2 * i + 1] = order[i] / (int32_t)w;
  }
  e.pdf.assign(N, 0.0f);
  const size_t nb = e.bins2.size() / 2;
  for (size_t b = 0; b < nb; b++) {
    int32_t h0 = e.bins2[2 * b], h1 = e.bins2[2 * b + 1];
    for (int32_t i = h0; i < h1; i++) {
      double bin_pdf = 1.0 / (double)nb;
      double coord_pdf = (double)N / (double)(h1 - h0);
      double sphere_pdf = 1.0 / (M_PI * M_PI * 2.0);
      double pdf = bin_pdf * coord_pdf * sphere_pdf;
      e.pdf[order[i]] = (float)pdf;
    }
  }
}
static inline EnvTables build_env(const uint8_t* rgbe, uint32_t w, uint32_t h) {
  EnvTables e;
  e.w = w; e.h = h;
  const size_t N = (size_t)w * h;
  e.rgbe.assign(rgbe, rgbe + 4 * N);
  std::vector<double> rad(N);
  // _getRadiance = 2^(a-128) * luma / 255.
  for (size_t i = 0; i < N; i++) {
    const uint8_t* c = rgbe + 4 * i;
    double power = std::ldexp(1.0, (int)c[3] - 128);
    double luma = 0.2126 * c[0] + 0.7152 * c[1] + 0.0722 * c[2];
    rad[i] = power * luma / 255.0;
  }
  build_env_from_rad(e, rad);
  return e;
}
// The same tables for an FP32 RGB map (the differentiable renderer's
// sampling environment, pk_diff_set_env_sampling): radiance = luma of the
// stored values in double, negative or NaN radiance taken as 0.
static inline EnvTables build_env_f32(const float* rgb, uint32_t w, uint32_t h) {
  EnvTables e;
  e.w = w; e.h = h;
  const size_t N = (size_t)w * h;
  std::vector<double> rad(N);
  for (size_t i = 0; i < N; i++) {
    const double r = 0.2126 * (double)rgb[3 * i] + 0.7152 * (double)rgb[3 * i + 1] + 0.0722 * (double)rgb[3 * i + 2];
    rad[i] = r > 0.0 ? r : 0.0;
  }
  build_env_from_rad(e, rad);
  return e;
}

}  // namespace om
