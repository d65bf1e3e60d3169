// om_render.h -- oracle restatement of Pike's per-frame passes.
//
// TEST INFRASTRUCTURE ONLY (see om_math.h).  Parity unpinned (see om_build.h).
//
// Follows line by line:
//   render/shader/camera.wgsl:46-92        hash, rand, createPrimaryRay, main
//   render/shader/trace.wgsl:83-213        rayBoxIntersect, rayTriangleIntersect, processLeaf,
//                                          stack, intersectScene (closest hit), main
//   render/shader/trace_shadow.wgsl:82-207 any-hit variant (EPSILON 1e-7, early exit)
//   render/shader/shade_hit.wgsl:153-483   surface interaction, GGX/Lambert, env sampling, MIS
//   render/shader/shade_miss.wgsl:37-57    env lookup
//   render/shader/accumulate.wgsl:20-34    running mean
//   render/shader/postprocess.wgsl:36-99   ACES fit, saturation, sRGB
//   render/passes/camera_pass.js:3-77      RenderState counters and clears
//   render/pike.js:120-162                 tick(): pass order per frame
// Invocation order is serial: atomics are incremented in increasing global
// invocation id, which is the order a stable compaction produces.
#pragma once
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "om_math.h"
#include "om_render64.h"

namespace om {

struct DeferredRay { float o[3]; float d[3]; float tp[4]; };
struct Hit { float t; int32_t index; uint32_t bary; DeferredRay ray; };
struct CameraState {
  float pos[3]; float dir[3]; uint32_t dims_mask; float fov; float focal_depth;
  float aperture; float distortion; float bokeh; uint32_t invocation_offset;
};

struct Stats { uint64_t node_fetch = 0, tri_tests = 0, rays = 0; uint32_t max_stack = 0; };

template <class F>
static inline void parallel_for(size_t n, int nthreads, F fn) {
  if (nthreads <= 1 || n < 2048) { fn(0, n, 0); return; }
  std::vector<std::thread> th;
  size_t chunk = (n + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; t++) {
    size_t b = t * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    th.emplace_back([=]() { fn(b, e, t); });
  }
  for (auto& x : th) x.join();
}

struct Hash {
  uint32_t seed;
  // camera.wgsl:46-52 (Jarzynski & Olano PCG-style hash)
  uint32_t hash() {
    uint32_t state = seed;
    seed = seed * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
  }
  float rand() { return (float)hash() / 4294967296.0f; }
};

static const float TAU_F = 6.283185307179586f;
static const float INV_PI_F = 0.3183098861837907f;
static const float MAX_T = 100000.0f;

struct Renderer {
  // configuration
  uint32_t W = 0, H = 0, B = 0;
  int nthreads = 1;
  // RenderState (camera_pass.js:3-77)
  int32_t samples = 0; float env_theta = 0.0f;
  uint32_t num_hits = 0, num_misses = 0, num_rays = 0, num_shadow = 0;
  std::vector<float> color, temp, display;
  std::vector<uint8_t> display8;
  std::vector<DeferredRay> ray_buffer, miss_buffer;
  std::vector<Hit> hit_buffer;
  uint32_t overflow = 0;
  // scene
  std::vector<int32_t> nodes5, tri4;
  std::vector<float> verts4;
  std::vector<uint32_t> attrs4;
  std::vector<int32_t> mat4;
  std::vector<uint8_t> layers;   // rgba8, atlas_res x atlas_res per layer
  int32_t atlas_res = 1;
  // env
  uint32_t env_w = 0, env_h = 0;
  std::vector<uint8_t> env_rgbe;
  std::vector<int32_t> env_bins2, env_coords2;
  std::vector<float> env_pdf;
  bool sample_env_light = true;
  CameraState cam{};
  float exposure = 1.0f, saturation = 1.0f;
  Stats trace_stats, shadow_stats;
  // FP64 companion (om_render64.h): per-ray FP64 throughput of the ray,
  // hit and miss buffers (3 doubles per slot), the frame's FP64 colour, its
  // running mean (accumulate.wgsl in double) and Welford moments of the
  // per-frame colour since set_track64.
  bool track64 = false;
  // With share_texels, the FP64 evaluation takes the texel indices of the
  // two nearest-texel lookups (envPdf's pdf texel for the bounce MIS weight,
  // envColor's texel on a miss) from the FP32 evaluation, and keeps its own
  // FP64 arithmetic everywhere else.  A texel choice is a discontinuous
  // function of the direction: near a texel boundary any rounding flips it.
  bool share_texels = false;
  std::vector<double> ray64, hit64, miss64, color64, accum64, mean64, m2_64;
  uint64_t frames64 = 0;
  void alloc64() {
    ray64.assign(3 * ray_buffer.size(), 0.0);
    hit64.assign(3 * hit_buffer.size(), 0.0);
    miss64.assign(3 * miss_buffer.size(), 0.0);
    color64.assign(4 * (size_t)W * H, 0.0);
    accum64.assign(4 * (size_t)W * H, 0.0);
    mean64.assign(4 * (size_t)W * H, 0.0);
    m2_64.assign(4 * (size_t)W * H, 0.0);
    frames64 = 0;
  }
  void set_track64(bool on, bool shared_texels = false) {
    track64 = on;
    share_texels = on && shared_texels;
    if (on) alloc64();
  }
  // envPdf's (shade_hit.wgsl:202-210) and envColor's (shade_miss.wgsl:37-43)
  // texel indices as the FP32 passes compute them for direction d.
  void pdf_texel_index32(V3 dir, int32_t* cx, int32_t* cy) const {
    float a = 1.0f + env_theta + atan2_(dir.z, dir.x) / TAU_F;
    float u = a - std::trunc(a);
    float v = acos_(dir.y) * INV_PI_F;
    *cx = f2i(u * (float)env_w);
    *cy = f2i(v * (float)env_h);
  }
  void color_texel_index32(V3 dir, int32_t* x, int32_t* y) const {
    float u = env_theta + atan2_(dir.z, dir.x) / TAU_F;
    float v = acos_(dir.y) * INV_PI_F;
    *x = f2i(std::floor(u * (float)env_w));
    *y = f2i(std::floor(v * (float)env_h));
  }

  // Queues hold the camera dispatch of a batch, rounded up to 128 invocations
  // (camera.wgsl's workgroup size), as the GPU's do.
  void configure(uint32_t w, uint32_t h, uint32_t batch) {
    W = w; H = h; B = batch;
    const size_t cap = round_up(B, 128);
    color.assign(4 * (size_t)W * H, 0.0f);
    temp.assign(4 * (size_t)W * H, 0.0f);
    display.assign(4 * (size_t)W * H, 0.0f);
    display8.assign(4 * (size_t)W * H, 0);
    ray_buffer.assign(3 * cap, DeferredRay{});
    miss_buffer.assign(2 * cap, DeferredRay{});
    hit_buffer.assign(cap, Hit{});
    if (track64) alloc64();
  }
  static uint32_t round_up(uint32_t n, uint32_t m) { return (n + m - 1) / m * m; }

  // ---------------- camera.wgsl ----------------
  V3 create_primary_ray_dir(Hash& h, float px, float py, float rx, float ry, V3* origin_out) const {
    const float k = cam.distortion;
    float jx = h.rand();
    float jy = h.rand();
    float ux = (2.0f * ((px + jx) / rx) - 1.0f) * (rx / ry);
    float uy = (2.0f * ((py + jy) / ry) - 1.0f) * -1.0f;
    float rd = std::sqrt(ux * ux + uy * uy);
    float ru = rd * (1.0f + k * rd * rd);
    float l = std::sqrt(ux * ux + uy * uy);
    float nx = ux / l, ny = uy / l;
    ux = ru * nx; uy = ru * ny;
    V3 eye_o = v3(cam.pos[0], cam.pos[1], cam.pos[2]);
    V3 eye_d = v3(cam.dir[0], cam.dir[1], cam.dir[2]);
    V3 up = v3(0.0f, 1.0f, 0.0f);
    float tf = tan_(cam.fov * 0.5f);
    V3 bx = scale(normalize(cross(eye_d, up)), tf);
    V3 by = scale(normalize(cross(bx, eye_d)), tf);
    float theta = h.rand() * TAU_F;
    float pw = pow_(h.rand(), cam.bokeh);
    V3 dof = scale(scale(add(scale(bx, cos_(theta)), scale(by, sin_(theta))), cam.aperture), pw);
    V3 screen = add(add(add(scale(bx, ux), scale(by, uy)), eye_d), eye_o);
    V3 dir = normalize(sub(add(screen, scale(dof, cam.focal_depth)), add(eye_o, dof)));
    *origin_out = add(dof, eye_o);
    return dir;
  }
  void pass_camera() {
    const uint32_t Wd = cam.dims_mask >> 16, Hd = cam.dims_mask & 0xffffu;
    const uint32_t n = round_up(B, 128);
    std::vector<uint8_t> valid(n, 0);
    std::vector<DeferredRay> out(n);
    parallel_for(n, nthreads, [&](size_t b, size_t e, int) {
      for (size_t gid = b; gid < e; gid++) {
        uint32_t idx = (uint32_t)gid + cam.invocation_offset;
        uint32_t px = idx % Wd, py = idx / Wd;
        if (px >= Wd || py >= Hd) continue;
        Hash h;
        h.seed = (px * 1973u + py * 9277u + (uint32_t)samples * 26699u) | 1u;
        h.seed = h.hash();
        V3 o;
        V3 d = create_primary_ray_dir(h, (float)px, (float)py, (float)Wd, (float)Hd, &o);
        DeferredRay r;
        r.o[0] = o.x; r.o[1] = o.y; r.o[2] = o.z;
        r.d[0] = d.x; r.d[1] = d.y; r.d[2] = d.z;
        r.tp[0] = r.tp[1] = r.tp[2] = 1.0f;
        r.tp[3] = u2f(idx);
        out[gid] = r;
        valid[gid] = 1;
      }
    });
    for (uint32_t gid = 0; gid < n; gid++) {
      if (!valid[gid]) continue;
      if (gid < ray_buffer.size()) {
        ray_buffer[gid] = out[gid];
        if (track64) ray64[3 * gid] = ray64[3 * gid + 1] = ray64[3 * gid + 2] = 1.0;
      } else {
        overflow |= 1;
      }
      num_rays++;
    }
  }

  // ---------------- trace.wgsl / trace_shadow.wgsl ----------------
  static float box_hit(const int32_t* node, V3 o, V3 inv) {
    float xr0, xr1, yr0, yr1, zr0, zr1;
    unpack2x16snorm((uint32_t)node[2], &xr0, &xr1);
    unpack2x16snorm((uint32_t)node[3], &yr0, &yr1);
    unpack2x16snorm((uint32_t)node[4], &zr0, &zr1);
    V3 t1 = mul(sub(v3(xr0, yr0, zr0), o), inv);
    V3 t2 = mul(sub(v3(xr1, yr1, zr1), o), inv);
    V3 mn = v3(fmin_(t1.x, t2.x), fmin_(t1.y, t2.y), fmin_(t1.z, t2.z));
    V3 mx = v3(fmax_(t1.x, t2.x), fmax_(t1.y, t2.y), fmax_(t1.z, t2.z));
    float tmax = fmin_(fmin_(mx.x, mx.y), mx.z);
    float tmin = fmax_(fmax_(mn.x, mn.y), mn.z);
    return (tmax >= tmin && tmax > 0.0f) ? tmin : MAX_T;
  }
  V3 vert(int32_t i) const { return v3(verts4[4 * (size_t)i], verts4[4 * (size_t)i + 1], verts4[4 * (size_t)i + 2]); }
  float tri_hit(V3 o, V3 d, const int32_t* tri, float eps, uint32_t* bary) const {
    V3 v0 = vert(tri[0]);
    V3 e1 = sub(vert(tri[1]), v0);
    V3 e2 = sub(vert(tri[2]), v0);
    V3 p = cross(d, e2);
    float det = dot(e1, p);
    if (std::fabs(det) < eps) return MAX_T;
    float inv_det = 1.0f / det;
    V3 t = sub(o, v0);
    float u = dot(t, p) * inv_det;
    if (u < 0.0f || u > 1.0f) return MAX_T;
    V3 q = cross(t, e1);
    float v = dot(d, q) * inv_det;
    if (v < 0.0f || u + v > 1.0f) return MAX_T;
    float dist = dot(e2, q) * inv_det;
    *bary = pack2x16unorm(u, v);
    return dist > eps ? dist : MAX_T;
  }
  // The watertight test of form (1) (Woop, Benthin & Wald, JCGT 2013), the
  // device's wt_setup / wt_test restated: kz = axis of largest |d| (first of
  // equals), kx, ky cyclic after it and swapped when d[kz] < 0; shear
  // S = (d[kx]/d[kz], d[ky]/d[kz], 1/d[kz]); an edge function exactly 0 is
  // recomputed in double; t = T/det accepted when t > eps; (u, v) = (V, W)/det.
  struct WtRay { int kx, ky, kz; float sx, sy, sz; float o[3]; };
  static WtRay wt_setup(V3 o, V3 d) {
    const float dv[3] = {d.x, d.y, d.z}, ov[3] = {o.x, o.y, o.z};
    const float ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
    int kz = 0;
    float m = ax;
    if (ay > m) { kz = 1; m = ay; }
    if (az > m) kz = 2;
    int kx = kz == 2 ? 0 : kz + 1;
    int ky = kx == 2 ? 0 : kx + 1;
    if (dv[kz] < 0.0f) std::swap(kx, ky);
    WtRay w;
    w.kx = kx; w.ky = ky; w.kz = kz;
    w.sx = dv[kx] / dv[kz];
    w.sy = dv[ky] / dv[kz];
    w.sz = 1.0f / dv[kz];
    w.o[0] = ov[kx]; w.o[1] = ov[ky]; w.o[2] = ov[kz];
    return w;
  }
  float tri_hit_wt(const WtRay& r, const int32_t* tri, float eps, uint32_t* bary) const {
    float p[3][3];
    for (int k = 0; k < 3; k++) {
      const V3 v = vert(tri[k]);
      const float c[3] = {v.x, v.y, v.z};
      p[k][0] = c[r.kx] - r.o[0];
      p[k][1] = c[r.ky] - r.o[1];
      p[k][2] = c[r.kz] - r.o[2];
    }
    const float Ax = p[0][0] - r.sx * p[0][2], Ay = p[0][1] - r.sy * p[0][2];
    const float Bx = p[1][0] - r.sx * p[1][2], By = p[1][1] - r.sy * p[1][2];
    const float Cx = p[2][0] - r.sx * p[2][2], Cy = p[2][1] - r.sy * p[2][2];
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
      U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
      V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
      W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return MAX_T;
    const float det = U + V + W;
    if (det == 0.0f) return MAX_T;
    const float Az = r.sz * p[0][2], Bz = r.sz * p[1][2], Cz = r.sz * p[2][2];
    const float T = U * Az + V * Bz + W * Cz;
    const float t = T / det;
    if (!(t > eps)) return MAX_T;
    *bary = pack2x16unorm(V / det, W / det);
    return t;
  }
  struct TravResult { float t; int32_t index; uint32_t bary; uint32_t fetch, tests, max_stack; };
  // Order-independent answer: every triangle tested with the watertight test,
  // closest = min (t, slot), any = some triangle accepted.  Used in place of
  // intersect() when `canonical` is set (the reference of form (1)'s 8-wide
  // and FP32 binary traversals).
  bool canonical = false;
  template <bool ANY>
  TravResult brute(V3 o, V3 d) const {
    const float eps = ANY ? 1e-7f : 1e-8f;
    TravResult r{MAX_T, -1, 0u, 0u, 0u, 0u};
    const size_t nt = tri4.size() / 4;
    const WtRay wr = wt_setup(o, d);
    for (size_t k = 0; k < nt; k++) {
      uint32_t bary = 0u;
      const float res = tri_hit_wt(wr, &tri4[4 * k], eps, &bary);
      if (res < r.t) {
        r.t = res;
        r.index = (int32_t)k;
        r.bary = bary;
        if (ANY) break;
      }
    }
    return r;
  }
  template <bool ANY>
  TravResult intersect(V3 o, V3 d, std::vector<int32_t>& stack) const {
    const float eps = ANY ? 1e-7f : 1e-8f;
    TravResult r{MAX_T, -1, 0u, 0u, 0u, 0u};
    V3 inv = v3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    stack.clear();
    stack.push_back(-1);
    int32_t idx = 0;
    for (;;) {
      if (idx <= -1) break;
      const int32_t* cur = &nodes5[5 * (size_t)idx];
      r.fetch++;
      if (cur[1] > -1) {
        const int32_t leaf_size = cur[1] >> 24;
        const int32_t base = cur[1] & 0x00ffffff;
        for (int32_t i = 0; i < leaf_size; i++) {
          uint32_t bary = 0;
          r.tests++;
          float res = tri_hit(o, d, &tri4[4 * (size_t)(base + i)], eps, &bary);
          if (res < r.t) { r.index = base + i; r.t = res; r.bary = bary; }
        }
        if (ANY && r.index != -1) return r;
      } else {
        int32_t li = cur[0], ri = li + 1;
        r.fetch += 2;
        float lh = box_hit(&nodes5[5 * (size_t)li], o, inv);
        float rh = box_hit(&nodes5[5 * (size_t)ri], o, inv);
        if (lh < r.t && rh < r.t) {
          int32_t deferred;
          if (lh > rh) { idx = ri; deferred = li; } else { idx = li; deferred = ri; }
          stack.push_back(deferred);
          r.max_stack = std::max<uint32_t>(r.max_stack, (uint32_t)stack.size() - 1);
          continue;
        } else {
          if (lh < r.t) { idx = li; continue; }
          if (rh < r.t) { idx = ri; continue; }
        }
      }
      idx = stack.back();
      stack.pop_back();
    }
    return r;
  }
  void pass_trace() {
    num_hits = 0; num_misses = 0;   // TracePass.generateCommands: clearNumHitsAndMisses
    const uint32_t n = std::min<uint32_t>(num_rays, shadow_offset());
    std::vector<TravResult> res(n);
    parallel_for(n, nthreads, [&](size_t b, size_t e, int) {
      std::vector<int32_t> stack;
      for (size_t j = b; j < e; j++) {
        const DeferredRay& r = ray_buffer[j];
        res[j] = canonical ? brute<false>(v3(r.o[0], r.o[1], r.o[2]), v3(r.d[0], r.d[1], r.d[2]))
                           : intersect<false>(v3(r.o[0], r.o[1], r.o[2]), v3(r.d[0], r.d[1], r.d[2]), stack);
      }
    });
    for (uint32_t j = 0; j < n; j++) {
      trace_stats.node_fetch += res[j].fetch;
      trace_stats.tri_tests += res[j].tests;
      trace_stats.max_stack = std::max(trace_stats.max_stack, res[j].max_stack);
      trace_stats.rays++;
      if (res[j].index != -1) {
        uint32_t k = num_hits++;
        if (k < hit_buffer.size()) hit_buffer[k] = Hit{res[j].t, res[j].index, res[j].bary, ray_buffer[j]}; else overflow |= 2;
        if (track64 && k < hit_buffer.size()) copy64(&hit64[3 * (size_t)k], &ray64[3 * (size_t)j]);
      } else {
        uint32_t k = num_misses++;
        if (k < miss_buffer.size()) miss_buffer[k] = ray_buffer[j]; else overflow |= 4;
        if (track64 && k < miss_buffer.size()) copy64(&miss64[3 * (size_t)k], &ray64[3 * (size_t)j]);
      }
    }
  }
  uint32_t shadow_offset() const { return (uint32_t)(ray_buffer.size() / 2); }
  void pass_trace_shadow() {
    const uint32_t off = shadow_offset();
    const uint32_t n = std::min<uint32_t>(num_shadow, (uint32_t)(ray_buffer.size() - off));
    std::vector<TravResult> res(n);
    parallel_for(n, nthreads, [&](size_t b, size_t e, int) {
      std::vector<int32_t> stack;
      for (size_t j = b; j < e; j++) {
        const DeferredRay& r = ray_buffer[off + j];
        res[j] = canonical ? brute<true>(v3(r.o[0], r.o[1], r.o[2]), v3(r.d[0], r.d[1], r.d[2]))
                           : intersect<true>(v3(r.o[0], r.o[1], r.o[2]), v3(r.d[0], r.d[1], r.d[2]), stack);
      }
    });
    for (uint32_t j = 0; j < n; j++) {
      shadow_stats.node_fetch += res[j].fetch;
      shadow_stats.tri_tests += res[j].tests;
      shadow_stats.max_stack = std::max(shadow_stats.max_stack, res[j].max_stack);
      shadow_stats.rays++;
      if (res[j].index == -1) {
        uint32_t k = num_misses++;
        if (k < miss_buffer.size()) miss_buffer[k] = ray_buffer[off + j]; else overflow |= 4;
        if (track64 && k < miss_buffer.size()) copy64(&miss64[3 * (size_t)k], &ray64[3 * ((size_t)off + j)]);
      }
    }
  }

  // ---------------- shade_hit.wgsl ----------------
  struct SI {
    V3 b1, b2, n;  // basis columns
    V3 wo, origin, normal, base, spec, emission;
    float metallic, opacity, alpha;
  };
  struct Sample { V3 wi; float pdf; };
  // textureSampleLevel(atlas, linear sampler with repeat addressing, uv, layer, 0)
  // on rgba8unorm layers (shade_hit.wgsl:184-197; sampler: shade_hit_pass.js:83-90).
  // A 1x1 layer returns its texel.  Larger layers filter bilinearly: texel
  // space x = u*R - 0.5, i0 = floor(x), fx = x - i0, indices wrap, and
  // mix(mix(t00, t10, fx), mix(t01, t11, fx), fy) with mix(a,b,t) = a(1-t) + bt.
  void texel_at(int32_t l, int32_t i, int32_t j, float* c) const {
    const int32_t R = atlas_res;
    i = ((i % R) + R) % R;
    j = ((j % R) + R) % R;
    const uint8_t* p = &layers[4 * (((size_t)l * R + (size_t)j) * R + (size_t)i)];
    for (int k = 0; k < 4; k++) c[k] = (float)p[k] / 255.0f;
  }
  void texel(int32_t layer, float u, float v, float* c) const {
    const int32_t R = atlas_res;
    const int32_t nl = (int32_t)(layers.size() / (4 * (size_t)R * R));
    const int32_t l = layer < 0 ? 0 : (layer >= nl ? nl - 1 : layer);
    if (R == 1) { texel_at(l, 0, 0, c); return; }
    const float x = u * (float)R - 0.5f, y = v * (float)R - 0.5f;
    const float x0 = std::floor(x), y0 = std::floor(y);
    const float fx = x - x0, fy = y - y0;
    const int32_t i0 = f2i(x0), j0 = f2i(y0);
    float t00[4], t10[4], t01[4], t11[4];
    texel_at(l, i0, j0, t00);
    texel_at(l, i0 + 1, j0, t10);
    texel_at(l, i0, j0 + 1, t01);
    texel_at(l, i0 + 1, j0 + 1, t11);
    for (int k = 0; k < 4; k++) c[k] = mix1(mix1(t00[k], t10[k], fx), mix1(t01[k], t11[k], fx), fy);
  }
  static void onb(V3 n, V3* b1, V3* b2) {
    float sign = n.z > 0.0f ? 1.0f : -1.0f;
    float a = -1.0f / (sign + n.z);
    float b = n.x * n.y * a;
    *b1 = v3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
    *b2 = v3(b, sign + n.y * n.y * a, -n.y);
  }
  SI surface(const Hit& hit) const {
    SI si;
    V3 ro = v3(hit.ray.o[0], hit.ray.o[1], hit.ray.o[2]);
    V3 rd = v3(hit.ray.d[0], hit.ray.d[1], hit.ray.d[2]);
    const int32_t* tri = &tri4[4 * (size_t)hit.index];
    float u, v;
    unpack2x16unorm(hit.bary, &u, &v);
    V3 bary = v3(1.0f - u - v, u, v);
    V3 tg[3], bt[3], nm[3];
    float uvx[3], uvy[3];
    for (int k = 0; k < 3; k++) {
      const uint32_t* a = &attrs4[4 * (size_t)tri[k]];
      unpack4x8snorm3(a[0], &tg[k].x, &tg[k].y, &tg[k].z);
      unpack4x8snorm3(a[1], &bt[k].x, &bt[k].y, &bt[k].z);
      unpack4x8snorm3(a[2], &nm[k].x, &nm[k].y, &nm[k].z);
      unpack2x16snorm(a[3], &uvx[k], &uvy[k]);
    }
    V3 T = normalize(matvec(tg[0], tg[1], tg[2], bary));
    V3 Bt = normalize(matvec(bt[0], bt[1], bt[2], bary));
    V3 N = normalize(matvec(nm[0], nm[1], nm[2], bary));
    const float tu = uvx[0] * bary.x + uvx[1] * bary.y + uvx[2] * bary.z;  // uvs * bary (mat3x2 * vec3)
    const float tv = uvy[0] * bary.x + uvy[1] * bary.y + uvy[2] * bary.z;
    const int32_t* mat = &mat4[4 * (size_t)tri[3]];
    float nrm[4], dif[4], mr[4], em[4];
    texel(mat[2], tu, tv, nrm);
    V3 map_normal = mul(sub(v3(nrm[0], nrm[1], nrm[2]), v3(0.5f, 0.5f, 0.0f)), v3(2.0f, 2.0f, 1.0f));
    si.normal = normalize(matvec(T, Bt, N, map_normal));
    si.origin = add(ro, scale(rd, hit.t - 1e-7f * 40.0f));
    si.n = si.normal;
    onb(si.normal, &si.b1, &si.b2);
    si.wo = vecmat(neg(rd), si.b1, si.b2, si.n);
    texel(mat[0], tu, tv, dif);
    si.base = v3(dif[0], dif[1], dif[2]);
    si.opacity = dif[3];
    texel(mat[1], tu, tv, mr);
    si.metallic = mr[2];
    si.alpha = mr[1] * mr[1];
    texel(mat[3], tu, tv, em);
    si.emission = v3(em[0], em[1], em[2]);
    si.spec = v3(mix1(1.0f, si.base.x, si.metallic), mix1(1.0f, si.base.y, si.metallic), mix1(1.0f, si.base.z, si.metallic));
    return si;
  }
  float pdf_texel(int32_t x, int32_t y) const {
    if (x < 0 || y < 0 || x >= (int32_t)env_w || y >= (int32_t)env_h) return 0.0f;
    return env_pdf[(size_t)x + (size_t)env_w * (size_t)y];
  }
  float env_pdf_dir(V3 dir) const {
    float dx = (float)env_w, dy = (float)env_h;
    float a = 1.0f + env_theta + atan2_(dir.z, dir.x) / TAU_F;
    float u = a - std::trunc(a);
    float v = acos_(dir.y) * INV_PI_F;
    int32_t cx = f2i(u * dx), cy = f2i(v * dy);
    float phi = v * PI_F;
    float sin_phi = sin_(phi);
    return pdf_texel(cx, cy) / sin_phi;
  }
  // Alias-table sampling of the library's PK_ENV_ALIAS (no reference
  // counterpart): per texel {keep threshold, alias}; env_pdf then holds the
  // table's pdf texture.  Empty: the reference's histogram.
  std::vector<uint32_t> env_alias2;
  Sample sample_env(Hash& h, const SI& si) const {
    float dx = (float)env_w, dy = (float)env_h;
    int32_t cx, cy;
    if (!env_alias2.empty()) {
      const uint32_t n = env_w * env_h;
      const uint32_t i = h.hash() % n;
      const uint32_t thr = env_alias2[2 * (size_t)i], al = env_alias2[2 * (size_t)i + 1];
      const uint32_t r = h.hash();
      const uint32_t k = (thr == 0xffffffffu || r < thr) ? i : al;
      cx = (int32_t)(k % env_w);
      cy = (int32_t)(k / env_w);
    } else {
      uint32_t nb = (uint32_t)(env_bins2.size() / 2);
      int32_t idx = (int32_t)(h.hash() % nb);
      int32_t h0 = env_bins2[2 * idx], h1 = env_bins2[2 * idx + 1];
      int32_t ci = (int32_t)(h.hash() % (uint32_t)(h1 - h0)) + h0;
      cx = env_coords2[2 * (size_t)ci];
      cy = env_coords2[2 * (size_t)ci + 1];
    }
    float u = -env_theta + ((0.5f + (float)cx) / dx);
    float v = (0.5f + (float)cy) / dy;
    float theta = u * TAU_F;
    float phi = v * PI_F;
    float sin_phi = sin_(phi);
    V3 dir = v3(cos_(theta) * sin_phi, cos_(phi), sin_(theta) * sin_phi);
    float pdf = pdf_texel(cx, cy) / sin_phi;
    return Sample{vecmat(dir, si.b1, si.b2, si.n), pdf};
  }
  // sampleEnv's direction for texel (cx, cy) (shade_hit.wgsl:218-224, before
  // the ONB) and envPdf's texel index for that direction (:202-206).
  void env_roundtrip(int32_t cx, int32_t cy, float* dir3, int32_t* ix, int32_t* iy) const {
    const float dx = (float)env_w, dy = (float)env_h;
    const float u = -env_theta + ((0.5f + (float)cx) / dx);
    const float v = (0.5f + (float)cy) / dy;
    const float theta = u * TAU_F, phi = v * PI_F, sin_phi = sin_(phi);
    const V3 dir = v3(cos_(theta) * sin_phi, cos_(phi), sin_(theta) * sin_phi);
    dir3[0] = dir.x; dir3[1] = dir.y; dir3[2] = dir.z;
    pdf_texel_index32(dir, ix, iy);
  }
  static float lambert_pdf(V3 wi) { return fmax_(wi.z, 1e-7f) * INV_PI_F; }
  static Sample sample_lambert(Hash& h) {
    float r = std::sqrt(h.rand());
    float phi = TAU_F * h.rand();
    float x = r * cos_(phi);
    float y = r * sin_(phi);
    float z = std::sqrt(fmax_(0.0f, 1.0f - x * x - y * y));
    V3 d = v3(x, y, z);
    return Sample{d, lambert_pdf(d)};
  }
  static V3 eval_lambert(const SI& si, const Sample& s) {
    float w = fmax_(1e-7f, s.wi.z);
    return v3(si.base.x * INV_PI_F * w / s.pdf, si.base.y * INV_PI_F * w / s.pdf, si.base.z * INV_PI_F * w / s.pdf);
  }
  static float ggx_d(V3 m, float au, float av) {
    float auv = au * av;
    float tx = m.x / au;
    float ty = m.y / av;
    float ell = tx * tx + ty * ty + m.z * m.z;
    return 1.0f / (PI_F * auv * ell * ell);
  }
  static float ggx_g1(V3 w, V3 m, float au, float av) {
    float ax = w.x * au;
    float ay = w.y * av;
    float axy2 = ax * ax + ay * ay;
    float tan_theta = axy2 / (w.z * w.z);
    float result = 2.0f / (1.0f + std::sqrt(1.0f + tan_theta));
    return (dot(w, m) * dot(w, v3(0.0f, 0.0f, 1.0f)) <= 0.0f) ? 0.0f : result;
  }
  static V3 sample_ggx(Hash& h, const SI& si) {
    float au = si.alpha, av = si.alpha;
    V3 vh = normalize(v3(au * si.wo.x, av * si.wo.y, si.wo.z));
    float lensq = vh.x * vh.x + vh.y * vh.y;
    V3 t1v = lensq > 0.0f ? scale(v3(-vh.y, vh.x, 0.0f), inverse_sqrt(lensq)) : v3(1.0f, 0.0f, 0.0f);
    V3 t2v = cross(vh, t1v);
    float r = std::sqrt(h.rand());
    float phi = TAU_F * h.rand();
    float t1 = r * cos_(phi);
    float t2 = r * sin_(phi);
    float s = 0.5f * (1.0f + vh.z);
    t2 = (1.0f - s) * std::sqrt(1.0f - t1 * t1) + s * t2;
    V3 nh = add(add(scale(t1v, t1), scale(t2v, t2)), scale(vh, std::sqrt(fmax_(0.0f, 1.0f - t1 * t1 - t2 * t2))));
    return normalize(v3(au * nh.x, av * nh.y, fmax_(0.0f, nh.z)));
  }
  static float specular_pdf(const SI& si, V3 m) {
    float a = si.alpha;
    return fmax_(1e-7f, ggx_d(m, a, a) * ggx_g1(si.wo, m, a, a) / (4.0f * si.wo.z));
  }
  static V3 eval_specular(const SI& si, const Sample& s) {
    float a = si.alpha;
    V3 hv = normalize(add(si.wo, s.wi));
    float D = ggx_d(hv, a, a);
    float G = ggx_g1(s.wi, hv, a, a) * ggx_g1(si.wo, hv, a, a);
    float k = fmax_(D * G / (4.0f * si.wo.z * s.pdf), 0.0f);
    return scale(si.spec, k);
  }
  static float power_heuristic(float p0, float p1) { float p02 = p0 * p0; return p02 / (p02 + p1 * p1); }
  static float schlick(float cos_theta, float ior) {
    float r0 = (1.0f - ior) / (1.0f + ior);
    r0 = r0 * r0;
    float tmp = 1.0f - cos_theta;
    float tmp2 = tmp * tmp;
    return r0 + (1.0f - r0) * tmp2 * tmp2 * tmp;
  }
  static DeferredRay material_sample_ray(const SI& si, const Sample& s, float f, const float* tp) {
    float lw = power_heuristic(s.pdf, lambert_pdf(s.wi));
    V3 el = eval_lambert(si, s);
    V3 sc = scale(v3((1.0f - f) * el.x, (1.0f - f) * el.y, (1.0f - f) * el.z), lw);
    V3 hv = normalize(add(si.wo, s.wi));
    float sw = power_heuristic(s.pdf, specular_pdf(si, hv));
    V3 es = eval_specular(si, s);
    sc = add(sc, scale(v3(f * es.x, f * es.y, f * es.z), sw));
    V3 dir = matvec(si.b1, si.b2, si.n, s.wi);
    DeferredRay r;
    r.o[0] = si.origin.x; r.o[1] = si.origin.y; r.o[2] = si.origin.z;
    r.d[0] = dir.x; r.d[1] = dir.y; r.d[2] = dir.z;
    r.tp[0] = sc.x * tp[0]; r.tp[1] = sc.y * tp[1]; r.tp[2] = sc.z * tp[2]; r.tp[3] = tp[3];
    return r;
  }
  struct ShadeOut {
    bool bounce = false, shadow = false, emit = false;
    bool passthru = false, diffuse = false;  // the branches taken (read by shade_one64)
    DeferredRay bounce_ray, shadow_ray;
    float add[4];
    uint32_t pixel = 0;
  };
  ShadeOut shade_one(uint32_t tid) const {
    ShadeOut out;
    const Hit& hit = hit_buffer[tid];
    V3 ro = v3(hit.ray.o[0], hit.ray.o[1], hit.ray.o[2]);
    V3 rd = v3(hit.ray.d[0], hit.ray.d[1], hit.ray.d[2]);
    uint32_t mask = f2u(hit.ray.tp[3]);
    uint32_t color_idx = mask & 0x0fffffffu;
    uint32_t ray_type = mask & 0xf0000000u;
    V3 ctp = v3(hit.ray.tp[0], hit.ray.tp[1], hit.ray.tp[2]);
    out.pixel = color_idx;
    Hash h;
    h.seed = (tid * 1973u + color_idx * 9277u + (uint32_t)samples * 26699u) | 1u;
    h.seed = h.hash();
    SI si = surface(hit);
    if (h.rand() > si.opacity) {
      V3 ao = add(ro, scale(rd, hit.t + 1e-7f * 40.0f));
      DeferredRay r = hit.ray;
      r.o[0] = ao.x; r.o[1] = ao.y; r.o[2] = ao.z;
      out.bounce = true; out.bounce_ray = r;
      out.passthru = true;
      return out;
    }
    if (dot(si.emission, v3(1.0f, 1.0f, 1.0f)) > 0.0f) {
      float att = fmax_(dot(si.normal, matvec(si.b1, si.b2, si.n, si.wo)), 0.0f);
      out.emit = true;
      out.add[0] = 50.0f * si.emission.x * ctp.x * att;
      out.add[1] = 50.0f * si.emission.y * ctp.y * att;
      out.add[2] = 50.0f * si.emission.z * ctp.z * att;
      out.add[3] = 1.0f;
      return out;
    }
    if (ray_type == 0x10000000u) return out;
    V3 m = sample_ggx(h, si);
    float f = mix1(schlick(fmax_(dot(si.wo, m), 0.0f), 1.5f), 1.0f, si.metallic);
    Sample bs;
    V3 bsdf;
    if (h.rand() > f) {
      bs = sample_lambert(h);
      bsdf = eval_lambert(si, bs);
      out.diffuse = true;
    } else {
      bs = Sample{reflect(neg(si.wo), m), 0.0f};
      bs.pdf = specular_pdf(si, m);
      bsdf = eval_specular(si, bs);
    }
    if (bs.wi.z > 0.0f) {
      V3 dir = matvec(si.b1, si.b2, si.n, bs.wi);
      float weight = sample_env_light ? power_heuristic(bs.pdf, env_pdf_dir(dir)) : 1.0f;
      DeferredRay r;
      r.o[0] = si.origin.x; r.o[1] = si.origin.y; r.o[2] = si.origin.z;
      r.d[0] = dir.x; r.d[1] = dir.y; r.d[2] = dir.z;
      r.tp[0] = bsdf.x * ctp.x * weight;
      r.tp[1] = bsdf.y * ctp.y * weight;
      r.tp[2] = bsdf.z * ctp.z * weight;
      r.tp[3] = hit.ray.tp[3];
      out.bounce = true; out.bounce_ray = r;
    }
    if (sample_env_light) {
      Sample es = sample_env(h, si);
      if (dot(es.wi, m) > 0.0f && es.wi.z > 0.0f) {
        out.shadow = true;
        out.shadow_ray = material_sample_ray(si, es, f, hit.ray.tp);
      }
    }
    return out;
  }
  void add_color(uint32_t idx, const float* c) {
    if ((size_t)idx >= (size_t)W * H) { overflow |= 8; return; }
    float* p = &color[4 * (size_t)idx];
    for (int i = 0; i < 4; i++) p[i] = p[i] + c[i];
  }
  void pass_shade_hit() {
    num_rays = 0; num_shadow = 0;   // ShadeHitPass.generateCommands: clearNumRays
    const uint32_t n = std::min<uint32_t>(num_hits, (uint32_t)hit_buffer.size());
    std::vector<ShadeOut> res(n);
    std::vector<Shade64> r64(track64 ? n : 0);
    parallel_for(n, nthreads, [&](size_t b, size_t e, int) {
      for (size_t j = b; j < e; j++) {
        res[j] = shade_one((uint32_t)j);
        if (track64) r64[j] = shade_one64((uint32_t)j, res[j]);
      }
    });
    const uint32_t off = shadow_offset();
    for (uint32_t j = 0; j < n; j++) {
      const ShadeOut& o = res[j];
      if (o.emit) {
        add_color(o.pixel, o.add);
        if (track64) add_color64(o.pixel, r64[j].add);
      }
      if (o.bounce) {
        uint32_t k = num_rays++;
        if (k < ray_buffer.size()) ray_buffer[k] = o.bounce_ray; else overflow |= 1;
        if (track64 && k < ray_buffer.size()) copy64(&ray64[3 * (size_t)k], r64[j].bounce);
      }
      if (o.shadow) {
        uint32_t k = num_shadow++ + off;
        if (k < ray_buffer.size()) ray_buffer[k] = o.shadow_ray; else overflow |= 1;
        if (track64 && k < ray_buffer.size()) copy64(&ray64[3 * (size_t)k], r64[j].shadow);
      }
    }
  }

  // ---------------- FP64 companion (om_render64.h) ----------------
  static void copy64(double* d, const double* s) { d[0] = s[0]; d[1] = s[1]; d[2] = s[2]; }
  void add_color64(uint32_t idx, const double* c) {
    if ((size_t)idx >= (size_t)W * H) return;
    double* p = &color64[4 * (size_t)idx];
    p[0] += c[0]; p[1] += c[1]; p[2] += c[2]; p[3] += 1.0;
  }
  void texel64(int32_t layer, double u, double v, double* c) const {
    const int32_t R = atlas_res;
    const int32_t nl = (int32_t)(layers.size() / (4 * (size_t)R * R));
    const int32_t l = layer < 0 ? 0 : (layer >= nl ? nl - 1 : layer);
    auto at = [&](int32_t i, int32_t j, double* t) {
      i = ((i % R) + R) % R;
      j = ((j % R) + R) % R;
      const uint8_t* p = &layers[4 * (((size_t)l * R + (size_t)j) * R + (size_t)i)];
      for (int k = 0; k < 4; k++) t[k] = (double)p[k] / 255.0;
    };
    if (R == 1) { at(0, 0, c); return; }
    const double x = u * R - 0.5, y = v * R - 0.5;
    const double x0 = std::floor(x), y0 = std::floor(y);
    const double fx = x - x0, fy = y - y0;
    const int32_t i0 = (int32_t)x0, j0 = (int32_t)y0;
    double t00[4], t10[4], t01[4], t11[4];
    at(i0, j0, t00);
    at(i0 + 1, j0, t10);
    at(i0, j0 + 1, t01);
    at(i0 + 1, j0 + 1, t11);
    for (int k = 0; k < 4; k++) c[k] = mixd(mixd(t00[k], t10[k], fx), mixd(t01[k], t11[k], fx), fy);
  }
  SI64 surface64(const Hit& hit) const { return surface64_at(hit.index, hit.bary, d3f(hit.ray.d)); }
  // getSurfaceInteraction in double for triangle `index`, the stored
  // (unorm16) barycentrics and ray direction rd
  SI64 surface64_at(int32_t index, uint32_t bary_word, D3 rd) const {
    SI64 si;
    const int32_t* tri = &tri4[4 * (size_t)index];
    const double u = unorm16d(bary_word, 0), v = unorm16d(bary_word, 1);
    const D3 bary = d3(1.0 - u - v, u, v);
    D3 tg[3], bt[3], nm[3];
    double uvx[3], uvy[3];
    for (int k = 0; k < 3; k++) {
      const uint32_t* a = &attrs4[4 * (size_t)tri[k]];
      tg[k] = d3(snorm8d(a[0], 0), snorm8d(a[0], 1), snorm8d(a[0], 2));
      bt[k] = d3(snorm8d(a[1], 0), snorm8d(a[1], 1), snorm8d(a[1], 2));
      nm[k] = d3(snorm8d(a[2], 0), snorm8d(a[2], 1), snorm8d(a[2], 2));
      uvx[k] = snorm16d(a[3], 0);
      uvy[k] = snorm16d(a[3], 1);
    }
    const D3 T = normalize(matvec(tg[0], tg[1], tg[2], bary));
    const D3 Bt = normalize(matvec(bt[0], bt[1], bt[2], bary));
    const D3 N = normalize(matvec(nm[0], nm[1], nm[2], bary));
    const double tu = uvx[0] * bary.x + uvx[1] * bary.y + uvx[2] * bary.z;
    const double tv = uvy[0] * bary.x + uvy[1] * bary.y + uvy[2] * bary.z;
    const int32_t* mat = &mat4[4 * (size_t)tri[3]];
    double nrm[4], dif[4], mr[4], em[4];
    texel64(mat[2], tu, tv, nrm);
    const D3 map_normal = mul(sub(d3(nrm[0], nrm[1], nrm[2]), d3(0.5, 0.5, 0.0)), d3(2.0, 2.0, 1.0));
    si.normal = normalize(matvec(T, Bt, N, map_normal));
    si.n = si.normal;
    onb64(si.normal, &si.b1, &si.b2);
    si.wo = vecmat(neg(rd), si.b1, si.b2, si.n);
    texel64(mat[0], tu, tv, dif);
    si.base = d3(dif[0], dif[1], dif[2]);
    si.opacity = dif[3];
    texel64(mat[1], tu, tv, mr);
    si.metallic = mr[2];
    si.alpha = mr[1] * mr[1];
    texel64(mat[3], tu, tv, em);
    si.emission = d3(em[0], em[1], em[2]);
    si.spec = d3(mixd(1.0, si.base.x, si.metallic), mixd(1.0, si.base.y, si.metallic), mixd(1.0, si.base.z, si.metallic));
    return si;
  }
  double pdf_texel64(int32_t x, int32_t y) const {
    if (x < 0 || y < 0 || x >= (int32_t)env_w || y >= (int32_t)env_h) return 0.0;
    return (double)env_pdf[(size_t)x + (size_t)env_w * (size_t)y];
  }
  static double acos_clamped(double y) { return std::acos(y < -1.0 ? -1.0 : (y > 1.0 ? 1.0 : y)); }
  // texel32: the FP32 direction whose texel is used (share_texels), or null
  double env_pdf_dir64(D3 dir, const V3* texel32 = nullptr) const {
    const double a = 1.0 + (double)env_theta + std::atan2(dir.z, dir.x) / TAU_D;
    const double u = a - std::trunc(a);
    const double v = acos_clamped(dir.y) / PI_D;
    int32_t cx = (int32_t)(u * (double)env_w), cy = (int32_t)(v * (double)env_h);
    if (texel32) pdf_texel_index32(*texel32, &cx, &cy);
    return pdf_texel64(cx, cy) / std::sin(v * PI_D);
  }
  Sample64 sample_env64(Hash& h, const SI64& si) const {
    const uint32_t nb = (uint32_t)(env_bins2.size() / 2);
    const int32_t idx = (int32_t)(h.hash() % nb);
    const int32_t h0 = env_bins2[2 * idx], h1 = env_bins2[2 * idx + 1];
    const int32_t ci = (int32_t)(h.hash() % (uint32_t)(h1 - h0)) + h0;
    const int32_t cx = env_coords2[2 * (size_t)ci], cy = env_coords2[2 * (size_t)ci + 1];
    const double u = -(double)env_theta + (0.5 + cx) / (double)env_w;
    const double v = (0.5 + cy) / (double)env_h;
    const double theta = u * TAU_D, phi = v * PI_D, sp = std::sin(phi);
    const D3 dir = d3(std::cos(theta) * sp, std::cos(phi), std::sin(theta) * sp);
    return Sample64{vecmat(dir, si.b1, si.b2, si.n), pdf_texel64(cx, cy) / sp};
  }
  D3 env_color64(D3 dir, const V3* texel32 = nullptr) const {
    const double u = (double)env_theta + std::atan2(dir.z, dir.x) / TAU_D;
    const double v = acos_clamped(dir.y) / PI_D;
    int32_t x = (int32_t)std::floor(u * (double)env_w), y = (int32_t)std::floor(v * (double)env_h);
    if (texel32) color_texel_index32(*texel32, &x, &y);
    x = ((x % (int32_t)env_w) + (int32_t)env_w) % (int32_t)env_w;
    y = ((y % (int32_t)env_h) + (int32_t)env_h) % (int32_t)env_h;
    const uint8_t* c = &env_rgbe[4 * ((size_t)y * env_w + (size_t)x)];
    const double p = std::ldexp(1.0, (int)c[3] - 128);
    return d3((double)c[0] / 255.0 * p, (double)c[1] / 255.0 * p, (double)c[2] / 255.0 * p);
  }
  struct Shade64 { double bounce[3] = {0, 0, 0}, shadow[3] = {0, 0, 0}, add[3] = {0, 0, 0}; };
  // shade_hit.wgsl:407-483 in FP64 along the branches the FP32 shading took
  Shade64 shade_one64(uint32_t tid, const ShadeOut& o) const {
    Shade64 r;
    const Hit& hit = hit_buffer[tid];
    const double* ctp = &hit64[3 * (size_t)tid];
    if (o.passthru) { copy64(r.bounce, ctp); return r; }
    const uint32_t mask = f2u(hit.ray.tp[3]);
    const uint32_t color_idx = mask & 0x0fffffffu;
    if (!o.emit && (mask & 0xf0000000u) == 0x10000000u) return r;
    Hash h;
    h.seed = (tid * 1973u + color_idx * 9277u + (uint32_t)samples * 26699u) | 1u;
    h.seed = h.hash();
    (void)h.rand();  // opacity
    const SI64 si = surface64(hit);
    if (o.emit) {
      const double att = fmaxd(dot(si.normal, matvec(si.b1, si.b2, si.n, si.wo)), 0.0);
      r.add[0] = 50.0 * si.emission.x * ctp[0] * att;
      r.add[1] = 50.0 * si.emission.y * ctp[1] * att;
      r.add[2] = 50.0 * si.emission.z * ctp[2] * att;
      return r;
    }
    const double g1 = (double)h.rand(), g2 = (double)h.rand();
    const D3 m = sample_ggx64(si, g1, g2);
    const double f = mixd(schlick64(fmaxd(dot(si.wo, m), 0.0), 1.5), 1.0, si.metallic);
    (void)h.rand();  // lobe choice (o.diffuse)
    Sample64 bs;
    D3 bsdf;
    if (o.diffuse) {
      const double l1 = (double)h.rand(), l2 = (double)h.rand();
      bs = sample_lambert64(l1, l2);
      bsdf = eval_lambert64(si, bs);
    } else {
      bs.wi = reflect(neg(si.wo), m);
      bs.pdf = specular_pdf64(si, m);
      bsdf = eval_specular64(si, bs);
    }
    if (o.bounce) {
      const V3 dir32 = v3(o.bounce_ray.d[0], o.bounce_ray.d[1], o.bounce_ray.d[2]);
      const double w = sample_env_light ? power_heuristic64(bs.pdf, env_pdf_dir64(matvec(si.b1, si.b2, si.n, bs.wi),
                                                                                  share_texels ? &dir32 : nullptr))
                                        : 1.0;
      r.bounce[0] = bsdf.x * ctp[0] * w;
      r.bounce[1] = bsdf.y * ctp[1] * w;
      r.bounce[2] = bsdf.z * ctp[2] * w;
    }
    if (sample_env_light) {
      const Sample64 es = sample_env64(h, si);
      if (o.shadow) {
        const D3 sc = material_sample64(si, es, f);
        r.shadow[0] = sc.x * ctp[0];
        r.shadow[1] = sc.y * ctp[1];
        r.shadow[2] = sc.z * ctp[2];
      }
    }
    return r;
  }

  // ---------------- shade_miss.wgsl ----------------
  V3 env_color(V3 dir) const {
    float u = env_theta + atan2_(dir.z, dir.x) / TAU_F;
    float v = acos_(dir.y) * INV_PI_F;
    // nearest texel, repeat addressing: floor(u*W) wrapped into [0, W)
    int32_t x = f2i(std::floor(u * (float)env_w)), y = f2i(std::floor(v * (float)env_h));
    x = ((x % (int32_t)env_w) + (int32_t)env_w) % (int32_t)env_w;
    y = ((y % (int32_t)env_h) + (int32_t)env_h) % (int32_t)env_h;
    const uint8_t* c = &env_rgbe[4 * ((size_t)y * env_w + (size_t)x)];
    float r = (float)c[0] / 255.0f, g = (float)c[1] / 255.0f, b = (float)c[2] / 255.0f, a = (float)c[3] / 255.0f;
    float p = pow_(2.0f, a * 255.0f - 128.0f);
    return v3(r * p, g * p, b * p);
  }
  void pass_shade_miss() {
    const uint32_t n = std::min<uint32_t>(num_misses, (uint32_t)miss_buffer.size());
    std::vector<V3> res(n);
    parallel_for(n, nthreads, [&](size_t b, size_t e, int) {
      for (size_t j = b; j < e; j++) {
        const DeferredRay& r = miss_buffer[j];
        res[j] = env_color(v3(r.d[0], r.d[1], r.d[2]));
      }
    });
    for (uint32_t j = 0; j < n; j++) {
      const DeferredRay& r = miss_buffer[j];
      float c[4] = {res[j].x * r.tp[0], res[j].y * r.tp[1], res[j].z * r.tp[2], 1.0f};
      add_color(f2u(r.tp[3]) & 0x0fffffffu, c);
      if (track64) {
        const V3 dir32 = v3(r.d[0], r.d[1], r.d[2]);
        const D3 e = env_color64(d3f(r.d), share_texels ? &dir32 : nullptr);
        const double* t = &miss64[3 * (size_t)j];
        const double c64[3] = {e.x * t[0], e.y * t[1], e.z * t[2]};
        add_color64(f2u(r.tp[3]) & 0x0fffffffu, c64);
      }
    }
  }

  // ---------------- accumulate.wgsl / postprocess.wgsl ----------------
  void pass_accumulate() {
    const size_t n = (size_t)W * H;
    const float s = (float)samples, s1 = (float)(samples + 1);
    for (size_t i = 0; i < n; i++) {
      float* a = &temp[4 * i];
      const float* c = &color[4 * i];
      for (int k = 0; k < 3; k++) a[k] = (fmax_(c[k], 0.0f) + a[k] * s) / s1;
      a[3] = 1.0f;
    }
    if (track64) {
      frames64++;
      const double sd = (double)samples, sd1 = (double)samples + 1.0;
      for (size_t i = 0; i < n; i++)
        for (int k = 0; k < 3; k++) {
          const size_t q = 4 * i + k;
          const double x = fmaxd(color64[q], 0.0);
          accum64[q] = (x + accum64[q] * sd) / sd1;
          const double delta = x - mean64[q];
          mean64[q] += delta / (double)frames64;
          m2_64[q] += delta * (x - mean64[q]);
        }
    }
  }
  static V3 rrt_odt_fit(V3 v) {
    V3 a = v3(v.x * (v.x + 0.0245786f) - 0.000090537f, v.y * (v.y + 0.0245786f) - 0.000090537f,
              v.z * (v.z + 0.0245786f) - 0.000090537f);
    V3 b = v3(v.x * (0.983729f * v.x + 0.4329510f) + 0.238081f, v.y * (0.983729f * v.y + 0.4329510f) + 0.238081f,
              v.z * (0.983729f * v.z + 0.4329510f) + 0.238081f);
    return v3(a.x / b.x, a.y / b.y, a.z / b.z);
  }
  V3 tonemap(V3 c) const {
    c = scale(c, exposure);
    V3 o = vecmat(c, v3(0.59719f, 0.35458f, 0.04823f), v3(0.07600f, 0.90834f, 0.01566f), v3(0.02840f, 0.13383f, 0.83777f));
    o = rrt_odt_fit(o);
    o = vecmat(o, v3(1.60475f, -0.53108f, -0.07367f), v3(-0.10208f, 1.10813f, -0.00605f), v3(-0.00327f, -0.07276f, 1.07602f));
    o = v3(clamp_(o.x, 0.0f, 1.0f), clamp_(o.y, 0.0f, 1.0f), clamp_(o.z, 0.0f, 1.0f));
    const float oms = 1.0f - saturation;
    V3 red = add(v3(0.3086f * oms, 0.3086f * oms, 0.3086f * oms), v3(saturation, 0.0f, 0.0f));
    V3 green = add(v3(0.6094f * oms, 0.6094f * oms, 0.6094f * oms), v3(0.0f, saturation, 0.0f));
    V3 blue = add(v3(0.0820f * oms, 0.0820f * oms, 0.0820f * oms), v3(0.0f, 0.0f, saturation));
    o = matvec(red, green, blue, o);
    float ch[3] = {o.x, o.y, o.z};
    for (int k = 0; k < 3; k++) {
      float cut = ch[k] <= 0.0031308f ? 1.0f : 0.0f;
      float higher = 1.055f * pow_(ch[k], 1.0f / 2.4f) - 0.055f;
      float lower = ch[k] * 12.92f;
      ch[k] = higher * (1.0f - cut) + lower * cut;
    }
    return v3(ch[0], ch[1], ch[2]);
  }
  void pass_postprocess() {
    const size_t n = (size_t)W * H;
    for (size_t i = 0; i < n; i++) {
      V3 c = tonemap(v3(temp[4 * i], temp[4 * i + 1], temp[4 * i + 2]));
      float ch[4] = {c.x, c.y, c.z, 1.0f};
      for (int k = 0; k < 4; k++) {
        display[4 * i + k] = ch[k];
        display8[4 * i + k] = (uint8_t)std::floor(clamp_(ch[k], 0.0f, 1.0f) * 255.0f + 0.5f);
      }
    }
  }

  // ---------------- frame driver (pike.js tick) ----------------
  void begin_frame() {
    // RenderState.generateCommands: clearColorBuffer + header upload {samples, theta, 0, 0, 0};
    // then tick() clears the colour buffer and, per batch, hits/misses and ray counts.
    std::fill(color.begin(), color.end(), 0.0f);
    if (track64) std::fill(color64.begin(), color64.end(), 0.0);
    num_hits = num_misses = num_rays = 0;
    num_shadow = 0;
  }
  // One batch of tick() at the camera's own invocationOffset (a band of the
  // frame: the bounded CPU sample of the benchmark).
  void tick_batch(uint32_t bounces) {
    begin_frame();
    pass_camera();
    for (uint32_t i = 0; i < bounces; i++) {
      pass_trace();
      pass_shade_hit();
      pass_trace_shadow();
      pass_shade_miss();
    }
    pass_accumulate();
    pass_postprocess();
    samples++;
  }
  // pike.js:133-154: W*H pixels in batches of B, each with its own counters,
  // camera invocationOffset j*B and bounces; one colour buffer per frame.
  void tick(uint32_t bounces) {
    begin_frame();
    const uint32_t nbatch = (uint32_t)(((uint64_t)W * H + B - 1) / B);
    const uint32_t saved = cam.invocation_offset;
    for (uint32_t j = 0; j < nbatch; j++) {
      num_hits = num_misses = num_rays = 0;
      num_shadow = 0;
      cam.invocation_offset = j * B;
      pass_camera();
      for (uint32_t i = 0; i < bounces; i++) {
        pass_trace();
        pass_shade_hit();
        pass_trace_shadow();
        pass_shade_miss();
      }
    }
    cam.invocation_offset = saved;
    pass_accumulate();
    pass_postprocess();
    samples++;
  }
};

}  // namespace om
