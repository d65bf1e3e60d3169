// om_render_f64.h -- the reference path rendered in binary64 end to end.
//
// TEST INFRASTRUCTURE ONLY (see om_math.h).  Not part of the product.
//
// Unlike om_render64.h (which re-evaluates in FP64 the light paths the FP32
// passes decided), this renderer makes every decision itself in double: the
// camera rays (camera.wgsl:58-93), the BVH traversal and Moller-Trumbore test
// (trace.wgsl:83-213, trace_shadow.wgsl:146-207: same node words, same
// EPSILON constants), its own hit/miss queues in serial invocation order (so
// a shading seed's slot is this renderer's own queue slot), every branch of
// shade_hit.wgsl:407-483 (opacity, lobe choice, the two `wi.z > 0` tests),
// shade_miss.wgsl and the running mean of accumulate.wgsl.  Random numbers
// come from the same counter-based hash streams (camera.wgsl:46-56) as
// hash / 2^32 in double.  What stays as the reference stores it: the scene's
// f32 vertex positions, the snorm16 node boxes, the snorm8 / snorm16 vertex
// attributes, the rgba8 atlas, the RGBE environment and its f32 pdf table,
// and the unorm16 barycentrics of the Hit record (pack2x16unorm), all read
// exactly into double.  Math is the C library's double sin, cos, tan, atan2,
// acos, pow, sqrt.
//
// Its converged image is therefore the reference estimator computed in
// binary64: independent of the FP32 arithmetic (paths diverge where an FP32
// decision flips), and the per-frame colours give each pixel's Monte Carlo
// standard deviation for the 3-sigma band test of the FP32 image.
#pragma once
#include <cmath>
#include <cstdint>
#include <vector>

#include "om_render.h"

namespace om {

struct Render64 {
  const Renderer& s;  // scene, environment, camera, sizes (read only)
  uint32_t W, H, B;
  int nthreads;
  int32_t samples = 0;
  double env_theta = 0.0;
  struct Ray { double o[3], d[3], tp[3]; uint32_t pixel, type; };
  struct HitD { double t; int32_t index; uint32_t bary; Ray ray; };
  std::vector<Ray> rays, shadow, misses;
  std::vector<HitD> hits;
  std::vector<double> color, accum, mean, m2;
  uint64_t frames = 0;

  explicit Render64(const Renderer& r)
      : s(r), W(r.W), H(r.H), B(r.B), nthreads(r.nthreads), samples(r.samples), env_theta((double)r.env_theta) {
    color.assign(4 * (size_t)W * H, 0.0);
    accum.assign(4 * (size_t)W * H, 0.0);
    mean.assign(4 * (size_t)W * H, 0.0);
    m2.assign(4 * (size_t)W * H, 0.0);
  }

  struct HashD {
    Hash h;
    double rand() { return (double)h.hash() / 4294967296.0; }
    uint32_t hash() { return h.hash(); }
  };
  static HashD seeded(uint32_t a, uint32_t b, int32_t samples) {
    HashD r;
    r.h.seed = (a * 1973u + b * 9277u + (uint32_t)samples * 26699u) | 1u;
    r.h.seed = r.h.hash();
    return r;
  }

  // ---------------- camera.wgsl ----------------
  void camera(uint32_t offset) {
    const CameraState& cam = s.cam;
    const uint32_t Wd = cam.dims_mask >> 16, Hd = cam.dims_mask & 0xffffu;
    const uint32_t n = Renderer::round_up(B, 128);
    std::vector<Ray> out(n);
    std::vector<uint8_t> valid(n, 0);
    parallel_for(n, nthreads, [&](size_t b, size_t e, int) {
      for (size_t gid = b; gid < e; gid++) {
        const uint32_t idx = (uint32_t)gid + offset;
        const uint32_t px = idx % Wd, py = idx / Wd;
        if (px >= Wd || py >= Hd) continue;
        HashD h = seeded(px, py, samples);
        const double rx = Wd, ry = Hd, k = cam.distortion;
        const double jx = h.rand(), jy = h.rand();
        double ux = (2.0 * ((px + jx) / rx) - 1.0) * (rx / ry);
        double uy = (2.0 * ((py + jy) / ry) - 1.0) * -1.0;
        const double rd = std::sqrt(ux * ux + uy * uy);
        const double ru = rd * (1.0 + k * rd * rd);
        const double l = std::sqrt(ux * ux + uy * uy);
        const double nx = ux / l, ny = uy / l;
        ux = ru * nx;
        uy = ru * ny;
        const D3 eo = d3f(cam.pos), ed = d3f(cam.dir);
        const double tf = std::tan((double)cam.fov * 0.5);
        const D3 bx = scale(normalize(cross(ed, d3(0.0, 1.0, 0.0))), tf);
        const D3 by = scale(normalize(cross(bx, ed)), tf);
        const double theta = h.rand() * TAU_D;
        const double pw = std::pow(h.rand(), (double)cam.bokeh);
        const D3 dof = scale(scale(add(scale(bx, std::cos(theta)), scale(by, std::sin(theta))), cam.aperture), pw);
        const D3 screen = add(add(add(scale(bx, ux), scale(by, uy)), ed), eo);
        const D3 dir = normalize(sub(add(screen, scale(dof, cam.focal_depth)), add(eo, dof)));
        const D3 org = add(dof, eo);
        Ray r;
        r.o[0] = org.x; r.o[1] = org.y; r.o[2] = org.z;
        r.d[0] = dir.x; r.d[1] = dir.y; r.d[2] = dir.z;
        r.tp[0] = r.tp[1] = r.tp[2] = 1.0;
        r.pixel = idx;
        r.type = 0;
        out[gid] = r;
        valid[gid] = 1;
      }
    });
    for (uint32_t gid = 0; gid < n; gid++)
      if (valid[gid]) rays.push_back(out[gid]);
  }

  // ---------------- trace.wgsl / trace_shadow.wgsl in double ----------------
  static double snorm16(uint32_t w, int k) { return fmaxd((double)(int16_t)((w >> (16 * k)) & 0xffffu) / 32767.0, -1.0); }
  static double box_hit(const int32_t* node, D3 o, D3 inv) {
    const double xa = snorm16((uint32_t)node[2], 0), xb = snorm16((uint32_t)node[2], 1);
    const double ya = snorm16((uint32_t)node[3], 0), yb = snorm16((uint32_t)node[3], 1);
    const double za = snorm16((uint32_t)node[4], 0), zb = snorm16((uint32_t)node[4], 1);
    const double t1x = (xa - o.x) * inv.x, t2x = (xb - o.x) * inv.x;
    const double t1y = (ya - o.y) * inv.y, t2y = (yb - o.y) * inv.y;
    const double t1z = (za - o.z) * inv.z, t2z = (zb - o.z) * inv.z;
    auto mn = [](double a, double b) { return (a != a) ? b : ((b != b) ? a : (a < b ? a : b)); };
    auto mx = [](double a, double b) { return (a != a) ? b : ((b != b) ? a : (a > b ? a : b)); };
    const double tmax = mn(mn(mx(t1x, t2x), mx(t1y, t2y)), mx(t1z, t2z));
    const double tmin = mx(mx(mn(t1x, t2x), mn(t1y, t2y)), mn(t1z, t2z));
    return (tmax >= tmin && tmax > 0.0) ? tmin : 100000.0;
  }
  D3 vert(int32_t i) const {
    return d3(s.verts4[4 * (size_t)i], s.verts4[4 * (size_t)i + 1], s.verts4[4 * (size_t)i + 2]);
  }
  double tri_hit(D3 o, D3 d, const int32_t* tri, double eps, double* u_out, double* v_out) const {
    const D3 v0 = vert(tri[0]);
    const D3 e1 = sub(vert(tri[1]), v0), e2 = sub(vert(tri[2]), v0);
    const D3 p = cross(d, e2);
    const double det = dot(e1, p);
    if (std::fabs(det) < eps) return 100000.0;
    const double inv_det = 1.0 / det;
    const D3 t = sub(o, v0);
    const double u = dot(t, p) * inv_det;
    if (u < 0.0 || u > 1.0) return 100000.0;
    const D3 q = cross(t, e1);
    const double v = dot(d, q) * inv_det;
    if (v < 0.0 || u + v > 1.0) return 100000.0;
    const double dist = dot(e2, q) * inv_det;
    *u_out = u;
    *v_out = v;
    return dist > eps ? dist : 100000.0;
  }
  // pack2x16unorm component in double: floor(0.5 + 65535 * clamp(x, 0, 1))
  static uint32_t pack16(double x) {
    const double c = x < 0.0 ? 0.0 : (x > 1.0 ? 1.0 : x);
    return (uint32_t)std::floor(0.5 + 65535.0 * c);
  }
  // Returns the hit {t, index, bary}; index -1 on a miss.
  template <bool ANY>
  HitD intersect(const Ray& ray) const {
    const double eps = ANY ? 1e-7 : 1e-8;
    HitD r{100000.0, -1, 0u, ray};
    const D3 o = d3(ray.o[0], ray.o[1], ray.o[2]), d = d3(ray.d[0], ray.d[1], ray.d[2]);
    const D3 inv = d3(1.0 / d.x, 1.0 / d.y, 1.0 / d.z);
    std::vector<int32_t> stack{-1};
    int32_t idx = 0;
    while (idx > -1) {
      const int32_t* cur = &s.nodes5[5 * (size_t)idx];
      if (cur[1] > -1) {
        const int32_t size = cur[1] >> 24, base = cur[1] & 0x00ffffff;
        for (int32_t i = 0; i < size; i++) {
          double u = 0, v = 0;
          const double res = tri_hit(o, d, &s.tri4[4 * (size_t)(base + i)], eps, &u, &v);
          if (res < r.t) {
            r.t = res;
            r.index = base + i;
            r.bary = pack16(u) | (pack16(v) << 16);
          }
        }
        if (ANY && r.index != -1) return r;
      } else {
        const int32_t li = cur[0], ri = li + 1;
        const double lh = box_hit(&s.nodes5[5 * (size_t)li], o, inv);
        const double rh = box_hit(&s.nodes5[5 * (size_t)ri], o, inv);
        if (lh < r.t && rh < r.t) {
          if (lh > rh) { idx = ri; stack.push_back(li); } else { idx = li; stack.push_back(ri); }
          continue;
        }
        if (lh < r.t) { idx = li; continue; }
        if (rh < r.t) { idx = ri; continue; }
      }
      idx = stack.back();
      stack.pop_back();
    }
    return r;
  }

  // ---------------- shade_hit.wgsl in double ----------------
  double pdf_texel(int32_t x, int32_t y) const {
    if (x < 0 || y < 0 || x >= (int32_t)s.env_w || y >= (int32_t)s.env_h) return 0.0;
    return (double)s.env_pdf[(size_t)x + (size_t)s.env_w * (size_t)y];
  }
  static double acos_c(double y) { return std::acos(y < -1.0 ? -1.0 : (y > 1.0 ? 1.0 : y)); }
  double env_pdf_dir(D3 dir) const {
    const double a = 1.0 + env_theta + std::atan2(dir.z, dir.x) / TAU_D;
    const double u = a - std::trunc(a);
    const double v = acos_c(dir.y) / PI_D;
    const int32_t cx = (int32_t)(u * (double)s.env_w), cy = (int32_t)(v * (double)s.env_h);
    return pdf_texel(cx, cy) / std::sin(v * PI_D);
  }
  D3 env_color(D3 dir) const {
    const double u = env_theta + std::atan2(dir.z, dir.x) / TAU_D;
    const double v = acos_c(dir.y) / PI_D;
    int32_t x = (int32_t)std::floor(u * (double)s.env_w), y = (int32_t)std::floor(v * (double)s.env_h);
    x = ((x % (int32_t)s.env_w) + (int32_t)s.env_w) % (int32_t)s.env_w;
    y = ((y % (int32_t)s.env_h) + (int32_t)s.env_h) % (int32_t)s.env_h;
    const uint8_t* c = &s.env_rgbe[4 * ((size_t)y * s.env_w + (size_t)x)];
    const double p = std::ldexp(1.0, (int)c[3] - 128);
    return d3((double)c[0] / 255.0 * p, (double)c[1] / 255.0 * p, (double)c[2] / 255.0 * p);
  }
  SI64 surface(const HitD& hit, D3* origin) const {
    SI64 si = s.surface64_at(hit.index, hit.bary, d3(hit.ray.d[0], hit.ray.d[1], hit.ray.d[2]));
    const D3 ro = d3(hit.ray.o[0], hit.ray.o[1], hit.ray.o[2]), rd = d3(hit.ray.d[0], hit.ray.d[1], hit.ray.d[2]);
    *origin = add(ro, scale(rd, hit.t - 1e-7 * 40.0));
    return si;
  }
  struct ShadeOut {
    bool bounce = false, shadow = false, emit = false;
    Ray bounce_ray, shadow_ray;
    double add[3] = {0, 0, 0};
    uint32_t pixel = 0;
  };
  ShadeOut shade_one(uint32_t tid) const {
    ShadeOut out;
    const HitD& hit = hits[tid];
    const uint32_t color_idx = hit.ray.pixel, ray_type = hit.ray.type;
    out.pixel = color_idx;
    HashD h = seeded(tid, color_idx, samples);
    D3 origin;
    const SI64 si = surface(hit, &origin);
    if (h.rand() > si.opacity) {
      Ray r = hit.ray;
      for (int k = 0; k < 3; k++) r.o[k] = hit.ray.o[k] + hit.ray.d[k] * (hit.t + 1e-7 * 40.0);
      out.bounce = true;
      out.bounce_ray = r;
      return out;
    }
    if (si.emission.x + si.emission.y + si.emission.z > 0.0) {
      const double att = fmaxd(dot(si.normal, matvec(si.b1, si.b2, si.n, si.wo)), 0.0);
      out.emit = true;
      out.add[0] = 50.0 * si.emission.x * hit.ray.tp[0] * att;
      out.add[1] = 50.0 * si.emission.y * hit.ray.tp[1] * att;
      out.add[2] = 50.0 * si.emission.z * hit.ray.tp[2] * att;
      return out;
    }
    if (ray_type == 1u) return out;
    const double g1 = h.rand(), g2 = h.rand();
    const D3 m = sample_ggx64(si, g1, g2);
    const double f = mixd(schlick64(fmaxd(dot(si.wo, m), 0.0), 1.5), 1.0, si.metallic);
    Sample64 bs;
    D3 bsdf;
    if (h.rand() > f) {
      const double l1 = h.rand(), l2 = h.rand();
      bs = sample_lambert64(l1, l2);
      bsdf = eval_lambert64(si, bs);
    } else {
      bs.wi = reflect(neg(si.wo), m);
      bs.pdf = specular_pdf64(si, m);
      bsdf = eval_specular64(si, bs);
    }
    if (bs.wi.z > 0.0) {
      const D3 dir = matvec(si.b1, si.b2, si.n, bs.wi);
      const double w = s.sample_env_light ? power_heuristic64(bs.pdf, env_pdf_dir(dir)) : 1.0;
      Ray r;
      r.o[0] = origin.x; r.o[1] = origin.y; r.o[2] = origin.z;
      r.d[0] = dir.x; r.d[1] = dir.y; r.d[2] = dir.z;
      r.tp[0] = bsdf.x * hit.ray.tp[0] * w;
      r.tp[1] = bsdf.y * hit.ray.tp[1] * w;
      r.tp[2] = bsdf.z * hit.ray.tp[2] * w;
      r.pixel = hit.ray.pixel;
      r.type = hit.ray.type;
      out.bounce = true;
      out.bounce_ray = r;
    }
    if (s.sample_env_light) {
      const uint32_t nb = (uint32_t)(s.env_bins2.size() / 2);
      const int32_t bi = (int32_t)(h.hash() % nb);
      const int32_t h0 = s.env_bins2[2 * bi], h1 = s.env_bins2[2 * bi + 1];
      const int32_t ci = (int32_t)(h.hash() % (uint32_t)(h1 - h0)) + h0;
      const int32_t cx = s.env_coords2[2 * (size_t)ci], cy = s.env_coords2[2 * (size_t)ci + 1];
      const double u = -env_theta + (0.5 + cx) / (double)s.env_w;
      const double v = (0.5 + cy) / (double)s.env_h;
      const double theta = u * TAU_D, phi = v * PI_D, sp = std::sin(phi);
      const D3 dir = d3(std::cos(theta) * sp, std::cos(phi), std::sin(theta) * sp);
      const Sample64 es{vecmat(dir, si.b1, si.b2, si.n), pdf_texel(cx, cy) / sp};
      if (dot(es.wi, m) > 0.0 && es.wi.z > 0.0) {
        const D3 sc = material_sample64(si, es, f);
        const D3 wd = matvec(si.b1, si.b2, si.n, es.wi);
        Ray r;
        r.o[0] = origin.x; r.o[1] = origin.y; r.o[2] = origin.z;
        r.d[0] = wd.x; r.d[1] = wd.y; r.d[2] = wd.z;
        r.tp[0] = sc.x * hit.ray.tp[0];
        r.tp[1] = sc.y * hit.ray.tp[1];
        r.tp[2] = sc.z * hit.ray.tp[2];
        r.pixel = hit.ray.pixel;
        r.type = hit.ray.type;  // createMaterialSampleRay keeps tp.w
        out.shadow = true;
        out.shadow_ray = r;
      }
    }
    return out;
  }

  void add_color(uint32_t idx, const double* c) {
    if ((size_t)idx >= (size_t)W * H) return;
    double* p = &color[4 * (size_t)idx];
    p[0] += c[0]; p[1] += c[1]; p[2] += c[2]; p[3] += 1.0;
  }

  // One bounce: trace -> shade_hit -> trace_shadow -> shade_miss, queues in
  // serial invocation order.
  void bounce() {
    misses.clear();
    hits.clear();
    std::vector<HitD> res(rays.size());
    parallel_for(rays.size(), nthreads, [&](size_t b, size_t e, int) {
      for (size_t j = b; j < e; j++) res[j] = intersect<false>(rays[j]);
    });
    for (size_t j = 0; j < rays.size(); j++) {
      if (res[j].index != -1) hits.push_back(res[j]);
      else misses.push_back(rays[j]);
    }
    std::vector<ShadeOut> so(hits.size());
    parallel_for(hits.size(), nthreads, [&](size_t b, size_t e, int) {
      for (size_t j = b; j < e; j++) so[j] = shade_one((uint32_t)j);
    });
    rays.clear();
    shadow.clear();
    for (const ShadeOut& o : so) {
      if (o.emit) add_color(o.pixel, o.add);
      if (o.bounce) rays.push_back(o.bounce_ray);
      if (o.shadow) shadow.push_back(o.shadow_ray);
    }
    std::vector<HitD> sres(shadow.size());
    parallel_for(shadow.size(), nthreads, [&](size_t b, size_t e, int) {
      for (size_t j = b; j < e; j++) sres[j] = intersect<true>(shadow[j]);
    });
    for (size_t j = 0; j < shadow.size(); j++)
      if (sres[j].index == -1) misses.push_back(shadow[j]);
    std::vector<D3> env(misses.size());
    parallel_for(misses.size(), nthreads, [&](size_t b, size_t e, int) {
      for (size_t j = b; j < e; j++) env[j] = env_color(d3(misses[j].d[0], misses[j].d[1], misses[j].d[2]));
    });
    for (size_t j = 0; j < misses.size(); j++) {
      const double c[3] = {env[j].x * misses[j].tp[0], env[j].y * misses[j].tp[1], env[j].z * misses[j].tp[2]};
      add_color(misses[j].pixel, c);
    }
  }

  // pike.js tick: the frame's batches, each camera + bounces; then the
  // running mean (accumulate.wgsl) and the per-frame moments.
  void tick(uint32_t bounces) {
    std::fill(color.begin(), color.end(), 0.0);
    const uint32_t nbatch = (uint32_t)(((uint64_t)W * H + B - 1) / B);
    for (uint32_t j = 0; j < nbatch; j++) {
      rays.clear();
      shadow.clear();
      camera(j * B);
      for (uint32_t i = 0; i < bounces; i++) bounce();
    }
    frames++;
    const double sd = (double)samples, sd1 = (double)samples + 1.0;
    for (size_t i = 0; i < (size_t)W * H; i++)
      for (int k = 0; k < 3; k++) {
        const size_t q = 4 * i + k;
        const double x = fmaxd(color[q], 0.0);
        accum[q] = (x + accum[q] * sd) / sd1;
        const double delta = x - mean[q];
        mean[q] += delta / (double)frames;
        m2[q] += delta * (x - mean[q]);
      }
    samples++;
  }
};

}  // namespace om
