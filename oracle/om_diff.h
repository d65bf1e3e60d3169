// om_diff.h -- FP64 oracle of the differentiable renderer and its gradient
// (pike_gb300/csrc/pk_diff.cu): the drop-in's estimator path by path with
// per-material parameters, detached sampling and the VNDF density ratio.
//
// TEST INFRASTRUCTURE ONLY (see om_math.h).  Every decision of a path is
// taken with the device's binary32 operations (camera ray, traversal of the
// reference BVH, hit point and shading frame, the VNDF normal sampled with the
// sampling roughness, the Fresnel lobe choice, Lambert and reflection
// directions, the environment sample from the sampling tables, visibility,
// texel indices), so both sides follow identical paths.  The weights -- BSDF,
// pdfs, MIS weights, density ratio, environment pdf -- and the image are
// evaluated in binary64, and their derivatives come from forward-mode dual
// numbers (value + partials by the hit material's albedo r, g, b and
// roughness), not from the device's hand-written derivative formulas; the
// path's sum of products is then differentiated by the chain rule
// (L_v = Q_v + P_v L_{v+1}).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <vector>

#include "om_render.h"

namespace om {

// value and partials by (albedo r, albedo g, albedo b, roughness) of one vertex's material
struct D4 {
  double v;
  double d[4];
};
static inline D4 dc(double v) { return D4{v, {0, 0, 0, 0}}; }
static inline D4 operator+(D4 a, D4 b) { D4 r{a.v + b.v, {}}; for (int k = 0; k < 4; k++) r.d[k] = a.d[k] + b.d[k]; return r; }
static inline D4 operator-(D4 a, D4 b) { D4 r{a.v - b.v, {}}; for (int k = 0; k < 4; k++) r.d[k] = a.d[k] - b.d[k]; return r; }
static inline D4 operator*(D4 a, D4 b) {
  D4 r{a.v * b.v, {}};
  for (int k = 0; k < 4; k++) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
static inline D4 operator/(D4 a, D4 b) {
  D4 r{a.v / b.v, {}};
  for (int k = 0; k < 4; k++) r.d[k] = (a.d[k] * b.v - a.v * b.d[k]) / (b.v * b.v);
  return r;
}
static inline D4 operator*(D4 a, double s) { D4 r{a.v * s, {}}; for (int k = 0; k < 4; k++) r.d[k] = a.d[k] * s; return r; }
static inline D4 operator*(double s, D4 a) { return a * s; }
static inline D4 operator+(D4 a, double s) { a.v += s; return a; }
static inline D4 operator+(double s, D4 a) { a.v += s; return a; }
static inline D4 operator-(double s, D4 a) { D4 r{s - a.v, {}}; for (int k = 0; k < 4; k++) r.d[k] = -a.d[k]; return r; }
static inline D4 operator/(D4 a, double s) { return a * (1.0 / s); }
static inline D4 operator/(double s, D4 b) { return dc(s) / b; }
static inline D4 dsqrt(D4 a) {
  const double s = std::sqrt(a.v);
  D4 r{s, {}};
  for (int k = 0; k < 4; k++) r.d[k] = a.d[k] / (2.0 * s);
  return r;
}
static inline D4 dmax(D4 a, double floor_) { return a.v > floor_ ? a : dc(floor_); }  // max(a, floor), by value
static inline D4 dmax0(D4 a) { return a.v > 0.0 ? a : dc(0.0); }

struct P3 { double x, y, z; };
static inline P3 p3(V3 a) { return P3{(double)a.x, (double)a.y, (double)a.z}; }
static inline double pdot(P3 a, P3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline P3 pnorm(P3 a) {
  const double l = std::sqrt(pdot(a, a));
  return P3{a.x / l, a.y / l, a.z / l};
}

static const double EPS64 = (double)1e-7f;  // shade_hit.wgsl's EPSILON as the device holds it
static const double PI64 = 3.14159265358979323846;

// shade_hit.wgsl GGX_D / GGX_G1 (au = av = a), power heuristic, in binary64.
static inline D4 ggx_d64(P3 m, D4 a) {
  const D4 tx = m.x / a, ty = m.y / a;
  const D4 ell = tx * tx + ty * ty + m.z * m.z;
  return 1.0 / (PI64 * (a * a) * ell * ell);
}
static inline D4 ggx_g1_64(P3 w, P3 m, D4 a) {
  if (pdot(w, m) * w.z <= 0.0) return dc(0.0);
  const D4 ax = w.x * a, ay = w.y * a;
  const D4 t = (ax * ax + ay * ay) / (w.z * w.z);
  return 2.0 / (1.0 + dsqrt(1.0 + t));
}
static inline D4 power_heuristic64(D4 p0, D4 p1) { return (p0 * p0) / (p0 * p0 + p1 * p1); }

struct DiffScene {
  const Renderer* r;  // scene, BVH, atlas and camera (r->cam); r->env_theta = the environment rotation
  uint32_t W, H;
  const double* albedo;  // n_mats x 3
  const double* rough;   // evaluation roughness
  const double* rough0;  // sampling roughness
  const double* metal;
  uint32_t n_mats;
  const double* env;     // env_h x env_w x 3 (evaluation radiance)
  int env_w, env_h;
  const EnvTables* tab;  // sampling tables of the FP32 sampling environment (build_env_f32)
  int spp, depth;
  uint32_t sample_base;
};

static const float DIFF_TAU_F = 6.283185307179586f;

// pk_diff.cu clamp_y: the y component of an environment lookup direction
// clamped to [-1, 1] (where it rounds beyond, acos would be NaN).
static inline V3 clamp_y(V3 d) { return v3(d.x, fmin_(fmax_(d.y, -1.0f), 1.0f), d.z); }

// shade_miss.wgsl's texel choice on the parameter map (pk_diff.cu diff_env).
static inline int diff_env_texel(const DiffScene& S, V3 dir) {
  dir = clamp_y(dir);
  const float u = S.r->env_theta + atan2_(dir.z, dir.x) / DIFF_TAU_F;
  const float v = acos_(dir.y) * INV_PI_F;
  int x = f2i(std::floor(u * (float)S.env_w)), y = f2i(std::floor(v * (float)S.env_h));
  x = ((x % S.env_w) + S.env_w) % S.env_w;
  y = ((y % S.env_h) + S.env_h) % S.env_h;
  return y * S.env_w + x;
}
static inline float diff_pdf_texel(const DiffScene& S, int32_t x, int32_t y) {
  if (x < 0 || y < 0 || x >= S.env_w || y >= S.env_h) return 0.0f;
  return S.tab->pdf[(size_t)x + (size_t)S.env_w * (size_t)y];
}
// envPdf (shade_hit.wgsl:202-210) on the sampling tables: the texel chosen in
// binary32, the division by sin(phi) in binary64.
static inline double diff_env_pdf64(const DiffScene& S, V3 dir) {
  dir = clamp_y(dir);
  const float a = 1.0f + S.r->env_theta + atan2_(dir.z, dir.x) / DIFF_TAU_F;
  const float u = a - std::trunc(a);
  const float v = acos_(dir.y) * INV_PI_F;
  const int32_t cx = f2i(u * (float)S.env_w), cy = f2i(v * (float)S.env_h);
  return (double)diff_pdf_texel(S, cx, cy) / std::sin(std::acos((double)dir.y));
}

// One recorded vertex: throughput T, factor P to the next throughput,
// contribution factor Q (duals in this vertex's parameters), dQ/dE and texel.
struct DVert64 {
  double T[3];
  D4 P[3], Q[3];
  double QE[3];
  int tex, mat;
};

// One path (pk_diff.cu diff_path): returns its vertices.
static inline void diff_path64(const DiffScene& S, uint32_t px, uint32_t py, int32_t samples,
                               std::vector<DVert64>& V, std::vector<int32_t>& stack, uint64_t& nrays) {
  const Renderer& R = *S.r;
  V.clear();
  Hash hc;
  hc.seed = (px * 1973u + py * 9277u + (uint32_t)samples * 26699u) | 1u;
  hc.seed = hc.hash();
  V3 o;
  V3 d = R.create_primary_ray_dir(hc, (float)px, (float)py, (float)S.W, (float)S.H, &o);
  double T[3] = {1.0, 1.0, 1.0};
  const uint32_t pixel = py * S.W + px;
  for (int bounce = 0; bounce < S.depth; bounce++) {
    const Renderer::TravResult t = R.intersect<false>(o, d, stack);
    nrays++;
    if (t.index < 0) {
      DVert64 e{};
      const int tex = diff_env_texel(S, d);
      for (int c = 0; c < 3; c++) {
        e.T[c] = T[c];
        e.P[c] = dc(0.0);
        e.Q[c] = dc(S.env[3 * (size_t)tex + c]);
        e.QE[c] = 1.0;
      }
      e.tex = tex;
      e.mat = -1;
      V.push_back(e);
      return;
    }
    DeferredRay ray;
    ray.o[0] = o.x; ray.o[1] = o.y; ray.o[2] = o.z;
    ray.d[0] = d.x; ray.d[1] = d.y; ray.d[2] = d.z;
    ray.tp[0] = ray.tp[1] = ray.tp[2] = 1.0f;
    ray.tp[3] = u2f(pixel);
    const Hit hit{t.t, t.index, t.bary, ray};
    Hash h;
    h.seed = ((uint32_t)bounce * 1973u + pixel * 9277u + (uint32_t)samples * 26699u) | 1u;
    h.seed = h.hash();
    Renderer::SI si = R.surface(hit);
    int mat = R.tri4[4 * (size_t)t.index + 3];
    const int nm_scene = (int)(R.mat4.size() / 4);
    if (mat < 0 || mat >= nm_scene) mat = 0;  // surface()'s clamp
    const bool next = bounce + 1 < S.depth;
    if (h.rand() > si.opacity) {  // alpha pass-through
      if (!next) return;
      o = add(o, scale(d, t.t + 1e-7f * 40.0f));
      continue;
    }
    DVert64 vx{};
    for (int c = 0; c < 3; c++) vx.T[c] = T[c];
    vx.tex = -1;
    if (dot(si.emission, v3(1.0f, 1.0f, 1.0f)) > 0.0f) {
      const float att = fmax_(dot(si.normal, matvec(si.b1, si.b2, si.n, si.wo)), 0.0f);
      const double e3[3] = {si.emission.x, si.emission.y, si.emission.z};
      for (int c = 0; c < 3; c++) {
        vx.P[c] = dc(0.0);
        vx.Q[c] = dc(50.0 * e3[c] * (double)att);
        vx.QE[c] = 0.0;
      }
      vx.mat = -1;
      V.push_back(vx);
      return;
    }
    // binary32 decisions with the sampling roughness and the metallic value
    const float mu32 = (float)S.metal[mat], rho0_32 = (float)S.rough0[mat];
    Renderer::SI s0 = si;
    s0.alpha = rho0_32 * rho0_32;
    const V3 m = Renderer::sample_ggx(h, s0);
    const float f32 = mix1(Renderer::schlick(fmax_(dot(si.wo, m), 0.0f), 1.5f), 1.0f, mu32);
    bool lamb;
    V3 wi;
    if (h.rand() > f32) {
      wi = Renderer::sample_lambert(h).wi;
      lamb = true;
    } else {
      wi = reflect(neg(si.wo), m);
      lamb = false;
    }
    const bool bounce_ok = wi.z > 0.0f;
    V3 ndir = v3(0.0f, 0.0f, 0.0f);
    if (bounce_ok) ndir = matvec(si.b1, si.b2, si.n, wi);
    // the environment sample (sampleEnv on the sampling tables)
    bool nee = false;
    V3 ws = v3(0.0f, 0.0f, 0.0f), sdir = ws;
    double pe_s = 0.0;
    {
      const EnvTables& tb = *S.tab;
      const uint32_t nb = (uint32_t)(tb.bins2.size() / 2);
      const int32_t idx = (int32_t)(h.hash() % nb);
      const int32_t h0 = tb.bins2[2 * idx], h1 = tb.bins2[2 * idx + 1];
      const int32_t ci = (int32_t)(h.hash() % (uint32_t)(h1 - h0)) + h0;
      const int32_t cx = tb.coords2[2 * (size_t)ci], cy = tb.coords2[2 * (size_t)ci + 1];
      const float u = -R.env_theta + ((0.5f + (float)cx) / (float)S.env_w);
      const float v = (0.5f + (float)cy) / (float)S.env_h;
      const float th = u * TAU_F, phi = v * PI_F, sin_phi = sin_(phi);
      const V3 dir = v3(cos_(th) * sin_phi, cos_(phi), sin_(th) * sin_phi);
      ws = vecmat(dir, si.b1, si.b2, si.n);
      if (dot(ws, m) > 0.0f && ws.z > 0.0f) {
        nee = true;
        sdir = matvec(si.b1, si.b2, si.n, ws);
        pe_s = (double)diff_pdf_texel(S, cx, cy) / std::sin(((0.5 + (double)cy) / (double)S.env_h) * PI64);
      }
    }
    bool visible = false;
    int stex = -1;
    if (nee) {
      const Renderer::TravResult ts = R.intersect<true>(si.origin, sdir, stack);
      nrays++;
      visible = ts.index < 0;
      if (visible) stex = diff_env_texel(S, sdir);
    }
    // binary64 weights with duals in (albedo rgb, roughness) of this material
    D4 base[3], spec[3];
    for (int c = 0; c < 3; c++) {
      base[c] = dc(S.albedo[3 * (size_t)mat + c]);
      base[c].d[c] = 1.0;
      spec[c] = (1.0 - S.metal[mat]) + base[c] * S.metal[mat];
    }
    D4 rho = dc(S.rough[mat]);
    rho.d[3] = 1.0;
    const D4 a = rho * rho;
    const D4 a0 = dc(S.rough0[mat] * S.rough0[mat]);
    const P3 wo = p3(si.wo), mm = p3(m);
    // the VNDF density ratio, 1 where the density does not apply (decided in binary32)
    const D4 ratio = dot(si.wo, m) * si.wo.z > 0.0f
                         ? (ggx_g1_64(wo, mm, a) * ggx_d64(mm, a)) / (ggx_g1_64(wo, mm, a0) * ggx_d64(mm, a0))
                         : dc(1.0);
    const double mu = S.metal[mat];
    const double f = [&]() {
      const double ct = std::max(pdot(wo, mm), 0.0);
      double r0 = (1.0 - 1.5) / (1.0 + 1.5);
      r0 = r0 * r0;
      const double tmp = 1.0 - ct;
      const double sch = r0 + (1.0 - r0) * tmp * tmp * tmp * tmp * tmp;
      return sch * (1.0 - mu) + 1.0 * mu;
    }();
    for (int c = 0; c < 3; c++) vx.P[c] = dc(0.0);
    if (bounce_ok && next) {
      const P3 w = p3(wi);
      const double pe = diff_env_pdf64(S, ndir);
      if (lamb) {
        const double pdf = std::max(w.z, EPS64) / PI64;
        const double wgt = (pdf * pdf) / (pdf * pdf + pe * pe);
        for (int c = 0; c < 3; c++) vx.P[c] = base[c] * (std::max(EPS64, w.z) / PI64 / pdf * wgt) * ratio;
      } else {
        const D4 pdfS = dmax(ggx_d64(mm, a) * ggx_g1_64(wo, mm, a) / (4.0 * wo.z), EPS64);
        const P3 hv = pnorm(P3{wo.x + w.x, wo.y + w.y, wo.z + w.z});
        const D4 k = dmax0(ggx_d64(hv, a) * ggx_g1_64(w, hv, a) * ggx_g1_64(wo, hv, a) / (4.0 * wo.z * pdfS));
        const D4 wgt = power_heuristic64(pdfS, dc(pe));
        for (int c = 0; c < 3; c++) vx.P[c] = spec[c] * k * wgt * ratio;
      }
    }
    if (visible) {
      const P3 w = p3(ws);
      const double lpdf = std::max(w.z, EPS64) / PI64;
      const double lw = (pe_s * pe_s) / (pe_s * pe_s + lpdf * lpdf);
      const P3 hv = pnorm(P3{wo.x + w.x, wo.y + w.y, wo.z + w.z});
      const D4 Dh = ggx_d64(hv, a), G1o = ggx_g1_64(wo, hv, a);
      const D4 ks = dmax0(Dh * ggx_g1_64(w, hv, a) * G1o / (4.0 * wo.z * pe_s));
      const D4 p1 = dmax(Dh * G1o / (4.0 * wo.z), EPS64);
      const D4 sw = power_heuristic64(dc(pe_s), p1);
      for (int c = 0; c < 3; c++) {
        const D4 Sc = ratio * ((1.0 - f) * base[c] * (std::max(EPS64, w.z) / PI64 / pe_s * lw) + f * spec[c] * ks * sw);
        const double E = S.env[3 * (size_t)stex + c];
        vx.Q[c] = Sc * E;
        vx.QE[c] = Sc.v;
      }
      vx.tex = stex;
    } else {
      for (int c = 0; c < 3; c++) { vx.Q[c] = dc(0.0); vx.QE[c] = 0.0; }
    }
    vx.mat = mat;
    V.push_back(vx);
    if (!(bounce_ok && next)) return;
    for (int c = 0; c < 3; c++) T[c] *= vx.P[c].v;
    o = si.origin;
    d = ndir;
  }
}

// The device's forward pass in binary32, operation for operation (pk_diff.cu
// shade_diff / diff_path without the derivative factors): every rounding of
// the weights, throughputs and accumulation as the GPU performs them, so its
// image equals pk_diff_render's bit for bit.  `trace` (a pixel index, or -1)
// prints that pixel's events.
static inline float diff_pdf_dir32(const DiffScene& S, V3 dir) {
  dir = clamp_y(dir);
  const float a = 1.0f + S.r->env_theta + atan2_(dir.z, dir.x) / DIFF_TAU_F;
  const float u = a - std::trunc(a);
  const float v = acos_(dir.y) * INV_PI_F;
  const int32_t cx = f2i(u * (float)S.env_w), cy = f2i(v * (float)S.env_h);
  return diff_pdf_texel(S, cx, cy) / sin_(v * PI_F);
}
static inline V3 diff_env32(const DiffScene& S, const std::vector<float>& env32, V3 dir) {
  const int tex = diff_env_texel(S, dir);
  return v3(env32[3 * (size_t)tex], env32[3 * (size_t)tex + 1], env32[3 * (size_t)tex + 2]);
}
static inline void diff_path32(const DiffScene& S, const std::vector<float>& env32, uint32_t px, uint32_t py,
                               int32_t samples, float acc[3], std::vector<int32_t>& stack, uint64_t& nrays,
                               bool trace) {
  const Renderer& R = *S.r;
  Hash hc;
  hc.seed = (px * 1973u + py * 9277u + (uint32_t)samples * 26699u) | 1u;
  hc.seed = hc.hash();
  V3 o;
  V3 d = R.create_primary_ray_dir(hc, (float)px, (float)py, (float)S.W, (float)S.H, &o);
  float t4[3] = {1.0f, 1.0f, 1.0f};
  const uint32_t pixel = py * S.W + px;
  for (int bounce = 0; bounce < S.depth; bounce++) {
    const Renderer::TravResult t = R.intersect<false>(o, d, stack);
    nrays++;
    if (t.index < 0) {
      const V3 e = diff_env32(S, env32, d);
      acc[0] = acc[0] + e.x * t4[0];
      acc[1] = acc[1] + e.y * t4[1];
      acc[2] = acc[2] + e.z * t4[2];
      if (trace) std::printf("s%d b%d miss e=(%g %g %g) t4=(%g %g %g)\n", samples, bounce, e.x, e.y, e.z, t4[0], t4[1], t4[2]);
      return;
    }
    DeferredRay ray;
    ray.o[0] = o.x; ray.o[1] = o.y; ray.o[2] = o.z;
    ray.d[0] = d.x; ray.d[1] = d.y; ray.d[2] = d.z;
    ray.tp[0] = t4[0]; ray.tp[1] = t4[1]; ray.tp[2] = t4[2];
    ray.tp[3] = u2f(pixel);
    const Hit hit{t.t, t.index, t.bary, ray};
    Hash h;
    h.seed = ((uint32_t)bounce * 1973u + pixel * 9277u + (uint32_t)samples * 26699u) | 1u;
    h.seed = h.hash();
    Renderer::SI si = R.surface(hit);
    int mat = R.tri4[4 * (size_t)t.index + 3];
    const int nm_scene = (int)(R.mat4.size() / 4);
    if (mat < 0 || mat >= nm_scene) mat = 0;
    const float rho = (float)S.rough[mat], rho0 = (float)S.rough0[mat], mu = (float)S.metal[mat];
    si.base = v3((float)S.albedo[3 * (size_t)mat], (float)S.albedo[3 * (size_t)mat + 1], (float)S.albedo[3 * (size_t)mat + 2]);
    si.metallic = mu;
    si.alpha = rho * rho;
    si.spec = v3(mix1(1.0f, si.base.x, mu), mix1(1.0f, si.base.y, mu), mix1(1.0f, si.base.z, mu));
    const bool next = bounce + 1 < S.depth;
    if (h.rand() > si.opacity) {
      if (!next) return;
      o = add(o, scale(d, t.t + 1e-7f * 40.0f));
      continue;
    }
    float cr = 0.0f, cg = 0.0f, cb = 0.0f;
    if (dot(si.emission, v3(1.0f, 1.0f, 1.0f)) > 0.0f) {
      const float att = fmax_(dot(si.normal, matvec(si.b1, si.b2, si.n, si.wo)), 0.0f);
      cr = 50.0f * si.emission.x * t4[0] * att;
      cg = 50.0f * si.emission.y * t4[1] * att;
      cb = 50.0f * si.emission.z * t4[2] * att;
      acc[0] = acc[0] + cr; acc[1] = acc[1] + cg; acc[2] = acc[2] + cb;
      return;
    }
    Renderer::SI s0 = si;
    s0.alpha = rho0 * rho0;
    const V3 m = Renderer::sample_ggx(h, s0);
    const float f = mix1(Renderer::schlick(fmax_(dot(si.wo, m), 0.0f), 1.5f), 1.0f, si.metallic);
    const float a = si.alpha;
    const bool vndf = dot(si.wo, m) * si.wo.z > 0.0f;
    float ratio = 1.0f;
    if (vndf && s0.alpha != a)
      ratio = (Renderer::ggx_g1(si.wo, m, a, a) * Renderer::ggx_d(m, a, a)) /
              (Renderer::ggx_g1(si.wo, m, s0.alpha, s0.alpha) * Renderer::ggx_d(m, s0.alpha, s0.alpha));
    Renderer::Sample bs;
    V3 bsdf;
    if (h.rand() > f) {
      bs = Renderer::sample_lambert(h);
      bsdf = Renderer::eval_lambert(si, bs);
    } else {
      bs = Renderer::Sample{reflect(neg(si.wo), m), 0.0f};
      bs.pdf = Renderer::specular_pdf(si, m);
      bsdf = Renderer::eval_specular(si, bs);
    }
    bool eb = false;
    V3 ndir = v3(0.0f, 0.0f, 0.0f);
    float bt[3] = {0.0f, 0.0f, 0.0f};
    if (bs.wi.z > 0.0f) {
      ndir = matvec(si.b1, si.b2, si.n, bs.wi);
      const float pe = diff_pdf_dir32(S, ndir);
      const float weight = Renderer::power_heuristic(bs.pdf, pe);
      eb = true;
      bt[0] = bsdf.x * t4[0] * weight * ratio;
      bt[1] = bsdf.y * t4[1] * weight * ratio;
      bt[2] = bsdf.z * t4[2] * weight * ratio;
      if (trace)
        std::printf("s%d b%d hit mat %d m=(%g %g %g) wo=(%g %g %g) f=%g wi=(%g %g %g) pdf=%g pe=%g w=%g bsdf=(%g %g %g) bt=(%g %g %g)\n",
                    samples, bounce, mat, m.x, m.y, m.z, si.wo.x, si.wo.y, si.wo.z, f, bs.wi.x, bs.wi.y, bs.wi.z, bs.pdf,
                    pe, weight, bsdf.x, bsdf.y, bsdf.z, bt[0], bt[1], bt[2]);
    }
    {
      const EnvTables& tb = *S.tab;
      const uint32_t nb = (uint32_t)(tb.bins2.size() / 2);
      const int32_t idx = (int32_t)(h.hash() % nb);
      const int32_t h0 = tb.bins2[2 * idx], h1 = tb.bins2[2 * idx + 1];
      const int32_t ci = (int32_t)(h.hash() % (uint32_t)(h1 - h0)) + h0;
      const int32_t cx = tb.coords2[2 * (size_t)ci], cy = tb.coords2[2 * (size_t)ci + 1];
      const float u = -R.env_theta + ((0.5f + (float)cx) / (float)S.env_w);
      const float v = (0.5f + (float)cy) / (float)S.env_h;
      const float th = u * TAU_F, phi = v * PI_F, sin_phi = sin_(phi);
      const V3 dir = v3(cos_(th) * sin_phi, cos_(phi), sin_(th) * sin_phi);
      const Renderer::Sample es{vecmat(dir, si.b1, si.b2, si.n), diff_pdf_texel(S, cx, cy) / sin_phi};
      if (dot(es.wi, m) > 0.0f && es.wi.z > 0.0f) {
        const DeferredRay sr = Renderer::material_sample_ray(si, es, f, t4);
        const float st[3] = {sr.tp[0] * ratio, sr.tp[1] * ratio, sr.tp[2] * ratio};
        const V3 sdir = v3(sr.d[0], sr.d[1], sr.d[2]);
        const Renderer::TravResult ts = R.intersect<true>(si.origin, sdir, stack);
        nrays++;
        if (ts.index < 0) {
          const V3 e = diff_env32(S, env32, sdir);
          cr += e.x * st[0];
          cg += e.y * st[1];
          cb += e.z * st[2];
        }
        if (trace)
          std::printf("s%d b%d nee wi=(%g %g %g) pdf=%g st=(%g %g %g) vis=%d\n", samples, bounce, es.wi.x, es.wi.y,
                      es.wi.z, es.pdf, st[0], st[1], st[2], ts.index < 0 ? 1 : 0);
      }
    }
    acc[0] = acc[0] + cr;
    acc[1] = acc[1] + cg;
    acc[2] = acc[2] + cb;
    if (!(eb && next)) return;
    o = si.origin;
    d = ndir;
    t4[0] = bt[0]; t4[1] = bt[1]; t4[2] = bt[2];
  }
}
// Rows [y0, y1) of the binary32 image (W x (y1-y0) x 4, alpha 0).
static inline uint64_t diff_render32(const DiffScene& S, uint32_t y0, uint32_t y1, float* image4, int nthreads,
                                     int64_t trace_pixel) {
  std::vector<float> env32(3 * (size_t)S.env_w * S.env_h);
  for (size_t i = 0; i < env32.size(); i++) env32[i] = (float)S.env[i];
  std::vector<uint64_t> rays(std::max(nthreads, 1), 0);
  parallel_for((size_t)S.W * (y1 - y0), nthreads, [&](size_t b, size_t e, int tid) {
    std::vector<int32_t> stack;
    for (size_t k = b; k < e; k++) {
      const uint32_t px = (uint32_t)(k % S.W), py = y0 + (uint32_t)(k / S.W);
      float acc[3] = {0.0f, 0.0f, 0.0f};
      const bool tr = (int64_t)(py * S.W + px) == trace_pixel;
      for (int s = 0; s < S.spp; s++)
        diff_path32(S, env32, px, py, (int32_t)(S.sample_base + (uint32_t)s), acc, stack, rays[tid], tr);
      const float inv = 1.0f / (float)S.spp;
      image4[4 * k] = acc[0] * inv;
      image4[4 * k + 1] = acc[1] * inv;
      image4[4 * k + 2] = acc[2] * inv;
      image4[4 * k + 3] = 0.0f;
    }
  });
  uint64_t n = 0;
  for (uint64_t r : rays) n += r;
  return n;
}

// image3 (W x H x 3): the mean over spp of each path's contributions.
static inline uint64_t diff_render(const DiffScene& S, double* image3, int nthreads) {
  std::vector<uint64_t> rays(std::max(nthreads, 1), 0);
  parallel_for((size_t)S.W * S.H, nthreads, [&](size_t b, size_t e, int tid) {
    std::vector<int32_t> stack;
    std::vector<DVert64> V;
    for (size_t pix = b; pix < e; pix++) {
      const uint32_t px = (uint32_t)(pix % S.W), py = (uint32_t)(pix / S.W);
      double acc[3] = {0, 0, 0};
      for (int s = 0; s < S.spp; s++) {
        diff_path64(S, px, py, (int32_t)(S.sample_base + (uint32_t)s), V, stack, rays[tid]);
        for (const DVert64& v : V)
          for (int c = 0; c < 3; c++) acc[c] += v.T[c] * v.Q[c].v;
      }
      for (int c = 0; c < 3; c++) image3[3 * pix + c] = acc[c] / S.spp;
    }
  });
  uint64_t n = 0;
  for (uint64_t r : rays) n += r;
  return n;
}

// Gradient of sum(dimage3 * image3), added to the outputs.
static inline void diff_gradient(const DiffScene& S, const double* dimage3, double* g_albedo, double* g_rough,
                                 double* g_env, int nthreads) {
  const int T = std::max(nthreads, 1);
  std::vector<std::vector<double>> ga(T, std::vector<double>(3 * (size_t)S.n_mats, 0.0));
  std::vector<std::vector<double>> gr(T, std::vector<double>(S.n_mats, 0.0));
  std::vector<std::vector<double>> ge(T, std::vector<double>(3 * (size_t)S.env_w * S.env_h, 0.0));
  std::vector<uint64_t> rays(T, 0);
  parallel_for((size_t)S.W * S.H, T, [&](size_t b, size_t e, int tid) {
    std::vector<int32_t> stack;
    std::vector<DVert64> V;
    for (size_t pix = b; pix < e; pix++) {
      const uint32_t px = (uint32_t)(pix % S.W), py = (uint32_t)(pix / S.W);
      const double g[3] = {dimage3[3 * pix] / S.spp, dimage3[3 * pix + 1] / S.spp, dimage3[3 * pix + 2] / S.spp};
      for (int s = 0; s < S.spp; s++) {
        diff_path64(S, px, py, (int32_t)(S.sample_base + (uint32_t)s), V, stack, rays[tid]);
        double L[3] = {0, 0, 0};
        for (int v = (int)V.size() - 1; v >= 0; v--) {
          const DVert64& x = V[v];
          for (int c = 0; c < 3; c++) {
            const double gt = g[c] * x.T[c];
            if (x.mat >= 0)
              for (int k = 0; k < 4; k++) {
                const double dk = gt * (x.Q[c].d[k] + x.P[c].d[k] * L[c]);
                if (k < 3) ga[tid][3 * (size_t)x.mat + k] += dk;
                else gr[tid][x.mat] += dk;
              }
            if (x.tex >= 0) ge[tid][3 * (size_t)x.tex + c] += gt * x.QE[c];
            L[c] = x.Q[c].v + x.P[c].v * L[c];
          }
        }
      }
    }
  });
  for (int t = 0; t < T; t++) {
    for (size_t k = 0; k < ga[t].size(); k++) g_albedo[k] += ga[t][k];
    for (size_t k = 0; k < gr[t].size(); k++) g_rough[k] += gr[t][k];
    for (size_t k = 0; k < ge[t].size(); k++) g_env[k] += ge[t][k];
  }
}

}  // namespace om
