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

// shade_miss.wgsl's texel choice on the parameter map (pk_diff.cu diff_env).
static inline int diff_env_texel(const DiffScene& S, V3 dir) {
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
