// om_render64.h -- FP64 evaluation of the light paths the FP32 oracle traces.
//
// TEST INFRASTRUCTURE ONLY (see om_math.h).  Not part of the product.
//
// The FP32 passes of om_render.h decide every ray, hit, random number and
// branch; with Renderer::track64 set, each ray also carries its throughput in
// FP64 and every contribution (emission, environment on a miss, the shadow
// ray's MIS estimate) is recomputed in FP64 from the same inputs: the hit's
// quantised barycentrics, the snorm vertex attributes, the atlas and RGBE
// texels, and the same random numbers (the FP32 rand() values, exact in
// double).  The FP64 result is therefore the reference algorithm evaluated in
// double precision along the identical light paths, which separates the
// arithmetic error of the FP32 pipeline from Monte Carlo noise.  Math is the
// C library's double sin/cos/atan2/acos/sqrt/ldexp.
//
// Restates in double: shade_hit.wgsl:166-200 (ONB, surface interaction),
// :202-227 (envPdf, sampleEnv), :239-361 (Lambert, GGX, VNDF sampling,
// Schlick, MIS), shade_miss.wgsl:37-43 (envColor), accumulate.wgsl:20-34.
#pragma once
#include <cmath>
#include <cstdint>

namespace om {

struct D3 { double x, y, z; };
static inline D3 d3(double x, double y, double z) { return D3{x, y, z}; }
static inline D3 d3f(const float* p) { return D3{(double)p[0], (double)p[1], (double)p[2]}; }
static inline D3 add(D3 a, D3 b) { return d3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline D3 sub(D3 a, D3 b) { return d3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline D3 mul(D3 a, D3 b) { return d3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline D3 scale(D3 a, double s) { return d3(a.x * s, a.y * s, a.z * s); }
static inline D3 neg(D3 a) { return d3(-a.x, -a.y, -a.z); }
static inline double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline D3 cross(D3 a, D3 b) { return d3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline D3 normalize(D3 a) { const double l = std::sqrt(dot(a, a)); return d3(a.x / l, a.y / l, a.z / l); }
static inline D3 matvec(D3 c0, D3 c1, D3 c2, D3 v) { return add(add(scale(c0, v.x), scale(c1, v.y)), scale(c2, v.z)); }
static inline D3 vecmat(D3 v, D3 c0, D3 c1, D3 c2) { return d3(dot(v, c0), dot(v, c1), dot(v, c2)); }
static inline double mixd(double a, double b, double t) { return a * (1.0 - t) + b * t; }
static inline D3 reflect(D3 e1, D3 e2) { return sub(e1, scale(e2, 2.0 * dot(e2, e1))); }
static inline double fmaxd(double a, double b) { return (a != a) ? b : ((b != b) ? a : (a > b ? a : b)); }

static const double PI_D = 3.14159265358979323846;
static const double TAU_D = 6.28318530717958647692;

// snorm / unorm decodes of the stored words, in double
static inline double snorm8d(uint32_t w, int k) { return fmaxd((double)(int8_t)((w >> (8 * k)) & 0xffu) / 127.0, -1.0); }
static inline double snorm16d(uint32_t w, int k) {
  return fmaxd((double)(int16_t)((w >> (16 * k)) & 0xffffu) / 32767.0, -1.0);
}
static inline double unorm16d(uint32_t w, int k) { return (double)((w >> (16 * k)) & 0xffffu) / 65535.0; }

struct SI64 {
  D3 b1, b2, n, wo, normal, base, spec, emission;
  double metallic, opacity, alpha;
};
struct Sample64 { D3 wi; double pdf; };

static inline void onb64(D3 n, D3* b1, D3* b2) {
  const double sign = n.z > 0.0 ? 1.0 : -1.0;
  const double a = -1.0 / (sign + n.z);
  const double b = n.x * n.y * a;
  *b1 = d3(1.0 + sign * n.x * n.x * a, sign * b, -sign * n.x);
  *b2 = d3(b, sign + n.y * n.y * a, -n.y);
}
static inline double lambert_pdf64(D3 wi) { return fmaxd(wi.z, 1e-7) / PI_D; }
static inline D3 eval_lambert64(const SI64& si, const Sample64& s) {
  const double w = fmaxd(1e-7, s.wi.z);
  return d3(si.base.x / PI_D * w / s.pdf, si.base.y / PI_D * w / s.pdf, si.base.z / PI_D * w / s.pdf);
}
static inline double ggx_d64(D3 m, double a) {
  const double tx = m.x / a, ty = m.y / a;
  const double ell = tx * tx + ty * ty + m.z * m.z;
  return 1.0 / (PI_D * a * a * ell * ell);
}
static inline double ggx_g1_64(D3 w, D3 m, double a) {
  const double ax = w.x * a, ay = w.y * a;
  const double tan_theta = (ax * ax + ay * ay) / (w.z * w.z);
  const double result = 2.0 / (1.0 + std::sqrt(1.0 + tan_theta));
  return (dot(w, m) * w.z <= 0.0) ? 0.0 : result;
}
static inline double specular_pdf64(const SI64& si, D3 m) {
  return fmaxd(1e-7, ggx_d64(m, si.alpha) * ggx_g1_64(si.wo, m, si.alpha) / (4.0 * si.wo.z));
}
static inline D3 eval_specular64(const SI64& si, const Sample64& s) {
  const D3 hv = normalize(add(si.wo, s.wi));
  const double D = ggx_d64(hv, si.alpha);
  const double G = ggx_g1_64(s.wi, hv, si.alpha) * ggx_g1_64(si.wo, hv, si.alpha);
  const double k = fmaxd(D * G / (4.0 * si.wo.z * s.pdf), 0.0);
  return scale(si.spec, k);
}
static inline double power_heuristic64(double p0, double p1) { const double p02 = p0 * p0; return p02 / (p02 + p1 * p1); }
static inline double schlick64(double cos_theta, double ior) {
  double r0 = (1.0 - ior) / (1.0 + ior);
  r0 = r0 * r0;
  const double t = 1.0 - cos_theta, t2 = t * t;
  return r0 + (1.0 - r0) * t2 * t2 * t;
}
// sampleGGX (VNDF) from the two random numbers r1, r2 the FP32 path drew
static inline D3 sample_ggx64(const SI64& si, double r1, double r2) {
  const double a = si.alpha;
  const D3 vh = normalize(d3(a * si.wo.x, a * si.wo.y, si.wo.z));
  const double lensq = vh.x * vh.x + vh.y * vh.y;
  const D3 t1v = lensq > 0.0 ? scale(d3(-vh.y, vh.x, 0.0), 1.0 / std::sqrt(lensq)) : d3(1.0, 0.0, 0.0);
  const D3 t2v = cross(vh, t1v);
  const double r = std::sqrt(r1), phi = TAU_D * r2;
  const double t1 = r * std::cos(phi);
  double t2 = r * std::sin(phi);
  const double s = 0.5 * (1.0 + vh.z);
  t2 = (1.0 - s) * std::sqrt(1.0 - t1 * t1) + s * t2;
  const D3 nh = add(add(scale(t1v, t1), scale(t2v, t2)), scale(vh, std::sqrt(fmaxd(0.0, 1.0 - t1 * t1 - t2 * t2))));
  return normalize(d3(a * nh.x, a * nh.y, fmaxd(0.0, nh.z)));
}
static inline Sample64 sample_lambert64(double r1, double r2) {
  const double r = std::sqrt(r1), phi = TAU_D * r2;
  const double x = r * std::cos(phi), y = r * std::sin(phi);
  const D3 d = d3(x, y, std::sqrt(fmaxd(0.0, 1.0 - x * x - y * y)));
  return Sample64{d, lambert_pdf64(d)};
}
// createMaterialSampleRay's throughput for an environment sample
static inline D3 material_sample64(const SI64& si, const Sample64& s, double f) {
  const double lw = power_heuristic64(s.pdf, lambert_pdf64(s.wi));
  const D3 el = eval_lambert64(si, s);
  D3 sc = scale(d3((1.0 - f) * el.x, (1.0 - f) * el.y, (1.0 - f) * el.z), lw);
  const D3 hv = normalize(add(si.wo, s.wi));
  const double sw = power_heuristic64(s.pdf, specular_pdf64(si, hv));
  const D3 es = eval_specular64(si, s);
  return add(sc, scale(d3(f * es.x, f * es.y, f * es.z), sw));
}

}  // namespace om
