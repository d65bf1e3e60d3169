// pk_diff.cu -- form (3): the path-replay adjoint of the drop-in's estimator.
//
// No reference counterpart (the reference has no differentiation).  The
// forward pass renders, path by path, the estimator the drop-in's passes
// render: camera.wgsl's ray (the context's camera and sample index),
// trace.wgsl closest hits and trace_shadow.wgsl any hits on the drop-in's
// records, shade_hit.wgsl:407-483 at every hit (GGX VNDF sampling of a
// microfacet normal, the Fresnel lobe choice between Lambert and specular, the
// bounce ray weighted by the power heuristic against the environment pdf,
// next-event estimation of the environment with both lobes MIS-weighted) and
// shade_miss.wgsl's environment radiance for rays that leave.  Base colour,
// roughness and metallic come from per-material FP32 parameters instead of
// the atlas (normal map, opacity and emission still come from it), and the
// environment radiance from an FP32 RGB equirect map.  As in pk_batch, the
// shading random numbers are seeded with the bounce index where the wavefront
// uses the hit-queue slot (shade_hit.wgsl:421), so the images equal the
// drop-in's in distribution.
//
// Detached sampling.  Paths are sampled with the sampling roughness rho0 and
// with the environment tables of pk_diff_set_env_sampling, both held fixed,
// and every path is weighted by
//     prod_v V(m_v; alpha_v) / V(m_v; alpha0_v)  x  (the drop-in's weights at theta),
// V(m; a) = G1(wo, m; a) D(m; a) being the density of the sampled microfacet
// normal m up to factors that cancel (Heitz's VNDF; the ratio is taken as 1
// where that density does not apply, wo below the shading hemisphere).  At theta = theta0 every
// ratio is exactly 1 and the arithmetic is the drop-in's operation for
// operation; for any theta the weighted path is an importance-sampled
// estimate of the drop-in's expected image at theta, so its derivative at
// theta0 is an unbiased estimate of the image gradient: the derivative of the
// weights along the fixed path plus the score d log V / d alpha of every
// sampled normal.  The lobe choice depends on metallic only, which is not
// differentiated; the environment sampling tables, and the pdfs they give the
// MIS weights, are held fixed.  For fixed seeds and theta0 the estimator is a
// smooth function of theta (paths do not move), so its exact derivative is
// what central differences with common random numbers measure.
//
// Adjoint.  k_diff_adjoint replays every path from its seed (nothing is
// stored between the passes) and records per vertex the throughput T that
// reaches it, the factor P to the next vertex's throughput, the contribution
// factor Q of the vertex (next-event estimate, emission, or the environment
// when the ray leaves) and their derivatives; a backward sweep with
// L_v = Q_v + P_v L_{v+1} gives
//     dLoss/dtheta_v = sum_c g_c T_v,c (dQ_v,c + dP_v,c L_{v+1},c),
//     dLoss/dE_c(texel of v) = g_c T_v,c dQ_v,c/dE_c.
// Material terms go through warp-aggregated atomics into per-block FP32
// partials in shared memory, flushed with FP64 atomics; environment terms are
// warp-aggregated per texel and added in FP64.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <string>

#include "../../include/pike.h"
#include "pk_ctx.h"
#include "pk_math.cuh"
#include "pk_shade.cuh"
#include "pk_traverse.cuh"

namespace pk {

constexpr int DIFF_THREADS = 128;  // = TRACE_THREADS (traversal stack layout)
constexpr int DIFF_MAX_DEPTH = 8;
// traversal stack entries per lane in shared memory (the rest of 64 in local
// memory): a small shared stack leaves more of the SM's L1 to node records
constexpr int DIFF_SSTACK = 8;
// The forward inlines its traversal (twice: closest and shadow rays); the
// out-of-line copy the adjoint calls measured slower there (771-780 against
// 866-872 Mrays/s on the differentiation workload).
// 8 resident blocks per SM (64 registers, some spilled) for both kernels:
// forward 795 against 764 Mrays/s unconstrained, adjoint 592 against 531
// (the differentiation workload, same call; 6 blocks: 788 and 557).
#ifndef PK_DIFF_FWD_BLOCKS
#define PK_DIFF_FWD_BLOCKS 8
#endif
#ifndef PK_DIFF_ADJ_BLOCKS
#define PK_DIFF_ADJ_BLOCKS 8
#endif

struct DiffParams {
  const float* albedo;  // n_mats x 3 (base colour)
  const float* rough;   // roughness the weights are evaluated with
  const float* rough0;  // roughness the normals are sampled with
  const float* metal;
  uint32_t n_mats;
  const float* env;     // env_h x env_w x 3
  int env_w, env_h;
  int spp, depth;
  uint32_t sample_base;
};

// A unit direction's y component can round to just above 1 in magnitude,
// where acos (and with it envPdf in the drop-in) is NaN and the NaN poisons
// the pixel; the differentiable renderer clamps y to [-1, 1] in its
// environment lookups (the texel chosen is the one the drop-in reads).
__device__ __forceinline__ V3 clamp_y(V3 d) { return v3(d.x, fmin_(fmax_(d.y, -1.0f), 1.0f), d.z); }

// shade_miss.wgsl's texel choice (env_color) on the FP32 map; tex = its index.
__device__ __forceinline__ V3 diff_env(const DiffParams& P, float theta, V3 dir, int& tex) {
  dir = clamp_y(dir);
  const float u = theta + atan2_(dir.z, dir.x) / c::TAU;
  const float v = acos_(dir.y) * c::INV_PI;
  int x = f2i(floorf(u * (float)P.env_w)), y = f2i(floorf(v * (float)P.env_h));
  x = ((x % P.env_w) + P.env_w) % P.env_w;
  y = ((y % P.env_h) + P.env_h) % P.env_h;
  tex = y * P.env_w + x;
  const float* e = P.env + 3 * (size_t)tex;
  return v3(__ldg(e), __ldg(e + 1), __ldg(e + 2));
}

// d log D(m; a) / da of shade_hit.wgsl's GGX_D with au = av = a:
// D = 1 / (pi a^2 ell^2), ell = q / a^2 + mz^2, q = mx^2 + my^2.
__device__ __forceinline__ float dlog_ggx_d(V3 m, float a) {
  const float q = m.x * m.x + m.y * m.y, z = a * a * m.z * m.z;
  return 2.0f * (q - z) / (a * (q + z));
}
// d log G1(w, m; a) / da of GGX_G1: G1 = 2 / (1 + s), s = sqrt(1 + a^2 k),
// k = (wx^2 + wy^2) / wz^2; 0 where GGX_G1 is 0.
__device__ __forceinline__ float dlog_ggx_g1(V3 w, V3 m, float a) {
  if (dot(w, m) * w.z <= 0.0f) return 0.0f;
  const float k = (w.x * w.x + w.y * w.y) / (w.z * w.z);
  const float s = sqrtf(1.0f + a * a * k);
  return -a * k / (s * (1.0f + s));
}
// d/dp0 of the power heuristic p0^2 / (p0^2 + p1^2).
__device__ __forceinline__ float dph_dp0(float p0, float p1) {
  const float d = p0 * p0 + p1 * p1;
  if (!(d > 0.0f) || !isfinite(d)) return 0.0f;
  return 2.0f * (p0 / d) * (p1 * p1 / d);
}

// One shading event (shade_hit.wgsl main for one hit) with the material's
// parameters.  For the adjoint (DERIV) also the bounce factor P (bt = t4 * P),
// the shadow factor S (st = t4 * S) and the emission factor Qem (em = t4 *
// Qem), with their derivatives by the hit material's albedo (per channel, of
// the same channel) and roughness.
struct DiffShade {
  bool emitted, eb, es, pass;  // pass: the alpha pass-through (the ray goes on unchanged)
  V3 em;
  float4 bo, bd, bt, so, sd, st;
  V3 P, dPa, dPr, S, dSa, dSr, Qem;
  int mat;
};

template <bool DERIV>
__device__ __forceinline__ void shade_diff(const SceneDev& sc, const EnvDev& env, const DiffParams& P, float theta,
                                           int32_t samples, uint32_t r, float4 o4, float4 d4, float4 t4, uint4 hr,
                                           DiffShade& out) {
  const V3 zero = v3(0.0f, 0.0f, 0.0f);
  out.emitted = out.eb = out.es = out.pass = false;
  out.em = out.P = out.dPa = out.dPr = out.S = out.dSa = out.dSr = out.Qem = zero;
  const V3 ro = v3(o4.x, o4.y, o4.z), rd = v3(d4.x, d4.y, d4.z);
  const float ht = __uint_as_float(hr.x);
  const uint32_t mask = __float_as_uint(t4.w);
  const uint32_t color_idx = mask & 0x0fffffffu;
  const uint32_t ray_type = mask & 0xf0000000u;
  Hash h;
  h.seed = (r * 1973u + color_idx * 9277u + (uint32_t)samples * 26699u) | 1u;
  h.seed = h.next();
  SI si = surface(sc, ro, rd, ht, (int)hr.y, hr.z);
  int mat = __ldg(sc.tri4 + hr.y).w;
  if ((uint32_t)mat >= sc.n_mats) mat = 0;  // surface()'s clamp
  out.mat = mat;
  const float rho = __ldg(P.rough + mat), rho0 = __ldg(P.rough0 + mat), mu = __ldg(P.metal + mat);
  si.base = v3(__ldg(P.albedo + 3 * mat), __ldg(P.albedo + 3 * mat + 1), __ldg(P.albedo + 3 * mat + 2));
  si.metallic = mu;
  si.alpha = rho * rho;
  si.spec = v3(mix1(1.0f, si.base.x, mu), mix1(1.0f, si.base.y, mu), mix1(1.0f, si.base.z, mu));
  if (h.rand() > si.opacity) {  // alpha pass-through: same direction and throughput
    const V3 ao = add(ro, scale(rd, ht + SHADE_EPS * 40.0f));
    out.eb = out.pass = true;
    out.bo = make_float4(ao.x, ao.y, ao.z, 0.0f);
    out.bd = d4;
    out.bt = t4;
    out.P = v3(1.0f, 1.0f, 1.0f);
    return;
  }
  if (dot(si.emission, v3(1.0f, 1.0f, 1.0f)) > 0.0f) {
    const float att = fmax_(dot(si.n, matvec(si.b1, si.b2, si.n, si.wo)), 0.0f);
    out.em = v3(50.0f * si.emission.x * t4.x * att, 50.0f * si.emission.y * t4.y * att,
                50.0f * si.emission.z * t4.z * att);
    out.Qem = v3(50.0f * si.emission.x * att, 50.0f * si.emission.y * att, 50.0f * si.emission.z * att);
    out.emitted = true;
    return;
  }
  if (ray_type == 0x10000000u) return;
  SI s0 = si;
  s0.alpha = rho0 * rho0;
  const V3 m = sample_ggx(h, s0);
  const float f = mix1(schlick(fmax_(dot(si.wo, m), 0.0f), 1.5f), 1.0f, si.metallic);
  const float a = si.alpha;
  // V(m; a) / V(m; a0): exactly 1 when the two roughness values agree, and
  // taken as 1 where the VNDF density does not apply (G1(wo, m) = 0: the
  // view direction below the shading hemisphere)
  const bool vndf = dot(si.wo, m) * si.wo.z > 0.0f;
  float ratio = 1.0f;
  if (vndf && s0.alpha != a)
    ratio = (ggx_g1(si.wo, m, a, a) * ggx_d(m, a, a)) / (ggx_g1(si.wo, m, s0.alpha, s0.alpha) * ggx_d(m, s0.alpha, s0.alpha));
  const float dlv = DERIV && vndf ? dlog_ggx_d(m, a) + dlog_ggx_g1(si.wo, m, a) : 0.0f;
  const float dadr = 2.0f * rho;  // d alpha / d roughness
  Sample bs;
  V3 bsdf;
  bool lamb;
  if (h.rand() > f) {
    const float lr = sqrtf(h.rand());
    const float lphi = c::TAU * h.rand();
    const float x = lr * cos_(lphi);
    const float y = lr * sin_(lphi);
    const float z = sqrtf(fmax_(0.0f, 1.0f - x * x - y * y));
    bs.wi = v3(x, y, z);
    bs.pdf = lambert_pdf(bs.wi);
    bsdf = eval_lambert(si, bs);
    lamb = true;
  } else {
    bs.wi = reflect(neg(si.wo), m);
    bs.pdf = specular_pdf(si, m);
    bsdf = eval_specular(si, bs);
    lamb = false;
  }
  if (bs.wi.z > 0.0f) {
    const V3 dir = matvec(si.b1, si.b2, si.n, bs.wi);
    const float pe = env.enabled ? env_pdf_dir(env, theta, clamp_y(dir)) : 0.0f;
    const float weight = env.enabled ? power_heuristic(bs.pdf, pe) : 1.0f;
    out.eb = true;
    out.bo = make_float4(si.origin.x, si.origin.y, si.origin.z, 0.0f);
    out.bd = make_float4(dir.x, dir.y, dir.z, 0.0f);
    out.bt = make_float4(bsdf.x * t4.x * weight * ratio, bsdf.y * t4.y * weight * ratio,
                         bsdf.z * t4.z * weight * ratio, t4.w);
    if (DERIV) {
      out.P = v3(bsdf.x * weight * ratio, bsdf.y * weight * ratio, bsdf.z * weight * ratio);
      if (lamb) {  // base * INV_PI * max(eps, wi.z) / pdf; nothing else depends on theta
        const float k1 = c::INV_PI * fmax_(SHADE_EPS, bs.wi.z) / bs.pdf * weight * ratio;
        out.dPa = v3(k1, k1, k1);
        out.dPr = scale(out.P, dlv * dadr);
      } else {  // k * spec with k = max(D(h) G / (4 wo.z pdfS), 0), pdfS = specularPdf(m)
        const V3 hv = normalize(add(si.wo, bs.wi));
        const float D = ggx_d(hv, a, a), G = ggx_g1(bs.wi, hv, a, a) * ggx_g1(si.wo, hv, a, a);
        const float k = fmax_(D * G / (4.0f * si.wo.z * bs.pdf), 0.0f);
        const float praw = ggx_d(m, a, a) * ggx_g1(si.wo, m, a, a) / (4.0f * si.wo.z);
        const float dlp = praw > SHADE_EPS ? dlog_ggx_d(m, a) + dlog_ggx_g1(si.wo, m, a) : 0.0f;
        const float dk =
            k > 0.0f ? k * (dlog_ggx_d(hv, a) + dlog_ggx_g1(bs.wi, hv, a) + dlog_ggx_g1(si.wo, hv, a) - dlp) : 0.0f;
        const float dw = env.enabled ? dph_dp0(bs.pdf, pe) * bs.pdf * dlp : 0.0f;
        const float dkw = ratio * (dlv * k * weight + dk * weight + k * dw) * dadr;
        const float ka = ratio * k * si.metallic * weight;
        out.dPa = v3(ka, ka, ka);
        out.dPr = v3(si.spec.x * dkw, si.spec.y * dkw, si.spec.z * dkw);
      }
    }
  }
  if (env.enabled) {
    const Sample es_ = sample_env(env, theta, h, si);
    if (dot(es_.wi, m) > 0.0f && es_.wi.z > 0.0f) {
      // createMaterialSampleRay (shade_hit.wgsl:339-348)
      const float lw = power_heuristic(es_.pdf, lambert_pdf(es_.wi));
      const V3 el = eval_lambert(si, es_);
      V3 scv = scale(v3((1.0f - f) * el.x, (1.0f - f) * el.y, (1.0f - f) * el.z), lw);
      const V3 hv = normalize(add(si.wo, es_.wi));
      const float p1 = specular_pdf(si, hv);
      const float sw = power_heuristic(es_.pdf, p1);
      const V3 ev = eval_specular(si, es_);
      scv = add(scv, scale(v3(f * ev.x, f * ev.y, f * ev.z), sw));
      const V3 sdir = matvec(si.b1, si.b2, si.n, es_.wi);
      out.es = true;
      out.so = make_float4(si.origin.x, si.origin.y, si.origin.z, 0.0f);
      out.sd = make_float4(sdir.x, sdir.y, sdir.z, 0.0f);
      out.st = make_float4(scv.x * t4.x * ratio, scv.y * t4.y * ratio, scv.z * t4.z * ratio, t4.w);
      if (DERIV) {
        out.S = scale(scv, ratio);
        const float kl = (1.0f - f) * c::INV_PI * fmax_(SHADE_EPS, es_.wi.z) / es_.pdf * lw;
        const float D = ggx_d(hv, a, a), G1o = ggx_g1(si.wo, hv, a, a);
        const float ks = fmax_(D * ggx_g1(es_.wi, hv, a, a) * G1o / (4.0f * si.wo.z * es_.pdf), 0.0f);
        const float dlh = dlog_ggx_d(hv, a) + dlog_ggx_g1(si.wo, hv, a);
        const float dks = ks > 0.0f ? ks * (dlh + dlog_ggx_g1(es_.wi, hv, a)) : 0.0f;
        const float dp1 = D * G1o / (4.0f * si.wo.z) > SHADE_EPS ? p1 * dlh : 0.0f;
        const float dsw = -dph_dp0(p1, es_.pdf) * dp1;
        const float dsc = f * (dks * sw + ks * dsw);
        const float sa = ratio * (kl + f * ks * si.metallic * sw);
        out.dSa = v3(sa, sa, sa);
        out.dSr = v3(ratio * (dlv * scv.x + si.spec.x * dsc) * dadr, ratio * (dlv * scv.y + si.spec.y * dsc) * dadr,
                     ratio * (dlv * scv.z + si.spec.z * dsc) * dadr);
      }
    }
  }
}

// One recorded vertex of a path: the throughput T reaching it, its factor P
// to the next vertex's throughput, its contribution factor Q (contribution =
// T * Q), the derivatives of P and Q by the material's albedo (per channel)
// and roughness, dQ/dE (environment texel `tex`) and the material.  The
// backward sweep overwrites dQa with dLoss/dalbedo, dQr[0] with
// dLoss/droughness and QE with dLoss/dE.
struct DVert {
  float T[3], P[3], dPa[3], dPr[3], Q[3], dQa[3], dQr[3], QE[3];
  int tex, mat;
};

__device__ __forceinline__ void set3(float* d, V3 v) { d[0] = v.x; d[1] = v.y; d[2] = v.z; }
__device__ __forceinline__ void set3(float* d, float x, float y, float z) { d[0] = x; d[1] = y; d[2] = z; }

// trace.wgsl (any = false) or trace_shadow.wgsl (any = true) on the drop-in's records.
__device__ __forceinline__ void diff_trace(bool any, const SceneDev& sc, float4 o, float4 d, float& t, int& idx,
                                           uint32_t& bary, int (*sstack)[TRACE_THREADS], uint32_t* err) {
  uint32_t nf = 0, nt = 0;
  traverse_rt<false, TRACE_THREADS, DIFF_SSTACK>(any, sc, o.x, o.y, o.z, d.x, d.y, d.z, t, idx, bary, sstack, err, nf,
                                                nt);
}
// The adjoint calls the shading and the traversal out of line: with them
// inlined its path loop overflows the instruction cache (ncu: instruction
// fetch was its largest stall).  Measured on the differentiation workload:
// adjoint 648 against 587 Mrays/s inlined; the forward kernel is faster
// inlined (783 against 738), so it keeps them inline.
__device__ __noinline__ void diff_trace_out(bool any, const SceneDev& sc, float4 o, float4 d, float& t, int& idx,
                                            uint32_t& bary, int (*sstack)[TRACE_THREADS], uint32_t* err) {
  diff_trace(any, sc, o, d, t, idx, bary, sstack, err);
}
__device__ __noinline__ void shade_diff_out(const SceneDev& sc, const EnvDev& env, const DiffParams& P, float theta,
                                            int32_t samples, uint32_t r, float4 o4, float4 d4, float4 t4, uint4 hr,
                                            DiffShade& out) {
  shade_diff<true>(sc, env, P, theta, samples, r, o4, d4, t4, hr, out);
}

// One path of pixel (px, py) with camera.wgsl's sample index `samples`: the
// loop of k_batch (closest hit, shading, the shadow ray, the next bounce while
// fewer than depth closest-hit rays were traced).  acc += its contributions in
// the order the drop-in adds them; REC: V[0..nv) its vertices.
template <bool REC>
__device__ __forceinline__ void diff_path(const SceneDev& sc, const EnvDev& env, const CamState& cam,
                                          const DiffParams& P, float theta, uint32_t W, uint32_t H, uint32_t px,
                                          uint32_t py, int32_t samples, float acc[3], DVert* V, int& nv,
                                          int (*sstack)[TRACE_THREADS], uint32_t* err, uint32_t& nrays) {
  V3 org, dir;
  camera_ray(cam, px, py, W, H, samples, org, dir);
  float4 o4 = make_float4(org.x, org.y, org.z, 0.0f), d4 = make_float4(dir.x, dir.y, dir.z, 0.0f);
  float4 t4 = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(py * W + px));
  nv = 0;
  for (int bounce = 0; bounce < P.depth; bounce++) {
    float t;
    int idx;
    uint32_t bary;
    if (REC) diff_trace_out(false, sc, o4, d4, t, idx, bary, sstack, err);
    else diff_trace(false, sc, o4, d4, t, idx, bary, sstack, err);
    nrays++;
    if (idx < 0) {
      int tex;
      const V3 e = diff_env(P, theta, v3(d4.x, d4.y, d4.z), tex);
      acc[0] = acc[0] + e.x * t4.x;
      acc[1] = acc[1] + e.y * t4.y;
      acc[2] = acc[2] + e.z * t4.z;
      if (REC) {
        DVert& R = V[nv++];
        set3(R.T, t4.x, t4.y, t4.z);
        set3(R.Q, e);
        set3(R.QE, 1.0f, 1.0f, 1.0f);
        set3(R.P, 0.0f, 0.0f, 0.0f); set3(R.dPa, 0.0f, 0.0f, 0.0f); set3(R.dPr, 0.0f, 0.0f, 0.0f);
        set3(R.dQa, 0.0f, 0.0f, 0.0f); set3(R.dQr, 0.0f, 0.0f, 0.0f);
        R.tex = tex;
        R.mat = -1;
      }
      return;
    }
    DiffShade s;
    const uint4 hr = make_uint4(__float_as_uint(t), (uint32_t)idx, bary, 0u);
    if (REC) shade_diff_out(sc, env, P, theta, samples, (uint32_t)bounce, o4, d4, t4, hr, s);
    else shade_diff<false>(sc, env, P, theta, samples, (uint32_t)bounce, o4, d4, t4, hr, s);
    float cr = 0.0f, cg = 0.0f, cb = 0.0f;
    if (s.emitted) { cr = s.em.x; cg = s.em.y; cb = s.em.z; }
    int stex = -1;
    V3 se = v3(0.0f, 0.0f, 0.0f);
    if (s.es) {
      float ts;
      int is;
      uint32_t sb;
      if (REC) diff_trace_out(true, sc, s.so, s.sd, ts, is, sb, sstack, err);
      else diff_trace(true, sc, s.so, s.sd, ts, is, sb, sstack, err);
      nrays++;
      if (is < 0) {
        se = diff_env(P, theta, v3(s.sd.x, s.sd.y, s.sd.z), stex);
        cr += se.x * s.st.x;
        cg += se.y * s.st.y;
        cb += se.z * s.st.z;
      }
    }
    acc[0] = acc[0] + cr;
    acc[1] = acc[1] + cg;
    acc[2] = acc[2] + cb;
    const bool next = s.eb && bounce + 1 < P.depth;
    if (REC && !(s.pass && next)) {  // a pass-through that continues changes nothing: not recorded
      DVert& R = V[nv++];
      set3(R.T, t4.x, t4.y, t4.z);
      if (next) {
        set3(R.P, s.P); set3(R.dPa, s.dPa); set3(R.dPr, s.dPr);
      } else {
        set3(R.P, 0.0f, 0.0f, 0.0f); set3(R.dPa, 0.0f, 0.0f, 0.0f); set3(R.dPr, 0.0f, 0.0f, 0.0f);
      }
      if (s.emitted) {
        set3(R.Q, s.Qem);
        set3(R.dQa, 0.0f, 0.0f, 0.0f); set3(R.dQr, 0.0f, 0.0f, 0.0f); set3(R.QE, 0.0f, 0.0f, 0.0f);
        R.tex = -1;
        R.mat = -1;
      } else {
        set3(R.Q, s.S.x * se.x, s.S.y * se.y, s.S.z * se.z);
        set3(R.dQa, s.dSa.x * se.x, s.dSa.y * se.y, s.dSa.z * se.z);
        set3(R.dQr, s.dSr.x * se.x, s.dSr.y * se.y, s.dSr.z * se.z);
        set3(R.QE, s.S);
        R.tex = stex;
        R.mat = s.mat;
      }
    }
    if (!next) return;
    o4 = s.bo;
    d4 = s.bd;
    t4 = s.bt;
  }
}

__global__ void __launch_bounds__(DIFF_THREADS, PK_DIFF_FWD_BLOCKS) k_diff_forward(SceneDev sc, EnvDev env, CamState cam, DiffParams P,
                                                               float theta, uint32_t W, uint32_t H,
                                                               float4* __restrict__ image, uint32_t* err,
                                                               unsigned long long* rays) {
  __shared__ int sstack[DIFF_SSTACK][TRACE_THREADS];
  const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= W * H) return;
  const uint32_t px = pix % W, py = pix / W;
  float acc[3] = {0.0f, 0.0f, 0.0f};
  uint32_t nrays = 0;
  for (int s = 0; s < P.spp; s++) {
    int nv;
    diff_path<false>(sc, env, cam, P, theta, W, H, px, py, (int32_t)(P.sample_base + (uint32_t)s), acc, nullptr, nv,
                     sstack, err, nrays);
  }
  const float inv = 1.0f / (float)P.spp;
  image[pix] = make_float4(acc[0] * inv, acc[1] * inv, acc[2] * inv, 0.0f);
  atomicAdd(rays, (unsigned long long)nrays);
}

// Sum of v over the lanes of `mask` holding the same key; the lowest such lane
// receives it (others get 0).  Every lane of `mask` must call it.
__device__ __forceinline__ float group_sum(unsigned mask, int key, float v, bool& leader) {
  const unsigned peers = __match_any_sync(mask, key);
  float sum = 0.0f;
  for (unsigned m = peers; m; m &= m - 1u) sum += __shfl_sync(peers, v, __ffs(m) - 1);
  leader = (int)(threadIdx.x & 31u) == __ffs(peers) - 1;
  return sum;
}

__global__ void __launch_bounds__(DIFF_THREADS, PK_DIFF_ADJ_BLOCKS) k_diff_adjoint(SceneDev sc, EnvDev env, CamState cam, DiffParams P,
                                                               float theta, uint32_t W, uint32_t H,
                                                               const float4* __restrict__ dimage,
                                                               double* __restrict__ g_albedo,
                                                               double* __restrict__ g_rough,
                                                               double* __restrict__ g_env, uint32_t* err,
                                                               unsigned long long* rays) {
  __shared__ int sstack[DIFF_SSTACK][TRACE_THREADS];
  extern __shared__ float spart[];  // n_mats x 4: albedo rgb, roughness
  for (uint32_t i = threadIdx.x; i < 4 * P.n_mats; i += blockDim.x) spart[i] = 0.0f;
  __syncthreads();
  const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = pix < W * H;  // every lane stays for the warp-wide reductions
  const uint32_t px = live ? pix % W : 0u, py = live ? pix / W : 0u;
  float g[3] = {0.0f, 0.0f, 0.0f};
  if (live) {
    const float4 dv = dimage[pix];
    const float inv = 1.0f / (float)P.spp;
    g[0] = dv.x * inv; g[1] = dv.y * inv; g[2] = dv.z * inv;
  }
  DVert V[DIFF_MAX_DEPTH];
  uint32_t nrays = 0;
  for (int s = 0; s < P.spp; s++) {
    int nv = 0;
    float acc[3] = {0.0f, 0.0f, 0.0f};
    if (live)
      diff_path<true>(sc, env, cam, P, theta, W, H, px, py, (int32_t)(P.sample_base + (uint32_t)s), acc, V, nv,
                      sstack, err, nrays);
    // backward sweep
    float L[3] = {0.0f, 0.0f, 0.0f};
    for (int v = nv - 1; v >= 0; v--) {
      DVert& R = V[v];
      float dr = 0.0f;
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const float gt = g[c] * R.T[c];
        const float da = gt * (R.dQa[c] + R.dPa[c] * L[c]);
        dr += gt * (R.dQr[c] + R.dPr[c] * L[c]);
        R.QE[c] = gt * R.QE[c];
        L[c] = R.Q[c] + R.P[c] * L[c];
        R.dQa[c] = da;
      }
      R.dQr[0] = dr;
    }
    // scatter, record by record across the warp
    for (int v = 0; v < DIFF_MAX_DEPTH; v++) {
      if (!__any_sync(0xffffffffu, v < nv)) break;
      const bool on = v < nv;
      const int mkey = on ? V[v].mat : -1;
      bool lead;
      const float s0 = group_sum(0xffffffffu, mkey, mkey >= 0 ? V[v].dQa[0] : 0.0f, lead);
      const float s1 = group_sum(0xffffffffu, mkey, mkey >= 0 ? V[v].dQa[1] : 0.0f, lead);
      const float s2 = group_sum(0xffffffffu, mkey, mkey >= 0 ? V[v].dQa[2] : 0.0f, lead);
      const float s3 = group_sum(0xffffffffu, mkey, mkey >= 0 ? V[v].dQr[0] : 0.0f, lead);
      if (lead && mkey >= 0) {
        atomicAdd(&spart[4 * mkey + 0], s0);
        atomicAdd(&spart[4 * mkey + 1], s1);
        atomicAdd(&spart[4 * mkey + 2], s2);
        atomicAdd(&spart[4 * mkey + 3], s3);
      }
      const int tkey = on ? V[v].tex : -1;
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const float se = group_sum(0xffffffffu, tkey, tkey >= 0 ? V[v].QE[c] : 0.0f, lead);
        if (lead && tkey >= 0 && se != 0.0f) atomicAdd(g_env + 3 * (size_t)tkey + c, (double)se);
      }
    }
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < 4 * P.n_mats; i += blockDim.x) {
    const float v = spart[i];
    if (v != 0.0f) {
      if ((i & 3u) == 3u) atomicAdd(g_rough + (i >> 2), (double)v);
      else atomicAdd(g_albedo + 3 * (i >> 2) + (i & 3u), (double)v);
    }
  }
  if (live) atomicAdd(rays, (unsigned long long)nrays);
}

namespace {

int diff_fail(pk_ctx* c, int code, const char* msg) {
  c->err = msg;
  return code;
}

int diff_check(pk_ctx* c, const pk_diff_params* p, DiffParams& dp) {
  if (!c->bvh_ready) return diff_fail(c, PK_ERR_STATE, "pk_diff: no BVH");
  if (!c->W || !c->H) return diff_fail(c, PK_ERR_STATE, "pk_diff: call pk_configure first");
  if (!c->cam_set) return diff_fail(c, PK_ERR_STATE, "pk_diff: call pk_set_camera first");
  if (!c->diff_env_ready) return diff_fail(c, PK_ERR_STATE, "pk_diff: call pk_diff_set_env_sampling first");
  if (!p || !p->albedo3 || !p->roughness || !p->metallic || !p->env_rgb)
    return diff_fail(c, PK_ERR_ARG, "pk_diff: null argument");
  if (p->n_mats < c->n_mats || p->n_mats == 0 || p->n_mats > 4096)
    return diff_fail(c, PK_ERR_ARG, "pk_diff: n_mats must cover the scene's materials (at most 4096)");
  if (p->env_w != c->diff_env_w || p->env_h != c->diff_env_h)
    return diff_fail(c, PK_ERR_ARG, "pk_diff: env size differs from the sampling tables' (pk_diff_set_env_sampling)");
  if (!p->spp || p->spp > 65536 || p->depth < 1 || p->depth > DIFF_MAX_DEPTH)
    return diff_fail(c, PK_ERR_ARG, "pk_diff: bad spp or depth (1..8)");
  dp = DiffParams{p->albedo3, p->roughness, p->roughness_sampling ? p->roughness_sampling : p->roughness,
                  p->metallic, p->n_mats, p->env_rgb, (int)p->env_w, (int)p->env_h, (int)p->spp, (int)p->depth,
                  p->sample_base};
  return PK_OK;
}

EnvDev diff_env_dev(pk_ctx* c) {
  return EnvDev{nullptr, c->diff_bins.p, c->diff_coords.p, c->diff_pdf.p, (int)c->diff_env_w, (int)c->diff_env_h,
                (int)c->diff_env_nb, 1, nullptr};
}

// Runs the launch, waits, reads the error flag and the ray count.
template <class F>
int diff_run(pk_ctx* c, const char* what, F launch) {
  DevBuf<uint32_t> err(1);
  DevBuf<unsigned long long> rays(1);
  check(cudaMemsetAsync(err.p, 0, 4, c->stream), "memset");
  check(cudaMemsetAsync(rays.p, 0, 8, c->stream), "memset");
  launch(err.p, rays.p);
  check(cudaGetLastError(), what);
  uint32_t herr = 0;
  unsigned long long hr = 0;
  check(cudaMemcpyAsync(&herr, err.p, 4, cudaMemcpyDeviceToHost, c->stream), "D2H");
  check(cudaMemcpyAsync(&hr, rays.p, 8, cudaMemcpyDeviceToHost, c->stream), "D2H");
  check(cudaStreamSynchronize(c->stream), "sync");
  c->diff_rays = hr;
  if (herr) {
    c->err = std::string(what) + ": device error flags (traversal stack)";
    return PK_ERR_DEVICE;
  }
  return PK_OK;
}

}  // namespace
}  // namespace pk

using namespace pk;

extern "C" int pk_diff_set_env_sampling(pk_ctx* c, const float* env_rgb, uint32_t w, uint32_t h) {
  if (!c) return PK_ERR_ARG;
  try {
    check(cudaSetDevice(c->device), "cudaSetDevice");
    if (!env_rgb || !w || !h || (uint64_t)w * h > (1ull << 26))
      return diff_fail(c, PK_ERR_ARG, "pk_diff_set_env_sampling: null map or bad size");
    std::string why;
    uint32_t nb = 0;
    c->diff_env_ready = false;
    if (build_env_tables_gpu_f32(c->stream, env_rgb, w, h, c->diff_bins, nb, c->diff_coords, c->diff_pdf, why)) {
      c->err = "pk_diff_set_env_sampling: " + why;
      return PK_ERR_ARG;
    }
    c->diff_env_w = w;
    c->diff_env_h = h;
    c->diff_env_nb = nb;
    c->diff_env_ready = true;
    return PK_OK;
  } catch (CudaError& e) {
    c->err = e.what();
    return PK_ERR_CUDA;
  }
}

extern "C" int pk_diff_env_info(pk_ctx* c, uint32_t* w, uint32_t* h, uint32_t* nb) {
  if (!c || !w || !h || !nb) return PK_ERR_ARG;
  if (!c->diff_env_ready) return diff_fail(c, PK_ERR_STATE, "pk_diff_env_info: no sampling tables");
  *w = c->diff_env_w;
  *h = c->diff_env_h;
  *nb = c->diff_env_nb;
  return PK_OK;
}

extern "C" int pk_diff_env_download(pk_ctx* c, int32_t* bins2, int32_t* coords2, float* pdf) {
  if (!c || !bins2 || !coords2 || !pdf) return PK_ERR_ARG;
  if (!c->diff_env_ready) return diff_fail(c, PK_ERR_STATE, "pk_diff_env_download: no sampling tables");
  try {
    check(cudaSetDevice(c->device), "cudaSetDevice");
    const size_t n = (size_t)c->diff_env_w * c->diff_env_h;
    check(cudaMemcpyAsync(bins2, c->diff_bins.p, 8 * (size_t)c->diff_env_nb, cudaMemcpyDeviceToHost, c->stream), "D2H");
    check(cudaMemcpyAsync(coords2, c->diff_coords.p, 8 * n, cudaMemcpyDeviceToHost, c->stream), "D2H");
    check(cudaMemcpyAsync(pdf, c->diff_pdf.p, 4 * n, cudaMemcpyDeviceToHost, c->stream), "D2H");
    check(cudaStreamSynchronize(c->stream), "sync");
    return PK_OK;
  } catch (CudaError& e) {
    c->err = e.what();
    return PK_ERR_CUDA;
  }
}

extern "C" int pk_diff_render(pk_ctx* c, const pk_diff_params* p, float* image4) {
  if (!c) return PK_ERR_ARG;
  try {
    check(cudaSetDevice(c->device), "cudaSetDevice");
    DiffParams dp;
    const int rc = diff_check(c, p, dp);
    if (rc != PK_OK) return rc;
    if (!image4) return diff_fail(c, PK_ERR_ARG, "pk_diff_render: null image");
    const uint32_t n = c->W * c->H;
    return diff_run(c, "pk_diff_render", [&](uint32_t* err, unsigned long long* rays) {
      k_diff_forward<<<(n + DIFF_THREADS - 1) / DIFF_THREADS, DIFF_THREADS, 0, c->stream>>>(
          c->dropin_scene(), diff_env_dev(c), c->cam_host, dp, c->theta_next, c->W, c->H,
          reinterpret_cast<float4*>(image4), err, rays);
    });
  } catch (CudaError& e) {
    c->err = e.what();
    return PK_ERR_CUDA;
  }
}

extern "C" int pk_diff_backward(pk_ctx* c, const pk_diff_params* p, const float* d_image4, double* g_albedo3,
                                double* g_roughness, double* g_env_rgb) {
  if (!c) return PK_ERR_ARG;
  try {
    check(cudaSetDevice(c->device), "cudaSetDevice");
    DiffParams dp;
    const int rc = diff_check(c, p, dp);
    if (rc != PK_OK) return rc;
    if (!d_image4 || !g_albedo3 || !g_roughness || !g_env_rgb)
      return diff_fail(c, PK_ERR_ARG, "pk_diff_backward: null buffer");
    const uint32_t n = c->W * c->H;
    const size_t smem = 16 * (size_t)p->n_mats;
    if (smem > 48 * 1024)
      check(cudaFuncSetAttribute(k_diff_adjoint, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "attr");
    return diff_run(c, "pk_diff_backward", [&](uint32_t* err, unsigned long long* rays) {
      k_diff_adjoint<<<(n + DIFF_THREADS - 1) / DIFF_THREADS, DIFF_THREADS, smem, c->stream>>>(
          c->dropin_scene(), diff_env_dev(c), c->cam_host, dp, c->theta_next, c->W, c->H,
          reinterpret_cast<const float4*>(d_image4), g_albedo3, g_roughness, g_env_rgb, err, rays);
    });
  } catch (CudaError& e) {
    c->err = e.what();
    return PK_ERR_CUDA;
  }
}

extern "C" int pk_diff_rays(pk_ctx* c, unsigned long long* rays) {
  if (!c || !rays) return PK_ERR_ARG;
  *rays = c->diff_rays;
  return PK_OK;
}
