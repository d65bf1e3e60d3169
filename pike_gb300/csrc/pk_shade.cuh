// pk_shade.cuh -- the per-hit shading of shade_hit.wgsl, the camera ray of
// camera.wgsl and the environment lookup of shade_miss.wgsl as device
// functions, shared by the wavefront passes (pk_render.cu) and the
// differentiable path tracer (pk_diff.cu).  Every function reproduces the
// reference's operations in order under the arithmetic definition of
// pk_math.cuh.
#pragma once
#include "pk_internal.cuh"

namespace pk {

constexpr float SHADE_EPS = 1e-7f;

// =====================================================================
// camera.wgsl:75-93 main + createPrimaryRay (:58-73)
// =====================================================================
// camera.wgsl:54-76 createPrimaryRay for pixel (px, py) of a W x H image.
__device__ __forceinline__ void camera_ray(const CamState& cam, uint32_t px, uint32_t py, uint32_t W, uint32_t H,
                                           int32_t samples, V3& org, V3& dir) {
  Hash h;
  h.seed = (px * 1973u + py * 9277u + (uint32_t)samples * 26699u) | 1u;
  h.seed = h.next();
  const float fx = (float)px, fy = (float)py, rx = (float)W, ry = (float)H;
  const float k = cam.distortion;
  const float jx = h.rand();
  const float jy = h.rand();
  float ux = (2.0f * ((fx + jx) / rx) - 1.0f) * (rx / ry);
  float uy = (2.0f * ((fy + jy) / ry) - 1.0f) * -1.0f;
  const float rd = sqrtf(ux * ux + uy * uy);
  const float ru = rd * (1.0f + k * rd * rd);
  const float l = sqrtf(ux * ux + uy * uy);
  const float nx = ux / l, ny = uy / l;
  ux = ru * nx;
  uy = ru * ny;
  const V3 eo = v3(cam.pos[0], cam.pos[1], cam.pos[2]);
  const V3 ed = v3(cam.dir[0], cam.dir[1], cam.dir[2]);
  const float tf = tan_(cam.fov * 0.5f);
  const V3 bx = scale(normalize(cross(ed, v3(0.0f, 1.0f, 0.0f))), tf);
  const V3 by = scale(normalize(cross(bx, ed)), tf);
  const float theta = h.rand() * c::TAU;
  const float pw = pow_(h.rand(), cam.bokeh);
  const V3 dof = scale(scale(add(scale(bx, cos_(theta)), scale(by, sin_(theta))), cam.aperture), pw);
  const V3 screen = add(add(add(scale(bx, ux), scale(by, uy)), ed), eo);
  dir = normalize(sub(add(screen, scale(dof, cam.focal_depth)), add(eo, dof)));
  org = add(dof, eo);
}

// =====================================================================
// shade_miss.wgsl:37-43 envColor: nearest texel with repeat addressing.
// =====================================================================
__device__ __forceinline__ V3 env_color(const EnvDev& env, float theta, V3 dir) {
  const float u = theta + atan2_(dir.z, dir.x) / c::TAU;
  const float v = acos_(dir.y) * c::INV_PI;
  int x = f2i(floorf(u * (float)env.w)), y = f2i(floorf(v * (float)env.h));
  x = ((x % env.w) + env.w) % env.w;
  y = ((y % env.h) + env.h) % env.h;
  const uchar4 cc = env.rgbe[(size_t)y * env.w + x];
  const float r = unorm8(cc.x), g = unorm8(cc.y), b = unorm8(cc.z), a = unorm8(cc.w);
  const float p = pow_(2.0f, a * 255.0f - 128.0f);
  return v3(r * p, g * p, b * p);
}
// =====================================================================
// shade_hit.wgsl:153-483
// =====================================================================
struct SI {
  V3 b1, b2, n;
  V3 wo, origin, base, spec, emission;
  float metallic, opacity, alpha;
};
struct Sample {
  V3 wi;
  float pdf;
};
__device__ __forceinline__ float4 texel_at(const SceneDev& sc, int l, int i, int j) {
  const int R = sc.atlas_res;
  i = ((i % R) + R) % R;
  j = ((j % R) + R) % R;
  const uchar4 t = __ldg(sc.layers + ((size_t)l * R + (size_t)j) * R + (size_t)i);
  return make_float4(unorm8(t.x), unorm8(t.y), unorm8(t.z), unorm8(t.w));
}
// textureSampleLevel(atlas, linear + repeat sampler, uv, layer, 0) on rgba8unorm
// layers (shade_hit.wgsl:184-197): a 1x1 layer returns its texel; larger ones
// filter bilinearly around x = u*R - 0.5 with mix(a, b, t) = a(1-t) + bt.
__device__ __forceinline__ float4 texel(const SceneDev& sc, int layer, float u, float v) {
  const int l = layer < 0 ? 0 : (layer >= sc.n_layers ? sc.n_layers - 1 : layer);
  const int R = sc.atlas_res;
  if (R == 1) return texel_at(sc, l, 0, 0);
  const float x = u * (float)R - 0.5f, y = v * (float)R - 0.5f;
  const float x0 = floorf(x), y0 = floorf(y);
  const float fx = x - x0, fy = y - y0;
  const int i0 = f2i(x0), j0 = f2i(y0);
  const float4 a = texel_at(sc, l, i0, j0), b = texel_at(sc, l, i0 + 1, j0);
  const float4 c = texel_at(sc, l, i0, j0 + 1), d = texel_at(sc, l, i0 + 1, j0 + 1);
  return make_float4(mix1(mix1(a.x, b.x, fx), mix1(c.x, d.x, fx), fy), mix1(mix1(a.y, b.y, fx), mix1(c.y, d.y, fx), fy),
                     mix1(mix1(a.z, b.z, fx), mix1(c.z, d.z, fx), fy), mix1(mix1(a.w, b.w, fx), mix1(c.w, d.w, fx), fy));
}
__device__ __forceinline__ void unpack_snorm8x3(uint32_t w, V3& o) {
  o.x = snorm8((int)(int8_t)(w & 0xffu));
  o.y = snorm8((int)(int8_t)((w >> 8) & 0xffu));
  o.z = snorm8((int)(int8_t)((w >> 16) & 0xffu));
}
// branchlessONB (:166-177)
__device__ __forceinline__ void onb(V3 n, V3& b1, V3& b2) {
  const float sign = n.z > 0.0f ? 1.0f : -1.0f;
  const float a = -1.0f / (sign + n.z);
  const float b = n.x * n.y * a;
  b1 = v3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
  b2 = v3(b, sign + n.y * n.y * a, -n.y);
}
// getSurfaceInteraction (:179-200) + interpolateVertexAttribute (:363-394)
__device__ __forceinline__ SI surface(const SceneDev& sc, V3 ro, V3 rd, float t, int index, uint32_t bary_mask) {
  SI si;
  int4 tri = __ldg(sc.tri4 + index);
  if ((uint32_t)tri.x >= sc.n_verts || (uint32_t)tri.y >= sc.n_verts || (uint32_t)tri.z >= sc.n_verts) tri.x = tri.y = tri.z = 0;
  if ((uint32_t)tri.w >= sc.n_mats) tri.w = 0;
  const float u = unorm16(bary_mask & 0xffffu), v = unorm16(bary_mask >> 16);
  const V3 bary = v3(1.0f - u - v, u, v);
  const uint4 a0 = __ldg(sc.attrs + tri.x), a1 = __ldg(sc.attrs + tri.y), a2 = __ldg(sc.attrs + tri.z);
  V3 t0, t1, t2, q0, q1, q2, n0, n1, n2;
  unpack_snorm8x3(a0.x, t0); unpack_snorm8x3(a1.x, t1); unpack_snorm8x3(a2.x, t2);
  unpack_snorm8x3(a0.y, q0); unpack_snorm8x3(a1.y, q1); unpack_snorm8x3(a2.y, q2);
  unpack_snorm8x3(a0.z, n0); unpack_snorm8x3(a1.z, n1); unpack_snorm8x3(a2.z, n2);
  const V3 T = normalize(matvec(t0, t1, t2, bary));
  const V3 B = normalize(matvec(q0, q1, q2, bary));
  const V3 N = normalize(matvec(n0, n1, n2, bary));
  // uvs * bary (mat3x2 * vec3)
  const float tu = snorm16((int)(int16_t)(a0.w & 0xffffu)) * bary.x + snorm16((int)(int16_t)(a1.w & 0xffffu)) * bary.y +
                   snorm16((int)(int16_t)(a2.w & 0xffffu)) * bary.z;
  const float tv = snorm16((int)(int16_t)(a0.w >> 16)) * bary.x + snorm16((int)(int16_t)(a1.w >> 16)) * bary.y +
                   snorm16((int)(int16_t)(a2.w >> 16)) * bary.z;
  const int4 mat = __ldg(sc.mat4 + tri.w);
  const float4 nm = texel(sc, mat.z, tu, tv);
  const V3 map_normal = mul(sub(v3(nm.x, nm.y, nm.z), v3(0.5f, 0.5f, 0.0f)), v3(2.0f, 2.0f, 1.0f));
  si.n = normalize(matvec(T, B, N, map_normal));
  si.origin = add(ro, scale(rd, t - SHADE_EPS * 40.0f));
  onb(si.n, si.b1, si.b2);
  si.wo = vecmat(neg(rd), si.b1, si.b2, si.n);
  const float4 dif = texel(sc, mat.x, tu, tv);
  si.base = v3(dif.x, dif.y, dif.z);
  si.opacity = dif.w;
  const float4 mr = texel(sc, mat.y, tu, tv);
  si.metallic = mr.z;
  si.alpha = mr.y * mr.y;
  const float4 em = texel(sc, mat.w, tu, tv);
  si.emission = v3(em.x, em.y, em.z);
  si.spec = v3(mix1(1.0f, si.base.x, si.metallic), mix1(1.0f, si.base.y, si.metallic),
               mix1(1.0f, si.base.z, si.metallic));
  return si;
}
__device__ __forceinline__ float pdf_texel(const EnvDev& env, int x, int y) {
  if (x < 0 || y < 0 || x >= env.w || y >= env.h) return 0.0f;
  return __ldg(env.pdf + (size_t)x + (size_t)env.w * (size_t)y);
}
// envPdf (:202-210)
__device__ __forceinline__ float env_pdf_dir(const EnvDev& env, float theta, V3 dir) {
  const float a = 1.0f + theta + atan2_(dir.z, dir.x) / c::TAU;
  const float u = a - truncf(a);
  const float v = acos_(dir.y) * c::INV_PI;
  const int cx = f2i(u * (float)env.w), cy = f2i(v * (float)env.h);
  const float sin_phi = sin_(v * c::PI);
  return pdf_texel(env, cx, cy) / sin_phi;
}
// sampleEnv (:213-227)
__device__ __forceinline__ Sample sample_env(const EnvDev& env, float theta, Hash& h, const SI& si) {
  int2 cc;
  if (env.alias) {  // PK_ENV_ALIAS: a uniform texel, kept or replaced by its alias (same two draws)
    const uint32_t n = (uint32_t)env.w * (uint32_t)env.h;
    const uint32_t i = h.next() % n;
    const uint2 e = __ldg(env.alias + i);
    const uint32_t r = h.next();
    const uint32_t k = (e.x == 0xffffffffu || r < e.x) ? i : e.y;
    cc = make_int2((int)(k % (uint32_t)env.w), (int)(k / (uint32_t)env.w));
  } else {
    const int idx = (int)(h.next() % (uint32_t)env.nb);
    const int2 bin = __ldg(env.bins + idx);
    const int ci = (int)(h.next() % (uint32_t)(bin.y - bin.x)) + bin.x;
    cc = __ldg(env.coords + ci);
  }
  const float u = -theta + ((0.5f + (float)cc.x) / (float)env.w);
  const float v = (0.5f + (float)cc.y) / (float)env.h;
  const float th = u * c::TAU;
  const float phi = v * c::PI;
  const float sin_phi = sin_(phi);
  const V3 dir = v3(cos_(th) * sin_phi, cos_(phi), sin_(th) * sin_phi);
  Sample s;
  s.pdf = pdf_texel(env, cc.x, cc.y) / sin_phi;
  s.wi = vecmat(dir, si.b1, si.b2, si.n);
  return s;
}
__device__ __forceinline__ float lambert_pdf(V3 wi) { return fmax_(wi.z, SHADE_EPS) * c::INV_PI; }
__device__ __forceinline__ V3 eval_lambert(const SI& si, const Sample& s) {
  const float w = fmax_(SHADE_EPS, s.wi.z);
  return v3(si.base.x * c::INV_PI * w / s.pdf, si.base.y * c::INV_PI * w / s.pdf, si.base.z * c::INV_PI * w / s.pdf);
}
__device__ __forceinline__ float ggx_d(V3 m, float au, float av) {
  const float auv = au * av;
  const float tx = m.x / au;
  const float ty = m.y / av;
  const float ell = tx * tx + ty * ty + m.z * m.z;
  return 1.0f / (c::PI * auv * ell * ell);
}
__device__ __forceinline__ float ggx_g1(V3 w, V3 m, float au, float av) {
  const float ax = w.x * au;
  const float ay = w.y * av;
  const float axy2 = ax * ax + ay * ay;
  const float tan_theta = axy2 / (w.z * w.z);
  const float result = 2.0f / (1.0f + sqrtf(1.0f + tan_theta));
  return (dot(w, m) * dot(w, v3(0.0f, 0.0f, 1.0f)) <= 0.0f) ? 0.0f : result;
}
__device__ __forceinline__ float specular_pdf(const SI& si, V3 m) {
  const float a = si.alpha;
  return fmax_(SHADE_EPS, ggx_d(m, a, a) * ggx_g1(si.wo, m, a, a) / (4.0f * si.wo.z));
}
__device__ __forceinline__ V3 eval_specular(const SI& si, const Sample& s) {
  const float a = si.alpha;
  const V3 hv = normalize(add(si.wo, s.wi));
  const float D = ggx_d(hv, a, a);
  const float G = ggx_g1(s.wi, hv, a, a) * ggx_g1(si.wo, hv, a, a);
  const float k = fmax_(D * G / (4.0f * si.wo.z * s.pdf), 0.0f);
  return scale(si.spec, k);
}
__device__ __forceinline__ float power_heuristic(float p0, float p1) {
  const float p02 = p0 * p0;
  return p02 / (p02 + p1 * p1);
}
// sampleGGX (:295-316)
__device__ __forceinline__ V3 sample_ggx(Hash& h, const SI& si) {
  const float au = si.alpha, av = si.alpha;
  const V3 vh = normalize(v3(au * si.wo.x, av * si.wo.y, si.wo.z));
  const float lensq = vh.x * vh.x + vh.y * vh.y;
  const V3 t1v = lensq > 0.0f ? scale(v3(-vh.y, vh.x, 0.0f), 1.0f / sqrtf(lensq)) : v3(1.0f, 0.0f, 0.0f);
  const V3 t2v = cross(vh, t1v);
  const float r = sqrtf(h.rand());
  const float phi = c::TAU * h.rand();
  const float t1 = r * cos_(phi);
  float t2 = r * sin_(phi);
  const float s = 0.5f * (1.0f + vh.z);
  t2 = (1.0f - s) * sqrtf(1.0f - t1 * t1) + s * t2;
  const V3 nh = add(add(scale(t1v, t1), scale(t2v, t2)), scale(vh, sqrtf(fmax_(0.0f, 1.0f - t1 * t1 - t2 * t2))));
  return normalize(v3(au * nh.x, av * nh.y, fmax_(0.0f, nh.z)));
}
__device__ __forceinline__ float schlick(float cos_theta, float ior) {
  float r0 = (1.0f - ior) / (1.0f + ior);
  r0 = r0 * r0;
  const float tmp = 1.0f - cos_theta;
  const float tmp2 = tmp * tmp;
  return r0 + (1.0f - r0) * tmp2 * tmp2 * tmp;
}

}  // namespace pk
