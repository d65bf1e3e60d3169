// om_diff.h -- FP64 oracle of the differentiable path tracer and its gradient
// (pike_gb300/csrc/pk_diff.cu).
//
// TEST INFRASTRUCTURE ONLY (see om_math.h).  The paths are replayed with the
// same binary32 operations as the device (camera ray, traversal of the
// reference BVH, hit point, geometric normal, cosine sampling through the
// pinned sin/cos, texel lookup through the pinned atan2/acos), so both sides
// follow identical paths; the BSDF, its derivatives, the image and the
// gradient are evaluated and accumulated in binary64.
#pragma once
#include <cmath>
#include <cstdint>
#include <vector>

#include "om_render.h"

namespace om {

struct DiffCamera { float o[3], f[3], r[3], u[3]; };

struct DiffScene {
  const Renderer* r;  // scene, BVH and triangles (tri4.w = material)
  DiffCamera cam;
  uint32_t W, H;
  const double* albedo;  // n_mats x 3
  const double* rough;
  const double* metal;
  uint32_t n_mats;
  const double* env;     // env_h x env_w x 3
  int env_w, env_h;
  int spp, depth;
  uint32_t seed;
};

struct DiffVertex { V3 n, wo, wi; int mat; };

static const float DIFF_TAU = 6.283185307179586f;
static const float DIFF_PI = 3.141592653589793f;

static inline int diff_env_texel(const DiffScene& S, V3 d) {
  const float u = atan2_(d.z, d.x) / DIFF_TAU + 0.5f;
  const float v = acos_(fmin_(fmax_(d.y, -1.0f), 1.0f)) / DIFF_PI;
  int ix = f2i(u * (float)S.env_w), iy = f2i(v * (float)S.env_h);
  ix = ix < 0 ? 0 : (ix >= S.env_w ? S.env_w - 1 : ix);
  iy = iy < 0 ? 0 : (iy >= S.env_h ? S.env_h - 1 : iy);
  return iy * S.env_w + ix;
}

// Duff et al. 2017 branchless orthonormal basis (the device's `basis`).
static inline void diff_basis(V3 n, V3& b1, V3& b2) {
  const float sign = n.z >= 0.0f ? 1.0f : -1.0f;
  const float a = -1.0f / (sign + n.z);
  const float b = n.x * n.y * a;
  b1 = v3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
  b2 = v3(b, sign + n.y * n.y * a, -n.y);
}

// Replays one path; returns the escaped texel or -1 (pk_diff.cu trace_path).
static inline int diff_trace_path(const DiffScene& S, uint32_t px, uint32_t py, uint32_t s, DiffVertex* vtx, int& nv,
                                  std::vector<int32_t>& stack, uint64_t& nrays) {
  Hash h;
  h.seed = (px * 1973u + py * 9277u + (s + S.seed * 65536u) * 26699u) | 1u;
  h.seed = h.hash();
  const float jx = h.rand(), jy = h.rand();
  const float sx = 2.0f * (((float)px + jx) / (float)S.W) - 1.0f;
  const float sy = 1.0f - 2.0f * (((float)py + jy) / (float)S.H);
  V3 o = v3(S.cam.o[0], S.cam.o[1], S.cam.o[2]);
  V3 d = normalize(add(add(v3(S.cam.f[0], S.cam.f[1], S.cam.f[2]), scale(v3(S.cam.r[0], S.cam.r[1], S.cam.r[2]), sx)),
                       scale(v3(S.cam.u[0], S.cam.u[1], S.cam.u[2]), sy)));
  nv = 0;
  for (int b = 0; b < S.depth; b++) {
    const Renderer::TravResult t = S.r->intersect<false>(o, d, stack);
    nrays++;
    if (t.index < 0) return diff_env_texel(S, d);
    if (b == S.depth - 1) return -1;
    const int32_t* tri = &S.r->tri4[4 * (size_t)t.index];
    const V3 v0 = S.r->vert(tri[0]);
    V3 n = normalize(cross(sub(S.r->vert(tri[1]), v0), sub(S.r->vert(tri[2]), v0)));
    if (dot(n, d) > 0.0f) n = neg(n);
    const V3 p = add(add(o, scale(d, t.t)), scale(n, 1e-4f));
    const float u1 = h.rand(), u2 = h.rand();
    const float rr = std::sqrt(u1), phi = DIFF_TAU * u2;
    const float lz = std::sqrt(fmax_(1.0f - u1, 0.0f));
    V3 b1, b2;
    diff_basis(n, b1, b2);
    const V3 wi = add(add(scale(b1, rr * cos_(phi)), scale(b2, rr * sin_(phi))), scale(n, lz));
    int m = tri[3];
    m = (uint32_t)m < S.n_mats ? m : 0;
    vtx[nv] = DiffVertex{n, neg(d), wi, m};
    nv++;
    o = p;
    d = wi;
  }
  return -1;
}

// w = pi f and its derivatives, in binary64 (pk_diff.cu bsdf_gain).
static inline void diff_gain(const DiffScene& S, const DiffVertex& v, double w[3], double dwa[3], double dwr[3]) {
  const double nx = v.n.x, ny = v.n.y, nz = v.n.z;
  const double ox = v.wo.x, oy = v.wo.y, oz = v.wo.z, ix = v.wi.x, iy = v.wi.y, iz = v.wi.z;
  const double co = std::max(nx * ox + ny * oy + nz * oz, 1e-6), ci = std::max(nx * ix + ny * iy + nz * iz, 1e-6);
  double hx = ox + ix, hy = oy + iy, hz = oz + iz;
  const double hl = std::sqrt(hx * hx + hy * hy + hz * hz);
  hx /= hl; hy /= hl; hz /= hl;
  const double nh = std::max(nx * hx + ny * hy + nz * hz, 0.0);
  const double vh = std::min(std::max(ox * hx + oy * hy + oz * hz, 0.0), 1.0);
  const double r = S.rough[v.mat], mt = S.metal[v.mat];
  const double al = r * r, a2 = al * al, PI = 3.14159265358979323846;
  const double cx = ny * hz - nz * hy, cy = nz * hx - nx * hz, cz = nx * hy - ny * hx;
  const double Bd = (cx * cx + cy * cy + cz * cz) + nh * nh * a2;
  const double D = a2 / (PI * Bd * Bd);
  const double dD = (2.0 * al / (PI * Bd * Bd)) * (1.0 - 2.0 * a2 * nh * nh / Bd);
  const double So = std::sqrt(a2 + (1.0 - a2) * co * co), Si = std::sqrt(a2 + (1.0 - a2) * ci * ci);
  const double G1o = 2.0 * co / (co + So), G1i = 2.0 * ci / (ci + Si);
  const double dG1o = -2.0 * co * (al * (1.0 - co * co) / So) / ((co + So) * (co + So));
  const double dG1i = -2.0 * ci * (al * (1.0 - ci * ci) / Si) / ((ci + Si) * (ci + Si));
  const double G = G1o * G1i, dG = dG1o * G1i + G1o * dG1i;
  const double k5 = std::pow(1.0 - vh, 5.0);
  const double spec = 1.0 / (4.0 * co * ci);
  for (int c = 0; c < 3; c++) {
    const double a = S.albedo[3 * v.mat + c];
    const double F0 = 0.04 * (1.0 - mt) + a * mt;
    const double F = F0 + (1.0 - F0) * k5;
    const double dF = mt * (1.0 - k5);
    const double kd = (1.0 - mt) * (1.0 - F);
    w[c] = kd * a + PI * D * G * F * spec;
    dwa[c] = kd - (1.0 - mt) * dF * a + PI * D * G * dF * spec;
    dwr[c] = PI * F * spec * (dD * G + D * dG) * 2.0 * r;
  }
}

// image3 (W x H x 3), the mean over spp of each path's contribution.
static inline uint64_t diff_render(const DiffScene& S, double* image3, int nthreads) {
  std::vector<uint64_t> rays(std::max(nthreads, 1), 0);
  parallel_for((size_t)S.W * S.H, nthreads, [&](size_t b, size_t e, int tid) {
    std::vector<int32_t> stack;
    DiffVertex vtx[8];
    for (size_t pix = b; pix < e; pix++) {
      const uint32_t px = (uint32_t)(pix % S.W), py = (uint32_t)(pix / S.W);
      double acc[3] = {0, 0, 0};
      for (int s = 0; s < S.spp; s++) {
        int nv = 0;
        const int tex = diff_trace_path(S, px, py, (uint32_t)s, vtx, nv, stack, rays[tid]);
        if (tex < 0) continue;
        double beta[3] = {1, 1, 1};
        for (int i = 0; i < nv; i++) {
          double w[3], dwa[3], dwr[3];
          diff_gain(S, vtx[i], w, dwa, dwr);
          for (int c = 0; c < 3; c++) beta[c] *= w[c];
        }
        for (int c = 0; c < 3; c++) acc[c] += beta[c] * S.env[3 * (size_t)tex + c];
      }
      for (int c = 0; c < 3; c++) image3[3 * pix + c] = acc[c] / S.spp;
    }
  });
  uint64_t n = 0;
  for (uint64_t r : rays) n += r;
  return n;
}

// Gradient of sum(dimage3 * image3) (dimage3 = dLoss/dimage), added to the outputs.
static inline void diff_gradient(const DiffScene& S, const double* dimage3, double* g_albedo, double* g_rough,
                                 double* g_env, int nthreads) {
  const int T = std::max(nthreads, 1);
  std::vector<std::vector<double>> ga(T, std::vector<double>(3 * (size_t)S.n_mats, 0.0));
  std::vector<std::vector<double>> gr(T, std::vector<double>(S.n_mats, 0.0));
  std::vector<std::vector<double>> ge(T, std::vector<double>(3 * (size_t)S.env_w * S.env_h, 0.0));
  std::vector<uint64_t> rays(T, 0);
  parallel_for((size_t)S.W * S.H, T, [&](size_t b, size_t e, int tid) {
    std::vector<int32_t> stack;
    DiffVertex vtx[8];
    for (size_t pix = b; pix < e; pix++) {
      const uint32_t px = (uint32_t)(pix % S.W), py = (uint32_t)(pix / S.W);
      const double g[3] = {dimage3[3 * pix] / S.spp, dimage3[3 * pix + 1] / S.spp, dimage3[3 * pix + 2] / S.spp};
      for (int s = 0; s < S.spp; s++) {
        int nv = 0;
        const int tex = diff_trace_path(S, px, py, (uint32_t)s, vtx, nv, stack, rays[tid]);
        if (tex < 0) continue;
        double w[8][3], dwa[8][3], dwr[8][3];
        for (int i = 0; i < nv; i++) diff_gain(S, vtx[i], w[i], dwa[i], dwr[i]);
        const double* E = S.env + 3 * (size_t)tex;
        for (int c = 0; c < 3; c++) {
          double beta = 1.0;
          for (int i = 0; i < nv; i++) beta *= w[i][c];
          ge[tid][3 * (size_t)tex + c] += g[c] * beta;
        }
        for (int i = 0; i < nv; i++) {
          const int m = vtx[i].mat;
          for (int c = 0; c < 3; c++) {
            double other = E[c];
            for (int j = 0; j < nv; j++)
              if (j != i) other *= w[j][c];
            ga[tid][3 * (size_t)m + c] += g[c] * other * dwa[i][c];
            gr[tid][m] += g[c] * other * dwr[i][c];
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
