// pk_diff.cu -- form (3): differentiable rendering with a path-replay adjoint.
//
// No reference counterpart (the reference has no differentiation).  The
// forward estimator renders the current scene with continuous FP32 material
// parameters (albedo RGB, roughness, metallic per material slot) and an FP32
// RGB equirect environment:
//
//   per pixel, per sample: pinhole camera ray with jitter; up to `depth`
//   rays; at a hit (geometric normal facing the ray) the next direction is
//   cosine-sampled around the normal, independent of every parameter, so the
//   sampled paths are a fixed function of the seed; the throughput gains
//   w_c = pi * f_c (f = Lambert (1-metal)(1-F_c) albedo_c / pi + GGX D G F_c /
//   (4 cos_o cos_i), alpha = roughness^2, F0 = mix(0.04, albedo, metal),
//   D = alpha^2 / (pi (|n x h|^2 + (n.h)^2 alpha^2)^2),
//   Schlick F) multiply; a ray that escapes adds throughput * env(texel).
//
// Because the paths do not depend on the parameters, the estimator is a
// smooth function of them for fixed seeds: its derivative is what central
// finite differences with common random numbers measure.  The adjoint kernel
// replays every path from its seed (nothing is stored between the passes),
// forms the contribution C_c = E_c * prod_i w_{i,c} and scatters
//   dL/dalbedo_{m,c} += g_c * (C_c / w_{i,c}) * dw_{i,c}/dalbedo_c,
//   dL/droughness_m  += sum_c g_c * (C_c / w_{i,c}) * dw_{i,c}/dr,
//   dL/denv_{t,c}    += g_c * prod_i w_{i,c}
// (the products over the other vertices are taken directly, not divided).
// Material terms go through warp-aggregated atomics into per-block FP32
// partials in shared memory, flushed with FP64 atomics; environment terms
// are warp-aggregated per texel and added in FP64.
//
// Random numbers, directions, hit points and texel lookups use the pinned
// built-ins of pk_math.cuh, so the CPU oracle replays the same paths bit for
// bit and differs only in the precision of the BSDF and gradient arithmetic.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>

#include "../../include/pike.h"
#include "pk_ctx.h"
#include "pk_math.cuh"
#include "pk_traverse.cuh"

namespace pk {

constexpr int DIFF_THREADS = 128;  // = TRACE_THREADS (traversal stack layout)
constexpr int DIFF_MAX_DEPTH = 8;
constexpr float DIFF_OFFSET = 1e-4f;
constexpr float DIFF_TAU = 6.283185307179586f;
constexpr float DIFF_PI = 3.141592653589793f;

struct DiffCam {
  float o[3], f[3], r[3], u[3];
};
struct DiffParams {
  const float* albedo;  // n_mats x 3
  const float* rough;
  const float* metal;
  uint32_t n_mats;
  const float* env;     // env_h x env_w x 3
  int env_w, env_h;
  int spp, depth;
  uint32_t seed;
};

struct Vertex {
  V3 n, wo, wi;
  int mat;
};

__device__ __forceinline__ Hash path_rng(uint32_t px, uint32_t py, uint32_t s, uint32_t seed) {
  Hash h;
  h.seed = (px * 1973u + py * 9277u + (s + seed * 65536u) * 26699u) | 1u;
  h.seed = h.next();
  return h;
}

__device__ __forceinline__ int env_texel(const DiffParams& P, V3 d) {
  const float u = atan2_(d.z, d.x) / DIFF_TAU + 0.5f;
  const float v = acos_(fmin_(fmax_(d.y, -1.0f), 1.0f)) / DIFF_PI;
  int ix = f2i(u * (float)P.env_w), iy = f2i(v * (float)P.env_h);
  ix = ix < 0 ? 0 : (ix >= P.env_w ? P.env_w - 1 : ix);
  iy = iy < 0 ? 0 : (iy >= P.env_h ? P.env_h - 1 : iy);
  return iy * P.env_w + ix;
}

// Duff et al. 2017 branchless orthonormal basis around n.
__device__ __forceinline__ void basis(V3 n, V3& b1, V3& b2) {
  const float sign = n.z >= 0.0f ? 1.0f : -1.0f;
  const float a = -1.0f / (sign + n.z);
  const float b = n.x * n.y * a;
  b1 = v3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
  b2 = v3(b, sign + n.y * n.y * a, -n.y);
}

// One path: fills up to depth-1 vertices; returns the escaped texel or -1.
__device__ __forceinline__ int trace_path(const SceneDev& sc, const DiffCam& cam, const DiffParams& P, uint32_t px,
                                          uint32_t py, uint32_t s, uint32_t W, uint32_t H, Vertex* vtx, int& nv,
                                          int (*sstack)[TRACE_THREADS], uint32_t* err, uint32_t& nrays) {
  Hash h = path_rng(px, py, s, P.seed);
  const float jx = h.rand(), jy = h.rand();
  const float sx = 2.0f * (((float)px + jx) / (float)W) - 1.0f;
  const float sy = 1.0f - 2.0f * (((float)py + jy) / (float)H);
  V3 o = v3(cam.o[0], cam.o[1], cam.o[2]);
  V3 d = normalize(add(add(v3(cam.f[0], cam.f[1], cam.f[2]), scale(v3(cam.r[0], cam.r[1], cam.r[2]), sx)),
                       scale(v3(cam.u[0], cam.u[1], cam.u[2]), sy)));
  nv = 0;
  for (int b = 0; b < P.depth; b++) {
    float t;
    int idx;
    uint32_t bary, nf = 0, nt = 0;
    traverse<false, false>(sc, o.x, o.y, o.z, d.x, d.y, d.z, t, idx, bary, sstack, err, nf, nt);
    nrays++;
    if (idx < 0) return env_texel(P, d);
    if (b == P.depth - 1) return -1;
    const float4* tp = sc.tris + 3 * (size_t)idx;
    const float4 A = __ldg(tp), B = __ldg(tp + 1), Cc = __ldg(tp + 2);
    V3 n = normalize(cross(v3(A.w, B.x, B.y), v3(B.z, B.w, Cc.x)));
    if (dot(n, d) > 0.0f) n = neg(n);
    const V3 p = add(add(o, scale(d, t)), scale(n, DIFF_OFFSET));
    const float u1 = h.rand(), u2 = h.rand();
    const float rr = sqrtf(u1), phi = DIFF_TAU * u2;
    const float lz = sqrtf(fmax_(1.0f - u1, 0.0f));
    V3 b1, b2;
    basis(n, b1, b2);
    const V3 wi = add(add(scale(b1, rr * cos_(phi)), scale(b2, rr * sin_(phi))), scale(n, lz));
    int m = __ldg(sc.tri4 + idx).w;
    m = (uint32_t)m < P.n_mats ? m : 0;
    vtx[nv].n = n;
    vtx[nv].wo = neg(d);
    vtx[nv].wi = wi;
    vtx[nv].mat = m;
    nv++;
    o = p;
    d = wi;
  }
  return -1;
}

// Throughput gain w = pi f and its derivatives (per channel c for albedo_c,
// and d/droughness).
__device__ __forceinline__ void bsdf_gain(const DiffParams& P, const Vertex& v, float w[3], float dwa[3],
                                          float dwr[3]) {
  const float co = fmax_(dot(v.n, v.wo), 1e-6f), ci = fmax_(dot(v.n, v.wi), 1e-6f);
  const V3 hv = normalize(add(v.wo, v.wi));
  const float nh = fmax_(dot(v.n, hv), 0.0f), vh = fmin_(fmax_(dot(v.wo, hv), 0.0f), 1.0f);
  const float r = P.rough[v.mat], mt = P.metal[v.mat];
  const float al = r * r, a2 = al * al;
  // nh^2 (a2 - 1) + 1 written as |n x h|^2 + nh^2 a2: no cancellation near the peak
  const V3 nxh = cross(v.n, hv);
  const float Bd = dot(nxh, nxh) + nh * nh * a2;
  const float D = a2 / (DIFF_PI * Bd * Bd);
  const float dD = (2.0f * al / (DIFF_PI * Bd * Bd)) * (1.0f - 2.0f * a2 * nh * nh / Bd);
  const float So = sqrtf(a2 + (1.0f - a2) * co * co), Si = sqrtf(a2 + (1.0f - a2) * ci * ci);
  const float G1o = 2.0f * co / (co + So), G1i = 2.0f * ci / (ci + Si);
  const float dG1o = -2.0f * co * (al * (1.0f - co * co) / So) / ((co + So) * (co + So));
  const float dG1i = -2.0f * ci * (al * (1.0f - ci * ci) / Si) / ((ci + Si) * (ci + Si));
  const float G = G1o * G1i, dG = dG1o * G1i + G1o * dG1i;
  const float k5 = (1.0f - vh) * (1.0f - vh) * (1.0f - vh) * (1.0f - vh) * (1.0f - vh);
  const float spec = 1.0f / (4.0f * co * ci);
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const float a = P.albedo[3 * v.mat + c];
    const float F0 = 0.04f * (1.0f - mt) + a * mt;
    const float F = F0 + (1.0f - F0) * k5;
    const float dF = mt * (1.0f - k5);
    const float kd = (1.0f - mt) * (1.0f - F);
    w[c] = kd * a + DIFF_PI * D * G * F * spec;
    dwa[c] = kd - (1.0f - mt) * dF * a + DIFF_PI * D * G * dF * spec;
    dwr[c] = DIFF_PI * F * spec * (dD * G + D * dG) * 2.0f * r;
  }
}

__global__ void __launch_bounds__(DIFF_THREADS) k_diff_forward(SceneDev sc, DiffCam cam, DiffParams P, uint32_t W,
                                                               uint32_t H, float4* __restrict__ image,
                                                               uint32_t* err, unsigned long long* rays) {
  __shared__ int sstack[STACK_SMEM][TRACE_THREADS];
  const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= W * H) return;
  const uint32_t px = pix % W, py = pix / W;
  Vertex vtx[DIFF_MAX_DEPTH];
  float acc[3] = {0.0f, 0.0f, 0.0f};
  uint32_t nrays = 0;
  for (int s = 0; s < P.spp; s++) {
    int nv;
    const int tex = trace_path(sc, cam, P, px, py, (uint32_t)s, W, H, vtx, nv, sstack, err, nrays);
    if (tex < 0) continue;
    float beta[3] = {1.0f, 1.0f, 1.0f};
    for (int i = 0; i < nv; i++) {
      float w[3], dwa[3], dwr[3];
      bsdf_gain(P, vtx[i], w, dwa, dwr);
      beta[0] *= w[0]; beta[1] *= w[1]; beta[2] *= w[2];
    }
    const float* e = P.env + 3 * (size_t)tex;
    acc[0] += beta[0] * e[0];
    acc[1] += beta[1] * e[1];
    acc[2] += beta[2] * e[2];
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

__global__ void __launch_bounds__(DIFF_THREADS) k_diff_adjoint(SceneDev sc, DiffCam cam, DiffParams P, uint32_t W,
                                                               uint32_t H, const float4* __restrict__ dimage,
                                                               double* __restrict__ g_albedo,
                                                               double* __restrict__ g_rough,
                                                               double* __restrict__ g_env, uint32_t* err,
                                                               unsigned long long* rays) {
  __shared__ int sstack[STACK_SMEM][TRACE_THREADS];
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
  Vertex vtx[DIFF_MAX_DEPTH];
  uint32_t nrays = 0;
  for (int s = 0; s < P.spp; s++) {
    int nv = 0, tex = -1;
    if (live) tex = trace_path(sc, cam, P, px, py, (uint32_t)s, W, H, vtx, nv, sstack, err, nrays);
    if (tex < 0) nv = 0;
    float w[DIFF_MAX_DEPTH][3], dwa[DIFF_MAX_DEPTH][3], dwr[DIFF_MAX_DEPTH][3];
    for (int i = 0; i < nv; i++) bsdf_gain(P, vtx[i], w[i], dwa[i], dwr[i]);
    float e[3] = {0.0f, 0.0f, 0.0f};
    if (tex >= 0) {
      const float* ep = P.env + 3 * (size_t)tex;
      e[0] = ep[0]; e[1] = ep[1]; e[2] = ep[2];
    }
    // environment texel: g * prod_i w_i
    {
      float beta[3] = {1.0f, 1.0f, 1.0f};
      for (int i = 0; i < nv; i++) { beta[0] *= w[i][0]; beta[1] *= w[i][1]; beta[2] *= w[i][2]; }
      for (int c = 0; c < 3; c++) {
        bool lead;
        const float sum = group_sum(0xffffffffu, tex, tex >= 0 ? g[c] * beta[c] : 0.0f, lead);
        if (lead && tex >= 0) atomicAdd(g_env + 3 * (size_t)tex + c, (double)sum);
      }
    }
    // vertices: the product of the other vertices' gains times the env radiance
    for (int i = 0; i < DIFF_MAX_DEPTH - 1; i++) {
      if (!__any_sync(0xffffffffu, i < nv)) break;
      const bool on = i < nv;
      const int key = on ? vtx[i].mat : -1;
      float da[3] = {0.0f, 0.0f, 0.0f}, dr = 0.0f;
      if (on) {
        for (int c = 0; c < 3; c++) {
          float other = e[c];
          for (int j = 0; j < nv; j++)
            if (j != i) other *= w[j][c];
          da[c] = g[c] * other * dwa[i][c];
          dr += g[c] * other * dwr[i][c];
        }
      }
      bool lead;
      const float s0 = group_sum(0xffffffffu, key, da[0], lead);
      const float s1 = group_sum(0xffffffffu, key, da[1], lead);
      const float s2 = group_sum(0xffffffffu, key, da[2], lead);
      const float s3 = group_sum(0xffffffffu, key, dr, lead);
      if (lead && key >= 0) {
        atomicAdd(&spart[4 * key + 0], s0);
        atomicAdd(&spart[4 * key + 1], s1);
        atomicAdd(&spart[4 * key + 2], s2);
        atomicAdd(&spart[4 * key + 3], s3);
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

int diff_check(pk_ctx* c, const pk_diff_camera* cam, const pk_diff_params* p, DiffCam& dc, DiffParams& dp) {
  if (!c->bvh_ready) { c->err = "pk_diff: no BVH"; return PK_ERR_STATE; }
  if (!c->W || !c->H) { c->err = "pk_diff: call pk_configure first"; return PK_ERR_STATE; }
  if (!cam || !p || !p->albedo3 || !p->roughness || !p->metallic || !p->env_rgb) {
    c->err = "pk_diff: null argument";
    return PK_ERR_ARG;
  }
  if (p->n_mats < c->n_mats || p->n_mats == 0 || p->n_mats > 4096) {
    c->err = "pk_diff: n_mats must cover the scene's materials (at most 4096)";
    return PK_ERR_ARG;
  }
  if (!p->env_w || !p->env_h || (uint64_t)p->env_w * p->env_h > (1ull << 26) || !p->spp || p->spp > 65536 ||
      p->depth < 1 || p->depth > DIFF_MAX_DEPTH) {
    c->err = "pk_diff: bad env size, spp or depth (1..8)";
    return PK_ERR_ARG;
  }
  for (int k = 0; k < 3; k++) {
    dc.o[k] = cam->origin[k];
    dc.f[k] = cam->forward[k];
    dc.r[k] = cam->right[k];
    dc.u[k] = cam->up[k];
  }
  dp = DiffParams{p->albedo3, p->roughness, p->metallic, p->n_mats, p->env_rgb, (int)p->env_w, (int)p->env_h,
                  (int)p->spp, (int)p->depth, p->seed};
  return PK_OK;
}

}  // namespace
}  // namespace pk

using namespace pk;

extern "C" int pk_diff_render(pk_ctx* c, const pk_diff_camera* cam, const pk_diff_params* p, float* image4) {
  if (!c) return PK_ERR_ARG;
  try {
    check(cudaSetDevice(c->device), "cudaSetDevice");
    DiffCam dc;
    DiffParams dp;
    const int rc = diff_check(c, cam, p, dc, dp);
    if (rc != PK_OK) return rc;
    if (!image4) { c->err = "pk_diff_render: null image"; return PK_ERR_ARG; }
    DevBuf<uint32_t> err(1);
    DevBuf<unsigned long long> rays(1);
    check(cudaMemsetAsync(err.p, 0, 4, c->stream), "memset");
    check(cudaMemsetAsync(rays.p, 0, 8, c->stream), "memset");
    const uint32_t n = c->W * c->H;
    k_diff_forward<<<(n + DIFF_THREADS - 1) / DIFF_THREADS, DIFF_THREADS, 0, c->stream>>>(
        c->dropin_scene(), dc, dp, c->W, c->H, reinterpret_cast<float4*>(image4), err.p, rays.p);
    check(cudaGetLastError(), "k_diff_forward");
    uint32_t herr = 0;
    unsigned long long hr = 0;
    check(cudaMemcpyAsync(&herr, err.p, 4, cudaMemcpyDeviceToHost, c->stream), "D2H");
    check(cudaMemcpyAsync(&hr, rays.p, 8, cudaMemcpyDeviceToHost, c->stream), "D2H");
    check(cudaStreamSynchronize(c->stream), "sync");
    c->diff_rays = hr;
    if (herr) { c->err = "pk_diff_render: device error flags (traversal stack)"; return PK_ERR_DEVICE; }
    return PK_OK;
  } catch (CudaError& e) {
    c->err = e.what();
    return PK_ERR_CUDA;
  }
}

extern "C" int pk_diff_backward(pk_ctx* c, const pk_diff_camera* cam, const pk_diff_params* p,
                                const float* d_image4, double* g_albedo3, double* g_roughness, double* g_env_rgb) {
  if (!c) return PK_ERR_ARG;
  try {
    check(cudaSetDevice(c->device), "cudaSetDevice");
    DiffCam dc;
    DiffParams dp;
    const int rc = diff_check(c, cam, p, dc, dp);
    if (rc != PK_OK) return rc;
    if (!d_image4 || !g_albedo3 || !g_roughness || !g_env_rgb) { c->err = "pk_diff_backward: null buffer"; return PK_ERR_ARG; }
    DevBuf<uint32_t> err(1);
    DevBuf<unsigned long long> rays(1);
    check(cudaMemsetAsync(err.p, 0, 4, c->stream), "memset");
    check(cudaMemsetAsync(rays.p, 0, 8, c->stream), "memset");
    const uint32_t n = c->W * c->H;
    const size_t smem = 16 * (size_t)p->n_mats;
    if (smem > 48 * 1024)
      check(cudaFuncSetAttribute(k_diff_adjoint, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "attr");
    k_diff_adjoint<<<(n + DIFF_THREADS - 1) / DIFF_THREADS, DIFF_THREADS, smem, c->stream>>>(
        c->dropin_scene(), dc, dp, c->W, c->H, reinterpret_cast<const float4*>(d_image4), g_albedo3, g_roughness,
        g_env_rgb, err.p, rays.p);
    check(cudaGetLastError(), "k_diff_adjoint");
    uint32_t herr = 0;
    unsigned long long hr = 0;
    check(cudaMemcpyAsync(&herr, err.p, 4, cudaMemcpyDeviceToHost, c->stream), "D2H");
    check(cudaMemcpyAsync(&hr, rays.p, 8, cudaMemcpyDeviceToHost, c->stream), "D2H");
    check(cudaStreamSynchronize(c->stream), "sync");
    c->diff_rays = hr;
    if (herr) { c->err = "pk_diff_backward: device error flags (traversal stack)"; return PK_ERR_DEVICE; }
    return PK_OK;
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
