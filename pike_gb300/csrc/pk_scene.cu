// pk_scene.cu -- scene-side kernels: attribute quantisation (row S) and the
// conversion of the reference's serialised BVH into the traversal format.
#include <cuda_runtime.h>

#include "pk_internal.cuh"
#include "pk_render.h"
#include "pk_util.h"

namespace pk {

// ---- Row S: scene.js:456-470 per-vertex attributes ------------------------
// ECMAScript ToInt8/ToInt16: NaN/inf -> 0, truncate toward zero, wrap.
__device__ __forceinline__ int js_toint(double v, int bits) {
  if (!isfinite(v)) return 0;
  const double mod = (double)(1 << bits);
  double m = fmod(trunc(v), mod);
  if (m < 0.0) m += mod;
  int mi = (int)m;
  if (mi >= (1 << (bits - 1))) mi -= (1 << bits);
  return mi;
}
// Vec.normalize: v * (1 / sqrt((x*x + y*y) + z*z)), then _quantizeVec3ToInt.
__device__ __forceinline__ uint32_t quantize3(double x, double y, double z) {
  const double m = sqrt(x * x + y * y + z * z);
  const double s = 1.0 / m;
  const double v[3] = {x * s, y * s, z * s};
  uint32_t out = 0;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const int b = js_toint(v[i] * (v[i] > 0.0 ? 127.0 : 128.0), 8);
    out |= (uint32_t)(uint8_t)b << (8 * i);
  }
  return out;
}
__device__ __forceinline__ uint32_t quantize2(double a, double b) {
  const int s0 = js_toint(a * (a > 0.0 ? 32767.0 : 32768.0), 16);
  const int s1 = js_toint(b * (b > 0.0 ? 32767.0 : 32768.0), 16);
  return (uint32_t)(uint16_t)s0 | ((uint32_t)(uint16_t)s1 << 16);
}

// bn3/bt4 are the normal and signed tangent the bitangent is built from:
// scene.js:160 takes them before the prop's rotations, so a caller that rotates
// on the host passes both forms (pk_scene_flatten_tbn); otherwise they alias
// nrm3/tan4.
__global__ void k_flatten(const double* __restrict__ pos3, const double* __restrict__ nrm3,
                          const double* __restrict__ tan4, const double* __restrict__ bn3,
                          const double* __restrict__ bt4, const double* __restrict__ uv2, uint32_t n, double scl,
                          double tx, double ty, double tz, double* __restrict__ pos_out3, uint4* __restrict__ attrs) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* p = pos3 + 3 * (size_t)i;
  const double* nr = nrm3 + 3 * (size_t)i;
  const double* tg = tan4 + 4 * (size_t)i;
  const double* bn = bn3 + 3 * (size_t)i;
  const double* bt = bt4 + 4 * (size_t)i;
  pos_out3[3 * (size_t)i + 0] = p[0] * scl + tx;
  pos_out3[3 * (size_t)i + 1] = p[1] * scl + ty;
  pos_out3[3 * (size_t)i + 2] = p[2] * scl + tz;
  // normal / tangent pass through _applyVectorTransforms(v, t, true): v * 1 + 0
  const double nx = nr[0] * 1.0 + 0.0, ny = nr[1] * 1.0 + 0.0, nz = nr[2] * 1.0 + 0.0;
  const double ux = tg[0] * 1.0 + 0.0, uy = tg[1] * 1.0 + 0.0, uz = tg[2] * 1.0 + 0.0;
  // bitangent = normalize(cross(normalAt, tangentAt) * (w || 1)); cross.y = -(a0*b2 - a2*b0)
  double cx = bn[1] * bt[2] - bn[2] * bt[1];
  double cy = -(bn[0] * bt[2] - bn[2] * bt[0]);
  double cz = bn[0] * bt[1] - bn[1] * bt[0];
  const double w = bt[3];
  const double sg = (w != 0.0 && w == w) ? w : 1.0;
  cx = cx * sg; cy = cy * sg; cz = cz * sg;
  const double* uv = uv2 + 2 * (size_t)i;
  attrs[i] = make_uint4(quantize3(ux, uy, uz), quantize3(cx, cy, cz), quantize3(nx, ny, nz), quantize2(uv[0], uv[1]));
}

void launch_flatten(cudaStream_t s, const double* pos3, const double* nrm3, const double* tan4, const double* bn3,
                    const double* bt4, const double* uv2, uint32_t n, double scale, double tx, double ty, double tz,
                    double* pos_out3, uint4* attrs) {
  if (n == 0) return;
  k_flatten<<<(n + 255) / 256, 256, 0, s>>>(pos3, nrm3, tan4, bn3, bt4, uv2, n, scale, tx, ty, tz, pos_out3, attrs);
}

// ---- serialised BVH -> traversal format --------------------------------
__global__ void k_inner_flags(const int32_t* __restrict__ nodes5, uint32_t n, uint32_t* __restrict__ flag) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  // trace.wgsl:155: a node is a leaf iff triangles > -1
  flag[i] = nodes5[5 * (size_t)i + 1] > -1 ? 0u : 1u;
}

__device__ __forceinline__ void decode_box(const int32_t* nd, float* b6) {
  const uint32_t m[3] = {(uint32_t)nd[2], (uint32_t)nd[3], (uint32_t)nd[4]};
#pragma unroll
  for (int a = 0; a < 3; a++) {
    b6[2 * a + 0] = snorm16((int)(int16_t)(uint16_t)(m[a] & 0xffffu));  // x_range.x (quantised max)
    b6[2 * a + 1] = snorm16((int)(int16_t)(uint16_t)(m[a] >> 16));      // x_range.y (quantised min)
  }
}
// Leaf words must address triangles inside the leaf-ordered array.
__device__ __forceinline__ int child_code(const int32_t* __restrict__ nodes5, const uint32_t* __restrict__ rank,
                                          uint32_t i, uint32_t n_tris, uint32_t* err) {
  const int32_t tri = nodes5[5 * (size_t)i + 1];
  if (tri > -1) {
    const uint32_t size = (uint32_t)tri >> 24, base = (uint32_t)tri & 0x00ffffffu;
    if (size >= 128u || base + size > n_tris) {
      atomicOr(err, ERR_BVH);
      return (int)0x80000000u;  // an empty leaf
    }
    return (int)(0x80000000u | (uint32_t)tri);
  }
  return (int)rank[i];
}

// Children must come after their parent in BFS order (serializeTree), which
// also rules out cycles: every traversal step moves to a larger node index.
__global__ void k_inner_records(const int32_t* __restrict__ nodes5, uint32_t n, const uint32_t* __restrict__ rank,
                                uint32_t n_tris, float4* __restrict__ inner, int* __restrict__ root_code,
                                uint32_t* err) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t* nd = nodes5 + 5 * (size_t)i;
  if (i == 0) *root_code = child_code(nodes5, rank, 0, n_tris, err);
  if (nd[1] > -1) return;
  const int32_t l = nd[0];
  if (l < 1 || (uint32_t)l <= i || (uint32_t)l + 1 >= n) {
    atomicOr(err, ERR_BVH);
    float4* r = inner + 4 * (size_t)rank[i];
    const float4 none = make_float4(0.f, 0.f, 0.f, 0.f);
    r[0] = none; r[1] = none; r[2] = none;
    reinterpret_cast<int4*>(r)[3] = make_int4((int)0x80000000u, (int)0x80000000u, 0, 0);
    return;
  }
  float lb[6], rb[6];
  decode_box(nodes5 + 5 * (size_t)l, lb);
  decode_box(nodes5 + 5 * (size_t)(l + 1), rb);
  float4* r = inner + 4 * (size_t)rank[i];
  r[0] = make_float4(lb[0], lb[1], lb[2], lb[3]);
  r[1] = make_float4(lb[4], lb[5], rb[0], rb[1]);
  r[2] = make_float4(rb[2], rb[3], rb[4], rb[5]);
  reinterpret_cast<int4*>(r)[3] = make_int4(child_code(nodes5, rank, (uint32_t)l, n_tris, err),
                                            child_code(nodes5, rank, (uint32_t)l + 1, n_tris, err), 0, 0);
}

// 32-byte records: the children's reference masks and child codes.
__global__ void k_inner_records32(const int32_t* __restrict__ nodes5, uint32_t n, const uint32_t* __restrict__ rank,
                                  const float4* __restrict__ inner64, int4* __restrict__ inner32) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t* nd = nodes5 + 5 * (size_t)i;
  if (nd[1] > -1) return;
  const uint32_t r = rank[i];
  const int4 codes = reinterpret_cast<const int4*>(inner64 + 4 * (size_t)r)[3];  // validated child codes
  const int32_t l = nd[0];
  int4 q0 = make_int4(0, 0, 0, 0), q1 = make_int4(0, 0, codes.x, codes.y);
  if (l >= 1 && (uint32_t)l > i && (uint32_t)l + 1 < n) {
    const int32_t* a = nodes5 + 5 * (size_t)l;
    const int32_t* b = nodes5 + 5 * (size_t)(l + 1);
    q0 = make_int4(a[2], a[3], a[4], b[2]);
    q1 = make_int4(b[3], b[4], codes.x, codes.y);
  }
  inner32[2 * (size_t)r] = q0;
  inner32[2 * (size_t)r + 1] = q1;
}

__global__ void k_tri_edges(const int4* __restrict__ tri4, uint32_t n, const float4* __restrict__ verts4,
                            uint32_t n_verts, float4* __restrict__ tris, uint32_t* err) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int4 t = tri4[k];
  if (t.x < 0 || t.y < 0 || t.z < 0 || (uint32_t)t.x >= n_verts || (uint32_t)t.y >= n_verts ||
      (uint32_t)t.z >= n_verts) {
    atomicOr(err, ERR_BVH);
    tris[3 * (size_t)k + 0] = make_float4(0.f, 0.f, 0.f, 0.f);
    tris[3 * (size_t)k + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
    tris[3 * (size_t)k + 2] = make_float4(0.f, 0.f, 0.f, 0.f);
    return;
  }
  const float4 v0 = verts4[t.x], v1 = verts4[t.y], v2 = verts4[t.z];
  const float e1x = v1.x - v0.x, e1y = v1.y - v0.y, e1z = v1.z - v0.z;
  const float e2x = v2.x - v0.x, e2y = v2.y - v0.y, e2z = v2.z - v0.z;
  tris[3 * (size_t)k + 0] = make_float4(v0.x, v0.y, v0.z, e1x);
  tris[3 * (size_t)k + 1] = make_float4(e1y, e1z, e2x, e2y);
  tris[3 * (size_t)k + 2] = make_float4(e2z, 0.0f, 0.0f, 0.0f);
}

int convert_bvh(cudaStream_t s, const int32_t* nodes5, uint32_t n_nodes, const int4* tri4, uint32_t n_tris,
                const float4* verts4, uint32_t n_verts, float4* inner, int4* inner32, float4* tris, int* root_code,
                uint32_t* err) {
  DevBuf<uint32_t> flag(n_nodes), rank(n_nodes);
  // records in breadth-first order: the rank of an inner node among the inner
  // nodes in index order (a depth-first order was measured no faster: 3012-3015
  // against 3022-3032 Mrays/s at 1080p)
  k_inner_flags<<<(n_nodes + 255) / 256, 256, 0, s>>>(nodes5, n_nodes, flag.p);
  scan_exclusive_u32(s, flag.p, rank.p, n_nodes, nullptr);
  k_inner_records<<<(n_nodes + 255) / 256, 256, 0, s>>>(nodes5, n_nodes, rank.p, n_tris, inner, root_code, err);
  k_inner_records32<<<(n_nodes + 255) / 256, 256, 0, s>>>(nodes5, n_nodes, rank.p, inner, inner32);
  if (n_tris) k_tri_edges<<<(n_tris + 255) / 256, 256, 0, s>>>(tri4, n_tris, verts4, n_verts, tris, err);
  return cudaStreamSynchronize(s) == cudaSuccess ? 0 : 1;
}

}  // namespace pk
