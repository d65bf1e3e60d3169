// pk_env.cu -- EnvironmentGenerator tables (render/env_sampler.js:43-157):
// per-texel radiance, stable sort by descending radiance, equal-mass luminance
// bins and the per-texel pdf; and PK_ENV_ALIAS's alias table.  The total
// radiance (row-major sum) and the bin walk (a running sum reset at every bin)
// are sequentially rounded double sums in the reference, so they are one
// chain of dependent FP64 additions each.  On GB300 a chain of FP64 additions
// on one GPU lane runs about a hundred times slower than on a Grace core
// (2048x1024: 380 ms for the tables with both walks on one warp), so the two
// walks run on the host over the radiance the GPU computed; the radiance, the
// sort, the pdf texture and the coordinates stay on the GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "pk_internal.cuh"
#include "pk_util.h"

namespace pk {
namespace {

// _getRadiance (env_sampler.js:43-48): 2^(a-128) * luma(rgb) / 255, in double.
__global__ void k_env_radiance(const uchar4* __restrict__ rgbe, uint32_t n, double* __restrict__ rad,
                               unsigned long long* __restrict__ keys, uint32_t* __restrict__ vals) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uchar4 c = rgbe[i];
  const double power = ldexp(1.0, (int)c.w - 128);
  const double luma = 0.2126 * (double)c.x + 0.7152 * (double)c.y + 0.0722 * (double)c.z;
  const double r = power * luma / 255.0;
  rad[i] = r;
  // sort((a, b) => b.rad - a.rad): descending; radiance is finite and >= +0, so
  // the complemented bit pattern orders ascending keys by descending radiance.
  keys[i] = ~(unsigned long long)__double_as_longlong(r);
  vals[i] = i;
}

// The same radiance for an FP32 RGB map (the differentiable renderer's
// environment): luma of the stored values, in double.
__global__ void k_env_radiance_f32(const float* __restrict__ rgb, uint32_t n, double* __restrict__ rad,
                                   unsigned long long* __restrict__ keys, uint32_t* __restrict__ vals) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double r = 0.2126 * (double)rgb[3 * (size_t)i] + 0.7152 * (double)rgb[3 * (size_t)i + 1] +
                   0.0722 * (double)rgb[3 * (size_t)i + 2];
  const double v = r > 0.0 ? r : 0.0;  // negative or NaN radiance is never sampled
  rad[i] = v;
  keys[i] = ~(unsigned long long)__double_as_longlong(v);
  vals[i] = i;
}

// createPdfTexture / createEnvCoordBuffer (env_sampler.js:104-157).
__global__ void k_env_pdf(const uint32_t* __restrict__ order, uint32_t n, uint32_t w, const int2* __restrict__ bins,
                          uint32_t nb, int2* __restrict__ coords, float* __restrict__ pdf) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t lo = 0, hi = nb;  // the bin holding sorted position i
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) / 2;
    if ((uint32_t)bins[mid].x <= i) lo = mid; else hi = mid;
  }
  const int2 b = bins[lo];
  const double bin_pdf = 1.0 / (double)nb;
  const double coord_pdf = (double)n / (double)(b.y - b.x);
  const double sphere_pdf = 1.0 / (3.141592653589793 * 3.141592653589793 * 2.0);
  const uint32_t t = order[i];
  pdf[t] = (float)(bin_pdf * coord_pdf * sphere_pdf);
  coords[i] = make_int2((int)(t % w), (int)(t / w));
}

// ---------------- alias table (PK_ENV_ALIAS) -----------------------------
// Radiance in FP64 as k_env_radiance computes it.
__device__ __forceinline__ double texel_radiance(uchar4 c) {
  return ldexp(1.0, (int)c.w - 128) * (0.2126 * (double)c.x + 0.7152 * (double)c.y + 0.0722 * (double)c.z) / 255.0;
}

constexpr int ALIAS_THREADS = 256;
constexpr int ALIAS_PER_BLOCK = 4 * ALIAS_THREADS;

// Per-block sums of the radiance (fixed grouping: the total is the same
// double on every run).
__global__ void __launch_bounds__(ALIAS_THREADS) k_alias_partial(const uchar4* __restrict__ rgbe, uint32_t n,
                                                                double* __restrict__ partial) {
  __shared__ double s_warp[ALIAS_THREADS / 32];
  double v = 0.0;
  const uint32_t base = blockIdx.x * ALIAS_PER_BLOCK + threadIdx.x;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const uint32_t i = base + k * ALIAS_THREADS;
    if (i < n) v += texel_radiance(rgbe[i]);
  }
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) s_warp[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < ALIAS_THREADS / 32; k++) t += s_warp[k];
    partial[blockIdx.x] = t;
  }
}

// The total (one block, fixed grouping) and the fixed-point scale
// n * 2^frac / total; status 1 for a black or non-finite map.
__global__ void k_alias_total(const double* __restrict__ partial, uint32_t m, uint32_t n, int frac,
                              double* __restrict__ scale, uint32_t* __restrict__ status) {
  __shared__ double s[1024];
  double v = 0.0;
  for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) v += partial[i];
  s[threadIdx.x] = v;
  __syncthreads();
  for (uint32_t w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double t = s[0];
    const bool ok = t > 0.0 && isfinite(t);
    *status = ok ? 0u : 1u;
    *scale = ok ? ldexp((double)n, frac) / t : 0.0;
  }
}

// q_i = round(radiance_i * scale): the texel's weight in units of 2^-frac of
// the mean; light (q < one) or heavy.
__global__ void k_alias_weights(const uchar4* __restrict__ rgbe, uint32_t n, const double* __restrict__ scale,
                                unsigned long long one, unsigned long long* __restrict__ q,
                                uint32_t* __restrict__ light) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned long long w = __double2ull_rn(texel_radiance(rgbe[i]) * *scale);
  q[i] = w;
  light[i] = w < one ? 1u : 0u;
}

// Light texels in index order with their deficits (one - q), heavy texels
// with their excesses (q - one).
__global__ void k_alias_split(const unsigned long long* __restrict__ q, const uint32_t* __restrict__ light,
                              const uint32_t* __restrict__ lrank, uint32_t n, unsigned long long one,
                              uint32_t* __restrict__ lidx, unsigned long long* __restrict__ ldef,
                              uint32_t* __restrict__ hidx, unsigned long long* __restrict__ hexc) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t r = lrank[i];
  if (light[i]) {
    lidx[r] = i;
    ldef[r] = one - q[i];
  } else {
    hidx[i - r] = i;
    hexc[i - r] = q[i] - one;
  }
}

__device__ __forceinline__ uint32_t alias_threshold(unsigned long long prob, unsigned long long one, int frac) {
  if (prob >= one) return 0xffffffffu;
  const unsigned long long t = prob >> (frac - 32);
  return t > 0xfffffffeull ? 0xfffffffeu : (uint32_t)t;
}

// The sweep of Huebschle-Schneider & Sanders ("Parallel Weighted Random
// Sampling", 2022) without running it: with D(a) the deficits of the first a
// lights and E(b) the excesses of the first b heavies (exclusive prefix
// sums), heavy b serves light a iff E(b) < D(a) <= E(b + 1) (b = 0 needs only
// the right side), and heavy b turns light at the first light a with
// D(a) > E(b + 1), keeping q_b + E(b) - D(a) and taking heavy b + 1 as its
// alias; a = n_light (D of all lights) stands for the end of the sweep, where
// the heavy in hand still turns when its weight has fallen below one.
// Lights the heavies cannot serve, the last heavy and heavies that never
// turn keep probability 1 (they differ from 1 only by the rounding of the
// weights).
__global__ void k_alias_lights(const uint32_t* __restrict__ lidx, const unsigned long long* __restrict__ dsum,
                               uint32_t nl, const uint32_t* __restrict__ hidx,
                               const unsigned long long* __restrict__ esum, const unsigned long long* __restrict__ hexc,
                               uint32_t nh, const unsigned long long* __restrict__ q, unsigned long long one, int frac,
                               uint2* __restrict__ table) {
  const uint32_t a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nl) return;
  const unsigned long long d = dsum[a];
  uint32_t lo = 0, hi = nh;  // first b with E(b + 1) >= D(a)
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (esum[mid] + hexc[mid] >= d) hi = mid; else lo = mid + 1;
  }
  const uint32_t t = lidx[a];
  table[t] = lo < nh ? make_uint2(alias_threshold(q[t], one, frac), hidx[lo]) : make_uint2(0xffffffffu, t);
}

__global__ void k_alias_heavies(const uint32_t* __restrict__ hidx, const unsigned long long* __restrict__ esum,
                                const unsigned long long* __restrict__ hexc, uint32_t nh,
                                const unsigned long long* __restrict__ dsum, uint32_t nl, unsigned long long one,
                                int frac, uint2* __restrict__ table) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nh) return;
  const unsigned long long e1 = esum[b] + hexc[b];
  uint32_t lo = 0, hi = nl + 1;  // first a in [0, nl] with D(a) > E(b + 1); D(nl) = all deficits
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (dsum[mid] > e1) hi = mid; else lo = mid + 1;
  }
  const uint32_t t = hidx[b];
  if (lo <= nl && b + 1 < nh) {
    const unsigned long long keep = one + hexc[b] + esum[b] - dsum[lo];  // q_b + E(b) - D(a), in [0, one)
    table[t] = make_uint2(alias_threshold(keep, one, frac), hidx[b + 1]);
  } else {
    table[t] = make_uint2(0xffffffffu, t);
  }
}

// Exact selection mass of each texel under the quantised table, in units of
// 2^-32: its kept share plus what the entries aliased to it pass on.
__global__ void k_alias_mass(const uint2* __restrict__ table, uint32_t n, unsigned long long* __restrict__ mass) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint2 e = table[i];
  const unsigned long long keep = e.x == 0xffffffffu ? (1ull << 32) : (unsigned long long)e.x;
  atomicAdd(mass + i, keep);
  if (keep < (1ull << 32)) atomicAdd(mass + e.y, (1ull << 32) - keep);
}

// mass / 2^32 is the texel's density in (u, v); / (2 pi^2) gives the unit of
// the histogram pdf texture (solid angle once divided by sin(phi)).
__global__ void k_alias_pdf(const unsigned long long* __restrict__ mass, uint32_t n, float* __restrict__ pdf) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double unit = 1.0 / (2.0 * 3.141592653589793 * 3.141592653589793);
  pdf[i] = (float)((double)mass[i] / 4294967296.0 * unit);
}

double js_min(double a, double b) { return (a != a || b != b) ? NAN : (a < b ? a : (b < a ? b : (std::signbit(a) ? a : b))); }
double js_max(double a, double b) { return (a != a || b != b) ? NAN : (a > b ? a : (b > a ? b : (std::signbit(a) ? b : a))); }

}  // namespace

namespace {

// The tables from per-texel radiance `rad` with sort keys and values already
// set (the radiance kernels above).
int build_from_radiance(cudaStream_t s, uint32_t w, uint32_t h, DevBuf<double>& rad,
                        DevBuf<unsigned long long>& keys, DevBuf<uint32_t>& vals, DevBuf<int2>& bins_out,
                        uint32_t& nb_out, DevBuf<int2>& coords_out, DevBuf<float>& pdf_out, std::string& why) {
  const uint32_t n = w * h;
  DevBuf<unsigned long long> keys_tmp(n);
  DevBuf<uint32_t> vals_tmp(n);
  std::vector<double> r(n);
  check(cudaMemcpyAsync(r.data(), rad.p, (size_t)n * 8, cudaMemcpyDeviceToHost, s), "D2H");
  radix_sort_pairs_u64(s, reinterpret_cast<uint64_t*>(keys.p), vals.p, reinterpret_cast<uint64_t*>(keys_tmp.p),
                       vals_tmp.p, n, 64);
  std::vector<uint32_t> order(n);
  check(cudaMemcpyAsync(order.data(), vals.p, (size_t)n * 4, cudaMemcpyDeviceToHost, s), "D2H");
  check(cudaStreamSynchronize(s), "sync");
  // totalRadiance += rad (row-major) and brightestTexel = max(rad, brightest)
  double total = 0.0, brightest = 0.0;
  for (uint32_t i = 0; i < n; i++) {
    brightest = std::fmax(r[i], brightest);
    total = total + r[i];
  }
  // numBins = min(256, max(32, 2 * ceil(total / brightest))); binSize = total / numBins
  const double num_bins = js_min(256.0, js_max(32.0, 2.0 * std::ceil(total / brightest)));
  if (num_bins != num_bins) { why = "environment has no radiance"; return 1; }
  const double bin_size = total / num_bins;
  // createLuminanceHistogram (env_sampler.js:74-94): walk the sorted texels,
  // closing a bin when the running sum reaches binSize, then resetting it.
  std::vector<int2> bins;
  double current = 0.0;
  int32_t prev = 0;
  for (uint32_t k = 0; k < n; k++) {
    if (current >= bin_size) {
      bins.push_back(make_int2(prev, (int)k));
      prev = (int)k;
      current = 0.0;
    }
    current = current + r[order[k]];
  }
  bins.push_back(make_int2(prev, (int)n));
  const uint32_t nbh = (uint32_t)bins.size();
  if (nbh < 2) { why = "environment yields a single luminance bin"; return 1; }
  if (nbh > 1024) { why = "too many luminance bins"; return 1; }
  bins_out.alloc(nbh);
  check(cudaMemcpyAsync(bins_out.p, bins.data(), (size_t)nbh * 8, cudaMemcpyHostToDevice, s), "H2D");
  coords_out.alloc(n);
  pdf_out.alloc(n);
  k_env_pdf<<<(n + 255) / 256, 256, 0, s>>>(vals.p, n, w, bins_out.p, nbh, coords_out.p, pdf_out.p);
  check(cudaGetLastError(), "env pdf");
  check(cudaStreamSynchronize(s), "sync");  // the host vectors are freed on return
  nb_out = nbh;
  return 0;
}

}  // namespace

// Builds bins (<= 257 entries), sorted coordinates and the pdf for a w x h
// RGBE image already on the device.  Returns non-zero with a reason on failure.
int build_env_tables_gpu(cudaStream_t s, const uchar4* rgbe, uint32_t w, uint32_t h, DevBuf<int2>& bins_out,
                         uint32_t& nb_out, DevBuf<int2>& coords_out, DevBuf<float>& pdf_out, std::string& why) {
  const uint32_t n = w * h;
  DevBuf<double> rad(n);
  DevBuf<unsigned long long> keys(n);
  DevBuf<uint32_t> vals(n);
  k_env_radiance<<<(n + 255) / 256, 256, 0, s>>>(rgbe, n, rad.p, keys.p, vals.p);
  return build_from_radiance(s, w, h, rad, keys, vals, bins_out, nb_out, coords_out, pdf_out, why);
}

// PK_ENV_ALIAS's table for a w x h RGBE image on the device: per texel
// {keep threshold, alias} (keep the uniformly drawn texel when the next 32-bit
// random number is below the threshold, always when it is 0xffffffff) and
// the pdf texture of its exact selection probabilities.  The radiance total
// and the normalisation are FP64; the weights are then fixed point (2^-frac
// of the mean, frac = 61 - ceil(log2 n)), so the prefix sums of the sweep are
// exact integers.
int build_env_alias_gpu(cudaStream_t s, const uchar4* rgbe, uint32_t w, uint32_t h, DevBuf<uint2>& table_out,
                        DevBuf<float>& pdf_out, std::string& why) {
  const uint32_t n = w * h;
  if (n == 0 || n > (1u << 29)) { why = "environment size out of range"; return 1; }
  int lg = 0;
  while ((1ull << lg) < n) lg++;
  const int frac = 61 - lg;  // >= 32
  const unsigned long long one = 1ull << frac;
  const unsigned nblk = (n + ALIAS_PER_BLOCK - 1) / ALIAS_PER_BLOCK, grid = (n + 255) / 256;
  DevBuf<double> partial(nblk), scale(1);
  DevBuf<uint32_t> status(1), light(n), lrank(n), nl_dev(1), lidx(n), hidx(n);
  DevBuf<unsigned long long> q(n), ldef(n + 1), hexc(n), esum(n), mass(n);
  k_alias_partial<<<nblk, ALIAS_THREADS, 0, s>>>(rgbe, n, partial.p);
  k_alias_total<<<1, 1024, 0, s>>>(partial.p, nblk, n, frac, scale.p, status.p);
  k_alias_weights<<<grid, 256, 0, s>>>(rgbe, n, scale.p, one, q.p, light.p);
  check(cudaGetLastError(), "alias weights");
  scan_exclusive_u32(s, light.p, lrank.p, n, nl_dev.p);  // synchronises
  uint32_t st = 0, nl = 0;
  check(cudaMemcpyAsync(&st, status.p, 4, cudaMemcpyDeviceToHost, s), "D2H");
  check(cudaMemcpyAsync(&nl, nl_dev.p, 4, cudaMemcpyDeviceToHost, s), "D2H");
  check(cudaStreamSynchronize(s), "sync");
  if (st) { why = "black or non-finite environment"; return 1; }
  const uint32_t nh = n - nl;
  check(cudaMemsetAsync(ldef.p + nl, 0, 8, s), "memset");  // D(nl) after the scan: all deficits
  k_alias_split<<<grid, 256, 0, s>>>(q.p, light.p, lrank.p, n, one, lidx.p, ldef.p, hidx.p, hexc.p);
  check(cudaGetLastError(), "alias split");
  scan_exclusive_u64(s, ldef.p, ldef.p, (size_t)nl + 1);  // D(a), a = 0..nl
  scan_exclusive_u64(s, hexc.p, esum.p, nh);  // E(b)
  table_out.alloc(n);
  pdf_out.alloc(n);
  if (nl) k_alias_lights<<<(nl + 255) / 256, 256, 0, s>>>(lidx.p, ldef.p, nl, hidx.p, esum.p, hexc.p, nh, q.p, one,
                                                          frac, table_out.p);
  if (nh) k_alias_heavies<<<(nh + 255) / 256, 256, 0, s>>>(hidx.p, esum.p, hexc.p, nh, ldef.p, nl, one, frac,
                                                           table_out.p);
  check(cudaMemsetAsync(mass.p, 0, mass.bytes(), s), "memset");
  k_alias_mass<<<grid, 256, 0, s>>>(table_out.p, n, mass.p);
  k_alias_pdf<<<grid, 256, 0, s>>>(mass.p, n, pdf_out.p);
  check(cudaGetLastError(), "alias table");
  check(cudaStreamSynchronize(s), "sync");
  return 0;
}

// The same tables for an FP32 RGB map (w x h x 3 on the device).
int build_env_tables_gpu_f32(cudaStream_t s, const float* rgb, uint32_t w, uint32_t h, DevBuf<int2>& bins_out,
                             uint32_t& nb_out, DevBuf<int2>& coords_out, DevBuf<float>& pdf_out, std::string& why) {
  const uint32_t n = w * h;
  DevBuf<double> rad(n);
  DevBuf<unsigned long long> keys(n);
  DevBuf<uint32_t> vals(n);
  k_env_radiance_f32<<<(n + 255) / 256, 256, 0, s>>>(rgb, n, rad.p, keys.p, vals.p);
  return build_from_radiance(s, w, h, rad, keys, vals, bins_out, nb_out, coords_out, pdf_out, why);
}

}  // namespace pk
