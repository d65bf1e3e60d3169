// pk_env.cu -- EnvironmentGenerator tables on the GPU (render/env_sampler.js:43-157):
// per-texel radiance, stable sort by descending radiance, equal-mass luminance
// bins and the per-texel pdf.  The total radiance (row-major sum) and the bin
// walk (a running sum reset at every bin) are sequentially rounded double sums
// in the reference, so each is computed by one warp in order: the warp streams
// 32 values at a time into registers and lane 0 adds them one by one.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>

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

// totalRadiance += rad (row-major) and brightestTexel = max(rad, brightest).
__global__ void k_env_total(const double* __restrict__ rad, uint32_t n, double* __restrict__ out2) {
  const int lane = threadIdx.x;
  double total = 0.0, brightest = 0.0;
  for (uint32_t base = 0; base < n; base += 32) {
    const double v = base + lane < n ? rad[base + lane] : 0.0;
    const uint32_t m = min(32u, n - base);
    for (uint32_t k = 0; k < m; k++) {
      const double x = __shfl_sync(0xffffffffu, v, (int)k);
      brightest = fmax(x, brightest);
      total = total + x;
    }
  }
  if (lane == 0) { out2[0] = total; out2[1] = brightest; }
}

// createLuminanceHistogram (env_sampler.js:74-94): walk the sorted texels,
// closing a bin when the running sum reaches binSize, then resetting it.
__global__ void k_env_bins(const double* __restrict__ rad, const uint32_t* __restrict__ order, uint32_t n,
                           double bin_size, int2* __restrict__ bins, uint32_t max_bins, uint32_t* __restrict__ nb_out) {
  const int lane = threadIdx.x;
  double current = 0.0;
  uint32_t nb = 0;
  int32_t prev = 0;
  for (uint32_t base = 0; base < n; base += 32) {
    const double v = base + lane < n ? rad[order[base + lane]] : 0.0;
    const uint32_t m = min(32u, n - base);
    for (uint32_t k = 0; k < m; k++) {
      const double x = __shfl_sync(0xffffffffu, v, (int)k);
      if (current >= bin_size) {
        if (lane == 0 && nb < max_bins) bins[nb] = make_int2(prev, (int)(base + k));
        prev = (int)(base + k);
        nb++;
        current = 0.0;
      }
      current = current + x;
    }
  }
  if (lane == 0) {
    if (nb < max_bins) bins[nb] = make_int2(prev, (int)n);
    *nb_out = nb + 1;
  }
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
  DevBuf<double> tot(2);
  DevBuf<unsigned long long> keys_tmp(n);
  DevBuf<uint32_t> vals_tmp(n), nb(1);
  k_env_total<<<1, 32, 0, s>>>(rad.p, n, tot.p);
  check(cudaGetLastError(), "env radiance");
  radix_sort_pairs_u64(s, reinterpret_cast<uint64_t*>(keys.p), vals.p, reinterpret_cast<uint64_t*>(keys_tmp.p),
                       vals_tmp.p, n, 64);
  double th[2];
  check(cudaMemcpyAsync(th, tot.p, 16, cudaMemcpyDeviceToHost, s), "D2H");
  check(cudaStreamSynchronize(s), "sync");
  // numBins = min(256, max(32, 2 * ceil(total / brightest))); binSize = total / numBins
  const double num_bins = js_min(256.0, js_max(32.0, 2.0 * std::ceil(th[0] / th[1])));
  if (num_bins != num_bins) { why = "environment has no radiance"; return 1; }
  const double bin_size = th[0] / num_bins;
  const uint32_t max_bins = 1024;
  DevBuf<int2> bins(max_bins);
  k_env_bins<<<1, 32, 0, s>>>(rad.p, vals.p, n, bin_size, bins.p, max_bins, nb.p);
  uint32_t nbh = 0;
  check(cudaMemcpyAsync(&nbh, nb.p, 4, cudaMemcpyDeviceToHost, s), "D2H");
  check(cudaStreamSynchronize(s), "sync");
  if (nbh < 2) { why = "environment yields a single luminance bin"; return 1; }
  if (nbh > max_bins) { why = "too many luminance bins"; return 1; }
  coords_out.alloc(n);
  pdf_out.alloc(n);
  k_env_pdf<<<(n + 255) / 256, 256, 0, s>>>(vals.p, n, w, bins.p, nbh, coords_out.p, pdf_out.p);
  check(cudaGetLastError(), "env pdf");
  bins_out.alloc(nbh);
  check(cudaMemcpyAsync(bins_out.p, bins.p, (size_t)nbh * 8, cudaMemcpyDeviceToDevice, s), "D2D");
  check(cudaStreamSynchronize(s), "sync");
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
