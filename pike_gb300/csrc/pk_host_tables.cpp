// pk_host_tables.cpp -- material layers (row M) and environment importance
// tables (row E), built on the host once per scene like the reference does.
// Compiled with -ffp-contract=off: the double arithmetic below must round
// exactly as JavaScript's does.
#include "pk_host_tables.h"

#include <algorithm>
#include <cmath>
#include <numeric>

namespace pk {

namespace {

uint8_t unorm8(double c) {
  const double x = c != c ? 0.0 : std::min(1.0, std::max(0.0, c));
  return (uint8_t)std::floor(x * 255.0 + 0.5);
}

struct ColorKeys {
  std::vector<std::vector<double>> keys;
  std::vector<uint8_t>* layers;
  // TexturePacker.addColor: key = color.join(' '); equal numbers give equal keys.
  int add(std::initializer_list<double> color) {
    std::vector<double> c(color);
    for (size_t i = 0; i < keys.size(); i++) {
      if (keys[i].size() != c.size()) continue;
      size_t k = 0;
      while (k < c.size() && keys[i][k] == c[k]) k++;
      if (k == c.size()) return (int)i;
    }
    keys.push_back(c);
    layers->push_back(unorm8(c[0]));
    layers->push_back(unorm8(c[1]));
    layers->push_back(unorm8(c[2]));
    layers->push_back(255);  // drawColor clears with alpha 1.0
    return (int)keys.size() - 1;
  }
};

// JavaScript Math.min / Math.max on numbers (NaN propagates).
double js_min(double a, double b) { return (a != a || b != b) ? NAN : (a < b ? a : (b < a ? b : (std::signbit(a) ? a : b))); }
double js_max(double a, double b) { return (a != a || b != b) ? NAN : (a > b ? a : (b > a ? b : (std::signbit(a) ? b : a))); }

}  // namespace

void build_material_layers(const double* mats9, uint32_t n_mats, std::vector<int32_t>& index4,
                           std::vector<uint8_t>& layers_rgba8) {
  ColorKeys keys;
  keys.layers = &layers_rgba8;
  index4.clear();
  layers_rgba8.clear();
  for (uint32_t m = 0; m < n_mats; m++) {
    const double* p = mats9 + 9 * (size_t)m;
    index4.push_back(keys.add({p[0], p[1], p[2], p[3]}));   // getBaseColor (4 components)
    index4.push_back(keys.add({0.0, p[4], p[5]}));          // getMetallicRoughness = [0, rough, metal]
    index4.push_back(keys.add({0.5, 0.5, 1.0}));            // default normal map colour
    index4.push_back(keys.add({p[6], p[7], p[8]}));         // getEmissive
  }
}

int build_env_tables(const uint8_t* rgbe, uint32_t w, uint32_t h, EnvHostTables& out, std::string& why) {
  const size_t N = (size_t)w * h;
  std::vector<double> rad(N);
  double total = 0.0, brightest = 0.0;
  // _sortPixels: row-major accumulation of _getRadiance = 2^(a-128) * luma / 255
  for (size_t i = 0; i < N; i++) {
    const uint8_t* c = rgbe + 4 * i;
    const double power = std::ldexp(1.0, (int)c[3] - 128);
    const double luma = 0.2126 * c[0] + 0.7152 * c[1] + 0.0722 * c[2];
    const double r = power * luma / 255.0;
    brightest = js_max(r, brightest);
    total += r;
    rad[i] = r;
  }
  // sort((a, b) => b.rad - a.rad): stable, descending radiance
  std::vector<int32_t> order(N);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return rad[a] > rad[b]; });
  const double num_bins = js_min(256.0, js_max(32.0, 2.0 * std::ceil(total / brightest)));
  if (num_bins != num_bins) { why = "environment has no radiance"; return 1; }
  const double bin_size = total / num_bins;
  out.bins2.clear();
  double current = 0.0;
  for (size_t i = 0; i < N; i++) {
    if (current >= bin_size) {
      const int32_t prev = out.bins2.empty() ? 0 : out.bins2.back();
      out.bins2.push_back(prev);
      out.bins2.push_back((int32_t)i);
      current = 0.0;
    }
    current += rad[order[i]];
  }
  if (out.bins2.empty()) { why = "environment yields a single luminance bin"; return 1; }
  const int32_t last = out.bins2.back();
  out.bins2.push_back(last);
  out.bins2.push_back((int32_t)N);
  out.coords2.resize(2 * N);
  for (size_t i = 0; i < N; i++) {
    out.coords2[2 * i] = order[i] % (int32_t)w;
    out.coords2[2 * i + 1] = order[i] / (int32_t)w;
  }
  out.pdf.assign(N, 0.0f);
  const size_t nb = out.bins2.size() / 2;
  const double sphere_pdf = 1.0 / (M_PI * M_PI * 2.0);
  for (size_t b = 0; b < nb; b++) {
    const int32_t h0 = out.bins2[2 * b], h1 = out.bins2[2 * b + 1];
    const double bin_pdf = 1.0 / (double)nb;
    const double coord_pdf = (double)N / (double)(h1 - h0);
    const double pdf = bin_pdf * coord_pdf * sphere_pdf;
    for (int32_t i = h0; i < h1; i++) out.pdf[order[i]] = (float)pdf;
  }
  return 0;
}

}  // namespace pk
