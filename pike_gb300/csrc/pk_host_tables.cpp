// pk_host_tables.cpp -- material layers (row M), built on the host once per
// scene like the reference does (a few hundred entries at most).
#include "pk_host_tables.h"

#include <algorithm>
#include <cmath>

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

bool build_env_alias(const uint8_t* rgbe, uint32_t w, uint32_t h, std::vector<uint32_t>& table2,
                     std::vector<float>& pdf, std::string& why) {
  const size_t N = (size_t)w * h;
  std::vector<double> q(N);
  double sum = 0.0, comp = 0.0;  // Neumaier's compensated sum
  for (size_t i = 0; i < N; i++) {
    const uint8_t* c = rgbe + 4 * i;
    const double r = std::ldexp(1.0, (int)c[3] - 128) * (0.2126 * c[0] + 0.7152 * c[1] + 0.0722 * c[2]) / 255.0;
    q[i] = r;
    const double t = sum + r;
    comp += std::fabs(sum) >= std::fabs(r) ? (sum - t) + r : (r - t) + sum;
    sum = t;
  }
  sum += comp;
  if (!(sum > 0.0) || !std::isfinite(sum)) {
    why = "black or non-finite environment";
    return false;
  }
  const double scale = (double)N / sum;
  std::vector<uint32_t> small, large;
  small.reserve(N);
  large.reserve(N);
  for (size_t i = 0; i < N; i++) {
    q[i] *= scale;
    (q[i] < 1.0 ? small : large).push_back((uint32_t)i);
  }
  std::vector<double> prob(N, 1.0);
  std::vector<uint32_t> alias(N);
  for (size_t i = 0; i < N; i++) alias[i] = (uint32_t)i;
  while (!small.empty() && !large.empty()) {
    const uint32_t s = small.back(), l = large.back();
    small.pop_back();
    large.pop_back();
    prob[s] = q[s];
    alias[s] = l;
    q[l] = (q[l] + q[s]) - 1.0;
    (q[l] < 1.0 ? small : large).push_back(l);
  }
  // what remains in either list has probability 1 up to rounding
  table2.assign(2 * N, 0u);
  std::vector<double> keep(N);
  for (size_t i = 0; i < N; i++) {
    uint32_t thr;
    if (prob[i] >= 1.0) {
      thr = 0xffffffffu;
      keep[i] = 1.0;
    } else {
      const double t = std::floor(prob[i] * 4294967296.0);
      thr = (uint32_t)std::min(t, 4294967294.0);
      keep[i] = (double)thr / 4294967296.0;
    }
    table2[2 * i] = thr;
    table2[2 * i + 1] = alias[i];
  }
  // exact selection probability of each texel under the quantised table
  std::vector<double> p(N, 0.0);
  for (size_t i = 0; i < N; i++) {
    p[i] += keep[i];
    if (keep[i] < 1.0) p[alias[i]] += 1.0 - keep[i];
  }
  pdf.assign(N, 0.0f);
  // p[k] / N is texel k's probability, so p[k] is its density in (u, v);
  // / (2 pi^2) gives the histogram pdf's unit (solid angle once / sin(phi))
  const double unit = 1.0 / (2.0 * M_PI * M_PI);
  for (size_t i = 0; i < N; i++) pdf[i] = (float)(p[i] * unit);
  return true;
}

}  // namespace pk
