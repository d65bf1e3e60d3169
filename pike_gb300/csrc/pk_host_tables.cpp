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

}  // namespace pk
