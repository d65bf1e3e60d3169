// pk_host_tables.h -- small host-side tables built once at scene load.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace pk {

// Scene._createSceneMaterial (scene.js:43-70) for untextured materials with
// TexturePacker.addColor de-duplication (texture_packer.js:99-108) and one
// 1x1 rgba8 layer per distinct colour, drawn by gl.clearColor(r, g, b, 1) and
// read back (texture_packer.js:274-279): unorm8 = floor(clamp(c) * 255 + 0.5).
// mats9: base r,g,b,a, roughness, metallic, emissive r,g,b per material.
void build_material_layers(const double* mats9, uint32_t n_mats, std::vector<int32_t>& index4,
                           std::vector<uint8_t>& layers_rgba8);

// EnvironmentGenerator tables (env_sampler.js:43-157).
struct EnvHostTables {
  std::vector<int32_t> bins2;
  std::vector<int32_t> coords2;
  std::vector<float> pdf;
};
int build_env_tables(const uint8_t* rgbe, uint32_t w, uint32_t h, EnvHostTables& out, std::string& why);

}  // namespace pk
