// pk_host_tables.h -- the material table, built on the host once per scene (as the reference does).
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

}  // namespace pk
