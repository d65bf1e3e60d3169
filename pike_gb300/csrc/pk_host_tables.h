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

// Environment sampling by an alias table (form (1)'s alternative to the
// reference's equal-mass luminance histogram, env_sampler.js:74-157; no
// reference counterpart).  Texel k is drawn with probability L_k / sum L,
// L = env_sampler.js's radiance 2^(a-128) * luma(rgb) / 255, by Vose's
// method (M. D. Vose, "A linear algorithm for generating random numbers with
// a given distribution", IEEE TSE 17(9), 1991) on FP64 probabilities
// normalised by a compensated FP64 sum.  table2: per texel {keep threshold,
// alias}: a lookup draws texel i uniformly and keeps it when the next 32-bit
// random number r < threshold (threshold 0xffffffff: always), else takes
// alias.  pdf: the r32f texture of the reference's layout (texel x + w*y)
// holding the table's exact selection probability (recomputed in FP64 from
// the quantised thresholds) times N / (2 pi^2), the same unit as the
// histogram's pdf.  Returns false (with a reason) for a black environment.
bool build_env_alias(const uint8_t* rgbe, uint32_t w, uint32_t h, std::vector<uint32_t>& table2,
                     std::vector<float>& pdf, std::string& why);

}  // namespace pk
