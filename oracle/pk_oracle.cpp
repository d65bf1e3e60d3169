// pk_oracle.cpp -- C entry points of the CPU oracle (liboracle.so).
//
// TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the CPU
// baseline legs of bench.py load this library, and only as the checker or as
// the timed CPU restatement; the product (pike_gb300/, libpike.so) never does.
//
// Parity unpinned: the reference (JavaScript + WGSL on WebGPU) has no tests,
// no fixtures and cannot run here, so this restatement of its source is the
// definition that golden vectors are generated from.  See om_build.h and
// om_render.h for the reference lines each part follows.
#include <cstdio>
#include <cstring>
#include <exception>
#include <string>

#include "om_build.h"
#include "om_render.h"
#include "om_render_f64.h"
#include "om_diff.h"
#include "om_wide.h"

using namespace om;

static thread_local std::string g_err;

extern "C" {

const char* or_last_error(void) { return g_err.c_str(); }

// Row S: flatten n vertices (scene.js:456-470) with transform {scale, translate}.
int or_flatten(const double* pos3, const double* nrm3, const double* tan4, const double* uv2, size_t n,
               double scale_, const double* translate3, double* pos_out3, uint32_t* attr_out4) {
  for (size_t i = 0; i < n; i++) {
    FlatVertex fv = flatten_vertex(pos3 + 3 * i, nrm3 + 3 * i, tan4 + 4 * i, uv2 + 2 * i, scale_, translate3);
    for (int k = 0; k < 3; k++) pos_out3[3 * i + k] = fv.pos[k];
    attr_out4[4 * i + 0] = fv.tangent;
    attr_out4[4 * i + 1] = fv.bitangent;
    attr_out4[4 * i + 2] = fv.normal;
    attr_out4[4 * i + 3] = fv.uv;
  }
  return 0;
}

// pk_scene_flatten_tbn: final positions, rotated normal/tangent, bitangent sources.
int or_flatten_tbn(const double* pos3, const double* nrm3, const double* tan4, const double* bn3, const double* bt4,
                   const double* uv2, size_t n, double* pos_out3, uint32_t* attr_out4) {
  const double zero[3] = {0.0, 0.0, 0.0};
  for (size_t i = 0; i < n; i++) {
    FlatVertex fv = flatten_vertex(pos3 + 3 * i, nrm3 + 3 * i, tan4 + 4 * i, uv2 + 2 * i, 1.0, zero, bn3 + 3 * i,
                                   bt4 + 4 * i);
    for (int k = 0; k < 3; k++) pos_out3[3 * i + k] = fv.pos[k];
    attr_out4[4 * i + 0] = fv.tangent;
    attr_out4[4 * i + 1] = fv.bitangent;
    attr_out4[4 * i + 2] = fv.normal;
    attr_out4[4 * i + 3] = fv.uv;
  }
  return 0;
}

// Row M: materials {r,g,b,a, roughness, metallic, er,eg,eb} -> index table + 1x1 layers.
int or_materials(const double* mats9, size_t n_mats, int32_t* index_out4, uint8_t* layers_out,
                 size_t max_layers, size_t* n_layers_out) {
  MaterialTable t;
  for (size_t i = 0; i < n_mats; i++) t.add_material(mats9 + 9 * i);
  size_t nl = t.layers.size() / 4;
  *n_layers_out = nl;
  if (nl > max_layers) { g_err = "or_materials: layer buffer too small"; return 1; }
  std::memcpy(index_out4, t.index4.data(), t.index4.size() * 4);
  std::memcpy(layers_out, t.layers.data(), t.layers.size());
  return 0;
}

struct OrBVH { BVHBuild build; PackedBVH packed; std::vector<double> pos; std::vector<int32_t> tri4; };

void* or_bvh_build(const double* pos3, size_t n_verts, const int32_t* tri4, size_t n_tris) {
  try {
    OrBVH* b = new OrBVH();
    b->build = build_bvh(pos3, tri4, n_tris);
    b->packed = pack_bvh(b->build, pos3, n_verts, tri4);
    b->pos.assign(pos3, pos3 + 3 * n_verts);
    b->tri4.assign(tri4, tri4 + 4 * n_tris);
    return b;
  } catch (std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}
void or_bvh_free(void* h) { delete (OrBVH*)h; }
// info: n_nodes, n_leaf_tris, max_depth, largest_leaf
void or_bvh_info(void* h, uint64_t* info4) {
  OrBVH* b = (OrBVH*)h;
  info4[0] = b->packed.nodes5.size() / 5;
  info4[1] = b->packed.tri4.size() / 4;
  info4[2] = (uint64_t)b->build.max_depth;
  info4[3] = b->build.largest_leaf;
}
// norm7: root_min[3], root_max[3] are not returned; center[3], scale, and root bounds
void or_bvh_copy(void* h, int32_t* nodes5, int32_t* tri4, float* verts4, double* norm10) {
  OrBVH* b = (OrBVH*)h;
  std::memcpy(nodes5, b->packed.nodes5.data(), b->packed.nodes5.size() * 4);
  std::memcpy(tri4, b->packed.tri4.data(), b->packed.tri4.size() * 4);
  std::memcpy(verts4, b->packed.verts4.data(), b->packed.verts4.size() * 4);
  for (int i = 0; i < 3; i++) {
    norm10[i] = b->packed.center[i];
    norm10[4 + i] = b->packed.root_min[i];
    norm10[7 + i] = b->packed.root_max[i];
  }
  norm10[3] = b->packed.scale;
}

// Raycaster.cast of n rays (6 doubles each: origin, dir in the normalised frame).
void or_bvh_cast(void* h, const double* rays6, size_t n, double* t_out) {
  OrBVH* b = (OrBVH*)h;
  Raycaster rc{b->build, b->pos.data(), b->tri4.data(), {b->packed.center[0], b->packed.center[1], b->packed.center[2]},
               b->packed.scale, {0, 0, 0}, {0, 0, 0}};
  for (size_t i = 0; i < n; i++) {
    for (int k = 0; k < 3; k++) { rc.o[k] = rays6[6 * i + k]; rc.d[k] = rays6[6 * i + 3 + k]; }
    t_out[i] = rc.traverse(0, Raycaster::MAXT);
  }
}

void* or_env_build(const uint8_t* rgbe, uint32_t w, uint32_t h) {
  try {
    return new EnvTables(build_env(rgbe, w, h));
  } catch (std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}
void* or_env_build_f32(const float* rgb, uint32_t w, uint32_t h) {
  try {
    return new EnvTables(build_env_f32(rgb, w, h));
  } catch (std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}
void or_env_free(void* h) { delete (EnvTables*)h; }
size_t or_env_num_bins(void* h) { return ((EnvTables*)h)->bins2.size() / 2; }
void or_env_copy(void* h, int32_t* bins2, int32_t* coords2, float* pdf, double* total_brightest) {
  EnvTables* e = (EnvTables*)h;
  std::memcpy(bins2, e->bins2.data(), e->bins2.size() * 4);
  std::memcpy(coords2, e->coords2.data(), e->coords2.size() * 4);
  std::memcpy(pdf, e->pdf.data(), e->pdf.size() * 4);
  total_brightest[0] = e->total;
  total_brightest[1] = e->brightest;
}

// ---------------- renderer ----------------
void* or_renderer_new(uint32_t w, uint32_t h, uint32_t batch, int nthreads) {
  Renderer* r = new Renderer();
  r->nthreads = nthreads < 1 ? 1 : nthreads;
  r->configure(w, h, batch);
  return r;
}
void or_renderer_free(void* p) { delete (Renderer*)p; }
void or_set_threads(void* p, int n) { ((Renderer*)p)->nthreads = n < 1 ? 1 : n; }

int or_set_scene(void* p, const int32_t* nodes5, size_t n_nodes, const int32_t* tri4, size_t n_tris,
                 const float* verts4, size_t n_verts, const uint32_t* attrs4, const int32_t* mat4, size_t n_mats,
                 const uint8_t* layers, size_t n_layers) {
  Renderer* r = (Renderer*)p;
  r->nodes5.assign(nodes5, nodes5 + 5 * n_nodes);
  r->tri4.assign(tri4, tri4 + 4 * n_tris);
  r->verts4.assign(verts4, verts4 + 4 * n_verts);
  r->attrs4.assign(attrs4, attrs4 + 4 * n_verts);
  r->mat4.assign(mat4, mat4 + 4 * n_mats);
  r->layers.assign(layers, layers + 4 * n_layers);
  r->atlas_res = 1;
  return 0;
}
// Replace the 1x1 layers with res x res rgba8 atlas layers.
int or_set_atlas(void* p, const uint8_t* layers, uint32_t res, size_t n_layers) {
  Renderer* r = (Renderer*)p;
  r->layers.assign(layers, layers + 4 * (size_t)res * res * n_layers);
  r->atlas_res = (int32_t)res;
  return 0;
}
int or_set_env(void* p, const uint8_t* rgbe, uint32_t w, uint32_t h, const int32_t* bins2, size_t nb,
               const int32_t* coords2, const float* pdf) {
  Renderer* r = (Renderer*)p;
  r->env_w = w; r->env_h = h;
  const size_t N = (size_t)w * h;
  r->env_rgbe.assign(rgbe, rgbe + 4 * N);
  r->env_bins2.assign(bins2, bins2 + 2 * nb);
  r->env_coords2.assign(coords2, coords2 + 2 * N);
  r->env_pdf.assign(pdf, pdf + N);
  r->env_alias2.clear();  // a new environment samples by its histogram
  r->sample_env_light = true;
  return 0;
}
// cam15: pos[3], dir[3], dims_mask(u32 bits), fov, focal_depth, aperture, distortion, bokeh, offset(u32 bits)
void or_set_camera(void* p, const void* cam15) { std::memcpy(&((Renderer*)p)->cam, cam15, sizeof(CameraState)); }
void or_set_render_state(void* p, int32_t samples, float env_theta) {
  Renderer* r = (Renderer*)p;
  r->samples = samples;
  r->env_theta = env_theta;
}
void or_set_post(void* p, float exposure, float saturation) {
  Renderer* r = (Renderer*)p;
  r->exposure = exposure;
  r->saturation = saturation;
}
void or_begin_frame(void* p) { ((Renderer*)p)->begin_frame(); }
// RenderState.clearColorBuffer / clearNumHitsAndMisses / clearNumRays (camera_pass.js:66-77)
void or_clear_color(void* p) { Renderer* r = (Renderer*)p; std::fill(r->color.begin(), r->color.end(), 0.0f); }
void or_clear_hits_misses(void* p) { Renderer* r = (Renderer*)p; r->num_hits = 0; r->num_misses = 0; }
void or_clear_rays(void* p) { Renderer* r = (Renderer*)p; r->num_rays = 0; r->num_shadow = 0; }
void or_camera(void* p) { ((Renderer*)p)->pass_camera(); }
void or_trace(void* p) { ((Renderer*)p)->pass_trace(); }
void or_shade_hit(void* p) { ((Renderer*)p)->pass_shade_hit(); }
void or_trace_shadow(void* p) { ((Renderer*)p)->pass_trace_shadow(); }
void or_shade_miss(void* p) { ((Renderer*)p)->pass_shade_miss(); }
void or_accumulate(void* p) { ((Renderer*)p)->pass_accumulate(); }
void or_postprocess(void* p) { ((Renderer*)p)->pass_postprocess(); }
void or_tick(void* p, uint32_t bounces) { ((Renderer*)p)->tick(bounces); }
void or_tick_batch(void* p, uint32_t bounces) { ((Renderer*)p)->tick_batch(bounces); }

// samples, num_hits, num_misses, num_rays, num_shadow, overflow
void or_counters(void* p, uint32_t* out6) {
  Renderer* r = (Renderer*)p;
  out6[0] = (uint32_t)r->samples; out6[1] = r->num_hits; out6[2] = r->num_misses;
  out6[3] = r->num_rays; out6[4] = r->num_shadow; out6[5] = r->overflow;
}
size_t or_shadow_offset(void* p) { return ((Renderer*)p)->shadow_offset(); }
// 12 floats per ray in the WGSL DeferredRay layout (48 B): origin, pad, dir, pad, throughput.
static void put_ray(const DeferredRay& r, float* o) {
  o[0] = r.o[0]; o[1] = r.o[1]; o[2] = r.o[2]; o[3] = 0.0f;
  o[4] = r.d[0]; o[5] = r.d[1]; o[6] = r.d[2]; o[7] = 0.0f;
  o[8] = r.tp[0]; o[9] = r.tp[1]; o[10] = r.tp[2]; o[11] = r.tp[3];
}
void or_read_rays(void* p, size_t first, size_t count, float* out12) {
  Renderer* r = (Renderer*)p;
  for (size_t i = 0; i < count; i++) put_ray(r->ray_buffer[first + i], out12 + 12 * i);
}
void or_read_misses(void* p, size_t count, float* out12) {
  Renderer* r = (Renderer*)p;
  for (size_t i = 0; i < count; i++) put_ray(r->miss_buffer[i], out12 + 12 * i);
}
// 16 words per hit: t, index, bary, 0, ray[12]
void or_read_hits(void* p, size_t count, uint32_t* out16) {
  Renderer* r = (Renderer*)p;
  for (size_t i = 0; i < count; i++) {
    const Hit& h = r->hit_buffer[i];
    out16[16 * i + 0] = f2u(h.t);
    out16[16 * i + 1] = (uint32_t)h.index;
    out16[16 * i + 2] = h.bary;
    out16[16 * i + 3] = 0;
    put_ray(h.ray, (float*)(out16 + 16 * i + 4));
  }
}
void or_read_color(void* p, float* out) { Renderer* r = (Renderer*)p; std::memcpy(out, r->color.data(), r->color.size() * 4); }
void or_read_accum(void* p, float* out) { Renderer* r = (Renderer*)p; std::memcpy(out, r->temp.data(), r->temp.size() * 4); }
void or_read_display(void* p, float* out, uint8_t* out8) {
  Renderer* r = (Renderer*)p;
  std::memcpy(out, r->display.data(), r->display.size() * 4);
  std::memcpy(out8, r->display8.data(), r->display8.size());
}
// trace: fetch, tests, rays, max_stack; shadow: fetch, tests, rays, max_stack
void or_stats(void* p, uint64_t* out8) {
  Renderer* r = (Renderer*)p;
  out8[0] = r->trace_stats.node_fetch; out8[1] = r->trace_stats.tri_tests;
  out8[2] = r->trace_stats.rays; out8[3] = r->trace_stats.max_stack;
  out8[4] = r->shadow_stats.node_fetch; out8[5] = r->shadow_stats.tri_tests;
  out8[6] = r->shadow_stats.rays; out8[7] = r->shadow_stats.max_stack;
}
void or_reset_stats(void* p) {
  Renderer* r = (Renderer*)p;
  r->trace_stats = Stats();
  r->shadow_stats = Stats();
}

// Trace a caller-supplied ray list against the current scene (no queues):
// out4 per ray = {t bits, index, bary, node fetches}.
void or_trace_rays(void* p, const float* rays8, size_t n, int any_hit, uint32_t* out4) {
  Renderer* r = (Renderer*)p;
  parallel_for(n, r->nthreads, [&](size_t b, size_t e, int) {
    std::vector<int32_t> stack;
    for (size_t i = b; i < e; i++) {
      const float* q = rays8 + 8 * i;
      Renderer::TravResult t = any_hit ? r->intersect<true>(v3(q[0], q[1], q[2]), v3(q[4], q[5], q[6]), stack)
                                       : r->intersect<false>(v3(q[0], q[1], q[2]), v3(q[4], q[5], q[6]), stack);
      out4[4 * i + 0] = f2u(t.t);
      out4[4 * i + 1] = (uint32_t)t.index;
      out4[4 * i + 2] = t.bary;
      out4[4 * i + 3] = t.fetch;
    }
  });
}

// Brute-force ray queries over every leaf-ordered triangle with the
// reference's triangle test: closest = minimum of (t, slot), any = whether
// some triangle is accepted.  out4 = {t bits, slot, bary, 0} (any: t and slot
// of the lowest accepted slot).  The canonical answer an order-independent
// traversal must reproduce.
void or_brute_rays(void* p, const float* rays8, size_t n, int any_hit, uint32_t* out4) {
  Renderer* r = (Renderer*)p;
  parallel_for(n, r->nthreads, [&](size_t b, size_t e, int) {
    for (size_t i = b; i < e; i++) {
      const float* q = rays8 + 8 * i;
      const V3 o = v3(q[0], q[1], q[2]), d = v3(q[4], q[5], q[6]);
      const Renderer::TravResult t = any_hit ? r->brute<true>(o, d) : r->brute<false>(o, d);
      out4[4 * i + 0] = f2u(t.t);
      out4[4 * i + 1] = (uint32_t)t.index;
      out4[4 * i + 2] = t.bary;
      out4[4 * i + 3] = 0u;
    }
  });
}
void or_set_canonical(void* p, int on) { ((Renderer*)p)->canonical = on != 0; }

// FP64 companion (om_render64.h): which = 0 the FP64 accumulation
// (accumulate.wgsl in double), 1 the mean and 2 the sum of squared deviations
// of the per-frame FP64 colours since or_set_track64; W*H*4 doubles.
// sampleEnv's direction for texel (cx, cy) and envPdf's texel for it.
void or_env_roundtrip(void* p, int32_t cx, int32_t cy, float* dir3, int32_t* idx2) {
  ((Renderer*)p)->env_roundtrip(cx, cy, dir3, idx2, idx2 + 1);
}
// Alias-table environment sampling (table2: W*H {threshold, alias}; pdf: W*H
// r32f replacing the histogram's pdf texture); n = 0 restores nothing (set a
// new environment to return to the histogram).
void or_set_env_alias(void* p, const uint32_t* table2, const float* pdf, size_t n) {
  Renderer* r = (Renderer*)p;
  r->env_alias2.assign(table2, table2 + 2 * n);
  r->env_pdf.assign(pdf, pdf + n);
}
// on: 0 off, 1 FP64 evaluation, 2 FP64 evaluation with the FP32 texel choices
void or_set_track64(void* p, int on) { ((Renderer*)p)->set_track64(on != 0, on == 2); }
uint64_t or_frames64(void* p) { return ((Renderer*)p)->frames64; }
int or_read64(void* p, int which, double* out) {
  Renderer* r = (Renderer*)p;
  const std::vector<double>* v = which == 0 ? &r->accum64 : which == 1 ? &r->mean64 : which == 2 ? &r->m2_64 : nullptr;
  if (!v || !r->track64) return 1;
  std::memcpy(out, v->data(), v->size() * sizeof(double));
  return 0;
}

// The reference path rendered in binary64 end to end (om_render_f64.h), on
// the scene, environment, camera and sample index of a configured renderer.
void* or_render64_new(void* r) { return new Render64(*(Renderer*)r); }
void or_render64_free(void* p) { delete (Render64*)p; }
void or_render64_tick(void* p, uint32_t bounces) { ((Render64*)p)->tick(bounces); }
uint64_t or_render64_frames(void* p) { return ((Render64*)p)->frames; }
// which = 0 the running mean, 1 the mean and 2 the sum of squared deviations
// of the per-frame colours, 3 the last frame's colour; W*H*4 doubles.
int or_render64_read(void* p, int which, double* out) {
  Render64* r = (Render64*)p;
  const std::vector<double>* v = which == 0 ? &r->accum : which == 1 ? &r->mean : which == 2 ? &r->m2
                               : which == 3 ? &r->color : nullptr;
  if (!v) return 1;
  std::memcpy(out, v->data(), v->size() * sizeof(double));
  return 0;
}

// Differentiable renderer (pk_diff.cu) in binary64: image and gradient.  The
// renderer supplies scene, BVH, atlas, camera and env rotation; `tables` is an
// or_env_build_f32 handle of the sampling environment.
static DiffScene diff_scene(void* p, uint32_t W, uint32_t H, const double* albedo, const double* rough,
                            const double* rough0, const double* metal, uint32_t n_mats, const double* env,
                            uint32_t env_w, uint32_t env_h, void* tables, uint32_t spp, uint32_t depth,
                            uint32_t sample_base) {
  DiffScene S;
  S.r = (Renderer*)p;
  S.W = W; S.H = H;
  S.albedo = albedo; S.rough = rough; S.rough0 = rough0; S.metal = metal; S.n_mats = n_mats;
  S.env = env; S.env_w = (int)env_w; S.env_h = (int)env_h;
  S.tab = (const EnvTables*)tables;
  S.spp = (int)spp; S.depth = (int)depth; S.sample_base = sample_base;
  return S;
}
uint64_t or_diff_render(void* p, uint32_t W, uint32_t H, const double* albedo, const double* rough,
                        const double* rough0, const double* metal, uint32_t n_mats, const double* env, uint32_t env_w,
                        uint32_t env_h, void* tables, uint32_t spp, uint32_t depth, uint32_t sample_base,
                        double* image3) {
  const DiffScene S =
      diff_scene(p, W, H, albedo, rough, rough0, metal, n_mats, env, env_w, env_h, tables, spp, depth, sample_base);
  return diff_render(S, image3, ((Renderer*)p)->nthreads);
}
uint64_t or_diff_render32(void* p, uint32_t W, uint32_t H, const double* albedo, const double* rough,
                          const double* rough0, const double* metal, uint32_t n_mats, const double* env,
                          uint32_t env_w, uint32_t env_h, void* tables, uint32_t spp, uint32_t depth,
                          uint32_t sample_base, uint32_t y0, uint32_t y1, float* image4, int64_t trace_pixel) {
  const DiffScene S =
      diff_scene(p, W, H, albedo, rough, rough0, metal, n_mats, env, env_w, env_h, tables, spp, depth, sample_base);
  return diff_render32(S, y0, y1, image4, ((Renderer*)p)->nthreads, trace_pixel);
}
void or_diff_grad(void* p, uint32_t W, uint32_t H, const double* albedo, const double* rough, const double* rough0,
                  const double* metal, uint32_t n_mats, const double* env, uint32_t env_w, uint32_t env_h,
                  void* tables, uint32_t spp, uint32_t depth, uint32_t sample_base, const double* dimage3,
                  double* g_albedo, double* g_rough, double* g_env) {
  const DiffScene S =
      diff_scene(p, W, H, albedo, rough, rough0, metal, n_mats, env, env_w, env_h, tables, spp, depth, sample_base);
  diff_gradient(S, dimage3, g_albedo, g_rough, g_env, ((Renderer*)p)->nthreads);
}

// Form (1)'s builders restated on the host (om_wide.h).
void* or_wide_build(const int32_t* nodes5, uint32_t n_nodes, const int32_t* tri4, uint32_t n_tris,
                    const float* verts4, uint32_t n_verts) {
  om_wide::WideHost* w = new om_wide::WideHost();
  std::string why;
  if (om_wide::build_wide_bvh(nodes5, n_nodes, tri4, n_tris, verts4, n_verts, *w, why)) {
    g_err = why;
    delete w;
    return nullptr;
  }
  return w;
}
uint32_t or_wide_nodes(void* h) { return ((om_wide::WideHost*)h)->n_nodes; }
uint32_t or_wide_depth(void* h) { return ((om_wide::WideHost*)h)->max_depth; }
void or_wide_copy(void* h, float* nodes20, float* tris12) {
  const om_wide::WideHost* w = (const om_wide::WideHost*)h;
  std::memcpy(nodes20, w->nodes.data(), w->nodes.size() * 4);
  std::memcpy(tris12, w->tris.data(), w->tris.size() * 4);
}
void or_wide_free(void* h) { delete (om_wide::WideHost*)h; }
// records16: 16 floats per inner node (the caller sizes it), tris12: 12 per triangle.
int or_exact_build(const int32_t* nodes5, uint32_t n_nodes, const int32_t* tri4, uint32_t n_tris,
                   const float* verts4, uint32_t n_verts, float* records16, float* tris12, int32_t* root) {
  std::vector<float> rec, tris;
  std::string why;
  if (om_wide::build_exact_binary(nodes5, n_nodes, tri4, n_tris, verts4, n_verts, rec, tris, *root, why)) {
    g_err = why;
    return 1;
  }
  std::memcpy(records16, rec.data(), rec.size() * 4);
  std::memcpy(tris12, tris.data(), tris.size() * 4);
  return 0;
}

// Elementwise math probes for parity of the built-in definitions:
// fn 0 sin, 1 cos, 2 tan, 3 atan2(x, y), 4 acos, 5 exp2, 6 log2, 7 pow(x, y), 8 snorm16 decode.
void or_math(int fn, const float* x, const float* y, float* out, size_t n) {
  for (size_t i = 0; i < n; i++) {
    float a = x[i], b = y ? y[i] : 0.0f;
    float r = 0.0f;
    switch (fn) {
      case 0: r = sin_(a); break;
      case 1: r = cos_(a); break;
      case 2: r = tan_(a); break;
      case 3: r = atan2_(a, b); break;
      case 4: r = acos_(a); break;
      case 5: r = exp2_(a); break;
      case 6: r = log2_(a); break;
      case 7: r = pow_(a, b); break;
      case 8: r = snorm16((int32_t)f2u(a)); break;  // unpack2x16snorm of an integer held in the bits of a
      default: r = NAN;
    }
    out[i] = r;
  }
}

// Jarzynski-Olano hash stream: n outputs from seed.
void or_hash_stream(uint32_t seed, uint32_t* out, size_t n) {
  Hash h;
  h.seed = seed;
  for (size_t i = 0; i < n; i++) out[i] = h.hash();
}

}  // extern "C"
