// pk_api.cu -- the C ABI of libpike.so (declared in include/pike.h): context,
// device memory, scene/material/BVH/env upload, pass sequencing and readback.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "../../include/pike.h"
#include "pk_bvh.h"
#include "pk_ctx.h"
#include "pk_wide.h"
#include "pk_host_tables.h"
#include "pk_internal.cuh"
#include "pk_render.h"
#include "pk_util.h"

using namespace pk;

namespace {

int fail(pk_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

// Orders the API stream after every frame still in flight and after the last
// asynchronous display read, so what follows on it sees their results and may
// overwrite what they read.
void join_frames(pk_ctx* c) {
  for (FrameSlot& s : c->slot)
    if (s.busy) {
      check(cudaStreamWaitEvent(c->stream, s.ev_done, 0), "cudaStreamWaitEvent");
      s.busy = false;
    }
  if (c->read_pending) check(cudaStreamWaitEvent(c->stream, c->ev_read, 0), "cudaStreamWaitEvent");
  c->read_pending = false;
  c->tail_pending = false;
}

// Brings slot 0's counters and camera up to the render state the host holds
// (pk_set_render_state, pk_set_camera, frames rendered since).
void apply_state(pk_ctx* c) {
  if (!c->state_dirty || !c->ctr.p) return;
  launch_set_state(c->stream, c->ctr.p, c->cam.p, c->samples_next, c->theta_next, c->cam_host, c->cam_set);
  check(cudaGetLastError(), "k_set_state");
  c->state_dirty = false;
}

template <bool JOIN, class F>
int guarded_impl(pk_ctx* c, F fn) {
  if (!c) return PK_ERR_ARG;
  try {
    check(cudaSetDevice(c->device), "cudaSetDevice");
    if (JOIN) {
      join_frames(c);
      apply_state(c);
    }
    return fn();
  } catch (CudaError& e) {
    return fail(c, PK_ERR_CUDA, e.what());
  } catch (std::exception& e) {
    return fail(c, PK_ERR_ARG, e.what());
  }
}
// Entry points that touch device state run after the frames in flight.
template <class F>
int guarded(pk_ctx* c, F fn) {
  return guarded_impl<true>(c, fn);
}
// Frame submission, render state and asynchronous reads order themselves.
template <class F>
int guarded_nojoin(pk_ctx* c, F fn) {
  return guarded_impl<false>(c, fn);
}

// Buffers of frame slot k, sized for the current configuration.
void alloc_slot(pk_ctx* c, int k) {
  FrameSlot& s = c->slot[k];
  s.drop_graph();
  if (!s.ctr.p) {
    s.ctr.alloc(1);
    check(cudaMemsetAsync(s.ctr.p, 0, sizeof(Counters), c->stream), "memset");
  }
  if (!s.cam.p) s.cam.alloc(1);
  for (int i = 0; i < 3; i++) {
    s.rq[0][i].alloc(c->cap);
    s.rq[1][i].alloc(c->cap);
    s.sq[i].alloc(c->cap);
  }
  s.hrec.alloc(c->cap);
  s.hflags.alloc(c->cap / 32 + 1);
  s.sflags.alloc(c->cap / 32 + 1);
  s.hit_list.alloc(c->cap);
  s.color.alloc(c->npix);
  s.tickets.alloc(4 * MAX_BOUNCES);
  s.tiles.alloc((size_t)MAX_BOUNCES * (2 * c->ct + c->st));
  check(cudaMemsetAsync(s.color.p, 0, s.color.bytes(), c->stream), "memset");
  check(cudaMemsetAsync(s.hflags.p, 0, s.hflags.bytes(), c->stream), "memset");
  check(cudaMemsetAsync(s.sflags.p, 0, s.sflags.bytes(), c->stream), "memset");
  check(cudaMemsetAsync(s.hit_list.p, 0, s.hit_list.bytes(), c->stream), "memset");
  check(cudaMemsetAsync(s.hrec.p, 0, s.hrec.bytes(), c->stream), "memset");
  check(cudaMemsetAsync(&s.ctr.p->num_hits, 0, 16, c->stream), "memset");
  s.cur = 0;
  s.cap = c->cap;
}

void release_slot(FrameSlot& s) {
  s.drop_graph();
  for (int i = 0; i < 3; i++) {
    s.rq[0][i].release();
    s.rq[1][i].release();
    s.sq[i].release();
  }
  s.hrec.release();
  s.hflags.release();
  s.sflags.release();
  s.hit_list.release();
  s.color.release();
  s.tickets.release();
  s.tiles.release();
  s.cap = 0;
}

template <class T>
void upload(DevBuf<T>& d, const void* host, size_t count, cudaStream_t s) {
  d.alloc(count);
  if (count) check(cudaMemcpyAsync(d.p, host, count * sizeof(T), cudaMemcpyHostToDevice, s), "H2D");
}

void require_config(pk_ctx* c) {
  if (!c->cap) throw std::runtime_error("pk_configure has not been called");
}
void require_render(pk_ctx* c) {
  require_config(c);
  if (!c->bvh_ready) throw std::runtime_error("no BVH: call pk_bvh_build or pk_bvh_upload");
  if (!c->n_mats || !c->n_layers) throw std::runtime_error("no materials: call pk_materials_set/upload");
  if (!c->attrs.p) throw std::runtime_error("no scene attributes: call pk_scene_flatten/upload");
  if (c->bvh_verts > c->n_verts) throw std::runtime_error("BVH vertices exceed the scene's vertex attributes");
  if (!c->cam_set) throw std::runtime_error("no camera: call pk_set_camera");
}

}  // namespace

extern "C" {

int pk_version(void) { return 10000; }

int pk_create(pk_ctx** out, int device) {
  if (!out) return PK_ERR_ARG;
  *out = nullptr;
  pk_ctx* c = new pk_ctx();
  c->device = device;
  int rc = guarded(c, [&]() {
    int n = 0;
    check(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
    if (device < 0 || device >= n) throw std::runtime_error("no such CUDA device");
    check(cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device), "attr");
    check(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    check(cudaStreamCreateWithFlags(&c->copy, cudaStreamNonBlocking), "cudaStreamCreate");
    for (cudaEvent_t* e : {&c->ev_api, &c->ev_tail, &c->ev_read})
      check(cudaEventCreateWithFlags(e, cudaEventDisableTiming), "cudaEventCreate");
    for (FrameSlot& s : c->slot) {
      check(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking), "cudaStreamCreate");
      check(cudaStreamCreateWithFlags(&s.side, cudaStreamNonBlocking), "cudaStreamCreate");
      for (cudaEvent_t* e : {&s.ev_shaded, &s.ev_shadow, &s.ev_done})
        check(cudaEventCreateWithFlags(e, cudaEventDisableTiming), "cudaEventCreate");
    }
    c->ctr.alloc(1);
    c->cam.alloc(1);
    c->cast_scratch = noalloc_scratch_address();
    check(cudaMemsetAsync(c->ctr.p, 0, sizeof(Counters), c->stream), "memset");
    check(cudaStreamSynchronize(c->stream), "sync");
    return PK_OK;
  });
  if (rc != PK_OK) {
    std::fprintf(stderr, "pk_create: %s\n", c->err.c_str());
    delete c;
    return rc;
  }
  *out = c;
  return PK_OK;
}

int pk_destroy(pk_ctx* c) {
  if (!c) return PK_ERR_ARG;
  cudaSetDevice(c->device);
  for (FrameSlot& s : c->slot) {
    if (s.stream) cudaStreamSynchronize(s.stream);
    if (s.side) cudaStreamSynchronize(s.side);
  }
  if (c->copy) cudaStreamSynchronize(c->copy);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (FrameSlot& s : c->slot) {
    s.drop_graph();
    for (cudaEvent_t e : {s.ev_shaded, s.ev_shadow, s.ev_done})
      if (e) cudaEventDestroy(e);
    if (s.side) cudaStreamDestroy(s.side);
    if (s.stream) cudaStreamDestroy(s.stream);
  }
  for (cudaEvent_t e : {c->ev_api, c->ev_tail, c->ev_read})
    if (e) cudaEventDestroy(e);
  if (c->copy) cudaStreamDestroy(c->copy);
  for (auto& p : c->events) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
  for (auto e : c->event_pool) cudaEventDestroy(e);
  if (c->t0) cudaEventDestroy(c->t0);
  if (c->t1) cudaEventDestroy(c->t1);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return PK_OK;
}

const char* pk_last_error(const pk_ctx* c) { return c ? c->err.c_str() : "null context"; }

int pk_configure(pk_ctx* c, uint32_t width, uint32_t height, uint32_t batch) {
  return guarded(c, [&]() {
    c->invalidate_graph();
    if (!width || !height || width > 0xffff || height > 0xffff) return fail(c, PK_ERR_ARG, "resolution out of range");
    if ((uint64_t)width * height >= (1ull << 28)) return fail(c, PK_ERR_ARG, "more than 2^28 pixels");
    if (!batch || batch > (1u << 28)) return fail(c, PK_ERR_ARG, "batch size out of range");
    c->W = width; c->H = height; c->B = batch;
    c->cap = (batch + 127u) / 128u * 128u;
    c->npix = width * height;
    if (c->kahan) {
      c->accum_sum.alloc(c->npix);
      c->accum_comp.alloc(c->npix);
    }
    c->ct = compact_tiles(c->cap);
    c->st = shade_tiles(c->cap);
    kernel_grids(c->sms, c->cap, &c->g_trace, &c->g_compact, &c->g_shade, &c->g_trace_wide);
    for (int i = 0; i < 3; i++) c->mq[i].alloc(2 * (size_t)c->cap);
    alloc_slot(c, 0);
    for (int k = 1; k < MAX_IN_FLIGHT; k++) release_slot(c->slot[k]);  // sized again on first use
    c->next_slot = c->last_slot = 0;
    c->accum.alloc(c->npix);
    c->display.alloc(c->npix);
    c->display8.alloc(c->npix);
    check(cudaMemsetAsync(c->accum.p, 0, c->accum.bytes(), c->stream), "memset");
    check(cudaMemsetAsync(c->display.p, 0, c->display.bytes(), c->stream), "memset");
    check(cudaMemsetAsync(c->display8.p, 0, c->display8.bytes(), c->stream), "memset");
    check(cudaStreamSynchronize(c->stream), "sync");
    return PK_OK;
  });
}

// ---------------- scene ----------------
namespace {
int flatten_impl(pk_ctx* c, const double* pos3, const double* nrm3, const double* tan4, const double* bn3,
                 const double* bt4, const double* uv2, uint32_t n_verts, const int32_t* tri4, uint32_t n_tris,
                 double scale, const double translate[3]) {
  return guarded(c, [&]() {
    if (!pos3 || !nrm3 || !tan4 || !uv2 || !tri4 || !n_verts || !n_tris) return fail(c, PK_ERR_ARG, "empty scene");
    for (uint32_t t = 0; t < n_tris; t++)
      for (int k = 0; k < 3; k++)
        if (tri4[4 * t + k] < 0 || (uint32_t)tri4[4 * t + k] >= n_verts) return fail(c, PK_ERR_ARG, "vertex index out of range");
    DevBuf<double> p, n, t, u, bn, bt;
    upload(p, pos3, 3 * (size_t)n_verts, c->stream);
    upload(n, nrm3, 3 * (size_t)n_verts, c->stream);
    upload(t, tan4, 4 * (size_t)n_verts, c->stream);
    upload(u, uv2, 2 * (size_t)n_verts, c->stream);
    if (bn3) upload(bn, bn3, 3 * (size_t)n_verts, c->stream);
    if (bt4) upload(bt, bt4, 4 * (size_t)n_verts, c->stream);
    c->pos.alloc(3 * (size_t)n_verts);
    c->attrs.alloc(n_verts);
    const double tr[3] = {translate ? translate[0] : 0.0, translate ? translate[1] : 0.0, translate ? translate[2] : 0.0};
    launch_flatten(c->stream, p.p, n.p, t.p, bn3 ? bn.p : n.p, bt4 ? bt.p : t.p, u.p, n_verts, scale, tr[0], tr[1],
                   tr[2], c->pos.p, c->attrs.p);
    check(cudaGetLastError(), "k_flatten");
    upload(c->tri4, tri4, n_tris, c->stream);
    check(cudaStreamSynchronize(c->stream), "sync");
    c->n_verts = n_verts;
    c->n_tris = n_tris;
    c->bvh_ready = false;
    c->invalidate_graph();
    return PK_OK;
  });
}
}  // namespace

int pk_scene_flatten(pk_ctx* c, const double* pos3, const double* nrm3, const double* tan4, const double* uv2,
                     uint32_t n_verts, const int32_t* tri4, uint32_t n_tris, double scale, const double translate[3]) {
  return flatten_impl(c, pos3, nrm3, tan4, nullptr, nullptr, uv2, n_verts, tri4, n_tris, scale, translate);
}

int pk_scene_flatten_tbn(pk_ctx* c, const double* pos3, const double* nrm3, const double* tan4, const double* bn3,
                         const double* bt4, const double* uv2, uint32_t n_verts, const int32_t* tri4, uint32_t n_tris) {
  if (c && (!bn3 || !bt4)) return fail(c, PK_ERR_ARG, "bitangent sources missing");
  const double zero[3] = {0.0, 0.0, 0.0};
  return flatten_impl(c, pos3, nrm3, tan4, bn3, bt4, uv2, n_verts, tri4, n_tris, 1.0, zero);
}

int pk_scene_upload(pk_ctx* c, const int32_t* tri4, uint32_t n_tris, const double* pos3, const uint32_t* attr4,
                    uint32_t n_verts) {
  return guarded(c, [&]() {
    if (!tri4 || !pos3 || !attr4 || !n_tris || !n_verts) return fail(c, PK_ERR_ARG, "empty scene");
    for (uint32_t t = 0; t < n_tris; t++)
      for (int k = 0; k < 3; k++)
        if (tri4[4 * t + k] < 0 || (uint32_t)tri4[4 * t + k] >= n_verts) return fail(c, PK_ERR_ARG, "vertex index out of range");
    upload(c->tri4, tri4, n_tris, c->stream);
    upload(c->pos, pos3, 3 * (size_t)n_verts, c->stream);
    upload(c->attrs, attr4, n_verts, c->stream);
    check(cudaStreamSynchronize(c->stream), "sync");
    c->n_verts = n_verts;
    c->n_tris = n_tris;
    c->bvh_ready = false;
    c->invalidate_graph();
    return PK_OK;
  });
}

int pk_scene_download(pk_ctx* c, double* pos3, uint32_t* attr4) {
  return guarded(c, [&]() {
    if (!c->attrs.p) return fail(c, PK_ERR_STATE, "no scene");
    if (pos3) check(cudaMemcpyAsync(pos3, c->pos.p, c->pos.bytes(), cudaMemcpyDeviceToHost, c->stream), "D2H");
    if (attr4) check(cudaMemcpyAsync(attr4, c->attrs.p, c->attrs.bytes(), cudaMemcpyDeviceToHost, c->stream), "D2H");
    check(cudaStreamSynchronize(c->stream), "sync");
    return PK_OK;
  });
}

int pk_materials_set(pk_ctx* c, const double* mats9, uint32_t n_mats) {
  return guarded(c, [&]() {
    if (!mats9 || !n_mats) return fail(c, PK_ERR_ARG, "no materials");
    std::vector<int32_t> index4;
    std::vector<uint8_t> layers;
    build_material_layers(mats9, n_mats, index4, layers);
    upload(c->mat4, index4.data(), n_mats, c->stream);
    upload(c->layers, layers.data(), layers.size() / 4, c->stream);
    check(cudaStreamSynchronize(c->stream), "sync");
    c->n_mats = n_mats;
    c->n_layers = (uint32_t)(layers.size() / 4);
    c->atlas_res = 1;
    c->invalidate_graph();
    return PK_OK;
  });
}

int pk_materials_upload(pk_ctx* c, const int32_t* mat4, uint32_t n_mats, const uint8_t* layers, uint32_t n_layers) {
  return guarded(c, [&]() {
    if (!mat4 || !layers || !n_mats || !n_layers) return fail(c, PK_ERR_ARG, "no materials");
    upload(c->mat4, mat4, n_mats, c->stream);
    upload(c->layers, layers, n_layers, c->stream);
    check(cudaStreamSynchronize(c->stream), "sync");
    c->n_mats = n_mats;
    c->n_layers = n_layers;
    c->atlas_res = 1;
    c->invalidate_graph();
    return PK_OK;
  });
}

int pk_atlas_upload(pk_ctx* c, const uint8_t* layers, uint32_t res, uint32_t n_layers) {
  return guarded(c, [&]() {
    if (!layers || !res || !n_layers || res > 16384) return fail(c, PK_ERR_ARG, "bad atlas");
    if ((uint64_t)res * res * n_layers >= (1ull << 32)) return fail(c, PK_ERR_ARG, "atlas too large");
    upload(c->layers, layers, (size_t)res * res * n_layers, c->stream);
    check(cudaStreamSynchronize(c->stream), "sync");
    c->n_layers = n_layers;
    c->atlas_res = res;
    c->invalidate_graph();
    return PK_OK;
  });
}

int pk_materials_download(pk_ctx* c, uint32_t* n_mats, uint32_t* n_layers, int32_t* mat4, uint8_t* layers) {
  return guarded(c, [&]() {
    if (n_mats) *n_mats = c->n_mats;
    if (n_layers) *n_layers = c->n_layers;
    if (mat4 && c->n_mats) check(cudaMemcpyAsync(mat4, c->mat4.p, c->mat4.bytes(), cudaMemcpyDeviceToHost, c->stream), "D2H");
    if (layers && c->n_layers && c->atlas_res == 1)
      check(cudaMemcpyAsync(layers, c->layers.p, c->layers.bytes(), cudaMemcpyDeviceToHost, c->stream), "D2H");
    check(cudaStreamSynchronize(c->stream), "sync");
    return PK_OK;
  });
}

// ---------------- BVH ----------------
// The compressed 8-wide BVH and its triangle records, built on the GPU.
static int build_wide(pk_ctx* c) {
  std::string why;
  uint32_t n = 0, depth = 0;
  if (build_wide_bvh_gpu(c->stream, c->nodes5.p, c->n_nodes, c->tri4_leaf.p, c->n_leaf_tris, c->verts4.p,
                         c->bvh_verts, c->wide, c->wide_tris, n, depth, why))
    return fail(c, PK_ERR_ARG, "wide BVH: " + why);
  c->wide_nodes = n;
  c->wide_depth = depth;
  c->wide_ready = true;
  c->invalidate_graph();
  return PK_OK;
}

// Binary records with outward-rounded FP32 boxes and the binary leaf order's
// triangle records for PK_TRACE_EXACT, built on the GPU.
static int build_exact(pk_ctx* c) {
  int32_t root = 0;
  std::string why;
  if (build_exact_binary_gpu(c->stream, c->nodes5.p, c->n_nodes, c->tri4_leaf.p, c->n_leaf_tris, c->verts4.p,
                             c->bvh_verts, c->exact, c->exact_tris, root, why))
    return fail(c, PK_ERR_ARG, "exact binary records: " + why);
  c->exact_root = root;
  c->exact_ready = true;
  c->invalidate_graph();
  return PK_OK;
}

static int finish_bvh(pk_ctx* c) {
  c->wide_ready = false;
  c->wide.release();
  c->wide_tris.release();
  c->exact_ready = false;
  c->exact.release();
  c->exact_tris.release();
  c->inner.alloc(4 * (size_t)std::max<uint32_t>(c->n_nodes, 1u));
  c->inner32.alloc(2 * (size_t)std::max<uint32_t>(c->n_nodes, 1u));
  c->tris.alloc(3 * (size_t)std::max<uint32_t>(c->n_leaf_tris, 1u));
  DevBuf<int> root(1);
  DevBuf<uint32_t> err(1);
  check(cudaMemsetAsync(err.p, 0, 4, c->stream), "memset");
  if (convert_bvh(c->stream, c->nodes5.p, c->n_nodes, c->tri4_leaf.p, c->n_leaf_tris, c->verts4.p, c->bvh_verts,
                  c->inner.p, c->inner32.p, c->tris.p, root.p, err.p))
    throw CudaError(std::string("convert_bvh: ") + cudaGetErrorString(cudaGetLastError()));
  uint32_t herr = 0;
  check(cudaMemcpy(&c->root, root.p, 4, cudaMemcpyDeviceToHost), "D2H");
  check(cudaMemcpy(&herr, err.p, 4, cudaMemcpyDeviceToHost), "D2H");
  if (herr) return fail(c, PK_ERR_ARG, "malformed BVH (child index, leaf size >= 128 or vertex index out of range)");
  c->bvh_ready = true;
  if (c->trace_mode & TRACE_WIDE) {
    const int rc = build_wide(c);
    if (rc != PK_OK) return rc;
  }
  if (c->trace_mode & TRACE_EXACT) {
    const int rc = build_exact(c);
    if (rc != PK_OK) return rc;
  }
  c->invalidate_graph();
  return PK_OK;
}

int pk_wide_info(pk_ctx* c, uint32_t* n_nodes, uint32_t* depth) {
  return guarded(c, [&]() {
    if (!c->wide_ready) return fail(c, PK_ERR_STATE, "no wide BVH: set PK_TRACE_WIDE after building a BVH");
    if (n_nodes) *n_nodes = c->wide_nodes;
    if (depth) *depth = c->wide_depth;
    return PK_OK;
  });
}

int pk_wide_download(pk_ctx* c, float* nodes20, float* tris12) {
  return guarded(c, [&]() {
    if (!c->wide_ready) return fail(c, PK_ERR_STATE, "no wide BVH");
    if (!nodes20) return fail(c, PK_ERR_ARG, "null output");
    check(cudaMemcpy(nodes20, c->wide.p, 80 * (size_t)c->wide_nodes, cudaMemcpyDeviceToHost), "D2H");
    if (tris12 && c->n_leaf_tris)
      check(cudaMemcpy(tris12, c->wide_tris.p, 48 * (size_t)c->n_leaf_tris, cudaMemcpyDeviceToHost), "D2H");
    return PK_OK;
  });
}

int pk_exact_download(pk_ctx* c, float* records16, float* tris12, int32_t* root_code) {
  return guarded(c, [&]() {
    if (!c->exact_ready) return fail(c, PK_ERR_STATE, "no FP32 binary records: set PK_TRACE_EXACT after building a BVH");
    if (!records16 || !root_code) return fail(c, PK_ERR_ARG, "null output");
    check(cudaMemcpy(records16, c->exact.p, c->exact.bytes(), cudaMemcpyDeviceToHost), "D2H");
    if (tris12 && c->n_leaf_tris)
      check(cudaMemcpy(tris12, c->exact_tris.p, 48 * (size_t)c->n_leaf_tris, cudaMemcpyDeviceToHost), "D2H");
    *root_code = c->exact_root;
    return PK_OK;
  });
}

int pk_bvh_upload(pk_ctx* c, const int32_t* nodes5, uint32_t n_nodes, const int32_t* tri4_leaf, uint32_t n_leaf_tris,
                  const float* verts4, uint32_t n_verts) {
  return guarded(c, [&]() {
    if (!nodes5 || !n_nodes || !verts4 || !n_verts) return fail(c, PK_ERR_ARG, "empty BVH");
    upload(c->nodes5, nodes5, 5 * (size_t)n_nodes, c->stream);
    c->node_box_d.release();
    upload(c->tri4_leaf, tri4_leaf, n_leaf_tris, c->stream);
    upload(c->verts4, verts4, n_verts, c->stream);
    c->n_nodes = n_nodes;
    c->n_leaf_tris = n_leaf_tris;
    c->bvh_verts = n_verts;
    for (double& x : c->norm) x = 0;
    return finish_bvh(c);
  });
}

int pk_bvh_build(pk_ctx* c, int mode) {
  return guarded(c, [&]() {
    if (mode != PK_BVH_SWEEP && mode != PK_BVH_BINNED) return fail(c, PK_ERR_UNSUPPORTED, "unknown BVH mode");
    if (!c->pos.p || !c->n_tris) return fail(c, PK_ERR_STATE, "no scene");
    BvhOut out;
    std::string why;
    const int rc = mode == PK_BVH_SWEEP
                       ? build_bvh_sweep(c->stream, c->pos.p, c->n_verts, c->tri4.p, c->n_tris, out, why)
                       : build_bvh_binned(c->stream, c->pos.p, c->n_verts, c->tri4.p, c->n_tris, out, why);
    if (rc) return fail(c, PK_ERR_ARG, "pk_bvh_build: " + why);
    c->nodes5 = std::move(out.nodes5);
    c->node_box_d = std::move(out.node_box);
    c->tri4_leaf = std::move(out.tri4_leaf);
    c->verts4 = std::move(out.verts4);
    c->n_nodes = out.n_nodes;
    c->n_leaf_tris = out.n_leaf_tris;
    c->bvh_verts = c->n_verts;
    for (int i = 0; i < 4; i++) c->norm[i] = out.norm[i];
    return finish_bvh(c);
  });
}

int pk_bvh_info(pk_ctx* c, uint32_t* n_nodes, uint32_t* n_leaf_tris, double norm4[4]) {
  return guarded(c, [&]() {
    if (!c->bvh_ready) return fail(c, PK_ERR_STATE, "no BVH");
    if (n_nodes) *n_nodes = c->n_nodes;
    if (n_leaf_tris) *n_leaf_tris = c->n_leaf_tris;
    if (norm4) for (int i = 0; i < 4; i++) norm4[i] = c->norm[i];
    return PK_OK;
  });
}

int pk_bvh_download(pk_ctx* c, int32_t* nodes5, int32_t* tri4_leaf, float* verts4) {
  return guarded(c, [&]() {
    if (!c->bvh_ready) return fail(c, PK_ERR_STATE, "no BVH");
    if (nodes5) check(cudaMemcpyAsync(nodes5, c->nodes5.p, c->nodes5.bytes(), cudaMemcpyDeviceToHost, c->stream), "D2H");
    if (tri4_leaf && c->n_leaf_tris)
      check(cudaMemcpyAsync(tri4_leaf, c->tri4_leaf.p, c->tri4_leaf.bytes(), cudaMemcpyDeviceToHost, c->stream), "D2H");
    if (verts4) check(cudaMemcpyAsync(verts4, c->verts4.p, c->verts4.bytes(), cudaMemcpyDeviceToHost, c->stream), "D2H");
    check(cudaStreamSynchronize(c->stream), "sync");
    return PK_OK;
  });
}

// ---------------- env ----------------
// The alias table of PK_ENV_ALIAS from the current environment's texels.
static int build_alias(pk_ctx* c) {
  std::string why;
  if (build_env_alias_gpu(c->stream, c->rgbe.p, c->env_w, c->env_h, c->env_alias, c->alias_pdf, why))
    return fail(c, PK_ERR_ARG, "alias table: " + why);
  c->alias_ready = true;
  c->invalidate_graph();
  return PK_OK;
}
// After an environment change: the alias table follows it.
static int env_changed(pk_ctx* c) {
  c->alias_ready = false;
  return c->env_sampling == PK_ENV_ALIAS ? build_alias(c) : PK_OK;
}

static int env_set(pk_ctx* c, const uint8_t* rgbe, uint32_t w, uint32_t h, const int32_t* bins2, uint32_t nb,
                   const int32_t* coords2, const float* pdf) {
  upload(c->rgbe, rgbe, (size_t)w * h, c->stream);
  upload(c->bins, bins2, nb, c->stream);
  upload(c->coords, coords2, (size_t)w * h, c->stream);
  upload(c->pdf, pdf, (size_t)w * h, c->stream);
  check(cudaStreamSynchronize(c->stream), "sync");
  c->env_w = w; c->env_h = h; c->env_nb = nb;
  c->env_ready = true;
  c->invalidate_graph();
  return env_changed(c);
}

int pk_env_build(pk_ctx* c, const uint8_t* rgbe, uint32_t w, uint32_t h) {
  return guarded(c, [&]() {
    if (!rgbe || !w || !h) return fail(c, PK_ERR_ARG, "empty environment");
    if ((uint64_t)w * h >= (1ull << 31)) return fail(c, PK_ERR_ARG, "environment too large");
    upload(c->rgbe, rgbe, (size_t)w * h, c->stream);
    std::string why;
    uint32_t nb = 0;
    if (build_env_tables_gpu(c->stream, c->rgbe.p, w, h, c->bins, nb, c->coords, c->pdf, why)) {
      c->env_ready = false;
      return fail(c, PK_ERR_ARG, "pk_env_build: " + why);
    }
    c->env_w = w; c->env_h = h; c->env_nb = nb;
    c->env_ready = true;
    c->invalidate_graph();
    return env_changed(c);
  });
}

int pk_set_env_sampling(pk_ctx* c, int mode) {
  return guarded(c, [&]() {
    if (mode != PK_ENV_HISTOGRAM && mode != PK_ENV_ALIAS) return fail(c, PK_ERR_ARG, "unknown env sampling mode");
    if (mode == PK_ENV_ALIAS && !c->alias_ready) {
      if (!c->env_ready) return fail(c, PK_ERR_STATE, "PK_ENV_ALIAS needs an environment");
      const int rc = build_alias(c);
      if (rc != PK_OK) return rc;
    }
    c->env_sampling = mode;
    c->invalidate_graph();
    return PK_OK;
  });
}

int pk_env_alias_download(pk_ctx* c, uint32_t* table2, float* pdf) {
  return guarded(c, [&]() {
    if (!c->alias_ready) return fail(c, PK_ERR_STATE, "no alias table: set PK_ENV_ALIAS first");
    const size_t N = (size_t)c->env_w * c->env_h;
    if (table2) check(cudaMemcpyAsync(table2, c->env_alias.p, 8 * N, cudaMemcpyDeviceToHost, c->stream), "D2H");
    if (pdf) check(cudaMemcpyAsync(pdf, c->alias_pdf.p, 4 * N, cudaMemcpyDeviceToHost, c->stream), "D2H");
    check(cudaStreamSynchronize(c->stream), "sync");
    return PK_OK;
  });
}

int pk_env_upload(pk_ctx* c, const uint8_t* rgbe, uint32_t w, uint32_t h, const int32_t* bins2, uint32_t nb,
                  const int32_t* coords2, const float* pdf) {
  return guarded(c, [&]() {
    if (!rgbe || !bins2 || !coords2 || !pdf || !w || !h || !nb) return fail(c, PK_ERR_ARG, "empty environment");
    const uint64_t N = (uint64_t)w * h;
    for (uint32_t b = 0; b < nb; b++)
      if (bins2[2 * b] < 0 || bins2[2 * b] >= bins2[2 * b + 1] || (uint64_t)bins2[2 * b + 1] > N)
        return fail(c, PK_ERR_ARG, "malformed luminance bin");
    for (uint64_t i = 0; i < N; i++)
      if (coords2[2 * i] < 0 || (uint32_t)coords2[2 * i] >= w || coords2[2 * i + 1] < 0 || (uint32_t)coords2[2 * i + 1] >= h)
        return fail(c, PK_ERR_ARG, "env coordinate out of range");
    return env_set(c, rgbe, w, h, bins2, nb, coords2, pdf);
  });
}

int pk_env_info(pk_ctx* c, uint32_t* w, uint32_t* h, uint32_t* nb) {
  return guarded(c, [&]() {
    if (w) *w = c->env_w;
    if (h) *h = c->env_h;
    if (nb) *nb = c->env_nb;
    return PK_OK;
  });
}

int pk_env_download(pk_ctx* c, int32_t* bins2, int32_t* coords2, float* pdf) {
  return guarded(c, [&]() {
    if (!c->env_ready) return fail(c, PK_ERR_STATE, "no environment");
    if (bins2) check(cudaMemcpyAsync(bins2, c->bins.p, c->bins.bytes(), cudaMemcpyDeviceToHost, c->stream), "D2H");
    if (coords2) check(cudaMemcpyAsync(coords2, c->coords.p, c->coords.bytes(), cudaMemcpyDeviceToHost, c->stream), "D2H");
    if (pdf) check(cudaMemcpyAsync(pdf, c->pdf.p, c->pdf.bytes(), cudaMemcpyDeviceToHost, c->stream), "D2H");
    check(cudaStreamSynchronize(c->stream), "sync");
    return PK_OK;
  });
}

// ---------------- render state ----------------
// The render state and camera are kept on the host and handed to each frame
// by value (and to slot 0 before a pass), so setting them never waits for a
// frame in flight.
int pk_set_render_state(pk_ctx* c, int32_t samples, float env_theta) {
  return guarded_nojoin(c, [&]() {
    c->samples_next = samples;
    c->theta_next = env_theta;
    c->state_dirty = true;
    return PK_OK;
  });
}

int pk_set_camera(pk_ctx* c, const pk_camera_state* cam) {
  return guarded_nojoin(c, [&]() {
    require_config(c);
    if (!cam) return fail(c, PK_ERR_ARG, "null camera");
    CamState s;
    std::memcpy(s.pos, cam->pos, 12);
    std::memcpy(s.dir, cam->dir, 12);
    // camera_pass.js:118-125: setUint16(0, H) | setUint16(2, W) -> W << 16 | H
    s.dims_mask = (c->W << 16) | (c->H & 0xffffu);
    s.fov = cam->fov;
    s.focal_depth = cam->focal_depth;
    s.aperture = cam->aperture_size;
    s.distortion = cam->distortion;
    s.bokeh = cam->bokeh;
    s.invocation_offset = cam->invocation_offset;
    c->cam_host = s;
    c->cam_set = true;
    c->state_dirty = true;
    return PK_OK;
  });
}

int pk_set_postprocess(pk_ctx* c, float exposure, float saturation) {
  return guarded(c, [&]() {
    c->invalidate_graph();
    c->exposure = exposure;
    c->saturation = saturation;
    return PK_OK;
  });
}

int pk_clear_color(pk_ctx* c) {
  return guarded(c, [&]() {
    c->last_slot = 0;
    require_config(c);
    check(cudaMemsetAsync(c->color.p, 0, c->color.bytes(), c->stream), "memset");
    return PK_OK;
  });
}
int pk_clear_hits_misses(pk_ctx* c) {
  return guarded(c, [&]() {
    c->last_slot = 0;
    check(cudaMemsetAsync(&c->ctr.p->num_hits, 0, 8, c->stream), "memset");
    return PK_OK;
  });
}
int pk_clear_rays(pk_ctx* c) {
  return guarded(c, [&]() {
    c->last_slot = 0;
    check(cudaMemsetAsync(&c->ctr.p->num_rays, 0, 8, c->stream), "memset");
    return PK_OK;
  });
}

// ---------------- passes ----------------
static void reset_slot(pk_ctx* c, uint32_t slot) {
  check(cudaMemsetAsync(c->ticket(slot, 0), 0, 16, c->stream), "memset");
  check(cudaMemsetAsync(c->tiles_compact(slot), 0, (size_t)(2 * c->ct + c->st) * 8, c->stream), "memset");
}

int pk_camera(pk_ctx* c) {
  return guarded(c, [&]() {
    c->last_slot = 0;
    require_config(c);
    if (!c->cam_set) return fail(c, PK_ERR_STATE, "no camera");
    LaunchCtx L = c->launch();
    c->cur = 0;
    c->timed(K_CAMERA, [&]() { launch_camera(L, c->R(c->cur), c->cap); });
    check(cudaGetLastError(), "k_camera");
    return PK_OK;
  });
}

int pk_trace(pk_ctx* c) {
  return guarded(c, [&]() {
    c->last_slot = 0;
    require_render(c);
    LaunchCtx L = c->launch();
    reset_slot(c, 0);
    check(cudaMemsetAsync(&c->ctr.p->num_hits, 0, 8, c->stream), "memset");  // clearNumHitsAndMisses
    c->timed(K_TRACE, [&]() {
      launch_trace(L, false, false, c->counting, &c->ctr.p->num_rays, c->R(c->cur), c->hrec.p, c->hflags.p,
                   c->ticket(0, 0));
    });
    c->timed(K_COMPACT, [&]() {
      launch_compact_trace(L, true, c->hflags.p, c->hit_list.p, c->R(c->cur), c->M(), c->ticket(0, 1),
                           c->tiles_compact(0), nullptr);
    });
    check(cudaGetLastError(), "trace");
    return PK_OK;
  });
}

int pk_shade_hit(pk_ctx* c) {
  return guarded(c, [&]() {
    c->last_slot = 0;
    require_render(c);
    LaunchCtx L = c->launch();
    reset_slot(c, 0);
    c->timed(K_SHADE, [&]() {
      launch_shade(L, c->hit_list.p, c->hrec.p, c->R(c->cur), c->R(c->cur ^ 1), c->S(), c->ticket(0, 2),
                   c->tiles_shade(0));
    });
    c->cur ^= 1;
    check(cudaGetLastError(), "shade");
    return PK_OK;
  });
}

int pk_trace_shadow(pk_ctx* c) {
  return guarded(c, [&]() {
    c->last_slot = 0;
    require_render(c);
    LaunchCtx L = c->launch();
    reset_slot(c, 0);
    c->timed(K_SHADOW, [&]() {
      launch_trace(L, true, false, c->counting, &c->ctr.p->num_shadow, c->S(), nullptr, c->sflags.p, c->ticket(0, 3));
    });
    c->timed(K_COMPACT, [&]() { launch_compact_shadow(L, c->sflags.p, c->S(), c->M(), c->ticket(0, 1), c->tiles_shadow(0)); });
    check(cudaGetLastError(), "trace_shadow");
    return PK_OK;
  });
}

int pk_shade_miss(pk_ctx* c) {
  return guarded(c, [&]() {
    c->last_slot = 0;
    require_config(c);
    if (!c->env_ready) return fail(c, PK_ERR_STATE, "no environment");
    LaunchCtx L = c->launch();
    c->timed(K_OTHER, [&]() { launch_shade_miss(L, c->M()); });
    check(cudaGetLastError(), "shade_miss");
    return PK_OK;
  });
}

int pk_accumulate(pk_ctx* c) {
  return guarded(c, [&]() {
    c->last_slot = 0;
    require_config(c);
    LaunchCtx L = c->launch();
    c->timed(K_ACCUM, [&]() { launch_accumulate(L); });
    check(cudaGetLastError(), "accumulate");
    return PK_OK;
  });
}

int pk_postprocess(pk_ctx* c) {
  return guarded(c, [&]() {
    c->last_slot = 0;
    require_config(c);
    LaunchCtx L = c->launch();
    c->timed(K_POST, [&]() { launch_postprocess(L, c->exposure, c->saturation); });
    check(cudaGetLastError(), "postprocess");
    return PK_OK;
  });
}

// Persistent grids, in tenths of the full grid, when other frames run beside
// a frame's kernels: a persistent kernel that fills every SM until its last
// rays finish keeps the other frames' kernels waiting, and a smaller grid
// leaves them room.  1080p, eight frames in flight, closest-hit / any-hit
// traversal: 10/10 3756-3780 Mrays/s, 10/4 3811, 10/2 3878-3887, 6/4
// 3907-3920, 6/2 3905-3914, 6/1 3908-3940, 4/2 3876-3908, 3/2 3847-3871;
// the shade kernel then (10/10 3889-3902, 7/10 3911-3948, 5/10 3915-3932,
// 3/10 3877-3914), and with it closest/any 6/4 3916-3922, 5/3 3938-3968, 6/3
// 3923-3924, 7/4 3892-3912; the compaction grid at 5/10 or 7/10 within the
// noise of 10/10.  One frame with its shadow traversal overlapped: any-hit
// 10/10 2351, 4/10 2373; a smaller closest-hit grid costs there (6/2 2286,
// 4/2 2119).  The 8-wide traversal takes the same fractions of its grid.
#ifndef PK_CLOSEST_TENTHS_PIPED
#define PK_CLOSEST_TENTHS_PIPED 5
#endif
#ifndef PK_ANY_TENTHS_PIPED
#define PK_ANY_TENTHS_PIPED 3
#endif
#ifndef PK_SHADE_TENTHS_PIPED
#define PK_SHADE_TENTHS_PIPED 7
#endif
#ifndef PK_COMPACT_TENTHS_PIPED
#define PK_COMPACT_TENTHS_PIPED 10
#endif
#ifndef PK_ANY_TENTHS_OVERLAP
#define PK_ANY_TENTHS_OVERLAP 4
#endif

// One frame of slot k as its launch sequence on `st`.  With overlap
// (persistent or 8-wide traversal, no per-kernel timing) each bounce's shadow
// traversal forks onto the slot's side stream after shading and joins before
// the next bounce's compaction; that bounce's closest-hit misses are parked
// in their hit records and added by the compaction, so every pixel still
// receives its contributions in the serial order (shadow of bounce b before
// the miss of bounce b+1).  `tail`: accumulate, postprocess and the sample
// count too (frames in flight issue those outside, ordered across slots).
static void render_frame_launches(pk_ctx* c, int k, cudaStream_t st, uint32_t bounces, bool tail) {
  FrameSlot& fs = c->slot[k];
  LaunchCtx L = c->launch(k, st);
  // PK_OVERLAP_AUTO: overlap when frames render one at a time or are small
  // (below 2^20 rays); several large frames in flight already fill the shadow
  // tails (1080p, four frames: 2596-2599 Mrays/s with, 2610-2612 without; one
  // frame: +19% with; the batching workload's small requests one at a time
  // through four frames in flight: 644 ms with, 708 ms without)
  const bool want = c->overlap == PK_OVERLAP_AUTO ? (c->in_flight == 1 || c->cap < (1u << 20)) : c->overlap != 0;
  const bool ov = want && !c->timing && (c->trace_mode & (pk::TRACE_PERSISTENT | pk::TRACE_WIDE)) != 0;
  L.defer_miss = ov;
  // Persistent grids beside concurrent work (the constants above).
  if (c->in_flight > 1 && !c->timing) {
    L.closest_tenths = PK_CLOSEST_TENTHS_PIPED;
    L.any_tenths = PK_ANY_TENTHS_PIPED;
    L.shade_tenths = PK_SHADE_TENTHS_PIPED;
    L.compact_tenths = PK_COMPACT_TENTHS_PIPED;
  } else if (ov) {
    L.any_tenths = PK_ANY_TENTHS_OVERLAP;
  }
  LaunchCtx Ls = L;
  Ls.stream = fs.side;
  bool forked = false;
  auto join = [&]() {
    if (forked) check(cudaStreamWaitEvent(st, fs.ev_shadow, 0), "cudaStreamWaitEvent");
    forked = false;
  };
  // tick() renders W*H pixels in batches of BATCH_SIZE (pk_configure's batch;
  // pike.js:133-154), each with its own counters, camera offset and bounces.
  const uint32_t nbatch = (uint32_t)(((uint64_t)c->npix + c->B - 1) / c->B);
  const uint64_t steps = (uint64_t)nbatch * bounces;
  const uint32_t nb = (uint32_t)std::min<uint64_t>(steps, MAX_BOUNCES);
  // RenderState.generateCommands + tick(): clear colour, hit/miss and ray counts
  check(cudaMemsetAsync(fs.color.p, 0, fs.color.bytes(), st), "memset");
  check(cudaMemsetAsync(&fs.ctr.p->num_hits, 0, 16, st), "memset");
  check(cudaMemsetAsync(fs.tickets.p, 0, fs.tickets.bytes(), st), "memset");
  check(cudaMemsetAsync(fs.tiles.p, 0, (size_t)std::max(nb, 1u) * (2 * c->ct + c->st) * 8, st), "memset");
  uint64_t seq = 0;  // (batch, bounce) steps so far: their ticket and tile slots
  for (uint32_t batch = 0; batch < nbatch; batch++) {
    if (batch) {
      join();  // the previous batch's shadow traversal still reads its counts
      check(cudaMemsetAsync(&fs.ctr.p->num_hits, 0, 16, st), "memset");  // clearNumHitsAndMisses, clearNumRays
    }
    fs.cur = 0;
    c->timed(K_CAMERA, [&]() { launch_camera(L, fs.R(0), c->cap, (int64_t)batch * c->B); });
    for (uint32_t b = 0; b < bounces; b++, seq++) {
      const uint32_t slot = (uint32_t)(seq % MAX_BOUNCES);
      if (seq && slot == 0) {
        join();  // the shadow traversal in flight still uses its slot's ticket
        check(cudaMemsetAsync(fs.tickets.p, 0, fs.tickets.bytes(), st), "memset");
        check(cudaMemsetAsync(fs.tiles.p, 0, fs.tiles.bytes(), st), "memset");
      }
      c->timed(K_TRACE, [&]() {
        launch_trace(L, false, true, c->counting, &fs.ctr.p->num_rays, fs.R(fs.cur), fs.hrec.p, fs.hflags.p,
                     fs.ticket(slot, 0));
      });
      join();
      c->timed(K_COMPACT, [&]() {
        launch_compact_trace(L, false, fs.hflags.p, fs.hit_list.p, fs.R(fs.cur), c->M(), fs.ticket(slot, 1),
                             c->tiles_compact(slot, k), ov ? fs.hrec.p : nullptr);
      });
      c->timed(K_SHADE, [&]() {
        launch_shade(L, fs.hit_list.p, fs.hrec.p, fs.R(fs.cur), fs.R(fs.cur ^ 1), fs.S(), fs.ticket(slot, 2),
                     c->tiles_shade(slot, k));
      });
      fs.cur ^= 1;
      if (ov) {
        check(cudaEventRecord(fs.ev_shaded, st), "cudaEventRecord");
        check(cudaStreamWaitEvent(fs.side, fs.ev_shaded, 0), "cudaStreamWaitEvent");
        launch_trace(Ls, true, true, c->counting, &fs.ctr.p->num_shadow, fs.S(), nullptr, fs.sflags.p,
                     fs.ticket(slot, 3));
        check(cudaEventRecord(fs.ev_shadow, fs.side), "cudaEventRecord");
        forked = true;
      } else {
        c->timed(K_SHADOW, [&]() {
          launch_trace(L, true, true, c->counting, &fs.ctr.p->num_shadow, fs.S(), nullptr, fs.sflags.p,
                       fs.ticket(slot, 3));
        });
      }
    }
  }
  join();
  if (tail) {
    c->timed(K_ACCUM, [&]() { launch_accumulate(L); });
    c->timed(K_POST, [&]() { launch_postprocess(L, c->exposure, c->saturation); });
    c->timed(K_OTHER, [&]() { launch_end_frame(L); });
  }
  check(cudaGetLastError(), "render_frame");
}

// pk_render_frame.  A frame's launches are captured once per slot into a CUDA
// graph and replayed (the sequence only reads device-side counts).  With
// several frames in flight, frames take the slots in turn, each on its stream: each waits
// for the API stream, takes the render state by value, replays its graph,
// then accumulates and postprocesses after the previous frame did (the
// accumulation and display buffers are shared) and after the last
// asynchronous display read.  With per-kernel timing the launches are issued
// directly on the API stream.
static void render_frame(pk_ctx* c, uint32_t bounces) {
  const bool piped = c->in_flight > 1 && !c->timing;
  const int k = piped ? c->next_slot : 0;
  FrameSlot& fs = c->slot[k];
  if (fs.cap != c->cap) alloc_slot(c, k);
  const cudaStream_t st = piped ? fs.stream : c->stream;
  if (piped) {
    check(cudaEventRecord(c->ev_api, c->stream), "cudaEventRecord");
    check(cudaStreamWaitEvent(st, c->ev_api, 0), "cudaStreamWaitEvent");
  } else if (c->read_pending) {  // the display is rewritten below
    check(cudaStreamWaitEvent(st, c->ev_read, 0), "cudaStreamWaitEvent");
    c->read_pending = false;
  }
  launch_set_state(st, fs.ctr.p, fs.cam.p, c->samples_next, c->theta_next, c->cam_host, true);
  if (c->timing) {
    render_frame_launches(c, k, st, bounces, true);
  } else {
    const bool tail = !piped;
    if (!fs.graph || fs.graph_bounces != bounces || fs.graph_counting != c->counting ||
        fs.graph_key != c->state_version || fs.graph_tail != tail) {
      fs.drop_graph();
      cudaGraph_t g = nullptr;
      check(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
      try {
        render_frame_launches(c, k, st, bounces, tail);
      } catch (...) {
        cudaStreamEndCapture(st, &g);
        if (g) cudaGraphDestroy(g);
        throw;
      }
      check(cudaStreamEndCapture(st, &g), "cudaStreamEndCapture");
      cudaGraphExec_t e = nullptr;
      const cudaError_t ie = cudaGraphInstantiate(&e, g, 0);
      cudaGraphDestroy(g);
      check(ie, "cudaGraphInstantiate");
      fs.graph = e;
      fs.graph_bounces = bounces;
      fs.graph_counting = c->counting;
      fs.graph_key = c->state_version;
      fs.graph_tail = tail;
    }
    check(cudaGraphLaunch(fs.graph, st), "cudaGraphLaunch");
  }
  if (piped) {
    LaunchCtx L = c->launch(k, st);
    if (c->tail_pending) check(cudaStreamWaitEvent(st, c->ev_tail, 0), "cudaStreamWaitEvent");
    launch_accumulate(L);
    if (c->read_pending) check(cudaStreamWaitEvent(st, c->ev_read, 0), "cudaStreamWaitEvent");
    launch_postprocess(L, c->exposure, c->saturation);
    launch_end_frame(L);
    check(cudaGetLastError(), "render_frame");
    check(cudaEventRecord(c->ev_tail, st), "cudaEventRecord");
    check(cudaEventRecord(fs.ev_done, st), "cudaEventRecord");
    c->tail_pending = true;
    fs.busy = true;
    c->next_slot = (c->next_slot + 1) % c->in_flight;
  }
  c->last_slot = k;
  c->samples_next++;
  c->state_dirty = true;
  c->frames++;
}

int pk_render_frame(pk_ctx* c, uint32_t bounces) {
  return guarded_nojoin(c, [&]() {
    require_render(c);
    if (!c->env_ready) return fail(c, PK_ERR_STATE, "no environment");
    render_frame(c, bounces);
    return PK_OK;
  });
}

int pk_render_frames(pk_ctx* c, uint32_t frames, uint32_t bounces) {
  return guarded_nojoin(c, [&]() {
    require_render(c);
    if (!c->env_ready) return fail(c, PK_ERR_STATE, "no environment");
    for (uint32_t f = 0; f < frames; f++) render_frame(c, bounces);
    return PK_OK;
  });
}

// ---------------- readback ----------------
int pk_sync(pk_ctx* c) {
  return guarded(c, [&]() {
    check(cudaStreamSynchronize(c->stream), "sync");
    c->collect_events();
    uint32_t err = 0;
    for (FrameSlot& fs : c->slot) {
      if (!fs.ctr.p) continue;
      uint32_t e = 0;
      check(cudaMemcpy(&e, &fs.ctr.p->err, 4, cudaMemcpyDeviceToHost), "D2H");
      err |= e;
    }
    if (err) {
      char buf[96];
      std::snprintf(buf, sizeof buf, "device error flags 0x%x", err);
      return fail(c, PK_ERR_DEVICE, buf);
    }
    return PK_OK;
  });
}

int pk_read_counters(pk_ctx* c, uint32_t out8[8]) {
  return guarded(c, [&]() {
    if (!out8) return fail(c, PK_ERR_ARG, "null output");
    Counters h;
    check(cudaStreamSynchronize(c->stream), "sync");
    check(cudaMemcpy(&h, c->slot[c->last_slot].ctr.p, sizeof(h), cudaMemcpyDeviceToHost), "D2H");
    for (int k = 0; k < MAX_IN_FLIGHT; k++) {
      if (k == c->last_slot || !c->slot[k].ctr.p) continue;
      Counters o;
      check(cudaMemcpy(&o, c->slot[k].ctr.p, sizeof(o), cudaMemcpyDeviceToHost), "D2H");
      h.rays_traced += o.rays_traced;
      h.err |= o.err;
    }
    out8[0] = (uint32_t)h.samples; out8[1] = h.num_hits; out8[2] = h.num_misses; out8[3] = h.num_rays;
    out8[4] = h.num_shadow; out8[5] = h.err;
    out8[6] = (uint32_t)(h.rays_traced & 0xffffffffu); out8[7] = (uint32_t)(h.rays_traced >> 32);
    return PK_OK;
  });
}

static void gather_rays(pk_ctx* c, RayQ q, uint32_t first, uint32_t count, float* out12) {
  std::vector<float4> o(count), d(count), t(count);
  check(cudaStreamSynchronize(c->stream), "sync");
  check(cudaMemcpy(o.data(), q.o + first, count * 16, cudaMemcpyDeviceToHost), "D2H");
  check(cudaMemcpy(d.data(), q.d + first, count * 16, cudaMemcpyDeviceToHost), "D2H");
  check(cudaMemcpy(t.data(), q.t + first, count * 16, cudaMemcpyDeviceToHost), "D2H");
  for (uint32_t i = 0; i < count; i++) {
    float* r = out12 + 12 * (size_t)i;
    r[0] = o[i].x; r[1] = o[i].y; r[2] = o[i].z; r[3] = 0.0f;
    r[4] = d[i].x; r[5] = d[i].y; r[6] = d[i].z; r[7] = 0.0f;
    r[8] = t[i].x; r[9] = t[i].y; r[10] = t[i].z; r[11] = t[i].w;
  }
}

int pk_read_rays(pk_ctx* c, int queue, uint32_t first, uint32_t count, float* out12) {
  return guarded(c, [&]() {
    require_config(c);
    const uint64_t limit = queue == PK_QUEUE_MISS ? 2ull * c->cap : c->cap;
    if (!out12 || (uint64_t)first + count > limit) return fail(c, PK_ERR_ARG, "range outside the queue");
    if (queue != PK_QUEUE_RAYS && queue != PK_QUEUE_SHADOW && queue != PK_QUEUE_MISS) return fail(c, PK_ERR_ARG, "bad queue");
    if (count) gather_rays(c, queue == PK_QUEUE_RAYS ? c->R(c->cur) : queue == PK_QUEUE_SHADOW ? c->S() : c->M(), first, count, out12);
    return PK_OK;
  });
}

int pk_read_hits(pk_ctx* c, uint32_t first, uint32_t count, uint32_t* out16) {
  return guarded(c, [&]() {
    require_config(c);
    if (!out16 || (uint64_t)first + count > c->cap) return fail(c, PK_ERR_ARG, "range outside the hit queue");
    if (!count) return PK_OK;
    std::vector<uint32_t> list(count);
    check(cudaStreamSynchronize(c->stream), "sync");
    check(cudaMemcpy(list.data(), c->hit_list.p + first, count * 4, cudaMemcpyDeviceToHost), "D2H");
    uint32_t maxj = 0;
    for (uint32_t j : list) maxj = std::max(maxj, j);
    if (maxj >= c->cap) return fail(c, PK_ERR_STATE, "hit list entry out of range");
    std::vector<uint4> hr(maxj + 1);
    std::vector<float> rays(12 * (size_t)(maxj + 1));
    check(cudaMemcpy(hr.data(), c->hrec.p, hr.size() * 16, cudaMemcpyDeviceToHost), "D2H");
    gather_rays(c, c->R(c->cur), 0, maxj + 1, rays.data());
    for (uint32_t i = 0; i < count; i++) {
      const uint32_t j = list[i];
      uint32_t* o = out16 + 16 * (size_t)i;
      o[0] = hr[j].x; o[1] = hr[j].y; o[2] = hr[j].z; o[3] = 0;
      std::memcpy(o + 4, &rays[12 * (size_t)j], 48);
    }
    return PK_OK;
  });
}

static int read_px(pk_ctx* c, const void* src, void* dst, size_t bytes) {
  return guarded(c, [&]() {
    require_config(c);
    if (!dst) return fail(c, PK_ERR_ARG, "null output");
    check(cudaStreamSynchronize(c->stream), "sync");
    check(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost), "D2H");
    return PK_OK;
  });
}
int pk_read_color(pk_ctx* c, float* out) {
  return c ? read_px(c, c->slot[c->last_slot].color.p, out, c->color.bytes()) : PK_ERR_ARG;
}
int pk_read_accum(pk_ctx* c, float* out) { return c ? read_px(c, c->accum.p, out, c->accum.bytes()) : PK_ERR_ARG; }
int pk_write_accum(pk_ctx* c, const float* in) {
  return guarded(c, [&]() {
    require_config(c);
    if (!in) return fail(c, PK_ERR_ARG, "null input");
    check(cudaMemcpyAsync(c->accum.p, in, c->accum.bytes(), cudaMemcpyHostToDevice, c->stream), "H2D");
    check(cudaStreamSynchronize(c->stream), "sync");
    return PK_OK;
  });
}
int pk_read_display(pk_ctx* c, float* out, uint8_t* out8) {
  return guarded(c, [&]() {
    require_config(c);
    check(cudaStreamSynchronize(c->stream), "sync");
    if (out) check(cudaMemcpy(out, c->display.p, c->display.bytes(), cudaMemcpyDeviceToHost), "D2H");
    if (out8) check(cudaMemcpy(out8, c->display8.p, c->display8.bytes(), cudaMemcpyDeviceToHost), "D2H");
    return PK_OK;
  });
}

// ---------------- measurement ----------------
int pk_set_counting(pk_ctx* c, int on) { return guarded(c, [&]() { c->counting = on != 0; return PK_OK; }); }
int pk_reset_stats(pk_ctx* c) {
  return guarded(c, [&]() {
    for (FrameSlot& fs : c->slot)
      if (fs.ctr.p)
        check(cudaMemsetAsync(&fs.ctr.p->rays_traced, 0, sizeof(Counters) - offsetof(Counters, rays_traced), c->stream),
              "memset");
    check(cudaStreamSynchronize(c->stream), "sync");
    c->collect_events();
    for (int k = 0; k < N_KINDS; k++) { c->kind_ms[k] = 0; c->kind_n[k] = 0; }
    c->frames = 0;
    return PK_OK;
  });
}
int pk_read_stats(pk_ctx* c, uint64_t out10[10]) {
  return guarded(c, [&]() {
    if (!out10) return fail(c, PK_ERR_ARG, "null output");
    check(cudaStreamSynchronize(c->stream), "sync");
    for (int i = 0; i < 9; i++) out10[i] = 0;
    for (FrameSlot& fs : c->slot) {
      if (!fs.ctr.p) continue;
      Counters h;
      check(cudaMemcpy(&h, fs.ctr.p, sizeof(h), cudaMemcpyDeviceToHost), "D2H");
      for (int i = 0; i < 8; i++) out10[i] += h.stat[i];
      out10[8] += h.rays_traced;
    }
    out10[9] = c->frames;
    return PK_OK;
  });
}
int pk_set_trace_mode(pk_ctx* c, int mode) {
  return guarded(c, [&]() {
    c->invalidate_graph();
    const int sched = mode & 1;
    if (mode & ~(1 | PK_TRACE_COMPACT_RECORDS | PK_TRACE_WIDE | PK_TRACE_EXACT))
      return fail(c, PK_ERR_ARG, "unknown trace mode");
    if ((mode & PK_TRACE_WIDE) && (mode & PK_TRACE_EXACT))
      return fail(c, PK_ERR_ARG, "PK_TRACE_WIDE and PK_TRACE_EXACT exclude each other");
    if ((mode & PK_TRACE_EXACT) && !(mode & PK_TRACE_PERSISTENT))
      return fail(c, PK_ERR_ARG, "PK_TRACE_EXACT needs PK_TRACE_PERSISTENT");
    if ((mode & PK_TRACE_WIDE) && !c->wide_ready) {
      if (!c->bvh_ready) return fail(c, PK_ERR_STATE, "PK_TRACE_WIDE needs a BVH");
      const int rc = build_wide(c);
      if (rc != PK_OK) return rc;
    }
    if ((mode & PK_TRACE_EXACT) && !c->exact_ready) {
      if (!c->bvh_ready) return fail(c, PK_ERR_STATE, "PK_TRACE_EXACT needs a BVH");
      const int rc = build_exact(c);
      if (rc != PK_OK) return rc;
    }
    c->trace_mode = sched | (mode & PK_TRACE_WIDE ? TRACE_WIDE : 0) | (mode & PK_TRACE_EXACT ? TRACE_EXACT : 0);
    c->compact_nodes = (mode & PK_TRACE_COMPACT_RECORDS) != 0;
    return PK_OK;
  });
}
int pk_set_accumulation(pk_ctx* c, int mode) {
  return guarded(c, [&]() {
    if (mode != PK_ACCUM_RUNNING_MEAN && mode != PK_ACCUM_COMPENSATED) return fail(c, PK_ERR_ARG, "unknown accumulation mode");
    require_config(c);
    c->kahan = mode == PK_ACCUM_COMPENSATED;
    if (c->kahan && c->accum_sum.n != c->npix) {
      c->accum_sum.alloc(c->npix);
      c->accum_comp.alloc(c->npix);
    }
    c->invalidate_graph();
    return PK_OK;
  });
}

int pk_set_frame_overlap(pk_ctx* c, int on) {
  return guarded(c, [&]() {
    if (on != PK_OVERLAP_AUTO && on != 0 && on != 1) return fail(c, PK_ERR_ARG, "overlap must be 0, 1 or PK_OVERLAP_AUTO");
    c->overlap = on;
    c->invalidate_graph();
    return PK_OK;
  });
}

int pk_set_frames_in_flight(pk_ctx* c, int n) {
  return guarded(c, [&]() {
    if (n < 1 || n > MAX_IN_FLIGHT) return fail(c, PK_ERR_ARG, "frames in flight must be 1 to 16");
    c->in_flight = n;
    c->next_slot = 0;
    c->invalidate_graph();
    return PK_OK;
  });
}

int pk_set_timing(pk_ctx* c, int on) { return guarded(c, [&]() { c->timing = on != 0; return PK_OK; }); }
int pk_read_timing(pk_ctx* c, float out16[16]) {
  return guarded(c, [&]() {
    if (!out16) return fail(c, PK_ERR_ARG, "null output");
    check(cudaStreamSynchronize(c->stream), "sync");
    c->collect_events();
    for (int k = 0; k < N_KINDS; k++) { out16[k] = c->kind_ms[k]; out16[8 + k] = c->kind_n[k]; }
    return PK_OK;
  });
}

int pk_stream_timer(pk_ctx* c, int op, float* ms) {
  return guarded(c, [&]() {
    if (!c->t0) check(cudaEventCreate(&c->t0), "cudaEventCreate");
    if (!c->t1) check(cudaEventCreate(&c->t1), "cudaEventCreate");
    if (op == 0) {
      check(cudaEventRecord(c->t0, c->stream), "cudaEventRecord");
      return PK_OK;
    }
    if (op != 1 || !ms) return fail(c, PK_ERR_ARG, "pk_stream_timer: op must be 0 or 1 with an output");
    check(cudaEventRecord(c->t1, c->stream), "cudaEventRecord");
    check(cudaEventSynchronize(c->t1), "cudaEventSynchronize");
    check(cudaEventElapsedTime(ms, c->t0, c->t1), "cudaEventElapsedTime");
    return PK_OK;
  });
}

int pk_host_alloc(pk_ctx* c, size_t bytes, void** out) {
  return guarded(c, [&]() {
    if (!out) return fail(c, PK_ERR_ARG, "null output");
    check(cudaHostAlloc(out, bytes ? bytes : 1, cudaHostAllocDefault), "cudaHostAlloc");
    return PK_OK;
  });
}

int pk_host_free(pk_ctx* c, void* p) {
  return guarded(c, [&]() {
    if (p) check(cudaFreeHost(p), "cudaFreeHost");
    return PK_OK;
  });
}

// On the copy stream, after the API stream and the last frame's postprocess;
// the next frame's postprocess waits for it.  Complete after pk_sync.
int pk_read_display_async(pk_ctx* c, uint8_t* out8) {
  return guarded_nojoin(c, [&]() {
    require_config(c);
    if (!out8) return fail(c, PK_ERR_ARG, "null output");
    check(cudaEventRecord(c->ev_api, c->stream), "cudaEventRecord");
    check(cudaStreamWaitEvent(c->copy, c->ev_api, 0), "cudaStreamWaitEvent");
    if (c->tail_pending) check(cudaStreamWaitEvent(c->copy, c->ev_tail, 0), "cudaStreamWaitEvent");
    check(cudaMemcpyAsync(out8, c->display8.p, c->display8.bytes(), cudaMemcpyDeviceToHost, c->copy), "D2H");
    check(cudaEventRecord(c->ev_read, c->copy), "cudaEventRecord");
    c->read_pending = true;
    return PK_OK;
  });
}

int pk_math_eval(pk_ctx* c, int fn, const float* x, const float* y, float* out, uint32_t n) {
  return guarded(c, [&]() {
    if (!x || !out) return fail(c, PK_ERR_ARG, "null array");
    DevBuf<float> dx, dy, dout(n);
    upload(dx, x, n, c->stream);
    if (y) upload(dy, y, n, c->stream);
    launch_math(c->stream, fn, dx.p, y ? dy.p : nullptr, dout.p, n);
    check(cudaGetLastError(), "k_math");
    check(cudaMemcpyAsync(out, dout.p, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream), "D2H");
    check(cudaStreamSynchronize(c->stream), "sync");
    return PK_OK;
  });
}

}  // extern "C"
