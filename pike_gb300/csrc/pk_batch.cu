// pk_batch.cu -- form (2): many render requests over several resident scenes
// in one persistent launch (k_batch in pk_render.cu), replayed per frame from
// a captured CUDA graph, with a measured choice of block size, shared-memory
// stack depth and queue chunk.  No reference counterpart.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pike.h"
#include "pk_ctx.h"
#include "pk_render.h"
#include "pk_util.h"

using namespace pk;

struct pk_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  std::vector<pk_ctx*> ctxs;
  std::vector<BatchScene> scenes;
  std::vector<BatchReq> reqs;
  DevBuf<BatchScene> d_scenes;
  DevBuf<BatchReq> d_reqs;
  DevBuf<float4> accum;
  DevBuf<unsigned long long> counter;
  DevBuf<uint32_t> frame, errflag;
  DevBuf<unsigned long long> remaining, remaining_init, done_ns;  // per request; done_ns[n] = launch start
  unsigned long long total = 0, n_accum = 0;
  BatchConfig cfg{128, 32, 4};
  unsigned grid = 1;
  int sms = 1;
  cudaGraphExec_t graph = nullptr;
  uint32_t frames = 0;
  float last_ms = 0.0f;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  void drop_graph() {
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
  }
};

namespace {

int bfail(pk_batch* b, int code, const std::string& m) {
  b->err = m;
  return code;
}

template <class F>
int bguard(pk_batch* b, F fn) {
  if (!b) return PK_ERR_ARG;
  try {
    check(cudaSetDevice(b->device), "cudaSetDevice");
    return fn();
  } catch (CudaError& e) {
    b->err = e.what();
    return PK_ERR_CUDA;
  } catch (std::exception& e) {
    b->err = e.what();
    return PK_ERR_STATE;
  }
}

unsigned grid_for_cfg(pk_batch* b, const BatchConfig& c) {
  const int per_sm = std::max(batch_blocks_per_sm(c), 1);
  return (unsigned)(b->sms * per_sm);
}

void enqueue_frame(pk_batch* b, const BatchConfig& c, unsigned grid, unsigned long long total) {
  check(cudaMemsetAsync(b->counter.p, 0, 8, b->stream), "memset");
  check(cudaMemcpyAsync(b->remaining.p, b->remaining_init.p, b->remaining.bytes(), cudaMemcpyDeviceToDevice,
                        b->stream), "D2D");
  check(cudaMemsetAsync(b->done_ns.p, 0, b->done_ns.bytes(), b->stream), "memset");
  launch_batch(b->stream, c, grid, b->d_scenes.p, (int)b->scenes.size(), b->d_reqs.p, (int)b->reqs.size(), total,
               b->counter.p, b->frame.p, b->accum.p, b->n_accum, b->errflag.p, b->remaining.p, b->done_ns.p);
  check(cudaGetLastError(), "k_batch");
  launch_batch_next_frame(b->stream, b->frame.p);
}

void reset_accum(pk_batch* b) {
  if (b->accum.p) check(cudaMemsetAsync(b->accum.p, 0, b->accum.bytes(), b->stream), "memset");
  check(cudaMemsetAsync(b->frame.p, 0, 4, b->stream), "memset");
  b->frames = 0;
}

}  // namespace

extern "C" {

int pk_batch_create(pk_batch** out, pk_ctx* const* scenes, uint32_t n_scenes) {
  if (!out || !scenes || n_scenes == 0 || n_scenes > (uint32_t)BATCH_MAX_SCENES) return PK_ERR_ARG;
  *out = nullptr;
  pk_batch* b = new pk_batch();
  b->device = scenes[0]->device;
  const int rc = bguard(b, [&]() {
    for (uint32_t i = 0; i < n_scenes; i++) {
      pk_ctx* c = scenes[i];
      if (!c || c->device != b->device) return bfail(b, PK_ERR_ARG, "scenes must be contexts on one device");
      if (!c->bvh_ready || !c->env_ready || !c->attrs.p || !c->mat4.p)
        return bfail(b, PK_ERR_STATE, "every scene needs a BVH, materials and an environment");
      const LaunchCtx L = c->launch();
      b->ctxs.push_back(c);
      b->scenes.push_back(BatchScene{c->dropin_scene(), L.env, 0.0f});
    }
    check(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device), "attr");
    check(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "stream");
    check(cudaEventCreate(&b->e0), "event");
    check(cudaEventCreate(&b->e1), "event");
    b->d_scenes.alloc(b->scenes.size());
    check(cudaMemcpy(b->d_scenes.p, b->scenes.data(), b->d_scenes.bytes(), cudaMemcpyHostToDevice), "H2D");
    b->counter.alloc(1);
    b->frame.alloc(1);
    b->errflag.alloc(1);
    check(cudaMemset(b->errflag.p, 0, 4), "memset");
    check(cudaMemset(b->frame.p, 0, 4), "memset");
    return PK_OK;
  });
  if (rc != PK_OK) {
    std::fprintf(stderr, "pk_batch_create: %s\n", b->err.c_str());
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return rc;
  }
  *out = b;
  return PK_OK;
}

int pk_batch_destroy(pk_batch* b) {
  if (!b) return PK_ERR_ARG;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  b->drop_graph();
  if (b->e0) cudaEventDestroy(b->e0);
  if (b->e1) cudaEventDestroy(b->e1);
  b->d_scenes.release();
  b->d_reqs.release();
  b->accum.release();
  b->counter.release();
  b->frame.release();
  b->errflag.release();
  b->remaining.release();
  b->remaining_init.release();
  b->done_ns.release();
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return PK_OK;
}

const char* pk_batch_last_error(pk_batch* b) { return b ? b->err.c_str() : "null batch"; }

int pk_batch_set_requests(pk_batch* b, const pk_batch_request* reqs, uint32_t n) {
  return bguard(b, [&]() {
    if (!reqs || n == 0 || n > (uint32_t)BATCH_MAX_REQ) return bfail(b, PK_ERR_ARG, "1..1024 requests");
    std::vector<BatchReq> v(n);
    unsigned long long paths = 0, pixels = 0;
    for (uint32_t i = 0; i < n; i++) {
      const pk_batch_request& r = reqs[i];
      if (r.scene >= b->scenes.size()) return bfail(b, PK_ERR_ARG, "request names an unknown scene");
      if (!r.width || !r.height || r.width > 16384 || r.height > 16384 || !r.spp || r.spp > 65536 || !r.depth ||
          r.depth > MAX_BOUNCES)
        return bfail(b, PK_ERR_ARG, "request size, spp or depth out of range");
      BatchReq& q = v[i];
      std::memset(&q.cam, 0, sizeof(q.cam));
      for (int k = 0; k < 3; k++) { q.cam.pos[k] = r.camera.pos[k]; q.cam.dir[k] = r.camera.dir[k]; }
      q.cam.dims_mask = (r.width << 16) | r.height;
      q.cam.fov = r.camera.fov;
      q.cam.focal_depth = r.camera.focal_depth;
      q.cam.aperture = r.camera.aperture_size;
      q.cam.distortion = r.camera.distortion;
      q.cam.bokeh = r.camera.bokeh;
      q.cam.invocation_offset = 0;
      q.scene = r.scene;
      q.W = r.width;
      q.H = r.height;
      q.spp = r.spp;
      q.depth = r.depth;
      q.path_begin = paths;
      q.out_offset = pixels;
      paths += (unsigned long long)r.width * r.height * r.spp;
      pixels += (unsigned long long)r.width * r.height;
    }
    if (pixels > (1ull << 31)) return bfail(b, PK_ERR_ARG, "requests exceed 2^31 output pixels");
    b->drop_graph();
    b->reqs = v;
    b->total = paths;
    b->n_accum = pixels;
    b->d_reqs.alloc(n);
    check(cudaMemcpyAsync(b->d_reqs.p, v.data(), n * sizeof(BatchReq), cudaMemcpyHostToDevice, b->stream), "H2D");
    std::vector<unsigned long long> counts(n);
    for (uint32_t i = 0; i < n; i++) counts[i] = (unsigned long long)v[i].W * v[i].H * v[i].spp;
    b->remaining.alloc(n);
    b->remaining_init.alloc(n);
    b->done_ns.alloc(n + 1);
    check(cudaMemcpyAsync(b->remaining_init.p, counts.data(), n * 8, cudaMemcpyHostToDevice, b->stream), "H2D");
    b->accum.alloc(pixels);
    reset_accum(b);
    check(cudaStreamSynchronize(b->stream), "sync");
    return PK_OK;
  });
}

int pk_batch_set_config(pk_batch* b, int block, int stack, int chunk) {
  return bguard(b, [&]() {
    const BatchConfig c{block, stack, chunk};
    if (!batch_config_ok(c)) return bfail(b, PK_ERR_ARG, "unsupported configuration (block 64/128/256, stack 16/32, chunk 1..64)");
    b->cfg = c;
    b->drop_graph();
    return PK_OK;
  });
}

int pk_batch_get_config(pk_batch* b, int* block, int* stack, int* chunk) {
  if (!b || !block || !stack || !chunk) return PK_ERR_ARG;
  *block = b->cfg.block;
  *stack = b->cfg.stack;
  *chunk = b->cfg.chunk;
  return PK_OK;
}

int pk_batch_autotune(pk_batch* b, uint64_t sample_paths, float* best_ms) {
  return bguard(b, [&]() {
    if (b->reqs.empty()) return bfail(b, PK_ERR_STATE, "set requests first");
    const unsigned long long total = sample_paths ? std::min<unsigned long long>(sample_paths, b->total) : b->total;
    const int blocks[3] = {64, 128, 256}, stacks[3] = {8, 16, 32}, chunks[3] = {1, 4, 16};
    float best = 1e30f;
    BatchConfig pick = b->cfg;
    for (int bl : blocks)
      for (int st : stacks)
        for (int ch : chunks) {
          const BatchConfig c{bl, st, ch};
          const unsigned grid = grid_for_cfg(b, c);
          enqueue_frame(b, c, grid, total);  // warm
          check(cudaEventRecord(b->e0, b->stream), "event");
          enqueue_frame(b, c, grid, total);
          check(cudaEventRecord(b->e1, b->stream), "event");
          check(cudaEventSynchronize(b->e1), "sync");
          float ms = 0.0f;
          check(cudaEventElapsedTime(&ms, b->e0, b->e1), "elapsed");
          if (ms < best) { best = ms; pick = c; }
        }
    b->cfg = pick;
    b->drop_graph();
    reset_accum(b);
    uint32_t e = 0;
    check(cudaMemcpyAsync(&e, b->errflag.p, 4, cudaMemcpyDeviceToHost, b->stream), "D2H");
    check(cudaStreamSynchronize(b->stream), "sync");
    if (best_ms) *best_ms = best;
    if (e) return bfail(b, PK_ERR_DEVICE, "device error flags during autotuning");
    return PK_OK;
  });
}

int pk_batch_render(pk_batch* b, uint32_t frames) {
  return bguard(b, [&]() {
    if (b->reqs.empty()) return bfail(b, PK_ERR_STATE, "set requests first");
    if (!b->graph) {
      b->grid = grid_for_cfg(b, b->cfg);
      cudaGraph_t g = nullptr;
      check(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "capture");
      enqueue_frame(b, b->cfg, b->grid, b->total);
      check(cudaStreamEndCapture(b->stream, &g), "capture");
      const cudaError_t ie = cudaGraphInstantiate(&b->graph, g, 0);
      cudaGraphDestroy(g);
      check(ie, "cudaGraphInstantiate");
    }
    check(cudaEventRecord(b->e0, b->stream), "event");
    for (uint32_t f = 0; f < frames; f++) check(cudaGraphLaunch(b->graph, b->stream), "cudaGraphLaunch");
    check(cudaEventRecord(b->e1, b->stream), "event");
    uint32_t e = 0;
    check(cudaMemcpyAsync(&e, b->errflag.p, 4, cudaMemcpyDeviceToHost, b->stream), "D2H");
    check(cudaStreamSynchronize(b->stream), "sync");
    check(cudaEventElapsedTime(&b->last_ms, b->e0, b->e1), "elapsed");
    b->frames += frames;
    if (e) return bfail(b, PK_ERR_DEVICE, "device error flags (traversal stack or accumulation index)");
    return PK_OK;
  });
}

int pk_batch_reset(pk_batch* b) {
  return bguard(b, [&]() {
    reset_accum(b);
    check(cudaStreamSynchronize(b->stream), "sync");
    return PK_OK;
  });
}

int pk_batch_read(pk_batch* b, uint32_t req, float* rgba_mean) {
  return bguard(b, [&]() {
    if (req >= b->reqs.size() || !rgba_mean) return bfail(b, PK_ERR_ARG, "bad request index or null output");
    const BatchReq& q = b->reqs[req];
    const size_t n = (size_t)q.W * q.H;
    check(cudaMemcpyAsync(rgba_mean, b->accum.p + q.out_offset, n * 16, cudaMemcpyDeviceToHost, b->stream), "D2H");
    check(cudaStreamSynchronize(b->stream), "sync");
    const float inv = b->frames ? 1.0f / ((float)b->frames * (float)q.spp) : 0.0f;
    for (size_t i = 0; i < 4 * n; i++) rgba_mean[i] *= inv;
    return PK_OK;
  });
}

int pk_batch_latencies(pk_batch* b, float* ms) {
  return bguard(b, [&]() {
    if (!ms || b->reqs.empty()) return bfail(b, PK_ERR_ARG, "no requests or null output");
    std::vector<unsigned long long> t(b->reqs.size() + 1);
    check(cudaMemcpyAsync(t.data(), b->done_ns.p, t.size() * 8, cudaMemcpyDeviceToHost, b->stream), "D2H");
    check(cudaStreamSynchronize(b->stream), "sync");
    const unsigned long long t0 = t[b->reqs.size()];
    for (size_t i = 0; i < b->reqs.size(); i++) ms[i] = t[i] >= t0 ? (float)((double)(t[i] - t0) * 1e-6) : -1.0f;
    return PK_OK;
  });
}

int pk_batch_info(pk_batch* b, uint64_t* total_paths, uint32_t* frames, float* last_ms) {
  if (!b) return PK_ERR_ARG;
  if (total_paths) *total_paths = b->total;
  if (frames) *frames = b->frames;
  if (last_ms) *last_ms = b->last_ms;
  return PK_OK;
}

}  // extern "C"
