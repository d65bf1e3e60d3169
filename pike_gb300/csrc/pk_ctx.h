// pk_ctx.h -- the library context behind the opaque pk_ctx handle (internal).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "pk_internal.cuh"
#include "pk_render.h"
#include "pk_util.h"

namespace pk {

constexpr uint32_t MAX_BOUNCES = 16;
constexpr int MAX_IN_FLIGHT = 16;  // frame slots
constexpr int N_KINDS = 8;
enum Kind { K_CAMERA = 0, K_TRACE, K_COMPACT, K_SHADE, K_SHADOW, K_ACCUM, K_POST, K_OTHER };

struct EventPair {
  int kind;
  cudaEvent_t a, b;
};

// The transient state of one frame of pk_render_frame.  Several slots let
// several frames be in flight: each renders on its own stream (plus a side stream for
// its shadow traversals) from its own counters, camera, colour buffer and
// queues; the scene, BVH, environment, accumulation and display buffers are
// shared.  Slot 0 is also the state of the pass-by-pass API.
struct FrameSlot {
  DevBuf<Counters> ctr;
  DevBuf<CamState> cam;
  DevBuf<float4> color;
  DevBuf<float4> rq[2][3], sq[3];
  DevBuf<uint4> hrec;
  DevBuf<uint32_t> hflags, sflags, hit_list;
  DevBuf<uint32_t> tickets;          // 4 per bounce slot
  DevBuf<unsigned long long> tiles;  // per bounce slot: ct (compact) + st (shade) + ct (shadow compact)
  int cur = 0;
  uint32_t cap = 0;                  // queue capacity the buffers were sized for (0: none)
  cudaStream_t stream = nullptr;     // frames of this slot when two are in flight
  cudaStream_t side = nullptr;       // shadow traversals (frame overlap)
  cudaEvent_t ev_shaded = nullptr, ev_shadow = nullptr, ev_done = nullptr;
  bool busy = false;                 // a frame was issued here since the last join
  // CUDA graph of this slot's frame; rebuilt when any captured pointer or
  // launch parameter changes.
  cudaGraphExec_t graph = nullptr;
  uint32_t graph_bounces = 0;
  bool graph_counting = false, graph_tail = false;
  unsigned long long graph_key = 0;

  RayQ R(int i) { return RayQ{rq[i][0].p, rq[i][1].p, rq[i][2].p}; }
  RayQ S() { return RayQ{sq[0].p, sq[1].p, sq[2].p}; }
  uint32_t* ticket(uint32_t bounce_slot, int k) { return tickets.p + 4 * bounce_slot + k; }
  void drop_graph() {
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
  }
};

// Device address of pk_cast_rays_noalloc's static scratch array on the
// current device (pk_cast.cu).
void* noalloc_scratch_address();

}  // namespace pk

struct pk_ctx {
  using RayQ = pk::RayQ;
  using LaunchCtx = pk::LaunchCtx;
  using Counters = pk::Counters;
  using CamState = pk::CamState;
  template <class T>
  using DevBuf = pk::DevBuf<T>;
  using EventPair = pk::EventPair;
  int device = 0;
  int sms = 0;
  cudaStream_t stream = nullptr;  // the API stream: uploads, passes, readbacks, serial frames
  cudaStream_t copy = nullptr;    // pk_read_display_async
  cudaEvent_t ev_api = nullptr, ev_tail = nullptr, ev_read = nullptr;
  int overlap = PK_OVERLAP_AUTO;  // shadow traversal beside the next closest-hit traversal
  int in_flight = 4;  // frames of pk_render_frame in flight (1..MAX_IN_FLIGHT)
  int next_slot = 0, last_slot = 0;
  bool tail_pending = false;      // ev_tail: accumulate/postprocess of the last pipelined frame
  bool read_pending = false;      // ev_read: the last asynchronous display read
  std::string err;
  // configuration
  uint32_t W = 0, H = 0, B = 0, cap = 0, npix = 0;
  uint32_t ct = 0, st = 0;  // look-back tiles per compaction / shade launch
  unsigned g_trace = 1, g_compact = 1, g_shade = 1, g_trace_wide = 1;  // persistent grid sizes
  int trace_mode = pk::TRACE_PERSISTENT;
  unsigned long long state_version = 1;
  pk::FrameSlot slot[pk::MAX_IN_FLIGHT];
  void invalidate_graph() {
    for (pk::FrameSlot& s : slot) s.drop_graph();
    state_version++;
  }
  // render state for the next frame (pk_set_render_state / pk_set_camera);
  // each frame receives it by value, pk_render_frame advances samples.
  int32_t samples_next = 0;
  float theta_next = 0.0f;
  CamState cam_host{};
  bool state_dirty = false;  // slot 0's device copy is stale
  DevBuf<Counters>& ctr = slot[0].ctr;
  DevBuf<CamState>& cam = slot[0].cam;
  bool cam_set = false;
  float exposure = 1.0f, saturation = 1.0f;
  DevBuf<float4>& color = slot[0].color;
  DevBuf<float4> accum, display;
  DevBuf<float4> accum_sum, accum_comp;  // compensated accumulation buffers
  bool kahan = false;
  DevBuf<uchar4> display8;
  DevBuf<float4> mq[3];
  int& cur = slot[0].cur;
  DevBuf<uint4>& hrec = slot[0].hrec;
  DevBuf<uint32_t>& hflags = slot[0].hflags;
  DevBuf<uint32_t>& sflags = slot[0].sflags;
  DevBuf<uint32_t>& hit_list = slot[0].hit_list;
  DevBuf<uint32_t>& tickets = slot[0].tickets;
  DevBuf<unsigned long long>& tiles = slot[0].tiles;
  // scene
  uint32_t n_verts = 0, n_tris = 0;
  DevBuf<double> pos;
  DevBuf<uint4> attrs;
  DevBuf<int4> tri4;
  uint32_t n_mats = 0, n_layers = 0, atlas_res = 1;
  DevBuf<int4> mat4;
  DevBuf<uchar4> layers;
  // bvh
  uint32_t n_nodes = 0, n_leaf_tris = 0, n_inner = 0, bvh_verts = 0;
  double norm[4] = {0, 0, 0, 0};
  DevBuf<int32_t> nodes5;
  DevBuf<int4> tri4_leaf;
  DevBuf<float4> verts4, inner, tris;
  DevBuf<int4> inner32;
  DevBuf<double> node_box_d;  // exact double node bounds (pk_bvh_build only)
  bool compact_nodes = false;  // traverse 32-byte records (same boxes as the 64-byte ones)
  DevBuf<float4> wide;         // compressed 8-wide BVH nodes (built on first use of PK_TRACE_WIDE)
  DevBuf<float4> wide_tris;    // its triangle records, in its own leaf order
  DevBuf<float4> exact;        // binary records with outward-rounded FP32 boxes (PK_TRACE_EXACT)
  DevBuf<float4> exact_tris;   // triangle records of the binary leaf order (PK_TRACE_EXACT)
  int exact_root = 0;
  bool exact_ready = false;
  uint32_t wide_nodes = 0, wide_depth = 0;
  bool wide_ready = false;
  int root = 0;
  bool bvh_ready = false;
  // env
  uint32_t env_w = 0, env_h = 0, env_nb = 0;
  DevBuf<uchar4> rgbe;
  DevBuf<int2> bins, coords;
  DevBuf<float> pdf;
  bool env_ready = false;
  int env_sampling = 0;       // PK_ENV_HISTOGRAM or PK_ENV_ALIAS
  DevBuf<uint2> env_alias;    // PK_ENV_ALIAS: {keep threshold, alias} per texel
  DevBuf<float> alias_pdf;    // and its pdf texture
  bool alias_ready = false;
  // measurement
  bool counting = false;
  bool timing = false;
  std::vector<EventPair> events;
  std::vector<cudaEvent_t> event_pool;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  float kind_ms[pk::N_KINDS] = {0};
  float kind_n[pk::N_KINDS] = {0};
  unsigned long long frames = 0;
  unsigned long long diff_rays = 0;  // rays of the last differentiable render / adjoint
  // the differentiable renderer's environment sampling tables (pk_diff_set_env_sampling)
  uint32_t diff_env_w = 0, diff_env_h = 0, diff_env_nb = 0;
  DevBuf<int2> diff_bins, diff_coords;
  DevBuf<float> diff_pdf;
  bool diff_env_ready = false;
  void* cast_scratch = nullptr;  // pk_cast_rays_noalloc's static scratch on this device (set by pk_create)

  RayQ R(int i) { return slot[0].R(i); }
  RayQ S() { return slot[0].S(); }
  RayQ M() { return RayQ{mq[0].p, mq[1].p, mq[2].p}; }
  uint32_t* ticket(uint32_t b, int k) { return slot[0].ticket(b, k); }
  unsigned long long* tiles_compact(uint32_t b, int k = 0) { return slot[k].tiles.p + (size_t)b * (2 * ct + st); }
  unsigned long long* tiles_shade(uint32_t b, int k = 0) { return tiles_compact(b, k) + ct; }
  unsigned long long* tiles_shadow(uint32_t b, int k = 0) { return tiles_compact(b, k) + ct + st; }

  // Launch parameters for frame slot k on stream s (default: slot 0 on the API stream).
  LaunchCtx launch(int k = 0, cudaStream_t s = nullptr) {
    LaunchCtx L;
    L.stream = s ? s : stream;
    L.ctr = slot[k].ctr.p;
    L.cam = slot[k].cam.p;
    const bool ex = (trace_mode & pk::TRACE_EXACT) && exact_ready;
    L.scene = pk::SceneDev{ex ? exact.p : inner.p, (compact_nodes && !ex) ? inner32.p : nullptr, tris.p, tri4_leaf.p,
                           attrs.p, mat4.p, layers.p, (int)n_layers, (int)atlas_res, ex ? exact_root : root,
                       n_leaf_tris, n_verts, n_mats, wide_ready ? wide.p : nullptr,
                       (trace_mode & pk::TRACE_WIDE) && wide_ready ? wide_tris.p : (ex ? exact_tris.p : nullptr)};
    const bool al = env_sampling == PK_ENV_ALIAS && alias_ready;
    L.env = pk::EnvDev{rgbe.p, bins.p, coords.p, al ? alias_pdf.p : pdf.p, (int)env_w, (int)env_h, (int)env_nb,
                       env_ready ? 1 : 0, al ? env_alias.p : nullptr};
    L.color = slot[k].color.p;
    L.accum = accum.p;
    L.display = display.p;
    L.display8 = display8.p;
    L.npix = npix;
    L.capacity = cap;
    L.miss_capacity = 2 * cap;
    L.trace_blocks = g_trace;
    L.trace_blocks_wide = g_trace_wide;
    L.accum_sum = kahan ? accum_sum.p : nullptr;
    L.accum_comp = kahan ? accum_comp.p : nullptr;
    L.compact_blocks = g_compact;
    L.shade_blocks = g_shade;
    L.trace_mode = trace_mode;
    return L;
  }
  // The drop-in's traversal records (the reference's snorm16 boxes and root),
  // whatever the trace mode.  The ray-query, batch and differentiable kernels
  // use the drop-in's box test and strict `<` hit test, which are defined on
  // these records only; PK_TRACE_EXACT's outward-rounded records need the
  // slack and (t, slot) ties of the exact traversal.
  pk::SceneDev dropin_scene() {
    pk::SceneDev s = launch().scene;
    s.inner = inner.p;
    s.inner32 = compact_nodes ? inner32.p : nullptr;
    s.root = root;
    return s;
  }
  cudaEvent_t take_event() {
    if (!event_pool.empty()) {
      cudaEvent_t e = event_pool.back();
      event_pool.pop_back();
      return e;
    }
    cudaEvent_t e;
    pk::check(cudaEventCreate(&e), "cudaEventCreate");
    return e;
  }
  template <class F>
  void timed(int kind, F fn) {
    if (!timing) {
      fn();
      return;
    }
    EventPair p{kind, take_event(), take_event()};
    pk::check(cudaEventRecord(p.a, stream), "cudaEventRecord");
    fn();
    pk::check(cudaEventRecord(p.b, stream), "cudaEventRecord");
    events.push_back(p);
  }
  void collect_events() {
    for (EventPair& p : events) {
      float ms = 0;
      pk::check(cudaEventElapsedTime(&ms, p.a, p.b), "cudaEventElapsedTime");
      kind_ms[p.kind] += ms;
      kind_n[p.kind] += 1;
      event_pool.push_back(p.a);
      event_pool.push_back(p.b);
    }
    events.clear();
  }
};

