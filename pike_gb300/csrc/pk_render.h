// pk_render.h -- host-side launchers of the per-frame kernels (pk_render.cu).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "pk_internal.cuh"

namespace pk {

// Traversal scheduling: fixed 32-ray chunks per warp, or persistent lanes with
// batched refill.  Both visit every ray's nodes in the reference order.
enum TraceMode : int { TRACE_CHUNKED = 0, TRACE_PERSISTENT = 1, TRACE_WIDE = 4, TRACE_EXACT = 8 };

// Everything a launch needs that is fixed for a configured context.
struct LaunchCtx {
  cudaStream_t stream;
  Counters* ctr;
  const CamState* cam;
  SceneDev scene;
  EnvDev env;
  float4* color;
  float4* accum;
  float4* display;
  uchar4* display8;
  uint32_t npix;
  uint32_t capacity;       // ray / hit / shadow queue capacity (batch rounded up to 128)
  uint32_t miss_capacity;  // 2 * capacity
  unsigned trace_blocks, compact_blocks, shade_blocks, trace_blocks_wide;
  float4* accum_sum = nullptr;   // compensated accumulation (pk_set_accumulation), else null
  float4* accum_comp = nullptr;
  int trace_mode;
  // Closest-hit misses park their contribution in the hit record for the
  // compaction to add (frames whose shadow traversal overlaps the next bounce).
  bool defer_miss = false;
  // Persistent grid of the binary traversals in tenths of trace_blocks:
  // smaller when other work runs beside them (frames in flight, overlap).
  unsigned closest_tenths = 10, any_tenths = 10;
  unsigned shade_tenths = 10, compact_tenths = 10;  // the same for the shade and compaction grids
};

// offset >= 0: invocation offset of the rays (else the camera state's own)
void launch_camera(const LaunchCtx& L, RayQ R, uint32_t n_threads, int64_t offset = -1);
// Kernels that claim work through an atomic ticket take it as `ticket`; the
// look-back kernels also take a zeroed tile-state array (one word per tile).
void launch_trace(const LaunchCtx& L, bool any_hit, bool fused, bool count, const uint32_t* countp, RayQ R,
                  uint4* hrec, uint32_t* flags, uint32_t* ticket);
// miss_rec: the hit records of a trace launched with L.defer_miss (whose parked
// miss contributions this compaction adds), else null.
void launch_compact_trace(const LaunchCtx& L, bool missq, const uint32_t* flags, uint32_t* hit_list, RayQ src,
                          RayQ M, uint32_t* ticket, unsigned long long* tiles, const uint4* miss_rec);
void launch_compact_shadow(const LaunchCtx& L, const uint32_t* flags, RayQ S, RayQ M, uint32_t* ticket,
                           unsigned long long* tiles);
void launch_shade(const LaunchCtx& L, const uint32_t* hit_list, const uint4* hrec, RayQ Rin, RayQ Rout, RayQ S,
                  uint32_t* ticket, unsigned long long* tiles);
// Grid sizes for a queue capacity on a GPU with `sms` multiprocessors.
void kernel_grids(int sms, uint32_t capacity, unsigned* trace, unsigned* compact, unsigned* shade,
                  unsigned* trace_wide);
// Tile counts the look-back kernels need for a given queue capacity.
uint32_t compact_tiles(uint32_t capacity);
uint32_t shade_tiles(uint32_t capacity);
void launch_shade_miss(const LaunchCtx& L, RayQ M);
void launch_accumulate(const LaunchCtx& L);
void launch_postprocess(const LaunchCtx& L, float exposure, float saturation);
void launch_end_frame(const LaunchCtx& L);
// Sets a frame's sample index, environment rotation and (with_cam) camera.
void launch_set_state(cudaStream_t s, Counters* ctr, CamState* cam, int32_t samples, float theta, const CamState& cs,
                      bool with_cam);
void launch_math(cudaStream_t s, int fn, const float* x, const float* y, float* out, uint32_t n);

// pk_scene.cu
// Convert the reference 20-byte BFS nodes + leaf-ordered triangles + 16-byte
// vertices into the traversal format (inner records, v0/e1/e2 triangles).
int convert_bvh(cudaStream_t s, const int32_t* nodes5, uint32_t n_nodes, const int4* tri4, uint32_t n_tris,
                const float4* verts4, uint32_t n_verts, float4* inner, int4* inner32, float4* tris, int* root_code,
                uint32_t* err);
// Row S: per-vertex attribute quantisation (scene.js:456-470).
void launch_flatten(cudaStream_t s, const double* pos3, const double* nrm3, const double* tan4, const double* bn3,
                    const double* bt4, const double* uv2, uint32_t n, double scale, double tx, double ty, double tz,
                    double* pos_out3, uint4* attrs);

// ---- form (2): persistent multi-request batch (pk_batch.cu drives it) ----
struct BatchScene {
  SceneDev sc;
  EnvDev env;
  float theta;
};
struct BatchReq {
  CamState cam;
  uint32_t scene, W, H, spp, depth;
  unsigned long long path_begin;  // first path id of this request
  unsigned long long out_offset;  // first accumulation pixel of this request
};
constexpr int BATCH_MAX_SCENES = 8;
constexpr int BATCH_MAX_REQ = 1024;
struct BatchConfig {
  int block, stack, chunk;  // threads per block, shared-memory stack entries, warp grab = chunk * 32 paths
};
// false for a configuration without a kernel instantiation
bool batch_config_ok(const BatchConfig& c);
int batch_blocks_per_sm(const BatchConfig& c);
void launch_batch(cudaStream_t s, const BatchConfig& c, unsigned grid, const BatchScene* scenes, int nscenes,
                  const BatchReq* reqs, int nreq, unsigned long long total, unsigned long long* counter,
                  uint32_t* frame, float4* accum, unsigned long long n_accum, uint32_t* err,
                  unsigned long long* remaining, unsigned long long* done_ns);
void launch_batch_next_frame(cudaStream_t s, uint32_t* frame);

}  // namespace pk
