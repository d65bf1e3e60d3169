/* pike.h -- C ABI of libpike.so, the GB300 (sm_103a) implementation of Pike's
 * wavefront path tracer.
 *
 * The reference drives its passes from JavaScript through WebGPU: pass objects
 * with a `static async create(device, ...)` factory and a
 * `generateCommands(commandEncoder)` method (the files of render/passes), sequenced by
 * PikeRenderer.tick() (render/pike.js:120-162).  Each entry point below names
 * the reference interface it replaces.  A JavaScript host binds them through
 * an N-API addon; the Python package pike_gb300 binds them through ctypes.
 *
 * Conventions
 *  - Every function returns a status: PK_OK (0) or an error code; the message
 *    of the last failure on a context is returned by pk_last_error().
 *  - The library owns all device memory.  Host input pointers are read before
 *    the call returns; output pointers must hold the documented element counts.
 *  - A context is single-threaded.  Uploads, passes and reads enqueue on its
 *    stream; pk_render_frame renders up to pk_set_frames_in_flight frames
 *    concurrently on further streams of its own, and every other call orders
 *    itself after them.  Entry points enqueue work and return; pk_sync() waits
 *    and reports device-side error flags (queue/stack overflow, bounded-wait
 *    timeouts) as PK_ERR_DEVICE.
 *  - Results are bit-identical to the CPU oracle's restatement of the reference
 *    (IEEE binary32, no FMA contraction, built-ins defined in pk_math.cuh).
 */
#ifndef PIKE_H_
#define PIKE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PK_OK 0
#define PK_ERR_ARG 1      /* invalid argument or size */
#define PK_ERR_CUDA 2     /* CUDA runtime error (message in pk_last_error) */
#define PK_ERR_STATE 3    /* call out of order (e.g. trace before a scene) */
#define PK_ERR_DEVICE 4   /* a kernel raised an error flag (see pk_read_counters) */
#define PK_ERR_UNSUPPORTED 5

/* Device-side error bits, reported in pk_read_counters()[5]. */
#define PK_DEVERR_STACK 1u
#define PK_DEVERR_LOOKBACK 2u
#define PK_DEVERR_QUEUE 4u
#define PK_DEVERR_PIXEL 8u
#define PK_DEVERR_BVH 16u

typedef struct pk_ctx pk_ctx;

/* CameraPass.setCameraState({pos, dir, fov, focalDepth, apertureSize,
 * distortion, bokeh, invocationOffset}) (render/passes/camera_pass.js:118-125),
 * packed as CameraStateStuct (render/util/structs.js:235-249).  fov is the
 * vertical field of view in radians; positions are in the normalised frame
 * the passes render in (trace_pass.js:202-211). */
typedef struct pk_camera_state {
  float pos[3];
  float dir[3];
  float fov;
  float focal_depth;
  float aperture_size;
  float distortion;
  float bokeh;
  uint32_t invocation_offset;
} pk_camera_state;

/* ---- lifetime ----------------------------------------------------------
 * navigator.gpu.requestAdapter()/requestDevice() (render/pike.js:92-97). */
int pk_create(pk_ctx** out, int cuda_device);
int pk_destroy(pk_ctx* ctx);
const char* pk_last_error(const pk_ctx* ctx);
/* Library version as 10000*major + 100*minor + patch. */
int pk_version(void);

/* CameraPass.create(device, resolution, batchSize) together with the
 * RenderState it owns (render/passes/camera_pass.js:3-19,79-91) and the ray,
 * hit and miss queues of TracePass (trace_pass.js:40-54).  batch_size is
 * BATCH_SIZE of pike.js:18 (W*H for one batch per frame). */
int pk_configure(pk_ctx* ctx, uint32_t width, uint32_t height, uint32_t batch_size);

/* ---- scene (rows S and M) -----------------------------------------------
 * Scene._createBuffers (render/scene.js:120-181) for vertices whose glTF
 * node matrix is the identity and whose prop transform is {scale, translate}
 * without rotations: quantises tangent/bitangent/normal to snorm8x4 and uv to
 * snorm16x2 on the GPU.  pos3/nrm3: n_verts*3 doubles, tan4: n_verts*4
 * (w = handedness), uv2: n_verts*2; tri4: n_tris*{i0, i1, i2, matId}. */
int pk_scene_flatten(pk_ctx* ctx, const double* pos3, const double* nrm3, const double* tan4, const double* uv2,
                     uint32_t n_verts, const int32_t* tri4, uint32_t n_tris, double scale,
                     const double translate[3]);
/* The same for props whose transforms rotate (scene.js:83-93): the host has
 * applied the glTF node matrices and the prop's rotate/scale/translate.
 * pos3 are final positions (used as is), nrm3/tan4 the rotated normal and
 * tangent (tan4.w unused), and bn3/bt4 the normal and signed tangent before
 * the prop's rotations, from which scene.js:160 builds the bitangent. */
int pk_scene_flatten_tbn(pk_ctx* ctx, const double* pos3, const double* nrm3, const double* tan4, const double* bn3,
                         const double* bt4, const double* uv2, uint32_t n_verts, const int32_t* tri4, uint32_t n_tris);
/* Upload already-flattened scene tables (scene.indices / scene.attributes). */
int pk_scene_upload(pk_ctx* ctx, const int32_t* tri4, uint32_t n_tris, const double* pos3, const uint32_t* attr4,
                    uint32_t n_verts);
/* Read back the flattened tables: pos3 (n_verts*3 doubles), attr4 (n_verts*4). */
int pk_scene_download(pk_ctx* ctx, double* pos3, uint32_t* attr4);
/* Scene._createSceneMaterial (scene.js:43-70) for untextured glTF materials
 * plus TexturePacker.addColor dedup and 1x1 layers (texture_packer.js:87-136).
 * mats9 per material: base r,g,b,a, roughness, metallic, emissive r,g,b. */
int pk_materials_set(pk_ctx* ctx, const double* mats9, uint32_t n_mats);
/* Upload a material index table {diffMap, metRoughMap, normMap, emitMap}
 * (MaterialIndexStruct, structs.js:251-260) and 1x1 rgba8 atlas layers. */
int pk_materials_upload(pk_ctx* ctx, const int32_t* mat4, uint32_t n_mats, const uint8_t* layers_rgba8,
                        uint32_t n_layers);
/* Textured atlas (TexturePacker.getPixels, texture_packer.js:121-136): n_layers
 * rgba8 layers of res x res texels, row-major, sampled by the shading pass with
 * textureSampleLevel's linear filter and repeat addressing (shade_hit.wgsl:
 * 184-197).  Replaces the layers of pk_materials_set/upload; material indices
 * stay as uploaded. */
int pk_atlas_upload(pk_ctx* ctx, const uint8_t* layers, uint32_t res, uint32_t n_layers);
/* n_layers, then mat4 (n_mats*4) and layers (n_layers*4 bytes, 1x1 layers only); either pointer may be NULL. */
int pk_materials_download(pk_ctx* ctx, uint32_t* n_mats, uint32_t* n_layers, int32_t* mat4, uint8_t* layers_rgba8);

/* ---- BVH (rows BVH and Q) ----------------------------------------------
 * new BVH(scene) + TracePass.initBVHBuffer (render/bvh.js:12-74,
 * render/passes/trace_pass.js:202-263) on the GPU.
 * mode PK_BVH_SWEEP: the reference's full-sweep object SAH (same topology,
 * primitive order and quantised boxes as bvh.js). */
#define PK_BVH_SWEEP 0
/* mode PK_BVH_BINNED: a binned SAH build (16 bins per axis, leaves of at
 * most 8 triangles) in the same layout; NOT the reference's topology, so
 * frames differ from the reference's; for callers that want a fast build
 * (no reference counterpart). */
#define PK_BVH_BINNED 1
int pk_bvh_build(pk_ctx* ctx, int mode);
/* Upload a BVH serialised by the reference: nodes5 = n_nodes * BVHNodeStruct
 * {childBaseIdx, triangles, xMask, yMask, zMask} (20 B), tri4_leaf = leaf-ordered
 * VertexIndexStruct, verts4 = normalised VertexPositionStruct (16 B stride). */
int pk_bvh_upload(pk_ctx* ctx, const int32_t* nodes5, uint32_t n_nodes, const int32_t* tri4_leaf,
                  uint32_t n_leaf_tris, const float* verts4, uint32_t n_verts);
/* n_nodes, n_leaf_tris, and the normaliser {center x,y,z, scale} (only set by pk_bvh_build). */
int pk_bvh_info(pk_ctx* ctx, uint32_t* n_nodes, uint32_t* n_leaf_tris, double norm4[4]);
/* Size (8-wide nodes, levels) and records of the compressed wide BVH (no
 * reference counterpart; the layout of pike_gb300/csrc/pk_wide.h): nodes20 =
 * 20 floats per node, tris12 (optional) = 12 floats per triangle record in the
 * wide BVH's order; PK_ERR_STATE before PK_TRACE_WIDE was set. */
int pk_wide_info(pk_ctx* ctx, uint32_t* n_nodes, uint32_t* depth);
int pk_wide_download(pk_ctx* ctx, float* nodes20, float* tris12);
/* Records of the FP32 binary reference (PK_TRACE_EXACT; no reference
 * counterpart): records16 = 16 floats per inner node of the binary BVH (both
 * children's outward-rounded boxes {hi, lo} per axis, then the two child
 * codes), tris12 = 12 floats per triangle in the binary leaf order, root_code
 * = the root's code; PK_ERR_STATE before PK_TRACE_EXACT was set. */
int pk_exact_download(pk_ctx* ctx, float* records16, float* tris12, int32_t* root_code);
int pk_bvh_download(pk_ctx* ctx, int32_t* nodes5, int32_t* tri4_leaf, float* verts4);

/* ---- environment (row E) --------------------------------------------------
 * new EnvironmentGenerator(img) (render/env_sampler.js:8-29,59-157): luminance
 * histogram, sorted texel coordinates and pdf texture from an RGBE-in-rgba8
 * equirect image (w*h*4 bytes, row-major). */
int pk_env_build(pk_ctx* ctx, const uint8_t* rgbe, uint32_t w, uint32_t h);
int pk_env_upload(pk_ctx* ctx, const uint8_t* rgbe, uint32_t w, uint32_t h, const int32_t* bins2, uint32_t nb,
                  const int32_t* coords2, const float* pdf);
int pk_env_info(pk_ctx* ctx, uint32_t* w, uint32_t* h, uint32_t* nb);
int pk_env_download(pk_ctx* ctx, int32_t* bins2, int32_t* coords2, float* pdf);

/* ---- render state ----------------------------------------------------
 * RenderState.generateCommands header upload {samples, envTheta}
 * (camera_pass.js:53-64); setEnvRotation/resetSamples. */
int pk_set_render_state(pk_ctx* ctx, int32_t samples, float env_theta);
int pk_set_camera(pk_ctx* ctx, const pk_camera_state* cam);
/* PostProcessPass.setExposure / setSaturation (postprocess_pass.js). */
int pk_set_postprocess(pk_ctx* ctx, float exposure, float saturation);
/* RenderState.clearColorBuffer / clearNumHitsAndMisses / clearNumRays (camera_pass.js:66-77). */
int pk_clear_color(pk_ctx* ctx);
int pk_clear_hits_misses(pk_ctx* ctx);
int pk_clear_rays(pk_ctx* ctx);

/* ---- passes (one call per generateCommands) ------------------------------ */
int pk_camera(pk_ctx* ctx);        /* CameraPass.generateCommands      (camera_pass.js:209-220, camera.wgsl) */
int pk_trace(pk_ctx* ctx);         /* TracePass.generateCommands       (trace_pass.js:265-276, trace.wgsl) */
int pk_shade_hit(pk_ctx* ctx);     /* ShadeHitPass.generateCommands    (shade_hit_pass.js:169-181, shade_hit.wgsl) */
int pk_trace_shadow(pk_ctx* ctx);  /* TraceShadowPass.generateCommands (trace_shadow_pass.js, trace_shadow.wgsl) */
int pk_shade_miss(pk_ctx* ctx);    /* ShadeMissPass.generateCommands   (shade_miss_pass.js, shade_miss.wgsl) */
int pk_accumulate(pk_ctx* ctx);    /* AccumulatePass.generateCommands  (accumulate_pass.js, accumulate.wgsl) */
int pk_postprocess(pk_ctx* ctx);   /* PostProcessPass: ACES + saturation + sRGB into a headless buffer */

/* ---- whole frames ------------------------------------------------------
 * PikeRenderer.tick() (pike.js:120-162) for one batch: clear, camera,
 * `bounces` x (trace, shade, shadow, miss), accumulate, postprocess, then
 * samples += 1.  Misses are shaded inside the traversal kernels instead of
 * through a materialised miss queue; results are identical to the pass path. */
int pk_render_frame(pk_ctx* ctx, uint32_t bounces);
int pk_render_frames(pk_ctx* ctx, uint32_t frames, uint32_t bounces);

/* ---- ray queries -------------------------------------------------------
 * Trace n rays held in caller-owned DEVICE buffers against the context's BVH:
 * the GPU form of the reference's autofocus Raycaster (render/raycaster.js:
 * 114-131, pike.js:88-90), with trace.wgsl closest-hit (any_hit = 0) or
 * trace_shadow.wgsl any-hit (any_hit = 1) semantics.  ray_o4 / ray_d4: n
 * float4 each (xyz used, normalised frame); hits4: n * {t bits, triangle index
 * or 0xffffffff, bary_mask, 0}; hit_index: the indices of the rays that hit,
 * increasing; n_hits: one u32 (device).  Runs on the context's stream and
 * returns when the results are written.  Always traverses the drop-in's
 * snorm16 node records, whatever pk_set_trace_mode selected.  Any hit reports
 * the closest triangle of the first leaf that has a hit, as trace_shadow.wgsl
 * does (its :154-158); the render passes' any-hit traversal only needs
 * visibility and stops at the first accepted triangle of that leaf (same
 * occluded/unoccluded answer, possibly another triangle). */
int pk_cast_rays(pk_ctx* ctx, const float* ray_o4, const float* ray_d4, uint32_t n, int any_hit, uint32_t* hits4,
                 uint32_t* hit_index, uint32_t* n_hits);
/* pk_cast_rays without any device allocation.  No counterpart in the reference.
 * For callers that must not allocate device memory when they query: a host
 * that handed its device memory budget to its own pool up front, or a
 * latency-sensitive render thread, where cudaMalloc can fail and cudaFree
 * waits for the whole device (stalling work queued by other threads).  It
 * makes no cudaMalloc/cudaFree call: its scratch is a 132,352-byte static
 * device array that every GPU loading the library keeps until the process
 * exits.  Limit: at most 1,048,576 rays per call (more returns PK_ERR_ARG).
 * pk_create looks up that array's device address (with the context's device
 * current) and the context keeps it, so it lives as long as the context.  All
 * calls share the array (each call re-zeroes what must start at zero): calls
 * that overlap on the GPU race.  Same arguments and results as pk_cast_rays;
 * like it, the call synchronises the context's stream before it returns. */
int pk_cast_rays_noalloc(pk_ctx* ctx, const float* ray_o4, const float* ray_d4, uint32_t n, int any_hit,
                         uint32_t* hits4, uint32_t* hit_index, uint32_t* n_hits);

/* Autofocus: Raycaster.cast (render/raycaster.js:13-131) of one ray in the
 * normalised frame, in double precision against the unquantised triangles
 * (Möller-Trumbore, epsilon 1e-12; 1e6 when nothing is hit), and the focal
 * depth 1 - 1/t that PikeRenderer.focusCamera derives from it (pike.js:88-90).
 * Needs the normaliser of pk_bvh_build.  focal_depth_out may be NULL. */
int pk_focus_distance(pk_ctx* ctx, const double origin[3], const double dir[3], double* t_out,
                      double* focal_depth_out);

/* ---- readback ---------------------------------------------------------- */
int pk_sync(pk_ctx* ctx);
/* samples, num_hits, num_misses, num_rays, num_shadow, device error bits,
 * rays traced (low, high 32 bits) since the last pk_reset_stats. */
int pk_read_counters(pk_ctx* ctx, uint32_t out8[8]);
/* queue 0: current ray queue, 1: shadow rays, 2: miss queue; 12 floats per ray
 * in the reference's DeferredRay layout {origin, 0, dir, 0, throughput}. */
#define PK_QUEUE_RAYS 0
#define PK_QUEUE_SHADOW 1
#define PK_QUEUE_MISS 2
int pk_read_rays(pk_ctx* ctx, int queue, uint32_t first, uint32_t count, float* out12);
/* Hit entries in the reference layout: {t bits, index, bary_mask, 0, ray[12]} (64 B). */
int pk_read_hits(pk_ctx* ctx, uint32_t first, uint32_t count, uint32_t* out16);
/* W*H*4 floats: colour buffer, running mean, tonemapped display; W*H*4 bytes: display8. */
int pk_read_color(pk_ctx* ctx, float* out);
int pk_read_accum(pk_ctx* ctx, float* out);
int pk_write_accum(pk_ctx* ctx, const float* in);
int pk_read_display(pk_ctx* ctx, float* out, uint8_t* out8);

/* ---- measurement --------------------------------------------------------
 * counting != 0 selects traversal kernels that also count, per ray kind, the
 * node fetches and triangle tests of the reference algorithm (trace.wgsl:
 * the current node plus both children per inner step, one per leaf).
 * pk_read_stats: closest {fetch, tests}, shadow {fetch, tests}, rays
 * {closest, shadow}, hits {closest, occluded shadow} (counting kernels only),
 * then rays traced by all kernels and frames rendered. */
int pk_set_counting(pk_ctx* ctx, int counting);
int pk_reset_stats(pk_ctx* ctx);
int pk_read_stats(pk_ctx* ctx, uint64_t out10[10]);
/* timing != 0 records CUDA events around every kernel of pk_render_frame on the
 * context's stream; pk_read_timing returns summed milliseconds and launch
 * counts per kernel kind: camera, trace, compact, shade, shadow, accumulate,
 * postprocess, other (16 floats: 8 times then 8 counts). */
/* Accumulation: PK_ACCUM_RUNNING_MEAN is accumulate.wgsl's running mean (the
 * default, bit-exact with the reference); PK_ACCUM_COMPENSATED keeps Kahan
 * sums of max(c, 0) per pixel and writes sum / n to the accumulation buffer
 * (the precision form; no reference counterpart).  pk_write_accum only seeds
 * the running mean. */
#define PK_ACCUM_RUNNING_MEAN 0
#define PK_ACCUM_COMPENSATED 1
int pk_set_accumulation(pk_ctx* ctx, int mode);
/* Environment light sampling of the shade pass: PK_ENV_HISTOGRAM is
 * env_sampler.js's equal-mass luminance histogram (env_sampler.js:74-157,
 * sampleEnv shade_hit.wgsl:213-227; the default, bit-exact with the
 * reference); PK_ENV_ALIAS draws texels from an alias table (Walker) with
 * probability proportional to their radiance, built on the GPU: the total
 * and the normalisation in FP64, then the weights in fixed point and the
 * sweep of Huebschle-Schneider & Sanders from exact integer prefix sums (the
 * precision form; no reference counterpart).  The alias mode makes the same
 * two hash draws and uses its own pdf texture for envPdf (shade_hit.wgsl:
 * 202-210), so MIS stays consistent.  pk_env_alias_download returns the
 * table (per texel {keep threshold, alias}: keep the uniformly drawn texel
 * when the next 32-bit random number is below the threshold, always when it
 * is 0xffffffff) and the pdf texture, W*H entries each. */
#define PK_ENV_HISTOGRAM 0
#define PK_ENV_ALIAS 1
int pk_set_env_sampling(pk_ctx* ctx, int mode);
int pk_env_alias_download(pk_ctx* ctx, uint32_t* table2, float* pdf);
/* overlap = 1 lets pk_render_frame run each bounce's shadow traversal
 * concurrently with the next bounce's closest-hit traversal on a second stream
 * of its graph, 0 runs them in sequence, PK_OVERLAP_AUTO (the default) does
 * the former when one frame is in flight or the ray queue holds fewer than
 * 2^20 rays (several large frames in flight already fill the shadow
 * traversals' tails).  Images are bit-identical either
 * way (pixels receive their contributions in the same order).  Applies to the
 * persistent and 8-wide traversal modes without per-kernel timing. */
#define PK_OVERLAP_AUTO (-1)
int pk_set_frame_overlap(pk_ctx* ctx, int overlap);
/* Frames of pk_render_frame in flight, 1 to 16 (4 by default): with 2 or more,
 * consecutive frames render on separate sets of queues and streams so one
 * frame's kernels fill the idle time of another's; accumulation and
 * postprocessing stay in frame order and images are bit-identical to 1 (one
 * frame at a time).  Every
 * other call (passes, uploads, reads, pk_sync) first waits for the frames in
 * flight; pk_set_render_state, pk_set_camera and pk_read_display_async do not.
 * pk_read_color returns the colour buffer of the last frame rendered. */
int pk_set_frames_in_flight(pk_ctx* ctx, int frames);
int pk_set_timing(pk_ctx* ctx, int timing);
int pk_read_timing(pk_ctx* ctx, float out16[16]);
/* CUDA events on the context's stream: op 0 records the start event, op 1
 * records the stop event, waits for it and returns the elapsed milliseconds. */
int pk_stream_timer(pk_ctx* ctx, int op, float* ms);
/* Read-bandwidth probe for the roofline denominators (no reference
 * counterpart): reads a zero-filled device buffer of `bytes` reps times with
 * 128-bit L2-only loads from every SM (after one untimed pass) and returns GB/s.
 * A buffer well inside the 129 MB L2 measures the L2 read rate.  Allocates the
 * buffer for the duration of the call. */
int pk_probe_read_bandwidth(pk_ctx* ctx, uint64_t bytes, uint32_t reps, float* gbs);
/* Page-locked host memory for the asynchronous readback below. */
int pk_host_alloc(pk_ctx* ctx, size_t bytes, void** out);
int pk_host_free(pk_ctx* ctx, void* p);
/* Enqueue a copy of the W*H*4-byte display image into host memory (pinned for
 * the copy to overlap); completes at the next pk_sync or stop timer. */
int pk_read_display_async(pk_ctx* ctx, uint8_t* out8);
/* Traversal scheduling of pk_trace / pk_trace_shadow / pk_render_frame:
 * PK_TRACE_CHUNKED gives each warp 32 consecutive rays at a time;
 * PK_TRACE_PERSISTENT (default) keeps warps resident and refills idle lanes in
 * batches.  OR PK_TRACE_COMPACT_RECORDS to traverse 32-byte inner records that
 * keep the reference's snorm16 boxes (decoded in the kernel) instead of the
 * default 64-byte records with the same boxes pre-decoded: half the node bytes,
 * more instructions per step.  Every combination gives identical results. */
#define PK_TRACE_CHUNKED 0
#define PK_TRACE_PERSISTENT 1
#define PK_TRACE_COMPACT_RECORDS 2
/* OR PK_TRACE_WIDE to trace an 8-wide BVH with 8-bit child boxes, collapsed
 * from the binary BVH on first use (no reference counterpart: the precision
 * form beside the drop-in).  Its closest hit is the minimum of (t, triangle
 * slot) over every triangle the reference's test accepts, with the same t, u,
 * v bits; the drop-in traversal keeps the reference's first-found order and
 * its inward-truncated snorm16 boxes, so the two differ only on rays where
 * those boxes lose a hit or two triangles tie on t. */
#define PK_TRACE_WIDE 4
/* OR PK_TRACE_EXACT (with PK_TRACE_PERSISTENT) to trace the same binary BVH
 * with FP32 boxes rounded outward from the triangles (plus a margin), slack in
 * the box tests and (t, slot) ties: the FP32 binary reference of the wide
 * traversal; both give the brute-force closest hit (no reference counterpart). */
#define PK_TRACE_EXACT 8
int pk_set_trace_mode(pk_ctx* ctx, int mode);
/* Elementwise evaluation of the library's built-in definitions on the GPU
 * (fn 0 sin, 1 cos, 2 tan, 3 atan2(x, y), 4 acos, 5 exp2, 6 log2, 7 pow(x, y)),
 * and of the integer decodes on bit-cast integer inputs (fn 8 the node-box
 * snorm16, 9 snorm8, 10 unorm8, 11 unorm16, 12 the attribute snorm16). */
int pk_math_eval(pk_ctx* ctx, int fn, const float* x, const float* y, float* out, uint32_t n);

/* ---- form (3): differentiable rendering (no reference counterpart) -------
 * The drop-in's estimator rendered path by path over the loaded scene and BVH
 * (camera.wgsl rays from pk_set_camera, trace.wgsl / trace_shadow.wgsl
 * traversal, shade_hit.wgsl shading with GGX VNDF sampling, the Fresnel lobe
 * choice, environment next-event estimation and power-heuristic MIS,
 * shade_miss.wgsl), with base colour, roughness and metallic taken from
 * per-material FP32 parameters and the environment radiance from an FP32 RGB
 * equirect map (environment rotation: pk_set_render_state's env_theta), and
 * its path-replay adjoint.  Shading random numbers are seeded with the bounce
 * index (as in pk_batch) instead of the wavefront's hit-queue slot.
 * Sampling is detached: normals are sampled with roughness_sampling and
 * environment directions from the tables of pk_diff_set_env_sampling; each
 * path is weighted by the ratio of the VNDF densities at roughness and at
 * roughness_sampling, so with roughness == roughness_sampling the estimator is
 * the drop-in's and, with the paths held fixed, a smooth function of the
 * parameters whose exact derivative pk_diff_backward returns (what central
 * differences with common random numbers measure, moving roughness only).
 * All array pointers are DEVICE pointers owned by the caller (e.g. torch
 * tensors); the calls block until the work on the library's stream is done,
 * so the caller must finish its own writes to the inputs first.  Resolution
 * comes from pk_configure. */
typedef struct pk_diff_params {
  const float* albedo3;             /* n_mats x 3: base colour */
  const float* roughness;           /* n_mats, alpha = roughness^2 */
  const float* metallic;            /* n_mats (not differentiated) */
  const float* roughness_sampling;  /* n_mats, or NULL (= roughness): the roughness normals are sampled with */
  uint32_t n_mats;                  /* >= the scene's material count, <= 4096 */
  const float* env_rgb;             /* env_h x env_w x 3 equirect radiance */
  uint32_t env_w, env_h;            /* the size given to pk_diff_set_env_sampling */
  uint32_t spp, depth;              /* depth = closest-hit rays per path, 1..8 */
  uint32_t sample_base;             /* sample s uses camera.wgsl's `samples` = sample_base + s */
} pk_diff_params;
/* Environment sampling tables (env_sampler.js's histogram and pdf, from the
 * luma of an FP32 RGB map, w x h x 3 on the device), held until the next call. */
int pk_diff_set_env_sampling(pk_ctx* ctx, const float* env_rgb, uint32_t w, uint32_t h);
int pk_diff_env_info(pk_ctx* ctx, uint32_t* w, uint32_t* h, uint32_t* nb);
/* Host copies: bins2 (nb x 2), coords2 (w*h x 2), pdf (w*h). */
int pk_diff_env_download(pk_ctx* ctx, int32_t* bins2, int32_t* coords2, float* pdf);
/* image4: width x height x 4 floats (rgb, 0), the mean over spp. */
int pk_diff_render(pk_ctx* ctx, const pk_diff_params* params, float* image4);
/* d_image4: dLoss/dimage (width x height x 4); the gradients are ADDED to
 * g_albedo3 (n_mats x 3), g_roughness (n_mats) and g_env_rgb (env_h x env_w x 3). */
int pk_diff_backward(pk_ctx* ctx, const pk_diff_params* params, const float* d_image4, double* g_albedo3,
                     double* g_roughness, double* g_env_rgb);
/* Rays traced (closest hit and shadow) by the last pk_diff_render / pk_diff_backward call. */
int pk_diff_rays(pk_ctx* ctx, unsigned long long* rays);

/* ---- form (2): batched rendering (no reference counterpart) -------------
 * Many render requests over up to 8 resident scenes in one persistent launch:
 * lanes draw paths (request, sample, pixel) from a shared queue and advance
 * one bounce per step with the drop-in's shading (shade_hit.wgsl), so a batch
 * of uneven requests keeps the GPU full.  A frame of the batch (every request
 * at its spp) is captured once as a CUDA graph and replayed per frame.  The
 * scene contexts must stay alive and unchanged while the batch exists.
 * Images are statistically, not bitwise, equal to the drop-in's: the RNG seed
 * of a hit uses the bounce index where the reference uses the hit-queue slot. */
typedef struct pk_batch pk_batch;
typedef struct pk_batch_request {
  uint32_t scene;            /* index into the scenes of pk_batch_create */
  uint32_t width, height;
  uint32_t spp;              /* samples per frame */
  uint32_t depth;            /* bounces, 1..16 */
  pk_camera_state camera;    /* invocation_offset ignored */
} pk_batch_request;
int pk_batch_create(pk_batch** out, pk_ctx* const* scenes, uint32_t n_scenes);
int pk_batch_destroy(pk_batch* batch);
const char* pk_batch_last_error(pk_batch* batch);
int pk_batch_set_requests(pk_batch* batch, const pk_batch_request* requests, uint32_t n);
/* Threads per block (64/128/256), shared-memory traversal stack entries
 * (8/16/32) and queue chunk (a warp claims chunk*32 paths per atomic, 1..64). */
int pk_batch_set_config(pk_batch* batch, int block, int stack, int chunk);
int pk_batch_get_config(pk_batch* batch, int* block, int* stack, int* chunk);
/* Times every supported configuration on the first sample_paths paths of the
 * batch (0 = all), keeps the fastest, and clears the accumulation. */
int pk_batch_autotune(pk_batch* batch, uint64_t sample_paths, float* best_ms);
/* Renders `frames` frames of every request (graph replay); device time of the
 * call in pk_batch_info. */
int pk_batch_render(pk_batch* batch, uint32_t frames);
int pk_batch_reset(pk_batch* batch);
/* Mean radiance (width x height x 4 floats) of request `req` over the frames rendered. */
int pk_batch_read(pk_batch* batch, uint32_t req, float* rgba_mean);
int pk_batch_info(pk_batch* batch, uint64_t* total_paths, uint32_t* frames, float* last_ms);
/* Completion time of each request in the last rendered frame, in ms from the
 * start of that frame's launch (the lane that retires a request's last path
 * stamps the GPU global timer).  Requests are served in the order given, so
 * listing small requests first lowers the mean latency. */
int pk_batch_latencies(pk_batch* batch, float* ms);

#ifdef __cplusplus
}
#endif
#endif /* PIKE_H_ */
