/*
 * C ABI of the GB300 path integrator (libnarval_gb300.so).
 *
 * It replaces the reference's CPU render path at the point where OfflineEngine
 * hands camera rays to the integrator:
 *   OfflineEngine::renderTile / coreLoop  (core/OfflineEngine.cpp:54-113)   -> ne_render
 *   Integrator::Li(Ray, Scene*)           (integrators/Integrator.h:13-25)   -> ne_li_batch
 *   Scene::intersectScene                 (core/Scene.cpp:30-56)            -> ne_trace_closest
 *   SceneReader::loadScene                (io/SceneReader.cpp:10-54)        -> ne_scene_host_load_json
 * Every function returns ne_status (0 = success, negative = failure) and never
 * aborts; the reference instead stops the process with LOG(FATAL) on bad input.
 * Buffers are owned by the caller; device memory of a scene is owned by the library.
 * A context owns one CUDA stream. A context and its scenes must not be used from
 * two threads at once; separate contexts are independent.
 */
#ifndef NARVAL_GB300_H_
#define NARVAL_GB300_H_

#include <stddef.h>
#include <stdint.h>
#include "narval_scene.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t ne_status;
#define NE_OK 0
#define NE_ERR_INVALID_ARG (-1)
#define NE_ERR_PARSE (-2)
#define NE_ERR_MISSING_ASSET (-3)
#define NE_ERR_CUDA (-4)
#define NE_ERR_TIMEOUT (-5)
#define NE_ERR_UNSUPPORTED (-6)
#define NE_ERR_NO_DEVICE (-7)
#define NE_ERR_OUT_OF_MEMORY (-8)

typedef struct ne_context ne_context;
typedef struct ne_scene ne_scene;
typedef struct ne_scene_host ne_scene_host;

/* A ray as the reference's Ray (primitives/Ray.h:17-32). */
typedef struct ne_ray {
  float o[3];
  float d[3];
} ne_ray;

/* Identity of a camera path: pixel = y * width + x, sample = index in the pixel. */
typedef struct ne_path_key {
  uint32_t pixel;
  uint32_t sample;
} ne_path_key;

/* Closest hit, the fields of RayIntersection (primitives/Ray.h:8-15) the integrator uses. */
typedef struct ne_hit {
  float t_near, t_far;
  float point[3];
  float normal[3];
  int32_t instance;  /* index into ne_scene_desc.instances, -1 on a miss */
  int32_t primitive; /* index into ne_scene_desc.prims, -1 on a miss */
  int32_t hit;       /* 1 when Scene::intersectScene returned true */
  int32_t pad;
} ne_hit;

/* ne_render_params.flags */
#define NE_RENDER_OUT_DEVICE (1u << 0)   /* out_rgb is device memory */
#define NE_RENDER_REF_TILES (1u << 1)    /* render only the 40x10 tile grid the reference covers */
#define NE_RENDER_COUNT_WORK (1u << 2)   /* count density lookups and scene queries (slower) */
#define NE_RENDER_NO_SYNC (1u << 3)      /* return after enqueueing; stats carry no timings */
#define NE_RENDER_DROP_NONFINITE (1u << 4) /* ne_render_accumulate: skip paths whose radiance is
                                              not finite (counted in dropped_paths) */

typedef struct ne_render_params {
  uint64_t seed;
  int32_t spp;            /* <= 0: SceneSettings::spp */
  int32_t bounces;        /* < 0: SceneSettings::bounces */
  int32_t rr;             /* < 0: scene setting, 0: off, 1: on */
  int32_t rr_after;       /* used when rr == 1 */
  uint32_t sample_offset; /* index of the first sample (progressive rendering) */
  uint32_t flags;
} ne_render_params;

typedef struct ne_render_stats {
  double kernel_ms;           /* CUDA-event time of the path kernel */
  double total_ms;            /* CUDA-event time of the whole call, copies included */
  uint64_t paths;             /* camera paths traced */
  uint64_t density_lookups;   /* trilinear density lookups (NE_RENDER_COUNT_WORK) */
  uint64_t scene_queries;     /* Scene::intersectScene calls (NE_RENDER_COUNT_WORK) */
  uint64_t bvh_nodes;         /* BVH nodes visited (NE_RENDER_COUNT_WORK) */
  uint64_t prim_tests;        /* ray-triangle tests (NE_RENDER_COUNT_WORK) */
  uint32_t kernel_launches;   /* kernels this call launched */
  uint32_t dropped_paths;     /* paths skipped by NE_RENDER_DROP_NONFINITE */
} ne_render_stats;

/* ---- host-side scene description (no GPU needed) ---- */

/* Parses a reference JSON scene descriptor (SceneReader semantics). resources_dir
 * plays the role of RESOURCES_DIR for relative asset paths (.vol and .vdb grids, textures). */
ne_status ne_scene_host_load_json(const char* path, const char* resources_dir, ne_scene_host** out,
                                  char* err, size_t err_len);
ne_status ne_scene_host_load_json_string(const char* json, const char* resources_dir, ne_scene_host** out,
                                         char* err, size_t err_len);
const ne_scene_desc* ne_scene_host_desc(const ne_scene_host* s);
/* Camera::Camera (core/Camera.cpp:7-26) as SceneReader sets it up (io/SceneReader.cpp:650-675:
 * aperture 0.0001, up (0, 1, 0)); focus 3 reproduces "autoFocus". For views built in code. */
ne_status ne_camera_look_at(const float position[3], const float look_at[3], float vfov_deg, int width,
                            int height, float focus, ne_camera* out);
void ne_scene_host_destroy(ne_scene_host* s);

/* Image files of a width*height*3 float image, row y*width+x (materials/Texture.h:44-75
 * saveImage): PNG with each channel clamped to [0, 1] and stored as (uint8)(v * 255), and EXR
 * with FP32 R, G, B channels. */
ne_status ne_save_png(const char* path, const float* rgb, int width, int height);
ne_status ne_save_exr(const char* path, const float* rgb, int width, int height);

/* Decodes an image file to 8-bit RGBA the way the reference loads textures (stbi_load with four
 * channels, core/ResourceManager.cpp:288-315): PNG (every colour type and bit depth, Adam7 or
 * not; 16-bit samples keep their high byte) and binary PNM (P5, P6). Sets width and height;
 * with out != NULL also copies the width*height*4 bytes (cap: bytes available). JPEG and HDR
 * files give NE_ERR_UNSUPPORTED. */
ne_status ne_image_load_rgba8(const char* path, int32_t* width, int32_t* height, uint8_t* out, size_t cap);

/* ---- device ---- */

ne_status ne_context_create(int device, ne_context** out);
/* Destroys the context and every scene still uploaded to it; their handles become invalid. */
void ne_context_destroy(ne_context* ctx);
const char* ne_last_error(const ne_context* ctx);
/* Device memory that scenes and renders release stays cached in the context for their
 * successors (no counterpart in the reference): at most `bytes` of it (by default a quarter
 * of the device's memory, at least 16 GiB); the excess is freed now, largest buffers first.
 * 0 frees the whole cache and caches nothing from then on. */
ne_status ne_context_set_cache_limit(ne_context* ctx, size_t bytes);

/* Copies a scene description to the device (grids, primitives, BVHs). */
ne_status ne_scene_upload(ne_context* ctx, const ne_scene_desc* desc, ne_scene** out);
void ne_scene_destroy(ne_scene* scene);

/* Renders every pixel (or the reference's tile grid) and writes the per-pixel mean
 * radiance, before tone mapping, as width*height*3 floats, pixel y*width+x. */
ne_status ne_render(ne_scene* scene, const ne_render_params* params, float* out_rgb, ne_render_stats* stats);

/* ne_render without allocation: no counterpart in the reference (whose CPU render
 * allocates freely). For callers that cannot call cudaMalloc while rendering: a host
 * application that has reserved the device's memory for its own pool (cudaMalloc then
 * fails) and frame loops that must not stall on cudaFree, which synchronises the device.
 * The image (width*height*3 floats, as ne_render) must be DEVICE memory owned by the
 * caller; NE_RENDER_OUT_DEVICE is implied and NE_RENDER_NO_SYNC is ignored (the call waits
 * for the render to read its error flag). Per-path
 * scratch comes from a fixed array of the library of NE_NOALLOC_MAX_PATHS paths (12 MiB),
 * held on every GPU that loads the library until the process exits; a call with more
 * paths (covered pixels x spp) fails with NE_ERR_INVALID_ARG. Kernel: the scene's tuned
 * path kernel, except that a scene tuned to the split kernel (kernel 3, the default after
 * ne_scene_autotune on most scenes) renders with the one-pass kernel (kernel 0) at that
 * kernel's occupancy: the split kernel's deferred-path queues are sized to the render and do
 * not fit the fixed array. The image is the same bits either way; the one-pass kernel is
 * several times slower on scenes with media (about 4x on the 512^2 x 64 spp medium scene).
 * The first call on a device after a context is created on it looks up the array's address
 * (cudaGetSymbolAddress) and should come before any stream capture. All calls on a device
 * share the array, which keeps the last call's contents: calls whose work overlaps on the GPU
 * (contexts on one device, unordered streams) race and must be serialised by the caller. */
#define NE_NOALLOC_MAX_PATHS (1u << 20)
ne_status ne_render_noalloc(ne_scene* scene, const ne_render_params* params, float* out_rgb_device,
                            ne_render_stats* stats);

/* Adds the radiance of samples [sample_offset, sample_offset + spp) of every pixel to a
 * width*height*3 FP64 accumulator, each path converted to double and summed in sample order
 * (for converged reference images; divide by the total sample count). With
 * NE_RENDER_OUT_DEVICE the accumulator is device memory, else host memory. */
ne_status ne_render_accumulate(ne_scene* scene, const ne_render_params* params, double* accum,
                               ne_render_stats* stats);

/* Camera path per key: camera ray (draws 0-3) then Li (draws from 4). out_L: n*3 floats. */
ne_status ne_trace_paths(ne_scene* scene, const ne_render_params* params, const ne_path_key* keys, size_t n,
                         float* out_L);

/* Integrator::Li for n given rays; draw numbering of each path starts at first_dim. */
ne_status ne_li_batch(ne_scene* scene, const ne_render_params* params, const ne_ray* rays,
                      const ne_path_key* keys, size_t n, uint32_t first_dim, float* out_L);

/* Scene::intersectScene for n rays with the given tMin/tMax. */
ne_status ne_trace_closest(ne_scene* scene, const ne_ray* rays, size_t n, float t_min, float t_max,
                           ne_hit* out);

/* Launch configuration of the path kernels of one scene (picked by an autotuner or by hand).
 * kernel: 0 = straight kernel (warps take 32 paths and run them to completion), 1 = regrouped
 * state-machine kernel (a warp steps tracking walks together while at least track_share/32 of
 * its live lanes are in one), 2 = straight kernel whose lanes take a new path as soon as
 * theirs ends, 3 = split: a first pass finishes every path that ends at its first event and
 * queues the others (at their first scattering in a grid medium, or after their first surface
 * bounce); each further pass resumes the queued paths packed together and queues them again
 * one bounce (or half a bounce) later, the last runs them to the end. blocks_per_sm:
 * persistent blocks per SM, 0 = as many as fit. Every configuration renders the same bits.
 * A new scene starts with kernel 3, split_half 1, 16 passes. */
typedef struct ne_tuning {
  int32_t kernel;
  int32_t track_share;
  int32_t blocks_per_sm;
  int32_t split_passes;  /* kernel 3: passes, 2..64 (0: 16 with split_half, else 8); pass p > 0
                            resumes the paths queued at deferral point p - 1 and queues them
                            again at point p, the last runs them to the end */
  int32_t split_half;    /* kernel 3: 0 = deferral points once a bounce (point b: bounce b's
                            scattering event in a medium, or the end of surface bounce b);
                            1 = every half bounce (point 2b: bounce b's free-flight sample,
                            2b + 1: the end of bounce b, after its light sampling), so passes
                            alternate between the two variable-length walks */
  int32_t queue_quarters; /* kernel 3: room for deferred paths, in quarters of the render's paths
                            (1..8, 0 = 3: two thirds for the paths whose next light is the first
                            kind, one third for the other); paths beyond it continue in the pass
                            that has them */
  int32_t pretrace;      /* kernel 3 by bounce (split_half 0), scenes without media: 1 = before
                            each resume pass, k_trace intersects the queued paths' bounce rays and
                            stores the hits, so the pass starts from them; 2 = the camera rays too
                            (a first pass queues every new path before its first intersection;
                            the queues then hold 1.5 x the render's paths); 3 = the light samples'
                            shadow rays too (a path stops at its visibility test and the next
                            pass runs that bounce again with the result: each pass takes a path
                            one traversal further). Same image */
} ne_tuning;

ne_status ne_scene_set_tuning(ne_scene* scene, const ne_tuning* tuning);
ne_status ne_scene_get_tuning(const ne_scene* scene, ne_tuning* tuning);
/* Autotuner: renders the scene with `params` under each candidate (straight, lane refill,
 * regrouped with thresholds of 8, 16 and 24 32nds, split with 3..24 passes by bounce or 12..32
 * by half bounce; resident blocks as many as fit), then, if a split configuration won, its
 * deferred-path capacity at 2 and 4 quarters; `repeats` timed renders after one warm-up each,
 * keeps the fastest path-kernel time and returns it. Every candidate renders the same bits. The
 * split kernel's best pass count depends on the number of paths a render has: tune with the
 * frame's own sample count. */
ne_status ne_scene_autotune(ne_scene* scene, const ne_render_params* params, int repeats, ne_tuning* best,
                            double* best_ms);

/* ---- timing utilities on the context's stream (for benchmarks) ---- */

/* Records CUDA event `slot` (0-7) on the context's stream. */
ne_status ne_context_event_record(ne_context* ctx, int slot);
/* Milliseconds between two recorded events; waits for the later one. */
ne_status ne_context_event_elapsed(ne_context* ctx, int slot_begin, int slot_end, float* ms);
ne_status ne_context_synchronize(ne_context* ctx);
/* Writes `bytes` of scratch memory on the context's stream, evicting the L2 cache. */
ne_status ne_context_flush_l2(ne_context* ctx, size_t bytes);
/* Read bandwidth of this GPU for a buffer of `bytes` (no counterpart in the reference; a
 * roofline denominator for benchmarks): one warm-up pass, then `iters` back-to-back launches
 * of a read-only kernel (16-byte loads that bypass L1, one CTA per SM times the resident
 * count), each reading the whole buffer as many times as makes at least 1 GiB, event-timed;
 * *gbs = bytes read / time. A buffer well inside the 129 MB L2 measures L2 bandwidth, one
 * well beyond it HBM bandwidth. */
ne_status ne_measure_read_bandwidth(ne_context* ctx, size_t bytes, int iters, double* gbs);
/* Rate of random 32-byte reads from a `bytes` buffer, the access a density-cell lookup makes
 * (two 16-byte loads of one 32-byte-aligned record at a hashed index): *reads_per_s, the best
 * over 2, 4, 8 and 16 independent reads in flight per thread, each timed over `iters` launches.
 * Sized like a scene's cell array, it is the ceiling for that scene's lookups; bytes / 32 must
 * fit in 32 bits. */
ne_status ne_measure_random_read(ne_context* ctx, size_t bytes, int iters, double* reads_per_s);

/* Device copies of the shared elementary functions, for bit-exactness checks.
 * fn: 0 log, 1 exp, 2 sin, 3 cos, 4 acos, 5 pow5, 6 atan2(x[i], x[i ^ 1]) (elements paired;
 * an unpaired last element is paired with 1), 7 log(1 - x) for draws x = k 2^-24. */
ne_status ne_debug_fmath(ne_context* ctx, int fn, const float* x, size_t n, float* out);

/* Device copy of the shared counter-based generator: u01 for (seed, pixel, sample, dim). */
ne_status ne_debug_rng(ne_context* ctx, uint64_t seed, const ne_path_key* keys, const uint32_t* dims, size_t n,
                       float* out);

/* ---- many views in one launch (no counterpart in the reference) ----
 * A batch of cameras over one scene, each with its own resolution and samples per pixel,
 * rendered by one persistent kernel launch (optionally replayed as a CUDA graph). Each view
 * uses its own random stream. Completion latency = time from the launch's first warp to the
 * view's last path. A batch belongs to its scene and is destroyed with it. */
typedef struct ne_view {
  ne_camera camera;
  int32_t width, height, spp, pad;
} ne_view;
typedef struct ne_views ne_views;
typedef struct ne_views_tuning {
  uint32_t fetch;          /* path indices a warp takes at a time, multiple of 32 (default 32) */
  int32_t blocks_per_sm;   /* resident blocks per SM, 0 = as many as fit */
  int32_t order;           /* views in the launch: 0 as given, 1 largest first, 2 smallest first */
  int32_t graph;           /* 1: capture the launch sequence once and replay it as a CUDA graph */
  int32_t split_passes;    /* as ne_tuning.split_passes: 1 = one pass, 2..64, 0 = 6 */
  int32_t split_half;      /* as ne_tuning.split_half: 1 = deferral points every half bounce */
  int32_t groups;          /* 1..16 (0 = 1): the views, in launch order, are cut into this many
                              groups of about equal paths, each run through all its passes
                              before the next starts, so the views of early groups complete
                              early (per-view latency) at some cost in throughput */
  int32_t pretrace;        /* 1: before each pass after the first, k_trace intersects the bounce
                              rays of the paths queued at the top of a bounce; 2: the camera rays
                              too (a first pass queues every path; the queues grow to the largest
                              group's paths) (as ne_tuning) */
} ne_views_tuning;
typedef struct ne_views_stats {
  double ms;               /* CUDA-event time of the batch */
  uint64_t paths;
  float latency_p50_ms, latency_p99_ms, latency_max_ms;
  uint32_t kernel_launches;  /* kernels per batch (a graph launch counts its kernels) */
} ne_views_stats;
ne_status ne_views_create(ne_scene* scene, const ne_view* views, uint32_t n, const ne_render_params* params,
                          ne_views** out);
void ne_views_destroy(ne_views* views);
ne_status ne_views_set_tuning(ne_views* views, const ne_views_tuning* tuning);
ne_status ne_views_get_tuning(const ne_views* views, ne_views_tuning* tuning);
/* Times every candidate configuration (fetch 32/128; largest-first order in one group, or
 * smallest-first order in 1, 2 or 4 groups; 8 passes by bounce or 12/16 by half bounce; as a
 * graph) `repeats` times after one warm-up batch; among those within 3% of the fastest it keeps
 * the one with the lowest median view latency, and returns it with its time. */
ne_status ne_views_autotune(ne_views* views, int repeats, ne_views_tuning* best, double* best_ms);
ne_status ne_views_render(ne_views* views, ne_views_stats* stats);
/* Completion latency of each view of the last batch, in the caller's order (n floats, ms). */
ne_status ne_views_latency(const ne_views* views, float* ms);
/* Per-pixel mean radiance of view v of the last batch (width*height*3 floats, host memory). */
ne_status ne_views_image(const ne_views* views, uint32_t v, float* out_rgb);

/* ---- learned radiance cache (no counterpart in the reference) ----
 * A small network (features 96 -> 4 x 64 ReLU -> RGB) that predicts the radiance a medium
 * path would still gather from a scattering vertex (position in the medium's object space,
 * incoming direction), trained online on the integrator's own path suffixes with BF16
 * tensor-core products and FP32 accumulation. Parameters: NE_CACHE_PARAMS floats, per layer
 * W[out][in] then b[out] (96->64, 64->64 x3, 64->16 with output rows 0..2 = RGB). Arrays are
 * host memory unless NE_CACHE_DEVICE_PTRS is set. A context destroys its caches with it. */
typedef struct ne_cache ne_cache;
#define NE_CACHE_PARAMS 19728
#define NE_CACHE_DEVICE_PTRS (1u << 0)
/* He-uniform initial weights from `seed`, zero biases, Adam state cleared. */
ne_status ne_cache_create(ne_context* ctx, uint64_t seed, ne_cache** out);
void ne_cache_destroy(ne_cache* cache);
/* Replaces the parameters and clears the optimiser state. */
ne_status ne_cache_set_params(ne_cache* cache, const float* params);
ne_status ne_cache_get_params(ne_cache* cache, float* params);
/* The 96 input features of n queries (pos: n*3 object-space positions, dirs: n*3 unit). */
ne_status ne_cache_encode(ne_cache* cache, const float* pos, const float* dirs, size_t n, float* feats);
/* Raw network outputs (n*3). Queries as pos/dirs, or as precomputed features (n*96). */
ne_status ne_cache_infer(ne_cache* cache, const float* pos, const float* dirs, const float* feats, size_t n,
                         float* rgb, uint32_t flags);
/* One training step on n samples (targets n*3): forward, relative-L2 loss, backward, and
 * with apply != 0 an Adam step (lr 1e-2, betas 0.9/0.99). loss (optional) receives the mean
 * loss, grads (optional, NE_CACHE_PARAMS) the summed gradient. */
ne_status ne_cache_train(ne_cache* cache, const float* pos, const float* dirs, const float* feats,
                         const float* targets, size_t n, int apply, float* loss, float* grads, uint32_t flags);

/* Rendering with the cache: paths reaching a scattering vertex in a grid medium at or
 * after `bounce` stop there and add throughput x cache(vertex); one path in train_stride
 * (hashed over the path index) runs to the end instead, contributes its full radiance, and
 * records the radiance it gathered after that vertex as a training sample. After the image
 * is formed the cache takes train_steps optimiser steps on the frame's samples. */
typedef struct ne_cache_render_params {
  int32_t bounce;         /* 2: paths end at their third scattering event */
  uint32_t train_stride;  /* 0: no training paths */
  int32_t train_steps;
  uint32_t train_batch;   /* samples per optimiser step; 0: all of the frame's samples */
  int32_t train_suffix;   /* 0: a training path runs to its end; n > 0: it ends in the cache too,
                             at its first scattering vertex n or more bounces after the recorded
                             one: it adds throughput x cache(end vertex) to the image, and its
                             training sample's target gets (throughput ratio) x cache(end vertex)
                             added (the network's own prediction for the rest of the path) */
} ne_cache_render_params;
typedef struct ne_cache_render_stats {
  uint64_t queries;        /* paths that ended in the cache */
  uint64_t train_samples;  /* training samples recorded this frame */
  float loss;              /* mean loss of the last optimiser step (0 without training) */
  float path_ms, infer_ms, train_ms;
} ne_cache_render_stats;
/* As ne_render (same flags, output and stats) for scenes whose media are grid media;
 * NE_ERR_UNSUPPORTED for other scenes. */
ne_status ne_render_cached(ne_scene* scene, ne_cache* cache, const ne_render_params* params,
                           const ne_cache_render_params* cache_params, float* out_rgb, ne_render_stats* stats,
                           ne_cache_render_stats* cache_stats);

/* BVH::init (primitives/BVH.cpp:6-106) as ne_scene_upload builds it, on the host (no GPU
 * needed), over triangles prims[first, first + count): 9 words per node (min, max, then start,
 * count, rightOffset as uint32 bits) and the primitive order. */
ne_status ne_debug_bvh(const ne_primitive* prims, uint32_t first, uint32_t count, float* nodes, size_t cap,
                       uint32_t* order, size_t* n_nodes);

/* The world-space boxes ne_scene_upload bounds the scene's media with (on the host, no GPU
 * needed): 6 floats per box (min xyz, max xyz), `cap` boxes at most. The kernels for meshes with
 * media skip intersectTr's walk (integrators/VolumetricPathIntegrator.cpp:10-32) for an MIS ray
 * whose line misses every box. *n_boxes = -1: no boxes (every ray walks); 0: no medium. */
ne_status ne_debug_medium_boxes(const ne_scene_desc* desc, float* boxes, size_t cap, int32_t* n_boxes);

/* The BVH of model `model` of an uploaded scene, read back from the device in ne_debug_bvh's
 * format (an interior node's start and count are 0) with its primitive order (the model's
 * prim_count global primitive indices). nodes = NULL: sets *n_nodes only (0: no BVH). Lets a
 * CPU check traverse the tree the GPU built ("bvh": "sah"). */
ne_status ne_scene_bvh(const ne_scene* scene, uint32_t model, float* nodes, size_t cap, uint32_t* order,
                       size_t* n_nodes);

/* Failure detection of the tensor-core kernels' bounded waits (no counterpart in the
 * reference, a test hook): one block allocates tensor memory, initialises an mbarrier as the
 * radiance-cache kernels do, and waits for a completion that nothing signals, giving up after
 * `max_polls` (1 .. 2^20) polls instead of the kernels' 2^24. Returns NE_ERR_TIMEOUT, with the
 * tensor memory released and the context usable, when the wait ran out as intended. */
ne_status ne_debug_wait_timeout(ne_context* ctx, uint32_t max_polls);

/* One 128 x n x k tensor-core product D = A * B^T (BF16 bit patterns, row-major A[128][k],
 * B[n][k]; FP32 D[128][n]) through the same shared-memory and tensor-memory conventions as
 * the radiance-cache kernels. n in 16..256 step 16, k in 16..128 step 16. */
ne_status ne_debug_mma(ne_context* ctx, const uint16_t* a, const uint16_t* b, int n, int k, float* d);
/* The same product with operands staged in the MN-major layout the radiance-cache backward
 * pass reads transposed operands through: layout bit 0 = A, bit 1 = B; n, k in 16..64,
 * multiples of 16. */
ne_status ne_debug_mma_layout(ne_context* ctx, const uint16_t* a, const uint16_t* b, int n, int k, uint32_t layout,
                              float* d);

#ifdef __cplusplus
}
#endif

#endif /* NARVAL_GB300_H_ */
