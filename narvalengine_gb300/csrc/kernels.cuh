// Path kernels and their launchers.
//
// Two path kernels: k_paths (straight: one path per lane to completion, warps take 32
// work items at a time) and k_sched (regrouped state machine, pt_sched.cuh). Each is
// specialised on the scene's feature set K (pt_device.cuh: K_VOLUME, K_SURFACE, K_MESH,
// K_GENERAL) and instantiated in its own translation unit (k_path_<kernel>_<set>.cu) so the
// build compiles them in parallel; the counting variants (K | K_COUNT) use K_GENERAL.
#pragma once
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "narval_gb300.h"
#include "pt_device.cuh"
#include "pt_sched.cuh"

namespace nedev {

constexpr int kThreads = 128;
// Resident blocks per SM the path kernels are compiled for: 7 x 128 threads caps them at 72
// registers. The spills this costs are cheaper than the latency stalls that fewer resident
// warps leave exposed. Measured (Mpaths/s, medium / dense cloud / Cornell / mesh, split by half
// bounce): 6 blocks 1467 / 286 / 581 / 156, 7 blocks 1530 / 304 / 561 / 169, 8 blocks
// 1468 / 309 / 558 / 170, 10 blocks 1350 / 282 / 531 / 176; split by bounce (medium /
// Cornell / dense cloud): 6 blocks 1338 / 589 / 264, 8 blocks 1316 / 573 / 282, 10 blocks
// 1186 / 546 / 252; one pass (medium / mesh): uncapped 123 registers 339 / 113, 8 blocks
// 383 / 127, 10 blocks 397 / 139.
#ifndef NE_PATH_MIN_BLOCKS
#define NE_PATH_MIN_BLOCKS 7
#endif
constexpr int kPathMinBlocks = NE_PATH_MIN_BLOCKS;
#ifndef NE_MESH_MIN_BLOCKS
#define NE_MESH_MIN_BLOCKS 16
#endif
#ifndef NE_MESH_MEDIA_MIN_BLOCKS
#define NE_MESH_MEDIA_MIN_BLOCKS 16
#endif
#ifndef NE_SURFACE_MIN_BLOCKS
#define NE_SURFACE_MIN_BLOCKS 7
#endif
// Triangle meshes run best with as many resident warps as an SM holds (16 blocks of 128
// threads, a 32-register cap) to hide their instruction-fetch and traversal latency, despite
// the spills: without media (the mesh feature set; mesh scene: 6 blocks 373, 8 416, 10 443,
// 12 471, 16 502 Mpaths/s) and with media (the general set; 64 views of the medium and the
// mesh: 8 blocks 104, 16 blocks 126). Surfaces without meshes or media (the surface set;
// Cornell box: 7 blocks 947, 16 blocks 836) and volumes: 7.
__host__ __device__ constexpr int pathMinBlocks(uint32_t K) {
  return (K & FT_TRI) ? ((K & FT_GRID) ? NE_MESH_MEDIA_MIN_BLOCKS : NE_MESH_MIN_BLOCKS)
                      : ((K & (FT_GRID | FT_HOMOG | FT_VOLBSDF)) ? kPathMinBlocks : NE_SURFACE_MIN_BLOCKS);
}

// Per-view completion accounting of a batch of views (see views.cuh): the path range of
// every view in launch order, finished-path counts and completion times.
struct ViewSpan {
  unsigned long long path_begin, paths;
};
struct ViewDone {
  const ViewSpan* spans;
  uint32_t n;
  unsigned long long* done;
  unsigned long long* t_done;
};

__device__ __forceinline__ unsigned long long globalTimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t findSpan(const ViewSpan* v, uint32_t n, unsigned long long idx) {
  uint32_t lo = 0, hi = n - 1;
  while (lo < hi) {
    uint32_t mid = (lo + hi + 1) >> 1;
    if (v[mid].path_begin <= idx) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Counts finished paths per view (one atomic per group of lanes of the same view; all 32
// lanes call it, `v` = 0xffffffff for lanes without a finished path) and stamps the time of
// each view's last path.
__device__ __forceinline__ void countViewDone(const ViewDone& vd, uint32_t v) {
  unsigned same = __match_any_sync(0xffffffffu, v);
  const int lane = threadIdx.x & 31;
  if (v != 0xffffffffu && lane == __ffs(same) - 1) {
    unsigned long long n = (unsigned long long)__popc(same);
    unsigned long long before = atomicAdd(&vd.done[v], n);
    if (before + n == vd.spans[v].paths) vd.t_done[v] = globalTimer();
  }
}

struct PathArgs {
  PathParams P;
  nerng::PathKey base;
  unsigned long long total;  // work items
  uint32_t spp;
  uint32_t sample_offset;
  uint32_t cover_w;          // rendered rectangle width (pixels)
  const ne_path_key* keys;   // explicit keys (ne_trace_paths) or null
  float* out;                // total * 3 floats
  int track_share;           // regrouped kernel: tracking-phase threshold in 32nds of live lanes
  const CacheIO* cache = nullptr;  // K_CACHE kernels: device copy of the cache buffers
  // K_SPLIT kernels: queues (device memory) the pass reads from and defers into, and the
  // bounce at whose scattering event paths are deferred (-1: run to the end)
  const DeferQueue* defer_in = nullptr;
  const DeferQueue* defer_out = nullptr;
  int defer_at = -1;
  int defer_half = 0;  // 1: deferral points every half bounce
  // first pass of a split render whose bounce rays are traced ahead (k_trace): every path
  // stops at the top of bounce 0, before its camera ray is intersected
  int defer_top = 0;
  // resume passes of a surface scene whose shadow rays are traced ahead too: a path stops at
  // its light sample's visibility test (and at the end of every bounce)
  int defer_shadow = 0;
  const ViewDone* views = nullptr;  // resume passes of a batch of views: completion accounting
};

// Training paths of a cached render: a multiplicative hash of the path index, so training
// paths spread over pixels and samples.
__device__ __forceinline__ bool isTrainingPath(unsigned long long idx, uint32_t stride) {
  return stride && (((uint32_t)idx * 0x9E3779B1u) >> 8) % stride == 0;
}

template <uint32_t K>
__global__ void __launch_bounds__(kThreads) k_sched(const __grid_constant__ DScene s, const PathArgs a,
                                                    unsigned long long* __restrict__ counter, uint32_t* err) {
  schedLoop<K>(s, a.P, a.base, a.total, a.spp, a.sample_offset, a.cover_w, a.keys, a.out, counter, err,
               a.track_share);
}

template <uint32_t K>
__device__ __forceinline__ void flushCounters(const Counters& cn, unsigned long long* g) {
  if (!(K & K_COUNT)) return;
  unsigned long long v[4] = {cn.lookups, cn.queries, cn.nodes, cn.tests};
#pragma unroll
  for (int k = 0; k < 4; k++) {
    unsigned long long x = v[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0 && x) atomicAdd(&g[1 + k], x);
  }
}

template <uint32_t K>
__global__ void __launch_bounds__(kThreads, pathMinBlocks(K)) k_paths(const __grid_constant__ DScene s, const PathArgs a,
                                                    unsigned long long* __restrict__ counter, uint32_t* err) {
  Ctx<K> c{s, Sampler{}, Counters{0, 0, 0, 0}, err, 0u, false, a.cache, a.defer_out, 0ull, false, a.defer_at,
           a.defer_half};
  c.deferTop = a.defer_top != 0;
  const int lane = threadIdx.x & 31;
  for (;;) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(&counter[0], 32ull);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= a.total) break;
    unsigned long long idx = base + (unsigned long long)lane;
    if (idx < a.total) {
      if (K & K_CACHE) {
        c.pidx = (uint32_t)idx;
        c.train = isTrainingPath(idx, a.cache->train_stride);
      }
      if (K & K_SPLIT) {
        c.idx = idx;
        c.deferred = false;
      }
      uint32_t pixel, sample;
      if (a.keys) {
        ne_path_key k = a.keys[idx];
        pixel = k.pixel;
        sample = k.sample + a.sample_offset;
      } else {
        uint32_t pi = (uint32_t)(idx / a.spp);
        sample = (uint32_t)(idx % a.spp) + a.sample_offset;
        pixel = (pi / a.cover_w) * (uint32_t)s.width + (pi % a.cover_w);
      }
      V3 L = cameraPath(c, a.P, a.base, pixel, sample);
      if (!((K & K_SPLIT) && c.deferred)) {
        a.out[3 * idx + 0] = L.x;
        a.out[3 * idx + 1] = L.y;
        a.out[3 * idx + 2] = L.z;
      }
    }
  }
  flushCounters<K>(c.c, counter);
}

// Later passes of a split render: warps take 32 deferred paths at a time from the input
// queue and run each from its saved scattering point, deferring it again at the scattering
// event of bounce a.defer_at (or running it to the end when that is -1): the same operations
// and draws as an undivided path.
template <uint32_t K>
__global__ void __launch_bounds__(kThreads, pathMinBlocks(K)) k_resume(const __grid_constant__ DScene s,
                                                                     const PathArgs a,
                                                                     unsigned long long* __restrict__ counter,
                                                                     uint32_t* err) {
  Ctx<K> c{s, Sampler{}, Counters{0, 0, 0, 0}, err, 0u, false, a.cache, a.defer_out, 0ull, false, a.defer_at,
           a.defer_half};
  c.deferShadow = a.defer_shadow != 0;
  const DeferQueue& q = *a.defer_in;
  const unsigned long long n0 = min(*q.count, q.cap);
  const unsigned long long n = n0 + (q.count_hi ? min(*q.count_hi, q.cap_hi) : 0u);
  const int lane = threadIdx.x & 31;
  for (;;) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(&counter[0], 32ull);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= n) break;
    unsigned long long i = base + (unsigned long long)lane;
    uint32_t finishedView = 0xffffffffu;
    if (i < n) {
      const PathState ps = loadState(q, i < n0 ? i : q.cap + (i - n0));
      LiVars v = ps.v;
      c.S.reset(ps.key, ps.dim);
      c.idx = ps.idx;
      c.deferred = false;
      if (K & K_CACHE) {
        c.pidx = (uint32_t)ps.idx;
        c.train = isTrainingPath(ps.idx, a.cache->train_stride);
      }
      // hit known (3, and 5-7: a stop at a shadow ray comes after the bounce's hit), no hit (4);
      // a shadow ray's result known (6 visible, 7 blocked)
      const int pre = (ps.mode == kModeHit || ps.mode >= kModeShadow) ? 1 : (ps.mode == kModeMiss ? 2 : 0);
      c.shadowVis = ps.mode == kModeVisible ? 1 : (ps.mode == kModeBlocked ? 2 : 0);
      c.shadowSlot = -1;
      V3 L = liLoop(c, a.P, v, ps.mode == 0, pre);
      if (!c.deferred) {
        a.out[3 * ps.idx + 0] = L.x;
        a.out[3 * ps.idx + 1] = L.y;
        a.out[3 * ps.idx + 2] = L.z;
        if (a.views) finishedView = findSpan(a.views->spans, a.views->n, ps.idx);
      }
    }
    if (a.views) {
      __syncwarp();
      countViewDone(*a.views, finishedView);
    }
  }
}

// The bounce rays of a queue of paths deferred at the top of a bounce (mode 1), intersected
// ahead of the pass that resumes them: Scene::intersectScene per ray, the hit stored into the
// path's state (mode 3, or 4 for no hit) so that the resume skips the call. The warps run
// nothing but the traversal. Each path's words 1, 2 (the ray), 4-6 (the previous hit, which a
// miss leaves in place but for its primitive) and 9 (the mode) are read, words 4-6 and 9
// written back. In surface-only kernels a path stopped at its light sample's visibility test
// (mode 5) gets the test's answer (visibilityTr from the hit to the point on the light in word
// 3; mode 6 visible, 7 blocked), and only word 9 is written.
template <uint32_t K>
__global__ void __launch_bounds__(kThreads, 8) k_trace(const __grid_constant__ DScene s, const DeferQueue* qp,
                                                  unsigned long long* __restrict__ counter, uint32_t* err) {
  Ctx<K> c{s, Sampler{}, Counters{0, 0, 0, 0}, err, 0u, false, nullptr, nullptr, 0ull, false, -1, 0};
  const DeferQueue q = *qp;
  const unsigned long long n0 = min(*q.count, q.cap);
  const unsigned long long n = n0 + (q.count_hi ? min(*q.count_hi, q.cap_hi) : 0u);
  const size_t plane = (size_t)q.cap + q.cap_hi;
  uint4* words = reinterpret_cast<uint4*>(q.items);
  const float inf = __int_as_float(0x7f800000);
  for (;;) {
    const int lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(&counter[0], 32ull);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= n) break;
    const unsigned long long i = base + (unsigned long long)lane;
    if (i >= n) continue;
    const size_t e = i < n0 ? i : q.cap + (i - n0);
    uint4 w9 = words[9 * plane + e];
    if constexpr (shadowQueue<K>()) {
      if (w9.x == kModeShadow) {
        // the light sample's visibility test: visibilityTr from the hit to the point on the light
        const uint4 w3 = words[3 * plane + e], w4 = words[4 * plane + e], w5 = words[5 * plane + e];
        const V3 p = v3(__uint_as_float(w4.z), __uint_as_float(w4.w), __uint_as_float(w5.x));
        const V3 lightPoint = v3(__uint_as_float(w3.x), __uint_as_float(w3.y), __uint_as_float(w3.z));
        w9.x = isBlack(visibilityTr(c, p, lightPoint)) ? kModeBlocked : kModeVisible;
        words[9 * plane + e] = w9;
        continue;
      }
    }
    if (w9.x != kModeTop) continue;
    const uint4 w1 = words[1 * plane + e], w2 = words[2 * plane + e];
    uint4 w4 = words[4 * plane + e];
    const uint4 w5 = words[5 * plane + e], w6 = words[6 * plane + e];
    Ray ray{v3(__uint_as_float(w1.z), __uint_as_float(w1.w), __uint_as_float(w2.x)),
            v3(__uint_as_float(w2.y), __uint_as_float(w2.z), __uint_as_float(w2.w))};
    Hit h;
    h.hitPoint = v3(__uint_as_float(w4.z), __uint_as_float(w4.w), __uint_as_float(w5.x));
    h.normal = v3(__uint_as_float(w5.y), __uint_as_float(w5.z), __uint_as_float(w5.w));
    h.tNear = __uint_as_float(w6.x);
    h.tFar = __uint_as_float(w6.y);
    h.inst = (int)w6.z;
    h.prim = (int)w6.w;
    const bool did = intersectScene(c, ray, h, kEps12F, inf);
    w4.z = __float_as_uint(h.hitPoint.x);
    w4.w = __float_as_uint(h.hitPoint.y);
    words[4 * plane + e] = w4;
    words[5 * plane + e] = make_uint4(__float_as_uint(h.hitPoint.z), __float_as_uint(h.normal.x),
                                      __float_as_uint(h.normal.y), __float_as_uint(h.normal.z));
    words[6 * plane + e] = make_uint4(__float_as_uint(h.tNear), __float_as_uint(h.tFar), (uint32_t)h.inst,
                                      (uint32_t)h.prim);
    w9.x = did ? kModeHit : kModeMiss;
    words[9 * plane + e] = w9;
  }
}

// Straight kernel with lane-level refill: a lane that finishes its path takes the next
// work item at once, together with whichever lanes finish at the same time (coalesced-group
// atomic), instead of waiting for the longest path of its warp.
template <uint32_t K>
__global__ void __launch_bounds__(kThreads, pathMinBlocks(K)) k_lanes(const __grid_constant__ DScene s, const PathArgs a,
                                                    unsigned long long* __restrict__ counter, uint32_t* err) {
  namespace cg = cooperative_groups;
  Ctx<K> c{s, Sampler{}, Counters{0, 0, 0, 0}, err, 0u, false, nullptr, nullptr, 0ull, false, -1, 0};
  for (;;) {
    cg::coalesced_group g = cg::coalesced_threads();
    unsigned long long base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(&counter[0], (unsigned long long)g.size());
    unsigned long long idx = g.shfl(base, 0) + g.thread_rank();
    if (idx >= a.total) break;
    uint32_t pixel, sample;
    if (a.keys) {
      ne_path_key k = a.keys[idx];
      pixel = k.pixel;
      sample = k.sample + a.sample_offset;
    } else {
      uint32_t pi = (uint32_t)(idx / a.spp);
      sample = (uint32_t)(idx % a.spp) + a.sample_offset;
      pixel = (pi / a.cover_w) * (uint32_t)s.width + (pi % a.cover_w);
    }
    V3 L = cameraPath(c, a.P, a.base, pixel, sample);
    a.out[3 * idx + 0] = L.x;
    a.out[3 * idx + 1] = L.y;
    a.out[3 * idx + 2] = L.z;
  }
  __syncwarp();
  flushCounters<K>(c.c, counter);
}

// One launcher per (kernel, feature set); KERNEL 0 = k_paths, 1 = k_sched, 2 = k_lanes.
template <int KERNEL, uint32_t K>
cudaError_t launchPathKernel(int blocks, cudaStream_t st, const DScene& s, const PathArgs& a,
                             unsigned long long* counter, uint32_t* err) {
  if (KERNEL == 0)
    k_paths<K><<<blocks, kThreads, 0, st>>>(s, a, counter, err);
  else if (KERNEL == 1)
    k_sched<K><<<blocks, kThreads, 0, st>>>(s, a, counter, err);
  else
    k_lanes<K><<<blocks, kThreads, 0, st>>>(s, a, counter, err);
  return cudaGetLastError();
}

template <int KERNEL, uint32_t K>
cudaError_t pathKernelOccupancy(int* blocks_per_sm) {
  if (KERNEL == 0) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_paths<K>, kThreads, 0);
  if (KERNEL == 1) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_sched<K>, kThreads, 0);
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_lanes<K>, kThreads, 0);
}

#define NE_PATH_KERNEL_INSTANCE(EXT, KERNEL, K)                                                              \
  EXT template cudaError_t launchPathKernel<KERNEL, K>(int, cudaStream_t, const DScene&, const PathArgs&,    \
                                                       unsigned long long*, uint32_t*);                      \
  EXT template cudaError_t pathKernelOccupancy<KERNEL, K>(int*);

#define NE_PATH_KERNEL_ALL(EXT)                          \
  NE_PATH_KERNEL_INSTANCE(EXT, 0, K_VOLUME)              \
  NE_PATH_KERNEL_INSTANCE(EXT, 0, K_SURFACE)             \
  NE_PATH_KERNEL_INSTANCE(EXT, 0, K_MESH)                \
  NE_PATH_KERNEL_INSTANCE(EXT, 0, K_GENERAL)             \
  NE_PATH_KERNEL_INSTANCE(EXT, 1, K_VOLUME)              \
  NE_PATH_KERNEL_INSTANCE(EXT, 1, K_SURFACE)             \
  NE_PATH_KERNEL_INSTANCE(EXT, 1, K_MESH)                \
  NE_PATH_KERNEL_INSTANCE(EXT, 1, K_GENERAL)             \
  NE_PATH_KERNEL_INSTANCE(EXT, 2, K_VOLUME)              \
  NE_PATH_KERNEL_INSTANCE(EXT, 2, K_SURFACE)             \
  NE_PATH_KERNEL_INSTANCE(EXT, 2, K_MESH)                \
  NE_PATH_KERNEL_INSTANCE(EXT, 2, K_GENERAL)             \
  NE_PATH_KERNEL_INSTANCE(EXT, 0, K_GENERAL | K_COUNT)   \
  NE_PATH_KERNEL_INSTANCE(EXT, 1, K_GENERAL | K_COUNT)   \
  NE_PATH_KERNEL_INSTANCE(EXT, 2, K_GENERAL | K_COUNT)

// Declared here, instantiated in the k_path_*.cu units only.
NE_PATH_KERNEL_ALL(extern)

}  // namespace nedev

// Dispatch over the instantiated kernels. features: the scene's FT_* bits; the smallest
// compiled set covering them is used (K_GENERAL covers everything).
uint32_t ne_feature_set_for(uint32_t features);
cudaError_t ne_launch_path_kernel(int kernel, uint32_t set, bool count, int blocks, cudaStream_t st,
                                  const nedev::DScene& s, const nedev::PathArgs& a, unsigned long long* counter,
                                  uint32_t* err);
cudaError_t ne_path_kernel_occupancy(int kernel, uint32_t set, int* blocks_per_sm);
// Split render (kernel 3) of a feature set: pass 0 = the first pass (k_paths deferring at
// bounce a.defer_at into a.defer_out), else a resume pass over a.defer_in; counter[0] must be
// zero before each.
cudaError_t ne_launch_path_split(int pass, uint32_t set, int blocks, cudaStream_t st, const nedev::DScene& s,
                                 const nedev::PathArgs& a, unsigned long long* counter, uint32_t* err);
cudaError_t ne_path_split_occupancy(uint32_t set, int* blocks_per_sm);
namespace nedev {
// Bounce rays of the paths a surface split pass queued at the top of a bounce (k_trace), one
// wave of resident blocks on `sm_count` SMs; counter[0] must be zero before the launch.
cudaError_t launchTrace_mesh(int sm_count, cudaStream_t st, const DScene& s, const DeferQueue* q,
                             unsigned long long* counter, uint32_t* err);
cudaError_t launchTrace_surface(int sm_count, cudaStream_t st, const DScene& s, const DeferQueue* q,
                                unsigned long long* counter, uint32_t* err);
cudaError_t launchTrace_general(int sm_count, cudaStream_t st, const DScene& s, const DeferQueue* q,
                                unsigned long long* counter, uint32_t* err);
}  // namespace nedev
// Grid-medium scenes with paths ending in the radiance cache, split like kernel 3: pass 0 =
// first pass, else a resume pass (see ne_launch_path_split).
cudaError_t ne_launch_path_kernel_cache(int pass, int blocks, cudaStream_t st, const nedev::DScene& s,
                                        const nedev::PathArgs& a, unsigned long long* counter, uint32_t* err);
cudaError_t ne_path_cache_occupancy(int* blocks_per_sm);
cudaError_t ne_launch_li(int blocks, cudaStream_t st, const nedev::DScene& s, nedev::PathParams P, nerng::PathKey base,
                         const ne_ray* rays, const ne_path_key* keys, size_t n, uint32_t first_dim, float* out,
                         uint32_t* err);
cudaError_t ne_launch_closest(int blocks, cudaStream_t st, const nedev::DScene& s, const ne_ray* rays, size_t n,
                              float tmin, float tmax, ne_hit* out, uint32_t* err);
