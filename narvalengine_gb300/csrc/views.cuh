// Many views of one scene in one persistent launch.
//
// The work of all views is one range of path indices: view v owns [begin[v], begin[v+1]),
// laid out pixel-major with spp consecutive samples per pixel as in k_paths. A launch covers
// the range of one group of consecutive views. Warps take `fetch` consecutive indices at a
// time from a global counter, so a warp's lanes share a view and usually a pixel, and views
// of every size drain through the same resident warps.
// The view the caller passed at index v uses random stream v + 1 (stream 0 is the
// single-camera render), so no two views share random numbers and the launch order does not
// change any image. Each view counts its finished paths (one atomic per group of
// lanes of the same view); the lane that completes the view stores the global timer, which
// with the launch's start time gives the view's completion latency.
#pragma once
#include "kernels.cuh"

namespace nedev {

struct DView {
  DCamera cam;
  int32_t width, height;
  uint32_t spp;
  uint32_t pix_begin;             // first pixel of this view in the concatenated images
  uint32_t stream;                // random stream: caller's view index + 1
  uint32_t pad;
  unsigned long long path_begin;  // first path index
  unsigned long long paths;
};

struct ViewArgs {
  PathParams P;
  nerng::PathKey base;
  const DView* views;       // in processing order
  uint32_t n_views;
  unsigned long long first; // path indices [first, total) of this launch (one group of views)
  unsigned long long total;
  uint32_t fetch;           // path indices per warp fetch, a multiple of 32
  float* out;               // total x 3 per-path radiance
  unsigned long long* done; // per view: finished paths
  unsigned long long* t_done;   // per view: global timer (ns) when its last path finished
  unsigned long long* t_start;  // global timer when the first warp started
  const DeferQueue* defer_out;  // split batches: queue of paths deferred at their first event
  int defer_half;               // 1: deferral points every half bounce
  int defer_top = 0;            // 1: every path is queued before its camera ray is intersected
};

// Index of the view owning path `idx` (views sorted by path_begin).
__device__ __forceinline__ uint32_t findView(const DView* v, uint32_t n, unsigned long long idx) {
  uint32_t lo = 0, hi = n - 1;
  while (lo < hi) {
    uint32_t mid = (lo + hi + 1) >> 1;
    if (v[mid].path_begin <= idx) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

template <uint32_t K>
__global__ void __launch_bounds__(kThreads, pathMinBlocks(K)) k_views(const __grid_constant__ DScene s,
                                                                    const ViewArgs a,
                                                                    unsigned long long* __restrict__ counter,
                                                                    uint32_t* err) {
  Ctx<K> c{s, Sampler{}, Counters{0, 0, 0, 0}, err, 0u, false, nullptr, a.defer_out, 0ull, false, 0, a.defer_half};
  c.deferTop = a.defer_top != 0;
  const int lane = threadIdx.x & 31;
  if (threadIdx.x == 0 && blockIdx.x == 0) atomicMin(a.t_start, globalTimer());
  for (;;) {
    unsigned long long base = 0;
    if (lane == 0) base = a.first + atomicAdd(&counter[0], (unsigned long long)a.fetch);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= a.total) break;
    for (uint32_t k = 0; k < a.fetch; k += 32) {
      unsigned long long idx = base + k + (unsigned long long)lane;
      bool live = idx < a.total;
      uint32_t v = live ? findView(a.views, a.n_views, idx) : 0xffffffffu;
      if (live) {
        const DView& vw = a.views[v];
        unsigned long long local = idx - vw.path_begin;
        uint32_t pixel = (uint32_t)(local / vw.spp), sample = (uint32_t)(local % vw.spp);
        if (K & K_SPLIT) {
          c.idx = idx;
          c.deferred = false;
        }
        V3 L = cameraPathCam(c, a.P, a.base, vw.cam, vw.width, vw.height, pixel, sample, vw.stream);
        if ((K & K_SPLIT) && c.deferred) {
          v = 0xffffffffu;  // counted when a resume pass finishes it
        } else {
          a.out[3 * idx + 0] = L.x;
          a.out[3 * idx + 1] = L.y;
          a.out[3 * idx + 2] = L.z;
        }
      }
      __syncwarp();
      unsigned same = __match_any_sync(0xffffffffu, v);
      if (v != 0xffffffffu && lane == __ffs(same) - 1) {
        unsigned long long n = (unsigned long long)__popc(same);
        unsigned long long before = atomicAdd(&a.done[v], n);
        if (before + n == a.views[v].paths) a.t_done[v] = globalTimer();
      }
    }
  }
}

}  // namespace nedev

// Launchers (k_views.cu): the general feature set covers every scene. split: the first pass
// of a split batch (paths deferred into a.defer_out at their first event).
cudaError_t ne_launch_views(bool split, int blocks, cudaStream_t st, const nedev::DScene& s,
                            const nedev::ViewArgs& a, unsigned long long* counter, uint32_t* err);
cudaError_t ne_views_occupancy(int* blocks_per_sm);
cudaError_t ne_launch_reduce_views(int blocks, cudaStream_t st, const float* paths, const nedev::DView* views,
                                   uint32_t n_views, uint32_t total_pixels, float* out);
