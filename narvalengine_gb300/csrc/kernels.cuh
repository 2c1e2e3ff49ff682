// Path kernels and their launchers. Each heavy kernel is instantiated in its own
// translation unit (k_paths_plain.cu, k_paths_count.cu, k_query.cu) so the build
// compiles them in parallel.
#pragma once
#include <cuda_runtime.h>

#include "narval_gb300.h"
#include "pt_device.cuh"
#include "pt_sched.cuh"

namespace nedev {

constexpr int kThreads = 128;

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
};

template <bool C>
__global__ void __launch_bounds__(kThreads) k_sched(const __grid_constant__ DScene s, const PathArgs a,
                                                    unsigned long long* __restrict__ counter, uint32_t* err) {
  schedLoop<C>(s, a.P, a.base, a.total, a.spp, a.sample_offset, a.cover_w, a.keys, a.out, counter, err,
               a.track_share);
}

template <bool C>
__device__ __forceinline__ void flushCounters(const Counters& cn, unsigned long long* g) {
  if (!C) return;
  unsigned long long v[4] = {cn.lookups, cn.queries, cn.nodes, cn.tests};
#pragma unroll
  for (int k = 0; k < 4; k++) {
    unsigned long long x = v[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0 && x) atomicAdd(&g[1 + k], x);
  }
}

// MINB > 1 caps registers per thread (65536 / (128 * MINB)) so more warps stay resident.
template <bool C, int MINB>
__global__ void __launch_bounds__(kThreads, MINB) k_paths(const __grid_constant__ DScene s, const PathArgs a,
                                                      unsigned long long* __restrict__ counter, uint32_t* err) {
  Ctx<C> c{s, Sampler{}, Counters{0, 0, 0, 0}, err};
  const int lane = threadIdx.x & 31;
  for (;;) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(&counter[0], 32ull);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= a.total) break;
    unsigned long long idx = base + (unsigned long long)lane;
    if (idx < a.total) {
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
  }
  flushCounters<C>(c.c, counter);
}


}  // namespace nedev

// Launchers (defined next to each kernel instantiation).
// variant: 0 = compiler's register choice, 1 = at most 80 registers, 2 = at most 64 registers,
// 3 = regrouped state-machine kernel (k_sched).
cudaError_t ne_launch_paths(bool count, int variant, int blocks, cudaStream_t st, const nedev::DScene& s,
                            const nedev::PathArgs& a, unsigned long long* counter, uint32_t* err);
cudaError_t ne_paths_occupancy(int variant, int* blocks_per_sm);
cudaError_t ne_launch_paths_variant(int variant, int blocks, cudaStream_t st, const nedev::DScene& s,
                                    const nedev::PathArgs& a, unsigned long long* counter, uint32_t* err);
cudaError_t ne_paths_occupancy_variant(int variant, int* blocks_per_sm);
cudaError_t ne_launch_sched(bool count, int blocks, cudaStream_t st, const nedev::DScene& s, const nedev::PathArgs& a,
                            unsigned long long* counter, uint32_t* err);
cudaError_t ne_sched_occupancy(int* blocks_per_sm);
cudaError_t ne_launch_li(int blocks, cudaStream_t st, const nedev::DScene& s, nedev::PathParams P, nerng::PathKey base,
                         const ne_ray* rays, const ne_path_key* keys, size_t n, uint32_t first_dim, float* out,
                         uint32_t* err);
cudaError_t ne_launch_closest(int blocks, cudaStream_t st, const nedev::DScene& s, const ne_ray* rays, size_t n,
                              float tmin, float tmax, ne_hit* out, uint32_t* err);
