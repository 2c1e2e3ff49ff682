// Multi-view kernel instantiation unit (see views.cuh).
#include "views.cuh"

namespace nedev {

// Per-pixel mean of every view's samples in sample order, into the concatenated images.
__global__ void k_reduce_views(const float* __restrict__ paths, const DView* __restrict__ views, uint32_t n_views,
                               uint32_t total_pixels, float* __restrict__ out) {
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < total_pixels; p += gridDim.x * blockDim.x) {
    uint32_t lo = 0, hi = n_views - 1;
    while (lo < hi) {
      uint32_t mid = (lo + hi + 1) >> 1;
      if (views[mid].pix_begin <= p) lo = mid;
      else hi = mid - 1;
    }
    const DView& v = views[lo];
    uint32_t local = p - v.pix_begin;
    const float* src = paths + 3 * (v.path_begin + (unsigned long long)local * v.spp);
    float r = 0, g = 0, b = 0;
    for (uint32_t k = 0; k < v.spp; k++) {
      r = r + src[3 * k + 0];
      g = g + src[3 * k + 1];
      b = b + src[3 * k + 2];
    }
    float fs = (float)v.spp;
    out[3 * (size_t)p + 0] = r / fs;
    out[3 * (size_t)p + 1] = g / fs;
    out[3 * (size_t)p + 2] = b / fs;
  }
}

}  // namespace nedev

cudaError_t ne_launch_views(bool split, int blocks, cudaStream_t st, const nedev::DScene& s,
                            const nedev::ViewArgs& a, unsigned long long* counter, uint32_t* err) {
  if (split)
    nedev::k_views<nedev::K_GENERAL | nedev::K_SPLIT><<<blocks, nedev::kThreads, 0, st>>>(s, a, counter, err);
  else
    nedev::k_views<nedev::K_GENERAL><<<blocks, nedev::kThreads, 0, st>>>(s, a, counter, err);
  return cudaGetLastError();
}

cudaError_t ne_views_occupancy(int* blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, nedev::k_views<nedev::K_GENERAL>,
                                                       nedev::kThreads, 0);
}

cudaError_t ne_launch_reduce_views(int blocks, cudaStream_t st, const float* paths, const nedev::DView* views,
                                   uint32_t n_views, uint32_t total_pixels, float* out) {
  nedev::k_reduce_views<<<blocks, 256, 0, st>>>(paths, views, n_views, total_pixels, out);
  return cudaGetLastError();
}
