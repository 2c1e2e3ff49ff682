// k_paths with capped registers: 6 (<= 80 registers) or 8 (<= 64 registers) blocks of 128
// threads resident per SM, trading spills for more warps to hide lookup latency.
#include "kernels.cuh"

using namespace nedev;

cudaError_t ne_paths_occupancy_variant(int variant, int* blocks_per_sm) {
  if (variant == 1) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_paths<false, 6>, kThreads, 0);
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_paths<false, 8>, kThreads, 0);
}

cudaError_t ne_launch_paths_variant(int variant, int blocks, cudaStream_t st, const DScene& s, const PathArgs& a,
                                    unsigned long long* counter, uint32_t* err) {
  if (variant == 1)
    k_paths<false, 6><<<blocks, kThreads, 0, st>>>(s, a, counter, err);
  else
    k_paths<false, 8><<<blocks, kThreads, 0, st>>>(s, a, counter, err);
  return cudaGetLastError();
}
