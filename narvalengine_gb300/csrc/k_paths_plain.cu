// k_paths without work counters (the timed render kernel), compiler-chosen registers.
#include "kernels.cuh"

using namespace nedev;

cudaError_t ne_paths_occupancy(int variant, int* blocks_per_sm) {
  if (variant != 0) return ne_paths_occupancy_variant(variant, blocks_per_sm);
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_paths<false, 1>, kThreads, 0);
}

cudaError_t ne_launch_paths_plain(int variant, int blocks, cudaStream_t st, const DScene& s, const PathArgs& a,
                                  unsigned long long* counter, uint32_t* err) {
  if (variant != 0) return ne_launch_paths_variant(variant, blocks, st, s, a, counter, err);
  k_paths<false, 1><<<blocks, kThreads, 0, st>>>(s, a, counter, err);
  return cudaGetLastError();
}
