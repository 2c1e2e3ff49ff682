// k_paths without work counters (the timed render kernel).
#include "kernels.cuh"

using namespace nedev;

cudaError_t ne_paths_occupancy(int* blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_paths<false>, kThreads, 0);
}

cudaError_t ne_launch_paths_plain(int blocks, cudaStream_t st, const DScene& s, const PathArgs& a,
                                  unsigned long long* counter, uint32_t* err) {
  k_paths<false><<<blocks, kThreads, 0, st>>>(s, a, counter, err);
  return cudaGetLastError();
}
