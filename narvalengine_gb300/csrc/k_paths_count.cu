// k_paths with work counters (density lookups, scene queries, BVH nodes, primitive
// tests), used to measure the algorithmic traffic of a render outside the timed run.
#include "kernels.cuh"

using namespace nedev;

cudaError_t ne_launch_paths_plain(int variant, int blocks, cudaStream_t st, const DScene& s, const PathArgs& a,
                                  unsigned long long* counter, uint32_t* err);

cudaError_t ne_launch_paths(bool count, int variant, int blocks, cudaStream_t st, const DScene& s, const PathArgs& a,
                            unsigned long long* counter, uint32_t* err) {
  if (!count) return ne_launch_paths_plain(variant, blocks, st, s, a, counter, err);
  k_paths<true, 1><<<blocks, kThreads, 0, st>>>(s, a, counter, err);
  return cudaGetLastError();
}
