// Path kernel instantiation unit (see kernels.cuh): grid-medium scenes rendered in two
// passes, paths that scatter deferred to the second.
#include "kernels.cuh"

namespace nedev {
constexpr uint32_t kSplitSet = K_VOLUME | K_SPLIT;
}  // namespace nedev

cudaError_t ne_launch_path_split(int pass, int blocks, cudaStream_t st, const nedev::DScene& s,
                                 const nedev::PathArgs& a, unsigned long long* counter, uint32_t* err) {
  if (pass == 0)
    nedev::k_paths<nedev::kSplitSet><<<blocks, nedev::kThreads, 0, st>>>(s, a, counter, err);
  else
    nedev::k_resume<nedev::kSplitSet><<<blocks, nedev::kThreads, 0, st>>>(s, a, counter, err);
  return cudaGetLastError();
}

cudaError_t ne_path_split_occupancy(int* blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, nedev::k_paths<nedev::kSplitSet>,
                                                       nedev::kThreads, 0);
}
