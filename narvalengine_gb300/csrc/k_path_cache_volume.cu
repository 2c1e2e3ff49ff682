// Path kernel instantiation unit (see kernels.cuh): grid-medium scenes, paths ending in
// the learned radiance cache, rendered in split passes.
#include "kernels.cuh"

cudaError_t ne_launch_path_kernel_cache(int pass, int blocks, cudaStream_t st, const nedev::DScene& s,
                                        const nedev::PathArgs& a, unsigned long long* counter, uint32_t* err) {
  constexpr uint32_t K = nedev::K_VOLUME | nedev::K_CACHE | nedev::K_SPLIT;
  if (pass == 0)
    nedev::k_paths<K><<<blocks, nedev::kThreads, 0, st>>>(s, a, counter, err);
  else
    nedev::k_resume<K><<<blocks, nedev::kThreads, 0, st>>>(s, a, counter, err);
  return cudaGetLastError();
}

cudaError_t ne_path_cache_occupancy(int* blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      blocks_per_sm, nedev::k_paths<nedev::K_VOLUME | nedev::K_CACHE | nedev::K_SPLIT>, nedev::kThreads, 0);
}
