// Path kernel instantiation unit (see kernels.cuh): grid-medium scenes, paths ending in
// the learned radiance cache.
#include "kernels.cuh"

namespace nedev {

NE_PATH_KERNEL_INSTANCE(, 0, K_VOLUME | K_CACHE)

}  // namespace nedev

cudaError_t ne_launch_path_kernel_cache(int blocks, cudaStream_t st, const nedev::DScene& s, const nedev::PathArgs& a,
                                        unsigned long long* counter, uint32_t* err) {
  return nedev::launchPathKernel<0, nedev::K_VOLUME | nedev::K_CACHE>(blocks, st, s, a, counter, err);
}
