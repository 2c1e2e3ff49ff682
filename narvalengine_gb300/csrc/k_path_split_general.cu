// Path kernel instantiation unit (see kernels.cuh): split render, K_GENERAL feature set.
#include "kernels.cuh"

namespace nedev {

cudaError_t launchSplit_general(int pass, int blocks, cudaStream_t st, const DScene& s, const PathArgs& a,
                             unsigned long long* counter, uint32_t* err) {
  constexpr uint32_t K = K_GENERAL | K_SPLIT;
  if (pass == 0)
    k_paths<K><<<blocks, kThreads, 0, st>>>(s, a, counter, err);
  else
    k_resume<K><<<blocks, kThreads, 0, st>>>(s, a, counter, err);
  return cudaGetLastError();
}

cudaError_t occupancySplit_general(int* blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_paths<K_GENERAL | K_SPLIT>, kThreads, 0);
}

cudaError_t launchTrace_general(int sm_count, cudaStream_t st, const DScene& s, const DeferQueue* q,
                                unsigned long long* counter, uint32_t* err) {
  static const int fit = [] {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_trace<K_GENERAL | K_SPLIT>, kThreads, 0) != cudaSuccess)
      b = 0;
    return b;
  }();
  k_trace<K_GENERAL | K_SPLIT><<<sm_count * (fit > 0 ? fit : 1), kThreads, 0, st>>>(s, q, counter, err);
  return cudaGetLastError();
}

}  // namespace nedev
