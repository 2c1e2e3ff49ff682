// The regrouped state-machine path kernel (pt_sched.cuh), plain and counting.
#include "kernels.cuh"

using namespace nedev;

cudaError_t ne_sched_occupancy(int* blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_sched<false>, kThreads, 0);
}

cudaError_t ne_launch_sched(bool count, int blocks, cudaStream_t st, const DScene& s, const PathArgs& a,
                            unsigned long long* counter, uint32_t* err) {
  if (count)
    k_sched<true><<<blocks, kThreads, 0, st>>>(s, a, counter, err);
  else
    k_sched<false><<<blocks, kThreads, 0, st>>>(s, a, counter, err);
  return cudaGetLastError();
}
