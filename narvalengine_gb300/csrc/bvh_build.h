// GPU binned-SAH BVH build (bvh_build.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "device_scene.h"

namespace nedev {

// Builds the BVH of triangles prims[first, first + n) (device memory) on `st`: nodes in
// depth-first order in DNode form (leaf starts index `slots`), slots = global primitive
// indices in leaf order. Synchronises `st`. On failure returns the CUDA error, or
// cudaErrorUnknown with a message in `err`.
cudaError_t buildSahBvh(cudaStream_t st, const DPrim* prims, uint32_t first, uint32_t n, std::vector<DNode>& nodes,
                        std::vector<uint32_t>& slots, std::string& err);

}  // namespace nedev
