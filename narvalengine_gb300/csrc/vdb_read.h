// OpenVDB density grids (.vdb) for grid media, read by the library itself (OpenVDB is not
// available here): the dense array core/ResourceManager.cpp:165-218 (loadVDBasTexture) makes
// of a file's float grid named "density" with OpenVDB 6.2.
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "narval_gb300.h"

namespace nevdb {

// Reads the first grid named "density" of the OpenVDB file at `path` and fills `grid` with the
// dense array of loadVDBasTexture: the box from (-|min.x|, -|min.y|, -|min.z|) with
// |min| + |max| voxels per axis (one more where the active box straddles 0), min and max the
// corners of the active voxels' bounding box, every voxel the tree's value there (active or
// not), z fastest; `res` = (voxels along z, along y, along x), the texture's width, height and
// depth. NE_ERR_MISSING_ASSET if the file cannot be read; NE_ERR_UNSUPPORTED for files before
// format 222, Blosc streams other than LZ4 with byte shuffle, grids that are not
// Tree_float_5_4_3 and instanced grids; NE_ERR_PARSE for a corrupt file, a file without a
// "density" grid, a grid without active voxels or an empty dense box. `err` says which.
ne_status loadDensity(const std::string& path, uint32_t res[3], std::vector<float>& grid, std::string& err);

}  // namespace nevdb
