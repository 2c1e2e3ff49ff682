// Seeded procedural inputs for the synthetic scenes: simplex-noise fBm density grids
// and displaced icosphere meshes. Host code; results are identical on every host
// (double arithmetic with +, -, *, /, floor and sqrt only).
#pragma once
#include <stdint.h>

#include <vector>

namespace negen {

struct FbmParams {
  int octaves = 5;
  double frequency = 4.0 / 128.0;  // per voxel
  double lacunarity = 2.0;
  double gain = 0.5;
  double falloff_radius = 64.0;    // voxels; density *= max(0, 1 - r / R)
  uint64_t seed = 0x4E415256ull;
};

// Fills a res[0] x res[1] x res[2] grid (index z*W*H + y*W + x) with
// max(0, fbm(voxel centre)) * max(0, 1 - r / R), r = distance to the grid centre.
void fbm_grid(const uint32_t res[3], const FbmParams& p, std::vector<float>& out);

struct IcoParams {
  int subdivisions = 3;
  double amplitude = 0.0;  // radial displacement: r = 1 + amplitude * noise(frequency * v)
  double frequency = 1.0;
  uint64_t seed = 0x4E415256ull;
};

// Unit icosphere subdivided n times (20 * 4^n triangles, 10 * 4^n + 2 vertices).
void icosphere(const IcoParams& p, std::vector<float>& positions, std::vector<uint32_t>& indices);

// Seeded uniform number in [0, 1) for index i.
double hash_u01(uint64_t seed, uint64_t i);

// 3-D simplex noise in [-1, 1] for a seeded permutation (exposed for tests).
struct Simplex {
  uint8_t perm[512];
  explicit Simplex(uint64_t seed);
  double noise(double x, double y, double z) const;
};

}  // namespace negen
