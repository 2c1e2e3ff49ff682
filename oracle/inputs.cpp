// Seeded synthetic inputs for the oracle's own scene reader (oracle/scene_reader.py).
//
// TEST INFRASTRUCTURE ONLY. The configurations' density grids and meshes are procedural:
// seeded simplex fBm grids and displaced icospheres. They are inputs, not part of the path
// under test, and both sides must consume the same ones, so this file exposes the seeded
// generator source (narvalengine_gb300/csrc/scene_gen.cpp, compiled into liboracle.so as a
// separate copy) to the oracle's reader. The generator is pinned by the fBm checksum
// fixture (tests/golden/fbm_checksum.json). Everything that reads the scene descriptor —
// transforms, camera, materials, lights, primitive layouts — is restated independently in
// Python by the oracle's reader.
#include <stdint.h>
#include <string.h>

#include <vector>

#include "scene_gen.h"

extern "C" {

// FbmParams fields in order; out holds res[0] * res[1] * res[2] floats.
void orc_gen_fbm(const uint32_t res[3], int octaves, double frequency, double lacunarity, double gain,
                 double falloff_radius, uint64_t seed, float* out) {
  negen::FbmParams p;
  p.octaves = octaves;
  p.frequency = frequency;
  p.lacunarity = lacunarity;
  p.gain = gain;
  p.falloff_radius = falloff_radius;
  p.seed = seed;
  std::vector<float> g;
  negen::fbm_grid(res, p, g);
  memcpy(out, g.data(), g.size() * sizeof(float));
}

// Icosphere with 20 * 4^n triangles and 10 * 4^n + 2 vertices; positions 3 floats per
// vertex, indices 3 per triangle.
void orc_gen_icosphere(int subdivisions, double amplitude, double frequency, uint64_t seed, float* positions,
                       uint32_t* indices) {
  negen::IcoParams p;
  p.subdivisions = subdivisions;
  p.amplitude = amplitude;
  p.frequency = frequency;
  p.seed = seed;
  std::vector<float> pos;
  std::vector<uint32_t> idx;
  negen::icosphere(p, pos, idx);
  memcpy(positions, pos.data(), pos.size() * sizeof(float));
  memcpy(indices, idx.data(), idx.size() * sizeof(uint32_t));
}

double orc_gen_hash_u01(uint64_t seed, uint64_t i) { return negen::hash_u01(seed, i); }

}  // extern "C"
