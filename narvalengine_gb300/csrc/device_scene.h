// Device-side layout of a scene (built from ne_scene_desc by api.cu).
//
// All arrays live in HBM; the DScene header itself is a kernel parameter, so its
// fields sit in the constant bank and every warp reads them without a memory access.
// Index conventions are those of ne_scene_desc (instances: instancedModels first,
// then lights).
#pragma once
#include <stdint.h>

#include "narval_scene.h"

namespace nedev {

// Affine part of a glm::mat4: columns 0..3, rows 0..2 (row 3 is (0,0,0,1) for every
// transform the scene reader builds; mul4 reads m[12..14] for the w term).
struct DInstance {
  float wcs[12];    // transformToWCS columns c0.xyz c1.xyz c2.xyz c3.xyz
  float ocs[12];    // invTransformToWCS, same layout
  float scale[3];   // getScale(transformToWCS) (utils/Math.h:874-912), for Rectangle::pdf
  uint32_t model;
  int32_t collision;
  // 1: no ray can hit this instance (its model holds only points and lights whose Le is a
  // non-black constant, which Model::intersect skips), so scene queries leave it out
  int32_t never_hit;
  int32_t pad[2];
};

enum : int32_t { DPRIM_GRID_MEDIUM = 1 };  // primitive whose material has a GridMedia

struct DPrim {
  int32_t type;
  int32_t material;
  int32_t flags;
  float radius;
  float p0[3];
  float p1[3];
  float p2[3];
  float area;  // Triangle::area
};

struct DModel {
  uint32_t prim_begin, prim_count;
  uint32_t light_begin, light_count;
  uint32_t mat_begin, mat_count;
  int32_t has_bbox;
  int32_t use_bvh;
  float bbox_min[3];
  float bbox_max[3];
  uint32_t bvh_node0;  // first node of this model's BVH in DScene::bvh
  uint32_t bvh_slot0;  // first slot of this model's leaf order in DScene::bvh_prims
};

// BVH node, 32 bytes: lo = (min.xyz, a), hi = (max.xyz, b). Leaf: a = start slot
// (relative to the model), b = count | 0x80000000. Interior: a = rightOffset, b = 0.
struct DNode {
  float lo[4];
  float hi[4];
};

struct DMaterial {
  int32_t bsdf, light, medium, phase;
  float g;
  float albedo[3];
  float roughness, metallic;
  float normal_map[3];
  int32_t tex_present, tex_types;
  int32_t albedo_w, albedo_h;  // albedo texture (RGBA8, row-major from the top row); 0: constant
  int32_t pad;
  const uchar4* albedo_tex;
};

struct DLight {
  int32_t type, primitive;
  float li[3], le[3], direction[3], env_radiance[3];
  float env_map_pdf;
  // InfiniteAreaLight with a texture (env_w > 0): RGBA8 texels and its Distribution2D
  // (utils/Sampling.h:71-112) as the reference builds it: `env_h` conditional rows of
  // `env_h` values each (Sampling.h:87 passes the height as every row's length), their CDFs
  // (env_h + 1 each) and integrals, and the marginal over the rows' integrals.
  int32_t env_w, env_h;
  float env_marg_int;
  const uchar4* env_tex;
  const float* env_cond_func;  // env_h x env_h
  const float* env_cond_cdf;   // env_h x (env_h + 1)
  const float* env_cond_int;   // env_h
  const float* env_marg_func;  // env_h
  const float* env_marg_cdf;   // env_h + 1
};

struct DMedium {
  int32_t type;
  float sigma_s[3];
  float sigma_t[3];      // absorption + scattering
  float density;         // density multiplier
  float inv_max_density; // 1 / max(grid)
  float mu;              // avg(sigma_t * density), the tracking rate
  uint32_t res[3];
  float resf[3];
  const float* grid;     // dense voxels, index z*W*H + y*W + x
  const float4* cells;   // (W+1)(H+1)(D+1) cells x 2 float4: the 8 corner densities
};

struct DCamera {
  float position[3], lower_left[3], horizontal[3], vertical[3], side[3], up[3];
  float lens_radius;
};

struct DScene {
  const DInstance* instances;
  const DModel* models;
  const DPrim* prims;
  const DMaterial* materials;
  const uint32_t* model_materials;
  const DLight* lights;
  const DMedium* media;
  const DNode* bvh;
  const uint32_t* bvh_prims;  // leaf slot -> primitive index
  uint32_t n_instances, n_light_instances;
  uint32_t n_prims, n_media;
  // world-space boxes (min xyz, max xyz) bounding every primitive whose material has a medium,
  // widened against rounding; -1: not known, every ray may reach a medium
  const float* medium_boxes;
  int32_t n_medium_boxes;
  DCamera camera;
  int32_t width, height;
};

}  // namespace nedev
