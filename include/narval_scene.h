/*
 * Plain-data description of a NarvalEngine scene, as the path integrator sees it.
 *
 * The reference keeps its scene as an object graph (core/Scene.h:12-36):
 *   Scene::instancedModels, Scene::lights   -> InstancedModel (transformToWCS, its inverse, Model*)
 *   Model::primitives, Model::lights, Model::materials (primitives/Model.h:68-77)
 *   Primitive::material (primitives/Primitive.h:14) -> Material {bsdf, medium, light, textures}
 *   Light::primitive (lights/Light.h:9), GridMedia {grid texture, sigma_s, sigma_a, density}
 * This header flattens that graph into arrays indexed by 32-bit ids, in the same
 * order the reference iterates them, so that a GPU copy and a CPU restatement can
 * both be built from one description. Every field names the reference member it
 * carries. The description is produced from the reference's JSON scene format by
 * ne_scene_host_load_json() (narval_gb300.h) or assembled by a caller directly.
 *
 * Matrices are 4x4 column-major, element (row r, column c) at m[c * 4 + r], the
 * memory layout of glm::mat4.
 */
#ifndef NARVAL_SCENE_H_
#define NARVAL_SCENE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Primitive kinds (primitives/Sphere.h, Rectangle.h, AABB.h, Triangle.h, Point.h). */
enum ne_prim_type {
  NE_PRIM_SPHERE = 0,    /* p0 = centre (OCS), radius */
  NE_PRIM_RECTANGLE = 1, /* p0 = vertexData[0], p1 = vertexData[1] (the opposite corner), p2 = normal */
  NE_PRIM_AABB = 2,      /* p0 = min, p1 = max */
  NE_PRIM_TRIANGLE = 3,  /* p0, p1, p2 = vertices (OCS); area = Triangle::area */
  NE_PRIM_POINT = 4      /* p0 = position */
};

typedef struct ne_primitive {
  int32_t type;
  int32_t material; /* index into materials, -1 when Primitive::material is null */
  float p0[3];
  float p1[3];
  float p2[3];
  float radius;
  float area;
} ne_primitive;

/* One Model: its primitive list, its emissive primitive list and its materials. */
typedef struct ne_model {
  uint32_t prim_begin, prim_count;   /* Model::primitives, contiguous in prims[] */
  uint32_t light_begin, light_count; /* Model::lights, contiguous in prims[] */
  uint32_t mat_begin, mat_count;     /* Model::materials, contiguous in model_materials[] */
  int32_t has_bbox;                  /* Model::boundingBox set (meshes) */
  float bbox_min[3], bbox_max[3];
  int32_t use_bvh;                   /* Model::bvh built (meshes loaded from files) */
} ne_model;

/* One InstancedModel (primitives/InstancedModel.h:11-33). */
typedef struct ne_instance {
  float to_wcs[16];  /* transformToWCS */
  float to_ocs[16];  /* invTransformToWCS */
  uint32_t model;
  int32_t collision; /* isCollisionEnabled */
} ne_instance;

enum ne_bsdf_kind { NE_BSDF_NONE = 0, NE_BSDF_GLOSSY = 1, NE_BSDF_VOLUME = 2 };
enum ne_phase_kind { NE_PHASE_ISOTROPIC = 0, NE_PHASE_HG = 1 };

/* Texture slots of a Material (core/RendererAPI.h:233-243 TextureName bits). */
enum ne_tex_bits {
  NE_TEX_ALBEDO = 1 << 1,
  NE_TEX_ROUGHNESS = 1 << 2,
  NE_TEX_METALLIC = 1 << 3,
  NE_TEX_NORMAL = 1 << 5,
  NE_TEX_TEX1 = 1 << 7
};

/* One Material (materials/Material.h:9-70). Textures are the 1x1 constants SceneReader
 * creates for "microfacet" and "emitter" materials (io/SceneReader.cpp:92-130,147). */
typedef struct ne_material {
  int32_t bsdf;        /* ne_bsdf_kind: GlossyBSDF or VolumeBSDF behind Material::bsdf */
  int32_t light;       /* index into lights, -1 when Material::light is null */
  int32_t medium;      /* index into media, -1 when Material::medium is null */
  int32_t phase;       /* ne_phase_kind of the VolumeBSDF */
  float g;             /* HG asymmetry */
  float albedo[3];     /* ALBEDO texture value */
  float roughness;     /* ROUGHNESS texture value */
  float metallic;      /* METALLIC texture value */
  float normal_map[3]; /* NORMAL texture value */
  int32_t tex_present; /* ne_tex_bits of the non-null Material::textures slots */
  int32_t tex_types;   /* Material::textureTypes (the bits hasTexture() tests) */
  /* A microfacet albedo given as an image file (io/SceneReader.cpp:80-103, loaded by
   * ResourceManager::loadTexture, core/ResourceManager.cpp:288-313, as 8-bit RGBA with the
   * mirror wrap and nearest lookup of Texture::sample): its texels row-major from the top
   * row. albedo_width = 0: the constant albedo[] above. */
  int32_t albedo_width, albedo_height;
  const uint8_t* albedo_texels;
} ne_material;

enum ne_light_kind { NE_LIGHT_DIFFUSE = 0, NE_LIGHT_DIRECTIONAL = 1, NE_LIGHT_INFINITE = 2 };

/* One Light (lights/Light.h:7-53 and subclasses). */
typedef struct ne_light {
  int32_t type;          /* ne_light_kind */
  int32_t primitive;     /* Light::primitive, index into prims */
  float li[3];           /* Light::li */
  float le[3];           /* Light::le */
  float direction[3];    /* DirectionalLight::direction (pointing from the light) */
  float env_radiance[3]; /* InfiniteAreaLight without a texture: value of its (1x1, constant) map */
  float env_map_pdf;     /* InfiniteAreaLight without a texture: pdf Distribution2D returns for
                            that map (1, or 0) */
  /* InfiniteAreaLight with a texture (lights/InfiniteAreaLight.h:20-40): its 8-bit RGBA texels
   * as the reference's loader gives them, row-major from the top row, sampled with the mirror
   * wrap and nearest lookup of Texture::sample. env_width = 0: no texture. The library builds
   * the light's Distribution2D from them at upload. */
  int32_t env_width, env_height;
  const uint8_t* env_texels;
} ne_light;

enum ne_medium_kind { NE_MEDIUM_GRID = 0, NE_MEDIUM_HOMOGENEOUS = 1 };

/* One Medium (materials/GridMedia.h:14-90, materials/HomogeneousMedia.h). */
typedef struct ne_medium {
  int32_t type;        /* ne_medium_kind */
  float sigma_s[3];    /* scattering */
  float sigma_a[3];    /* absorption */
  float density;       /* GridMedia::densityMultiplier or HomogeneousMedia::density */
  uint32_t res[3];     /* grid width, height, depth */
  const float* grid;   /* R32F voxels, index z*W*H + y*W + x (utils/Math.h:104-106) */
} ne_medium;

/* Camera basis after Camera::Camera (core/Camera.cpp:7-26). */
typedef struct ne_camera {
  float position[3];
  float lower_left[3];
  float horizontal[3];
  float vertical[3];
  float side[3];
  float up[3];
  float lens_radius;
} ne_camera;

/* SceneSettings (core/Settings.h:12-17) plus the documented extensions. */
typedef struct ne_settings {
  int32_t width, height;
  int32_t spp;
  int32_t bounces;
  int32_t hdr;
  int32_t rr_enabled; /* extension: Russian roulette on the path throughput */
  int32_t rr_after;   /* extension: first bounce index (exclusive) where it applies */
  int32_t bvh_build;  /* extension: 0 = BVH::init's midpoint build on the host (the reference's
                         tree), 1 = binned-SAH build on the GPU (same layout and leaf size) */
} ne_settings;

typedef struct ne_scene_desc {
  uint32_t n_instances;       /* Scene::instancedModels, first in instances[] */
  uint32_t n_light_instances; /* Scene::lights, after them */
  const ne_instance* instances;
  uint32_t n_models;
  const ne_model* models;
  uint32_t n_prims;
  const ne_primitive* prims;
  uint32_t n_materials;
  const ne_material* materials;
  uint32_t n_model_materials;
  const uint32_t* model_materials;
  uint32_t n_lights;
  const ne_light* lights;
  uint32_t n_media;
  const ne_medium* media;
  ne_camera camera;
  ne_settings settings;
} ne_scene_desc;

#ifdef __cplusplus
}
#endif

#endif /* NARVAL_SCENE_H_ */
