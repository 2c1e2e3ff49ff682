/*
 * CPU oracle of the NarvalEngine path-tracing hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This library restates, on the CPU, the reference's
 * VolumetricPathIntegrator and everything it calls per path (oracle.cpp cites the
 * reference file:line of every function). It exists to check the GPU library: the
 * parity tests, the smoke check and the CPU-baseline leg of bench.py call it as the
 * checker, never as the thing measured or shipped. The product never links or loads it.
 *
 * Deliberate deviations from the reference, shared with the GPU code:
 *  - random() (utils/Math.h:51-66) is replaced by the counter-based generator of
 *    ne_rng.h, in the reference's draw order;
 *  - libm's log/sin/cos/acos/pow are replaced by ne_fmath.h.
 */
#ifndef NARVAL_ORACLE_H_
#define NARVAL_ORACLE_H_

#include <stddef.h>
#include <stdint.h>
#include "narval_scene.h"
#include "narval_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_scene orc_scene;

orc_scene* orc_scene_create(const ne_scene_desc* desc);
void orc_scene_destroy(orc_scene* s);

/* Camera path per key (camera draws 0-3, Li from 4), like ne_trace_paths. */
void orc_trace_paths(const orc_scene* s, const ne_render_params* p, const ne_path_key* keys, size_t n, float* out_L,
                     int n_threads);
/* Camera paths of a view (camera, size, random stream), like one view of ne_views. */
void orc_trace_view_paths(const orc_scene* s, const ne_render_params* p, const ne_camera* cam, int width, int height,
                          uint32_t stream, const ne_path_key* keys, size_t n, float* out_L, int n_threads);
/* Integrator::Li for given rays, like ne_li_batch. */
void orc_li_batch(const orc_scene* s, const ne_render_params* p, const ne_ray* rays, const ne_path_key* keys,
                  size_t n, uint32_t first_dim, float* out_L, int n_threads);
/* OfflineEngine::coreLoop without tone mapping: per-pixel mean radiance. Returns wall
 * seconds. Tiles are taken from a shared queue by n_threads std::threads. */
double orc_render(const orc_scene* s, const ne_render_params* p, float* out_rgb, int n_threads);
/* Renders only pixels [pixel_begin, pixel_begin + n_pixels) (all spp), returns seconds. */
double orc_render_pixels(const orc_scene* s, const ne_render_params* p, uint32_t pixel_begin, uint32_t n_pixels,
                         float* out_rgb, int n_threads, uint64_t* density_lookups);
/* Renders the listed pixels (all spp each) into out_rgb (3 floats per listed pixel). */
double orc_render_pixel_list(const orc_scene* s, const ne_render_params* p, const uint32_t* pixels, uint32_t n_pixels,
                             float* out_rgb, int n_threads, uint64_t* density_lookups);
void orc_trace_closest(const orc_scene* s, const ne_ray* rays, size_t n, float t_min, float t_max, ne_hit* out);

/* BVH::init result of model m: 9 words per node (min, max, start, count, rightOffset). */
size_t orc_model_bvh(const orc_scene* s, uint32_t m, float* nodes, size_t cap, uint32_t* order);
int orc_model_set_bvh(orc_scene* s, uint32_t m, const float* nodes, size_t n, const uint32_t* order, size_t n_order);

/* Unit-level restatements for known-answer tests. */
int orc_triangle_intersect(const float* v0, const float* v1, const float* v2, const ne_ray* r, float* t_near,
                           float* t_far, float* point, float* normal);
int orc_aabb_intersect(const float* mn, const float* mx, const ne_ray* r, float* t_near, float* t_far,
                       float* point, float* normal);
void orc_orthonormal(const float* n, float* v, float* u);
void orc_to_lcs(const float* v, const float* ns, const float* ss, const float* ts, float* out);
void orc_to_world(const float* v, const float* ns, const float* ss, const float* ts, float* out);
void orc_sample_unit_sphere(float e1, float e2, float* out);
float orc_hg_eval(float g, const float* wi, const float* wo);
void orc_hg_sample(float g, float u0, float u1, float* out);
float orc_iso_pdf(void);
void orc_barycentric(const float* p, const float* a, const float* b, const float* c, float* out);
float orc_triangle_area(const float* v0, const float* v1, const float* v2);
int orc_triangle_contains(const float* v0, const float* v1, const float* v2, const float* p);
int orc_point_in_triangle_range(const float* p, const float* a, const float* b, const float* c);
/* Model(vertexData, indexData) of triangles (primitives/Model.cpp:36-79) + Model::intersect. */
int orc_triangle_model_intersect(const float* verts, uint32_t n_verts, const uint32_t* idx, uint32_t n_idx,
                                 const ne_ray* r, float t_min, float t_max, float* t_hit);
/* BVH::init over a triangle soup; returns node count; bvh hit via orc_bvh_intersect. */
uint32_t orc_bvh_build_count(const float* verts, const uint32_t* idx, uint32_t n_tris);

/* Elementary functions of ne_fmath.h as compiled on the host. fn as ne_debug_fmath. */
void orc_fmath(int fn, const float* x, size_t n, float* out);
void orc_rng(uint64_t seed, const ne_path_key* keys, const uint32_t* dims, size_t n, float* out);
void orc_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out);

/* Seeded synthetic inputs (inputs.cpp) for the oracle's own scene reader. */
void orc_gen_fbm(const uint32_t res[3], int octaves, double frequency, double lacunarity, double gain,
                 double falloff_radius, uint64_t seed, float* out);
void orc_gen_icosphere(int subdivisions, double amplitude, double frequency, uint64_t seed, float* positions,
                       uint32_t* indices);
double orc_gen_hash_u01(uint64_t seed, uint64_t i);

#ifdef __cplusplus
}
#endif

#endif
