/*
 * ORACLE - test infrastructure only (parity checker and CPU baseline).
 * Nothing in the product library includes, links or calls this code; only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * liborc.so.
 *
 * A plain-C restatement of the reference's per-sample path tracer
 * (src/tfg-pathtracer/kernel.cu:54-481 and the __host__ __device__ headers
 * it uses), with the reference's own BVH (BVH.hpp: depth 18, 14-bin SAH) and
 * traversal, so that hit IDs and shading follow the reference's arithmetic
 * and quirks.  The random numbers are this project's counter-based stream
 * (Philox-4x32-10), not cuRAND's.
 */
#ifndef ORC_H
#define ORC_H

#include <stdint.h>
#include "orc_math.h"
#include "../include/eleven.h"

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_BVH_DEPTH 18 /* Definitions.h:13 */
#define ORC_SAH_BINS 14  /* Definitions.h:14 */

/* Tri.hpp:13-19 */
typedef struct {
  v3 v[3], uv[3], n[3], tg[3];
  float tsign;
  int32_t id; /* the triangle's index in the desc (reference: objectID slot) */
} orc_tri;

/* Hit.hpp:6-13 */
typedef struct {
  v3 position, normal, tangent, bitangent;
  int valid;
  int32_t id;
  float tu, tv;
} orc_hit;

/* BVH.hpp:29-48 */
typedef struct {
  v3 b1, b2;
  int32_t from, to, idx, depth;
  int32_t valid;
} orc_node;

/* Texture.hpp:196-214 (filter is always NO_FILTER on the hot path) */
typedef struct {
  int32_t w, h;
  const float* data;
  float xTile, yTile, xOffset, yOffset;
} orc_tex;

/* kernel.h:46-69 HitData, same member order (27 floats). */
typedef struct {
  float metallic, roughness, clearcoatGloss, clearcoat, anisotropic, eta,
      transmission, specular, specularTint, sheenTint, subsurface, sheen;
  v3 emission, albedo, normal, tangent, bitangent;
} orc_hitdata;

typedef struct {
  v3 origin, direction;
} orc_ray;

typedef struct orc_scene {
  er_camera cam;
  int64_t ntri;
  orc_tri* tris;
  uint32_t* tie_key;
  int32_t* tri_mat; /* material of each triangle (object -> material) */
  /* reference BVH */
  orc_node* nodes;
  int64_t nnodes;
  int32_t* tri_indices;
  int32_t nmat;
  er_material* mats;
  int32_t ntex;
  orc_tex* texs;
  float** tex_store;
  int32_t nlights;
  er_point_light* lights;
  orc_tex env;
  float* env_store;
  float* cdf; /* w*h+1 */
  float radianceSum;
} orc_scene;

/* ---- scene ---- */
orc_scene* orc_scene_new(const er_scene_desc* d);
void orc_scene_free(orc_scene* s);
int64_t orc_bvh_node_count(const orc_scene* s);
/* boxes: n*6 (b1, b2); meta: n*5 (from, to, idx, depth, valid) */
void orc_bvh_export(const orc_scene* s, float* boxes, int32_t* meta, int32_t* tri_indices);

/* ---- geometry ---- */
int orc_tri_hit(const orc_tri* t, const orc_ray* r, orc_hit* h);
orc_ray orc_make_ray(v3 o, v3 d); /* Ray.hpp:14-18 */
void orc_transverse(const orc_scene* s, orc_ray r, orc_hit* nearest);
/* mode 0: reference BVH traversal; 1: all triangles in index order;
 * 2: all triangles, lowest tie key wins on exactly equal distance */
void orc_trace(const orc_scene* s, const float* rays, int64_t n, int32_t mode,
               int32_t normalize, int32_t* tri, float* dist, float* uv, int32_t nthreads);

/* ---- shading pieces ---- */
v3 orc_tex_coord(const orc_tex* t, int32_t x, int32_t y);
v3 orc_tex_uv(const orc_tex* t, float u, float v);
void orc_spherical_mapping(v3 p, float* u, float* v);
v3 orc_reverse_spherical(float u, float v);
void orc_inverse_transform_uv(const orc_tex* t, float u, float v, float* nu, float* nv);
void orc_hdri_cdf(const orc_tex* t, float* cdf, float* radianceSum);
int32_t orc_hdri_search(const float* cdf, float value, int32_t length);
float orc_hdri_pdf(const orc_tex* t, float radianceSum, int32_t x, int32_t y);
float orc_disney_pdf(const orc_ray* r, const orc_hitdata* hd, v3 L);
v3 orc_disney_sample(const orc_ray* r, const orc_hitdata* hd, float r1, float r2, float r3);
v3 orc_disney_eval(const orc_ray* r, const orc_hitdata* hd, v3 L);
orc_ray orc_camera_ray(const er_camera* c, int32_t x, int32_t y, float r1, float r2, float r3, float r4, float r5);

/* ---- RNG: Philox-4x32-10 (Salmon et al., SC'11) ---- */
void orc_philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1, uint32_t out[4]);
float orc_u01(uint32_t x);

/* ---- render ---- */
typedef struct {
  int32_t spp, sample_begin, max_depth, aov;
  uint64_t seed;
  int32_t nthreads;      /* 0 = all */
  int32_t pixel_stride;  /* >1: render only pixels p with p % stride == 0 (bounded samples) */
} orc_render_opts;

/* One sample of one pixel (kernel.cu:369-481 before accumulation).
 * Returns the bounce count; light (before clamp) and first-hit AOVs. */
int32_t orc_sample(const orc_scene* s, int32_t x, int32_t y, int32_t sample, int32_t max_depth,
                   uint64_t seed, v3* light, v3* nrm, v3* tan, v3* bit);
/* Full render with the reference FP32 running mean (kernel.cu:445-478).
 * passes: 4 arrays of W*H*4 (beauty, normal, tangent, bitangent; any NULL). */
void orc_render(const orc_scene* s, const orc_render_opts* o, float* beauty, float* normal,
                float* tangent, float* bitangent, uint32_t* samples, uint32_t* pathcount);
/* Per-path radiance/bounces for samples [sample_begin, sample_begin+spp):
 * radiance [s][p][3], bounces [s][p], p = output pixel index. */
void orc_render_paths(const orc_scene* s, const orc_render_opts* o, float* radiance, int32_t* bounces);

/* ---- FP64 restatement of the estimator (orc64.c) ---- */
typedef struct orc64_scene orc64_scene;
orc64_scene* orc64_new(const orc_scene* s);
void orc64_free(orc64_scene* S);
void orc64_render_pixels(const orc64_scene* S, const int32_t* idx, int64_t n, int32_t spp, int32_t sample_begin,
                         int32_t max_depth, uint64_t seed, double* rgb, uint32_t* counts, int32_t nthreads);
void orc64_trace(const orc64_scene* S, const float* rays, int64_t n, int32_t* tri, double* dist, int32_t nthreads);
/* the detached estimator: sampling from the scene, BRDF values and env
 * radiance from eval_mat (n_materials x 5) / eval_env (w*h*3), NULL = the
 * scene's (as er_render_replay) */
void orc64_render_pixels_eval(const orc64_scene* S, const int32_t* idx, int64_t n, int32_t spp, int32_t sample_begin,
                              int32_t max_depth, uint64_t seed, const float* eval_mat, const float* eval_env,
                              double* rgb, uint32_t* counts, int32_t nthreads);

/* ---- post-processing (PostProcessing.cpp), in place on W*H*4 floats ---- */
void orc_postprocess(float* pix, int32_t w, int32_t h, const er_post_opts* o);

/* ---- output (main.cpp:150-165) ---- */
double orc_fastpow(double a, double b);
void orc_encode_ldr(const float* rgba, int64_t n, uint8_t* out);

#ifdef __cplusplus
}
#endif
#endif
