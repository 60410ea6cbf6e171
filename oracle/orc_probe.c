/*
 * ORACLE - test infrastructure only.  Batched, ctypes-friendly entry points
 * over the restated reference functions.  oracle/ref_shim.cpp exports the
 * same signatures (prefix ref_p_) on top of the reference's own headers, so
 * the tests can pin this restatement against the reference bit for bit.
 *
 * Packed layouts (floats):
 *   tri  : 37 = vertices 9, uv 9 (Vector3 per vertex), normals 9,
 *          tangents 9, tangent sign 1                        (Tri.hpp:13-17)
 *   hit  : 17 = valid, position 3, normal 3, tangent 3, bitangent 3, tu, tv,
 *          distance |position - origin|                      (Hit.hpp:6-13)
 *   hd   : 27 = HitData in member order                      (kernel.h:46-69)
 */
#include <string.h>
#include "orc.h"

static v3 g3(const float* p) { return V3(p[0], p[1], p[2]); }
static void p3(float* o, v3 a) { o[0] = a.x; o[1] = a.y; o[2] = a.z; }

static void unpack_tri(const float* q, orc_tri* t) {
  for (int k = 0; k < 3; k++) {
    t->v[k] = g3(q + 3 * k);
    t->uv[k] = g3(q + 9 + 3 * k);
    t->n[k] = g3(q + 18 + 3 * k);
    t->tg[k] = g3(q + 27 + 3 * k);
  }
  t->tsign = q[36];
  t->id = 0;
}

static void unpack_hd(const float* q, orc_hitdata* h) { memcpy(h, q, sizeof(orc_hitdata)); }

/* Tri::hit on ray (o, d) after the Ray constructor (normalize != 0) or as is */
void orc_p_tri_hit(int64_t n, const float* tris, const float* rays, int32_t normalize, float* out) {
  for (int64_t i = 0; i < n; i++) {
    orc_tri t;
    unpack_tri(tris + 37 * i, &t);
    orc_ray r;
    r.origin = g3(rays + 6 * i);
    r.direction = g3(rays + 6 * i + 3);
    if (normalize) r = orc_make_ray(r.origin, r.direction);
    orc_hit h;
    memset(&h, 0, sizeof h);
    float* o = out + 17 * i;
    memset(o, 0, 17 * sizeof(float));
    if (orc_tri_hit(&t, &r, &h)) {
      o[0] = 1;
      p3(o + 1, h.position); p3(o + 4, h.normal); p3(o + 7, h.tangent); p3(o + 10, h.bitangent);
      o[13] = h.tu; o[14] = h.tv;
      o[15] = vlen(vsub(h.position, r.origin));
    }
  }
}

/* out 7 per item: DisneyEval rgb, DisneyPdf, DisneySample xyz.
 * dirs are the incoming ray directions (used as given). */
void orc_p_disney(int64_t n, const float* hd, const float* dirs, const float* Ls, const float* rnd, float* out) {
  for (int64_t i = 0; i < n; i++) {
    orc_hitdata h;
    unpack_hd(hd + 27 * i, &h);
    orc_ray r;
    r.origin = V1(0);
    r.direction = g3(dirs + 3 * i);
    v3 L = g3(Ls + 3 * i);
    float* o = out + 7 * i;
    p3(o, orc_disney_eval(&r, &h, L));
    o[3] = orc_disney_pdf(&r, &h, L);
    p3(o + 4, orc_disney_sample(&r, &h, rnd[3 * i], rnd[3 * i + 1], rnd[3 * i + 2]));
  }
}

/* out 6 per item: ray origin and (normalised) direction */
void orc_p_camera(const er_camera* c, int64_t n, const int32_t* xy, const float* rnd, float* out) {
  for (int64_t i = 0; i < n; i++) {
    const float* u = rnd + 5 * i;
    orc_ray r = orc_camera_ray(c, xy[2 * i], xy[2 * i + 1], u[0], u[1], u[2], u[3], u[4]);
    p3(out + 6 * i, r.origin);
    p3(out + 6 * i + 3, r.direction);
  }
}

/* out 2 per item: sphericalMapping(u, v) of the points */
void orc_p_spherical(int64_t n, const float* pts, float* out) {
  for (int64_t i = 0; i < n; i++) orc_spherical_mapping(g3(pts + 3 * i), out + 2 * i, out + 2 * i + 1);
}

/* out 3 per item: reverseSphericalMapping of (u, v) */
void orc_p_reverse_spherical(int64_t n, const float* uv, float* out) {
  for (int64_t i = 0; i < n; i++) p3(out + 3 * i, orc_reverse_spherical(uv[2 * i], uv[2 * i + 1]));
}

/* cdf has length w*h+1; radiance_sum receives HDRI::radianceSum */
void orc_p_hdri_cdf(const er_texture* t, float* cdf, float* radiance_sum) {
  orc_tex x = {t->width, t->height, t->data, t->x_tile, t->y_tile, t->x_offset, t->y_offset};
  orc_hdri_cdf(&x, cdf, radiance_sum);
}

/* out 8 per item for uniform r: texel index, pdf, direction xyz, env rgb
 * (HDRI::sample -> hdriLight direction / value / pdf, kernel.cu:236-254) */
void orc_p_hdri_sample(const er_texture* t, const float* cdf, float radiance_sum, int64_t n, const float* r,
                       float* out) {
  orc_tex x = {t->width, t->height, t->data, t->x_tile, t->y_tile, t->x_offset, t->y_offset};
  for (int64_t i = 0; i < n; i++) {
    int32_t count = orc_hdri_search(cdf, r[i], x.w * x.h);
    float tx = (float)(count % x.w), ty = (float)(count / x.w);
    float iu, iv;
    orc_inverse_transform_uv(&x, tx / (float)x.w, ty / (float)x.h, &iu, &iv);
    v3 d = vneg(vnormalized(orc_reverse_spherical(iu, iv)));
    float* o = out + 8 * i;
    o[0] = (float)count;
    o[1] = orc_hdri_pdf(&x, radiance_sum, f2i_dev(iu * (float)x.w), f2i_dev(iv * (float)x.h));
    p3(o + 2, d);
    p3(o + 5, orc_tex_uv(&x, iu, iv));
  }
}

/* Effective texel distribution of HDRI::binarySearch (HDRI.hpp:130-142)
 * over the renderer's uniform grid r = k * 2^-24, k = 1..2^24: counts[t]
 * receives how many k select texel t (counts has w*h entries, zeroed here). */
void orc_p_hdri_counts(const float* cdf, int32_t n, uint32_t* counts) {
  for (int32_t i = 0; i < n; i++) counts[i] = 0;
  for (int64_t k = 0; k < ((int64_t)1 << 24); k++) {
    int32_t t = orc_hdri_search(cdf, (float)(k + 1) * (1.0f / 16777216.0f), n);
    if (t >= 0 && t < n) counts[t]++;
  }
}

/* texture fetch by uv (nearest, with tile/offset), out 3 per item */
void orc_p_tex_uv(const er_texture* t, int64_t n, const float* uv, float* out) {
  orc_tex x = {t->width, t->height, t->data, t->x_tile, t->y_tile, t->x_offset, t->y_offset};
  for (int64_t i = 0; i < n; i++) p3(out + 3 * i, orc_tex_uv(&x, uv[2 * i], uv[2 * i + 1]));
}

/* Full per-sample path with explicit uniforms instead of the RNG, so that a
 * restatement over the reference headers can replay it.  u holds
 * 5 + 4*max_depth uniforms: camera r1..r5, then per vertex DisneySample
 * r1..r3 and the shade r1.  out: light rgb, bounce count. */
int32_t orc_sample_u(const orc_scene* s, int32_t x, int32_t y, int32_t max_depth, const float* u, float* out);

void orc_p_sample_u(const orc_scene* s, int64_t n, const int32_t* xy, int32_t max_depth, const float* u,
                    float* out) {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 8)
#endif
  for (int64_t i = 0; i < n; i++)
    orc_sample_u(s, xy[2 * i], xy[2 * i + 1], max_depth, u + (int64_t)(5 + 4 * max_depth) * i, out + 4 * i);
}

void orc_p_philox(int64_t n, const uint32_t* ctr, uint32_t k0, uint32_t k1, uint32_t* out) {
  for (int64_t i = 0; i < n; i++)
    orc_philox(ctr[4 * i], ctr[4 * i + 1], ctr[4 * i + 2], ctr[4 * i + 3], k0, k1, out + 4 * i);
}
