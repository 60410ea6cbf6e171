/*
 * ORACLE - test infrastructure only.  Restatement of the reference's
 * per-sample path loop and its device helpers (src/tfg-pathtracer/
 * kernel.cu:54-119 generateHitData, 152-173 throwRay, 175-205 pointLight,
 * 210-258 hdriLight, 339-367 shade/calculateBounce, 369-481
 * renderingKernel), the FP32 running-mean accumulation (kernel.cu:445-478)
 * and the LDR output step (main.cpp:150-165).
 *
 * Defined behaviour where the reference has none:
 *  - hdriLight leaves its pdf unset when the shadow ray is blocked
 *    (kernel.cu:247-248 return before :254); here the texel pdf is always
 *    computed, as it is independent of visibility.
 *  - pointLight indexes lights[(int)(n*r1)] and r1 can be exactly 1
 *    (kernel.cu:185); the index is clamped to n-1.
 *
 * Random numbers: Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel
 * random numbers: as easy as 1, 2, 3", SC'11), counter = (pixel, sample,
 * dimension block, 0), key = seed.  Block 0 and 1 feed the camera
 * (5 uniforms), block 2+i feeds vertex i: three BRDF-sample uniforms and
 * the shared light/HDRI uniform (kernel.cu:429,431; r2/r3 of shade are
 * unused by the reference with HDRIIS on).
 */
#include <stdlib.h>
#include <string.h>
#include "orc.h"
#ifdef _OPENMP
#include <omp.h>
#endif

void orc_philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1, uint32_t out[4]) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)M0 * c0;
    uint64_t p1 = (uint64_t)M1 * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += W0; k1 += W1;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* uniform in (0, 1], 24-bit resolution (the range of curand_uniform) */
float orc_u01(uint32_t x) { return (float)((x >> 8) + 1u) * (1.0f / 16777216.0f); }

/* ---------------------------------------------------------------- shading */

/* kernel.cu:152-173 with USEBVH */
static orc_hit throw_ray(const orc_scene* s, orc_ray r) {
  orc_hit h;
  memset(&h, 0, sizeof h);
  orc_transverse(s, r, &h);
  return h;
}

/* kernel.cu:54-119 */
static void hit_data(const orc_scene* s, const er_material* m, orc_hitdata* hd, const orc_hit* hit) {
  hd->albedo = m->albedo_tex < 0 ? V3(m->albedo[0], m->albedo[1], m->albedo[2])
                                 : orc_tex_uv(&s->texs[m->albedo_tex], hit->tu, hit->tv);
  hd->emission = m->emission_tex < 0 ? V3(m->emission[0], m->emission[1], m->emission[2])
                                     : orc_tex_uv(&s->texs[m->emission_tex], hit->tu, hit->tv);
  hd->roughness = m->roughness_tex < 0 ? m->roughness : orc_tex_uv(&s->texs[m->roughness_tex], hit->tu, hit->tv).x;
  hd->metallic = m->metallic_tex < 0 ? m->metallic : orc_tex_uv(&s->texs[m->metallic_tex], hit->tu, hit->tv).x;
  if (m->normal_tex < 0) {
    hd->normal = hit->normal;
  } else {
    v3 c = orc_tex_uv(&s->texs[m->normal_tex], hit->tu, hit->tv);
    v3 ln = vsub(vscale(c, 2.0f), V1(1.0f));
    hd->normal = vnormalized(vadd(vsub(vscale(hit->tangent, ln.x), vscale(hit->bitangent, ln.y)), vscale(hit->normal, ln.z)));
  }
  hd->roughness = powf(hd->roughness, 2.2f);
  hd->metallic = powf(hd->metallic, 2.2f);
  hd->clearcoatGloss = m->clearcoat_gloss;
  hd->clearcoat = m->clearcoat;
  hd->anisotropic = m->anisotropic;
  hd->eta = m->eta;
  hd->transmission = m->transmission;
  hd->specular = m->specular;
  hd->specularTint = m->specular_tint;
  hd->sheenTint = m->sheen_tint;
  hd->subsurface = m->subsurface;
  hd->sheen = m->sheen;
  hd->tangent = hit->tangent;
  hd->bitangent = hit->bitangent;
}

/* kernel.cu:175-205 */
static v3 point_light(const orc_scene* s, const orc_ray* ray, const orc_hitdata* hd, v3 point, float* pdf, float r1) {
  if (s->nlights <= 0) { *pdf = 0; return V1(0); }
  *pdf = (float)((double)(float)s->nlights / (2.0 * (double)ORC_PI));
  int32_t li = f2i_dev((float)s->nlights * r1);
  if (li > s->nlights - 1) li = s->nlights - 1;
  const er_point_light* L = &s->lights[li];
  v3 lp = V3(L->position[0], L->position[1], L->position[2]);
  v3 newDir = vnormalized(vsub(lp, point));
  float dist = vlen(vsub(lp, point));
  orc_ray sr = orc_make_ray(vadd(point, vscale(newDir, (float)0.001)), newDir);
  orc_hit sh = throw_ray(s, sr);
  float shadowDist = vlen(vsub(sh.position, point));
  if (sh.valid && shadowDist < dist) return V1(0);
  v3 plv = vdivs(V3(L->radiance[0], L->radiance[1], L->radiance[2]), dist * dist);
  v3 f = orc_disney_eval(ray, hd, newDir);
  return vdivs(vscale(vmul(plv, f), fabsf(vdot(newDir, hd->normal))), *pdf);
}

/* kernel.cu:210-258, HDRIIS branch */
static v3 hdri_light(const orc_scene* s, const orc_ray* ray, v3 point, const orc_hitdata* hd, float r1, float* pdf) {
  const orc_tex* t = &s->env;
  int32_t count = orc_hdri_search(s->cdf, r1, t->w * t->h);
  float tx = (float)(count % t->w), ty = (float)(count / t->w);
  float nu = tx / (float)t->w, nv = ty / (float)t->h;
  float iu, iv;
  orc_inverse_transform_uv(t, nu, nv, &iu, &iv);
  v3 newDir = vneg(vnormalized(orc_reverse_spherical(iu, iv)));
  *pdf = orc_hdri_pdf(t, s->radianceSum, f2i_dev(iu * (float)t->w), f2i_dev(iv * (float)t->h));
  orc_ray sr = orc_make_ray(vadd(point, vscale(newDir, (float)0.001)), newDir);
  orc_hit sh = throw_ray(s, sr);
  if (sh.valid) return V1(0);
  v3 hv = orc_tex_uv(t, iu, iv);
  v3 f = orc_disney_eval(ray, hd, newDir);
  return vdivs(vmul(vscale(f, fabsf(vdot(newDir, hd->normal))), hv), *pdf);
}

/* kernel.cu:369-443 for one pixel; u holds 5 + 4*max_depth uniforms
 * (camera r1..r5, then per vertex DisneySample r1..r3 and the shade r1). */
static int32_t path_core(const orc_scene* s, int32_t x, int32_t y, int32_t max_depth, const float* u,
                         v3* light_out, v3* nrm, v3* tan, v3* bit) {
  const er_camera* c = &s->cam;
  orc_ray ray = orc_camera_ray(c, x, y, u[0], u[1], u[2], u[3], u[4]);
  v3 light = V1(0), normal = V1(0), tangent = V1(0), bitangent = V1(0);
  v3 reduction = V1(1);
  int32_t i;
  for (i = 0; i < max_depth; i++) {
    orc_hit hit = throw_ray(s, ray);
    if (!hit.valid) {
      float eu, ev;
      orc_spherical_mapping(vscale(ray.direction, -1.0f), &eu, &ev);
      light = vadd(light, vmul(orc_tex_uv(&s->env, eu, ev), reduction));
      break;
    }
    const er_material* m = &s->mats[s->tri_mat[hit.id]];
    orc_hitdata hd;
    hit_data(s, m, &hd, &hit);
    const float* q = u + 5 + 4 * i;
    v3 dir = orc_disney_sample(&ray, &hd, q[0], q[1], q[2]);
    float r1 = q[3];
    /* shade, kernel.cu:339-358 */
    v3 f = orc_disney_eval(&ray, &hd, dir);
    float brdfPdf = orc_disney_pdf(&ray, &hd, dir);
    float hdriPdf, pointPdf = 0;
    v3 hdriC = hdri_light(s, &ray, hit.position, &hd, r1, &hdriPdf);
    v3 pointC = point_light(s, &ray, &hd, hit.position, &pointPdf, r1);
    v3 brdfC = vdivs(vmul(vscale(f, fabsf(vdot(dir, hd.normal))), hd.emission), brdfPdf);
    float w1 = hdriPdf / (hdriPdf + pointPdf + brdfPdf);
    float w2 = pointPdf / (hdriPdf + pointPdf + brdfPdf);
    float w3 = brdfPdf / (hdriPdf + pointPdf + brdfPdf);
    v3 hl = vmul(vadd(vadd(vscale(hdriC, w1), vscale(pointC, w2)), vscale(brdfC, w3)), reduction);
    reduction = vmul(reduction, vdivs(vscale(f, fabsf(vdot(dir, hd.normal))), brdfPdf));
    light = vadd(light, hl);
    if (i == 0) { normal = hit.normal; tangent = hit.tangent; bitangent = hit.bitangent; }
    ray = orc_make_ray(vadd(hit.position, vscale(dir, (float)0.001)), dir);
  }
  *light_out = light;
  if (nrm) *nrm = normal;
  if (tan) *tan = tangent;
  if (bit) *bit = bitangent;
  return i;
}

#define ORC_MAX_DEPTH 64

int32_t orc_sample(const orc_scene* s, int32_t x, int32_t y, int32_t sample, int32_t max_depth,
                   uint64_t seed, v3* light_out, v3* nrm, v3* tan, v3* bit) {
  const er_camera* c = &s->cam;
  uint32_t idx = (uint32_t)(c->x_res * (c->y_res - y - 1) + x); /* kernel.cu:378 */
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  float u[5 + 4 * ORC_MAX_DEPTH];
  uint32_t q[4];
  if (max_depth > ORC_MAX_DEPTH) max_depth = ORC_MAX_DEPTH;
  orc_philox(idx, (uint32_t)sample, 0, 0, k0, k1, q);
  for (int k = 0; k < 4; k++) u[k] = orc_u01(q[k]);
  orc_philox(idx, (uint32_t)sample, 1, 0, k0, k1, q);
  u[4] = orc_u01(q[0]);
  for (int32_t i = 0; i < max_depth; i++) {
    orc_philox(idx, (uint32_t)sample, 2u + (uint32_t)i, 0, k0, k1, q);
    for (int k = 0; k < 4; k++) u[5 + 4 * i + k] = orc_u01(q[k]);
  }
  return path_core(s, x, y, max_depth, u, light_out, nrm, tan, bit);
}

int32_t orc_sample_u(const orc_scene* s, int32_t x, int32_t y, int32_t max_depth, const float* u, float* out) {
  v3 L;
  int32_t b = path_core(s, x, y, max_depth, u, &L, NULL, NULL, NULL);
  out[0] = L.x; out[1] = L.y; out[2] = L.z; out[3] = (float)b;
  return b;
}

/* kernel.cu:445-478: FP32 running mean, NaN samples dropped */
static void accumulate(float* pass, uint32_t sa, v3 val) {
  if (!pass) return;
  if (sa > 0) {
    float k = ((float)sa) / ((float)(sa + 1));
    pass[0] *= k; pass[1] *= k; pass[2] *= k;
  }
  pass[0] += val.x / ((float)sa + 1);
  pass[1] += val.y / ((float)sa + 1);
  pass[2] += val.z / ((float)sa + 1);
}

void orc_render(const orc_scene* s, const orc_render_opts* o, float* beauty, float* normal,
                float* tangent, float* bitangent, uint32_t* samples, uint32_t* pathcount) {
  const int32_t W = s->cam.x_res, H = s->cam.y_res;
  int32_t stride = o->pixel_stride > 1 ? o->pixel_stride : 1;
  int64_t np = (int64_t)W * H;
  float* passes[4] = {beauty, normal, tangent, bitangent};
  for (int k = 0; k < 4; k++)
    if (passes[k])
      for (int64_t p = 0; p < np; p++) {
        passes[k][4 * p] = 0; passes[k][4 * p + 1] = 0; passes[k][4 * p + 2] = 0; passes[k][4 * p + 3] = 1;
      }
  if (samples) memset(samples, 0, (size_t)np * sizeof(uint32_t));
  if (pathcount) memset(pathcount, 0, (size_t)np * sizeof(uint32_t));
#ifdef _OPENMP
  if (o->nthreads > 0) omp_set_num_threads(o->nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (int64_t q = 0; q < np; q += stride) {
    int32_t x = (int32_t)(q % W), y = (int32_t)(q / W);
    int64_t idx = (int64_t)W * (H - y - 1) + x;
    uint32_t sa = 0, pc = 0;
    for (int32_t sm = 0; sm < o->spp; sm++) {
      v3 L, N, T, B;
      int32_t b = orc_sample(s, x, y, o->sample_begin + sm, o->max_depth, o->seed, &L, &N, &T, &B);
      pc += (uint32_t)b;
      L = vclamp(L, 0, 10);
      if (!(L.x != L.x) && !(L.y != L.y) && !(L.z != L.z)) {
        accumulate(beauty ? beauty + 4 * idx : NULL, sa, L);
        if (o->aov) {
          accumulate(normal ? normal + 4 * idx : NULL, sa, N);
          accumulate(tangent ? tangent + 4 * idx : NULL, sa, T);
          accumulate(bitangent ? bitangent + 4 * idx : NULL, sa, B);
        }
        sa++;
      }
    }
    if (samples) samples[idx] = sa;
    if (pathcount) pathcount[idx] = pc;
  }
}

void orc_render_paths(const orc_scene* s, const orc_render_opts* o, float* radiance, int32_t* bounces) {
  const int32_t W = s->cam.x_res, H = s->cam.y_res;
  int64_t np = (int64_t)W * H;
#ifdef _OPENMP
  if (o->nthreads > 0) omp_set_num_threads(o->nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (int64_t q = 0; q < np; q++) {
    int32_t x = (int32_t)(q % W), y = (int32_t)(q / W);
    int64_t idx = (int64_t)W * (H - y - 1) + x;
    for (int32_t sm = 0; sm < o->spp; sm++) {
      v3 L;
      int32_t b = orc_sample(s, x, y, o->sample_begin + sm, o->max_depth, o->seed, &L, NULL, NULL, NULL);
      int64_t j = (int64_t)sm * np + idx;
      radiance[3 * j] = L.x; radiance[3 * j + 1] = L.y; radiance[3 * j + 2] = L.z;
      bounces[j] = b;
    }
  }
}

/* stb_image.h:127-135 (Ankerl's approximate pow on the high word of a
 * double, published at martin.ankerl.com, 2012).  Little-endian layout. */
double orc_fastpow(double a, double b) {
  union { double d; int32_t x[2]; } u;
  u.d = a;
  u.x[1] = (int32_t)(b * (double)(u.x[1] - 1072632447) + 1072632447);
  u.x[0] = 0;
  return u.d;
}

/* main.cpp:99 clampPixels then main.cpp:156-158 */
void orc_encode_ldr(const float* rgba, int64_t n, uint8_t* out) {
  for (int64_t i = 0; i < n; i++) {
    float v = clampf_(rgba[i], 0.0f, 1.0f);
    double e = orc_fastpow((double)v, 1.0 / 2.2) * 255.0;
    if (!(e >= 0.0 && e < 256.0)) e = 0.0; /* NaN input: defined as 0 */
    out[i] = (uint8_t)(int32_t)e;
  }
}
