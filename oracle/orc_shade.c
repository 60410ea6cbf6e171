/*
 * ORACLE - test infrastructure only.  Restatement of the reference's shading
 * pieces: textures (src/tfg-pathtracer/Texture.hpp:95-207), the HDRI CDF,
 * search and pdf (HDRI.hpp:107-162), the sampling helpers (Sampling.hpp),
 * the BRDF-only Disney model (Disney.hpp:41-253) and the thin-lens camera
 * ray (kernel.cu:260-337).  Literal types follow the reference: a double
 * literal in a float expression promotes that expression to double and the
 * result is rounded when stored to float.
 */
#include "orc.h"

/* Texture.hpp:95-112: tile/offset, truncation, C remainder.  A negative
 * remainder (u < 0, negative offsets) makes the reference read outside the
 * texel array; it is wrapped into range here instead (defined behaviour,
 * identical to the reference for every in-range index). */
v3 orc_tex_coord(const orc_tex* t, int32_t x, int32_t y) {
  x = f2i_dev(t->xTile * ((float)x + t->xOffset * (float)t->w)) % t->w;
  y = f2i_dev(t->yTile * ((float)y + t->yOffset * (float)t->h)) % t->h;
  if (x < 0) x += t->w;
  if (y < 0) y += t->h;
  int64_t i = 3 * ((int64_t)y * t->w + x);
  return V3(t->data[i], t->data[i + 1], t->data[i + 2]);
}

/* Texture.hpp:114-116 (getValueFromUV == getValueFromUVFiltered with the
 * NO_FILTER default of Texture.hpp:21) */
v3 orc_tex_uv(const orc_tex* t, float u, float v) {
  return orc_tex_coord(t, f2i_dev(u * (float)t->w), f2i_dev(v * (float)t->h));
}

/* Texture.hpp:144-156 with origin 0 and radius 1 */
void orc_spherical_mapping(v3 p, float* u, float* v) {
  float theta = acosf(-p.y);
  float phi = atan2f(-p.z, p.x) + ORC_PI;
  *u = phi / (2.0f * ORC_PI);
  *v = theta / ORC_PI;
  limit_uv(u, v);
}

/* Texture.hpp:195-207 */
v3 orc_reverse_spherical(float u, float v) {
  float phi = u * 2.0f * ORC_PI;
  float theta = v * ORC_PI;
  float px = cosf(phi - ORC_PI);
  float py = -cosf(theta);
  float pz = -sinf(phi - ORC_PI);
  float a = sqrtf(1.0f - py * py);
  return V3(a * px, py, a * pz);
}

/* Texture.hpp:177-193 */
void orc_inverse_transform_uv(const orc_tex* t, float u, float v, float* nu, float* nv) {
  int32_t x = f2i_dev(u * (float)t->w);
  int32_t y = f2i_dev(v * (float)t->h);
  x = f2i_dev(t->xTile * ((float)x - t->xOffset * (float)t->w)) % t->w;
  y = f2i_dev(t->yTile * ((float)y - t->yOffset * (float)t->h)) % t->h;
  *nu = (float)x / (float)t->w;
  *nv = (float)y / (float)t->h;
  limit_uv(nu, nv);
}

/* HDRI.hpp:107-128: FP32 running sums in row-major order. */
void orc_hdri_cdf(const orc_tex* t, float* cdf, float* radianceSum) {
  float sum = 0;
  cdf[0] = 0;
  for (int32_t j = 0; j < t->h; j++)
    for (int32_t i = 0; i < t->w; i++) {
      v3 d = orc_tex_coord(t, i, j);
      sum += d.x + d.y + d.z;
    }
  int64_t c = 0;
  for (int32_t j = 0; j < t->h; j++)
    for (int32_t i = 0; i < t->w; i++) {
      v3 d = orc_tex_coord(t, i, j);
      cdf[c + 1] = cdf[c] + (d.x + d.y + d.z) / sum;
      c++;
    }
  *radianceSum = sum;
}

/* HDRI.hpp:130-142: returns `to`, not an exact lower bound.  Bounded to 64
 * steps: with a NaN CDF (all-black environment, zero sum) the reference's
 * loop never ends. */
int32_t orc_hdri_search(const float* arr, float value, int32_t length) {
  int32_t from = 0, to = length - 1;
  for (int it = 0; it < 64 && to - from > 0; it++) {
    int32_t m = from + (to - from) / 2;
    if (value == arr[m]) return m;
    if (value < arr[m]) to = m - 1;
    if (value > arr[m]) from = m + 1;
  }
  return to;
}

/* HDRI.hpp:145-152: theta from the texel's top edge. */
float orc_hdri_pdf(const orc_tex* t, float radianceSum, int32_t x, int32_t y) {
  v3 dv = orc_tex_coord(t, x, y);
  float theta = ((float)y / (float)t->h) * ORC_PI;
  float a = ((dv.x + dv.y + dv.z) / radianceSum) * (float)t->w * (float)t->h;
  return (float)((double)a / (2.0 * (double)ORC_PI * (double)sinf(theta)));
}

/* ---------------------------------------------------------------- Disney */

/* Disney.hpp:41-45: degenerate (zero) basis when the normal is +-y */
static void create_basis(v3 n, v3* t, v3* b) {
  *t = vnormalized(vcross(V3(0, 1, 0), n));
  *b = vnormalized(vcross(n, *t));
}

/* Disney.hpp:47-51 */
static float schlick(float u) {
  float m = clampf_((float)(1.0 - (double)u), 0.0f, 1.0f);
  float m2 = m * m;
  return m2 * m2 * m;
}

/* Disney.hpp:68-74 */
static float gtr1(float NDotH, float a) {
  if (a >= 1.0) return 1.0f / ORC_PI;
  float a2 = a * a;
  float t = (float)(1.0 + ((double)a2 - 1.0) * (double)NDotH * (double)NDotH);
  return (float)(((double)a2 - 1.0) / (double)(ORC_PI * logf(a2) * t));
}

/* Disney.hpp:82-87 */
static float gtr2_aniso(float NDotH, float HDotX, float HDotY, float ax, float ay) {
  float a = HDotX / ax;
  float b = HDotY / ay;
  float c = a * a + b * b + NDotH * NDotH;
  return (float)(1.0 / (double)(ORC_PI * ax * ay * c * c));
}

/* Disney.hpp:89-93 */
static float smith_ggx(float NDotV, float alphaG) {
  float a = alphaG * alphaG;
  float b = NDotV * NDotV;
  return (float)(1.0 / (double)(NDotV + sqrtf(a + b - a * b)));
}

/* Disney.hpp:95-100 */
static float smith_ggx_aniso(float NDotV, float VDotX, float VDotY, float ax, float ay) {
  float a = VDotX * ax;
  float b = VDotY * ay;
  float c = NDotV;
  return (float)(1.0 / (double)(NDotV + sqrtf(a * a + b * b + c * c)));
}

/* Disney.hpp:108-147 (returns 1 when N.L <= 0) */
float orc_disney_pdf(const orc_ray* ray, const orc_hitdata* hd, v3 L) {
  v3 N = hd->normal;
  v3 Vv = vscale(ray->direction, -1.0f);
  v3 H = vnormalized(vadd(L, Vv));
  v3 T, B;
  create_basis(hd->normal, &T, &B);
  float NDotH = fabsf(vdot(N, H));
  if (vdot(N, L) <= 0.0) return 1.0f;
  float clearcoatAlpha = lerpf_((float)0.1, (float)0.001, hd->clearcoatGloss);
  float diffuseRatio = (float)(0.5 * (1.0 - (double)hd->metallic));
  float specularRatio = (float)(1.0 - (double)diffuseRatio);
  float aspect = (float)sqrt(1.0 - (double)hd->anisotropic * 0.9);
  float ax = maxf_((float)0.001, hd->roughness / aspect);
  float ay = maxf_((float)0.001, hd->roughness * aspect);
  float pdfGTR2 = gtr2_aniso(NDotH, vdot(H, T), vdot(H, B), ax, ay) * NDotH;
  float pdfGTR1 = gtr1(NDotH, clearcoatAlpha) * NDotH;
  float ratio = (float)(1.0 / (1.0 + (double)hd->clearcoat));
  float pdfSpec = (float)((double)lerpf_(pdfGTR1, pdfGTR2, ratio) / (4.0 * (double)fabsf(vdot(L, H))));
  float pdfDiff = (float)((double)fabsf(vdot(L, N)) * (1.0 / (double)ORC_PI));
  return diffuseRatio * pdfDiff + specularRatio * pdfSpec;
}

/* Sampling.hpp:31-41 */
static v3 cosine_hemisphere(float u1, float u2) {
  v3 d;
  float r = sqrtf(u1);
  float phi = (float)(2.0 * (double)ORC_PI * (double)u2);
  d.x = r * cosf(phi);
  d.y = r * sinf(phi);
  d.z = sqrtf(maxf_(0.0f, (float)(1.0 - (double)(d.x * d.x) - (double)(d.y * d.y))));
  return d;
}

/* Sampling.hpp:43-54: roughness used as alpha directly */
static v3 importance_ggx(float rgh, float r1, float r2) {
  float a = maxf_((float)0.001, rgh);
  float phi = r1 * ORC_PI * 2.0f;
  float cosTheta = (float)sqrt((1.0 - (double)r2) / (1.0 + ((double)(a * a) - 1.0) * (double)r2));
  float sinTheta = clampf_((float)sqrt(1.0 - (double)(cosTheta * cosTheta)), 0.0f, 1.0f);
  float sinPhi = sinf(phi);
  float cosPhi = cosf(phi);
  return V3(sinTheta * cosPhi, sinTheta * sinPhi, cosTheta);
}

/* Disney.hpp:150-177: the result is not re-normalised here. */
v3 orc_disney_sample(const orc_ray* ray, const orc_hitdata* hd, float r1, float r2, float r3) {
  v3 N = hd->normal;
  v3 Vv = vscale(ray->direction, -1.0f);
  v3 T, B;
  create_basis(hd->normal, &T, &B);
  float diffuseRatio = (float)(0.5 * (1.0 - (double)hd->metallic));
  if (r3 < diffuseRatio) {
    v3 H = cosine_hemisphere(r1, r2);
    return vadd(vadd(vscale(T, H.x), vscale(B, H.y)), vscale(N, H.z));
  }
  v3 H = importance_ggx(hd->roughness, r1, r2);
  H = vadd(vadd(vscale(T, H.x), vscale(B, H.y)), vscale(N, H.z));
  return vreflect(vscale(Vv, -1.0f), H);
}

/* Disney.hpp:179-253 */
v3 orc_disney_eval(const orc_ray* ray, const orc_hitdata* hd, v3 L) {
  v3 Vv = vscale(ray->direction, -1.0f);
  v3 T, B;
  create_basis(hd->normal, &T, &B);
  v3 H = vnormalized(vadd(L, Vv));
  float NDotL = fabsf(vdot(hd->normal, L));
  float NDotV = fabsf(vdot(hd->normal, Vv));
  float NDotH = fabsf(vdot(hd->normal, H));
  float LDotH = fabsf(vdot(L, H));
  v3 brdf = V1(0.0f);
  if (hd->transmission < 1.0 && vdot(hd->normal, L) > 0.0 && vdot(hd->normal, Vv) > 0.0) {
    v3 Cdlin = hd->albedo;
    float Cdlum = (float)(0.3 * (double)Cdlin.x + 0.6 * (double)Cdlin.y + 0.1 * (double)Cdlin.z);
    v3 Ctint = Cdlum > 0.0 ? vdivs(Cdlin, Cdlum) : V1(1.0f);
    v3 Cspec0 = vlerp(vscale(vlerp(V1(1.0f), Ctint, hd->specularTint), (float)((double)hd->specular * 0.08)),
                      Cdlin, hd->metallic);
    v3 Csheen = vlerp(V1(1.0f), Ctint, hd->sheenTint);
    float FL = schlick(NDotL);
    float FV = schlick(NDotV);
    float Fd90 = (float)(0.5 + 2.0 * (double)LDotH * (double)LDotH * (double)hd->roughness);
    float Fd = lerpf_(1.0f, Fd90, FL) * lerpf_(1.0f, Fd90, FV);
    float Fss90 = LDotH * LDotH * hd->roughness;
    float Fss = lerpf_(1.0f, Fss90, FL) * lerpf_(1.0f, Fss90, FV);
    float ss = (float)(1.25 * ((double)Fss * (1.0 / (double)(NDotL + NDotV) - 0.5) + 0.5));
    float aspect = (float)sqrt(1.0 - (double)hd->anisotropic * 0.9);
    float ax = maxf_((float)0.001, hd->roughness / aspect);
    float ay = maxf_((float)0.001, hd->roughness * aspect);
    float Ds = gtr2_aniso(NDotH, vdot(H, T), vdot(H, B), ax, ay);
    float FH = schlick(LDotH);
    v3 Fs = vlerp(Cspec0, V1(1.0f), FH);
    float Gs = smith_ggx_aniso(NDotL, vdot(L, T), vdot(L, B), ax, ay);
    Gs *= smith_ggx_aniso(NDotV, vdot(Vv, T), vdot(Vv, B), ax, ay);
    v3 Fsheen = vscale(Csheen, FH * hd->sheen);
    float Dr = gtr1(NDotH, lerpf_((float)0.1, (float)0.001, hd->clearcoatGloss));
    float Fr = lerpf_((float)0.04, 1.0f, FH);
    float Gr = smith_ggx(NDotL, 0.25f) * smith_ggx(NDotV, 0.25f);
    float kd = (float)((1.0 / (double)ORC_PI) * (double)lerpf_(Fd, ss, hd->subsurface));
    v3 diff = vscale(vadd(vscale(Cdlin, kd), Fsheen), (float)(1.0 - (double)hd->metallic));
    v3 spec = vscale(vscale(Fs, Gs), Ds);
    float cc = (float)(0.25 * (double)hd->clearcoat * (double)Gr * (double)Fr * (double)Dr);
    brdf = vadds(vadd(diff, spec), cc);
  }
  return brdf;
}

/* Sampling.hpp:10-19 (unused on the hot path with HDRIIS on) */
static v3 uniform_sphere(float u1, float u2) {
  float z = (float)(1.0 - 2.0 * (double)u1);
  float r = sqrtf(maxf_(0.f, (float)(1.0 - (double)(z * z))));
  float phi = (float)(2.0 * (double)ORC_PI * (double)u2);
  return V3(r * cosf(phi), r * sinf(phi), z);
}

static void circle_sample(float u1, float u2, float u3, float* x, float* y);

/* Probe: out 12 per item (see ref_p_sampling in ref_shim.cpp) */
void orc_p_sampling(int64_t n, const float* u, float* out) {
  for (int64_t i = 0; i < n; i++) {
    const float* q = u + 3 * i;
    float* o = out + 12 * i;
    v3 a = uniform_sphere(q[0], q[1]);
    v3 b = cosine_hemisphere(q[0], q[1]);
    v3 c = importance_ggx(q[2], q[0], q[1]);
    o[0] = a.x; o[1] = a.y; o[2] = a.z;
    o[3] = b.x; o[4] = b.y; o[5] = b.z;
    o[6] = c.x; o[7] = c.y; o[8] = c.z;
    circle_sample(q[0], q[1], q[2], &o[9], &o[10]);
    o[11] = 0;
  }
}

/* ---------------------------------------------------------------- camera */

/* Sampling.hpp:21-29: radius u2+u3 folded at 1 */
static void circle_sample(float u1, float u2, float u3, float* x, float* y) {
  float t = 2.0f * ORC_PI * u1;
  float u = u2 + u3;
  float r = u > 1 ? 2 - u : u;
  *x = r * cosf(t);
  *y = r * sinf(t);
}

/* kernel.cu:260-337 */
orc_ray orc_camera_ray(const er_camera* c, int32_t x, int32_t y, float r1, float r2, float r3, float r4, float r5) {
  float dx = c->position[0] + ((float)x) / ((float)c->x_res) * c->sensor_width;
  float dy = c->position[1] + ((float)y) / ((float)c->y_res) * c->sensor_height;
  float odx = (float)((double)(-c->sensor_width) / 2.0 + (double)dx);
  float ody = (float)((double)(-c->sensor_height) / 2.0 + (double)dy);
  float rx = (float)((1.0 / (double)(float)c->x_res) * ((double)r1 - 0.5) * (double)c->sensor_width);
  float ry = (float)((1.0 / (double)(float)c->y_res) * ((double)r2 - 0.5) * (double)c->sensor_height);
  float SPx = odx + rx;
  float SPy = ody + ry;
  float SPz = c->position[2] + c->focal_length;
  float k = (float)((double)ORC_PI / 180.0);
  v3 rot = V3(c->rotation[0] * k, c->rotation[1] * k, c->rotation[2] * k);
  v3 pos = V3(c->position[0], c->position[1], c->position[2]);
  v3 d = vsub(V3(SPx, SPy, SPz), pos);
  v3 dX = V3(d.x, d.y * cosf(rot.x) - d.z * sinf(rot.x), d.y * sinf(rot.x) + d.z * cosf(rot.x));
  v3 dY = V3(dX.x * cosf(rot.y) + dX.z * sinf(rot.y), dX.y, dX.z * cosf(rot.y) - dX.x * sinf(rot.y));
  v3 dZ = V3(dY.x * cosf(rot.z) - dY.y * sinf(rot.z), dY.x * sinf(rot.z) + dY.y * cosf(rot.z), dY.z);
  orc_ray ray = orc_make_ray(pos, dZ);
  if (c->bokeh) {
    float rIPx, rIPy;
    float diameter = c->focal_length / c->aperture;
    float l = c->focus_distance + c->focal_length;
    v3 focus = vadd(ray.origin, vscale(ray.direction, l));
    circle_sample(r3, r4, r5, &rIPx, &rIPy);
    rIPx = (float)((double)rIPx * ((double)diameter * 0.5));
    rIPy = (float)((double)rIPy * ((double)diameter * 0.5));
    v3 orig = vadd(pos, V3(rIPx, rIPy, 0));
    ray = orc_make_ray(orig, vsub(focus, orig));
  }
  return ray;
}
