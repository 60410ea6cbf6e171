// Device shading: textures, environment (HDRI) sampling, the BRDF-only
// Disney model and the thin-lens camera, following the reference
// (Texture.hpp:95-207, HDRI.hpp:130-162, Disney.hpp:41-253,
// Sampling.hpp:21-54, kernel.cu:260-337) in FP32.
#pragma once

#include "common.cuh"
#include "internal.h"

namespace er {

// Texture.hpp:95-112 (nearest texel, tile/offset, C remainder; a negative
// remainder is wrapped into range instead of reading outside the array).
__device__ __forceinline__ f3 tex_coord(const DevScene& S, const DevTex& t, int32_t x, int32_t y) {
  x = __float2int_rz(t.x_tile * ((float)x + t.x_offset * (float)t.w)) % t.w;
  y = __float2int_rz(t.y_tile * ((float)y + t.y_offset * (float)t.h)) % t.h;
  if (x < 0) x += t.w;
  if (y < 0) y += t.h;
  float4 c = __ldg(S.texels + t.offset + (int64_t)y * t.w + x);
  return mk(c.x, c.y, c.z);
}
__device__ __forceinline__ f3 tex_uv(const DevScene& S, const DevTex& t, float u, float v) {
  return tex_coord(S, t, __float2int_rz(u * (float)t.w), __float2int_rz(v * (float)t.h));
}

// Texture.hpp:144-156
__device__ __forceinline__ void spherical_mapping(f3 p, float& u, float& v) {
  float theta = acosf(-p.y);
  float phi = atan2f(-p.z, p.x) + ER_PI;
  u = __fdiv_rn(phi, 2.0f * ER_PI);
  v = __fdiv_rn(theta, ER_PI);
  limit_uv(u, v);
}

// Texture.hpp:195-207
__device__ __forceinline__ f3 reverse_spherical(float u, float v) {
  float phi = u * 2.0f * ER_PI;
  float theta = v * ER_PI;
  float px = cosf(phi - ER_PI);
  float py = -cosf(theta);
  float pz = -sinf(phi - ER_PI);
  float a = sqrtf(1.0f - py * py);
  return mk(a * px, py, a * pz);
}

// HDRI.hpp:130-142 (returns `to`, not an exact lower bound).  The loop is
// bounded: with a NaN CDF (an all-black environment divides by a zero sum)
// the reference's search never terminates.
__device__ __forceinline__ int32_t hdri_search(const float* __restrict__ arr, float value, int32_t length) {
  int32_t from = 0, to = length - 1;
  for (int it = 0; it < 64 && to - from > 0; it++) {
    int32_t m = from + (to - from) / 2;
    float a = __ldg(arr + m);
    if (value == a) return m;
    if (value < a) to = m - 1;
    if (value > a) from = m + 1;
  }
  return to;
}

// HDRI.hpp:145-152 (theta from the texel's top edge)
// dv: the environment value at storage coordinates (x, y) (tex_coord).
__device__ __forceinline__ float hdri_pdf(const DevScene& S, f3 dv, int32_t y) {
  const DevTex& t = S.env;
  float theta = __fdiv_rn((float)y, (float)t.h) * ER_PI;
  float a = __fdiv_rn((dv.x + dv.y) + dv.z, S.radiance_sum) * (float)t.w * (float)t.h;
  return a / (2.0f * ER_PI * sinf(theta));
}

struct HitData {  // kernel.h:46-69
  float metallic, roughness, clearcoatGloss, clearcoat, anisotropic, transmission, specular, specularTint,
      sheenTint, subsurface, sheen;
  f3 emission, albedo, normal;
};

// Disney.hpp:41-45: zero basis when the normal is +-y
__device__ __forceinline__ void create_basis(f3 n, f3& t, f3& b) {
  t = normalized(cross(mk(0.f, 1.f, 0.f), n));
  b = normalized(cross(n, t));
}
__device__ __forceinline__ float schlick(float u) {
  float m = clampf_(1.0f - u, 0.0f, 1.0f);
  float m2 = m * m;
  return m2 * m2 * m;
}
__device__ __forceinline__ float gtr1(float NDotH, float a) {
  if (a >= 1.0f) return 1.0f / ER_PI;
  float a2 = a * a;
  float t = 1.0f + (a2 - 1.0f) * NDotH * NDotH;
  return (a2 - 1.0f) / (ER_PI * logf(a2) * t);
}
__device__ __forceinline__ float gtr2_aniso(float NDotH, float HDotX, float HDotY, float ax, float ay) {
  float a = HDotX / ax, b = HDotY / ay;
  float c = a * a + b * b + NDotH * NDotH;
  return 1.0f / (ER_PI * ax * ay * c * c);
}
__device__ __forceinline__ float smith_ggx(float NDotV, float alphaG) {
  float a = alphaG * alphaG, b = NDotV * NDotV;
  return 1.0f / (NDotV + sqrtf(a + b - a * b));
}
__device__ __forceinline__ float smith_ggx_aniso(float NDotV, float VDotX, float VDotY, float ax, float ay) {
  float a = VDotX * ax, b = VDotY * ay, c = NDotV;
  return 1.0f / (NDotV + sqrtf(a * a + b * b + c * c));
}

// Per-hit constants shared by the three DisneyEval calls of a vertex.
struct DisneyCtx {
  f3 N, V, T, B;
  float ax, ay, diffuseRatio, specularRatio, clearcoatAlpha, ccRatio;
};

__device__ __forceinline__ DisneyCtx disney_ctx(const HitData& hd, f3 raydir) {
  DisneyCtx c;
  c.N = hd.normal;
  c.V = -raydir;
  create_basis(hd.normal, c.T, c.B);
  float aspect = sqrtf(1.0f - hd.anisotropic * 0.9f);
  c.ax = maxf_(0.001f, hd.roughness / aspect);
  c.ay = maxf_(0.001f, hd.roughness * aspect);
  c.diffuseRatio = 0.5f * (1.0f - hd.metallic);
  c.specularRatio = 1.0f - c.diffuseRatio;
  c.clearcoatAlpha = lerpf_(0.1f, 0.001f, hd.clearcoatGloss);
  c.ccRatio = 1.0f / (1.0f + hd.clearcoat);
  return c;
}

// Disney.hpp:108-147 (1 when N.L <= 0)
__device__ __forceinline__ float disney_pdf(const DisneyCtx& c, f3 L) {
  f3 H = normalized(L + c.V);
  float NDotH = fabsf(dot(c.N, H));
  if (dot(c.N, L) <= 0.0f) return 1.0f;
  float pdfGTR2 = gtr2_aniso(NDotH, dot(H, c.T), dot(H, c.B), c.ax, c.ay) * NDotH;
  float pdfGTR1 = gtr1(NDotH, c.clearcoatAlpha) * NDotH;
  float pdfSpec = lerpf_(pdfGTR1, pdfGTR2, c.ccRatio) / (4.0f * fabsf(dot(L, H)));
  float pdfDiff = fabsf(dot(L, c.N)) * (1.0f / ER_PI);
  return c.diffuseRatio * pdfDiff + c.specularRatio * pdfSpec;
}

// Disney.hpp:150-177 + Sampling.hpp:31-54 (not re-normalised)
__device__ __forceinline__ f3 disney_sample(const HitData& hd, const DisneyCtx& c, float r1, float r2, float r3) {
  if (r3 < c.diffuseRatio) {
    float r = sqrtf(r1);
    float phi = 2.0f * ER_PI * r2;
    float hx = r * cosf(phi), hy = r * sinf(phi);
    float hz = sqrtf(maxf_(0.0f, 1.0f - hx * hx - hy * hy));
    return c.T * hx + c.B * hy + c.N * hz;
  }
  float a = maxf_(0.001f, hd.roughness);
  float phi = r1 * ER_PI * 2.0f;
  float cosTheta = sqrtf((1.0f - r2) / (1.0f + (a * a - 1.0f) * r2));
  float sinTheta = clampf_(sqrtf(1.0f - cosTheta * cosTheta), 0.0f, 1.0f);
  f3 H = c.T * (sinTheta * cosf(phi)) + c.B * (sinTheta * sinf(phi)) + c.N * cosTheta;
  f3 v = -c.V;
  return v - H * (2.0f * dot(v, H));
}

// DisneyEval's condition for a non-zero value (Disney.hpp:200): outside it
// the value and every partial are zero.
__device__ __forceinline__ bool disney_gate(const HitData& hd, const DisneyCtx& c, f3 L) {
  return hd.transmission < 1.0f && dot(c.N, L) > 0.0f && dot(c.N, c.V) > 0.0f;
}

// Disney.hpp:179-253
__device__ __forceinline__ f3 disney_eval(const HitData& hd, const DisneyCtx& c, f3 L) {
  f3 brdf = mk1(0.0f);
  if (disney_gate(hd, c, L)) {
    f3 H = normalized(L + c.V);
    float NDotL = fabsf(dot(c.N, L));
    float NDotV = fabsf(dot(c.N, c.V));
    float NDotH = fabsf(dot(c.N, H));
    float LDotH = fabsf(dot(L, H));
    f3 Cdlin = hd.albedo;
    float Cdlum = 0.3f * Cdlin.x + 0.6f * Cdlin.y + 0.1f * Cdlin.z;
    f3 Ctint = Cdlum > 0.0f ? Cdlin / Cdlum : mk1(1.0f);
    f3 Cspec0 = lerp3(lerp3(mk1(1.0f), Ctint, hd.specularTint) * (hd.specular * 0.08f), Cdlin, hd.metallic);
    f3 Csheen = lerp3(mk1(1.0f), Ctint, hd.sheenTint);
    float FL = schlick(NDotL), FV = schlick(NDotV);
    float Fd90 = 0.5f + 2.0f * LDotH * LDotH * hd.roughness;
    float Fd = lerpf_(1.0f, Fd90, FL) * lerpf_(1.0f, Fd90, FV);
    float Fss90 = LDotH * LDotH * hd.roughness;
    float Fss = lerpf_(1.0f, Fss90, FL) * lerpf_(1.0f, Fss90, FV);
    float ss = 1.25f * (Fss * (1.0f / (NDotL + NDotV) - 0.5f) + 0.5f);
    float Ds = gtr2_aniso(NDotH, dot(H, c.T), dot(H, c.B), c.ax, c.ay);
    float FH = schlick(LDotH);
    f3 Fs = lerp3(Cspec0, mk1(1.0f), FH);
    float Gs = smith_ggx_aniso(NDotL, dot(L, c.T), dot(L, c.B), c.ax, c.ay);
    Gs *= smith_ggx_aniso(NDotV, dot(c.V, c.T), dot(c.V, c.B), c.ax, c.ay);
    f3 Fsheen = Csheen * (FH * hd.sheen);
    float Dr = gtr1(NDotH, c.clearcoatAlpha);
    float Fr = lerpf_(0.04f, 1.0f, FH);
    float Gr = smith_ggx(NDotL, 0.25f) * smith_ggx(NDotV, 0.25f);
    float kd = (1.0f / ER_PI) * lerpf_(Fd, ss, hd.subsurface);
    f3 diff = (Cdlin * kd + Fsheen) * (1.0f - hd.metallic);
    f3 spec = Fs * Gs * Ds;
    float cc = 0.25f * hd.clearcoat * Gr * Fr * Dr;
    brdf = diff + spec + mk1(cc);
  }
  return brdf;
}

// kernel.cu:260-337 with the rotation trigonometry hoisted.  The two
// expressions the reference evaluates in double are kept in double (one
// camera ray per sample).
__device__ __forceinline__ void camera_ray(const DevCamera& c, int32_t x, int32_t y, float r1, float r2, float r3,
                                           float r4, float r5, f3& o, f3& d) {
  float dx = __fadd_rn(c.px, __fmul_rn(__fdiv_rn((float)x, (float)c.x_res), c.sensor_width));
  float dy = __fadd_rn(c.py, __fmul_rn(__fdiv_rn((float)y, (float)c.y_res), c.sensor_height));
  float odx = __fadd_rn(__fmul_rn(-c.sensor_width, 0.5f), dx);
  float ody = __fadd_rn(__fmul_rn(-c.sensor_height, 0.5f), dy);
  float rx = (float)((1.0 / (double)(float)c.x_res) * ((double)r1 - 0.5) * (double)c.sensor_width);
  float ry = (float)((1.0 / (double)(float)c.y_res) * ((double)r2 - 0.5) * (double)c.sensor_height);
  float SPx = __fadd_rn(odx, rx), SPy = __fadd_rn(ody, ry), SPz = __fadd_rn(c.pz, c.focal_length);
  f3 pos = mk(c.px, c.py, c.pz);
  f3 dir = xsub(mk(SPx, SPy, SPz), pos);
  f3 dX = mk(dir.x, __fsub_rn(__fmul_rn(dir.y, c.cx), __fmul_rn(dir.z, c.sx)),
             __fadd_rn(__fmul_rn(dir.y, c.sx), __fmul_rn(dir.z, c.cx)));
  f3 dY = mk(__fadd_rn(__fmul_rn(dX.x, c.cy), __fmul_rn(dX.z, c.sy)), dX.y,
             __fsub_rn(__fmul_rn(dX.z, c.cy), __fmul_rn(dX.x, c.sy)));
  f3 dZ = mk(__fsub_rn(__fmul_rn(dY.x, c.cz), __fmul_rn(dY.y, c.sz)),
             __fadd_rn(__fmul_rn(dY.x, c.sz), __fmul_rn(dY.y, c.cz)), dY.z);
  o = pos;
  d = xnormalize(dZ);
  if (c.bokeh) {
    float diameter = __fdiv_rn(c.focal_length, c.aperture);
    float l = __fadd_rn(c.focus_distance, c.focal_length);
    f3 focus = xadd(o, xscale(d, l));
    float t = __fmul_rn(__fmul_rn(2.0f, ER_PI), r3);
    float u = __fadd_rn(r4, r5);
    float r = u > 1.0f ? __fsub_rn(2.0f, u) : u;
    float rIPx = __fmul_rn(__fmul_rn(r, cosf(t)), __fmul_rn(diameter, 0.5f));
    float rIPy = __fmul_rn(__fmul_rn(r, sinf(t)), __fmul_rn(diameter, 0.5f));
    f3 orig = xadd(pos, mk(rIPx, rIPy, 0.0f));
    o = orig;
    d = xnormalize(xsub(focus, orig));
  }
}

}  // namespace er
