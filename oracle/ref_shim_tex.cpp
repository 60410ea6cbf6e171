// ORACLE - test infrastructure only.  Texture / HDRI half of the reference
// header shim (see ref_shim.cpp).  Built at -O0 -fno-unreachable-traps: the
// reference's limitUV (Math.hpp:38-41) falls off the end of a non-void
// function, which gcc otherwise turns into a trap or unreachable code.
#include "kernel.h"
#include "HDRI.hpp"
#include "Math.hpp"

#include <cstdint>
#include <cstring>

#include "../include/eleven.h"

namespace {

Vector3 g3(const float* p) { return Vector3(p[0], p[1], p[2]); }
void p3(float* o, const Vector3& a) { o[0] = a.x; o[1] = a.y; o[2] = a.z; }

Texture make_texture(const er_texture* t) {
  Texture x;
  x.data = const_cast<float*>(t->data);
  x.width = t->width;
  x.height = t->height;
  x.xTile = t->x_tile;
  x.yTile = t->y_tile;
  x.xOffset = t->x_offset;
  x.yOffset = t->y_offset;
  return x;
}

}  // namespace

extern "C" {

void ref_p_spherical(int64_t n, const float* pts, float* out) {
  for (int64_t i = 0; i < n; i++) Texture::sphericalMapping(Vector3(), g3(pts + 3 * i), 1, out[2 * i], out[2 * i + 1]);
}

void ref_p_reverse_spherical(int64_t n, const float* uv, float* out) {
  Texture t;
  for (int64_t i = 0; i < n; i++) p3(out + 3 * i, t.reverseSphericalMapping(uv[2 * i], uv[2 * i + 1]));
}

void ref_p_hdri_cdf(const er_texture* t, float* cdf, float* radiance_sum) {
  HDRI h;
  h.texture = make_texture(t);
  h.cdf = cdf;
  h.generateCDF();
  *radiance_sum = h.radianceSum;
}

// HDRI::sample, Texture::inverseTransformUV / reverseSphericalMapping /
// getValueFromUV and HDRI::pdf composed as hdriLight does.
void ref_p_hdri_sample(const er_texture* t, const float* cdf, float radiance_sum, int64_t n, const float* r,
                       float* out) {
  HDRI h;
  h.texture = make_texture(t);
  h.cdf = const_cast<float*>(cdf);
  h.radianceSum = radiance_sum;
  for (int64_t i = 0; i < n; i++) {
    Vector3 tc = h.sample(r[i]);
    float nu = tc.x / (float)h.texture.width;
    float nv = tc.y / (float)h.texture.height;
    float iu = h.texture.inverseTransformUV(nu, nv).x;
    float iv = h.texture.inverseTransformUV(nu, nv).y;
    Vector3 d = -h.texture.reverseSphericalMapping(iu, iv).normalized();
    float* o = out + 8 * i;
    o[0] = tc.x + tc.y * (float)h.texture.width;
    o[1] = h.pdf(iu * h.texture.width, iv * h.texture.height);
    p3(o + 2, d);
    p3(o + 5, h.texture.getValueFromUV(iu, iv));
  }
}

void ref_p_tex_uv(const er_texture* t, int64_t n, const float* uv, float* out) {
  Texture x = make_texture(t);
  for (int64_t i = 0; i < n; i++) p3(out + 3 * i, x.getValueFromUVFiltered(uv[2 * i], uv[2 * i + 1]));
}

}  // extern "C"
