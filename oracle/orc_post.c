/*
 * ORACLE - test infrastructure only.  Restatement of the reference's
 * PostProcessing.cpp functions (applyExposure :3-6, flipX :19-28 / flipY :8-17,
 * clampPixels :30-33, reinhardTonemap :35-39, acesTonemap :41-52,
 * applysRGB :54-57, basicBlur :132-211) in the order the product's
 * er_postprocess applies them, with the reference's literal types (double
 * where its expressions hold a double literal).  basicBlur's uninitialised
 * reads (the alpha of below-threshold pixels, the blur of border pixels)
 * are defined as 0.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "orc.h"

static float clampr(float a, float b, float c) { return a < b ? b : a > c ? c : a; }

/* opts: exposure, tonemap (0 none, 1 Reinhard, 2 ACES), clamp, srgb,
 * flip_x, flip_y, bloom threshold, power, radius; pix: W*H*4 in/out */
void orc_postprocess(float* pix, int32_t w, int32_t h, const er_post_opts* o) {
  const int64_t n = (int64_t)w * h;
  for (int64_t i = 0; i < 4 * n; i++) pix[i] *= o->exposure;
  if (o->bloom_power != 0.0f) {
    int32_t blurSize = (int32_t)(o->bloom_radius / 2);
    float sd = o->bloom_radius;
    float kernelSize = (float)(blurSize * 2 + 1);
    int32_t ks = blurSize * 2 + 1;
    float* kernel = (float*)malloc(sizeof(float) * ks * ks);
    float* thr = (float*)calloc((size_t)(4 * n), sizeof(float));
    float* blur = (float*)calloc((size_t)(4 * n), sizeof(float));
    for (int32_t x = 0; x < ks; x++)
      for (int32_t y = 0; y < ks; y++) {
        float t1 = (float)(1.0 / ((2.0 * (double)ORC_PI) * (double)(sd * sd)));
        float tx = (float)(x - (int32_t)(kernelSize / 2.0));
        float ty = (float)(y - (int32_t)(kernelSize / 2.0));
        float t2 = (float)(-(double)(tx * tx + ty * ty) / (2.0 * (double)sd * (double)sd));
        kernel[x + y * ks] = t1 * expf(t2);
      }
    for (int64_t i = 0; i < n; i++) {
      float v = 0;
      v = (float)((double)v + (double)pix[4 * i] / 3.0);
      v = (float)((double)v + (double)pix[4 * i + 1] / 3.0);
      v = (float)((double)v + (double)pix[4 * i + 2] / 3.0);
      if (!(v < o->bloom_threshold)) memcpy(&thr[4 * i], &pix[4 * i], 16);
    }
    for (int32_t x = blurSize; x < w - blurSize; x++)
      for (int32_t y = blurSize; y < h - blurSize; y++) {
        float v[4] = {0, 0, 0, 0};
        int32_t ii = 0;
        for (int32_t i = x - blurSize; i <= x + blurSize; i++, ii++) {
          int32_t jj = 0;
          for (int32_t j = y - blurSize; j <= y + blurSize; j++, jj++)
            for (int k = 0; k < 4; k++) v[k] += thr[(int64_t)(i + j * w) * 4 + k] * kernel[ii + jj * ks];
        }
        memcpy(&blur[(int64_t)(x + y * w) * 4], v, 16);
      }
    for (int64_t i = 0; i < 4 * n; i++) pix[i] += blur[i] * o->bloom_power;
    free(kernel); free(thr); free(blur);
  }
  for (int64_t i = 0; i < 4 * n; i++) {
    float x = pix[i];
    if (o->tonemap == 1) {
      x = x / (1.0f + x);
    } else if (o->tonemap == 2) {
      const float a = 2.51f, b = 0.03f, c = 2.43f, d = 0.59f, e = 0.14f;
      x = clampr((float)(((double)x * 0.6 * ((double)(a * x) * 0.6 + b)) /
                         ((double)x * 0.6 * ((double)(c * x) * 0.6 + d) + e)),
                 0.0f, 1.0f);
    }
    if (o->clamp) x = clampr(x, 0.0f, 1.0f);
    if (o->srgb) x = (float)pow((double)x, 1.0 / 2.2);
    pix[i] = x;
  }
  if (o->flip_x || o->flip_y) {
    float* t = (float*)malloc(sizeof(float) * 4 * n);
    memcpy(t, pix, sizeof(float) * 4 * n);
    for (int32_t y = 0; y < h; y++)
      for (int32_t x = 0; x < w; x++) {
        int32_t sx = o->flip_x ? w - 1 - x : x, sy = o->flip_y ? h - 1 - y : y;
        memcpy(&pix[(int64_t)(x + y * w) * 4], &t[(int64_t)(sx + sy * w) * 4], 16);
      }
    free(t);
  }
}
