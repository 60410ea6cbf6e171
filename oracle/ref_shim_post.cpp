// ORACLE - test infrastructure only.  Built by oracle/Makefile (target
// `ref`) only where the reference sources are present, into oracle/_ref/.
//
// The reference's own post-processing functions (PostProcessing.cpp,
// compiled for the host from the reference tree next to this file) applied
// in the order er_postprocess applies them: applyExposure (:3-6), basicBlur
// (:132-211), reinhardTonemap (:35-39) or acesTonemap (:41-52), clampPixels
// (:30-33), applysRGB (:54-57), flipX (:19-28), flipY (:8-17).
//
// basicBlur reads memory it never writes: the alpha of the threshold image
// for pixels below the threshold (:165-168 write channel 2 twice), and the
// blur of pixels within blurSize of the border (:180-181 skip them), both
// from fresh `new float[]` arrays.  Its output there is whatever the heap
// held; golden vectors made here keep only the pixels and channels it
// defines.
#include "PostProcessing.h"

#include <cstdint>

#include "../include/eleven.h"

extern "C" void ref_postprocess(float* pix, int32_t w, int32_t h, const er_post_opts* o) {
  applyExposure(pix, w, h, o->exposure);
  if (o->bloom_power != 0.0f) basicBlur(pix, w, h, o->bloom_threshold, o->bloom_power, o->bloom_radius);
  if (o->tonemap == ER_TONEMAP_REINHARD) reinhardTonemap(pix, w, h);
  if (o->tonemap == ER_TONEMAP_ACES) acesTonemap(pix, w, h);
  if (o->clamp) clampPixels(pix, w, h);
  if (o->srgb) applysRGB(pix, w, h);
  if (o->flip_x) flipX(pix, w, h);
  if (o->flip_y) flipY(pix, w, h);
}
