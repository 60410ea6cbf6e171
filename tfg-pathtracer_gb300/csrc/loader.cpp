// Scene-folder loader (SceneLoader.hpp:7-143): placeholder until the
// JSON / OBJ / MTL / BMP / HDR readers land.
#include "internal.h"

extern "C" er_status er_scene_load(const char* dir, const er_scene_opts* opts, er_scene** out) {
  (void)opts;
  if (out) *out = nullptr;
  if (!dir || !out) return er::fail(ER_ERR_INVALID_ARG, "NULL argument");
  return er::fail(ER_ERR_UNSUPPORTED, "scene-folder loading is not built yet");
}
