// ORACLE - test infrastructure only.  Built by oracle/Makefile (target
// `ref`) only where the reference sources are present, into oracle/_ref/.
//
// The reference's own scene-folder loader -- loadScene (SceneLoader.hpp:7-143)
// with its .mtl / .obj reader (ObjLoader.hpp:20-206), the JSON parser it
// vendors (RSJparser.hpp), the stb_image decode behind Texture
// (Texture.hpp:41-68) and HDRI (HDRI.hpp:42-60), and the tangents it runs per
// object (CalcTangents, linked from ref_shim_mikk.cpp) -- compiled for the
// host from the reference tree, with the loaded Scene exported as flat
// arrays.  Used to write golden vectors that pin er_scene_folder_read.
//
// loadScene appends a Windows separator to its argument (SceneLoader.hpp:11,
// 54) and the .mtl names textures relative to the working directory
// (SceneLoader.hpp:75,104): ref_folder_load runs it from inside the folder
// with an empty path, so the folder must also hold the names "\scene.json",
// "\scene.mtl", "\scene.obj" and "\HDRI\<name>.hdr" (links to the real
// files; the golden generator makes them).
//
// stb_image keeps its vertical-flip switch in a global that the first
// texture load turns on (Texture.hpp:49): in the reference's one-scene
// process the HDR environment, loaded before any texture, is read unflipped.
// The switch is cleared before each load so that every load here starts from
// that state.
#include "SceneLoader.hpp"

#include <unistd.h>

#include <climits>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../include/eleven.h"

namespace {

struct Loaded {
  Scene scene;
};

void p3(float* o, const Vector3& a) {
  o[0] = a.x;
  o[1] = a.y;
  o[2] = a.z;
}

}  // namespace

extern "C" {

void* ref_folder_load(const char* dir) {
  char cwd[PATH_MAX];
  if (!getcwd(cwd, sizeof cwd)) return nullptr;
  if (chdir(dir) != 0) return nullptr;
  stbi_set_flip_vertically_on_load(false);
  Loaded* L = new Loaded();
  L->scene = loadScene("");
  if (chdir(cwd) != 0) {
    delete L;
    return nullptr;
  }
  return L;
}

void ref_folder_free(void* h) { delete (Loaded*)h; }

// c: triangles, objects, materials, textures, point lights, env width, env height
void ref_folder_counts(void* h, int64_t* c) {
  Scene& s = ((Loaded*)h)->scene;
  c[0] = (int64_t)s.tris.size();
  c[1] = (int64_t)s.meshObjects.size();
  c[2] = (int64_t)s.materials.size();
  c[3] = (int64_t)s.textures.size();
  c[4] = (int64_t)s.pointLights.size();
  c[5] = s.hdri.texture.width;
  c[6] = s.hdri.texture.height;
}

// Per triangle: 9 positions, 9 normals, 9 uv (Vector3 per corner as the
// reference stores them), 9 tangents, the tangent sign and the object id.
void ref_folder_tris(void* h, float* pos, float* nrm, float* uv, float* tan, float* sign, int32_t* obj) {
  Scene& s = ((Loaded*)h)->scene;
  for (size_t i = 0; i < s.tris.size(); i++) {
    const Tri& t = s.tris[i];
    for (int k = 0; k < 3; k++) {
      p3(pos + 9 * i + 3 * k, t.vertices[k]);
      p3(nrm + 9 * i + 3 * k, t.normals[k]);
      p3(uv + 9 * i + 3 * k, t.uv[k]);
      p3(tan + 9 * i + 3 * k, t.tangents[k]);
    }
    sign[i] = t.tangentsSign;
    obj[i] = t.objectID;
  }
}

void ref_folder_objects(void* h, int32_t* material, int32_t* tri_count) {
  Scene& s = ((Loaded*)h)->scene;
  for (size_t i = 0; i < s.meshObjects.size(); i++) {
    material[i] = s.meshObjects[i].materialID;
    tri_count[i] = (int32_t)s.meshObjects[i].triCount;
  }
}

// Material i in the C-ABI's layout (the same fields kernel_shim.cpp copies).
void ref_folder_material(void* h, int32_t i, er_material* e) {
  const Material& m = ((Loaded*)h)->scene.materials[(size_t)i];
  e->albedo_tex = m.albedoTextureID;
  e->emission_tex = m.emissionTextureID;
  e->roughness_tex = m.roughnessTextureID;
  e->metallic_tex = m.metallicTextureID;
  e->normal_tex = m.normalTextureID;
  p3(e->albedo, m.albedo);
  p3(e->emission, m.emission);
  e->roughness = m.roughness;
  e->metallic = m.metallic;
  e->clearcoat_gloss = m.clearcoatGloss;
  e->clearcoat = m.clearcoat;
  e->anisotropic = m.anisotropic;
  e->eta = m.eta;
  e->transmission = m.transmission;
  e->specular = m.specular;
  e->specular_tint = m.specularTint;
  e->sheen_tint = m.sheenTint;
  e->subsurface = m.subsurface;
  e->sheen = m.sheen;
}

// Texture i: wh = (width, height); data (may be NULL) = width*height*3 floats.
void ref_folder_texture(void* h, int32_t i, int32_t* wh, float* data) {
  const Texture& t = ((Loaded*)h)->scene.textures[(size_t)i];
  wh[0] = t.width;
  wh[1] = t.height;
  if (data) std::memcpy(data, t.data, sizeof(float) * 3 * (size_t)t.width * t.height);
}

// Environment texels (width*height*3) and (x_tile, y_tile, x_offset, y_offset).
void ref_folder_env(void* h, float* data, float* tile_offset) {
  const Texture& t = ((Loaded*)h)->scene.hdri.texture;
  if (data) std::memcpy(data, t.data, sizeof(float) * 3 * (size_t)t.width * t.height);
  tile_offset[0] = t.xTile;
  tile_offset[1] = t.yTile;
  tile_offset[2] = t.xOffset;
  tile_offset[3] = t.yOffset;
}

void ref_folder_camera(void* h, er_camera* c) {
  const Camera& k = ((Loaded*)h)->scene.camera;
  c->x_res = (int32_t)k.xRes;
  c->y_res = (int32_t)k.yRes;
  c->focal_length = k.focalLength;
  c->sensor_width = k.sensorWidth;
  c->sensor_height = k.sensorHeight;
  c->aperture = k.aperture;
  c->focus_distance = k.focusDistance;
  p3(c->position, k.position);
  p3(c->rotation, k.rotation);
  c->bokeh = k.bokeh ? 1 : 0;
}

void ref_folder_lights(void* h, er_point_light* out) {
  Scene& s = ((Loaded*)h)->scene;
  for (size_t i = 0; i < s.pointLights.size(); i++) {
    p3(out[i].position, s.pointLights[i].position);
    p3(out[i].radiance, s.pointLights[i].radiance);
  }
}

}  // extern "C"
