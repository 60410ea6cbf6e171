// Drop-in replacement for the host API of the reference's kernel.cu
// (declared in its kernel.h:78-84) on top of libeleven's C-ABI.
//
// A maintainer compiles this file INSIDE the reference tree, in place of
// kernel.cu, and links libeleven.so:
//
//   g++ -std=c++17 -c kernel_shim.cpp -I<reference>/src/tfg-pathtracer \
//       -I<this repo>/include -I/usr/local/cuda/include
//   g++ main.o kernel_shim.o ... -L<this repo>/tfg-pathtracer_gb300 -leleven
//
// main.cpp (main.cpp:40-56, 89-109) keeps calling renderSetup, renderCuda on
// its worker thread, and getBuffers / getSamples from the polling thread;
// the calls are serialised here with a mutex and renderCuda renders in
// chunks so progressive readback still sees intermediate images.
#include <algorithm>
#include <cstdio>
#include <mutex>
#include <vector>

#include "Definitions.h"
#include "kernel.h"

#include "eleven.h"

namespace {

std::mutex g_lock;
er_scene* g_scene = nullptr;
int g_width = 0, g_height = 0;
int g_samples_done = 0;

cudaError_t to_cuda(er_status s) {
  if (s == ER_OK) return cudaSuccess;
  std::fprintf(stderr, "eleven: %s: %s\n", er_status_string(s), er_last_error());
  return s == ER_ERR_OOM ? cudaErrorMemoryAllocation : cudaErrorUnknown;
}

er_texture texture_of(Texture& t) {
  er_texture e;
  e.width = t.width;
  e.height = t.height;
  e.data = t.data;
  e.x_tile = t.xTile;
  e.y_tile = t.yTile;
  e.x_offset = t.xOffset;
  e.y_offset = t.yOffset;
  return e;
}

}  // namespace

// kernel.cu:566-661
cudaError_t renderSetup(Scene* scene) {
  std::lock_guard<std::mutex> lk(g_lock);
  er_scene_desc d{};
  Camera& c = scene->camera;
  d.camera.x_res = (int32_t)c.xRes;
  d.camera.y_res = (int32_t)c.yRes;
  d.camera.focal_length = c.focalLength;
  d.camera.sensor_width = c.sensorWidth;
  d.camera.sensor_height = c.sensorHeight;
  d.camera.aperture = c.aperture;
  d.camera.focus_distance = c.focusDistance;
  d.camera.position[0] = c.position.x; d.camera.position[1] = c.position.y; d.camera.position[2] = c.position.z;
  d.camera.rotation[0] = c.rotation.x; d.camera.rotation[1] = c.rotation.y; d.camera.rotation[2] = c.rotation.z;
  d.camera.bokeh = c.bokeh ? 1 : 0;

  std::vector<Tri>& tris = scene->tris;
  size_t T = tris.size();
  std::vector<float> pos(9 * T), nrm(9 * T), uv(6 * T), tan(9 * T), sgn(T);
  std::vector<int32_t> obj(T);
  for (size_t i = 0; i < T; i++) {
    for (int k = 0; k < 3; k++) {
      const Tri& t = tris[i];
      pos[9 * i + 3 * k + 0] = t.vertices[k].x; pos[9 * i + 3 * k + 1] = t.vertices[k].y; pos[9 * i + 3 * k + 2] = t.vertices[k].z;
      nrm[9 * i + 3 * k + 0] = t.normals[k].x; nrm[9 * i + 3 * k + 1] = t.normals[k].y; nrm[9 * i + 3 * k + 2] = t.normals[k].z;
      tan[9 * i + 3 * k + 0] = t.tangents[k].x; tan[9 * i + 3 * k + 1] = t.tangents[k].y; tan[9 * i + 3 * k + 2] = t.tangents[k].z;
      uv[6 * i + 2 * k + 0] = t.uv[k].x; uv[6 * i + 2 * k + 1] = t.uv[k].y;
    }
    sgn[i] = tris[i].tangentsSign;
    obj[i] = tris[i].objectID;  // stamped by Scene::addMeshObject (Scene.hpp:75-93)
  }
  std::vector<int32_t> objmat(scene->meshObjects.size());
  for (size_t i = 0; i < objmat.size(); i++) objmat[i] = scene->meshObjects[i].materialID;
  std::vector<er_material> mats(scene->materials.size());
  for (size_t i = 0; i < mats.size(); i++) {
    const Material& m = scene->materials[i];
    er_material& e = mats[i];
    e.albedo_tex = m.albedoTextureID; e.emission_tex = m.emissionTextureID; e.roughness_tex = m.roughnessTextureID;
    e.metallic_tex = m.metallicTextureID; e.normal_tex = m.normalTextureID;
    e.albedo[0] = m.albedo.x; e.albedo[1] = m.albedo.y; e.albedo[2] = m.albedo.z;
    e.emission[0] = m.emission.x; e.emission[1] = m.emission.y; e.emission[2] = m.emission.z;
    e.roughness = m.roughness; e.metallic = m.metallic; e.clearcoat_gloss = m.clearcoatGloss;
    e.clearcoat = m.clearcoat; e.anisotropic = m.anisotropic; e.eta = m.eta; e.transmission = m.transmission;
    e.specular = m.specular; e.specular_tint = m.specularTint; e.sheen_tint = m.sheenTint;
    e.subsurface = m.subsurface; e.sheen = m.sheen;
  }
  std::vector<er_texture> texs;
  for (Texture& t : scene->textures) texs.push_back(texture_of(t));
  std::vector<er_point_light> lights(scene->pointLights.size());
  for (size_t i = 0; i < lights.size(); i++) {
    const PointLight& l = scene->pointLights[i];
    lights[i].position[0] = l.position.x; lights[i].position[1] = l.position.y; lights[i].position[2] = l.position.z;
    lights[i].radiance[0] = l.radiance.x; lights[i].radiance[1] = l.radiance.y; lights[i].radiance[2] = l.radiance.z;
  }
  d.tri_count = (int64_t)T;
  d.positions = pos.data();
  d.normals = nrm.data();
  d.uvs = uv.data();
  d.tangents = tan.data();
  d.tangent_sign = sgn.data();
  d.tri_object = obj.data();
  d.object_count = (int32_t)objmat.size();
  d.object_material = objmat.data();
  d.material_count = (int32_t)mats.size();
  d.materials = mats.data();
  d.texture_count = (int32_t)texs.size();
  d.textures = texs.data();
  d.light_count = (int32_t)lights.size();
  d.lights = lights.data();
  d.env = texture_of(scene->hdri.texture);
  if (g_scene) er_scene_free(g_scene);
  g_scene = nullptr;
  g_width = (int)c.xRes;
  g_height = (int)c.yRes;
  g_samples_done = 0;
  return to_cuda(er_scene_create(&d, nullptr, &g_scene));
}

// kernel.cu:665-686: sampleTarget more samples per pixel, MAXBOUNCES deep.
cudaError_t renderCuda(Scene*, int sampleTarget) {
  // 8 samples per call: two waves in flight at 1080p (a 4-sample call is a
  // single wave), and the polling thread still sees a new image every ~30 ms
  const int chunk = 8;
  for (int done = 0; done < sampleTarget; done += chunk) {
    std::lock_guard<std::mutex> lk(g_lock);
    er_render_opts o{};
    o.spp = std::min(chunk, sampleTarget - done);
    o.sample_begin = g_samples_done;
    o.max_depth = MAXBOUNCES;
    o.flags = ER_RENDER_NO_OUTPUT | ER_RENDER_AOV | (g_samples_done ? ER_RENDER_CONTINUE : 0u);
    er_status s = er_render(g_scene, &o, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
    if (s != ER_OK) return to_cuda(s);
    g_samples_done += o.spp;
  }
  return cudaSuccess;
}

// kernel.cu:688-710 (passes BEAUTY, NORMAL, TANGENT, BITANGENT; DENOISE is
// left to the caller as in the reference).
cudaError_t getBuffers(RenderData& rd, int* pathcountBuffer, int size) {
  std::lock_guard<std::mutex> lk(g_lock);
  if (!g_scene || g_samples_done == 0) return cudaSuccess;
  if (size != g_width * g_height) return cudaErrorInvalidValue;
  return to_cuda(er_film_read(g_scene, 0, rd.passes[BEAUTY], rd.passes[NORMAL], rd.passes[TANGENT],
                              rd.passes[BITANGENT], nullptr, reinterpret_cast<uint32_t*>(pathcountBuffer)));
}

// kernel.cu:712-724: samples of the first pixel.
int getSamples() {
  std::lock_guard<std::mutex> lk(g_lock);
  if (!g_scene || g_samples_done == 0) return 0;
  std::vector<uint32_t> s((size_t)g_width * g_height);
  if (er_film_read(g_scene, 0, nullptr, nullptr, nullptr, nullptr, s.data(), nullptr) != ER_OK) return 0;
  return (int)s[0];
}
