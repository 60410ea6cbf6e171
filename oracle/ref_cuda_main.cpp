// ORACLE - test infrastructure only: a headless caller of the reference's
// own CUDA renderer, built by oracle/Makefile (target `refcuda`) from a
// scratch copy of the reference tree with the patches that Makefile lists,
// into oracle/_ref/.  It stands in for the reference's main.cpp, which needs
// a window, OpenGL and OIDN: it builds the reference's Scene from a flat
// scene file (the same arrays er_scene_create takes, written by
// oracle/refcuda_scene.py), then runs the reference's renderSetup
// (kernel.cu:566-661, which builds its BVH on the host), renderCuda
// (kernel.cu:665-686, one renderingKernel launch per sample) and
// getBuffers / getSamples (kernel.cu:688-724), as main.cpp:51-53,97-102 do.
//
//   ref_cuda <scene file> <warm-up spp> <timed spp> [beauty out]
//
// Prints one JSON line: timed milliseconds (CUDA events on the reference's
// kernelStream around renderCuda), samples, the reference's path counter
// (sum of bounce counts, kernel.cu:445) and the set-up times.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "Definitions.h"
#include "kernel.h"
#include "mikktspaceCallback.hpp"

extern cudaStream_t kernelStream;  // kernel.cu:49

namespace {

// er_material's layout (include/eleven.h): five texture ids, albedo,
// emission, then roughness, metallic, clearcoatGloss, clearcoat,
// anisotropic, eta, transmission, specular, specularTint, sheenTint,
// subsurface, sheen.
struct er_material_raw {
  int32_t tex[5];
  float albedo[3];
  float emission[3];
  float f[12];
};
static_assert(sizeof(er_material_raw) == 92, "material record");

struct Reader {
  FILE* f;
  bool ok = true;
  template <class T>
  T get() {
    T v{};
    ok = ok && std::fread(&v, sizeof(T), 1, f) == 1;
    return v;
  }
  template <class T>
  void arr(std::vector<T>& v, size_t n) {
    v.resize(n);
    ok = ok && (n == 0 || std::fread(v.data(), sizeof(T), n, f) == n);
  }
};

Vector3 v3(const float* p) { return Vector3(p[0], p[1], p[2]); }

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

bool read_texture(Reader& r, Texture& t) {
  int32_t w = r.get<int32_t>(), h = r.get<int32_t>();
  if (!r.ok || w <= 0 || h <= 0) return false;
  std::vector<float> data;
  r.arr(data, (size_t)w * h * 3);
  float to[4];
  for (float& x : to) x = r.get<float>();
  if (!r.ok) return false;
  t.width = w;
  t.height = h;
  t.data = new float[(size_t)w * h * 3];
  std::memcpy(t.data, data.data(), data.size() * sizeof(float));
  t.xTile = to[0];
  t.yTile = to[1];
  t.xOffset = to[2];
  t.yOffset = to[3];
  return true;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: %s <scene file> <warm-up spp> <timed spp> [beauty out]\n", argv[0]);
    return 2;
  }
  const int warm = std::atoi(argv[2]), spp = std::atoi(argv[3]);
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 3;
  Reader r{f};
  char magic[4];
  if (std::fread(magic, 1, 4, f) != 4 || std::memcmp(magic, "ERSC", 4) != 0) return 3;
  double t0 = now_ms();

  Scene scene;
  // camera (Camera.hpp:29-37 then the fields loadScene sets, SceneLoader.hpp:40-46)
  int32_t xres = r.get<int32_t>(), yres = r.get<int32_t>();
  if (xres <= 0 || yres <= 0 || xres > 1920 || yres > 1080) return 4;  // static buffers, kernel.cu:41-45
  scene.camera = Camera(xres, yres);
  scene.camera.focalLength = r.get<float>();
  scene.camera.sensorWidth = r.get<float>();
  scene.camera.sensorHeight = r.get<float>();
  scene.camera.aperture = r.get<float>();
  scene.camera.focusDistance = r.get<float>();
  float pr[6];
  for (float& x : pr) x = r.get<float>();
  scene.camera.position = v3(pr);
  scene.camera.rotation = v3(pr + 3);
  scene.camera.bokeh = r.get<int32_t>() != 0;

  // triangles, grouped into mesh objects (Scene::addMeshObject, Scene.hpp:75-93)
  int64_t T = r.get<int64_t>();
  std::vector<float> pos, nrm, uv, tan, sgn;
  std::vector<int32_t> tobj;
  r.arr(pos, (size_t)T * 9);
  r.arr(nrm, (size_t)T * 9);
  r.arr(uv, (size_t)T * 6);
  r.arr(tan, (size_t)T * 9);
  r.arr(sgn, (size_t)T);
  r.arr(tobj, (size_t)T);
  int32_t n_obj = r.get<int32_t>();
  std::vector<int32_t> omat;
  r.arr(omat, (size_t)n_obj);
  int32_t n_mat = r.get<int32_t>();
  std::vector<er_material_raw> mats;
  r.arr(mats, (size_t)n_mat);
  if (!r.ok) return 5;
  for (const er_material_raw& e : mats) {
    Material m;
    m.albedoTextureID = e.tex[0];
    m.emissionTextureID = e.tex[1];
    m.roughnessTextureID = e.tex[2];
    m.metallicTextureID = e.tex[3];
    m.normalTextureID = e.tex[4];
    m.albedo = v3(e.albedo);
    m.emission = v3(e.emission);
    m.roughness = e.f[0]; m.metallic = e.f[1]; m.clearcoatGloss = e.f[2]; m.clearcoat = e.f[3];
    m.anisotropic = e.f[4]; m.eta = e.f[5]; m.transmission = e.f[6]; m.specular = e.f[7];
    m.specularTint = e.f[8]; m.sheenTint = e.f[9]; m.subsurface = e.f[10]; m.sheen = e.f[11];
    scene.addMaterial(m);
  }
  std::vector<std::vector<Tri>> per_obj((size_t)n_obj);
  for (int64_t i = 0; i < T; i++) {
    if (tobj[(size_t)i] < 0 || tobj[(size_t)i] >= n_obj) return 5;
    Tri t;
    for (int k = 0; k < 3; k++) {
      t.vertices[k] = v3(&pos[(size_t)i * 9 + 3 * k]);
      t.normals[k] = v3(&nrm[(size_t)i * 9 + 3 * k]);
      t.tangents[k] = v3(&tan[(size_t)i * 9 + 3 * k]);
      t.uv[k] = Vector3(uv[(size_t)i * 6 + 2 * k], uv[(size_t)i * 6 + 2 * k + 1], 0);
    }
    t.tangentsSign = sgn[(size_t)i];
    per_obj[(size_t)tobj[(size_t)i]].push_back(t);
  }
  scene.tris.reserve((size_t)T);  // addMeshObject re-points every object into tris
  for (int32_t o = 0; o < n_obj; o++) {
    MeshObject mo;
    mo.tris = per_obj[(size_t)o].data();
    mo.triCount = (unsigned int)per_obj[(size_t)o].size();
    mo.materialID = omat[(size_t)o];
    scene.addMeshObject(mo);
  }
  // textures, environment (HDRI.hpp:42-60: texels, then generateCDF), lights
  int32_t n_tex = r.get<int32_t>();
  for (int32_t i = 0; i < n_tex; i++) {
    Texture t;
    if (!read_texture(r, t)) return 6;
    scene.addTexture(t);
  }
  HDRI h;
  if (!read_texture(r, h.texture)) return 6;
  h.cdf = new float[(size_t)h.texture.width * h.texture.height + 1];
  h.generateCDF();
  scene.hdri = h;
  int32_t n_light = r.get<int32_t>();
  for (int32_t i = 0; i < n_light; i++) {
    float l[6];
    for (float& x : l) x = r.get<float>();
    scene.addPointLight(PointLight(v3(l), v3(l + 3)));
  }
  std::fclose(f);
  if (!r.ok) return 5;
  double t1 = now_ms();

  renderSetup(&scene);
  if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return 7;
  double t2 = now_ms();
  // renderCuda returns an uninitialised status (kernel.cu:667 is shadowed
  // by :679): errors are read from the runtime instead
  if (warm > 0) renderCuda(&scene, warm);
  if (cudaDeviceSynchronize() != cudaSuccess) return 8;
  const int n = xres * yres;
  RenderData rd;
  std::vector<float> pass[PASSES_COUNT];
  for (int i = 0; i < PASSES_COUNT; i++) {
    pass[i].assign((size_t)4 * n, 0.0f);
    rd.passes[i] = pass[i].data();
  }
  std::vector<int> pc0(n), pc1(n);
  getBuffers(rd, pc0.data(), n);
  if (cudaDeviceSynchronize() != cudaSuccess) return 9;

  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, kernelStream);
  double w0 = now_ms();
  renderCuda(&scene, spp);
  cudaEventRecord(e1, kernelStream);
  cudaEventSynchronize(e1);
  double w1 = now_ms();
  if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return 8;
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  getBuffers(rd, pc1.data(), n);
  int samples = getSamples();
  if (cudaDeviceSynchronize() != cudaSuccess) return 9;
  long long paths = 0;
  for (int i = 0; i < n; i++) paths += (long long)pc1[(size_t)i] - pc0[(size_t)i];
  if (argc > 4) {
    FILE* o = std::fopen(argv[4], "wb");
    if (!o) return 10;
    std::fwrite(pass[BEAUTY].data(), sizeof(float), pass[BEAUTY].size(), o);
    std::fclose(o);
  }
  std::printf("{\"ms\": %.4f, \"wall_ms\": %.3f, \"spp\": %d, \"warmup_spp\": %d, \"width\": %d, \"height\": %d, "
              "\"samples_first_pixel\": %d, \"path_vertices\": %lld, \"max_bounces\": %d, \"triangles\": %lld, "
              "\"scene_build_ms\": %.1f, \"render_setup_ms\": %.1f}\n",
              ms, w1 - w0, spp, warm, xres, yres, samples, paths, MAXBOUNCES, (long long)T, t1 - t0, t2 - t1);
  return 0;
}
