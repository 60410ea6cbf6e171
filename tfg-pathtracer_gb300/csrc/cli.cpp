// eleven <scene_dir> <spp> <out> [--max-depth N] [--seed S] [--bmp] [--fp64]
//
// Headless equivalent of the reference's main (main.cpp:111-194, README.md:11):
// load the scene folder, render <spp> samples per pixel, write the clamped,
// gamma-encoded beauty pass.  Like the reference, the file is PNG whatever its
// name; --bmp writes a real 24-bit BMP.  Prints the reference's progress
// figure, kPaths/s = sum of path vertices / ms (main.cpp:105-106,172), and
// Msamples/s.  MAXBOUNCES defaults to the reference's 5 (Definitions.h:9).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "eleven.h"

static int die(er_status s, const char* what) {
  std::fprintf(stderr, "eleven: %s: %s (%s)\n", what, er_status_string(s), er_last_error());
  return 1;
}

int main(int argc, char** argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: %s <scene_dir> <spp> <out> [--max-depth N] [--seed S] [--bmp] [--fp64]\n", argv[0]);
    return 2;
  }
  int spp = std::atoi(argv[2]);
  int depth = 5;
  unsigned long long seed = 0;
  bool bmp = false, fp64 = false;
  for (int i = 4; i < argc; i++) {
    if (!std::strcmp(argv[i], "--max-depth") && i + 1 < argc) depth = std::atoi(argv[++i]);
    else if (!std::strcmp(argv[i], "--seed") && i + 1 < argc) seed = std::strtoull(argv[++i], nullptr, 10);
    else if (!std::strcmp(argv[i], "--bmp")) bmp = true;
    else if (!std::strcmp(argv[i], "--fp64")) fp64 = true;
    else {
      std::fprintf(stderr, "eleven: unknown option %s\n", argv[i]);
      return 2;
    }
  }
  if (spp <= 0 || depth <= 0 || depth > 64) {
    std::fprintf(stderr, "eleven: spp and --max-depth must be positive (depth <= 64)\n");
    return 2;
  }
  auto t0 = std::chrono::steady_clock::now();
  er_scene* scene = nullptr;
  er_status st = er_scene_load(argv[1], nullptr, &scene);
  if (st != ER_OK) return die(st, "loading the scene");
  er_scene_info info;
  er_scene_info_get(scene, &info);
  er_camera cam;
  er_scene_get_camera(scene, &cam);
  auto t1 = std::chrono::steady_clock::now();
  std::printf("scene %s: %lld triangles, %dx%d, BVH %lld nodes (%.0f ms), load %.0f ms\n", argv[1],
              (long long)info.tri_count, cam.x_res, cam.y_res, (long long)info.node_count, info.bvh_build_ms,
              std::chrono::duration<double, std::milli>(t1 - t0).count());
  const size_t np = (size_t)cam.x_res * cam.y_res;
  std::vector<float> beauty(np * 4);
  std::vector<uint32_t> pathcount(np);
  er_render_opts o{};
  o.spp = spp;
  o.max_depth = depth;
  o.seed = seed;
  o.flags = fp64 ? ER_RENDER_ACCUM_FP64 : 0;
  er_render_stats rs;
  st = er_render(scene, &o, beauty.data(), nullptr, nullptr, nullptr, nullptr, pathcount.data(), &rs);
  if (st != ER_OK) return die(st, "rendering");
  double vertices = 0;
  for (uint32_t p : pathcount) vertices += p;
  std::printf("%d spp, depth %d: %.1f ms, %.2f Msamples/s, kPaths/s %.1f\n", spp, depth, rs.ms,
              (double)rs.samples / rs.ms / 1e3, vertices / rs.ms);
  std::vector<uint8_t> ldr(np * 4);
  if ((st = er_encode_ldr(beauty.data(), cam.x_res, cam.y_res, ldr.data())) != ER_OK) return die(st, "encoding");
  if ((st = er_write_image(argv[3], ldr.data(), cam.x_res, cam.y_res, bmp ? 1 : 0)) != ER_OK)
    return die(st, "writing the image");
  std::printf("saved %s\n", argv[3]);
  er_scene_free(scene);
  return 0;
}
