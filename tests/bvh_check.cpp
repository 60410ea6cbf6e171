// Host check of the SAH BVH4 builder (tfg-pathtracer_gb300/csrc/bvh_build.cpp),
// compiled and run by tests/test_bvh_host.py.
//
// Input: a file of float32 triangles (T x 3 vertices x 3).  Builds the
// FP32 tree and its 8-bit form and prints one line of key=value pairs:
// nodes, leaves, depth, slots (leaf slots), missing (triangles in no leaf),
// repeated (triangles in more than one leaf), outside (vertices outside
// their leaf's box), badref (child references out of range or a node
// reached twice), maxleaf (largest leaf), q8_loose (8-bit child boxes that
// do not contain the FP32 box when decoded as the traversal does).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"

namespace er {
er_status fail(er_status s, const std::string&) { return s; }
}  // namespace er

using namespace er;

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  std::fseek(f, 0, SEEK_END);
  const long n = std::ftell(f) / 36;
  std::fseek(f, 0, SEEK_SET);
  std::vector<float> P((size_t)n * 9);
  if (n > 0 && std::fread(P.data(), 36, (size_t)n, f) != (size_t)n) return 2;
  std::fclose(f);
  er_scene_desc d;
  std::memset(&d, 0, sizeof d);
  d.tri_count = n;
  d.positions = P.data();
  BuildResult r;
  if (build_bvh4(&d, 4, &r) != ER_OK) return 3;
  quantize_bvh4(&r);

  std::vector<int> seen((size_t)n, 0), visits((size_t)r.node_count, 0);
  long leaves = 0, outside = 0, badref = 0, maxleaf = 0, q8_loose = 0;
  std::vector<int32_t> stack{0};
  while (!stack.empty()) {
    const int32_t node = stack.back();
    stack.pop_back();
    if (node < 0 || node >= r.node_count || visits[(size_t)node]++) {
      badref++;
      continue;
    }
    const float* nd = &r.nodes[(size_t)node * 32];
    const QNode& q = r.qnodes[(size_t)node];
    for (int s = 0; s < 4; s++) {
      int32_t c;
      std::memcpy(&c, &nd[24 + s], 4);
      if (c == kEmpty) continue;
      // the 8-bit box, decoded as origin + q * 2^e in float, holds the FP32 box
      const float org[3] = {q.ox, q.oy, q.oz};
      const uint8_t* lo[3] = {q.qlx, q.qly, q.qlz};
      const uint8_t* hi[3] = {q.qhx, q.qhy, q.qhz};
      for (int a = 0; a < 3; a++) {
        const float sc = std::ldexp(1.0f, (int)((q.ex >> (8 * a)) & 0xFFu) - 127);
        if (!(org[a] + (float)lo[a][s] * sc <= nd[8 * a + s]) || !(org[a] + (float)hi[a][s] * sc >= nd[8 * a + 4 + s]))
          q8_loose++;
      }
      if (c >= 0) {
        stack.push_back(c);
        continue;
      }
      const uint32_t first = (uint32_t)c & kLeafFirstMask, cnt = (((uint32_t)c >> kLeafCountShift) & 15u) + 1u;
      leaves++;
      maxleaf = std::max<long>(maxleaf, (long)cnt);
      if (first + cnt > r.order.size()) {
        badref++;
        continue;
      }
      for (uint32_t k = 0; k < cnt; k++) {
        const int32_t t = r.order[first + k];
        if (t < 0 || t >= n) {
          badref++;
          continue;
        }
        seen[(size_t)t]++;
        for (int v = 0; v < 3; v++)
          for (int a = 0; a < 3; a++) {
            const float p = P[(size_t)t * 9 + 3 * v + a];
            if (p < nd[8 * a + s] || p > nd[8 * a + 4 + s]) outside++;
          }
      }
    }
  }
  long missing = 0, repeated = 0, unreached = 0;
  for (long t = 0; t < n; t++) {
    missing += seen[(size_t)t] == 0;
    repeated += seen[(size_t)t] > 1;
  }
  for (long i = 0; i < r.node_count; i++) unreached += visits[(size_t)i] == 0;
  std::printf("nodes=%lld leaves=%ld depth=%d slots=%zu missing=%ld repeated=%ld outside=%ld badref=%ld "
              "unreached=%ld maxleaf=%ld q8_loose=%ld\n",
              (long long)r.node_count, leaves, r.depth, r.order.size(), missing, repeated, outside, badref, unreached,
              maxleaf, q8_loose);
  return 0;
}
