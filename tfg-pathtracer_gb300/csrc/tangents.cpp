// Per-corner tangents for normal mapping, in the manner of MikkTSpace
// (M. S. Mikkelsen, "Simulation of wrinkled surfaces revisited", 2008), which
// the reference runs on every loaded object (ObjLoader.hpp:167-168 through
// mikktspaceCallback.hpp):
//
//  1. corners with bit-identical position, normal and texture coordinate are
//     one vertex;
//  2. each triangle's texture-space tangent is sign(A) * (dv2 e1 - dv1 e2),
//     normalised, with e1, e2 its edges, dv1, dv2 the v deltas of the
//     texture coordinates and A their signed area (A > 0: the triangle keeps
//     its orientation in texture space);
//  3. a corner's contribution is that tangent projected onto the plane of
//     the corner's normal, weighted by the corner angle measured between
//     the two edges projected onto the same plane;
//  4. the corners of one vertex with the same orientation share the
//     normalised sum; the sign is +1 for orientation-preserving triangles,
//     -1 otherwise.
//
// The reference stores one sign per triangle (set_tspace_basic writes
// Tri::tangentsSign for every corner), which is the triangle's orientation.
#include <cmath>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "internal.h"

namespace er {
namespace {

struct V3d {
  double x, y, z;
};
inline V3d sub(V3d a, V3d b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3d add(V3d a, V3d b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3d scl(V3d a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(V3d a, V3d b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double len(V3d a) { return std::sqrt(dot(a, a)); }
inline V3d nrm(V3d a) {
  double l = len(a);
  return l > 0 ? scl(a, 1.0 / l) : a;
}
inline V3d ld(const float* p) { return {p[0], p[1], p[2]}; }
// projection onto the plane with normal n (unit or zero)
inline V3d on_plane(V3d v, V3d n) { return sub(v, scl(n, dot(n, v))); }

struct CornerKey {
  uint32_t w[8];
  bool operator==(const CornerKey& o) const { return std::memcmp(w, o.w, sizeof w) == 0; }
};
struct CornerHash {
  size_t operator()(const CornerKey& k) const {
    uint64_t h = 1469598103934665603ull;
    for (uint32_t v : k.w) h = (h ^ v) * 1099511628211ull;
    return (size_t)h;
  }
};

}  // namespace

void compute_tangents(int64_t n_tris, const float* pos, const float* nrm_in, const float* uv, float* tangents,
                      float* sign) {
  // 1. weld corners
  std::unordered_map<CornerKey, int32_t, CornerHash> ids;
  ids.reserve((size_t)(3 * n_tris));
  std::vector<int32_t> vid((size_t)(3 * n_tris));
  for (int64_t c = 0; c < 3 * n_tris; c++) {
    CornerKey k;
    std::memcpy(&k.w[0], pos + 3 * c, 12);
    std::memcpy(&k.w[3], nrm_in + 3 * c, 12);
    std::memcpy(&k.w[6], uv + 2 * c, 8);
    auto it = ids.emplace(k, (int32_t)ids.size()).first;
    vid[(size_t)c] = it->second;
  }
  // 2.-3. accumulate per (vertex, orientation)
  std::vector<V3d> acc(2 * ids.size(), V3d{0, 0, 0});
  std::vector<uint8_t> orient((size_t)n_tris);
  for (int64_t f = 0; f < n_tris; f++) {
    const float* P = pos + 9 * f;
    const float* T = uv + 6 * f;
    V3d p0 = ld(P), p1 = ld(P + 3), p2 = ld(P + 6);
    double s1x = (double)T[2] - T[0], s1y = (double)T[3] - T[1];
    double s2x = (double)T[4] - T[0], s2y = (double)T[5] - T[1];
    double area = s1x * s2y - s1y * s2x;
    orient[(size_t)f] = area > 0;
    V3d e1 = sub(p1, p0), e2 = sub(p2, p0);
    V3d os = sub(scl(e1, s2y), scl(e2, s1y));
    os = nrm(scl(os, area < 0 ? -1.0 : 1.0));
    if (area == 0) os = V3d{0, 0, 0};
    const V3d pc[3] = {p0, p1, p2};
    for (int i = 0; i < 3; i++) {
      V3d n = nrm(ld(nrm_in + 9 * f + 3 * i));
      V3d t = nrm(on_plane(os, n));
      V3d a = nrm(on_plane(sub(pc[(i + 2) % 3], pc[i]), n));
      V3d b = nrm(on_plane(sub(pc[(i + 1) % 3], pc[i]), n));
      double c = dot(a, b);
      c = c < -1 ? -1 : c > 1 ? 1 : c;
      double ang = std::acos(c);
      size_t g = 2 * (size_t)vid[(size_t)(3 * f + i)] + orient[(size_t)f];
      acc[g] = add(acc[g], scl(t, ang));
    }
  }
  // 4. write
  for (int64_t f = 0; f < n_tris; f++) {
    for (int i = 0; i < 3; i++) {
      size_t g = 2 * (size_t)vid[(size_t)(3 * f + i)] + orient[(size_t)f];
      V3d t = nrm(acc[g]);
      float* o = tangents + 9 * f + 3 * i;
      o[0] = (float)t.x;
      o[1] = (float)t.y;
      o[2] = (float)t.z;
    }
    sign[f] = orient[(size_t)f] ? 1.0f : -1.0f;
  }
}

}  // namespace er

extern "C" er_status er_compute_tangents(int64_t tri_count, const float* positions, const float* normals,
                                         const float* uvs, float* tangents, float* tangent_sign) {
  return er::guarded("er_compute_tangents", [&]() -> er_status {
    if (tri_count < 0 || (tri_count > 0 && (!positions || !normals || !uvs || !tangents || !tangent_sign)))
      return er::fail(ER_ERR_INVALID_ARG, "bad tangent arguments");
    er::compute_tangents(tri_count, positions, normals, uvs, tangents, tangent_sign);
    return ER_OK;
  });
}
