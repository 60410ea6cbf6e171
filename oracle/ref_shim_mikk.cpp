// ORACLE - test infrastructure only.  Built by oracle/Makefile (target
// `ref`) only where the reference sources are present, into oracle/_ref/.
//
// The reference's own tangent generation -- the MikkTSpace generator
// (mikktspace.cpp) driven by CalcTangents (mikktspaceCallback.hpp), which
// ObjLoader.hpp:167-168 runs on every loaded object -- compiled for the
// host from the reference tree, behind a flat-array probe.
#include "mikktspaceCallback.hpp"

#include <cstdint>
#include <vector>

extern "C" void ref_p_tangents(int64_t n, const float* pos, const float* nrm, const float* uv, float* tan,
                               float* sign) {
  std::vector<Tri> tris((size_t)n);
  for (int64_t f = 0; f < n; f++) {
    Tri& t = tris[(size_t)f];
    for (int k = 0; k < 3; k++) {
      const float* p = pos + 9 * f + 3 * k;
      const float* q = nrm + 9 * f + 3 * k;
      t.vertices[k] = Vector3(p[0], p[1], p[2]);
      t.normals[k] = Vector3(q[0], q[1], q[2]);
      t.uv[k] = Vector3(uv[6 * f + 2 * k], uv[6 * f + 2 * k + 1], 0);
    }
  }
  MeshObject mo;
  mo.tris = tris.data();
  mo.triCount = (unsigned int)n;
  CalcTangents ct;
  ct.calc(&mo);
  for (int64_t f = 0; f < n; f++) {
    const Tri& t = tris[(size_t)f];
    for (int k = 0; k < 3; k++) {
      tan[9 * f + 3 * k] = t.tangents[k].x;
      tan[9 * f + 3 * k + 1] = t.tangents[k].y;
      tan[9 * f + 3 * k + 2] = t.tangents[k].z;
    }
    sign[f] = t.tangentsSign;
  }
}
