// ORACLE - test infrastructure only.  Built by oracle/Makefile (target
// `ref`) only where the reference sources are present, into oracle/_ref/.
//
// Exports, over the reference's OWN __host__ __device__ headers compiled for
// the host, the same batched probe signatures as oracle/orc_probe.c (prefix
// ref_p_ instead of orc_p_) plus the reference BVH build/traversal, so the
// tests can pin the plain-C restatement against the reference bit for bit.
// Only header-level reference code is exercised here; kernel.cu's device-only
// functions cannot be compiled for the host and are covered by the oracle's
// restatement alone.  Texture/HDRI probes live in ref_shim_tex.cpp: Math.hpp's
// limitUV (Math.hpp:38-41) is declared float but returns nothing, which gcc
// compiles into a trap (-O0) or into unreachable code (-O1+), so that unit
// is built at -O0 with -fno-unreachable-traps.
//
// The headers are included in kernel.cu's order (kernel.cu:6-15) so HitData
// is declared before Disney.hpp uses it.
#include "kernel.h"
#include "Camera.hpp"
#include "Material.hpp"
#include "Hit.hpp"
#include "Disney.hpp"
#include "PointLight.hpp"
#include "BVH.hpp"
#include "HDRI.hpp"
#include "Math.hpp"
#include "Definitions.h"

#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/eleven.h"

namespace {

struct RefScene {
  std::vector<Tri> tris;
  BVH* bvh = nullptr;
};

Vector3 g3(const float* p) { return Vector3(p[0], p[1], p[2]); }
void p3(float* o, const Vector3& a) { o[0] = a.x; o[1] = a.y; o[2] = a.z; }

void unpack_tri(const float* q, Tri& t) {
  for (int k = 0; k < 3; k++) {
    t.vertices[k] = g3(q + 3 * k);
    t.uv[k] = g3(q + 9 + 3 * k);
    t.normals[k] = g3(q + 18 + 3 * k);
    t.tangents[k] = g3(q + 27 + 3 * k);
  }
  t.tangentsSign = q[36];
  t.objectID = 0;
}

void unpack_hd(const float* q, HitData& h) {
  static_assert(sizeof(HitData) == 27 * sizeof(float), "HitData layout");
  std::memcpy(&h, q, sizeof(HitData));
}

}  // namespace

extern "C" {

void* ref_scene_new(const er_scene_desc* d) {
  RefScene* s = new RefScene();
  s->tris.resize((size_t)d->tri_count);
  for (int64_t i = 0; i < d->tri_count; i++) {
    Tri& t = s->tris[(size_t)i];
    for (int k = 0; k < 3; k++) {
      t.vertices[k] = g3(d->positions + 9 * i + 3 * k);
      t.normals[k] = d->normals ? g3(d->normals + 9 * i + 3 * k) : Vector3();
      t.tangents[k] = d->tangents ? g3(d->tangents + 9 * i + 3 * k) : Vector3();
      t.uv[k] = d->uvs ? Vector3(d->uvs[6 * i + 2 * k], d->uvs[6 * i + 2 * k + 1], 0) : Vector3();
    }
    t.tangentsSign = d->tangent_sign ? d->tangent_sign[i] : 1.0f;
    // Tri::hit copies objectID into Hit::objectID (Tri.hpp:157): storing the
    // triangle index there turns the reference traversal into a hit-ID query.
    t.objectID = (int)i;
  }
  s->bvh = new BVH();
  s->bvh->triIndices = new int[d->tri_count > 0 ? d->tri_count : 1];
  s->bvh->build(&s->tris);
  s->bvh->tris = s->tris.data();
  return s;
}

void ref_scene_free(void* p) {
  RefScene* s = (RefScene*)p;
  if (!s) return;
  delete[] s->bvh->triIndices;
  delete s->bvh;
  delete s;
}

int64_t ref_bvh_node_count(void* p) { return (int64_t)2 << BVH_DEPTH; }

void ref_bvh_export(void* p, float* boxes, int32_t* meta, int32_t* tri_indices) {
  RefScene* s = (RefScene*)p;
  int64_t nn = (int64_t)2 << BVH_DEPTH;
  for (int64_t i = 0; i < nn; i++) {
    const Node& n = s->bvh->nodes[i];
    if (n.valid) {
      boxes[6 * i + 0] = n.b1.x; boxes[6 * i + 1] = n.b1.y; boxes[6 * i + 2] = n.b1.z;
      boxes[6 * i + 3] = n.b2.x; boxes[6 * i + 4] = n.b2.y; boxes[6 * i + 5] = n.b2.z;
      meta[5 * i + 0] = n.from; meta[5 * i + 1] = n.to; meta[5 * i + 2] = n.idx;
      meta[5 * i + 3] = n.depth; meta[5 * i + 4] = 1;
    } else {
      for (int k = 0; k < 6; k++) boxes[6 * i + k] = 0;
      for (int k = 0; k < 5; k++) meta[5 * i + k] = 0;
    }
  }
  if (!s->tris.empty()) std::memcpy(tri_indices, s->bvh->triIndices, s->tris.size() * sizeof(int32_t));
}

// BVH::transverse (device-only in the reference, host-compiled here).
void ref_trace(void* p, const float* rays, int64_t n, int32_t normalize, int32_t* tri, float* dist) {
  RefScene* s = (RefScene*)p;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; i++) {
    const float* q = rays + 6 * i;
    Ray r;
    if (normalize) {
      r = Ray(g3(q), g3(q + 3));
    } else {
      r.origin = g3(q);
      r.direction = g3(q + 3);
    }
    Hit h = Hit();
    s->bvh->transverse(r, h);
    tri[i] = h.valid ? (int32_t)h.objectID : -1;
    if (dist) dist[i] = h.valid ? (h.position - r.origin).length() : 0.0f;
  }
}

void ref_p_tri_hit(int64_t n, const float* tris, const float* rays, int32_t normalize, float* out) {
  for (int64_t i = 0; i < n; i++) {
    Tri t;
    unpack_tri(tris + 37 * i, t);
    Ray r;
    if (normalize) {
      r = Ray(g3(rays + 6 * i), g3(rays + 6 * i + 3));
    } else {
      r.origin = g3(rays + 6 * i);
      r.direction = g3(rays + 6 * i + 3);
    }
    Hit h;
    float* o = out + 17 * i;
    std::memset(o, 0, 17 * sizeof(float));
    if (t.hit(r, h)) {
      o[0] = 1;
      p3(o + 1, h.position); p3(o + 4, h.normal); p3(o + 7, h.tangent); p3(o + 10, h.bitangent);
      o[13] = h.tu; o[14] = h.tv;
      o[15] = (h.position - r.origin).length();
    }
  }
}

void ref_p_disney(int64_t n, const float* hd, const float* dirs, const float* Ls, const float* rnd, float* out) {
  for (int64_t i = 0; i < n; i++) {
    HitData h;
    unpack_hd(hd + 27 * i, h);
    Ray r;
    r.origin = Vector3();
    r.direction = g3(dirs + 3 * i);
    Vector3 L = g3(Ls + 3 * i);
    float* o = out + 7 * i;
    p3(o, DisneyEval(r, h, L));
    o[3] = DisneyPdf(r, h, L);
    p3(o + 4, DisneySample(r, h, rnd[3 * i], rnd[3 * i + 1], rnd[3 * i + 2]));
  }
}

// Sampling.hpp helpers; out 3 per item for each function in turn:
// uniformSampleSphere(u1,u2), CosineSampleHemisphere(u1,u2),
// ImportanceSampleGGX(rgh=u3,u1,u2), uniformCircleSampling(u1,u2,u3) (x, y, 0)
void ref_p_sampling(int64_t n, const float* u, float* out) {
  for (int64_t i = 0; i < n; i++) {
    const float* q = u + 3 * i;
    float* o = out + 12 * i;
    p3(o, uniformSampleSphere(q[0], q[1]));
    p3(o + 3, CosineSampleHemisphere(q[0], q[1]));
    p3(o + 6, ImportanceSampleGGX(q[2], q[0], q[1]));
    float x, y;
    uniformCircleSampling(q[0], q[1], q[2], x, y);
    o[9] = x; o[10] = y; o[11] = 0;
  }
}

}  // extern "C"
