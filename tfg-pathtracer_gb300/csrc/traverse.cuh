// BVH4 traversal shared by the extension (closest-hit) and shadow kernels.
//
// Reference semantics being reproduced (BVH.hpp:120-175, Tri.hpp:38-92):
// every triangle whose Moller-Trumbore test passes is a candidate, and the
// winner is the one with the smallest |hit position - origin|, where the hit
// position is the smooth-shading position when the surface is locally convex
// (not t).  The reference visits every leaf its (unpruned) slab test accepts;
// ties go to the first found.  Here boxes are tested conservatively and
// pruned with  t_near > best + delta, delta being a per-child bound on
// |shading position - geometric hit|, so the same candidate set is ranked;
// exact ties go to the lowest tie key (the reference's visiting order when
// the caller supplies it, else the triangle index).
#pragma once

#include "common.cuh"
#include "internal.h"

namespace er {

enum TraceMode { kClosest = 0, kAny = 1, kPoint = 2 };

constexpr int kTravBlock = 128;
constexpr int kSmemStack = 16;
constexpr int kLocalStack = 80;
constexpr int kMaxStack = kSmemStack + kLocalStack;

struct TravStats {
  uint32_t nodes, boxes, tris;
};

// Tri.hpp:38-68 bit for bit: the epsilon is (float)0.0000001, 1.0/det is a
// double division rounded to float, which equals the IEEE float reciprocal
// (double rounding is innocuous for division when 53 >= 2*24+2).  NaNs pass
// the range checks exactly as they do in the reference.
__device__ __forceinline__ bool mt_hit(f3 v0, f3 v1, f3 v2, f3 o, f3 d, float& t, float& u, float& v) {
  const float EPS = 1.00000001e-07f;
  f3 e1 = xsub(v1, v0), e2 = xsub(v2, v0);
  f3 p = xcross(d, e2);
  float det = xdot(e1, p);
  if (det > -EPS && det < EPS) return false;
  float inv = __frcp_rn(det);
  f3 tv = xsub(o, v0);
  u = __fmul_rn(xdot(tv, p), inv);
  if (u < 0.0f || u > 1.0f) return false;
  f3 q = xcross(tv, e1);
  v = __fmul_rn(xdot(d, q), inv);
  if (v < 0.0f || __fadd_rn(u, v) > 1.0f) return false;
  t = __fmul_rn(xdot(e2, q), inv);
  if (t < 0.0f) return false;
  return true;
}

// Tri.hpp:72-91: geometric point, interpolated normal, per-vertex plane
// projections, convexity test.  Returns the hit position the reference
// ranks by.
__device__ __forceinline__ f3 ref_position(f3 o, f3 d, float t, float u, float v, f3 v0, f3 v1, f3 v2, f3 n0, f3 n1,
                                           f3 n2, f3* normal_out) {
  f3 geom = xadd(o, xscale(d, t));
  f3 sn = xadd(xadd(n0, xscale(xsub(n1, n0), u)), xscale(xsub(n2, n0), v));
  f3 p0 = xsub(geom, xscale(n0, xdot(xsub(geom, v0), n0)));
  f3 p1 = xsub(geom, xscale(n1, xdot(xsub(geom, v1), n1)));
  f3 p2 = xsub(geom, xscale(n2, xdot(xsub(geom, v2), n2)));
  f3 sp = xadd(xadd(p0, xscale(xsub(p1, p0), u)), xscale(xsub(p2, p0), v));
  bool convex = xdot(xsub(sp, geom), sn) > 0.0f;
  if (normal_out) *normal_out = sn;
  return convex ? sp : geom;
}

struct TravResult {
  int32_t slot;  // leaf slot of the winner, -1 = miss
  float t, u, v, dist;
  f3 pos;
  bool occluded;
};

__device__ __forceinline__ float byte_of(uint32_t w, int c) { return (float)((w >> (8 * c)) & 0xFFu); }

// One traversal.  MODE kClosest: closest hit by reference distance.
// kAny: any triangle hit (env shadow rays, kernel.cu:247-248).  kPoint:
// point-light shadow ray: occluded when the closest hit (by distance from
// the shadow origin o) lies closer than pdist to the shading point pp
// (kernel.cu:192-197); the search stops early once a hit proves it.
template <int MODE, bool Q8, bool STATS>
__device__ __forceinline__ TravResult traverse(const DevScene& S, f3 o, f3 d, f3 pp, float pdist, int2* sstk,
                                               TravStats& st, uint32_t* err) {
  int2 lstk[kLocalStack];
  TravResult R;
  R.slot = -1;
  R.t = R.u = R.v = 0.0f;
  R.dist = INFINITY;
  R.pos = mk1(0.0f);
  R.occluded = false;
  uint32_t bkey = 0xFFFFFFFFu;
  const f3 inv = mk(__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z));
  const float omax = fmaxf(fmaxf(fabsf(o.x), fabsf(o.y)), fabsf(o.z));
  const float slack = (omax + S.scene_eps) * 2.0e-6f;
  // point mode: |o - pp| bounds how far the distances from o and pp differ
  const float poff = (MODE == kPoint) ? xlen(xsub(o, pp)) * 1.000001f + slack : 0.0f;
  int sp = 0;
  int32_t node = 0;
  bool done = false;
  // A ray visits every node at most once; a longer walk means a corrupt
  // tree, reported through the error word instead of spinning.
  int64_t guard = S.n_nodes + 1;
  while (!done) {
    if (--guard < 0 || (uint64_t)node >= (uint64_t)S.n_nodes) {
      atomicOr(err, 4u);
      return R;
    }
    float4 lx, hx, ly, hy, lz, hz, dl;
    int4 ch;
    if (Q8) {
      const uint4* qn = S.qnodes + 4 * (size_t)node;
      uint4 a = __ldg(qn), b = __ldg(qn + 1), c = __ldg(qn + 2), e = __ldg(qn + 3);
      float ox = __uint_as_float(a.x), oy = __uint_as_float(a.y), oz = __uint_as_float(a.z);
      float sx = __uint_as_float((a.w & 0xFFu) << 23), sy = __uint_as_float(((a.w >> 8) & 0xFFu) << 23),
            sz = __uint_as_float(((a.w >> 16) & 0xFFu) << 23);
      lx = make_float4(ox + byte_of(b.x, 0) * sx, ox + byte_of(b.x, 1) * sx, ox + byte_of(b.x, 2) * sx, ox + byte_of(b.x, 3) * sx);
      hx = make_float4(ox + byte_of(b.y, 0) * sx, ox + byte_of(b.y, 1) * sx, ox + byte_of(b.y, 2) * sx, ox + byte_of(b.y, 3) * sx);
      ly = make_float4(oy + byte_of(b.z, 0) * sy, oy + byte_of(b.z, 1) * sy, oy + byte_of(b.z, 2) * sy, oy + byte_of(b.z, 3) * sy);
      hy = make_float4(oy + byte_of(b.w, 0) * sy, oy + byte_of(b.w, 1) * sy, oy + byte_of(b.w, 2) * sy, oy + byte_of(b.w, 3) * sy);
      lz = make_float4(oz + byte_of(c.x, 0) * sz, oz + byte_of(c.x, 1) * sz, oz + byte_of(c.x, 2) * sz, oz + byte_of(c.x, 3) * sz);
      hz = make_float4(oz + byte_of(c.y, 0) * sz, oz + byte_of(c.y, 1) * sz, oz + byte_of(c.y, 2) * sz, oz + byte_of(c.y, 3) * sz);
      ch = make_int4((int)c.z, (int)c.w, (int)e.x, (int)e.y);
      float dd = __uint_as_float(e.z);
      dl = make_float4(dd, dd, dd, dd);
    } else {
      const float4* nd = S.nodes + 8 * (size_t)node;
      lx = __ldg(nd + 0); hx = __ldg(nd + 1); ly = __ldg(nd + 2); hy = __ldg(nd + 3);
      lz = __ldg(nd + 4); hz = __ldg(nd + 5);
      float4 c4 = __ldg(nd + 6);
      ch = make_int4(__float_as_int(c4.x), __float_as_int(c4.y), __float_as_int(c4.z), __float_as_int(c4.w));
      dl = __ldg(nd + 7);
    }
    if (STATS) { st.nodes++; st.boxes += 4; }
    float tn[4];
    int32_t cc[4];
    const float lxa[4] = {lx.x, lx.y, lx.z, lx.w}, hxa[4] = {hx.x, hx.y, hx.z, hx.w};
    const float lya[4] = {ly.x, ly.y, ly.z, ly.w}, hya[4] = {hy.x, hy.y, hy.z, hy.w};
    const float lza[4] = {lz.x, lz.y, lz.z, lz.w}, hza[4] = {hz.x, hz.y, hz.z, hz.w};
    const float dla[4] = {dl.x, dl.y, dl.z, dl.w};
    const int32_t cha[4] = {ch.x, ch.y, ch.z, ch.w};
#pragma unroll
    for (int c = 0; c < 4; c++) {
      float t0x = (lxa[c] - o.x) * inv.x, t1x = (hxa[c] - o.x) * inv.x;
      float t0y = (lya[c] - o.y) * inv.y, t1y = (hya[c] - o.y) * inv.y;
      float t0z = (lza[c] - o.z) * inv.z, t1z = (hza[c] - o.z) * inv.z;
      float tnear = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fminf(t0z, t1z));
      float tfar = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fmaxf(t0z, t1z));
      tfar = tfar + fabsf(tfar) * 1.0e-6f + slack;
      bool hit = cha[c] != kEmpty && tnear <= tfar && tfar >= 0.0f;
      if (MODE != kAny) hit = hit && (tnear - dla[c]) <= R.dist * 1.000001f + slack;
      tn[c] = hit ? tnear - (MODE != kAny ? dla[c] : 0.0f) : INFINITY;
      cc[c] = hit ? cha[c] : kEmpty;
    }
    // leaves first
#pragma unroll
    for (int c = 0; c < 4; c++) {
      if (cc[c] == kEmpty || cc[c] >= 0) continue;
      if (!(tn[c] <= R.dist * 1.000001f + slack)) continue;  // best may have improved
      uint32_t lf = (uint32_t)cc[c];
      uint32_t first = lf & kLeafFirstMask, cnt = ((lf >> kLeafCountShift) & 0xFu) + 1u;
      for (uint32_t k = 0; k < cnt; k++) {
        uint32_t slot = first + k;
        const float4* tv = S.tri_v + 3 * (size_t)slot;
        float4 a = __ldg(tv), b = __ldg(tv + 1), e = __ldg(tv + 2);
        if (STATS) st.tris++;
        float t, u, v;
        f3 v0 = from4(a), v1 = from4(b), v2 = from4(e);
        if (!mt_hit(v0, v1, v2, o, d, t, u, v)) continue;
        if (MODE == kAny) {
          R.occluded = true;
          R.slot = (int32_t)slot;
          return R;
        }
        const float4* tnp = S.tri_n + 3 * (size_t)slot;
        f3 pos = ref_position(o, d, t, u, v, v0, v1, v2, from4(__ldg(tnp)), from4(__ldg(tnp + 1)),
                              from4(__ldg(tnp + 2)), nullptr);
        float dist = xlen(xsub(pos, o));
        uint32_t key = __float_as_uint(b.w);
        if (dist < R.dist || (dist == R.dist && key < bkey)) {
          R.dist = dist; R.slot = (int32_t)slot; R.t = t; R.u = u; R.v = v; R.pos = pos; bkey = key;
          if (MODE == kPoint && (dist + poff) * 1.000001f < pdist) {
            R.occluded = true;
            return R;
          }
        }
      }
      cc[c] = kEmpty;
    }
    // internal children: nearest first
    float k0 = cc[0] >= 0 && cc[0] != kEmpty ? tn[0] : INFINITY;
    float k1 = cc[1] >= 0 && cc[1] != kEmpty ? tn[1] : INFINITY;
    float k2 = cc[2] >= 0 && cc[2] != kEmpty ? tn[2] : INFINITY;
    float k3 = cc[3] >= 0 && cc[3] != kEmpty ? tn[3] : INFINITY;
    int32_t c0 = cc[0], c1 = cc[1], c2 = cc[2], c3 = cc[3];
#define ER_CSWAP(ka, ca, kb, cb)                         \
  if (kb < ka) {                                         \
    float tk = ka; ka = kb; kb = tk;                     \
    int32_t tc = ca; ca = cb; cb = tc;                   \
  }
    ER_CSWAP(k0, c0, k1, c1);
    ER_CSWAP(k2, c2, k3, c3);
    ER_CSWAP(k0, c0, k2, c2);
    ER_CSWAP(k1, c1, k3, c3);
    ER_CSWAP(k1, c1, k2, c2);
#undef ER_CSWAP
    int n = (k0 < INFINITY) + (k1 < INFINITY) + (k2 < INFINITY) + (k3 < INFINITY);
    if (n > 0) {
      // push the farther ones, farthest first
      if (sp + n - 1 > kMaxStack) {
        atomicOr(err, 1u);
        return R;
      }
      if (n > 3) { int2 e = make_int2(c3, __float_as_int(k3)); if (sp < kSmemStack) sstk[sp * kTravBlock] = e; else lstk[sp - kSmemStack] = e; sp++; }
      if (n > 2) { int2 e = make_int2(c2, __float_as_int(k2)); if (sp < kSmemStack) sstk[sp * kTravBlock] = e; else lstk[sp - kSmemStack] = e; sp++; }
      if (n > 1) { int2 e = make_int2(c1, __float_as_int(k1)); if (sp < kSmemStack) sstk[sp * kTravBlock] = e; else lstk[sp - kSmemStack] = e; sp++; }
      node = c0;
      continue;
    }
    // pop until an entry survives the (possibly tightened) bound
    done = true;
    while (sp > 0) {
      sp--;
      int2 e = sp < kSmemStack ? sstk[sp * kTravBlock] : lstk[sp - kSmemStack];
      if (MODE == kAny || __int_as_float(e.y) <= R.dist * 1.000001f + slack) {
        node = e.x;
        done = false;
        break;
      }
    }
  }
  if (MODE == kPoint && R.slot >= 0) {
    // kernel.cu:194-196 on the closest hit: |hit - point| < dist
    R.occluded = xlen(xsub(R.pos, pp)) < pdist;
  }
  return R;
}

}  // namespace er
