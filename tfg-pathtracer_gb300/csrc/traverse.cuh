// BVH4 traversal shared by the trace and er_trace_closest kernels.
//
// Reference semantics being reproduced (BVH.hpp:120-175, Tri.hpp:38-92):
// every triangle whose Moller-Trumbore test passes is a candidate, and the
// winner is the one with the smallest |hit position - origin|, where the hit
// position is the smooth-shading position when the surface is locally convex
// (not t).  The reference visits every leaf its (unpruned) slab test accepts;
// ties go to the first found.  Here boxes are tested conservatively and
// pruned with  t_near - delta > limit, delta being a per-child bound on
// |shading position - geometric hit|, so the same candidate set is ranked;
// exact ties go to the lowest tie key (the reference's visiting order when
// the caller supplies it, else the triangle index).
//
// Execution model: persistent warps, one ray per lane, lanes refilled from
// the queue when they finish (dynamic fetch), and "while-while" scheduling:
// a lane that reaches a leaf postpones it and keeps expanding nodes; the
// warp intersects leaves once every lane has one (or has no node left) or
// once several lanes wait with a leaf, so triangle tests run with many
// lanes active and node rounds do not idle on lanes that only wait.
#pragma once

#include "common.cuh"
#include "internal.h"

namespace er {

enum TraceMode { kClosest = 0, kAny = 1, kPoint = 2 };

#ifndef ER_TRAV_BLOCK
#define ER_TRAV_BLOCK 128
#endif
constexpr int kTravBlock = ER_TRAV_BLOCK;  // threads per traversal block
#ifndef ER_TRAV_MIN_BLOCKS
#define ER_TRAV_MIN_BLOCKS 7
#endif
constexpr int kTravMinBlocks = ER_TRAV_MIN_BLOCKS;  // blocks of 128 per SM the register budget allows
#ifndef ER_SMEM_STACK
#define ER_SMEM_STACK 16
#endif
constexpr int kSmemStack = ER_SMEM_STACK;   // stack entries per lane in shared memory
constexpr int kLocalStack = 96 - kSmemStack;  // the rest in local memory
constexpr int kMaxStack = kSmemStack + kLocalStack;
#ifndef ER_Q8_FOLD
#define ER_Q8_FOLD 1  // 8-bit nodes: plane decode folded into the slab fma
#endif

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

// Byte c of w as a float, exactly: the byte is placed in the low mantissa
// bits of 2^23 (byte permute) and 2^23 subtracted, two full-rate
// operations instead of a shift, a mask and an integer conversion.
__device__ __forceinline__ float byte_of(uint32_t w, int c) {
  return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7440u + (uint32_t)c)) - 8388608.0f;
}
// Byte c of w placed in mantissa bits 8..15 of 2^23: the float 2^23 + 256 q,
// exactly, from one byte permute.  Times a slab factor pre-scaled by 2^-8 it
// is 2^15 A + q A; the constant 2^15 A goes into the node's bias once, so a
// plane costs the permute and one fma.
__device__ __forceinline__ float byte_hi(uint32_t w, int c) {
  return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7404u + ((uint32_t)c << 4)));
}
// Decoded Q8 plane origin + q * scale: q * scale is exact (q <= 255, the
// scale a power of two), so the fused form rounds like the sum.
__device__ __forceinline__ float q8_plane(float org, uint32_t w, int c, float scale) {
  return fmaf(byte_of(w, c), scale, org);
}

// Three-input min / max (PTX ISA 8.8, sm_100+); a NaN input is ignored.
__device__ __forceinline__ float max3f(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

// MODE kClosest: closest hit by reference distance.  kAny: any triangle hit
// (env shadow rays, kernel.cu:247-248).  kPoint: point-light shadow ray:
// occluded when the closest hit (by distance from the shadow origin o) lies
// closer than pdist to the shading point pp (kernel.cu:192-197).  Only hits
// whose reference distance is below Tp = pdist + |o - pp| can occlude, and
// when one exists the closest hit is among them, so the search is pruned at
// Tp and stops at the first hit that already proves occlusion.
//
// Stack entries are (node or leaf reference, lower bound of the reference
// distance of anything below it); leaves and internal nodes share the stack.
template <int MODE, bool Q8, bool STATS>
struct Traverser {
  f3 o, d, inv, pp;
  // Slab planes are evaluated as fma(plane, inv, bias): the near-plane bias
  // is lowered and the far-plane bias raised by a bound on the rounding
  // error, so a box the exact ray touches is never culled.
  f3 bnear, bfar;
  uint32_t sgn;  // bit a set: direction component a is negative
  float slack, poff, pdist, tp;
  float best;       // reference distance of the current winner
  uint32_t bkey;
  int32_t slot;     // leaf slot of the winner, -1 = none
  float t, u, v;
  f3 pos;
  bool occluded;
  bool done;
  int sp;
  int32_t node;     // next internal node to expand, -1 = none
  int32_t leaf;     // postponed leaf reference, 0 = none
  float leaf_key;
  int32_t guard;

  __device__ __forceinline__ float limit() const {
    return MODE == kPoint ? fminf(best, tp) : best;
  }
  __device__ __forceinline__ bool survives(float key) const {
    return MODE == kAny || key <= limit() * 1.000001f + slack;
  }

  __device__ __forceinline__ void init(const DevScene& S, f3 o_, f3 d_, f3 pp_, float pdist_) {
    init_at(S, o_, d_, pp_, pdist_, 0, S.scene_eps);
  }

  // Starts at node `root` of a merged node array (a batch of scenes), with
  // that scene's coordinate extent `eps`.
  __device__ __forceinline__ void init_at(const DevScene& S, f3 o_, f3 d_, f3 pp_, float pdist_, int32_t root,
                                          float eps) {
    o = o_;
    d = d_;
    pp = pp_;
    pdist = pdist_;
    // A zero direction component gets a huge finite reciprocal (2^100) so
    // that fma(plane, inv, -o*inv) still separates planes on either side of
    // the origin instead of producing inf - inf.
    const float big = 1.26765060e30f;  // 2^100
    inv = mk(d.x != 0.0f ? __frcp_rn(d.x) : copysignf(big, d.x), d.y != 0.0f ? __frcp_rn(d.y) : copysignf(big, d.y),
             d.z != 0.0f ? __frcp_rn(d.z) : copysignf(big, d.z));
    float omax = fmaxf(fmaxf(fabsf(o.x), fabsf(o.y)), fabsf(o.z));
    slack = (omax + eps) * 2.0e-6f;
    // |error| of fma(plane, inv, -o*inv) <= (|o| + |plane|) |inv| 2^-23;
    // node planes lie within +-scene_eps.  Margin: 4x that.  It only widens
    // slabs whose plane lies within ~1e-5 (|o| + scene_eps) of the origin.
    const float k = 4.76837158e-7f;  // 2^-21
    float mx = (fabsf(o.x) + eps) * fabsf(inv.x) * k;
    float my = (fabsf(o.y) + eps) * fabsf(inv.y) * k;
    float mz = (fabsf(o.z) + eps) * fabsf(inv.z) * k;
    f3 oi = mk(-(o.x * inv.x), -(o.y * inv.y), -(o.z * inv.z));
    bnear = mk(oi.x - mx, oi.y - my, oi.z - mz);
    bfar = mk(oi.x + mx, oi.y + my, oi.z + mz);
    sgn = (__float_as_uint(inv.x) >> 31) | ((__float_as_uint(inv.y) >> 31) << 1) |
          ((__float_as_uint(inv.z) >> 31) << 2);
    poff = (MODE == kPoint) ? xlen(xsub(o, pp)) * 1.000001f + slack : 0.0f;
    tp = (MODE == kPoint) ? (pdist + poff) * 1.000001f + slack : INFINITY;
    best = INFINITY;
    bkey = 0xFFFFFFFFu;
    slot = -1;
    t = u = v = 0.0f;
    pos = mk1(0.0f);
    occluded = false;
    done = false;
    sp = 0;
    node = root;
    leaf = 0;
    leaf_key = 0.0f;
    // a ray visits every node at most once; a longer walk means a corrupt tree
    guard = (int32_t)min(S.n_nodes + 1, (int64_t)0x7FFFFFFF);
  }

  __device__ __forceinline__ bool push(int2* sstk, int2* lstk, int32_t ref, float key, uint32_t* err) {
    if (sp >= kMaxStack) {
      atomicOr(err, 1u);
      done = true;
      return false;
    }
    int2 e = make_int2(ref, __float_as_int(key));
    if (sp < kSmemStack) sstk[sp * kTravBlock] = e;
    else lstk[sp - kSmemStack] = e;
    sp++;
    return true;
  }

  __device__ __forceinline__ void finish() {
    done = true;
    if (MODE == kPoint && slot >= 0) occluded = xlen(xsub(pos, pp)) < pdist;  // kernel.cu:194-196
  }

  // Pops entries until an internal node survives the bound (-> node) or the
  // stack is empty.  A surviving leaf is taken as the postponed leaf when
  // the slot is free; with the slot taken it is pushed back and the lane
  // waits for the next leaf round.
  __device__ __forceinline__ void pop_next(int2* sstk, int2* lstk, uint32_t* err) {
    node = -1;
    while (sp > 0) {
      int2 e = (sp - 1) < kSmemStack ? sstk[(sp - 1) * kTravBlock] : lstk[sp - 1 - kSmemStack];
      float key = __int_as_float(e.y);
      if (!survives(key)) {
        sp--;
        continue;
      }
      if (e.x >= 0) {
        sp--;
        node = e.x;
        return;
      }
      if (leaf != 0) return;  // keep it on the stack
      sp--;
      leaf = e.x;
      leaf_key = key;
    }
    if (leaf == 0) finish();
  }

  // Expands `node`: tests its four child boxes, postpones / pushes leaf
  // children, pushes the other internal children and continues with the
  // nearest.
  __device__ __forceinline__ void node_step(const DevScene& S, int2* sstk, int2* lstk, TravStats& st, uint32_t* err) {
    if (--guard < 0 || (uint64_t)node >= (uint64_t)S.n_nodes) {
      atomicOr(err, 4u);
      done = true;
      return;
    }
    // slab distances of the four children: near / far plane per axis
    float tnx[4], tny[4], tnz[4], tfx[4], tfy[4], tfz[4];
    float4 dl;
    int4 ch;
    if (Q8) {
      const uint4* qn = S.qnodes + 4 * (size_t)node;
      uint4 a = __ldg(qn), b = __ldg(qn + 1), c = __ldg(qn + 2), e = __ldg(qn + 3);
      float ox = __uint_as_float(a.x), oy = __uint_as_float(a.y), oz = __uint_as_float(a.z);
      float sx = __uint_as_float((a.w & 0xFFu) << 23), sy = __uint_as_float(((a.w >> 8) & 0xFFu) << 23),
            sz = __uint_as_float(((a.w >> 16) & 0xFFu) << 23);
      uint32_t qnx = (sgn & 1u) ? b.y : b.x, qfx = (sgn & 1u) ? b.x : b.y;
      uint32_t qny = (sgn & 2u) ? b.w : b.z, qfy = (sgn & 2u) ? b.z : b.w;
      uint32_t qnz = (sgn & 4u) ? c.y : c.x, qfz = (sgn & 4u) ? c.x : c.y;
      // The decode folded into the slab: (o + q s) inv + bias =
      // q (s inv) + (o inv + bias), with s inv exact (s a power of two) and
      // one rounding each for o inv + bias and the final fma.  Their error
      // is below 2^-24 |inv| (3 extent + 2 |origin|), inside the bias
      // widening (8x 2^-24 |inv| (extent + |origin|)), which therefore also
      // covers the difference between the exact o + q s and its float the
      // builder checked against the FP32 box.  An s inv that overflows
      // (node extents beyond 2^35) takes the plain decode.
      const float Ax = sx * inv.x, Ay = sy * inv.y, Az = sz * inv.z;
#if ER_Q8_FOLD
      // Folded form: t = fma(2^23 + 256 q, A 2^-8, B - 2^15 A) with the
      // bias B - 2^15 A rounded down for near planes and up for far planes.
      // Its exact value lies on the outer side of q A + B, and rounding is
      // monotone, so every slab distance is at least as far out as the
      // unfolded form's (a widening below one ulp of 2^15 A, 2^-8 of a
      // quantisation step).  A 2^-8 and 2^15 A are exact while 2^-118 <=
      // |A| < 2^112; other nodes take the unfolded form.
      const float amax = max3f(fabsf(Ax), fabsf(Ay), fabsf(Az)), amin = min3f(fabsf(Ax), fabsf(Ay), fabsf(Az));
      if (amax < 0x1p112f && amin >= 0x1p-118f) {
        const float ax = Ax * 0x1p-8f, ay = Ay * 0x1p-8f, az = Az * 0x1p-8f;
        const float cx = Ax * -0x1p15f, cy = Ay * -0x1p15f, cz = Az * -0x1p15f;
        const float Bnx = __fadd_rd(fmaf(ox, inv.x, bnear.x), cx), Bfx = __fadd_ru(fmaf(ox, inv.x, bfar.x), cx);
        const float Bny = __fadd_rd(fmaf(oy, inv.y, bnear.y), cy), Bfy = __fadd_ru(fmaf(oy, inv.y, bfar.y), cy);
        const float Bnz = __fadd_rd(fmaf(oz, inv.z, bnear.z), cz), Bfz = __fadd_ru(fmaf(oz, inv.z, bfar.z), cz);
#pragma unroll
        for (int k = 0; k < 4; k++) {
          tnx[k] = fmaf(byte_hi(qnx, k), ax, Bnx);
          tfx[k] = fmaf(byte_hi(qfx, k), ax, Bfx);
          tny[k] = fmaf(byte_hi(qny, k), ay, Bny);
          tfy[k] = fmaf(byte_hi(qfy, k), ay, Bfy);
          tnz[k] = fmaf(byte_hi(qnz, k), az, Bnz);
          tfz[k] = fmaf(byte_hi(qfz, k), az, Bfz);
        }
      } else
#endif
      if (fabsf(Ax) < INFINITY && fabsf(Ay) < INFINITY && fabsf(Az) < INFINITY) {
        const float Bnx = fmaf(ox, inv.x, bnear.x), Bfx = fmaf(ox, inv.x, bfar.x);
        const float Bny = fmaf(oy, inv.y, bnear.y), Bfy = fmaf(oy, inv.y, bfar.y);
        const float Bnz = fmaf(oz, inv.z, bnear.z), Bfz = fmaf(oz, inv.z, bfar.z);
#pragma unroll
        for (int k = 0; k < 4; k++) {
          tnx[k] = fmaf(byte_of(qnx, k), Ax, Bnx);
          tfx[k] = fmaf(byte_of(qfx, k), Ax, Bfx);
          tny[k] = fmaf(byte_of(qny, k), Ay, Bny);
          tfy[k] = fmaf(byte_of(qfy, k), Ay, Bfy);
          tnz[k] = fmaf(byte_of(qnz, k), Az, Bnz);
          tfz[k] = fmaf(byte_of(qfz, k), Az, Bfz);
        }
      } else {
#pragma unroll
        for (int k = 0; k < 4; k++) {
          tnx[k] = fmaf(q8_plane(ox, qnx, k, sx), inv.x, bnear.x);
          tfx[k] = fmaf(q8_plane(ox, qfx, k, sx), inv.x, bfar.x);
          tny[k] = fmaf(q8_plane(oy, qny, k, sy), inv.y, bnear.y);
          tfy[k] = fmaf(q8_plane(oy, qfy, k, sy), inv.y, bfar.y);
          tnz[k] = fmaf(q8_plane(oz, qnz, k, sz), inv.z, bnear.z);
          tfz[k] = fmaf(q8_plane(oz, qfz, k, sz), inv.z, bfar.z);
        }
      }
      ch = make_int4((int)c.z, (int)c.w, (int)e.x, (int)e.y);
      float dd = __uint_as_float(e.z);
      dl = make_float4(dd, dd, dd, dd);
    } else {
      const float4* nd = S.nodes + 8 * (size_t)node;
      const float4 nx = __ldg(nd + (sgn & 1u)), fx = __ldg(nd + 1 - (sgn & 1u));
      const float4 ny = __ldg(nd + 2 + ((sgn >> 1) & 1u)), fy = __ldg(nd + 3 - ((sgn >> 1) & 1u));
      const float4 nz = __ldg(nd + 4 + ((sgn >> 2) & 1u)), fz = __ldg(nd + 5 - ((sgn >> 2) & 1u));
      float4 c4 = __ldg(nd + 6);
      ch = make_int4(__float_as_int(c4.x), __float_as_int(c4.y), __float_as_int(c4.z), __float_as_int(c4.w));
      dl = __ldg(nd + 7);
      const float nxa[4] = {nx.x, nx.y, nx.z, nx.w}, fxa[4] = {fx.x, fx.y, fx.z, fx.w};
      const float nya[4] = {ny.x, ny.y, ny.z, ny.w}, fya[4] = {fy.x, fy.y, fy.z, fy.w};
      const float nza[4] = {nz.x, nz.y, nz.z, nz.w}, fza[4] = {fz.x, fz.y, fz.z, fz.w};
#pragma unroll
      for (int k = 0; k < 4; k++) {
        tnx[k] = fmaf(nxa[k], inv.x, bnear.x);
        tfx[k] = fmaf(fxa[k], inv.x, bfar.x);
        tny[k] = fmaf(nya[k], inv.y, bnear.y);
        tfy[k] = fmaf(fya[k], inv.y, bfar.y);
        tnz[k] = fmaf(nza[k], inv.z, bnear.z);
        tfz[k] = fmaf(fza[k], inv.z, bfar.z);
      }
    }
    if (STATS) { st.nodes++; st.boxes += 4; }
    const float dla[4] = {dl.x, dl.y, dl.z, dl.w};
    const int32_t cha[4] = {ch.x, ch.y, ch.z, ch.w};
    const float lim = limit() * 1.000001f + slack;
    float ik[4];
    int32_t ic[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
      float tnear = max3f(tnx[c], tny[c], tnz[c]);
      float tfar = min3f(tfx[c], tfy[c], tfz[c]);
      // FP32 nodes reject empty slots by their inverted boxes; a Q8 empty
      // slot decodes to an inverted box too, but the bias widening could
      // reopen it on a tiny node, so it is checked
      bool hit = (!Q8 || cha[c] != kEmpty) && tnear <= tfar && tfar >= -slack;
      float key = MODE == kAny ? tnear : tnear - dla[c];
      if (MODE != kAny) hit = hit && key <= lim;
      bool is_leaf = cha[c] < 0;
      if (hit && is_leaf) {
        if (leaf == 0) {
          leaf = cha[c];
          leaf_key = key;
        } else if (!push(sstk, lstk, cha[c], key, err)) {
          return;
        }
      }
      ik[c] = hit && !is_leaf ? key : INFINITY;
      ic[c] = cha[c];
    }
    // internal children: the nearest is expanded next, the others are
    // pushed in slot order (their keys still prune them at the pop; a full
    // sort cost more than it saved: 2 % slower on the 1080p scene)
    float kmin = ik[0];
    int im = 0;
#pragma unroll
    for (int c = 1; c < 4; c++)
      if (ik[c] < kmin) { kmin = ik[c]; im = c; }
#pragma unroll
    for (int c = 3; c >= 0; c--)
      if (c != im && ik[c] < INFINITY && !push(sstk, lstk, ic[c], ik[c], err)) return;
    if (kmin < INFINITY) {
      node = ic[im];
      return;
    }
    pop_next(sstk, lstk, err);
  }

  // Intersects the triangles of the postponed leaf, then pops on if the lane
  // has no node left.
  __device__ __forceinline__ void leaf_step(const DevScene& S, int2* sstk, int2* lstk, TravStats& st, uint32_t* err) {
    uint32_t lf = (uint32_t)leaf;
    leaf = 0;
    if (survives(leaf_key)) {
      uint32_t first = lf & kLeafFirstMask, cnt = ((lf >> kLeafCountShift) & 0xFu) + 1u;
      for (uint32_t k = 0; k < cnt; k++) {
        uint32_t sl = first + k;
        const float4* tv = S.tri_v + 3 * (size_t)sl;
        float4 a = __ldg(tv), b = __ldg(tv + 1), e = __ldg(tv + 2);
        if (STATS) st.tris++;
        float tt, uu, vv;
        f3 v0 = from4(a), v1 = from4(b), v2 = from4(e);
        if (!mt_hit(v0, v1, v2, o, d, tt, uu, vv)) continue;
        if (MODE == kAny) {
          occluded = true;
          slot = (int32_t)sl;
          done = true;
          return;
        }
        const float4* tnp = S.tri_n + 3 * (size_t)sl;
        f3 p = ref_position(o, d, tt, uu, vv, v0, v1, v2, from4(__ldg(tnp)), from4(__ldg(tnp + 1)),
                            from4(__ldg(tnp + 2)), nullptr);
        float dist = xlen(xsub(p, o));
        uint32_t key = __float_as_uint(b.w);
        if (dist < best || (dist == best && key < bkey)) {
          best = dist; slot = (int32_t)sl; t = tt; u = uu; v = vv; pos = p; bkey = key;
          if (MODE == kPoint && (dist + poff) * 1.000001f < pdist) {
            occluded = true;  // the closest hit is at least this close
            done = true;
            return;
          }
        }
      }
    }
    if (node < 0) pop_next(sstk, lstk, err);
  }
};

#ifndef ER_REFILL_THRESHOLD
#define ER_REFILL_THRESHOLD 20
#endif
// Lanes below this many active rays make the warp refill from the queue.
constexpr int kRefillThreshold = ER_REFILL_THRESHOLD;
#ifndef ER_LEAF_ROUND_STUCK
#define ER_LEAF_ROUND_STUCK 8
#endif
// A leaf round also starts once this many lanes hold a postponed leaf and
// have no node left to expand (they would idle through node rounds).
constexpr int kLeafRoundStuck = ER_LEAF_ROUND_STUCK;

// Persistent, warp-refilling traversal over a queue of n items.  `load(i,
// tr)` initialises lane state for item i, `store(i, tr)` consumes a finished
// traversal.  Items are claimed in warp batches from *counter, which must be
// zero at launch.
template <int MODE, bool Q8, bool STATS, typename Load, typename Store>
__device__ __forceinline__ void persistent_traverse(const DevScene& S, int32_t n, int32_t* counter, int2* sstk,
                                                    TravStats& st, uint32_t* err, Load load, Store store) {
  // An empty queue claims nothing, so its counter stays zero for a later
  // launch of the same phase.
  if (n <= 0) return;
  int2 lstk[kLocalStack];
  Traverser<MODE, Q8, STATS> tr;
  const unsigned lane = threadIdx.x & 31u;
  int32_t item = -1;  // -1: needs an item; >= n: queue exhausted
  bool active = false;
  while (true) {
    bool need = item < 0;
    unsigned m = __ballot_sync(0xFFFFFFFFu, need);
    if (m) {
      int leader = __ffs(m) - 1;
      int32_t base = 0;
      if ((int)lane == leader) base = atomicAdd(counter, __popc(m));
      base = __shfl_sync(0xFFFFFFFFu, base, leader);
      if (need) {
        item = base + __popc(m & ((1u << lane) - 1u));
        if (item >= n) item = n;  // exhausted
        else {
          load(item, tr);
          active = true;
        }
      }
    }
    if (!__any_sync(0xFFFFFFFFu, active)) break;
    while (true) {
      // leaf round once no active lane is left with only node work, or once
      // enough lanes wait with a leaf (measured on the 1.18M-triangle
      // 1080p scene: lanes busy in node rounds 14 -> 18 of 32, 10 % less
      // traversal time than waiting for every lane)
      bool node_only = active && tr.node >= 0 && tr.leaf == 0;
      unsigned stuck = __ballot_sync(0xFFFFFFFFu, active && tr.leaf != 0 && tr.node < 0);
      bool leaf_round = !__any_sync(0xFFFFFFFFu, node_only) || __popc(stuck) >= kLeafRoundStuck;
      if (active) {
        if (leaf_round) {
          if (tr.leaf != 0) tr.leaf_step(S, sstk, lstk, st, err);
        } else if (tr.node >= 0) {
          tr.node_step(S, sstk, lstk, st, err);
        }
        if (tr.done) {
          store(item, tr);
          active = false;
          item = -1;
        }
      }
      unsigned am = __ballot_sync(0xFFFFFFFFu, active);
      unsigned want = __ballot_sync(0xFFFFFFFFu, item < 0);
      if (__popc(am) < kRefillThreshold && want) break;
      if (!am) break;
    }
  }
}

}  // namespace er
