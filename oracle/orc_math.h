/*
 * ORACLE - test infrastructure only.  Never linked into the product library;
 * only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use it.
 *
 * Scalar / vector helpers with the exact float semantics of the reference's
 * Vector3 (src/tfg-pathtracer/Vector.hpp:7-236) and Math.hpp helpers
 * (Math.hpp:22-66).  Build with -ffp-contract=off: the reference host code
 * has no fused multiply-adds, and every expression below must round like it.
 */
#ifndef ORC_MATH_H
#define ORC_MATH_H

#include <math.h>
#include <stdint.h>
#include <limits.h>

/* PI of Math.hpp:7 is a float literal. */
#define ORC_PI 3.14159265358979323846f

typedef struct { float x, y, z; } v3;

static inline v3 V3(float x, float y, float z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
static inline v3 V1(float a) { return V3(a, a, a); }
static inline v3 vadd(v3 a, v3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
/* Vector3*float and float*Vector3 (Vector.hpp:96,207,211): component * s */
static inline v3 vscale(v3 a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
/* Vector3*Vector3 (Vector.hpp:178), component-wise */
static inline v3 vmul(v3 a, v3 b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline v3 vdivs(v3 a, float s) { return V3(a.x / s, a.y / s, a.z / s); }
static inline v3 vneg(v3 a) { return vscale(a, -1.0f); }
/* Vector.hpp:203 Vector3 + float */
static inline v3 vadds(v3 a, float s) { return V3(a.x + s, a.y + s, a.z + s); }
/* Vector.hpp:156-158: ((x*x' + y*y') + z*z') */
static inline float vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
/* Vector.hpp:160-162: the middle component is negated explicitly */
static inline v3 vcross(v3 a, v3 b) {
  return V3(a.y * b.z - a.z * b.y, -(a.x * b.z - a.z * b.x), a.x * b.y - a.y * b.x);
}
/* Vector.hpp:92-94 */
static inline float vlen(v3 a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }
/* Vector.hpp:173-176: returns the input unchanged when its length is 0 */
static inline v3 vnormalized(v3 a) {
  if (vlen(a) == 0) return a;
  return vdivs(a, vlen(a));
}
/* Vector.hpp:164-171 (in-place form used by the Ray constructor) */
static inline v3 vnormalize(v3 a) {
  float l = vlen(a);
  if (l == 0) return a;
  a.x /= l; a.y /= l; a.z /= l;
  return a;
}
static inline float vcomp(v3 a, int n) { return n == 1 ? a.y : n == 2 ? a.z : a.x; }
/* reflect, Vector.hpp:218-220 */
static inline v3 vreflect(v3 a, v3 b) { return vsub(a, vscale(b, 2.0f * vdot(a, b))); }

/* Math.hpp:60-66: NaN selects the second operand */
static inline float minf_(float a, float b) { return a < b ? a : b; }
static inline float maxf_(float a, float b) { return a > b ? a : b; }
/* Math.hpp:30-32 */
static inline float clampf_(float a, float b, float c) { return a < b ? b : a > c ? c : a; }
static inline v3 vclamp(v3 v, float b, float c) { return V3(clampf_(v.x, b, c), clampf_(v.y, b, c), clampf_(v.z, b, c)); }
/* Math.hpp:43-50 with FAST_LERP */
static inline float lerpf_(float a, float b, float c) { return a + c * (b - a); }
static inline v3 vlerp(v3 a, v3 b, float c) { return V3(lerpf_(a.x, b.x, c), lerpf_(a.y, b.y, c), lerpf_(a.z, b.z, c)); }
/* Math.hpp:22-24 */
static inline float mapf_(float a, float b, float c, float d, float e) { return d + ((a - b) / (c - b)) * (e - d); }
/* Math.hpp:38-41: NOTE u < 0 moves u further down by one (the reference's
 * expression adds -1 in both cases). */
static inline void limit_uv(float* u, float* v) {
  *u += (float)(-(*u > 1) + -(*u < 0));
  *v += (float)(-(*v > 1) + -(*v < 0));
}

/* float -> int conversions.  The reference relies on the platform for
 * values outside int range and NaN:
 *   - host (x86-64 MSVC / gcc, cvttss2si): the "integer indefinite" INT_MIN;
 *   - device (cvt.rzi.s32.f32): NaN -> 0, saturation at INT_MIN / INT_MAX.
 * Host-side reference code (BVH build) uses f2i_host, device code f2i_dev. */
static inline int32_t f2i_host(float f) {
  if (!(f > -2147483904.0f && f < 2147483648.0f)) return INT_MIN;
  return (int32_t)f;
}
static inline int32_t f2i_dev(float f) {
  if (f != f) return 0;
  if (f >= 2147483648.0f) return INT_MAX;
  if (f <= -2147483904.0f) return INT_MIN;
  return (int32_t)f;
}

#endif
