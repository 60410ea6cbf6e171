// Device helpers shared by the kernels.
//
// Two flavours of 3-vector arithmetic:
//  - x*, the "exact" ops, use the IEEE round-to-nearest intrinsics, which
//    the compiler never contracts into FMAs.  They reproduce the reference's
//    host arithmetic bit for bit and are used wherever a result decides
//    which triangle is hit: the Ray normalisation (Ray.hpp:14-18), the
//    Moller-Trumbore test and the shading-position ranking distance
//    (Tri.hpp:38-92, BVH.hpp:159-175), and ray spawning (kernel.cu:442).
//  - plain operators for shading, where FMA contraction is allowed.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define ER_PI 3.14159265358979323846f

namespace er {

struct f3 {
  float x, y, z;
};

__device__ __forceinline__ f3 mk(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 mk1(float a) { return f3{a, a, a}; }
__device__ __forceinline__ f3 from4(float4 a) { return f3{a.x, a.y, a.z}; }

// ------------------------------------------------------------ exact ops --
__device__ __forceinline__ f3 xadd(f3 a, f3 b) { return mk(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)); }
__device__ __forceinline__ f3 xsub(f3 a, f3 b) { return mk(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)); }
__device__ __forceinline__ f3 xscale(f3 a, float s) { return mk(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s)); }
__device__ __forceinline__ float xdot(f3 a, f3 b) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
// Vector.hpp:160-162 (middle component negated explicitly)
__device__ __forceinline__ f3 xcross(f3 a, f3 b) {
  return mk(__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)), -__fsub_rn(__fmul_rn(a.x, b.z), __fmul_rn(a.z, b.x)),
            __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}
__device__ __forceinline__ float xlen(f3 a) { return __fsqrt_rn(xdot(a, a)); }
// Ray.hpp:17 via Vector.hpp:164-171 (unchanged when the length is 0)
__device__ __forceinline__ f3 xnormalize(f3 a) {
  float l = xlen(a);
  if (l == 0.0f) return a;
  return mk(__fdiv_rn(a.x, l), __fdiv_rn(a.y, l), __fdiv_rn(a.z, l));
}

// ------------------------------------------------------------ fast ops --
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 operator*(f3 a, f3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ f3 operator*(float s, f3 a) { return mk(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ f3 operator/(f3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ f3 operator-(f3 a) { return mk(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
  return mk(a.y * b.z - a.z * b.y, -(a.x * b.z - a.z * b.x), a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float len(f3 a) { return sqrtf(dot(a, a)); }
// Vector.hpp:173-176
__device__ __forceinline__ f3 normalized(f3 a) {
  float l = len(a);
  if (l == 0.0f) return a;
  return a / l;
}
__device__ __forceinline__ float minf_(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float maxf_(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float clampf_(float a, float b, float c) { return a < b ? b : a > c ? c : a; }
__device__ __forceinline__ float lerpf_(float a, float b, float c) { return a + c * (b - a); }
__device__ __forceinline__ f3 lerp3(f3 a, f3 b, float c) { return mk(lerpf_(a.x, b.x, c), lerpf_(a.y, b.y, c), lerpf_(a.z, b.z, c)); }

// Math.hpp:38-41: a value below 0 moves down by one more (as the reference)
__device__ __forceinline__ void limit_uv(float& u, float& v) {
  u += (float)(-(int)(u > 1.0f) + -(int)(u < 0.0f));
  v += (float)(-(int)(v > 1.0f) + -(int)(v < 0.0f));
}

// ------------------------------------------------------------------ RNG --
// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).
__device__ __forceinline__ uint4 philox(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}
// (0, 1], 24 bits
__device__ __forceinline__ float u01(uint32_t x) { return (float)((x >> 8) + 1u) * (1.0f / 16777216.0f); }

}  // namespace er
