/* ORACLE SENSITIVITY PROBE - test infrastructure only.
 *
 * Force-included (gcc -include) into a second build of the oracle sources,
 * oracle/liborc_ulp.so.  The oracle's single-precision transcendental calls
 * (sinf, cosf, acosf, atan2f, powf, logf) return their libm result moved by
 * a few units in the last place, chosen by a hash of the argument bits:
 *
 *   level 0  unchanged (the plain oracle),
 *   level 1  half of the calls moved by one ulp,
 *   level 2  every call moved by one or two ulps.
 *
 * Math libraries for GPUs implement these functions with error bounds of a
 * few ulps, so comparing the plain oracle with liborc_ulp.so measures how far
 * the per-path results of a scene move under rounding differences of that
 * size alone (tests/test_oracle_sensitivity.py).  Nothing else changes.
 */
#ifndef ORC_ULP_H
#define ORC_ULP_H
#include <math.h>
#include <stdint.h>
#include <string.h>

__attribute__((weak)) int orc_ulp_level = 0;

__attribute__((weak, visibility("default"))) void orc_ulp_set_level(int level) { orc_ulp_level = level; }

static inline uint32_t orc_ulp_bits(float x) {
  uint32_t u;
  memcpy(&u, &x, 4);
  return u;
}

static inline float orc_ulp_nudge(float r, uint32_t h) {
  if (orc_ulp_level <= 0) return r;
  h ^= h >> 16;  /* integer hash (xorshift-multiply) */
  h *= 0x7feb352dU;
  h ^= h >> 15;
  h *= 0x846ca68bU;
  h ^= h >> 16;
  const float dir = (h & 2u) ? INFINITY : -INFINITY;
  if (orc_ulp_level == 1) return (h & 1u) ? r : nextafterf(r, dir);
  r = nextafterf(r, dir);
  return (h & 1u) ? nextafterf(r, dir) : r;
}

static inline float orc_ulp_sinf(float x) { return orc_ulp_nudge(sinf(x), orc_ulp_bits(x) * 3u + 1u); }
static inline float orc_ulp_cosf(float x) { return orc_ulp_nudge(cosf(x), orc_ulp_bits(x) * 5u + 2u); }
static inline float orc_ulp_acosf(float x) { return orc_ulp_nudge(acosf(x), orc_ulp_bits(x) * 7u + 3u); }
static inline float orc_ulp_atan2f(float y, float x) {
  return orc_ulp_nudge(atan2f(y, x), orc_ulp_bits(y) * 9u + orc_ulp_bits(x));
}
static inline float orc_ulp_powf(float x, float y) {
  return orc_ulp_nudge(powf(x, y), orc_ulp_bits(x) * 11u + orc_ulp_bits(y));
}
static inline float orc_ulp_logf(float x) { return orc_ulp_nudge(logf(x), orc_ulp_bits(x) * 13u + 4u); }

#define sinf orc_ulp_sinf
#define cosf orc_ulp_cosf
#define acosf orc_ulp_acosf
#define atan2f orc_ulp_atan2f
#define powf orc_ulp_powf
#define logf orc_ulp_logf
#endif
