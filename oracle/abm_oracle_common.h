/* Shared inline helpers of the C oracle (TEST INFRASTRUCTURE ONLY): threefry2x32-20,
 * partitionable jax.random key/bit derivation and the float conversions of
 * jax.random.uniform / normal, restated from their published definitions. */
#ifndef ABM_ORACLE_COMMON_H
#define ABM_ORACLE_COMMON_H

#include <math.h>
#include <stdint.h>
#include <string.h>

/* ---- threefry2x32-20 (Salmon et al., SC'11) ---------------------------------------- */
static inline uint32_t rotl32(uint32_t x, int r) { return (x << r) | (x >> (32 - r)); }

#define RND(r)         \
  x0 += x1;            \
  x1 = rotl32(x1, r);  \
  x1 ^= x0;

static inline void tf(uint32_t k0, uint32_t k1, uint32_t c0, uint32_t c1, uint32_t* o0,
                      uint32_t* o1) {
  const uint32_t ks0 = k0, ks1 = k1, ks2 = k0 ^ k1 ^ 0x1BD11BDAu;
  uint32_t x0 = c0 + ks0, x1 = c1 + ks1;
  RND(13) RND(15) RND(26) RND(6)
  x0 += ks1; x1 += ks2 + 1u;
  RND(17) RND(29) RND(16) RND(24)
  x0 += ks2; x1 += ks0 + 2u;
  RND(13) RND(15) RND(26) RND(6)
  x0 += ks0; x1 += ks1 + 3u;
  RND(17) RND(29) RND(16) RND(24)
  x0 += ks1; x1 += ks2 + 4u;
  RND(13) RND(15) RND(26) RND(6)
  x0 += ks2; x1 += ks0 + 5u;
  *o0 = x0;
  *o1 = x1;
}
#undef RND

typedef struct { uint32_t a, b; } key_t2;

/* partitionable split(key, n)[i] */
static inline key_t2 split_at(key_t2 k, uint64_t i) {
  key_t2 r;
  tf(k.a, k.b, (uint32_t)(i >> 32), (uint32_t)i, &r.a, &r.b);
  return r;
}
/* partitionable bits(key, shape)[i] */
static inline uint32_t bits_at(key_t2 k, uint64_t i) {
  uint32_t y0, y1;
  tf(k.a, k.b, (uint32_t)(i >> 32), (uint32_t)i, &y0, &y1);
  return y0 ^ y1;
}

static inline float as_float(uint32_t u) {
  float f;
  memcpy(&f, &u, 4);
  return f;
}
static inline float unit_float(uint32_t b) { return as_float((b >> 9) | 0x3F800000u) - 1.0f; }

static inline float uniform_from_bits(uint32_t b, float lo, float hi) {
  const float span = hi - lo;
  float v = unit_float(b) * span;
  v = v + lo;
  return v > lo ? v : lo;
}

/* Giles (2011) single-precision erfinv, Horner with fused multiply-add. */
static inline float erfinv_giles(float x) {
  float w = -log1pf(-(x * x));
  float p;
  if (w < 5.0f) {
    w = w - 2.5f;
    p = 2.81022636e-08f;
    p = fmaf(p, w, 3.43273939e-07f);
    p = fmaf(p, w, -3.5233877e-06f);
    p = fmaf(p, w, -4.39150654e-06f);
    p = fmaf(p, w, 0.00021858087f);
    p = fmaf(p, w, -0.00125372503f);
    p = fmaf(p, w, -0.00417768164f);
    p = fmaf(p, w, 0.246640727f);
    p = fmaf(p, w, 1.50140941f);
  } else {
    w = sqrtf(w) - 3.0f;
    p = -0.000200214257f;
    p = fmaf(p, w, 0.000100950558f);
    p = fmaf(p, w, 0.00134934322f);
    p = fmaf(p, w, -0.00367342844f);
    p = fmaf(p, w, 0.00573950773f);
    p = fmaf(p, w, -0.0076224613f);
    p = fmaf(p, w, 0.00943887047f);
    p = fmaf(p, w, 1.00167406f);
    p = fmaf(p, w, 2.83297682f);
  }
  return p * x;
}

static const float kNormalLo = -0.99999994039535522461f;
static const float kSqrt2f = 1.41421353816986083984f;

static inline float normal_from_bits(uint32_t b) {
  return kSqrt2f * erfinv_giles(uniform_from_bits(b, kNormalLo, 1.0f));
}

/* float64 draw from the same bits: erfinv by Newton iteration on erf in double. */
static inline double erfinv_f64(double y) {
  if (y <= -1.0) return -INFINITY;
  if (y >= 1.0) return INFINITY;
  double x = (double)erfinv_giles((float)y);
  for (int it = 0; it < 4; ++it) {
    const double err = erf(x) - y;
    x -= err / (1.1283791670955126 * exp(-x * x));
  }
  return x;
}
static inline double normal_from_bits_f64(uint32_t b) {
  return 1.4142135623730951 * erfinv_f64((double)uniform_from_bits(b, kNormalLo, 1.0f));
}

static inline float mod1f(float v) {
  float r = fmodf(v, 1.0f);
  if (r != 0.0f && r < 0.0f) r = r + 1.0f;
  return r;
}
static inline double mod1d(double v) {
  double r = fmod(v, 1.0);
  if (r != 0.0 && r < 0.0) r = r + 1.0;
  return r;
}

#endif
