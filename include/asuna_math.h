/*
 * asuna_math.h — the float transcendental functions of the path tracer.
 *
 * The reference's GLSL leaves sin, cos, acos, atan, exp, log and pow to the driver
 * (GLSL 4.60 only bounds their error), so the reference's own sample streams
 * are defined up to those functions.  This library fixes them with one
 * implementation shared by the CUDA kernels and the CPU oracle, so a path
 * gives the same bits on both.  Methods (all float, no fused multiply-add:
 * compile device code with -fmad=false and host code with -ffp-contract=off):
 *   exp   Cody-Waite reduction x = n ln2 + r, |r| <= ln2/2, degree-7 Taylor
 *         polynomial of e^r, scaled by 2^n.
 *   sin,  reduction by pi/2 with a three-part Cody-Waite constant,
 *   cos   |r| <= pi/4, Taylor polynomials of degree 9 (sin) and 10 (cos).
 *   tan   the same reduction; the quotient of the two polynomials.
 *   atan2 the range reduction and degree-9 odd minimax polynomial of the
 *         Cephes library's atanf (S. L. Moshier, "Methods and Programs for
 *         Mathematical Functions", 1989), with IEEE quadrant handling.
 *   acos  acos(x) = atan2(sqrt((1 - x)(1 + x)), x).
 *   log2  x = m 2^e with m in [sqrt(1/2), sqrt(2)); ln m = 2 atanh(s),
 *         s = (m - 1) / (m + 1), odd series to s^9; times log2(e).
 *   log   the same ln m plus e ln 2 (ln 2 split in two parts).
 *   exp2  t = n + r, |r| <= 1/2: the exp polynomial at r ln 2, times 2^n.
 *   pow   exp2(y log2 x) (x > 0; GLSL leaves x < 0 undefined: NaN here).
 * Errors: sin, cos, exp within 1 ulp; tan within 3 ulp; atan2, acos, log2, log within 3 ulp; exp2
 * within 2 ulp; pow within 2 ulp plus |y log2 x| ulp of the exponent,
 * over the ranges the path tracer uses (tested against double precision).
 */
#ifndef ASUNA_MATH_H
#define ASUNA_MATH_H

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define ASUNA_MATH_FN __host__ __device__ __forceinline__
#else
#define ASUNA_MATH_FN static inline
#endif

#ifdef __cplusplus
extern "C++" {
namespace asuna_math {

ASUNA_MATH_FN float fl_floor(float x) {
#if defined(__CUDA_ARCH__)
  return floorf(x);
#else
  return __builtin_floorf(x);
#endif
}
ASUNA_MATH_FN float fl_sqrt(float x) {
#if defined(__CUDA_ARCH__)
  return __fsqrt_rn(x);
#else
  return __builtin_sqrtf(x);
#endif
}
ASUNA_MATH_FN float bits_to_float(uint32_t u) {
  float f;
  memcpy(&f, &u, 4);
  return f;
}
ASUNA_MATH_FN uint32_t float_to_bits(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
}
ASUNA_MATH_FN float fl_abs(float x) { return bits_to_float(float_to_bits(x) & 0x7fffffffu); }
ASUNA_MATH_FN float fl_copysign(float x, float s) {
  return bits_to_float((float_to_bits(x) & 0x7fffffffu) | (float_to_bits(s) & 0x80000000u));
}
ASUNA_MATH_FN int fl_isnan(float x) { return (float_to_bits(x) & 0x7fffffffu) > 0x7f800000u; }

/* 2^n for integer n in [-252, 254] as an exact float product. */
ASUNA_MATH_FN float pow2i(int n) {
  if (n > 127) return bits_to_float(uint32_t(127 + 127) << 23) * bits_to_float(uint32_t(n - 127 + 127) << 23);
  if (n < -126) return bits_to_float(uint32_t(-126 + 127) << 23) * bits_to_float(uint32_t(n + 126 + 127) << 23);
  return bits_to_float(uint32_t(n + 127) << 23);
}

ASUNA_MATH_FN float expf_(float x) {
  if (fl_isnan(x)) return x;
  if (x > 88.72283935546875f) return bits_to_float(0x7f800000u);
  if (x < -103.97207641601562f) return 0.0f;
  const float kLog2e = 0x1.715476p+0f;
  const float kLn2Hi = 0x1.62ep-1f, kLn2Lo = 0x1.0bfbe8p-15f;
  float n = fl_floor(x * kLog2e + 0.5f);
  float r = (x - n * kLn2Hi) - n * kLn2Lo;
  float p = 1.0f / 5040.0f;
  p = p * r + 1.0f / 720.0f;
  p = p * r + 1.0f / 120.0f;
  p = p * r + 1.0f / 24.0f;
  p = p * r + 1.0f / 6.0f;
  p = p * r + 0.5f;
  p = p * r + 1.0f;
  p = p * r + 1.0f;
  return p * pow2i((int)n);
}

/* x = k pi/2 + r with |r| <= pi/4 (|x| up to ~1e5). */
ASUNA_MATH_FN float reduce_pio2(float x, int* k) {
  const float k2OverPi = 0x1.45f306p-1f;
  const float kPio2Hi = 0x1.92p+0f, kPio2Mid = 0x1.fb4p-12f, kPio2Lo = 0x1.4442d2p-24f;
  float fk = fl_floor(x * k2OverPi + 0.5f);
  *k = (int)fk;
  return ((x - fk * kPio2Hi) - fk * kPio2Mid) - fk * kPio2Lo;
}
ASUNA_MATH_FN float sin_poly(float r) {
  float z = r * r;
  float p = 1.0f / 362880.0f;
  p = p * z - 1.0f / 5040.0f;
  p = p * z + 1.0f / 120.0f;
  p = p * z - 1.0f / 6.0f;
  return r + r * z * p;
}
ASUNA_MATH_FN float cos_poly(float r) {
  float z = r * r;
  float p = -1.0f / 3628800.0f;
  p = p * z + 1.0f / 40320.0f;
  p = p * z - 1.0f / 720.0f;
  p = p * z + 1.0f / 24.0f;
  p = p * z - 0.5f;
  return 1.0f + z * p;
}
ASUNA_MATH_FN float sinf_(float x) {
  if (fl_isnan(x) || fl_abs(x) == bits_to_float(0x7f800000u)) return bits_to_float(0x7fc00000u);
  int k;
  float r = reduce_pio2(x, &k);
  switch (k & 3) {
    case 0: return sin_poly(r);
    case 1: return cos_poly(r);
    case 2: return -sin_poly(r);
    default: return -cos_poly(r);
  }
}
ASUNA_MATH_FN float cosf_(float x) {
  if (fl_isnan(x) || fl_abs(x) == bits_to_float(0x7f800000u)) return bits_to_float(0x7fc00000u);
  int k;
  float r = reduce_pio2(x, &k);
  switch (k & 3) {
    case 0: return cos_poly(r);
    case 1: return -sin_poly(r);
    case 2: return -cos_poly(r);
    default: return sin_poly(r);
  }
}

/* tan = sin / cos of the one reduced argument: sin_poly(r) / cos_poly(r) for
 * an even quadrant, -cos_poly(r) / sin_poly(r) for an odd one. */
ASUNA_MATH_FN float tanf_(float x) {
  if (fl_isnan(x) || fl_abs(x) == bits_to_float(0x7f800000u)) return bits_to_float(0x7fc00000u);
  int k;
  float r = reduce_pio2(x, &k);
  return (k & 1) ? -cos_poly(r) / sin_poly(r) : sin_poly(r) / cos_poly(r);
}

/* atan of t >= 0 (Cephes atanf reduction and polynomial). */
ASUNA_MATH_FN float atan_pos(float t) {
  const float kPio2 = 0x1.921fb6p+0f, kPio4 = 0x1.921fb6p-1f;
  float y0 = 0.0f, u = t;
  if (t > 2.414213562373095f) {
    y0 = kPio2;
    u = -1.0f / t;
  } else if (t > 0.4142135623730950f) {
    y0 = kPio4;
    u = (t - 1.0f) / (t + 1.0f);
  }
  float z = u * u;
  float p = 8.05374449538e-2f;
  p = p * z - 1.38776856032e-1f;
  p = p * z + 1.99777106478e-1f;
  p = p * z - 3.33329491539e-1f;
  return y0 + (u + u * z * p);
}
ASUNA_MATH_FN float atan2f_(float y, float x) {
  const float kPi = 0x1.921fb6p+1f, kPio2 = 0x1.921fb6p+0f;
  if (fl_isnan(x) || fl_isnan(y)) return x + y;
  const int xneg = (float_to_bits(x) >> 31) != 0;
  if (y == 0.0f) return xneg ? fl_copysign(kPi, y) : fl_copysign(0.0f, y);
  if (x == 0.0f) return fl_copysign(kPio2, y);
  float ax = fl_abs(x), ay = fl_abs(y);
  float a = atan_pos(ay / ax);  /* ratio may overflow to inf: atan_pos(inf) = pi/2 */
  if (xneg) a = kPi - a;
  return fl_copysign(a, y);
}
ASUNA_MATH_FN float acosf_(float x) {
  if (fl_isnan(x) || x > 1.0f || x < -1.0f) return bits_to_float(0x7fc00000u);
  return atan2f_(fl_sqrt((1.0f - x) * (1.0f + x)), x);
}

// x = 2^e m, m in [sqrt(1/2), sqrt(2)): returns ln m (x finite, > 0)
ASUNA_MATH_FN float log_reduce(float x, int* eo) {
  int e = 0;
  uint32_t b = float_to_bits(x);
  if ((b >> 23) == 0) {  // subnormal: scale by 2^23 first
    b = float_to_bits(x * 8388608.0f);
    e = -23;
  }
  e += int(b >> 23) - 127;
  float m = bits_to_float((b & 0x007fffffu) | 0x3f800000u);  // [1, 2)
  if (m > 1.41421356f) {
    m = m * 0.5f;
    e += 1;
  }
  const float s = (m - 1.0f) / (m + 1.0f);
  const float s2 = s * s;
  float p = 1.0f / 9.0f;
  p = p * s2 + 1.0f / 7.0f;
  p = p * s2 + 1.0f / 5.0f;
  p = p * s2 + 1.0f / 3.0f;
  p = p * s2 + 1.0f;
  *eo = e;
  return 2.0f * s * p;
}

ASUNA_MATH_FN float log2f_(float x) {
  if (fl_isnan(x) || x < 0.0f) return bits_to_float(0x7fc00000u);
  if (x == 0.0f) return bits_to_float(0xff800000u);
  if (x == bits_to_float(0x7f800000u)) return x;
  int e;
  const float ln = log_reduce(x, &e);
  return float(e) + ln * 0x1.715476p+0f;
}

// natural logarithm: e ln 2 (two-part constant) + ln m
ASUNA_MATH_FN float logf_(float x) {
  if (fl_isnan(x) || x < 0.0f) return bits_to_float(0x7fc00000u);
  if (x == 0.0f) return bits_to_float(0xff800000u);
  if (x == bits_to_float(0x7f800000u)) return x;
  int e;
  const float ln = log_reduce(x, &e);
  const float fe = float(e);
  return fe * 0x1.62e400p-1f + (ln + fe * 0x1.7f7d1cp-20f);
}

ASUNA_MATH_FN float exp2f_(float t) {
  if (fl_isnan(t)) return t;
  if (t >= 128.0f) return bits_to_float(0x7f800000u);
  if (t < -150.0f) return 0.0f;
  const float n = fl_floor(t + 0.5f);
  const float r = (t - n) * 0x1.62e430p-1f;  // (t - n) is exact; times ln 2
  float p = 1.0f / 5040.0f;
  p = p * r + 1.0f / 720.0f;
  p = p * r + 1.0f / 120.0f;
  p = p * r + 1.0f / 24.0f;
  p = p * r + 1.0f / 6.0f;
  p = p * r + 0.5f;
  p = p * r + 1.0f;
  p = p * r + 1.0f;
  return p * pow2i((int)n);
}

ASUNA_MATH_FN float powf_(float x, float y) {
  if (fl_isnan(x) || fl_isnan(y)) return bits_to_float(0x7fc00000u);
  if (y == 0.0f) return 1.0f;
  if (x == 0.0f) return y > 0.0f ? 0.0f : bits_to_float(0x7f800000u);
  if (x < 0.0f) return bits_to_float(0x7fc00000u);
  return exp2f_(y * log2f_(x));
}

}  // namespace asuna_math
}  // extern "C++"
#endif /* __cplusplus */

#endif /* ASUNA_MATH_H */
