/*
 * sl_detmath.h -- deterministic fp32 natural log and exp, bit-identical on the host CPU and on the GPU.
 *
 * Why this exists: the splat pipeline's parity contract asks for bit-exact sort keys, per-tile ranges and per-pixel
 * contributor counts.  Those three depend on a transcendental function:
 *   - the 16-bit log-depth key  t = ln(depth / near) / ln(far / near)        (shaders/project.wgsl:366-367)
 *   - the cutoff radius         r = sqrt(2 ln(tau0 / tau_min))                (shaders/project.wgsl:290-295)
 *   - the fragment keep test    alpha >= 1/255, evaluated in its closed form q <= 2 ln(tau0 / tau_min)
 *                               (the bound project.wgsl:290-295 derives for the quad; splat.wgsl:68-73)
 * libm's logf/expf and CUDA's logf/expf round differently in the last place, so a CPU restatement and a GPU kernel
 * that call them disagree on a few keys and boundary fragments.  Both sides therefore evaluate these functions with
 * the code below, which uses only IEEE-754 operations that are correctly rounded on every target (add, sub, mul,
 * div, exact power-of-two scaling, floor): the same inputs give the same bits everywhere.
 *
 * Rules for callers (both are part of the contract):
 *   - host code that includes this header is compiled with -ffp-contract=off (gcc contracts a*b+c into fma on
 *     aarch64 otherwise);
 *   - device code that includes it is compiled with --fmad=false in the translation unit that needs bit parity.
 * No fma appears below, so the results do not depend on whether the target has a fused multiply-add.
 *
 * Methods (standard, published; the constants are the Taylor coefficients 1/k! and 1/(2k+1) and the two-part split
 * of ln 2, all derived from the mathematics, not copied from any library):
 *   exp: Cody & Waite, "Software Manual for the Elementary Functions" (1980), argument reduction
 *        x = n ln2 + r, |r| <= ln2/2, with ln2 split into a 24-bit-exact high part and a low correction; then
 *        exp(r) by its Taylor series to degree 8 in Horner form and exact scaling by 2^n (two steps below 2^-126, so
 *        gradual underflow is rounded once, by the final multiply).
 *   log: x = m 2^e with m in [sqrt(1/2), sqrt(2)); ln m = 2 atanh(s), s = (m - 1) / (m + 1), by the odd series
 *        2 (s + s^3/3 + ... + s^15/15); ln x = e ln2_hi + (e ln2_lo + ln m).
 *   atan/atan2/asin/acos: argument inversion and two angle halvings, then the odd Taylor series (see sl_atanf).
 * Accuracy: exp/log within 2 ulp of the correctly rounded result over the ranges the pipeline uses, atan family within
 * a few ulp (tested against double precision in the unit tests).  sl_expf is used where only a tolerance applies (blending weights in the CPU
 * restatement), so that restatement also gives the same bits on x86-64 and aarch64 hosts.
 */
#ifndef SL_DETMATH_H
#define SL_DETMATH_H

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define SL_DM_FN static __host__ __device__ __forceinline__
#else
#define SL_DM_FN static inline
#endif

SL_DM_FN float sl_bits_to_float(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}

SL_DM_FN uint32_t sl_float_to_bits(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
#endif
}

SL_DM_FN float sl_floorf(float x) {
#if defined(__CUDA_ARCH__)
  return floorf(x);
#else
  return __builtin_floorf(x);
#endif
}

/* 2^k as a float for -126 <= k <= 127 (exact). */
SL_DM_FN float sl_pow2i(int k) { return sl_bits_to_float((uint32_t)(k + 127) << 23); }

/* exp(x), fp32, deterministic.  Returns 0 below -104 and +inf above 88.8. */
SL_DM_FN float sl_expf(float x) {
  if (x != x) return x;
  if (x < -104.0f) return 0.0f;
  if (x > 88.8f) return sl_bits_to_float(0x7f800000u);
  const float kLog2e = 1.44269504088896341f;
  const float kLn2Hi = 0.693145751953125f;      /* 0x3f317200: ln2 rounded to 16 significant bits */
  const float kLn2Lo = 1.42860682030941723e-06f; /* ln2 - kLn2Hi */
  float fn = sl_floorf(x * kLog2e + 0.5f);
  int n = (int)fn;
  float r = (x - fn * kLn2Hi) - fn * kLn2Lo;
  /* Taylor series of exp(r) to r^8/8!, Horner form (|r| <= 0.347: truncation < 2e-10 relative) */
  float p = 2.48015873015873016e-05f;            /* 1/8! */
  p = p * r + 1.98412698412698413e-04f;          /* 1/7! */
  p = p * r + 1.38888888888888889e-03f;          /* 1/6! */
  p = p * r + 8.33333333333333333e-03f;          /* 1/5! */
  p = p * r + 4.16666666666666667e-02f;          /* 1/4! */
  p = p * r + 1.66666666666666667e-01f;          /* 1/3! */
  p = p * r + 0.5f;                              /* 1/2! */
  p = p * r + 1.0f;
  p = p * r + 1.0f;
  if (n > 127) return p * sl_pow2i(127) * sl_pow2i(n - 127);
  if (n < -126) return (p * sl_pow2i(n + 64)) * sl_pow2i(-64);
  return p * sl_pow2i(n);
}

/* natural log, fp32, deterministic.  x <= 0 gives -inf (x == 0) or NaN; +inf gives +inf; subnormals are scaled. */
SL_DM_FN float sl_logf(float x) {
  if (x != x) return x;
  if (x <= 0.0f) return x == 0.0f ? sl_bits_to_float(0xff800000u) : sl_bits_to_float(0x7fc00000u);
  uint32_t u = sl_float_to_bits(x);
  if (u >= 0x7f800000u) return x;
  int e = 0;
  if (u < 0x00800000u) { /* subnormal: scale by 2^24 (exact) */
    x = x * 16777216.0f;
    u = sl_float_to_bits(x);
    e = -24;
  }
  e += (int)(u >> 23) - 127;
  float m = sl_bits_to_float((u & 0x007fffffu) | 0x3f800000u); /* [1, 2) */
  if (m > 1.41421356237309505f) { m = m * 0.5f; e += 1; }     /* [sqrt(1/2), sqrt(2)] */
  float f = m - 1.0f;
  float s = f / (m + 1.0f);
  float z = s * s;
  /* atanh series: s + s^3/3 + ... ; |s| <= 0.1716, z <= 0.02944, truncation at s^17/17 < 1e-14 */
  float q = 6.66666666666666667e-02f;            /* 1/15 */
  q = q * z + 7.69230769230769231e-02f;          /* 1/13 */
  q = q * z + 9.09090909090909091e-02f;          /* 1/11 */
  q = q * z + 1.11111111111111111e-01f;          /* 1/9 */
  q = q * z + 1.42857142857142857e-01f;          /* 1/7 */
  q = q * z + 2.0e-01f;                          /* 1/5 */
  q = q * z + 3.33333333333333333e-01f;          /* 1/3 */
  float lnm = 2.0f * s + (2.0f * s) * (z * q);
  const float kLn2Hi = 0.693145751953125f;
  const float kLn2Lo = 1.42860682030941723e-06f;
  float fe = (float)e;
  return fe * kLn2Hi + (fe * kLn2Lo + lnm);
}

/* log2(x) = ln(x) / ln 2 (the lighting's mip-level selection). */
SL_DM_FN float sl_log2f(float x) { return sl_logf(x) * 1.44269504088896341f; }

/* atan(x), fp32, deterministic.  Method: for |x| > 1, atan(x) = sign(x) pi/2 - atan(1/x); then two angle halvings,
 * atan(t) = 2 atan(t / (1 + sqrt(1 + t^2))), bring |t| below tan(pi/16) = 0.199, where the odd Taylor series of atan
 * to t^15 is accurate to 1e-13; the result is 4 atan(t') (+ the pi/2 offset). */
SL_DM_FN float sl_atanf(float x) {
  if (x != x) return x;
  const float kHalfPi = 1.57079632679489662f;
  float ax = x < 0.0f ? -x : x;
  int inv = ax > 1.0f;
  float t = inv ? 1.0f / ax : ax;
  t = t / (1.0f + sqrtf(1.0f + t * t));
  t = t / (1.0f + sqrtf(1.0f + t * t));
  float z = t * t;
  float p = -6.66666666666666667e-02f;           /* -1/15 */
  p = p * z + 7.69230769230769231e-02f;          /* 1/13 */
  p = p * z - 9.09090909090909091e-02f;          /* -1/11 */
  p = p * z + 1.11111111111111111e-01f;          /* 1/9 */
  p = p * z - 1.42857142857142857e-01f;          /* -1/7 */
  p = p * z + 2.0e-01f;                          /* 1/5 */
  p = p * z - 3.33333333333333333e-01f;          /* -1/3 */
  float a = 4.0f * (t + t * (z * p));
  if (inv) a = kHalfPi - a;
  return x < 0.0f ? -a : a;
}

/* atan2(y, x) with the usual quadrant conventions (atan2(0, 0) = 0). */
SL_DM_FN float sl_atan2f(float y, float x) {
  const float kPi = 3.14159265358979324f;
  const float kHalfPi = 1.57079632679489662f;
  if (x != x || y != y) return x + y;
  if (x == 0.0f) {
    if (y > 0.0f) return kHalfPi;
    if (y < 0.0f) return -kHalfPi;
    return 0.0f;
  }
  float a = sl_atanf(y / x);
  if (x > 0.0f) return a;
  return y >= 0.0f ? a + kPi : a - kPi;
}

/* asin(x) = atan2(x, sqrt((1 - x)(1 + x))), acos(x) = atan2(sqrt((1 - x)(1 + x)), x), for x in [-1, 1]. */
SL_DM_FN float sl_asinf(float x) { return sl_atan2f(x, sqrtf((1.0f - x) * (1.0f + x))); }
SL_DM_FN float sl_acosf(float x) { return sl_atan2f(sqrtf((1.0f - x) * (1.0f + x)), x); }

#endif /* SL_DETMATH_H */
