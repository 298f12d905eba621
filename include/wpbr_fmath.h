/*
 * wpbr_fmath.h — portable, bit-reproducible elementary functions.
 *
 * The ray pipeline's transcendental calls (sphere parametrisation, microfacet
 * and light sampling, environment-map lookups) must give the same bits on the
 * GPU and on any host CPU, so that discrete decisions downstream (which
 * primitive a shadow ray hits, which strata a sample lands in) do not flip
 * between implementations. Library functions (CUDA's device math, glibc) make
 * no such promise, so every function here is written from the mathematics:
 *
 *   - argument reduction: Cody–Waite with a three-part split of pi/2
 *     (the first two parts carry 12 significant bits so k*P1, k*P2 are exact
 *     for |k| < 2^11);
 *   - kernels: minimax polynomials fitted for this file with a Remez exchange
 *     (mpmath, 50 digits) on the reduced intervals and rounded to float:
 *       sin  (sin r - r)/r^3        in r^2, r in [0, pi/4], max err 2.8e-11
 *       cos  (cos r - 1 + r^2/2)/r^4 in r^2,                max err 2.3e-12
 *       atan (atan t - t)/t^3        in t^2, t in [0, tan(pi/8)], 5.0e-10
 *       exp  (e^r - 1 - r)/r^2,      r in [-ln2/2, ln2/2]
 *       log  (log((1+s)/(1-s)) - 2s)/s^3 in s^2, |s| <= 3 - 2*sqrt(2)
 *   - double-precision sin/cos: Taylor series to degree 23 on [-pi/4, pi/4].
 *
 * Every function is a fixed sequence of IEEE-754 add/sub/mul/div/sqrt in a
 * fixed order. The results are reproducible only if the compiler does not
 * contract a*b+c into a fused multiply-add: host code that includes this file
 * is built with -ffp-contract=off and device code with nvcc -fmad=false.
 * Accuracy (checked against libm in the test suite): sin/cos/atan2/acos within
 * 2 ulp on their domains of use, exp/log within 2 ulp.
 */
#ifndef WPBR_FMATH_H
#define WPBR_FMATH_H

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define WPBR_HD __host__ __device__ __forceinline__
#else
#define WPBR_HD inline
#endif

namespace wpbr_fm {

WPBR_HD uint32_t f2u(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
#endif
}
WPBR_HD float u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}
WPBR_HD uint64_t d2u(double d) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t u;
  memcpy(&u, &d, 8);
  return u;
#endif
}
WPBR_HD double u2d(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double d;
  memcpy(&d, &u, 8);
  return d;
#endif
}

WPBR_HD bool is_nan(float x) { return x != x; }
WPBR_HD float fabs_(float x) { return u2f(f2u(x) & 0x7fffffffu); }
WPBR_HD float copysign_(float mag, float sgn) {
  return u2f((f2u(mag) & 0x7fffffffu) | (f2u(sgn) & 0x80000000u));
}
WPBR_HD bool signbit_(float x) { return (f2u(x) >> 31) != 0; }
WPBR_HD float inf_() { return u2f(0x7f800000u); }
WPBR_HD float nan_() { return u2f(0x7fc00000u); }

/* Round to nearest integer (ties away from zero); |x| < 2^22 assumed. */
WPBR_HD float rint_away(float x) {
  float a = fabs_(x);
  float r = (float)(int32_t)(a + 0.5f);
  return copysign_(r, x);
}

/* IEEE square root; correctly rounded on both sides (nvcc default
 * -prec-sqrt=true, x86/ARM hardware sqrt). */
WPBR_HD float sqrt_(float x) {
#if defined(__CUDA_ARCH__)
  return __fsqrt_rn(x);
#else
  return __builtin_sqrtf(x);
#endif
}
WPBR_HD double sqrt_d(double x) {
#if defined(__CUDA_ARCH__)
  return __dsqrt_rn(x);
#else
  return __builtin_sqrt(x);
#endif
}

/* ---- sin / cos (float) ------------------------------------------------- */
static constexpr float kTwoOverPi = 0x1.45f306p-1f;
static constexpr float kP1 = 0x1.92p+0f;        /* pi/2 split, 12 bits */
static constexpr float kP2 = 0x1.fb4p-12f;      /* next 12 bits        */
static constexpr float kP3 = 0x1.4442d2p-24f;   /* remainder           */

WPBR_HD float sin_kernel(float r) {
  float x = r * r;
  float p = 0x1.6dbe4ap-19f;
  p = p * x + -0x1.a013a8p-13f;
  p = p * x + 0x1.11110ep-7f;
  p = p * x + -0x1.555556p-3f;
  return r + (r * x) * p;
}
WPBR_HD float cos_kernel(float r) {
  float x = r * r;
  float p = -0x1.252474p-22f;
  p = p * x + 0x1.a015c6p-16f;
  p = p * x + -0x1.6c16cp-10f;
  p = p * x + 0x1.555556p-5f;
  return (1.0f - 0.5f * x) + (x * x) * p;
}

/* Reduce x to r in [-pi/4, pi/4] with x = r + q*pi/2; returns q mod 4. */
WPBR_HD int reduce_pio2(float x, float* r) {
  float a = fabs_(x);
  if (a <= 0x1.921fb6p-1f) { /* |x| <= pi/4 */
    *r = x;
    return 0;
  }
  if (a < 2048.0f) {
    float k = rint_away(x * kTwoOverPi);
    float y = ((x - k * kP1) - k * kP2) - k * kP3;
    *r = y;
    return ((int)k) & 3;
  }
  /* Large arguments: reduce in double (53-bit split of pi/2). */
  double xd = (double)x;
  double kd = (double)(int64_t)(xd * 0x1.45f306dc9c883p-1 + (xd < 0 ? -0.5 : 0.5));
  double yd = ((xd - kd * 0x1.921fb5p+0) - kd * 0x1.110b46p-26) - kd * 0x1.1a62633145c07p-54;
  *r = (float)yd;
  return ((int)(int64_t)kd) & 3;
}

WPBR_HD float sinf_(float x) {
  if (is_nan(x) || fabs_(x) == inf_()) return nan_();
  float r;
  int q = reduce_pio2(x, &r);
  switch (q) {
    case 0: return sin_kernel(r);
    case 1: return cos_kernel(r);
    case 2: return -sin_kernel(r);
    default: return -cos_kernel(r);
  }
}
WPBR_HD float cosf_(float x) {
  if (is_nan(x) || fabs_(x) == inf_()) return nan_();
  float r;
  int q = reduce_pio2(x, &r);
  switch (q) {
    case 0: return cos_kernel(r);
    case 1: return -sin_kernel(r);
    case 2: return -cos_kernel(r);
    default: return sin_kernel(r);
  }
}
WPBR_HD float tanf_(float x) { return sinf_(x) / cosf_(x); }

/* ---- atan / atan2 / acos (float) ---------------------------------------- */
WPBR_HD float atan_kernel(float t) { /* |t| <= tan(pi/8) */
  float x = t * t;
  float p = 0x1.9e89f2p-5f;
  p = p * x + -0x1.617b08p-4f;
  p = p * x + 0x1.c583eap-4f;
  p = p * x + -0x1.248a58p-3f;
  p = p * x + 0x1.99997cp-3f;
  p = p * x + -0x1.555556p-2f;
  return t + (t * x) * p;
}
static constexpr float kPiO2Hi = 0x1.921fb6p+0f, kPiO2Lo = -0x1.777a5cp-25f;
static constexpr float kPiHi = 0x1.921fb6p+1f, kPiLo = -0x1.777a5cp-24f;
static constexpr float kPiO4Hi = 0x1.921fb6p-1f, kPiO4Lo = -0x1.777a5cp-26f;

/* atan of t in [0, 1]. */
WPBR_HD float atan_01(float t) {
  if (t > 0x1.a8279ap-2f) {
    float u = (t - 1.0f) / (t + 1.0f);
    return kPiO4Hi + (atan_kernel(u) + kPiO4Lo);
  }
  return atan_kernel(t);
}

/* atan2 with the C library's conventions for zeros, infinities and NaN. */
WPBR_HD float atan2f_(float y, float x) {
  if (is_nan(x) || is_nan(y)) return nan_();
  float ax = fabs_(x), ay = fabs_(y);
  float a;
  if (ay == 0.0f) {
    a = signbit_(x) ? kPiHi : 0.0f;
    return copysign_(a, y);
  }
  if (ax == 0.0f) return copysign_(kPiO2Hi, y);
  if (ax == inf_() && ay == inf_()) {
    a = signbit_(x) ? 3.0f * kPiO4Hi : kPiO4Hi;
    return copysign_(a, y);
  }
  if (ax == inf_()) return copysign_(signbit_(x) ? kPiHi : 0.0f, y);
  if (ay == inf_()) return copysign_(kPiO2Hi, y);
  if (ay > ax) {
    a = atan_01(ax / ay);
    a = kPiO2Hi - (a - kPiO2Lo);
  } else {
    a = atan_01(ay / ax);
  }
  if (signbit_(x)) a = kPiHi - (a - kPiLo);
  return copysign_(a, y);
}
WPBR_HD float atanf_(float x) { return atan2f_(x, 1.0f); }

/* acos; NaN outside [-1, 1] like the C library. */
WPBR_HD float acosf_(float x) {
  if (!(fabs_(x) <= 1.0f)) return nan_();
  float s = sqrt_((1.0f - x) * (1.0f + x));
  return atan2f_(s, x);
}

/* ---- exp / log (float) --------------------------------------------------- */
WPBR_HD float ldexp_(float x, int e) {
  /* scale by 2^e in two steps to stay in range */
  while (e > 100) { x *= 0x1p100f; e -= 100; }
  while (e < -100) { x *= 0x1p-100f; e += 100; }
  return x * u2f((uint32_t)(127 + e) << 23);
}
WPBR_HD float expf_(float x) {
  if (is_nan(x)) return x;
  if (x > 88.8f) return inf_();
  if (x < -103.9f) return 0.0f;
  float k = rint_away(x * 0x1.715476p+0f);
  float r = (x - k * 0x1.62ep-1f) - k * 0x1.0bfbe8p-15f;
  float p = 0x1.6d753ap-10f;
  p = p * r + 0x1.120b66p-7f;
  p = p * r + 0x1.5554b8p-5f;
  p = p * r + 0x1.5554dcp-3f;
  p = p * r + 0x1p-1f;
  float e = (1.0f + r) + (r * r) * p;
  return ldexp_(e, (int)k);
}
WPBR_HD float logf_(float x) {
  if (is_nan(x) || x < 0.0f) return nan_();
  if (x == 0.0f) return -inf_();
  if (x == inf_()) return x;
  int ex = 0;
  if (x < 0x1p-126f) { x *= 0x1p24f; ex = -24; }
  uint32_t u = f2u(x);
  ex += (int)((u >> 23) & 0xff) - 127;
  float m = u2f((u & 0x007fffffu) | 0x3f800000u); /* [1, 2) */
  if (m > 0x1.6a09e6p+0f) { m *= 0.5f; ex += 1; }   /* [sqrt(1/2), sqrt(2)) */
  float f = m - 1.0f;
  float s = f / (2.0f + f);
  float z = s * s;
  float p = 0x1.ddd848p-3f;
  p = p * z + 0x1.245c0ep-2f;
  p = p * z + 0x1.9999ecp-2f;
  p = p * z + 0x1.555556p-1f;
  float lm = 2.0f * s + (s * z) * p;
  float k = (float)ex;
  return (k * 0x1.62ep-1f + lm) + k * 0x1.0bfbe8p-15f;
}

// log2 through logf_: log(x) / log(2) with the quotient taken in double.
WPBR_HD float log2f_(float x) { return (float)((double)logf_(x) * 1.4426950408889634); }

/* ---- double-precision sin / cos ------------------------------------------ */
WPBR_HD double sin_kernel_d(double r) {
  double x = r * r;
  double p = -0x1.761b41316381ap-75;
  p = p * x + 0x1.71b8ef6dcf572p-66;
  p = p * x + -0x1.2f49b46814157p-57;
  p = p * x + 0x1.952c77030ad4ap-49;
  p = p * x + -0x1.ae7f3e733b81fp-41;
  p = p * x + 0x1.6124613a86d09p-33;
  p = p * x + -0x1.ae64567f544e4p-26;
  p = p * x + 0x1.71de3a556c734p-19;
  p = p * x + -0x1.a01a01a01a01ap-13;
  p = p * x + 0x1.1111111111111p-7;
  p = p * x + -0x1.5555555555555p-3;
  return r + (r * x) * p;
}
WPBR_HD double cos_kernel_d(double r) {
  double x = r * r;
  double p = -0x1.0ce396db7f853p-70;
  p = p * x + 0x1.e542ba4020225p-62;
  p = p * x + -0x1.6827863b97d97p-53;
  p = p * x + 0x1.ae7f3e733b81fp-45;
  p = p * x + -0x1.93974a8c07c9dp-37;
  p = p * x + 0x1.1eed8eff8d898p-29;
  p = p * x + -0x1.27e4fb7789f5cp-22;
  p = p * x + 0x1.a01a01a01a01ap-16;
  p = p * x + -0x1.6c16c16c16c17p-10;
  p = p * x + 0x1.5555555555555p-5;
  return (1.0 - 0.5 * x) + (x * x) * p;
}
WPBR_HD int reduce_pio2_d(double x, double* r) {
  double a = x < 0 ? -x : x;
  if (a <= 0x1.921fb54442d18p-1) { *r = x; return 0; }
  double kd = (double)(int64_t)(x * 0x1.45f306dc9c883p-1 + (x < 0 ? -0.5 : 0.5));
  *r = ((x - kd * 0x1.921fb5p+0) - kd * 0x1.110b46p-26) - kd * 0x1.1a62633145c07p-54;
  return ((int)(int64_t)kd) & 3;
}
/* Valid for |x| < 2^26 (exact k*P1, k*P2); the pipeline only uses |x| < 8. */
WPBR_HD double sin_d(double x) {
  double r;
  int q = reduce_pio2_d(x, &r);
  switch (q) {
    case 0: return sin_kernel_d(r);
    case 1: return cos_kernel_d(r);
    case 2: return -sin_kernel_d(r);
    default: return -cos_kernel_d(r);
  }
}
WPBR_HD double cos_d(double x) {
  double r;
  int q = reduce_pio2_d(x, &r);
  switch (q) {
    case 0: return cos_kernel_d(r);
    case 1: return -sin_kernel_d(r);
    case 2: return -cos_kernel_d(r);
    default: return sin_kernel_d(r);
  }
}

}  // namespace wpbr_fm

#endif  // WPBR_FMATH_H
