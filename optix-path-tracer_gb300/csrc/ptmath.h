/*
 * ptmath.h - single-precision elementary functions that give the SAME bits
 * on the host (gcc, -ffp-contract=off) and on the GPU (nvcc, -fmad=false).
 *
 * Why: the reference path tracer calls sinf/cosf/tanf/atanf/atan2f/acosf/
 * asinf/powf in its sampling and shading code (e.g. programs/sampling.cuh:23,
 * programs/materials/microfacets.cuh:13-19, programs/miss.cu:64-77,
 * programs/hitables/sphere.cu:84-87, host_includes/camera.hpp:23-24).  The
 * CUDA and glibc versions of those functions differ in the last bits, so a
 * CPU transcription could never reproduce a GPU path bit for bit.  Both the
 * CUDA kernels and the CPU oracle therefore call the functions below, which
 * use only +, -, *, /, sqrt, floor and bit manipulation - all of which are
 * correctly rounded IEEE-754 operations on both sides.
 *
 * Methods (all from the open literature, coefficients derived here):
 *  - sin/cos/tan: Cody & Waite (1980) additive range reduction by pi/2 with a
 *    three-part split of pi/2, then the Taylor polynomials of sin and cos on
 *    [-pi/4, pi/4] (coefficients (-1)^k/(2k+1)! and (-1)^k/(2k)!).
 *  - atan/atan2/asin/acos: reduction |x|>1 -> pi/2 - atan(1/x) and
 *    x > tan(pi/8) -> pi/4 + atan((x-1)/(x+1)), then the Gregory series
 *    sum (-1)^k t^(2k+1)/(2k+1) on |t| <= tan(pi/8); asin/acos via atan2.
 *  - log2: exponent/mantissa split with mantissa in [sqrt(1/2), sqrt(2)),
 *    ln(m) = 2 atanh((m-1)/(m+1)) by its odd power series.
 *  - exp2: split into integer and fractional part in [-1/2, 1/2], Taylor
 *    series of e^(f ln2), integer part applied to the exponent field.
 *  - pow(x, y) = exp2(y log2 x) with the usual special cases.
 * Accuracy (checked by tests/test_ptmath.py against double precision): a few
 * ulp for sin/cos/atan family, ~1e-6 relative for pow at |y log2 x| < 30.
 */
#ifndef PT_MATH_H
#define PT_MATH_H

#include <stdint.h>

#if defined(__CUDACC__)
#define PTM_FN __host__ __device__ __forceinline__
#else
#define PTM_FN static inline
#include <string.h>
#endif

PTM_FN uint32_t ptm_f2u(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
#endif
}

PTM_FN float ptm_u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}

PTM_FN float ptm_floor(float x) {
#if defined(__CUDA_ARCH__)
  return floorf(x);
#else
  return __builtin_floorf(x);
#endif
}

PTM_FN float ptm_sqrt(float x) {
#if defined(__CUDA_ARCH__)
  return __fsqrt_rn(x);
#else
  return __builtin_sqrtf(x);
#endif
}

PTM_FN float ptm_fabs(float x) { return ptm_u2f(ptm_f2u(x) & 0x7fffffffu); }
PTM_FN int ptm_isnan(float x) { return (ptm_f2u(x) & 0x7fffffffu) > 0x7f800000u; }

#define PTM_PI 3.14159274101257324f       /* float(pi) */
#define PTM_PI_2 1.57079637050628662f     /* float(pi/2) */
#define PTM_PI_4 0.785398185253143311f    /* float(pi/4) */
#define PTM_2_PI 0.636619746685028076f    /* float(2/pi) */
#define PTM_TAN_PI_8 0.414213567972183228f
#define PTM_SQRT2 1.41421353816986084f
#define PTM_LOG2E 1.44269502162933350f
#define PTM_LN2 0.693147182464599609f

/* Cody-Waite reduction x = k*(pi/2) + r.  C1 and C2 have 12 significant bits
 * so k*C1 and k*C2 are exact for |k| < 2048 (|x| < ~3200). */
PTM_FN float ptm_reduce_pio2(float x, int *quadrant) {
  const float C1 = 1.5703125f;
  const float C2 = 4.837512969970703125e-4f;
  const float C3 = 7.549790126404332e-08f;
  float k = ptm_floor(x * PTM_2_PI + 0.5f);
  float r = x - k * C1;
  r = r - k * C2;
  r = r - k * C3;
  *quadrant = (int)k;
  return r;
}

/* Taylor polynomials on |r| <= ~pi/4 (Horner in r^2). */
PTM_FN float ptm_sin_poly(float r) {
  float z = r * r;
  float p = 2.75573192e-6f;          /*  1/9!  */
  p = p * z + -1.98412698e-4f;       /* -1/7!  */
  p = p * z + 8.33333333e-3f;        /*  1/5!  */
  p = p * z + -1.66666667e-1f;       /* -1/3!  */
  return r + r * (z * p);
}

PTM_FN float ptm_cos_poly(float r) {
  float z = r * r;
  float p = -2.75573192e-7f;         /* -1/10! */
  p = p * z + 2.48015873e-5f;        /*  1/8!  */
  p = p * z + -1.38888889e-3f;       /* -1/6!  */
  p = p * z + 4.16666667e-2f;        /*  1/4!  */
  p = p * z + -0.5f;                 /* -1/2!  */
  return 1.0f + z * p;
}

PTM_FN float pt_sinf(float x) {
  int q;
  float r = ptm_reduce_pio2(x, &q);
  float s = ptm_sin_poly(r), c = ptm_cos_poly(r);
  switch (q & 3) {
    case 0: return s;
    case 1: return c;
    case 2: return -s;
    default: return -c;
  }
}

PTM_FN float pt_cosf(float x) {
  int q;
  float r = ptm_reduce_pio2(x, &q);
  float s = ptm_sin_poly(r), c = ptm_cos_poly(r);
  switch (q & 3) {
    case 0: return c;
    case 1: return -s;
    case 2: return -c;
    default: return s;
  }
}

PTM_FN void pt_sincosf(float x, float *sn, float *cs) {
  int q;
  float r = ptm_reduce_pio2(x, &q);
  float s = ptm_sin_poly(r), c = ptm_cos_poly(r);
  switch (q & 3) {
    case 0: *sn = s; *cs = c; break;
    case 1: *sn = c; *cs = -s; break;
    case 2: *sn = -s; *cs = -c; break;
    default: *sn = -c; *cs = s; break;
  }
}

PTM_FN float pt_tanf(float x) {
  float s, c;
  pt_sincosf(x, &s, &c);
  return s / c;
}

/* atan on [0, 1]: one more reduction to |t| <= tan(pi/8), Gregory series. */
PTM_FN float ptm_atan01(float a) {
  float base = 0.0f, t = a;
  if (a > PTM_TAN_PI_8) {
    t = (a - 1.0f) / (a + 1.0f);
    base = PTM_PI_4;
  }
  float z = t * t;
  float p = 1.0f / 17.0f;
  p = p * z - 1.0f / 15.0f;
  p = p * z + 1.0f / 13.0f;
  p = p * z - 1.0f / 11.0f;
  p = p * z + 1.0f / 9.0f;
  p = p * z - 1.0f / 7.0f;
  p = p * z + 1.0f / 5.0f;
  p = p * z - 1.0f / 3.0f;
  return base + (t + t * (z * p));
}

PTM_FN float pt_atanf(float x) {
  if (ptm_isnan(x)) return x;
  float a = ptm_fabs(x), r;
  if (a > 1.0f)
    r = PTM_PI_2 - ptm_atan01(1.0f / a);
  else
    r = ptm_atan01(a);
  return x < 0.0f ? -r : r;
}

PTM_FN float pt_atan2f(float y, float x) {
  if (ptm_isnan(x) || ptm_isnan(y)) return x + y;
  float ax = ptm_fabs(x), ay = ptm_fabs(y), r;
  if (ax == 0.0f && ay == 0.0f) {
    r = 0.0f;
  } else if (ay <= ax) {
    r = ptm_atan01(ay / ax);
  } else {
    r = PTM_PI_2 - ptm_atan01(ax / ay);
  }
  if (ptm_f2u(x) >> 31) r = PTM_PI - r;   /* x < 0 (or -0) */
  return (ptm_f2u(y) >> 31) ? -r : r;
}

PTM_FN float pt_asinf(float x) {
  return pt_atan2f(x, ptm_sqrt((1.0f - x) * (1.0f + x)));
}

PTM_FN float pt_acosf(float x) {
  return pt_atan2f(ptm_sqrt((1.0f - x) * (1.0f + x)), x);
}

/* log2 for finite x > 0 (callers handle the special cases). */
PTM_FN float ptm_log2_pos(float x) {
  uint32_t u = ptm_f2u(x);
  int e = 0;
  if (u < 0x00800000u) { /* subnormal: scale by 2^23 */
    x = x * 8388608.0f;
    u = ptm_f2u(x);
    e = -23;
  }
  e += (int)((u >> 23) & 0xffu) - 127;
  float m = ptm_u2f((u & 0x007fffffu) | 0x3f800000u); /* [1, 2) */
  if (m > PTM_SQRT2) {
    m = m * 0.5f;
    e += 1;
  }
  float s = (m - 1.0f) / (m + 1.0f);
  float z = s * s;
  float p = 1.0f / 13.0f;
  p = p * z + 1.0f / 11.0f;
  p = p * z + 1.0f / 9.0f;
  p = p * z + 1.0f / 7.0f;
  p = p * z + 1.0f / 5.0f;
  p = p * z + 1.0f / 3.0f;
  float ln_m = 2.0f * (s + s * (z * p));
  return (float)e + ln_m * PTM_LOG2E;
}

PTM_FN float pt_exp2f(float y) {
  if (ptm_isnan(y)) return y;
  if (y > 128.0f) return ptm_u2f(0x7f800000u);
  if (y < -151.0f) return 0.0f;
  float k = ptm_floor(y + 0.5f);
  float f = y - k;                  /* [-0.5, 0.5], exact */
  float g = f * PTM_LN2;
  float p = 1.0f / 40320.0f;        /* e^g by Taylor to g^8 */
  p = p * g + 1.0f / 5040.0f;
  p = p * g + 1.0f / 720.0f;
  p = p * g + 1.0f / 120.0f;
  p = p * g + 1.0f / 24.0f;
  p = p * g + 1.0f / 6.0f;
  p = p * g + 0.5f;
  p = p * g + 1.0f;
  p = p * g + 1.0f;
  int ki = (int)k;
  /* multiply by 2^ki in at most two exact steps so subnormals come out right */
  if (ki > 127) {
    p = p * ptm_u2f(0x7f000000u); /* 2^127 */
    ki -= 127;
  } else if (ki < -126) {
    p = p * ptm_u2f(0x00800000u); /* 2^-126 */
    ki += 126;
  }
  return p * ptm_u2f((uint32_t)(ki + 127) << 23);
}

PTM_FN float pt_log2f(float x) {
  if (ptm_isnan(x) || x < 0.0f) return ptm_u2f(0x7fc00000u);
  if (x == 0.0f) return ptm_u2f(0xff800000u);
  if (ptm_f2u(x) == 0x7f800000u) return x;
  return ptm_log2_pos(x);
}

PTM_FN float pt_expf(float x) { return pt_exp2f(x * PTM_LOG2E); }
PTM_FN float pt_logf(float x) { return pt_log2f(x) * PTM_LN2; }

PTM_FN float pt_powf(float x, float y) {
  if (y == 0.0f || x == 1.0f) return 1.0f;
  if (ptm_isnan(x) || ptm_isnan(y)) return x + y;
  float ax = ptm_fabs(x);
  int neg = 0;
  if (x < 0.0f) {
    if (ptm_floor(y) != y) return ptm_u2f(0x7fc00000u);
    /* y integral: odd y keeps the sign */
    float h = y * 0.5f;
    neg = (ptm_floor(h) != h);
  }
  float r;
  if (ax == 0.0f) {
    r = y > 0.0f ? 0.0f : ptm_u2f(0x7f800000u);
  } else if (ptm_f2u(ax) == 0x7f800000u) {
    r = y > 0.0f ? ax : 0.0f;
  } else {
    r = pt_exp2f(y * ptm_log2_pos(ax));
  }
  return neg ? -r : r;
}

#endif /* PT_MATH_H */
