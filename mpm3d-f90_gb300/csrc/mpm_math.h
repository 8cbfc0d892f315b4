/*
 * mpm_math.h -- deterministic log / exp / pow in plain IEEE double arithmetic.
 *
 * Why: the reference evaluates Johnson-Cook hardening (Constitution.f90:998,
 * 1014-1015, 1066, 1080-1081, 1169, 1192-1193), the neo-Hookean log
 * (:753-755) and the JWL exponentials (:1491-1492) with the host libm. glibc
 * and the CUDA math library may differ by an ulp, and an ulp can flip the
 * REAL(4) rounding of the equivalent stress that the plastic return uses. The
 * "strict" build of the FP64 step therefore calls these functions on both the
 * CPU oracle and the GPU: the same sequence of correctly rounded + - * / on
 * both sides gives the same bits, provided the compilers do not contract
 * a*b+c into fused multiply-adds (host: -ffp-contract=off, device:
 * --fmad=false).
 *
 * Methods (textbook, written for this project):
 *   log: x = 2^k * m with m in [sqrt(1/2), sqrt(2)), s = (m-1)/(m+1),
 *        log m = 2 atanh(s) = 2 s (1 + s^2/3 + s^4/5 + ...), summed by Horner
 *        to s^26; k*ln2 added in two parts (Cody & Waite splitting).
 *   exp: k = nearest integer to x/ln2, r = (x - k ln2_hi) - k ln2_lo
 *        (Cody-Waite), exp r by its Taylor series to r^14 (|r| <= ln2/2),
 *        scaled by 2^k built from the exponent bits.
 *   pow: exp(y log x) for x > 0, with the IEEE special cases for 0, 1, inf,
 *        NaN and negative x with integral y.
 * Accuracy is a few ulp, which is all the parity argument needs: equality
 * between the two sides, not correct rounding.
 */
#ifndef MPM_MATH_H
#define MPM_MATH_H

#include <stdint.h>

#if defined(__CUDACC__)
#define MPM_HD __host__ __device__ __forceinline__
#else
#include <string.h>
#define MPM_HD static inline
#endif

MPM_HD int64_t mpm_d2bits(double x) {
#if defined(__CUDA_ARCH__)
  return __double_as_longlong(x);
#else
  int64_t b;
  memcpy(&b, &x, sizeof b);
  return b;
#endif
}

MPM_HD double mpm_bits2d(int64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double(b);
#else
  double x;
  memcpy(&x, &b, sizeof x);
  return x;
#endif
}

/* 2^k for -1022 <= k <= 1023 */
MPM_HD double mpm_pow2i(int k) { return mpm_bits2d((int64_t)(k + 1023) << 52); }

MPM_HD double mpm_log(double x) {
  const int64_t bits = mpm_d2bits(x);
  if (x != x) return x;
  if (x < 0.0) return mpm_bits2d(0x7ff8000000000000LL); /* NaN */
  if (x == 0.0) return -mpm_bits2d(0x7ff0000000000000LL);
  if (bits >= 0x7ff0000000000000LL) return x; /* +inf */
  int k = 0;
  int64_t b = bits;
  if (b < 0x0010000000000000LL) { /* subnormal: scale by 2^54 */
    b = mpm_d2bits(x * 18014398509481984.0);
    k = -54;
  }
  k += (int)((b >> 52) & 0x7ff) - 1023;
  double m = mpm_bits2d((b & 0x000fffffffffffffLL) | 0x3ff0000000000000LL); /* [1,2) */
  if (m > 1.4142135623730951) { m = m * 0.5; k += 1; }
  const double f = m - 1.0;
  const double s = f / (2.0 + f);
  const double z = s * s;
  /* 1 + z/3 + z^2/5 + ... + z^13/27 */
  double p = 1.0 / 27.0;
  p = p * z + 1.0 / 25.0;
  p = p * z + 1.0 / 23.0;
  p = p * z + 1.0 / 21.0;
  p = p * z + 1.0 / 19.0;
  p = p * z + 1.0 / 17.0;
  p = p * z + 1.0 / 15.0;
  p = p * z + 1.0 / 13.0;
  p = p * z + 1.0 / 11.0;
  p = p * z + 1.0 / 9.0;
  p = p * z + 1.0 / 7.0;
  p = p * z + 1.0 / 5.0;
  p = p * z + 1.0 / 3.0;
  const double two_s = s + s;
  const double tail = two_s * (p * z); /* 2s (z/3 + z^2/5 + ...) */
  const double ln2_hi = 6.93147180369123816490e-01; /* upper 32 bits of ln 2 */
  const double ln2_lo = 1.90821492927058770002e-10; /* ln 2 - ln2_hi */
  const double dk = (double)k;
  return dk * ln2_hi + ((two_s + (tail + dk * ln2_lo)));
}

MPM_HD double mpm_exp(double x) {
  if (x != x) return x;
  if (x > 709.782712893383973096) return mpm_bits2d(0x7ff0000000000000LL);
  if (x < -745.1332191019411) return 0.0;
  const double inv_ln2 = 1.44269504088896338700e+00;
  const double ln2_hi = 6.93147180369123816490e-01;
  const double ln2_lo = 1.90821492927058770002e-10;
  double t = x * inv_ln2;
  int k = (int)(t < 0.0 ? t - 0.5 : t + 0.5);
  const double dk = (double)k;
  const double r = (x - dk * ln2_hi) - dk * ln2_lo;
  /* Taylor series of e^r to r^14 */
  double p = 1.0 / 87178291200.0;   /* 1/14! */
  p = p * r + 1.0 / 6227020800.0;   /* 1/13! */
  p = p * r + 1.0 / 479001600.0;    /* 1/12! */
  p = p * r + 1.0 / 39916800.0;     /* 1/11! */
  p = p * r + 1.0 / 3628800.0;      /* 1/10! */
  p = p * r + 1.0 / 362880.0;       /* 1/9!  */
  p = p * r + 1.0 / 40320.0;        /* 1/8!  */
  p = p * r + 1.0 / 5040.0;         /* 1/7!  */
  p = p * r + 1.0 / 720.0;          /* 1/6!  */
  p = p * r + 1.0 / 120.0;          /* 1/5!  */
  p = p * r + 1.0 / 24.0;           /* 1/4!  */
  p = p * r + 1.0 / 6.0;            /* 1/3!  */
  p = p * r + 0.5;
  p = p * r + 1.0;
  p = p * r + 1.0;
  if (k > 1023) return p * mpm_pow2i(1023) * mpm_pow2i(k - 1023);
  if (k < -1022) return p * mpm_pow2i(k + 1000) * mpm_pow2i(-1000);
  return p * mpm_pow2i(k);
}

MPM_HD int mpm_is_int(double y) {
  /* |y| >= 2^52 are integers; else compare with truncation */
  double a = y < 0 ? -y : y;
  if (a >= 4503599627370496.0) return 1;
  return (double)(int64_t)y == y;
}

MPM_HD double mpm_pow(double x, double y) {
  const double inf = mpm_bits2d(0x7ff0000000000000LL);
  const double nan = mpm_bits2d(0x7ff8000000000000LL);
  if (y == 0.0) return 1.0;
  if (x == 1.0) return 1.0;
  if (x != x || y != y) return nan;
  if (x == 0.0) {
    if (y > 0.0) return 0.0;
    return inf;
  }
  if (x < 0.0) {
    if (!mpm_is_int(y)) return nan;
    double a = y < 0 ? -y : y;
    double r = mpm_exp(y * mpm_log(-x));
    int odd = (a < 9007199254740992.0) && (((int64_t)a) & 1);
    return odd ? -r : r;
  }
  if (x == inf) return y > 0.0 ? inf : 0.0;
  return mpm_exp(y * mpm_log(x));
}

#endif /* MPM_MATH_H */
