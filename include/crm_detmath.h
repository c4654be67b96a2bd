/*
 * crm_detmath.h -- deterministic double-precision exp, log and pow.
 *
 * The CRM calls exp, log and ** (pow) on the hot path: precip_init.F90:54-91
 * (per level and step), precip_proc.F90:75-125 and microphysics.F90:453-486
 * (per cell), ice_fall.F90:108, damping.F90:58, sat.F90:30,93 (below -80 C).
 * CUDA's libdevice and glibc's libm round these differently in the last bit,
 * and a one-ulp difference in a cell feeds the chaotic CRM integration.  To
 * make the FP64 device form bit-identical to a CPU run of the same
 * algorithm, both sides evaluate these three functions with the code below,
 * built only from IEEE-754 +, -, *, /, sqrt and fma (correctly rounded on
 * both sides when implicit contraction is off: nvcc -fmad=false, gcc
 * -ffp-contract=off).
 *
 * Methods (textbook, not taken from any vendor library):
 *  - exp: Cody-Waite reduction x = n*ln2 + r, |r| <= ln2/2, with ln2 split
 *    into a 32-bit head and a tail so n*ln2_head is exact; e^r from its
 *    Taylor series to degree 13 (truncation < 4e-18 relative) by Horner's
 *    rule; scaling by 2^n through the exponent field.
 *  - log: x = 2^e * m with m in [sqrt(1/2), sqrt(2)); f = m - 1,
 *    s = f/(2+f), log(m) = 2 atanh(s) = f - (f^2/2 - s*(f^2/2 + R)) with
 *    R = sum_{k=1..12} 2 s^(2k)/(2k+1) (truncation < 1e-19).
 *  - pow(x, y) = exp(y * log(x)) for x > 0; pow(0, y>0) = 0, with log(x)
 *    carried as an exact head e*ln2_head plus a tail and the product y*log x
 *    split exactly by one fused multiply-add (correctly rounded on both
 *    sides), so the result stays within a few ulp for large |y log x|.
 *  - atan: odd symmetry, atan(x) = pi/2 - atan(1/x) above 1, then
 *    atan(x) = pi/6 + atan((sqrt(3) x - 1)/(x + sqrt(3))) above tan(pi/12),
 *    and the Taylor series to t^29 on |t| <= tan(pi/12) (< 1e-18).
 * Accuracy on the CRM's arguments is checked against the platform libm in
 * tests/test_detmath.py (exp, log, pow <= 2 ulp, atan <= 4 ulp).
 */
#ifndef CRM_DETMATH_H
#define CRM_DETMATH_H

#if defined(__CUDACC__)
#define CRM_DM_FN __host__ __device__ __forceinline__
#else
#define CRM_DM_FN static inline
#include <string.h>
#endif

#ifdef __cplusplus
namespace crm_detmath {
#endif

CRM_DM_FN double dm_from_bits(long long b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double(b);
#else
  double d;
  memcpy(&d, &b, sizeof d);
  return d;
#endif
}

CRM_DM_FN long long dm_to_bits(double d) {
#if defined(__CUDA_ARCH__)
  return __double_as_longlong(d);
#else
  long long b;
  memcpy(&b, &d, sizeof b);
  return b;
#endif
}

/* ln 2 = DM_LN2_HI + DM_LN2_LO; the head has 32 trailing zero bits. */
#define DM_LN2_HI 6.93147180369123816490e-01
#define DM_LN2_LO 1.90821492927058770002e-10
#define DM_INV_LN2 1.44269504088896338700e+00

/* 2^n for -1022 <= n <= 1023 */
CRM_DM_FN double dm_pow2i(int n) {
  return dm_from_bits((long long)(n + 1023) << 52);
}

/* exp(hi + lo) for |lo| much smaller than |hi|: the tail enters the
 * reduced argument after the exact subtraction of n*ln2_head. */
CRM_DM_FN double det_exp2(double hi, double lo) {
  if (hi != hi) return hi;                  /* NaN */
  if (hi > 709.0) return dm_from_bits(0x7ff0000000000000LL);
  if (hi < -744.0) return 0.0;
  double fn = hi * DM_INV_LN2 + 0.5;
#if defined(__CUDA_ARCH__)
  fn = floor(fn);
#else
  fn = __builtin_floor(fn);
#endif
  int n = (int)fn;
  double r = ((hi - fn * DM_LN2_HI) + lo) - fn * DM_LN2_LO;
  /* Taylor coefficients 1/k!, k = 13 .. 0 */
  double p = 1.6059043836821614599e-10;   /* 1/13! */
  p = p * r + 2.0876756987868098979e-09;  /* 1/12! */
  p = p * r + 2.5052108385441718775e-08;  /* 1/11! */
  p = p * r + 2.7557319223985890653e-07;  /* 1/10! */
  p = p * r + 2.7557319223985892511e-06;  /* 1/9!  */
  p = p * r + 2.4801587301587301566e-05;  /* 1/8!  */
  p = p * r + 1.9841269841269841253e-04;  /* 1/7!  */
  p = p * r + 1.3888888888888889419e-03;  /* 1/6!  */
  p = p * r + 8.3333333333333332177e-03;  /* 1/5!  */
  p = p * r + 4.1666666666666664354e-02;  /* 1/4!  */
  p = p * r + 1.6666666666666665741e-01;  /* 1/3!  */
  p = p * r + 0.5;
  p = p * r + 1.0;
  p = p * r + 1.0;
  if (n < -1021) {                          /* gradual underflow */
    return (p * dm_pow2i(n + 600)) * dm_pow2i(-600);
  }
  if (n > 1023) return (p * dm_pow2i(n - 600)) * dm_pow2i(600);
  return p * dm_pow2i(n);
}

CRM_DM_FN double det_exp(double x) { return det_exp2(x, 0.0); }

/* log(x) as hi + lo: hi = e*ln2_head is exact, lo = e*ln2_tail + log(m).
 * Returns 0 and sets *hi to the special value for x <= 0, NaN and +Inf. */
CRM_DM_FN int det_log2(double x, double *hi, double *lo) {
  *lo = 0.0;
  if (x != x || x < 0.0) { *hi = dm_from_bits(0x7ff8000000000000LL); return 0; }
  if (x == 0.0) { *hi = -dm_from_bits(0x7ff0000000000000LL); return 0; }
  long long b = dm_to_bits(x);
  int e = 0;
  if ((b >> 52) == 0) {                     /* subnormal: scale by 2^54 */
    x = x * 18014398509481984.0;
    b = dm_to_bits(x);
    e = -54;
  }
  if ((b >> 52) >= 0x7ff) { *hi = x; return 0; }   /* +Inf */
  e += (int)((b >> 52) & 0x7ff) - 1023;
  b = (b & 0x000fffffffffffffLL) | 0x3ff0000000000000LL;   /* m in [1,2) */
  double m = dm_from_bits(b);
  if (m > 1.4142135623730951) {
    m = m * 0.5;
    e += 1;
  }
  double f = m - 1.0;
  double s = f / (2.0 + f);
  double z = s * s;
  /* R = sum_{k=1}^{12} 2 z^k / (2k+1) by Horner */
  double R = 8.0000000000000004441e-02;     /* 2/25 */
  R = R * z + 8.6956521739130432160e-02;    /* 2/23 */
  R = R * z + 9.5238095238095232808e-02;    /* 2/21 */
  R = R * z + 1.0526315789473683626e-01;    /* 2/19 */
  R = R * z + 1.1764705882352941013e-01;    /* 2/17 */
  R = R * z + 1.3333333333333333148e-01;    /* 2/15 */
  R = R * z + 1.5384615384615385469e-01;    /* 2/13 */
  R = R * z + 1.8181818181818182323e-01;    /* 2/11 */
  R = R * z + 2.2222222222222220989e-01;    /* 2/9  */
  R = R * z + 2.8571428571428569843e-01;    /* 2/7  */
  R = R * z + 4.0000000000000002220e-01;    /* 2/5  */
  R = R * z + 6.6666666666666662966e-01;    /* 2/3  */
  R = R * z;
  double hfsq = 0.5 * f * f;
  double de = (double)e;
  *hi = de * DM_LN2_HI;
  *lo = de * DM_LN2_LO - ((hfsq - s * (hfsq + R)) - f);
  return 1;
}

CRM_DM_FN double det_log(double x) {
  double hi, lo;
  if (!det_log2(x, &hi, &lo)) return hi;
  return hi + lo;
}

CRM_DM_FN double dm_fma(double a, double b, double c) {
#if defined(__CUDA_ARCH__)
  return fma(a, b, c);
#else
  return __builtin_fma(a, b, c);
#endif
}

CRM_DM_FN double det_pow(double x, double y) {
  if (y == 0.0) return 1.0;
  if (x == 0.0) return y > 0.0 ? 0.0 : dm_from_bits(0x7ff0000000000000LL);
  if (x < 0.0 || x != x || y != y) return dm_from_bits(0x7ff8000000000000LL);
  if (x == 1.0) return 1.0;
  double lh, ll;
  det_log2(x, &lh, &ll);
  double ph = y * lh;
  double pl = dm_fma(y, lh, -ph) + y * ll;  /* exact product tail */
  double h = ph + pl;                       /* renormalise the pair */
  double t = pl - (h - ph);
  return det_exp2(h, t);
}

CRM_DM_FN double det_atan(double x) {
  if (x != x) return x;
  double sgn = 1.0;
  if (x < 0.0) { x = -x; sgn = -1.0; }
  double base = 0.0, mul = 1.0;
  if (x > 1.0) { x = 1.0 / x; base = 1.5707963267948966; mul = -1.0; }
  double off = 0.0;
  if (x > 0.2679491924311227) {             /* tan(pi/12) */
    x = (1.7320508075688772 * x - 1.0) / (x + 1.7320508075688772);
    off = 0.52359877559829887;               /* pi/6 */
  }
  double z = x * x;
  /* sum_{k=0}^{14} (-1)^k z^k / (2k+1) */
  double s = 1.0 / 29.0;
  s = -s * z + 1.0 / 27.0;
  s = -s * z + 1.0 / 25.0;
  s = -s * z + 1.0 / 23.0;
  s = -s * z + 1.0 / 21.0;
  s = -s * z + 1.0 / 19.0;
  s = -s * z + 1.0 / 17.0;
  s = -s * z + 1.0 / 15.0;
  s = -s * z + 1.0 / 13.0;
  s = -s * z + 1.0 / 11.0;
  s = -s * z + 1.0 / 9.0;
  s = -s * z + 1.0 / 7.0;
  s = -s * z + 1.0 / 5.0;
  s = -s * z + 1.0 / 3.0;
  s = -s * z + 1.0;
  double r = off + x * s;
  return sgn * (base + mul * r);
}

#ifdef __cplusplus
} /* namespace crm_detmath */
#endif
#endif /* CRM_DETMATH_H */
