/* mcx_fmath.h - portable FP64 exp, log, log10 and pow.
 *
 * The plain FP64 balance is checked against a sequential C restatement to a
 * relative 1e-6 on every cell.  iterateT and ionBalance branch on their own
 * residuals (secant bracketing, X-iteration exits, the x1.2 steps), so a
 * one-ulp difference between two libraries' exp or pow can send a cell down
 * another branch and leave it a few per cent away.  Both sides therefore
 * evaluate the transcendental functions with the routines below, which use
 * only +, -, *, / (each correctly rounded in IEEE double on the host and on
 * the GPU), floor and exponent-field bit operations.  Compiled without FMA
 * contraction (nvcc --fmad=false, gcc -ffp-contract=off) they give the same
 * bits on x86, Arm and sm_103a.
 *
 * Methods (textbook, written from the mathematics):
 *   exp:  x = k ln2 + r with ln2 split into a 32-bit head and a tail (the
 *         Cody & Waite reduction, so k ln2_hi is exact), |r| <= ln2/2,
 *         e^r by its Taylor series to r^13 (truncation < 0.05 ulp), then
 *         scaled by 2^k through the exponent field.
 *   log:  x = m 2^e with m in (sqrt(1/2), sqrt(2)]; ln m = 2 atanh(s),
 *         s = (m - 1)/(m + 1), by its odd series to s^23 (|s| < 0.172).
 *   log10 = log / ln 10;  pow(x, y) = exp(y log x) for x > 0, with the
 *         C99 special cases for zero, negative bases with integral y,
 *         infinities and NaN.
 *   sin, cos: x = k pi/2 + r with pi/2 split into a 33-bit head and a tail,
 *         |r| <= pi/4, sin r and cos r by their Taylor series to r^19 and
 *         r^20, the quadrant k mod 4 choosing the sign and the function;
 *         meant for |x| < 1e6 (the transport's angles lie in [-pi, pi]).
 * Accuracy (tests/test_fmath_cpu.py, against the host's libm): exp and log
 * within 2 ulp, log10 within 3 ulp, pow within (2 |y ln x| + 4) ulp, sin
 * and cos within 2 ulp plus an absolute 1e-22 (the pi/2 reduction's error
 * near a zero of the function).
 */
#ifndef MCX_FMATH_H
#define MCX_FMATH_H

#include <stdint.h>

#include <string.h>

#if defined(__CUDACC__)
#define MCX_FM_FN static __host__ __device__ __forceinline__
#else
#define MCX_FM_FN static inline
#endif

#define MCX_FM_LN2_HI 6.93147180369123816490e-01  /* ln 2 with its low 21 mantissa bits cleared */
#define MCX_FM_LN2_LO 1.9082149292705877e-10      /* ln 2 - MCX_FM_LN2_HI */
#define MCX_FM_INV_LN2 1.4426950408889634
#define MCX_FM_INV_LN10 0.4342944819032518
#define MCX_FM_SQRT2 1.4142135623730951

MCX_FM_FN uint64_t mcx_fm_bits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  memcpy(&b, &x, sizeof b);
  return b;
#endif
}

MCX_FM_FN double mcx_fm_from_bits(uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double x;
  memcpy(&x, &b, sizeof x);
  return x;
#endif
}

MCX_FM_FN double mcx_fm_inf(void) { return mcx_fm_from_bits(0x7ff0000000000000ULL); }
MCX_FM_FN double mcx_fm_nan(void) { return mcx_fm_from_bits(0x7ff8000000000000ULL); }

/* 2^k as a double, for -1022 <= k <= 1023 */
MCX_FM_FN double mcx_fm_pow2i(int k) { return mcx_fm_from_bits((uint64_t)(k + 1023) << 52); }

/* p * 2^k for p in [0.5, 2): one rounding, also into the subnormal range */
MCX_FM_FN double mcx_fm_scale(double p, int k) {
  if (k > 1023) return p * mcx_fm_pow2i(1023) * mcx_fm_pow2i(k - 1023);
  if (k < -1021) return p * mcx_fm_pow2i(k + 1000) * mcx_fm_pow2i(-1000);
  return p * mcx_fm_pow2i(k);
}

MCX_FM_FN double mcx_fm_floor(double x) {
#if defined(__CUDA_ARCH__)
  return floor(x);
#else
  return __builtin_floor(x);
#endif
}

MCX_FM_FN double mcx_fm_exp(double x) {
  if (!(x == x)) return x;
  if (x > 709.782712893384) return mcx_fm_inf();
  if (x < -745.1332191019412) return 0.0;
  const double kd = mcx_fm_floor(x * MCX_FM_INV_LN2 + 0.5);
  const double r = (x - kd * MCX_FM_LN2_HI) - kd * MCX_FM_LN2_LO;
  double p = 1.6059043836821613e-10;          /* 1/13! */
  p = 2.08767569878681e-09 + r * p;           /* 1/12! */
  p = 2.505210838544172e-08 + r * p;          /* 1/11! */
  p = 2.755731922398589e-07 + r * p;          /* 1/10! */
  p = 2.7557319223985893e-06 + r * p;         /* 1/9!  */
  p = 2.48015873015873e-05 + r * p;           /* 1/8!  */
  p = 1.984126984126984e-04 + r * p;          /* 1/7!  */
  p = 1.388888888888889e-03 + r * p;          /* 1/6!  */
  p = 8.333333333333333e-03 + r * p;          /* 1/5!  */
  p = 4.1666666666666664e-02 + r * p;         /* 1/4!  */
  p = 1.6666666666666666e-01 + r * p;         /* 1/3!  */
  p = 0.5 + r * p;
  p = 1.0 + r * p;
  p = 1.0 + r * p;
  return mcx_fm_scale(p, (int)kd);
}

MCX_FM_FN double mcx_fm_log(double x) {
  if (!(x == x)) return x;
  if (x < 0.0) return mcx_fm_nan();
  if (x == 0.0) return -mcx_fm_inf();
  if (x == mcx_fm_inf()) return x;
  int e = 0;
  uint64_t b = mcx_fm_bits(x);
  if ((b >> 52) == 0) {                        /* subnormal: scale by 2^54 */
    b = mcx_fm_bits(x * mcx_fm_pow2i(54));
    e = -54;
  }
  e += (int)(b >> 52) - 1023;
  double m = mcx_fm_from_bits((b & 0x000fffffffffffffULL) | (1023ULL << 52));
  if (m > MCX_FM_SQRT2) {
    m = m * 0.5;
    e += 1;
  }
  const double f = m - 1.0;                    /* exact for m in [0.5, 2] */
  const double s = f / (2.0 + f);
  const double z = s * s;
  double R = 0.043478260869565216;             /* 1/23 */
  R = 0.047619047619047616 + z * R;            /* 1/21 */
  R = 0.05263157894736842 + z * R;             /* 1/19 */
  R = 0.058823529411764705 + z * R;            /* 1/17 */
  R = 0.06666666666666667 + z * R;             /* 1/15 */
  R = 0.07692307692307693 + z * R;             /* 1/13 */
  R = 0.09090909090909091 + z * R;             /* 1/11 */
  R = 0.1111111111111111 + z * R;              /* 1/9  */
  R = 0.14285714285714285 + z * R;             /* 1/7  */
  R = 0.2 + z * R;                             /* 1/5  */
  R = 0.3333333333333333 + z * R;              /* 1/3  */
  R = z * R;
  const double t = s + s * R;
  const double lm = t + t;
  const double ed = (double)e;
  return ed * MCX_FM_LN2_HI + (lm + ed * MCX_FM_LN2_LO);
}

MCX_FM_FN double mcx_fm_log10(double x) { return mcx_fm_log(x) * MCX_FM_INV_LN10; }

MCX_FM_FN double mcx_fm_pow(double x, double y) {
  if (y == 0.0 || x == 1.0) return 1.0;
  if (!(x == x) || !(y == y)) return mcx_fm_nan();
  const double inf = mcx_fm_inf();
  if (y == inf || y == -inf) {
    const double ax = x < 0.0 ? -x : x;
    if (ax == 1.0) return 1.0;
    return (ax > 1.0) == (y > 0.0) ? inf : 0.0;
  }
  double sign = 1.0;
  if (x < 0.0) {
    const double yi = mcx_fm_floor(y);
    if (yi != y) return mcx_fm_nan();
    const double half = y * 0.5;
    if (mcx_fm_floor(half) != half) sign = -1.0;   /* odd integral exponent */
    x = -x;
  }
  if (x == 0.0) return sign * (y > 0.0 ? 0.0 : inf);
  if (x == inf) return sign * (y > 0.0 ? inf : 0.0);
  return sign * mcx_fm_exp(y * mcx_fm_log(x));
}

#define MCX_FM_PIO2_HI 1.5707963267341256     /* pi/2 with its low 20 mantissa bits cleared */
#define MCX_FM_PIO2_LO 6.077100506506192e-11   /* pi/2 - MCX_FM_PIO2_HI */
#define MCX_FM_TWO_OVER_PI 0.6366197723675814

/* sin r and cos r for |r| <= pi/4 */
MCX_FM_FN double mcx_fm_sin_kernel(double r) {
  const double z = r * r;
  double p = -8.22063524662433e-18;            /* -1/19! */
  p = 2.8114572543455206e-15 + z * p;          /*  1/17! */
  p = -7.647163731819816e-13 + z * p;          /* -1/15! */
  p = 1.6059043836821613e-10 + z * p;          /*  1/13! */
  p = -2.505210838544172e-08 + z * p;          /* -1/11! */
  p = 2.7557319223985893e-06 + z * p;          /*  1/9!  */
  p = -1.984126984126984e-04 + z * p;          /* -1/7!  */
  p = 8.333333333333333e-03 + z * p;           /*  1/5!  */
  p = -1.6666666666666666e-01 + z * p;         /* -1/3!  */
  return r + (r * z) * p;
}

MCX_FM_FN double mcx_fm_cos_kernel(double r) {
  const double z = r * r;
  double p = 4.110317623312165e-19;            /*  1/20! */
  p = -1.5619206968586225e-16 + z * p;         /* -1/18! */
  p = 4.779477332387385e-14 + z * p;           /*  1/16! */
  p = -1.1470745597729725e-11 + z * p;         /* -1/14! */
  p = 2.08767569878681e-09 + z * p;            /*  1/12! */
  p = -2.755731922398589e-07 + z * p;          /* -1/10! */
  p = 2.48015873015873e-05 + z * p;            /*  1/8!  */
  p = -1.388888888888889e-03 + z * p;          /* -1/6!  */
  p = 4.1666666666666664e-02 + z * p;          /*  1/4!  */
  p = -0.5 + z * p;                            /* -1/2!  */
  return 1.0 + z * p;
}

/* x = k pi/2 + r; returns r and the quadrant k mod 4 */
MCX_FM_FN double mcx_fm_reduce_pio2(double x, int* quadrant) {
  const double kd = mcx_fm_floor(x * MCX_FM_TWO_OVER_PI + 0.5);
  const double r = (x - kd * MCX_FM_PIO2_HI) - kd * MCX_FM_PIO2_LO;
  const long long k = (long long)kd;
  *quadrant = (int)(((k % 4) + 4) % 4);
  return r;
}

MCX_FM_FN double mcx_fm_sin(double x) {
  if (!(x == x) || x == mcx_fm_inf() || x == -mcx_fm_inf()) return mcx_fm_nan();
  int q;
  const double r = mcx_fm_reduce_pio2(x, &q);
  switch (q) {
    case 0: return mcx_fm_sin_kernel(r);
    case 1: return mcx_fm_cos_kernel(r);
    case 2: return -mcx_fm_sin_kernel(r);
    default: return -mcx_fm_cos_kernel(r);
  }
}

MCX_FM_FN double mcx_fm_cos(double x) {
  if (!(x == x) || x == mcx_fm_inf() || x == -mcx_fm_inf()) return mcx_fm_nan();
  int q;
  const double r = mcx_fm_reduce_pio2(x, &q);
  switch (q) {
    case 0: return mcx_fm_cos_kernel(r);
    case 1: return -mcx_fm_sin_kernel(r);
    case 2: return -mcx_fm_cos_kernel(r);
    default: return mcx_fm_sin_kernel(r);
  }
}

/* TwoSum (Knuth): the rounding error of s = RN(a + b), exactly: a + b = s + err */
MCX_FM_FN double mcx_fm_two_sum_err(double a, double b, double s) {
  const double bb = s - a;
  return (a - (s - bb)) + (b - bb);
}

#endif /* MCX_FMATH_H */
