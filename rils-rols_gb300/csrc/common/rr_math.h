/*
 * FP64 element-wise functions of the fitness path: exp, log, sin, cos, pow.
 *
 * One definition compiled for the host (C99 / C++, -ffp-contract=off) and for
 * the device (CUDA, every operation an explicit round-to-nearest intrinsic),
 * so that the same input gives the same bits on x86, Arm and GB300.  This is
 * what lets the FP64 device path reproduce the CPU oracle bit for bit.
 * Methods (all published; constants are mathematical constants computed for
 * this file, rounded to double):
 *   exp  Cody & Waite argument reduction x = k ln2 + r (ln2 split in a 32-bit
 *        head and a tail), Taylor polynomial of e^r - 1 to degree 13,
 *        scaling by 2^k through the exponent field;
 *   log  x = m 2^e with m in (sqrt(1/2), sqrt(2)], log m = 2 atanh(s),
 *        s = (m-1)/(m+1), atanh series to s^23;
 *   sin, cos  Cody & Waite reduction by pi/2 (three-term split, FMA) for
 *        |x| < 2^20, Payne & Hanek reduction with the binary expansion of 2/pi
 *        above; Taylor polynomials of sin (to r^19) and cos (to r^20) on
 *        |r| <= pi/4 with a first-order correction for the reduced tail;
 *   pow  exp(b log|a|) with the sign and special-value rules of C's pow.
 * Accuracy: a few ulp (checked against the host libm by the CPU tests).
 */
#ifndef RR_MATH_H
#define RR_MATH_H

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define RRM_FN static __host__ __device__ __forceinline__
#else
#define RRM_FN static inline
#endif

#if defined(__CUDA_ARCH__)
#define RRM_ADD(a, b) __dadd_rn((a), (b))
#define RRM_SUB(a, b) __dsub_rn((a), (b))
#define RRM_MUL(a, b) __dmul_rn((a), (b))
#define RRM_DIV(a, b) __ddiv_rn((a), (b))
#define RRM_FMA(a, b, c) __fma_rn((a), (b), (c))
#else
#include <math.h>
#define RRM_ADD(a, b) ((a) + (b))
#define RRM_SUB(a, b) ((a) - (b))
#define RRM_MUL(a, b) ((a) * (b))
#define RRM_DIV(a, b) ((a) / (b))
#define RRM_FMA(a, b, c) fma((a), (b), (c))
#endif

RRM_FN uint64_t rrm_bits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  memcpy(&u, &x, sizeof u);
  return u;
#endif
}
RRM_FN double rrm_from_bits(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, sizeof x);
  return x;
#endif
}
RRM_FN double rrm_inf(void) { return rrm_from_bits(0x7ff0000000000000ull); }
RRM_FN double rrm_nan(void) { return rrm_from_bits(0x7ff8000000000000ull); }
RRM_FN double rrm_pow2(int e) { /* 2^e, -1022 <= e <= 1023 */
  return rrm_from_bits((uint64_t)(e + 1023) << 52);
}
RRM_FN int rrm_isnan(double x) { return x != x; }
RRM_FN double rrm_fabs(double x) { return rrm_from_bits(rrm_bits(x) & 0x7fffffffffffffffull); }

/* round to the nearest integer value (ties to even), |x| < 2^51 */
RRM_FN double rrm_rint(double x) {
  const double shift = 0x1.8p52;
  return RRM_SUB(RRM_ADD(x, shift), shift);
}

/* ------------------------------------------------------------------ exp -- */
RRM_FN double rr_exp(double x) {
  if (rrm_isnan(x)) return x;
  if (x > 0x1.62e42fefa39efp+9) return rrm_inf(); /* > log(DBL_MAX) */
  if (x < -0x1.74910d52d3052p+9) return 0.0;      /* < log of the least subnormal / 2 */
  const double kd = rrm_rint(RRM_MUL(x, 0x1.71547652b82fep+0));
  double r = RRM_FMA(-kd, 0x1.62e42fee00000p-1, x);
  r = RRM_FMA(-kd, 0x1.a39ef35793c76p-33, r);
  /* p = sum_{j=2}^{13} r^(j-2) / j! */
  double p = 0x1.6124613a86d09p-33;
  p = RRM_FMA(p, r, 0x1.1eed8eff8d898p-29);
  p = RRM_FMA(p, r, 0x1.ae64567f544e4p-26);
  p = RRM_FMA(p, r, 0x1.27e4fb7789f5cp-22);
  p = RRM_FMA(p, r, 0x1.71de3a556c734p-19);
  p = RRM_FMA(p, r, 0x1.a01a01a01a01ap-16);
  p = RRM_FMA(p, r, 0x1.a01a01a01a01ap-13);
  p = RRM_FMA(p, r, 0x1.6c16c16c16c17p-10);
  p = RRM_FMA(p, r, 0x1.1111111111111p-7);
  p = RRM_FMA(p, r, 0x1.5555555555555p-5);
  p = RRM_FMA(p, r, 0x1.5555555555555p-3);
  p = RRM_FMA(p, r, 0.5);
  const double em1 = RRM_FMA(RRM_MUL(r, r), p, r);
  double y = RRM_ADD(1.0, em1);
  int k = (int)kd;
  if (k > 1023) {
    y = RRM_MUL(y, rrm_pow2(1023));
    k -= 1023;
  }
  if (k < -1000) return RRM_MUL(RRM_MUL(y, rrm_pow2(k + 1000)), rrm_pow2(-1000));
  return RRM_MUL(y, rrm_pow2(k));
}

/* ------------------------------------------------------------------ log -- */
RRM_FN double rr_log(double x) {
  if (rrm_isnan(x)) return x;
  if (x < 0.0) return rrm_nan();
  if (x == 0.0) return -rrm_inf();
  if (x > 0x1.fffffffffffffp+1023) return x; /* +inf */
  uint64_t b = rrm_bits(x);
  int e = (int)((b >> 52) & 0x7ff);
  if (e == 0) { /* subnormal */
    x = RRM_MUL(x, 0x1p54);
    b = rrm_bits(x);
    e = (int)((b >> 52) & 0x7ff) - 54;
  }
  e -= 1023;
  double m = rrm_from_bits((b & 0x000fffffffffffffull) | 0x3ff0000000000000ull);
  if (m > 0x1.6a09e667f3bcdp+0) {
    m = RRM_MUL(m, 0.5);
    e += 1;
  }
  const double f = RRM_SUB(m, 1.0);
  const double s = RRM_DIV(f, RRM_ADD(2.0, f));
  const double z = RRM_MUL(s, s);
  /* q = sum_{j=1}^{11} z^(j-1) / (2j+1) */
  double q = 1.0 / 23.0;
  q = RRM_FMA(q, z, 1.0 / 21.0);
  q = RRM_FMA(q, z, 1.0 / 19.0);
  q = RRM_FMA(q, z, 1.0 / 17.0);
  q = RRM_FMA(q, z, 1.0 / 15.0);
  q = RRM_FMA(q, z, 1.0 / 13.0);
  q = RRM_FMA(q, z, 1.0 / 11.0);
  q = RRM_FMA(q, z, 1.0 / 9.0);
  q = RRM_FMA(q, z, 1.0 / 7.0);
  q = RRM_FMA(q, z, 1.0 / 5.0);
  q = RRM_FMA(q, z, 1.0 / 3.0);
  const double hs = RRM_ADD(s, s);
  const double lm = RRM_FMA(RRM_MUL(hs, z), q, hs);
  const double ed = (double)e;
  return RRM_FMA(ed, 0x1.62e42fee00000p-1, RRM_FMA(ed, 0x1.a39ef35793c76p-33, lm));
}

/* ------------------------------------------------------------ sin / cos -- */
/* binary expansion of 2/pi: 2/pi = sum_j word[j] 2^(-64 (j+1)) */
#define RR_2PI_WORDS                                                                                         \
  0xa2f9836e4e441529ull, 0xfc2757d1f534ddc0ull, 0xdb6295993c439041ull, 0xfe5163abdebbc561ull,              \
      0xb7246e3a424dd2e0ull, 0x06492eea09d1921cull, 0xfe1deb1cb129a73eull, 0xe88235f52ebb4484ull,          \
      0xe99c7026b45f7e41ull, 0x3991d639835339f4ull, 0x9c845f8bbdf9283bull, 0x1ff897ffde05980full,          \
      0xef2f118b5a0a6d1full, 0x6d367ecf27cb09b7ull, 0x4f463f669e5fea2dull, 0x7527bac7ebe5f17bull,          \
      0x3d0739f78a5292eaull, 0x6bfb5fb11f8d5d08ull, 0x56033046fc7b6babull, 0xf0cfbc209af4361dull,          \
      0xa9e391615ee61b08ull, 0x6599855f14a06840ull
#if defined(__CUDACC__)
__device__ __constant__ static const uint64_t RR_TWO_OVER_PI_D[22] = {RR_2PI_WORDS};
#endif
static const uint64_t RR_TWO_OVER_PI_H[22] = {RR_2PI_WORDS};

RRM_FN uint64_t rrm_two_over_pi(int j) {
#if defined(__CUDA_ARCH__)
  return RR_TWO_OVER_PI_D[j];
#else
  return RR_TWO_OVER_PI_H[j];
#endif
}

/* 64 x 64 -> 128 bit product */
RRM_FN void rrm_mul128(uint64_t a, uint64_t b, uint64_t* hi, uint64_t* lo) {
#if defined(__CUDA_ARCH__)
  *lo = a * b;
  *hi = __umul64hi(a, b);
#else
  const unsigned __int128 p = (unsigned __int128)a * b;
  *lo = (uint64_t)p;
  *hi = (uint64_t)(p >> 64);
#endif
}

/* 64 bits of the little-endian multi-word integer q starting at bit pos */
RRM_FN uint64_t rrm_bits_at(const uint64_t* q, int nw, int pos) {
  const int w = pos >> 6, off = pos & 63;
  const uint64_t lo = w < nw ? q[w] : 0;
  const uint64_t hi = w + 1 < nw ? q[w + 1] : 0;
  return off == 0 ? lo : ((lo >> off) | (hi << (64 - off)));
}

/* Reduces |x| (finite, >= 2^20) modulo pi/2 by Payne & Hanek: returns the
 * quadrant and r = rhi + rlo in [-pi/4, pi/4]. */
RRM_FN int rrm_reduce_large(double ax, double* rhi, double* rlo) {
  const uint64_t b = rrm_bits(ax);
  const int E = (int)((b >> 52) & 0x7ff) - 1075; /* ax = m 2^E */
  const uint64_t m = (b & 0x000fffffffffffffull) | 0x0010000000000000ull;
  int j0 = (E - 1 + 63) / 64 - 1; /* ceil((E-1)/64) - 1, E >= 20-52 */
  if (E - 1 <= 0) j0 = 0;
  if (j0 < 0) j0 = 0;
  /* P = m * (W[j0] W[j0+1] W[j0+2] W[j0+3]) as 5 little-endian words */
  uint64_t h[4], l[4];
  for (int i = 0; i < 4; ++i) rrm_mul128(m, rrm_two_over_pi(j0 + 3 - i), &h[i], &l[i]); /* i = 0: least significant */
  uint64_t q[5];
  q[0] = l[0];
  uint64_t c = 0, s;
  s = h[0] + l[1];
  c = s < h[0];
  q[1] = s;
  s = h[1] + l[2];
  uint64_t c2 = s < h[1];
  s += c;
  c2 += s < c;
  q[2] = s;
  s = h[2] + l[3];
  uint64_t c3 = s < h[2];
  s += c2;
  c3 += s < c2;
  q[3] = s;
  q[4] = h[3] + c3;
  const int sh = 64 * (j0 + 4) - E; /* binary point, 192 <= sh <= 255 */
  int quad = (int)(rrm_bits_at(q, 5, sh) & 3u);
  uint64_t fhi = rrm_bits_at(q, 5, sh - 64), flo = rrm_bits_at(q, 5, sh - 128);
  double sign = 1.0;
  if (fhi >> 63) { /* fraction >= 1/2: take f - 1 */
    quad = (quad + 1) & 3;
    sign = -1.0;
    flo = ~flo + 1;
    fhi = ~fhi + (flo == 0 ? 1 : 0);
  }
  const double a_hi = (double)(fhi >> 11) * 0x1p-53;
  const uint64_t mid = ((fhi & 0x7ffull) << 53) | (flo >> 11);
  const double a_lo = (double)mid * 0x1p-117;
  const double f_hi = RRM_ADD(a_hi, a_lo);
  const double f_lo = RRM_SUB(a_lo, RRM_SUB(f_hi, a_hi));
  /* r = f * pi/2 in double-double */
  const double PIO2_HI = 0x1.921fb54442d18p+0, PIO2_LO = 0x1.1a62633145c07p-54;
  const double p = RRM_MUL(f_hi, PIO2_HI);
  double e = RRM_FMA(f_hi, PIO2_HI, -p);
  e = RRM_FMA(f_hi, PIO2_LO, e);
  e = RRM_FMA(f_lo, PIO2_HI, e);
  const double r = RRM_ADD(p, e);
  *rhi = sign * r;
  *rlo = sign * RRM_SUB(e, RRM_SUB(r, p));
  return quad;
}

/* quadrant of |x| and r with |x| = quadrant * pi/2 + r (mod 2 pi) */
RRM_FN int rrm_reduce(double ax, double* rhi, double* rlo) {
  if (ax <= 0x1.921fb54442d18p-1) {
    *rhi = ax;
    *rlo = 0.0;
    return 0;
  }
  if (ax < 0x1p20) {
    const double kd = rrm_rint(RRM_MUL(ax, 0x1.45f306dc9c883p-1));
    double r = RRM_FMA(-kd, 0x1.921fb54400000p+0, ax);
    r = RRM_FMA(-kd, 0x1.0b4611a600000p-34, r);
    r = RRM_FMA(-kd, 0x1.3198a2e037073p-69, r);
    *rhi = r;
    *rlo = 0.0;
    return (int)((int64_t)kd & 3);
  }
  return rrm_reduce_large(ax, rhi, rlo);
}

RRM_FN double rrm_sin_k(double r, double rl) {
  const double z = RRM_MUL(r, r);
  double p = -0x1.2f49b46814157p-57;         /* -1/19! */
  p = RRM_FMA(p, z, 0x1.952c77030ad4ap-49);  /*  1/17! */
  p = RRM_FMA(p, z, -0x1.ae7f3e733b81fp-41); /* -1/15! */
  p = RRM_FMA(p, z, 0x1.6124613a86d09p-33);  /*  1/13! */
  p = RRM_FMA(p, z, -0x1.ae64567f544e4p-26); /* -1/11! */
  p = RRM_FMA(p, z, 0x1.71de3a556c734p-19);  /*  1/9!  */
  p = RRM_FMA(p, z, -0x1.a01a01a01a01ap-13); /* -1/7!  */
  p = RRM_FMA(p, z, 0x1.1111111111111p-7);   /*  1/5!  */
  p = RRM_FMA(p, z, -0x1.5555555555555p-3);  /* -1/3!  */
  const double corr = RRM_MUL(rl, RRM_FMA(-0.5, z, 1.0));
  return RRM_ADD(r, RRM_FMA(RRM_MUL(r, z), p, corr));
}

RRM_FN double rrm_cos_k(double r, double rl) {
  const double z = RRM_MUL(r, r);
  double p = 0x1.e542ba4020225p-62;          /*  1/20! */
  p = RRM_FMA(p, z, -0x1.6827863b97d97p-53); /* -1/18! */
  p = RRM_FMA(p, z, 0x1.ae7f3e733b81fp-45);  /*  1/16! */
  p = RRM_FMA(p, z, -0x1.93974a8c07c9dp-37); /* -1/14! */
  p = RRM_FMA(p, z, 0x1.1eed8eff8d898p-29);  /*  1/12! */
  p = RRM_FMA(p, z, -0x1.27e4fb7789f5cp-22); /* -1/10! */
  p = RRM_FMA(p, z, 0x1.a01a01a01a01ap-16);  /*  1/8!  */
  p = RRM_FMA(p, z, -0x1.6c16c16c16c17p-10); /* -1/6!  */
  p = RRM_FMA(p, z, 0x1.5555555555555p-5);   /*  1/4!  */
  const double w = RRM_MUL(0.5, z);
  const double h = RRM_SUB(1.0, w);
  const double tail = RRM_SUB(RRM_SUB(1.0, h), w);
  const double t = RRM_FMA(RRM_MUL(z, z), p, RRM_FMA(-r, rl, tail));
  return RRM_ADD(h, t);
}

RRM_FN double rr_sin(double x) {
  if (rrm_isnan(x)) return x;
  const double ax = rrm_fabs(x);
  if (ax > 0x1.fffffffffffffp+1023) return rrm_nan();
  double rh, rl;
  const int q = rrm_reduce(ax, &rh, &rl);
  double v = (q & 1) ? rrm_cos_k(rh, rl) : rrm_sin_k(rh, rl);
  if (q & 2) v = -v;
  return x < 0.0 ? -v : v;
}

RRM_FN double rr_cos(double x) {
  if (rrm_isnan(x)) return x;
  const double ax = rrm_fabs(x);
  if (ax > 0x1.fffffffffffffp+1023) return rrm_nan();
  double rh, rl;
  const int q = rrm_reduce(ax, &rh, &rl);
  double v = (q & 1) ? rrm_sin_k(rh, rl) : rrm_cos_k(rh, rl);
  if ((q + 1) & 2) v = -v;
  return v;
}

/* ------------------------------------------------------------------ pow -- */
RRM_FN int rrm_is_int(double b) { return rrm_fabs(b) >= 0x1p52 || rrm_rint(b) == b; }
RRM_FN int rrm_is_odd_int(double b) {
  if (rrm_fabs(b) >= 0x1p53 || rrm_rint(b) != b) return 0;
  const double h = RRM_MUL(b, 0.5);
  return rrm_rint(h) != h;
}

RRM_FN double rr_pow(double a, double b) {
  if (b == 0.0) return 1.0;
  if (a == 1.0) return 1.0;
  if (rrm_isnan(a) || rrm_isnan(b)) return rrm_nan();
  const double ab = rrm_fabs(a), bb = rrm_fabs(b);
  const int bodd = rrm_is_odd_int(b);
  if (bb > 0x1.fffffffffffffp+1023) { /* b = +-inf */
    if (ab == 1.0) return 1.0;
    return ((ab > 1.0) == (b > 0.0)) ? rrm_inf() : 0.0;
  }
  if (a == 0.0) {
    const double v = b < 0.0 ? rrm_inf() : 0.0;
    return (bodd && rrm_bits(a) >> 63) ? -v : v;
  }
  if (ab > 0x1.fffffffffffffp+1023) { /* a = +-inf */
    const double v = b < 0.0 ? 0.0 : rrm_inf();
    return (a < 0.0 && bodd) ? -v : v;
  }
  double sign = 1.0;
  if (a < 0.0) {
    if (!rrm_is_int(b)) return rrm_nan();
    if (bodd) sign = -1.0;
  }
  return sign * rr_exp(RRM_MUL(b, rr_log(ab)));
}

#endif
