/*
 * Double-float arithmetic ("df32"): a value is the unevaluated sum hi + lo of
 * two FP32 numbers with |lo| <= ulp(hi) / 2, about 48 significant bits over
 * FP32's exponent range.  It runs on the FP32 pipes, which on GB300 issue
 * 64 times as many operations per cycle as the FP64 pipe.
 *
 * Basic operations follow the double-word algorithms analysed by Joldes,
 * Muller and Popescu ("Tight and rigorous error bounds for basic building
 * blocks of double-word arithmetic", ACM TOMS 44(2), 2017): addition
 * (their Algorithm 6), multiplication with FMA (Algorithm 12), division
 * (Algorithm 17 form), the square root by one Karp-Markstein correction of
 * the FP32 root.  Elementary functions are our own: exp by Cody-Waite
 * reduction by ln 2 (three-part split), a Taylor polynomial on r / 16 and
 * four squarings; log by one Newton step on the FP32 logarithm using exp;
 * sin / cos by Cody-Waite reduction by pi / 2 (four-part split, |k| < 4096)
 * and Taylor polynomials on |r| <= pi / 4.  The constants are the Taylor
 * coefficients 1 / k! and splits of ln 2 and pi / 2, each rounded to a
 * double-float.  Relative accuracy is about 1e-13 (absolute for results
 * near zero, and only absolute, about 1e-38, for magnitudes below 1e-31,
 * where the low part leaves FP32's normal range); arguments that the
 * reductions do not cover give NaN, so that a caller treats the value as
 * not computed.
 *
 * Non-finite results carry lo = 0.  Host builds need -ffp-contract=off.
 */
#ifndef RR_DF32_H
#define RR_DF32_H

#include <math.h>

#if defined(__CUDACC__)
#define DFN static __host__ __device__ __forceinline__
#else
#define DFN static inline
#endif

#if defined(__CUDA_ARCH__)
#define DF_ADD(a, b) __fadd_rn((a), (b))
#define DF_SUB(a, b) __fsub_rn((a), (b))
#define DF_MUL(a, b) __fmul_rn((a), (b))
#define DF_DIV(a, b) __fdiv_rn((a), (b))
#define DF_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#define DF_SQRT(a) __fsqrt_rn(a)
#else
#define DF_ADD(a, b) ((float)((a) + (b)))
#define DF_SUB(a, b) ((float)((a) - (b)))
#define DF_MUL(a, b) ((float)((a) * (b)))
#define DF_DIV(a, b) ((float)((a) / (b)))
#define DF_FMA(a, b, c) fmaf((a), (b), (c))
#define DF_SQRT(a) sqrtf(a)
#endif

typedef struct {
  float hi, lo;
} dfl;

DFN dfl dfl_make(float h, float l) {
  dfl r;
  r.hi = h;
  r.lo = l;
  return r;
}
DFN int dfl_finite(float x) { return x - x == 0.0f; }
#if defined(__CUDA_ARCH__)
DFN float dfl_nanf(void) { return __int_as_float(0x7fc00000); }
DFN float dfl_inff(void) { return __int_as_float(0x7f800000); }
/* 2^e for e in [-126, 127] */
DFN float dfl_pow2(int e) { return __int_as_float((e + 127) << 23); }
#else
DFN float dfl_nanf(void) { return NAN; }
DFN float dfl_inff(void) { return INFINITY; }
DFN float dfl_pow2(int e) { return ldexpf(1.0f, e); }
#endif

/* ---- error-free transformations ---- */
DFN dfl dfl_fast_two_sum(float a, float b) {
  const float s = DF_ADD(a, b);
  const float z = DF_SUB(s, a);
  return dfl_make(s, DF_SUB(b, z));
}
DFN dfl dfl_two_sum(float a, float b) {
  const float s = DF_ADD(a, b);
  const float ap = DF_SUB(s, b);
  const float bp = DF_SUB(s, ap);
  return dfl_make(s, DF_ADD(DF_SUB(a, ap), DF_SUB(b, bp)));
}
DFN dfl dfl_two_prod(float a, float b) {
  const float p = DF_MUL(a, b);
  return dfl_make(p, DF_FMA(a, b, -p));
}
/* a non-finite leading part, or a low part made non-finite by an overflow in
 * an intermediate, leaves the value as its leading part */
DFN dfl dfl_guard(dfl r, float lead) {
  if (!dfl_finite(lead)) return dfl_make(lead, 0.0f);
  if (!dfl_finite(r.hi)) return dfl_make(r.hi, 0.0f);
  if (!dfl_finite(r.lo)) r.lo = 0.0f;
  return r;
}

/* ---- conversions ---- */
DFN dfl dfl_from_double(double x) {
  const float h = (float)x;
  if (!dfl_finite(h)) return dfl_make(h, 0.0f);
  return dfl_make(h, (float)(x - (double)h));
}
DFN double dfl_to_double(dfl a) { return (double)a.hi + (double)a.lo; }

/* ---- arithmetic ---- */
DFN dfl dfl_add(dfl x, dfl y) {
  const float lead = DF_ADD(x.hi, y.hi);
  if (!dfl_finite(lead)) return dfl_make(lead, 0.0f);
  const dfl s = dfl_two_sum(x.hi, y.hi);
  const dfl t = dfl_two_sum(x.lo, y.lo);
  const float c = DF_ADD(s.lo, t.hi);
  const dfl v = dfl_fast_two_sum(s.hi, c);
  const float w = DF_ADD(t.lo, v.lo);
  return dfl_guard(dfl_fast_two_sum(v.hi, w), lead);
}
DFN dfl dfl_neg(dfl x) { return dfl_make(-x.hi, -x.lo); }
DFN dfl dfl_sub(dfl x, dfl y) { return dfl_add(x, dfl_neg(y)); }
DFN dfl dfl_mul(dfl x, dfl y) {
  const dfl c = dfl_two_prod(x.hi, y.hi);
  if (!dfl_finite(c.hi)) return dfl_make(c.hi, 0.0f);
  const float tl0 = DF_MUL(x.lo, y.lo);
  const float tl1 = DF_FMA(x.hi, y.lo, tl0);
  const float cl2 = DF_FMA(x.lo, y.hi, tl1);
  const float cl3 = DF_ADD(c.lo, cl2);
  return dfl_guard(dfl_fast_two_sum(c.hi, cl3), c.hi);
}
DFN dfl dfl_mul_f(dfl x, float y) {
  const dfl c = dfl_two_prod(x.hi, y);
  if (!dfl_finite(c.hi)) return dfl_make(c.hi, 0.0f);
  const float cl3 = DF_FMA(x.lo, y, c.lo);
  return dfl_guard(dfl_fast_two_sum(c.hi, cl3), c.hi);
}
DFN dfl dfl_div(dfl x, dfl y) {
  const float th = DF_DIV(x.hi, y.hi);
  if (!dfl_finite(th) || y.hi == 0.0f || th == 0.0f) return dfl_make(th, 0.0f);
  const dfl r = dfl_mul_f(y, th);
  const float pih = DF_SUB(x.hi, r.hi);
  const float dl = DF_SUB(x.lo, r.lo);
  const float d = DF_ADD(pih, dl);
  const float tl = DF_DIV(d, y.hi);
  return dfl_guard(dfl_fast_two_sum(th, tl), th);
}
DFN dfl dfl_sqrt(dfl x) {
  if (!(x.hi > 0.0f) || !dfl_finite(x.hi)) return dfl_make(DF_SQRT(x.hi), 0.0f);
  const float s = DF_SQRT(x.hi);
  const dfl e = dfl_sub(x, dfl_two_prod(s, s));
  const float c = DF_DIV(e.hi, DF_MUL(2.0f, s));
  return dfl_guard(dfl_fast_two_sum(s, c), s);
}
DFN dfl dfl_scale(dfl x, float p2) { return dfl_make(DF_MUL(x.hi, p2), DF_MUL(x.lo, p2)); }

/* ---- comparisons (the semantics of the FP64 comparisons on hi + lo) ---- */
DFN int dfl_lt(dfl a, dfl b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
DFN int dfl_eq(dfl a, dfl b) { return a.hi == b.hi && a.lo == b.lo; }

/* ---- exp ---- */
DFN dfl dfl_exp(dfl x) {
  if (x.hi != x.hi) return dfl_make(dfl_nanf(), 0.0f);
  if (x.hi > 88.72f) return dfl_make(dfl_inff(), 0.0f);
  if (x.hi < -103.5f) return dfl_make(0.0f, 0.0f);
  const float k = rintf(DF_MUL(x.hi, 1.4426950216293335f));
  /* ln 2 = L1 + L2 + L3 (+ 9e-17): L1, L2 of 12 bits, k * L1 and k * L2 exact */
  dfl r = dfl_sub(x, dfl_make(DF_MUL(k, 0.693115234375f), 0.0f));
  r = dfl_sub(r, dfl_make(DF_MUL(k, 3.1948089599609375e-05f), 0.0f));
  r = dfl_sub(r, dfl_two_prod(k, -1.9046542121259336e-09f)); /* k * L3 */
  r = dfl_scale(r, 0.0625f);
  /* expm1(r) = r (1 + r (1/2 + r (1/6 + ... + r / 7!))) on |r| <= 0.022 */
  dfl p = dfl_make(0.00019841270113829523f, -2.725596874933456e-12f);
  p = dfl_add(dfl_mul(p, r), dfl_make(0.0013888889225199819f, -3.3631094437103215e-11f));
  p = dfl_add(dfl_mul(p, r), dfl_make(0.008333333767950535f, -4.34617203337595e-10f));
  p = dfl_add(dfl_mul(p, r), dfl_make(0.0416666679084301f, -1.2417634698280722e-09f));
  p = dfl_add(dfl_mul(p, r), dfl_make(0.1666666716337204f, -4.967053879312289e-09f));
  p = dfl_add(dfl_mul(p, r), dfl_make(0.5f, 0.0f));
  p = dfl_add(dfl_mul(p, r), dfl_make(1.0f, 0.0f));
  dfl em = dfl_mul(p, r);
  /* (1 + em)^2 - 1 = em (em + 2), four times */
  for (int i = 0; i < 4; ++i) em = dfl_mul(em, dfl_add(em, dfl_make(2.0f, 0.0f)));
  dfl e = dfl_add(em, dfl_make(1.0f, 0.0f));
  /* times 2^k in two exact steps (k in [-150, 128]) */
  const int ki = (int)k;
  const int k1 = ki / 2, k2 = ki - k1;
  e = dfl_scale(e, dfl_pow2(k1));
  e = dfl_scale(e, dfl_pow2(k2));
  if (!dfl_finite(e.hi)) e.lo = 0.0f;
  return e;
}

/* ---- log ---- */
/* x = m 2^e with m in [sqrt(1/2), sqrt(2)); x finite, > 0 and normal */
DFN dfl dfl_split_exp(dfl x, int* e) {
#if defined(__CUDA_ARCH__)
  int ex = ((__float_as_int(x.hi) >> 23) & 0xff) - 127;
#else
  int ex;
  frexpf(x.hi, &ex);
  ex -= 1;
#endif
  dfl m = dfl_scale(x, dfl_pow2(-ex));
  if (m.hi > 1.41421353816986083984f) {
    m = dfl_scale(m, 0.5f);
    ex += 1;
  }
  *e = ex;
  return m;
}
DFN dfl dfl_log(dfl x) {
  if (x.hi != x.hi || x.hi < 0.0f) return dfl_make(dfl_nanf(), 0.0f);
  if (x.hi == 0.0f) return dfl_make(-dfl_inff(), 0.0f);
  if (!dfl_finite(x.hi)) return dfl_make(dfl_inff(), 0.0f);
  int shift = 0;
  if (x.hi < 1e-30f) {  /* keep m and its low part normal: log(x) = log(x 2^64) - 64 ln 2 */
    x = dfl_scale(x, 18446744073709551616.0f);
    shift = 64;
  }
  int e;
  const dfl m = dfl_split_exp(x, &e);
  const float y0 = logf(m.hi);
  /* log(m) = y0 + m exp(-y0) - 1, one Newton step */
  const dfl t = dfl_mul(m, dfl_exp(dfl_make(-y0, 0.0f)));
  const dfl lm = dfl_add(dfl_make(y0, 0.0f), dfl_add(t, dfl_make(-1.0f, 0.0f)));
  /* + (e - shift) ln 2 */
  return dfl_add(lm, dfl_mul_f(dfl_make(0.6931471824645996f, -1.9046542121259336e-09f), (float)(e - shift)));
}

/* ---- sin / cos ---- */
/* r = x - k pi/2 with pi/2 = P1 + P2 + P3 + P4; returns the quadrant k mod 4,
 * or -1 when |k| >= 4096 (the reduction is not exact there) */
DFN int dfl_reduce_half_pi(dfl x, dfl* r) {
  const float k = rintf(DF_MUL(x.hi, 0.6366197466850281f));
  if (!(fabsf(k) < 4096.0f)) return -1;
  dfl t = dfl_sub(x, dfl_make(DF_MUL(k, 1.57080078125f), 0.0f));
  t = dfl_sub(t, dfl_make(DF_MUL(k, -4.453584551811218e-06f), 0.0f));
  t = dfl_sub(t, dfl_two_prod(k, -8.705515752716053e-10f));
  t = dfl_sub(t, dfl_two_prod(k, 5.721188916458728e-18f));
  *r = t;
  const int ki = (int)k;
  return ki & 3;
}
DFN dfl dfl_sin_kernel(dfl r) {
  const dfl z = dfl_mul(r, r);
  dfl p = dfl_make(2.8114573589663704e-15f, -1.0462084739763658e-22f);         /* 1/17! */
  p = dfl_sub(dfl_make(7.647163609812713e-13f, 1.2200710471178288e-20f), dfl_mul(p, z));   /* 1/15! */
  p = dfl_sub(dfl_make(1.6059044372074283e-10f, -5.352526511562726e-18f), dfl_mul(p, z));  /* 1/13! */
  p = dfl_sub(dfl_make(2.5052107943679403e-08f, 4.4176230446483665e-16f), dfl_mul(p, z));  /* 1/11! */
  p = dfl_sub(dfl_make(2.7557318844628753e-06f, 3.793571224297229e-14f), dfl_mul(p, z));   /* 1/9! */
  p = dfl_sub(dfl_make(0.00019841270113829523f, -2.725596874933456e-12f), dfl_mul(p, z));  /* 1/7! */
  p = dfl_sub(dfl_make(0.008333333767950535f, -4.34617203337595e-10f), dfl_mul(p, z));     /* 1/5! */
  p = dfl_sub(dfl_make(0.1666666716337204f, -4.967053879312289e-09f), dfl_mul(p, z));      /* 1/3! */
  p = dfl_sub(dfl_make(1.0f, 0.0f), dfl_mul(p, z));
  return dfl_mul(p, r);
}
DFN dfl dfl_cos_kernel(dfl r) {
  const dfl z = dfl_mul(r, r);
  dfl p = dfl_make(1.5619206814541513e-16f, 1.5404471465941993e-24f);          /* 1/18! */
  p = dfl_sub(dfl_make(4.7794772561329454e-14f, 7.62544404448643e-22f), dfl_mul(p, z));    /* 1/16! */
  p = dfl_sub(dfl_make(1.147074536050896e-11f, 2.372207689231238e-19f), dfl_mul(p, z));    /* 1/14! */
  p = dfl_sub(dfl_make(2.0876755879584152e-09f, 1.1082839147459852e-16f), dfl_mul(p, z));  /* 1/12! */
  p = dfl_sub(dfl_make(2.755731998149713e-07f, -7.575112209051195e-15f), dfl_mul(p, z));   /* 1/10! */
  p = dfl_sub(dfl_make(2.4801587642286904e-05f, -3.40699609366682e-13f), dfl_mul(p, z));   /* 1/8! */
  p = dfl_sub(dfl_make(0.0013888889225199819f, -3.3631094437103215e-11f), dfl_mul(p, z));  /* 1/6! */
  p = dfl_sub(dfl_make(0.0416666679084301f, -1.2417634698280722e-09f), dfl_mul(p, z));     /* 1/4! */
  p = dfl_sub(dfl_make(0.5f, 0.0f), dfl_mul(p, z));                                         /* 1/2! */
  return dfl_sub(dfl_make(1.0f, 0.0f), dfl_mul(p, z));
}
DFN dfl dfl_sin(dfl x) {
  if (!dfl_finite(x.hi)) return dfl_make(dfl_nanf(), 0.0f);
  dfl r;
  const int q = dfl_reduce_half_pi(x, &r);
  if (q < 0) return dfl_make(dfl_nanf(), 0.0f);
  const dfl v = (q & 1) ? dfl_cos_kernel(r) : dfl_sin_kernel(r);
  return (q & 2) ? dfl_neg(v) : v;
}
DFN dfl dfl_cos(dfl x) {
  if (!dfl_finite(x.hi)) return dfl_make(dfl_nanf(), 0.0f);
  dfl r;
  const int q = dfl_reduce_half_pi(x, &r);
  if (q < 0) return dfl_make(dfl_nanf(), 0.0f);
  const dfl v = (q & 1) ? dfl_sin_kernel(r) : dfl_cos_kernel(r);
  return ((q + 1) & 2) ? dfl_neg(v) : v;
}

#endif
