/*
 * FP64 element-wise functions of the fitness path: exp, log, sin, cos, pow.
 *
 * One definition compiled for the host (C99 / C++, -ffp-contract=off) and for
 * the device (CUDA, every operation an explicit round-to-nearest intrinsic),
 * so that the same input gives the same bits on x86, Arm and GB300.  This is
 * what lets the FP64 device path reproduce the CPU oracle bit for bit.
 * Methods (all published; constants are mathematical constants computed for
 * this file by gen_rr_math_tables.py, rounded to double):
 *   exp  table-driven (Tang): x = (64 k' + j) ln2/64 + r with ln2/64 split in
 *        a 36-bit head and a tail (Cody & Waite), |r| <= ln2/128; e^x =
 *        2^k' 2^(j/64) (1 + p(r)), 2^(j/64) from a table of double-double
 *        values, p the Taylor polynomial of e^r - 1 to degree 6; scaling by
 *        2^k' through the exponent field;
 *   log  table-driven (Tang): x = m 2^e with m in [sqrt(1/2), sqrt(2)), c =
 *        1 + j/64 the grid point nearest m, log x = e ln2 + log c +
 *        log1p(r), r = (m - c)/c formed as r_hi + r_lo (m - c exact, r_hi =
 *        (m - c) RN(1/c), r_lo from the exact remainder), log1p by its
 *        Taylor series to degree 9; e ln2 + log c summed exactly (heads on
 *        a 2^-42 grid), the rest by Fast2Sum;
 *   sin, cos  Cody & Waite reduction by pi/2 (three-term split, FMA) for
 *        |x| < 2^20, Payne & Hanek reduction with the binary expansion of 2/pi
 *        above; Taylor polynomials of sin (to r^19) and cos (to r^20) on
 *        |r| <= pi/4 with a first-order correction for the reduced tail;
 *   pow  exp(b log|a|) with log|a| and the product b log|a| carried as
 *        double-doubles, and the sign and special-value rules of C's pow.
 * Accuracy: exp, log and pow within 1 ulp (measured 0.51), sin and cos within
 * 2 ulp (checked against 60-digit arithmetic by tests/test_rr_math_cpu.py).
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

/* ------------------------------------------------------ exp / log tables -- */
/* exp: x = k ln2/64 + r; 64/ln2, ln2/64 = C1 + C2 (C1: 36 bits) */
#define RR_EXP_INV_L64 0x1.71547652b82fep+6
#define RR_EXP_C1 0x1.62e42fefa0000p-7
#define RR_EXP_C2 0x1.cf79abc9e3b3ap-46
/* 1/n!, n = 2..6 */
#define RR_EXP_F2 0x1.0000000000000p-1
#define RR_EXP_F3 0x1.5555555555555p-3
#define RR_EXP_F4 0x1.5555555555555p-5
#define RR_EXP_F5 0x1.1111111111111p-7
#define RR_EXP_F6 0x1.6c16c16c16c17p-10
/* 2^(j/64) = hi + lo, j = 0..63 */
#define RR_EXP_TAB { \
  {0x1.0000000000000p+0, 0x0.0p+0}, \
  {0x1.02c9a3e778061p+0, -0x1.19083535b085dp-56}, \
  {0x1.059b0d3158574p+0, 0x1.d73e2a475b465p-55}, \
  {0x1.0874518759bc8p+0, 0x1.186be4bb284ffp-57}, \
  {0x1.0b5586cf9890fp+0, 0x1.8a62e4adc610bp-54}, \
  {0x1.0e3ec32d3d1a2p+0, 0x1.03a1727c57b53p-59}, \
  {0x1.11301d0125b51p+0, -0x1.6c51039449b3ap-54}, \
  {0x1.1429aaea92de0p+0, -0x1.32fbf9af1369ep-54}, \
  {0x1.172b83c7d517bp+0, -0x1.19041b9d78a76p-55}, \
  {0x1.1a35beb6fcb75p+0, 0x1.e5b4c7b4968e4p-55}, \
  {0x1.1d4873168b9aap+0, 0x1.e016e00a2643cp-54}, \
  {0x1.2063b88628cd6p+0, 0x1.dc775814a8495p-55}, \
  {0x1.2387a6e756238p+0, 0x1.9b07eb6c70573p-54}, \
  {0x1.26b4565e27cddp+0, 0x1.2bd339940e9d9p-55}, \
  {0x1.29e9df51fdee1p+0, 0x1.612e8afad1255p-55}, \
  {0x1.2d285a6e4030bp+0, 0x1.0024754db41d5p-54}, \
  {0x1.306fe0a31b715p+0, 0x1.6f46ad23182e4p-55}, \
  {0x1.33c08b26416ffp+0, 0x1.32721843659a6p-54}, \
  {0x1.371a7373aa9cbp+0, -0x1.63aeabf42eae2p-54}, \
  {0x1.3a7db34e59ff7p+0, -0x1.5e436d661f5e3p-56}, \
  {0x1.3dea64c123422p+0, 0x1.ada0911f09ebcp-55}, \
  {0x1.4160a21f72e2ap+0, -0x1.ef3691c309278p-58}, \
  {0x1.44e086061892dp+0, 0x1.89b7a04ef80d0p-59}, \
  {0x1.486a2b5c13cd0p+0, 0x1.3c1a3b69062f0p-56}, \
  {0x1.4bfdad5362a27p+0, 0x1.d4397afec42e2p-56}, \
  {0x1.4f9b2769d2ca7p+0, -0x1.4b309d25957e3p-54}, \
  {0x1.5342b569d4f82p+0, -0x1.07abe1db13cadp-55}, \
  {0x1.56f4736b527dap+0, 0x1.9bb2c011d93adp-54}, \
  {0x1.5ab07dd485429p+0, 0x1.6324c054647adp-54}, \
  {0x1.5e76f15ad2148p+0, 0x1.ba6f93080e65ep-54}, \
  {0x1.6247eb03a5585p+0, -0x1.383c17e40b497p-54}, \
  {0x1.6623882552225p+0, -0x1.bb60987591c34p-54}, \
  {0x1.6a09e667f3bcdp+0, -0x1.bdd3413b26456p-54}, \
  {0x1.6dfb23c651a2fp+0, -0x1.bbe3a683c88abp-57}, \
  {0x1.71f75e8ec5f74p+0, -0x1.16e4786887a99p-55}, \
  {0x1.75feb564267c9p+0, -0x1.0245957316dd3p-54}, \
  {0x1.7a11473eb0187p+0, -0x1.41577ee04992fp-55}, \
  {0x1.7e2f336cf4e62p+0, 0x1.05d02ba15797ep-56}, \
  {0x1.82589994cce13p+0, -0x1.d4c1dd41532d8p-54}, \
  {0x1.868d99b4492edp+0, -0x1.fc6f89bd4f6bap-54}, \
  {0x1.8ace5422aa0dbp+0, 0x1.6e9f156864b27p-54}, \
  {0x1.8f1ae99157736p+0, 0x1.5cc13a2e3976cp-55}, \
  {0x1.93737b0cdc5e5p+0, -0x1.75fc781b57ebcp-57}, \
  {0x1.97d829fde4e50p+0, -0x1.d185b7c1b85d1p-54}, \
  {0x1.9c49182a3f090p+0, 0x1.c7c46b071f2bep-56}, \
  {0x1.a0c667b5de565p+0, -0x1.359495d1cd533p-54}, \
  {0x1.a5503b23e255dp+0, -0x1.d2f6edb8d41e1p-54}, \
  {0x1.a9e6b5579fdbfp+0, 0x1.0fac90ef7fd31p-54}, \
  {0x1.ae89f995ad3adp+0, 0x1.7a1cd345dcc81p-54}, \
  {0x1.b33a2b84f15fbp+0, -0x1.2805e3084d708p-57}, \
  {0x1.b7f76f2fb5e47p+0, -0x1.5584f7e54ac3bp-56}, \
  {0x1.bcc1e904bc1d2p+0, 0x1.23dd07a2d9e84p-55}, \
  {0x1.c199bdd85529cp+0, 0x1.11065895048ddp-55}, \
  {0x1.c67f12e57d14bp+0, 0x1.2884dff483cadp-54}, \
  {0x1.cb720dcef9069p+0, 0x1.503cbd1e949dbp-56}, \
  {0x1.d072d4a07897cp+0, -0x1.cbc3743797a9cp-54}, \
  {0x1.d5818dcfba487p+0, 0x1.2ed02d75b3707p-55}, \
  {0x1.da9e603db3285p+0, 0x1.c2300696db532p-54}, \
  {0x1.dfc97337b9b5fp+0, -0x1.1a5cd4f184b5cp-54}, \
  {0x1.e502ee78b3ff6p+0, 0x1.39e8980a9cc8fp-55}, \
  {0x1.ea4afa2a490dap+0, -0x1.e9c23179c2893p-54}, \
  {0x1.efa1bee615a27p+0, 0x1.dc7f486a4b6b0p-54}, \
  {0x1.f50765b6e4540p+0, 0x1.9d3e12dd8a18bp-54}, \
  {0x1.fa7c1819e90d8p+0, 0x1.74853f3a5931ep-55}, \
}
/* log: ln2 = HI + LO (HI a multiple of 2^-42) */
#define RR_LOG_LN2_HI 0x1.62e42fefa3800p-1
#define RR_LOG_LN2_LO 0x1.ef35793c76730p-45
/* (-1)^(n+1) / n, n = 2..9 */
#define RR_LOG_P2 -0x1.0000000000000p-1
#define RR_LOG_P3 0x1.5555555555555p-2
#define RR_LOG_P4 -0x1.0000000000000p-2
#define RR_LOG_P5 0x1.999999999999ap-3
#define RR_LOG_P6 -0x1.5555555555555p-3
#define RR_LOG_P7 0x1.2492492492492p-3
#define RR_LOG_P8 -0x1.0000000000000p-3
#define RR_LOG_P9 0x1.c71c71c71c71cp-4
/* c = 1 + j/64, j = -19..27: RN(1/c), log(c) = hi + lo (hi a multiple of 2^-42) */
#define RR_LOG_TAB { \
  {0x1.6c16c16c16c17p+0, -0x1.68ac83e9c7000p-2, 0x1.7af966c548a30p-44}, \
  {0x1.642c8590b2164p+0, -0x1.522ae0738a000p-2, -0x1.ebe708164c759p-45}, \
  {0x1.5c9882b931057p+0, -0x1.3c25277333000p-2, -0x1.83b54b606bd5cp-46}, \
  {0x1.5555555555555p+0, -0x1.269621134e000p-2, 0x1.1b61f10522625p-44}, \
  {0x1.4e5e0a72f0539p+0, -0x1.1178e8227e000p-2, -0x1.1ef78ce2d07f2p-44}, \
  {0x1.47ae147ae147bp+0, -0x1.f991c6cb3c000p-3, 0x1.90d04cd7cc834p-44}, \
  {0x1.4141414141414p+0, -0x1.d1037f2656000p-3, 0x1.84a7e75b6f6e4p-47}, \
  {0x1.3b13b13b13b14p+0, -0x1.a93ed3c8ae000p-3, 0x1.8724350562169p-45}, \
  {0x1.3521cfb2b78c1p+0, -0x1.823c16551a000p-3, -0x1.e0ddb9a631e83p-46}, \
  {0x1.2f684bda12f68p+0, -0x1.5bf406b544000p-3, 0x1.27023eb68981cp-46}, \
  {0x1.29e4129e4129ep+0, -0x1.365fcb015a000p-3, 0x1.fd3a0afb9691bp-44}, \
  {0x1.2492492492492p+0, -0x1.1178e8227e000p-3, -0x1.1ef78ce2d07f2p-45}, \
  {0x1.1f7047dc11f70p+0, -0x1.da72763844000p-4, -0x1.a89401fa71733p-46}, \
  {0x1.1a7b9611a7b96p+0, -0x1.9335e5d594000p-4, -0x1.3115c3abd47dap-45}, \
  {0x1.15b1e5f75270dp+0, -0x1.4d3115d208000p-4, 0x1.53a2582f4e1efp-48}, \
  {0x1.1111111111111p+0, -0x1.08598b59e4000p-4, 0x1.7e5dd7009902cp-46}, \
  {0x1.0c9714fbcda3bp+0, -0x1.894aa149f8000p-5, -0x1.9a19a8be97661p-44}, \
  {0x1.0842108421084p+0, -0x1.0415d89e78000p-5, 0x1.dddc7f461c516p-44}, \
  {0x1.0410410410410p+0, -0x1.0205658930000p-6, -0x1.611d27c8e8417p-44}, \
  {0x1.0000000000000p+0, 0x0.0p+0, 0x0.0p+0}, \
  {0x1.f81f81f81f820p-1, 0x1.fc0a8b0fc0000p-7, 0x1.f1e7cf6d3a69cp-50}, \
  {0x1.f07c1f07c1f08p-1, 0x1.f829b0e780000p-6, 0x1.980267c7e09e4p-45}, \
  {0x1.e9131abf0b767p-1, 0x1.77458f6330000p-5, -0x1.181dce586af09p-44}, \
  {0x1.e1e1e1e1e1e1ep-1, 0x1.f0a30c0118000p-5, -0x1.d599e83368e91p-45}, \
  {0x1.dae6076b981dbp-1, 0x1.341d7961bc000p-4, 0x1.1d09299837610p-44}, \
  {0x1.d41d41d41d41dp-1, 0x1.6f0d28ae58000p-4, -0x1.4b4641b664613p-44}, \
  {0x1.cd85689039b0bp-1, 0x1.a926d3a4ac000p-4, 0x1.563650bd22a9cp-44}, \
  {0x1.c71c71c71c71cp-1, 0x1.e27076e2b0000p-4, -0x1.a342c2af0003cp-45}, \
  {0x1.c0e070381c0e0p-1, 0x1.0d77e7cd08000p-3, 0x1.cb2cd2ee2f482p-44}, \
  {0x1.bacf914c1bad0p-1, 0x1.29552f8200000p-3, -0x1.5b967f4471dfcp-44}, \
  {0x1.b4e81b4e81b4fp-1, 0x1.44d2b6ccb8000p-3, -0x1.70cc16135783cp-46}, \
  {0x1.af286bca1af28p-1, 0x1.5ff3070a7a000p-3, -0x1.8586f183bebf2p-44}, \
  {0x1.a98ef606a63bep-1, 0x1.7ab890210e000p-3, -0x1.bdb9072534a58p-45}, \
  {0x1.a41a41a41a41ap-1, 0x1.9525a9cf46000p-3, -0x1.297137d9f158fp-44}, \
  {0x1.9ec8e951033d9p-1, 0x1.af3c94e80c000p-3, -0x1.a4e633fcd9066p-52}, \
  {0x1.999999999999ap-1, 0x1.c8ff7c79aa000p-3, -0x1.7794f689f8434p-45}, \
  {0x1.948b0fcd6e9e0p-1, 0x1.e27076e2b0000p-3, -0x1.a342c2af0003cp-44}, \
  {0x1.8f9c18f9c18fap-1, 0x1.fb9186d5e4000p-3, -0x1.d572aab993c87p-47}, \
  {0x1.8acb90f6bf3aap-1, 0x1.0a324e2739000p-2, 0x1.c6bee7ef4030ep-47}, \
  {0x1.8618618618618p-1, 0x1.1675cababa000p-2, 0x1.8380e731f55c4p-44}, \
  {0x1.8181818181818p-1, 0x1.22941fbcf8000p-2, -0x1.a6976f5eb0963p-44}, \
  {0x1.7d05f417d05f4p-1, 0x1.2e8e2bae12000p-2, -0x1.67b1e99b72bd8p-45}, \
  {0x1.78a4c8178a4c8p-1, 0x1.3a64c55694000p-2, 0x1.7a71cbcd735d0p-44}, \
  {0x1.745d1745d1746p-1, 0x1.4618bc21c6000p-2, -0x1.3d82f484c84ccp-46}, \
  {0x1.702e05c0b8170p-1, 0x1.51aad872e0000p-2, -0x1.f4bd8db0a7cc1p-44}, \
  {0x1.6c16c16c16c17p-1, 0x1.5d1bdbf581000p-2, -0x1.8d6bdc9c7c238p-44}, \
  {0x1.6816816816817p-1, 0x1.686c81e9b1000p-2, 0x1.2bb110af84054p-44}, \
}

#if defined(__CUDACC__)
static __device__ const double RR_EXP_T_D[64][2] = RR_EXP_TAB;
static __device__ const double RR_LOG_T_D[47][3] = RR_LOG_TAB;
#endif
static const double RR_EXP_T_H[64][2] = RR_EXP_TAB;
static const double RR_LOG_T_H[47][3] = RR_LOG_TAB;
#if defined(__CUDA_ARCH__)
#define RR_EXP_T(j, i) RR_EXP_T_D[j][i]
#define RR_LOG_T(j, i) RR_LOG_T_D[j][i]
#else
#define RR_EXP_T(j, i) RR_EXP_T_H[j][i]
#define RR_LOG_T(j, i) RR_LOG_T_H[j][i]
#endif

/* ------------------------------------------------------------------ exp -- */
/* y * 2^k for y in [0.99, 2.02], any k, with one rounding */
RRM_FN double rrm_scale(double y, int k) {
  if (k >= -1020 && k <= 1020) return rrm_from_bits(rrm_bits(y) + ((uint64_t)(int64_t)k << 52));
  if (k > 1023) {
    y = RRM_MUL(y, rrm_pow2(1023));
    k -= 1023;
    return k > 1023 ? rrm_inf() : RRM_MUL(y, rrm_pow2(k));
  }
  if (k < -1000) return RRM_MUL(RRM_MUL(y, rrm_pow2(k + 1000)), rrm_pow2(-1000));
  return RRM_MUL(y, rrm_pow2(k));
}

/* e^(x + xl) for |x| <= 745.2, xl a small correction used when has_lo */
RRM_FN double rrm_exp_core(double x, double xl, int has_lo) {
  /* kd = nearest integer to 64 x / ln2, read back from the low bits of the shifted sum */
  const double t = RRM_FMA(x, RR_EXP_INV_L64, 0x1.8p52);
  const int kd = (int)(int32_t)(uint32_t)rrm_bits(t);
  const double kdd = RRM_SUB(t, 0x1.8p52);
  double r = RRM_FMA(-kdd, RR_EXP_C1, x);
  r = RRM_FMA(-kdd, RR_EXP_C2, r);
  if (has_lo) r = RRM_ADD(r, xl);
  /* e^r - 1 = r + r^2 (1/2 + r/6 + r^2/24 + r^3/120 + r^4/720) */
  double q = RRM_FMA(r, RR_EXP_F6, RR_EXP_F5);
  q = RRM_FMA(q, r, RR_EXP_F4);
  q = RRM_FMA(q, r, RR_EXP_F3);
  q = RRM_FMA(q, r, RR_EXP_F2);
  const double p = RRM_FMA(RRM_MUL(r, r), q, r);
  const int j = kd & 63;
  const double th = RR_EXP_T(j, 0), tl = RR_EXP_T(j, 1);
  const double y = RRM_ADD(th, RRM_FMA(th, p, tl));
  return rrm_scale(y, (kd - j) / 64);
}

RRM_FN double rr_exp(double x) {
  if ((rrm_bits(x) & 0x7fffffffffffffffull) >= 0x4086200000000000ull) { /* |x| >= 708, inf or NaN */
    if (rrm_isnan(x)) return x;
    if (x > 0x1.62e42fefa39efp+9) return rrm_inf(); /* > log(DBL_MAX) */
    if (x < -0x1.74910d52d3052p+9) return 0.0;      /* < log of the least subnormal / 2 */
  }
  return rrm_exp_core(x, 0.0, 0);
}

/* ------------------------------------------------------------------ log -- */
/* log x = s + u for a positive normal x with its bits b and exponent offset e0
 * (|u| well below |s| unless s = 0) */
RRM_FN void rrm_log_parts(uint64_t b, int e0, double* s_out, double* u_out) {
  const uint64_t mant = b & 0x000fffffffffffffull;
  int e = e0 + (int)(b >> 52) - 1023;
  int j;
  double m;
  if (mant > 0x6a09e667f3bccull) { /* 1.mant > sqrt(2): m = 1.mant / 2 */
    m = rrm_from_bits(mant | 0x3fe0000000000000ull);
    e += 1;
    j = (int)((mant + (1ull << 46)) >> 47) - 32;
  } else {
    m = rrm_from_bits(mant | 0x3ff0000000000000ull);
    j = (int)((mant + (1ull << 45)) >> 46);
  }
  const double c = 1.0 + (double)j * 0x1p-6;
  const double invc = RR_LOG_T(j + 19, 0);
  const double f = RRM_SUB(m, c); /* exact */
  const double rh = RRM_MUL(f, invc);
  const double rl = RRM_MUL(RRM_FMA(-rh, c, f), invc);
  /* log1p(r) - r = r^2 (-1/2 + r/3 - r^2/4 + ... + r^7/9) */
  double q = RRM_FMA(rh, RR_LOG_P9, RR_LOG_P8);
  q = RRM_FMA(q, rh, RR_LOG_P7);
  q = RRM_FMA(q, rh, RR_LOG_P6);
  q = RRM_FMA(q, rh, RR_LOG_P5);
  q = RRM_FMA(q, rh, RR_LOG_P4);
  q = RRM_FMA(q, rh, RR_LOG_P3);
  q = RRM_FMA(q, rh, RR_LOG_P2);
  const double tail = RRM_FMA(RRM_MUL(rh, rh), q, rl);
  const double ed = (double)e;
  const double a = RRM_FMA(ed, RR_LOG_LN2_HI, RR_LOG_T(j + 19, 1)); /* exact */
  const double b0 = RRM_FMA(ed, RR_LOG_LN2_LO, RR_LOG_T(j + 19, 2));
  const double s = RRM_ADD(a, rh);
  const double t = RRM_ADD(RRM_SUB(a, s), rh); /* |a| >= |rh| or a = 0 */
  *s_out = s;
  *u_out = RRM_ADD(RRM_ADD(t, tail), b0);
}

RRM_FN double rr_log(double x) {
  uint64_t b = rrm_bits(x);
  int e0 = 0;
  if (b - 0x0010000000000000ull >= 0x7fe0000000000000ull) { /* not a positive normal number */
    if (rrm_isnan(x)) return x;
    if (x < 0.0) return rrm_nan();
    if (x == 0.0) return -rrm_inf();
    if (x > 0x1.fffffffffffffp+1023) return x; /* +inf */
    b = rrm_bits(RRM_MUL(x, 0x1p54));          /* subnormal */
    e0 = -54;
  }
  double s, u;
  rrm_log_parts(b, e0, &s, &u);
  return RRM_ADD(s, u);
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
  if (rrm_isnan(x) || x == 0.0) return x; /* sin(-0) = -0 */
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
  /* e^(b log|a|) with log|a| and the product carried as double-doubles */
  uint64_t bits = rrm_bits(ab);
  int e0 = 0;
  if (bits < 0x0010000000000000ull) { /* subnormal */
    bits = rrm_bits(RRM_MUL(ab, 0x1p54));
    e0 = -54;
  }
  double s, u;
  rrm_log_parts(bits, e0, &s, &u);
  const double lh = RRM_ADD(s, u);
  const double ll = RRM_ADD(RRM_SUB(s, lh), u);
  const double yh = RRM_MUL(b, lh);
  const double yl = RRM_FMA(b, ll, RRM_FMA(b, lh, -yh));
  if (rrm_isnan(yh)) return rrm_nan();
  if (yh > 0x1.62e42fefa39efp+9) return sign * rrm_inf();
  if (yh < -0x1.74910d52d3052p+9) return sign * 0.0;
  return sign * rrm_exp_core(yh, yl, 1);
}

#endif
