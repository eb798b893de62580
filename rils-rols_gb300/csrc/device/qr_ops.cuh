// Device helpers shared by the FP64 QR kernels (plain.cu, qr_cluster.cu).
#pragma once
#include <cstdint>

#include "common.cuh"

namespace rrd {

// Column j of candidate factor values: contiguous columns from a_col, or
// through the column map (shared factor table) when one is given.
__device__ __forceinline__ const double* factor_column(const double* A, int64_t n_pad, int64_t a_col, int j,
                                                       const int32_t* colmap) {
  return A + (colmap ? (int64_t)colmap[a_col + j] : a_col + j) * n_pad;
}

// a / b correctly rounded (the value of __ddiv_rn), for many a and one b,
// with y = RN(1 / b): q0 = RN(a y), Markstein's correction
// q1 = RN(q0 + (a - q0 b) y), and q1 is accepted when its exact remainder
// a - q1 b (one FMA) is below half an ulp of q1 times |b| in magnitude,
// which makes q1 the correctly rounded quotient.  A power-of-two q1 (whose
// lower neighbour is closer than half an ulp), a q1 outside the normal range
// and a bound outside the normal range take __ddiv_rn.
__device__ __forceinline__ double div_by(double a, double b, double y) {
  const double q0 = __dmul_rn(a, y);
  const double r = __fma_rn(-q0, b, a);
  const double q1 = __fma_rn(r, y, q0);
  const double r1 = __fma_rn(-q1, b, a);
  const long long qb = __double_as_longlong(q1);
  const int e = (int)((qb >> 52) & 0x7ff);
  const long long bb = __double_as_longlong(b) & 0x7fffffffffffffffll;
  const int eb = (int)(bb >> 52);
  const int el = eb + e - 1023 - 53;  // biased exponent of |b| * 2^(E(q1) - 53)
  if (e > 54 && e < 2045 && (qb & 0x000fffffffffffffll) != 0 && el > 1 && el < 2046) {
    // |r1| < lim on the bit patterns (both non-negative; a NaN r1 compares above)
    const long long lim = bb + ((long long)(e - 1023 - 53) << 52);
    if ((__double_as_longlong(r1) & 0x7fffffffffffffffll) < lim) return q1;
  }
  return __ddiv_rn(a, b);
}

}  // namespace rrd
