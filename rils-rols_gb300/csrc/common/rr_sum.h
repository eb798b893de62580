/*
 * The fixed summation order of the FP64 fitness path.
 *
 * RR256: a range [start, end) is summed by 256 lanes, lane t taking elements
 * start + t, start + t + 256, ... in increasing order; each group of 32 lanes
 * is folded by halving strides (16, 8, 4, 2, 1: lane t += lane t + stride),
 * and the eight group totals are added in order starting from 0.  This is the
 * order of a 256-thread CUDA block that sums with warp shuffles and then
 * across warps, so device and host results agree bit for bit.
 * CSUM: a whole column of n rows is summed as consecutive chunks of
 * RR_CHUNK rows, each by RR256, the chunk totals added in order from 0.
 * QSUM (the sums of the column-pivoted QR): a row range [start, end) is cut
 * at the absolute row multiples of RR_CHUNK; within a chunk, lane t takes
 * the rows i with i mod 256 = t in increasing order, the lanes are folded as
 * in RR256, and the chunk totals are added in order from 0.  A range from
 * row 0 is summed exactly as CSUM sums it.  The fixed lane of every row and
 * the independent chunks let a device spread one sum over as many blocks as
 * the range has chunks.
 * Every sum, mean, dot product and norm of the plain FP64 path uses one of
 * these (host code must be built with -ffp-contract=off).  Dot products and
 * sums of squares accumulate each product with a fused multiply-add, as the
 * reference's Eigen kernels do in its -O3 -march=native build on FMA hardware.
 */
#ifndef RR_SUM_H
#define RR_SUM_H

#include <math.h>

#define RR_LANES 256
#define RR_CHUNK 16384

static inline double rrs_fold(double* p) {
  for (int w = 0; w < RR_LANES / 32; ++w) {
    double* q = p + 32 * w;
    for (int off = 16; off > 0; off >>= 1)
      for (int t = 0; t < off; ++t) q[t] = q[t] + q[t + off];
  }
  double s = 0.0;
  for (int w = 0; w < RR_LANES / 32; ++w) s = s + p[32 * w];
  return s;
}

static inline double rr_sum256(const double* x, long start, long end) {
  double p[RR_LANES] = {0};
  for (long i = start; i < end; ++i) p[(i - start) & (RR_LANES - 1)] += x[i];
  return rrs_fold(p);
}

static inline double rr_sumsq256(const double* x, long start, long end) {
  double p[RR_LANES] = {0};
  for (long i = start; i < end; ++i) {
    double* q = &p[(i - start) & (RR_LANES - 1)];
    *q = fma(x[i], x[i], *q);
  }
  return rrs_fold(p);
}

static inline double rr_dot256(const double* a, const double* b, long start, long end) {
  double p[RR_LANES] = {0};
  for (long i = start; i < end; ++i) {
    double* q = &p[(i - start) & (RR_LANES - 1)];
    *q = fma(a[i], b[i], *q);
  }
  return rrs_fold(p);
}

/* streaming CSUM: add values in row order, then rr_csum_total */
typedef struct {
  double p[RR_LANES];
  long i;
  double total;
} rr_csum_acc;

static inline void rr_csum_init(rr_csum_acc* a) {
  for (int t = 0; t < RR_LANES; ++t) a->p[t] = 0.0;
  a->i = 0;
  a->total = 0.0;
}
static inline void rr_csum_add(rr_csum_acc* a, double v) {
  a->p[a->i % RR_CHUNK & (RR_LANES - 1)] += v;
  if (++a->i % RR_CHUNK == 0) {
    a->total = a->total + rrs_fold(a->p);
    for (int t = 0; t < RR_LANES; ++t) a->p[t] = 0.0;
  }
}
static inline double rr_csum_total(rr_csum_acc* a) {
  if (a->i % RR_CHUNK != 0) {
    a->total = a->total + rrs_fold(a->p);
    for (int t = 0; t < RR_LANES; ++t) a->p[t] = 0.0;
    a->i = (a->i / RR_CHUNK + 1) * RR_CHUNK;
  }
  return a->total;
}

/* QSUM sum of squares and dot product over rows [start, end) */
static inline double rr_qsumsq(const double* x, long start, long end) {
  double total = 0.0;
  for (long c0 = (start / RR_CHUNK) * RR_CHUNK; c0 < end; c0 += RR_CHUNK) {
    const long lo = c0 > start ? c0 : start, hi = c0 + RR_CHUNK < end ? c0 + RR_CHUNK : end;
    double p[RR_LANES] = {0};
    for (long i = lo; i < hi; ++i) {
      double* q = &p[i & (RR_LANES - 1)];
      *q = fma(x[i], x[i], *q);
    }
    total = total + rrs_fold(p);
  }
  return total;
}

static inline double rr_qdot(const double* a, const double* b, long start, long end) {
  double total = 0.0;
  for (long c0 = (start / RR_CHUNK) * RR_CHUNK; c0 < end; c0 += RR_CHUNK) {
    const long lo = c0 > start ? c0 : start, hi = c0 + RR_CHUNK < end ? c0 + RR_CHUNK : end;
    double p[RR_LANES] = {0};
    for (long i = lo; i < hi; ++i) {
      double* q = &p[i & (RR_LANES - 1)];
      *q = fma(a[i], b[i], *q);
    }
    total = total + rrs_fold(p);
  }
  return total;
}

static inline double rr_csum(const double* x, long n) {
  double s = 0.0;
  for (long c = 0; c < n; c += RR_CHUNK) s = s + rr_sum256(x, c, c + RR_CHUNK < n ? c + RR_CHUNK : n);
  return s;
}

#endif
