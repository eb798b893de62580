// ORACLE build support (test infrastructure only).
//
// Force-included (-include) by `oracle/build_ref.sh --stock`: the arithmetic
// the reference would run with a stock toolchain instead of the pinned one.
// Element-wise exp / log / sin / cos / pow are the C library's (glibc on
// this host), and every sum, dot product and norm adds its terms one after
// another in index order with separate multiplies and adds, as an
// unvectorised Eigen build does.  It takes the place of the product's
// csrc/common/rr_math.h and rr_sum.h by defining their include guards and
// functions first, so that the reference sources, the Eigen shim and
// oracle/colpiv_qr.h compile unchanged against it.  The library it makes
// (oracle/_ref/librr_ref_stock.so) measures how far the reference's results
// move under that arithmetic; nothing scores candidates with it.
#pragma once
#define RR_MATH_H
#define RR_SUM_H
#include <math.h>

#define RR_LANES 256
#define RR_CHUNK 16384

#define RRQ_UPDATE(a, b, c) ((a) * (b) + (c))

static inline double rr_sin(double x) { return sin(x); }
static inline double rr_cos(double x) { return cos(x); }
static inline double rr_log(double x) { return log(x); }
static inline double rr_exp(double x) { return exp(x); }
static inline double rr_pow(double x, double y) { return pow(x, y); }

static inline double rr_sum256(const double* x, long start, long end) {
  double s = 0.0;
  for (long i = start; i < end; ++i) s = s + x[i];
  return s;
}
static inline double rr_sumsq256(const double* x, long start, long end) {
  double s = 0.0;
  for (long i = start; i < end; ++i) {
    const double p = x[i] * x[i];
    s = s + p;
  }
  return s;
}
static inline double rr_dot256(const double* a, const double* b, long start, long end) {
  double s = 0.0;
  for (long i = start; i < end; ++i) {
    const double p = a[i] * b[i];
    s = s + p;
  }
  return s;
}
static inline double rr_qsumsq(const double* x, long start, long end) { return rr_sumsq256(x, start, end); }
static inline double rr_qdot(const double* a, const double* b, long start, long end) {
  return rr_dot256(a, b, start, end);
}
typedef struct {
  double total;
} rr_csum_acc;
static inline void rr_csum_init(rr_csum_acc* a) { a->total = 0.0; }
static inline void rr_csum_add(rr_csum_acc* a, double v) { a->total = a->total + v; }
static inline double rr_csum_total(rr_csum_acc* a) { return a->total; }
static inline double rr_csum(const double* x, long n) { return rr_sum256(x, 0, n); }
