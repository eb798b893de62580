// Operator semantics of node::evaluate_inner (node.cpp:23-95) in double-float
// arithmetic (csrc/common/df32.h): the factor-table evaluator and the probe
// share these.
#pragma once
#include <cstdint>

#include "../common/df32.h"
#include "../common/rr_math.h"
#include "common.cuh"

namespace rrd {

// heavy functions stay out of line so that the interpreters stay small
static __device__ __noinline__ dfl df_sin_call(dfl a) { return dfl_sin(a); }
static __device__ __noinline__ dfl df_cos_call(dfl a) { return dfl_cos(a); }
static __device__ __noinline__ dfl df_log_call(dfl a) { return dfl_log(a); }
static __device__ __noinline__ dfl df_exp_call(dfl a) { return dfl_exp(a); }
// pow is rare: evaluated in FP64 (the plain path's rr_pow) and rounded back
static __device__ __noinline__ dfl df_pow_call(dfl a, dfl b) {
  return dfl_from_double(rr_pow(dfl_to_double(a), dfl_to_double(b)));
}

__device__ __forceinline__ dfl df_unary(int op, dfl a) {
  switch (op) {
    case RRG_OP_SIN: return df_sin_call(a);
    case RRG_OP_COS: return df_cos_call(a);
    case RRG_OP_LN: return df_log_call(a);
    case RRG_OP_EXP: return df_exp_call(a);
    case RRG_OP_SQRT: return dfl_sqrt(a);
    default: return dfl_mul(a, a);  // RRG_OP_SQR
  }
}

// Division: the reciprocal form (dfl_div_nc) first; a zero, tiny or
// non-finite divisor or a non-finite quotient gives a non-finite leading part,
// and then the guarded dfl_div decides the row.  The two forms agree to about
// 2^-47 on finite quotients, and every evaluator (table and probe) takes the
// same form for the same row.
__device__ __forceinline__ dfl df_div(dfl a, dfl b) {
  const dfl r = dfl_div_nc(a, b);
  return dfl_finite(r.hi) ? r : dfl_div(a, b);
}

__device__ __forceinline__ dfl df_bin(int base, dfl a, dfl b) {
  switch (base) {
    case RRG_ADD: return dfl_add(a, b);
    case RRG_SUB: return dfl_sub(a, b);
    case RRG_MUL: return dfl_mul(a, b);
    case RRG_DIV: return df_div(a, b);
    case RRG_POW: return df_pow_call(a, b);
    case RRG_LT: return dfl_make(dfl_lt(a, b) ? 1.f : 0.f, 0.f);
    case RRG_EQ: return dfl_make(dfl_eq(a, b) ? 1.f : 0.f, 0.f);
    case RRG_NE: return dfl_make(dfl_eq(a, b) ? 0.f : 1.f, 0.f);
    case RRG_MIN: return dfl_lt(a, b) ? a : b;
    case RRG_MAX: return dfl_lt(b, a) ? a : b;
    default: return dfl_make(dfl_nanf(), 0.f);
  }
}

// Two rows at once (one dispatch).  Addition, subtraction, multiplication and
// squaring run without the non-finite guards first; a non-finite leading
// part means an operand or the result is not finite, and only then are the
// guarded operations (whose results are identical on finite values) run.
__device__ __forceinline__ void df_bin2(int base, dfl a0, dfl b0, dfl a1, dfl b1, dfl& r0, dfl& r1) {
  switch (base) {
    case RRG_ADD:
    case RRG_SUB:
      if (base == RRG_SUB) {
        b0 = dfl_neg(b0);
        b1 = dfl_neg(b1);
      }
      r0 = dfl_add_nc(a0, b0);
      r1 = dfl_add_nc(a1, b1);
      if (!(dfl_finite(r0.hi) && dfl_finite(r1.hi))) {
        r0 = dfl_add(a0, b0);
        r1 = dfl_add(a1, b1);
      }
      return;
    case RRG_MUL:
      r0 = dfl_mul_nc(a0, b0);
      r1 = dfl_mul_nc(a1, b1);
      if (!(dfl_finite(r0.hi) && dfl_finite(r1.hi))) {
        r0 = dfl_mul(a0, b0);
        r1 = dfl_mul(a1, b1);
      }
      return;
    case RRG_DIV:
      r0 = df_div(a0, b0);
      r1 = df_div(a1, b1);
      return;
    default:
      r0 = df_bin(base, a0, b0);
      r1 = df_bin(base, a1, b1);
  }
}

__device__ __forceinline__ void df_unary2(int op, dfl& t0, dfl& t1) {
  if (op == RRG_OP_SQR) {
    const dfl r0 = dfl_mul_nc(t0, t0), r1 = dfl_mul_nc(t1, t1);
    if (dfl_finite(r0.hi) && dfl_finite(r1.hi)) {
      t0 = r0;
      t1 = r1;
    } else {
      t0 = dfl_mul(t0, t0);
      t1 = dfl_mul(t1, t1);
    }
    return;
  }
  t0 = df_unary(op, t0);
  t1 = df_unary(op, t1);
}

// Scalar interpreter (one row) over double-float X and constants; false on
// a spill-stack violation.
__device__ inline bool eval_row_df(const uint32_t* code, int len, const float* K, const float* Klo,
                                   const DevData& ds, int64_t row, dfl& out) {
  dfl st[RRG_MAX_STACK];
  dfl tos = dfl_make(0.f, 0.f);
  int sp = 0;
  auto xval = [&](uint32_t j) {
    const int64_t i = (int64_t)j * ds.n_pad + row;
    return dfl_make(ds.X32[i], ds.X32lo[i]);
  };
  for (int pc = 0; pc < len; ++pc) {
    const uint32_t w = code[pc];
    const int op = (int)(w & 0xffu);
    const uint32_t arg = w >> 8;
    switch (op) {
      case RRG_OP_LDV: tos = xval(arg); break;
      case RRG_OP_LDC: tos = dfl_make(K[arg], Klo[arg]); break;
      case RRG_OP_PSV:
        if (sp >= RRG_MAX_STACK) return false;
        st[sp++] = tos;
        tos = xval(arg);
        break;
      case RRG_OP_PSC:
        if (sp >= RRG_MAX_STACK) return false;
        st[sp++] = tos;
        tos = dfl_make(K[arg], Klo[arg]);
        break;
      case RRG_OP_EMIT:
        out = tos;
        sp = 0;
        break;
      default:
        if (op >= RRG_OP_SIN && op <= RRG_OP_SQR) {
          tos = df_unary(op, tos);
        } else {
          const int kk = op - RRG_OP_BIN;
          const int base = kk >> 3, src = (kk & 7) >> 1, dir = kk & 1;
          dfl o;
          if (src == RRG_SRC_S) {
            if (sp <= 0) return false;
            o = st[--sp];
          } else if (src == RRG_SRC_V) {
            o = xval(arg);
          } else {
            o = dfl_make(K[arg], Klo[arg]);
          }
          tos = dir == RRG_DIR_N ? df_bin(base, o, tos) : df_bin(base, tos, o);
        }
    }
  }
  return true;
}

}  // namespace rrd
