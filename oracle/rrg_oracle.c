/*
 * ORACLE - test infrastructure only.  Only tests/, __graft_entry__.smoke() and
 * the CPU-baseline leg of bench.py may load this file's library; the product
 * path never does.
 *
 * A CPU restatement, in plain C99, of the reference's fitness path for one
 * candidate, consuming the same batch format as the device C ABI
 * (include/rils_rols_gb300.h):
 *   - factor evaluation: node::evaluate_all / evaluate_inner
 *       (rils_rols_cpp/node.cpp:5-95), element-wise FP64 (exp, log, sin, cos,
 *       pow from rils-rols_gb300/csrc/common/rr_math.h);
 *   - the OLS refit of tune_constants: A = [factor_1 .. factor_m, 1],
 *       coefs = A.colPivHouseholderQr().solve(y)  (rils_rols_cpp.cpp:474-484),
 *       by oracle/colpiv_qr.h;
 *   - the rebuilt sum with the drop / snap rules (rils_rols_cpp.cpp:488-517);
 *   - fitness: R2, RMSE and the NaN sentinel (rils_rols_cpp.cpp:40-49, 520-541),
 *       every sum in the fixed CSUM order of csrc/common/rr_sum.h.
 * The decoded programs are checked against the compiled reference through
 * the golden vectors in tests/golden/ (tree in -> fitness out).
 *
 * Exports the four functions of an rrh_backend (include/rils_rols_host.h) so
 * that the host search driver can run against it in tests, and a threaded
 * batch entry point for the CPU baseline.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/rils_rols_gb300.h"
#include "../rils-rols_gb300/csrc/common/rr_math.h"
#include "../rils-rols_gb300/csrc/common/rr_sum.h"
#include "colpiv_qr.h"

typedef struct {
  double* X; /* d columns of n */
  double* y;
  int64_t n;
  int32_t d;
} oracle_dataset;

static const double kEps = 1e-12; /* pow(10, -12), node.h:14 */

void* oracle_dataset_create(void* self, const double* X_col, const double* y, int64_t n, int32_t d) {
  (void)self;
  if (n <= 0 || d < 0) return NULL;
  oracle_dataset* ds = (oracle_dataset*)calloc(1, sizeof *ds);
  if (!ds) return NULL;
  ds->X = (double*)malloc(sizeof(double) * (size_t)(d > 0 ? d : 1) * (size_t)n);
  ds->y = (double*)malloc(sizeof(double) * (size_t)n);
  if (!ds->X || !ds->y) {
    free(ds->X);
    free(ds->y);
    free(ds);
    return NULL;
  }
  memcpy(ds->X, X_col, sizeof(double) * (size_t)d * (size_t)n);
  memcpy(ds->y, y, sizeof(double) * (size_t)n);
  ds->n = n;
  ds->d = d;
  return ds;
}

void oracle_dataset_destroy(void* p) {
  oracle_dataset* ds = (oracle_dataset*)p;
  if (!ds) return;
  free(ds->X);
  free(ds->y);
  free(ds);
}

/* binary operator of node.cpp:33-90 on (left, right) */
static double bin_op(int base, double a, double b) {
  switch (base) {
    case RRG_ADD: return a + b;
    case RRG_SUB: return a - b;
    case RRG_MUL: return a * b;
    case RRG_DIV: return a / b;
    case RRG_POW: return rr_pow(a, b);
    case RRG_LT: return a < b ? 1 : 0;
    case RRG_EQ: return a == b ? 1 : 0;
    case RRG_NE: return a != b ? 1 : 0;
    case RRG_MIN: return a < b ? a : b;
    case RRG_MAX: return a > b ? a : b;
    default: return NAN;
  }
}

/* Runs the code of one candidate on row `r`, writing one value per factor
 * slot.  Returns 0, or -1 on malformed code. */
static int run_row(const oracle_dataset* ds, const rrg_batch* b, const rrg_cand* c, int64_t r, double* fv) {
  double st[RRG_MAX_STACK + 1];
  int sp = 0;
  double tos = 0.0;
  const uint32_t* code = b->code + c->code_offset;
  for (int32_t pc = 0; pc < c->code_len; ++pc) {
    const uint32_t w = code[pc];
    const int op = (int)(w & 0xffu);
    const uint32_t arg = w >> 8;
    switch (op) {
      case RRG_OP_LDV: tos = ds->X[(size_t)arg * (size_t)ds->n + (size_t)r]; break;
      case RRG_OP_LDC: tos = b->consts[arg]; break;
      case RRG_OP_PSV:
        if (sp >= RRG_MAX_STACK) return -1;
        st[sp++] = tos;
        tos = ds->X[(size_t)arg * (size_t)ds->n + (size_t)r];
        break;
      case RRG_OP_PSC:
        if (sp >= RRG_MAX_STACK) return -1;
        st[sp++] = tos;
        tos = b->consts[arg];
        break;
      case RRG_OP_SIN: tos = rr_sin(tos); break;
      case RRG_OP_COS: tos = rr_cos(tos); break;
      case RRG_OP_LN: tos = rr_log(tos); break;
      case RRG_OP_EXP: tos = rr_exp(tos); break;
      case RRG_OP_SQRT: tos = sqrt(tos); break;
      case RRG_OP_SQR: tos = tos * tos; break;
      case RRG_OP_EMIT:
        fv[arg] = tos;
        sp = 0;
        break;
      default: {
        if (op < RRG_OP_BIN) return -1;
        const int k = op - RRG_OP_BIN;
        const int base = k / 8, src = (k % 8) / 2, dir = k % 2;
        if (base >= RRG_N_BASE) return -1;
        double other;
        if (src == RRG_SRC_S) {
          if (sp <= 0) return -1;
          other = st[--sp];
        } else if (src == RRG_SRC_V) {
          other = ds->X[(size_t)arg * (size_t)ds->n + (size_t)r];
        } else {
          other = b->consts[arg];
        }
        tos = dir == RRG_DIR_N ? bin_op(base, other, tos) : bin_op(base, tos, other);
      }
    }
  }
  return 0;
}

/* Scores candidate `ci`; `A` has room for n * (RRG_MAX_TERMS) doubles,
 * `work` for rrq_work_size(n, RRG_MAX_TERMS), `yp` for n. */
static int score_one(const oracle_dataset* ds, const rrg_batch* b, int ci, rrg_result* res, double* coefs, double* A,
                     double* work, double* yp) {
  const rrg_cand* c = &b->cands[ci];
  const int64_t n = ds->n;
  const int m = c->n_factors;
  const int tuned = c->mode == RRG_TUNED;
  const int k = tuned ? m + 1 : 1;
  double fv[RRG_MAX_TERMS];
  memset(res, 0, sizeof *res);
  if (k > RRG_MAX_TERMS || c->stack_need > RRG_MAX_STACK) {
    res->flags = RRG_F_TOO_LARGE;
    return -1;
  }
  for (int64_t r = 0; r < n; ++r) {
    if (run_row(ds, b, c, r, fv) != 0) return -1;
    for (int i = 0; i < m; ++i) A[(size_t)i * (size_t)n + (size_t)r] = fv[i];
  }
  int size = 0;
  if (tuned) {
    double* cf = coefs + c->coef_offset;
    for (int64_t r = 0; r < n; ++r) A[(size_t)m * (size_t)n + (size_t)r] = 1.0; /* free term */
    const long rank = rrq_lstsq(A, (long)n, (long)n, (long)k, ds->y, cf, work);
    /* the QR overwrote A: evaluate the factors again for the rebuilt sum */
    for (int64_t r = 0; r < n; ++r) {
      run_row(ds, b, c, r, fv);
      double acc = 0.0;
      int have = 0;
      for (int i = 0; i < k; ++i) {
        const double ci_ = cf[i];
        if (fabs(ci_) < kEps) continue;
        double term;
        if (i == m) term = ci_ * 1.0;
        else if (fabs(ci_ - 1) < kEps) term = fv[i];
        else term = ci_ * fv[i];
        acc = have ? acc + term : term;
        have = 1;
      }
      yp[r] = have ? acc : 0.0;
    }
    int kept = 0;
    for (int i = 0; i < k; ++i) {
      const double ci_ = cf[i];
      if (fabs(ci_) < kEps) continue;
      ++kept;
      if (i == m) size += 1;
      else if (fabs(ci_ - 1) < kEps) size += b->factors[c->first_factor + i].n_nodes;
      else size += 2 + b->factors[c->first_factor + i].n_nodes;
    }
    size = kept == 0 ? 1 : size + kept - 1;
    res->rank = (int32_t)rank;
    res->n_coef = k;
    if (rank < k) res->flags |= RRG_F_RANK_DEFICIENT;
  } else {
    for (int64_t r = 0; r < n; ++r) yp[r] = A[r];
    size = b->factors[c->first_factor].n_nodes;
  }
  /* R2 and RMSE, rils_rols_cpp.cpp:40-49 */
  const double ymean = rr_csum(ds->y, (long)n) / (double)n;
  rr_csum_acc acc;
  rr_csum_init(&acc);
  for (int64_t r = 0; r < n; ++r) {
    const double e = ds->y[r] - yp[r];
    rr_csum_add(&acc, e * e);
  }
  const double ssr = rr_csum_total(&acc);
  rr_csum_init(&acc);
  for (int64_t r = 0; r < n; ++r) {
    const double e = ds->y[r] - ymean;
    rr_csum_add(&acc, e * e);
  }
  const double sst = rr_csum_total(&acc);
  const double r2 = 1 - ssr / sst;
  const double rmse = sqrt(ssr / (double)n);
  if (r2 != r2 || rmse != rmse) {
    res->loss = 1000;
    res->rmse = 1000;
    res->size = 1000;
    res->flags |= RRG_F_NONFINITE;
  } else {
    res->loss = 1 - r2;
    res->rmse = rmse;
    res->size = size;
  }
  return 0;
}

typedef struct {
  const oracle_dataset* ds;
  const rrg_batch* b;
  rrg_result* res;
  double* coefs;
  int first, step, status;
} job_t;

static void* run_job(void* p) {
  job_t* j = (job_t*)p;
  const int64_t n = j->ds->n;
  double* A = (double*)malloc(sizeof(double) * (size_t)n * RRG_MAX_TERMS);
  double* work = (double*)malloc(sizeof(double) * (size_t)rrq_work_size(n, RRG_MAX_TERMS));
  double* yp = (double*)malloc(sizeof(double) * (size_t)n);
  if (!A || !work || !yp) {
    j->status = RRG_E_OOM;
  } else {
    for (int ci = j->first; ci < j->b->n_cand; ci += j->step)
      if (score_one(j->ds, j->b, ci, &j->res[ci], j->coefs, A, work, yp) != 0) j->status = RRG_E_INVALID;
  }
  free(A);
  free(work);
  free(yp);
  return NULL;
}

/* Scores every candidate of the batch with `threads` threads (candidates
 * interleaved over threads; results do not depend on the thread count). */
int32_t oracle_eval_threads(void* p, const rrg_batch* b, rrg_result* res, double* coefs, int32_t threads) {
  const oracle_dataset* ds = (const oracle_dataset*)p;
  if (!ds || !b || !res) return RRG_E_INVALID;
  if (threads < 1) threads = 1;
  if (threads > b->n_cand) threads = b->n_cand > 0 ? b->n_cand : 1;
  job_t* jobs = (job_t*)calloc((size_t)threads, sizeof(job_t));
  pthread_t* tids = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
  if (!jobs || !tids) {
    free(jobs);
    free(tids);
    return RRG_E_OOM;
  }
  for (int t = 0; t < threads; ++t) {
    jobs[t] = (job_t){ds, b, res, coefs, t, threads, RRG_OK};
    if (t > 0) pthread_create(&tids[t], NULL, run_job, &jobs[t]);
  }
  run_job(&jobs[0]);
  int32_t st = jobs[0].status;
  for (int t = 1; t < threads; ++t) {
    pthread_join(tids[t], NULL);
    if (jobs[t].status != RRG_OK) st = jobs[t].status;
  }
  free(jobs);
  free(tids);
  return st;
}

/* rrh_backend.eval; `precision` is ignored (the oracle is always FP64). */
int32_t oracle_eval(void* p, const rrg_batch* b, int32_t precision, rrg_result* res, double* coefs) {
  (void)precision;
  return oracle_eval_threads(p, b, res, coefs, 1);
}

/* rrh_backend.predict: values of candidate 0 on every row. */
int32_t oracle_predict(void* p, const rrg_batch* b, double* values) {
  const oracle_dataset* ds = (const oracle_dataset*)p;
  if (!ds || !b || b->n_cand < 1) return RRG_E_INVALID;
  double fv[RRG_MAX_TERMS];
  for (int64_t r = 0; r < ds->n; ++r) {
    if (run_row(ds, b, &b->cands[0], r, fv) != 0) return RRG_E_INVALID;
    values[r] = fv[0];
  }
  return RRG_OK;
}
