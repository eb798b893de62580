/*
 * rils_rols_gb300 - C ABI of the host search driver.
 *
 * Mirrors the pybind11 module `rils_rols_cpp` of the reference
 * (rils_rols_cpp/rils_rols_cpp.cpp:998-1007): one model object with the same
 * constructor arguments, fit / predict and the same getters.  The search
 * (iterated local search, rils_rols_cpp.cpp:601-859) runs on the host; every
 * fitness evaluation goes through a backend, by default the GB300 device
 * path of include/rils_rols_gb300.h, one batched call per local-search round.
 */
#ifndef RILS_ROLS_HOST_H
#define RILS_ROLS_HOST_H

#include <stdint.h>

#include "rils_rols_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Where fitness is computed.  The default backend is the device path; a
 * backend with the same signatures can be installed (tests use this to run
 * the search against a CPU restatement of the reference). */
typedef struct {
  void* self;
  void* (*dataset_create)(void* self, const double* X_col, const double* y, int64_t n, int32_t d);
  int32_t (*eval)(void* dataset, const rrg_batch* batch, int32_t precision, rrg_result* results, double* coefs);
  int32_t (*predict)(void* dataset, const rrg_batch* batch, double* values);
  void (*dataset_destroy)(void* dataset);
} rrh_backend;

typedef struct rrh_model rrh_model;

/* rils_rols(classification, max_fit_calls, max_seconds, complexity_penalty,
 *           max_complexity, sample_size, verbose, random_state)
 * rils_rols_cpp.cpp:646-657.  Returns NULL on failure (see rrh_last_error). */
rrh_model* rrh_create(int32_t classification, int32_t max_fit_calls, int32_t max_seconds,
                      double complexity_penalty, int32_t max_complexity, double sample_size, int32_t verbose,
                      int32_t random_state);
void rrh_destroy(rrh_model* m);

/* Install a backend (copied).  NULL restores the device backend. */
int32_t rrh_set_backend(rrh_model* m, const rrh_backend* be);
/* RRG_PLAIN_FP64 (default, the drop-in), RRG_MIXED_CERTIFIED (every fitness
 * within 1e-6 relative of the FP64 path's: decisions agree except between
 * candidates whose fitness values lie that close) or RRG_MIXED. */
int32_t rrh_set_precision(rrh_model* m, int32_t precision);
/* Run the device backend's rounds as CUDA graphs (rrg_context_set_graph);
 * off by default.  The same search and results either way.  No counterpart
 * in the reference. */
int32_t rrh_set_graph(rrh_model* m, int32_t on);
/* Keep factor columns across the device backend's rounds
 * (rrg_context_set_column_cache); on by default.  The same search and
 * results either way.  No counterpart in the reference. */
int32_t rrh_set_column_cache(rrh_model* m, int32_t on);

/* fit(X, y, data_cnt, feat_cnt), X row-major n x d (rils_rols_cpp.cpp:717-728).
 * Returns RRG_OK or an rrg_status; never exits the process. */
int32_t rrh_fit(rrh_model* m, const double* X_rowmajor, const double* y, int32_t n, int32_t d);
/* predict(X, data_cnt, feat_cnt) -> out[n] (rils_rols_cpp.cpp:730-750). */
int32_t rrh_predict(rrh_model* m, const double* X_rowmajor, int32_t n, int32_t d, double* out);

/* get_model_string (rils_rols_cpp.cpp:866-868); returns the length, or the
 * negated required capacity when `cap` is too small. */
int32_t rrh_model_string(const rrh_model* m, char* buf, int32_t cap);
/* The model in the prefix token form "add mul c:2.5 x0 c:1" (full precision). */
int32_t rrh_model_prefix(const rrh_model* m, char* buf, int32_t cap);
double rrh_best_time(const rrh_model* m);
double rrh_total_time(const rrh_model* m);
int32_t rrh_fit_calls(const rrh_model* m);
/* Counters beyond the reference's: [0] LS calls, [1] main-loop iterations,
 * [2] backend rounds, [3] candidates scored, [4] skipped and [5] all
 * perturbations, [6] nanoseconds spent in the fitness backend. */
int64_t rrh_counter(const rrh_model* m, int32_t which);
const char* rrh_last_error(void);

/* ---- inspection hooks on the tree IR (used by the parity tests) ---- */
/* all_candidates(tree, local_search) (rils_rols_cpp.cpp:348-443) for d features;
 * lines "<to_string>\t<prefix>\n". */
int32_t rrh_candidates(const char* tree_prefix, int32_t local_search, int32_t d, int32_t classification, char* out,
                       int32_t cap);
/* what: 0 to_string, 1 expand, 2 simplify, 3 normalize_factor_constants,
 *       4 candidate clean-up loop, 5 tune_constants factors (one per line). */
int32_t rrh_rewrite(const char* tree_prefix, int32_t what, char* out, int32_t cap);
/* Encode candidates (one prefix tree per line) into an rrg_batch held by the
 * library until the next call; mode as rrg_mode. */
int32_t rrh_encode(const char* trees, int32_t mode, rrg_batch* out);
/* Rebuild a tuned tree from its factors and coefficients; output "<to_string>\t<prefix>". */
int32_t rrh_rebuild(const char* tree_prefix, const double* coefs, int32_t n_coefs, char* out, int32_t cap);

#ifdef __cplusplus
}
#endif
#endif
