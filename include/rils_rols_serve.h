/*
 * rils_rols_gb300 - serving loop: whole fit jobs submitted as they arrive,
 * run concurrently on one GPU.
 *
 * No counterpart in the reference, whose pybind11 module runs one fit per
 * call with the GIL held (rils_rols_cpp/rils_rols_cpp.cpp:998-1007).  Each
 * job is one search of include/rils_rols_host.h (the reference's
 * rils_rols::fit, rils_rols_cpp.cpp:717-728) with its own device context:
 * its dataset stays resident in HBM for the whole search, and its rounds run
 * on its own CUDA stream, so the rounds of the jobs in flight overlap on the
 * device (continuous batching at round granularity).  A job is admitted when
 * a slot is free and its device-memory footprint (dataset plus working
 * tables, sized from n and d) fits the server's budget.  Jobs start in
 * arrival order, except that when the head of the queue does not fit, a
 * job among the next 16 that does fit may start first, at most 8 times past
 * the same head.  A worker keeps its device context (and its scratch) from
 * job to job.  A job's result does not depend on the other jobs: the same
 * search, on the same data, in the same arithmetic.
 */
#ifndef RILS_ROLS_SERVE_H
#define RILS_ROLS_SERVE_H

#include <stdint.h>

#include "rils_rols_host.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rrs_server rrs_server;

/* The arguments of rils_rols(...) (rils_rols_cpp.cpp:646-657) and the precision of
 * include/rils_rols_gb300.h. */
typedef struct {
  int32_t classification;
  int32_t max_fit_calls;
  int32_t max_seconds;
  double complexity_penalty;
  int32_t max_complexity;
  double sample_size;
  int32_t random_state;
  int32_t precision; /* RRG_PLAIN_FP64, RRG_MIXED or RRG_MIXED_CERTIFIED */
} rrs_job_params;

/* Job states. */
enum { RRS_QUEUED = 0, RRS_RUNNING = 1, RRS_DONE = 2, RRS_FAILED = 3 };

typedef struct {
  int32_t state;          /* RRS_* */
  int32_t fit_calls;      /* get_fit_calls */
  double queued_s;        /* submission to admission */
  double run_s;           /* admission to model */
  double time_to_model_s; /* submission to model */
  double best_time;       /* get_best_time */
  int64_t footprint_bytes;
  int64_t device_rounds;  /* batched device rounds of the search */
  int64_t candidates;     /* candidates scored */
} rrs_job_info;

typedef struct {
  int64_t submitted, done, failed, running, queued;
  double p50_time_to_model_s, p99_time_to_model_s, mean_time_to_model_s;
  double wall_s;          /* first submission to last completion */
  int64_t candidates;     /* scored by finished jobs */
  int64_t peak_running;   /* most jobs in flight at once */
} rrs_stats;

/* memory_budget_bytes: device memory the jobs in flight may hold together
 * (0: 80% of the free memory); max_active: jobs in flight at most. */
rrs_server* rrs_create(int32_t device, int64_t memory_budget_bytes, int32_t max_active);
/* Waits for the jobs in flight, drops the queued ones. */
void rrs_destroy(rrs_server* s);
/* Fitness backend of the jobs (NULL: the device path); tests run the loop
 * on a CPU backend.  Set before the first submission. */
int32_t rrs_set_backend(rrs_server* s, const rrh_backend* be);

/* Copies X (row-major n x d) and y; returns the job id (>= 0) or a negated
 * rrg_status. */
int64_t rrs_submit(rrs_server* s, const double* X_rowmajor, const double* y, int32_t n, int32_t d,
                   const rrs_job_params* params);
/* RRG_OK once the job finished (done or failed), RRG_E_TIMEOUT otherwise
 * (timeout_ms < 0: no limit). */
int32_t rrs_wait(rrs_server* s, int64_t job, int32_t timeout_ms);
/* Model string (get_model_string) of a finished job; returns its length or the
 * negated capacity needed; info may be NULL. */
int32_t rrs_result(rrs_server* s, int64_t job, char* model, int32_t cap, rrs_job_info* info);
int32_t rrs_stats_get(rrs_server* s, rrs_stats* out);
const char* rrs_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
