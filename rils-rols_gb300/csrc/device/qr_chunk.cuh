// Column-pivoted QR least squares of the plain FP64 path over whole-GPU
// passes (qr_chunk.cu).
#pragma once
#include "common.cuh"

namespace rrd {

constexpr int kQrMaxCols = RRG_MAX_TERMS + 1;  // [factors | 1 | y]

// Per-candidate factorisation state between passes (device memory).
struct QrState {
  int32_t active;   // 1: a tuned candidate this job factorises
  int32_t k;        // OLS columns (factors + free term); y is storage column k
  int32_t size;     // steps: min(rows, k)
  int32_t nonzero;  // rank (Eigen's m_nonzero_pivots rule)
  int32_t kk;       // the step the next pass A runs
  int32_t tau_zero;  // step kk's reflector is the identity (tail below DBL_MIN)
  int32_t upd_y;     // step kk's reflector reaches y (kk < rank)
  int32_t upd_y_next;
  int32_t rec_any;   // pass B of step kk recomputes down-dated norms
  int32_t nsum;      // columns whose sums pass B forms
  int32_t sum_store[kQrMaxCols];  // their storage columns
  int32_t sum_norm[kQrMaxCols];   // 1: also the norm over rows >= kk + 1
  int32_t pos2col[kQrMaxCols];    // pivot position -> storage column
  int32_t perm[kQrMaxCols];       // pivot position -> factor column
  double nupd[kQrMaxCols], ndir[kQrMaxCols];
  double ntmp[kQrMaxCols];  // by storage column: -(v^T a + a[kk]) of step kk
  double thr_helper, tau, beta, den, rden;
  unsigned int ticket;
  int32_t pad;
};

// One factorisation job: the tuned candidates list[list_off + t] for
// t < n (n = n_list, or min(n_list, *dcount - list_off) when the device
// decided the list's length).  Candidate c's factor column j is
// factor_column(A, n_pad, pc[c].a_col, j, colmap); its k + 1 working columns
// [factors | 1 | y] are at M + pc[c].m_col * n_pad, or, when slot_cols > 0,
// at M + t * slot_cols * n_pad.  Writes the coefficients (at the candidate's
// coef_offset) and res[c].rank; candidates that are untuned or whose pc pad
// bit 0 is set are left alone.
struct QrJob {
  DevBatch b;
  DevData ds;
  const PlainCand* pc;
  const int32_t* list;
  int32_t list_off, n_list;
  const int32_t* dcount;
  const double* A;
  const int32_t* colmap;
  double* M;
  int64_t slot_cols;
  double* coefs;
  rrg_result* res;
  uint32_t* status;
  int count_bytes;  // add the algorithmic bytes to the status block
  int max_cols;     // bound on k + 1 over the job's candidates (<= kQrMaxCols)
  int max_steps;    // bound on the steps (k) over them; 0: max_cols - 1
  int nch;          // row chunks: ceil(n / RR_CHUNK)
  QrState* state;   // n_list entries
  double* part;     // n_list * (nch + 1) * max_cols chunk totals
};

// Device scratch (state and chunk totals) of a job of n_list candidates.
size_t qr_chunk_scratch_bytes(int64_t n_list, int64_t rows, int max_cols);
// Fills the job's nch, state and part from `scratch` (qr_chunk_scratch_bytes).
void qr_chunk_bind(QrJob& job, void* scratch);
// Enqueues the factorisation: one pass copying the columns and forming the
// initial norms, two passes per step (Householder vector and dot products;
// rank-1 update and the next step's sums), one solve.  `blocks`: the grid of
// every pass (persistent blocks over candidate x row-chunk items).
// Results are bit-identical to launch_plain_qr's (the same QSUM order).
bool launch_qr_chunked(const QrJob& job, int blocks, cudaStream_t st, int64_t* launches);
// Blocks of 256 threads of the pass kernels that fit on one SM.
int qr_chunk_blocks_per_sm(int max_cols);

}  // namespace rrd
