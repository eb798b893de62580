// Kernels of the plain FP64 path (plain.cu).
#pragma once
#include "common.cuh"

namespace rrd {

constexpr int kMaxCodeSmem = 4096;  // program words staged in shared memory per block

struct ColStat;
// `list` (may be NULL) maps grid positions to candidates: candidate = list[cand0 + i].
// cst (may be NULL; one-column programs): column statistics of every
// written column, merged into cst[pc[c].a_col] (zeroed before the launch).
__global__ void plain_eval_kernel(DevBatch b, DevData ds, const PlainCand* pc, const int32_t* list, int cand0,
                                  double* A, uint32_t* status, ColStat* cst);
// colmap (may be NULL): factor column j of candidate c is column
// colmap[pc[c].a_col + j] of A (a shared factor table) instead of
// column pc[c].a_col + j.
// Column bucket (register footprint) of the QR kernel for k + 1 columns.
int plain_qr_bucket(int cols);
// One block per candidate of the launch (the whole factorisation in one
// launch; QSUM order, the bits of launch_qr_chunked); max_cols bounds k + 1.
bool launch_plain_qr(int max_cols, int grid, cudaStream_t st, DevBatch b, DevData ds, const PlainCand* pc,
                     const int32_t* list, int cand0, const double* A, double* M, double* coefs, rrg_result* res,
                     uint32_t* status, const int32_t* colmap);
// dcount (may be NULL): grid positions at or beyond *dcount do nothing (a
// list whose length the device decided; the grid covers its capacity).
__global__ void plain_resid_kernel(DevBatch b, DevData ds, const PlainCand* pc, const int32_t* list, int cand0,
                                   const double* A, const double* coefs, double* partial, const int32_t* colmap,
                                   const int32_t* dcount = nullptr);
// partial[c * nb + j]: per-candidate squared-residual partial sums; when
// sse_direct is given and sse_direct[c] >= 0 (or NaN) it is the SSE itself.
__global__ void finalize_kernel(DevBatch b, DevData ds, const int32_t* list, int cand0, int cand1,
                                const double* partial, int nb, const double* coefs, rrg_result* res,
                                uint32_t flags_or, const double* sse_direct, const int32_t* dcount = nullptr);

__global__ void clear_results_kernel(const int32_t* list, int n, rrg_result* res, const int32_t* dcount = nullptr);

// Column statistics of an FP64 table (gathered by plain_eval_kernel), for
// deciding the column-pivoted QR's outcome on non-finite data without running it.
struct ColStat {
  uint32_t flags;       // kCs* bits
  uint32_t pad;
  unsigned long long maxabs;  // bits of the largest finite |value| (non-negative doubles order as integers)
};
constexpr uint32_t kCsNaN = 1;   // a NaN value: the column's norm is NaN
constexpr uint32_t kCsBig = 2;   // an infinite value or one whose square overflows
constexpr uint32_t kCsTail = 4;  // a row after the first with |value| > 1e-150 or non-finite
// One thread per listed tuned candidate: where the QR's result is certain to
// be all-NaN coefficients at full rank (the fitness sentinel), writes that
// result, sets pc[c].pad = 1 (the QR and residual kernels skip it) and
// counts it in *decided.
// Finite columns (the free term included) of the Gram certificate for a NaN
// column beyond column 0; wider candidates are left to the QR.
constexpr int kGramCols = 9;
// grid (row blocks, listed candidates): per-block FP64 Gram sums of the finite
// columns of the candidates sentinel_classify_kernel marked (pad bit 1)
__global__ void nan_gram_kernel(const int32_t* list, int cnt, const PlainCand* pc, const int32_t* colmap,
                                const ColStat* cs, const double* T, int64_t n, int64_t n_pad, double* gpart,
                                const int32_t* dcount = nullptr);
// one thread per listed candidate: a well-conditioned Gram decides the
// all-NaN outcome (written, pad = 1); otherwise pad = 0 and the QR runs
__global__ void nan_gram_decide_kernel(DevBatch b, const int32_t* list, int cnt, PlainCand* pc, const int32_t* colmap,
                                       const ColStat* cs, int nbx, const double* gpart, double* coefs,
                                       rrg_result* res, uint32_t* decided, const int32_t* dcount = nullptr);
__global__ void sentinel_classify_kernel(DevBatch b, const int32_t* list, int cand0, int cnt, PlainCand* pc,
                                         const int32_t* colmap, const ColStat* cs, int64_t rows, double* coefs,
                                         rrg_result* res, uint32_t* decided, const int32_t* dcount = nullptr);
// Table columns listed in cols[0 .. *count) (one-column programs, pc[c].a_col
// = the column), with their column statistics into cst: a persistent grid of
// any size walks (column, row block) items, each column split into
// min(max_nbc, ceil(gridDim.x / count)) row blocks.  The values and
// statistics are those of plain_eval_kernel's one-column form.
__global__ void table_eval_list_kernel(DevBatch b, DevData ds, const PlainCand* pc, const int32_t* cols,
                                       const int32_t* count, int max_nbc, double* A, uint32_t* status, ColStat* cst);

size_t plain_eval_smem();
size_t plain_qr_smem();

}  // namespace rrd
