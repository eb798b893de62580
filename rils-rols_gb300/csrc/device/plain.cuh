// Kernels of the plain FP64 path (plain.cu).
#pragma once
#include "common.cuh"

namespace rrd {

constexpr int kMaxCodeSmem = 4096;  // program words staged in shared memory per block

// `list` (may be NULL) maps grid positions to candidates: candidate = list[cand0 + i].
__global__ void plain_eval_kernel(DevBatch b, DevData ds, const PlainCand* pc, const int32_t* list, int cand0,
                                  double* A, double* M, double* S, int tsqr, uint32_t* status);
// tsqr = 1: pivoted QR of the stacked slice triangles, and redo[c] = 1 when
// the candidate must be re-solved directly; tsqr = 0 with redo != NULL: only
// the flagged candidates, by the direct QR on [A | 1 | y].
__global__ void plain_qr_kernel(DevBatch b, DevData ds, const PlainCand* pc, const int32_t* list, int cand0,
                                const double* A, double* M, double* S, int tsqr, int nb, double* coefs,
                                rrg_result* res, uint32_t* status, uint8_t* redo);
__global__ void plain_resid_kernel(DevBatch b, DevData ds, const PlainCand* pc, const int32_t* list, int cand0,
                                   const double* A, const double* coefs, double* partial);
// partial[c * nb + j]: per-candidate squared-residual partial sums; when
// sse_direct is given and sse_direct[c] >= 0 (or NaN) it is the SSE itself.
__global__ void finalize_kernel(DevBatch b, DevData ds, const int32_t* list, int cand0, int cand1,
                                const double* partial, int nb, const double* coefs, rrg_result* res,
                                uint32_t flags_or, const double* sse_direct);

size_t plain_eval_smem();
size_t plain_qr_smem();

}  // namespace rrd
