// Shared device-side definitions of the GB300 fitness path.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../../include/rils_rols_gb300.h"

namespace rrd {

// Error bits a kernel may raise in the round's status word.
enum : uint32_t {
  ST_BAD_CODE = 0x1,       // unknown opcode or argument out of range
  ST_STACK = 0x2,          // spill stack over/underflow
  ST_WAIT_TIMEOUT = 0x4,   // a bounded mbarrier / flag wait ran out
  ST_TOO_LARGE = 0x8,      // candidate beyond the kernel's term limit
  ST_QR_STATE = 0x10       // a QR pass found its state inconsistent (a bug, never data)
};

// Batch of one round, resident on the device.
struct DevBatch {
  const rrg_cand* cands;
  const rrg_factor* factors;
  const uint32_t* code;
  const double* consts;
  const float* consts32;    // constants as double-floats: high parts
  const float* consts32lo;  // low parts
  int32_t n_cand, n_factors, n_code, n_consts;
};

// Resident dataset: d columns of n_pad values each (rows >= n are zero).
struct DevData {
  const double* X64;
  const float* X32;    // X as double-floats: high parts (the FP32 rounding of X)
  const float* X32lo;  // low parts
  const double* y64;
  const float* y32;    // y rounded to FP32 (high part)
  const float* y32lo;  // y - y32, rounded to FP32 (low part)
  int64_t n, n_pad;
  int32_t d;
  double ymean, sst, ysum, yy;  // mean(y), sum((y - mean)^2), sum(y), sum(y^2): FP64 sums
};

// Per-candidate scratch placement of a plain round.
struct PlainCand {
  int64_t a_col;   // first column of its factor values in the A arena (n_pad doubles per column)
  int64_t m_col;   // first column of its QR working copy (k+1 columns)
  int64_t s_off;   // offset of its stacked R blocks (TSQR only)
  int32_t k;       // OLS columns (factors + free term); 1 when untuned
  int32_t pad;
};

// Internal instructions of table programs (never in a submitted batch: the
// batch validation rejects them): read table column `arg` of the same rows.
constexpr int kOpLDT = 12;   // TOS = T[arg]
constexpr int kOpPST = 13;   // spill TOS; TOS = T[arg]
constexpr int kSrcT = 3;     // binary operand from table column `arg`

// word of the round's 16-word status block counting candidates whose QR outcome
// was decided from the table's column statistics (word 0 holds the error bits)
constexpr int kStatusSentinel = 8;
// words 10-11 of the status block: algorithmic bytes of the round's direct QRs (u64)
constexpr int kStatusQrBytes = 10;
constexpr double kEps12 = 1e-12;  // value_zero / value_one threshold (node.h:13-14)

__host__ __device__ inline int64_t round_up(int64_t a, int64_t b) { return (a + b - 1) / b * b; }

// After a kernel launch: true when it was accepted; otherwise the launch
// error is recorded as the thread's error text (rrg_last_error) and cleared,
// so the caller's own checks see it through the return value.
bool launch_ok(const char* what);

}  // namespace rrd
