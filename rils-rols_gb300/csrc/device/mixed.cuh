// Batched mixed-precision fitness path (mixed.cu).
#pragma once
#include "common.cuh"

namespace rrd {

constexpr int kMixedStackCap = 4;    // spill levels kept in shared memory per warp
constexpr int kMixedCodeCap = 128;   // program words staged per warp
constexpr int kMixedMaxM = 8;        // factors per candidate handled by the mixed kernels

// Per-candidate solve output consumed by the residual pass.
struct MixedTerm {
  float hi[16];  // coefficient as a double-float pair, k <= kMixedMaxM + 1 entries used
  float lo[16];
  int8_t kind[16];  // 0 drop, 1 free term, 2 bare factor, 3 scaled factor
};

// Why a mixed candidate was re-scored by the FP64 path (counters per round).
enum FallbackReason : int {
  FB_PROBE_NONFINITE = 0,  // FP32 non-finite where FP64 is finite (or the reverse) on a probe row
  FB_FP64_INF,             // FP64 overflow on a probe row
  FB_FP32_OVERFLOW,        // +-inf in the FP32 sums without NaN
  FB_NAN_RANK,             // NaN factor next to a rank-deficient rest
  FB_RANK,                 // rank cut
  FB_ILL_COND,             // pivot ratio below the conditioning bound
  FB_SNAP,                 // coefficient near 1 (snap rule ambiguous)
  FB_DROP,                 // coefficient near 0 (drop rule ambiguous)
  FB_ONE_PASS,             // Gram-identity SSE not accurate enough
  FB_CERT,                 // certified fitness bound above tolerance
  FB_OTHER_NAN,            // NaN outside the factor columns
  kFbReasons
};

// FP32-versus-FP64 comparison of every factor on the probe rows of a mixed
// round (mixed_probe_kernel), read by the certification in the solve.
constexpr int kProbeRows = 1024;  // every row when n <= kProbeRows
struct ProbeOut {
  float dev[kMixedMaxM];   // max |f32 - f64| over probe rows where both are finite
  float rms[kMixedMaxM];   // root mean square of f64 over those rows
  uint32_t nan64, inf64;   // factor masks: FP64 NaN / +-inf on some probe row
  uint32_t bad32;          // factor mask: FP32 non-finite where FP64 is finite, or the reverse
  uint32_t all_rows;       // 1 when every row of the dataset was probed
};

struct MixedArgs {
  DevBatch b;
  DevData ds;
  const int32_t* list;   // candidates of this launch (absolute indices)
  int32_t n_list;
  int32_t group;         // candidates per work unit
  int32_t n_tiles, tile; // row tiles
  int32_t n_units;
  float2* gram;          // [list index][tile][E] (gram pass)
  double* sse;           // [absolute candidate][tile] (residual pass)
  const MixedTerm* terms;  // [absolute candidate] (residual pass)
  uint32_t* status;
  int64_t* nanrow;         // [absolute candidate] first row with a NaN factor value (gram pass)
};

struct SolveArgs {
  DevBatch b;
  DevData ds;
  const int32_t* list;
  int32_t n_list, n_tiles, mmax;
  const float2* gram;
  double* coefs;
  MixedTerm* terms;
  rrg_result* res;
  int32_t* fallback;       // [0] count, [1..] candidates
  int32_t fallback_cap;
  double* sse1;            // [candidate] one-pass SSE, or -1 when the residual pass is needed
  uint8_t* pass2;          // [candidate] 1: run the residual pass
  const ProbeOut* probe;   // [candidate]
  uint32_t* reasons;       // [kFbReasons] counts of FP64 re-scoring reasons
  const int64_t* nanrow;   // [candidate] first row where FP32 gave a NaN factor value
  double rank_tol, fallback_tol, pass2_tol, cert_tol;
  int certify;             // 1: RRG_MIXED_CERTIFIED decisions
};

// Host launchers (mixed.cu).
bool launch_gram(int mmax, const MixedArgs& a, int grid, size_t smem, cudaStream_t st);
bool launch_resid(int mmax, const MixedArgs& a, int grid, size_t smem, cudaStream_t st);
bool launch_solve(const SolveArgs& a, cudaStream_t st);
bool launch_probe(const DevBatch& b, const DevData& ds, const int32_t* list, int32_t n_list, ProbeOut* out,
                  cudaStream_t st);
int mixed_threads(int mmax);
size_t mixed_smem(int mmax, int d, int tile, bool resid);
int mixed_gram_entries(int mmax);
bool launch_to_f32(const double* src, float* dst, int64_t n, cudaStream_t st);
bool launch_split_f32(const double* src, float* hi, float* lo, int64_t n, cudaStream_t st);

}  // namespace rrd

namespace rrd {
bool mixed_allow_smem();
}
