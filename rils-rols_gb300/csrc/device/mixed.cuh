// Mixed-precision fitness path: solve and probes (mixed.cu); the factor
// table kernels are in ftable.cu.
#pragma once
#include "common.cuh"

namespace rrd {

constexpr int kMixedStackCap = 4;    // spill levels of the double-float factor evaluator
constexpr int kMixedMaxM = 8;        // factors per candidate handled by the mixed solve

template <int MMAX>
struct GramSize {
  static constexpr int G = MMAX * (MMAX + 1) / 2;
  static constexpr int E = G + 2 * MMAX;
};
constexpr int kMixedE = GramSize<kMixedMaxM>::E;  // Gram entries per candidate in the pair map

// Per-candidate solve output consumed by the residual pass.
struct MixedTerm {
  float hi[16];  // coefficient as a double-float pair, k <= kMixedMaxM + 1 entries used
  float lo[16];
  int8_t kind[16];  // 0 drop, 1 free term, 2 bare factor, 3 scaled factor
};

// Why a mixed candidate was re-scored by the FP64 path (counters per round).
enum FallbackReason : int {
  FB_PROBE_NONFINITE = 0,  // double-float non-finite where FP64 is finite (or the reverse) on a probe row
  FB_FP64_INF,             // FP64 overflow on a probe row
  FB_FP32_OVERFLOW,        // +-inf in the double-float sums without NaN (FP32 exponent range)
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

// Double-float-versus-FP64 comparison on the probe rows, per distinct factor
// (fac_probe_kernel) and gathered per candidate (cand_probe_kernel).
constexpr int kProbeRows = 1024;  // every row when n <= kProbeRows
enum : uint32_t { FP_NAN64 = 1, FP_INF64 = 2, FP_BAD32 = 4, FP_FAIL = 8, FP_ALL_ROWS = 16 };
struct FacProbe {
  float dev;       // max |df - f64| over probe rows where both are finite
  float rms;       // root mean square of f64 over those rows
  uint32_t flags;  // FP_* bits
  uint32_t pad;
};
struct ProbeOut {
  float dev[kMixedMaxM];   // max |df - f64| over probe rows where both are finite
  float rms[kMixedMaxM];   // root mean square of f64 over those rows
  uint32_t nan64, inf64;   // factor masks: FP64 NaN / +-inf on some probe row
  uint32_t bad32;          // factor mask: double-float non-finite where FP64 is finite, or the reverse
  uint32_t all_rows;       // 1 when every row of the dataset was probed
};

struct SolveArgs {
  DevBatch b;
  DevData ds;
  const int32_t* list;     // mixed candidates (absolute indices)
  int32_t n_list;
  const int32_t* pair_of;  // [list index][kMixedE] pair index of each Gram entry, -1 for none
  const double* psum;      // [pair] FP64 sum over all rows (pair index >= 0)
  const double* pself;     // self sums by column: entry -2 - p of pair index p <= -2
  double* coefs;
  MixedTerm* terms;
  rrg_result* res;
  int32_t* fallback;       // [0] count, [1..] candidates
  int32_t fallback_cap;
  double* sse1;            // [candidate] one-pass SSE, or -1 when the residual pass is needed
  uint8_t* pass2;          // [candidate] 1: run the residual pass
  const ProbeOut* probe;   // [candidate]
  uint32_t* reasons;       // [kFbReasons] counts of FP64 re-scoring reasons
  const int64_t* nanrow;   // [candidate] first row where a factor value was NaN in the table
  double* cert_e;          // [candidate] certified rounds: per-row error bound for the residual-pass check
  double rank_tol;         // pivot cut: squared pivot below rank_tol x its column's squared norm
  double fallback_tol;     // smallest pivot ratio solved here; below it the FP64 path solves
  double pass2_tol, cert_tol;
  int certify;             // 1: RRG_MIXED_CERTIFIED decisions
};

// Host launchers (mixed.cu).
// omap (may be NULL): the record of program f goes to out[omap[f]]
bool launch_fac_probe(const uint32_t* code, const int2* meta, int32_t nf, const double* K64, const float* K32,
                      const float* K32lo, const DevData& ds, FacProbe* out, cudaStream_t st,
                      const int32_t* omap = nullptr);
// cand_fac: [list index][kMixedMaxM] factor ids of fp; fcol (may be NULL:
// the same ids): factor id -> column of fnan
bool launch_cand_probe(const rrg_cand* cands, const int32_t* list, int32_t n_list, const int32_t* cand_fac,
                       const int32_t* fcol, const FacProbe* fp, const unsigned long long* fnan, ProbeOut* out,
                       int64_t* nanrow, cudaStream_t st);
bool launch_solve(const SolveArgs& a, cudaStream_t st);
// Certified rounds: residual-pass SSE of the listed candidates against their bound.
// n2_dev (may be NULL): the device-decided length of list2 (<= n2).
bool launch_cert_resid(const int32_t* mlist, const int32_t* list2, int32_t n2, const double* sse_part, int nb,
                       const double* cert_e, const DevData& ds, double cert_tol, int32_t* fallback,
                       int32_t fallback_cap, uint32_t* reasons, cudaStream_t st, const int32_t* n2_dev = nullptr);
bool launch_to_f32(const double* src, float* dst, int64_t n, cudaStream_t st);
bool launch_split_f32(const double* src, float* hi, float* lo, int64_t n, cudaStream_t st);

}  // namespace rrd
