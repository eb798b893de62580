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
  double rank_tol, fallback_tol, pass2_tol;
};

// Host launchers (mixed.cu).
bool launch_gram(int mmax, const MixedArgs& a, int grid, size_t smem, cudaStream_t st);
bool launch_resid(int mmax, const MixedArgs& a, int grid, size_t smem, cudaStream_t st);
bool launch_solve(const SolveArgs& a, cudaStream_t st);
int mixed_threads(int mmax);
size_t mixed_smem(int mmax, int d, int tile, bool resid);
int mixed_gram_entries(int mmax);
bool launch_to_f32(const double* src, float* dst, int64_t n, cudaStream_t st);
bool launch_split_f32(const double* src, float* hi, float* lo, int64_t n, cudaStream_t st);

}  // namespace rrd

namespace rrd {
bool mixed_allow_smem();
}
