// Factor table of a mixed round (ftable.cu).
//
// The candidates of one local-search round are perturbations of the same
// model, so most of their top-level factors are shared: a round of the
// 1M-row regression search holds about six times fewer distinct factor
// programs than factor instances.  Each distinct factor is evaluated once
// in double-float arithmetic (csrc/common/df32.h) into HBM, and each
// distinct pair of factors is summed once.
#pragma once
#include <cuda.h>  // CUtensorMap: the tensor maps of the staged evaluator

#include "common.cuh"
#include "mixed.cuh"

namespace rrd {

constexpr int kFacThreads = 256;      // evaluator block: 2 or 4 rows per thread
constexpr int kFacStep = 4 * kFacThreads;
constexpr int kFacCodeSmem = 2048;    // program words of one evaluator group in shared memory
constexpr int kFacGroupMax = 64;      // factors per evaluator group
// Rows per evaluator block (a power of two, multiple of kFacStep): larger
// chunks spread each block's per-factor reductions over more rows, smaller
// ones keep the X rows that the resident blocks read within L2; about
// 24K (rows x features) per block, in [1024, 8192].  Measured per 1M-row
// round: d = 5, 2048 / 4096 / 8192 rows 56.8 / 52.4 / 51.9 ms; 100k rows,
// d = 10 (deeper programs): 92.3 / 98.1 / 110.9 ms.  It fixes the grouping
// of the self sums, so it depends on the data shape only.
inline int fac_chunk(int d) {
  int c = 8192;
  while (c > 1024 && (int64_t)c * (d + 1) > 24576) c >>= 1;
  return c;
}
constexpr int kPairThreads = 256;
constexpr int kPairBatch = 16;        // partners reduced together
constexpr int kPairRows = 4096;       // rows per pair-sum / residual block
constexpr int kResidThreads = 256;


// Staged evaluation (FacEvalArgs::stage): a block copies the rows of its
// chunk of the features its group reads, and of y, into shared memory with
// tensor copies (cp.async.bulk.tensor, boxes of kTmaRows rows of one
// feature) and evaluates from there; the same arithmetic on the same rows.
constexpr int kFacStageMax = 64;  // features one staged group may read (shared memory decides first)
constexpr int kTmaRows = 256;     // rows per tensor-copy box

// Self pairs of factor f sit at pair index 3f (f*f), 3f+1 (f*1), 3f+2 (f*y);
// cross pairs follow from 3 * n_factors.
struct FacEvalArgs {
  DevData ds;
  const uint32_t* code;      // distinct factor programs, each ending in EMIT 0
  const int2* meta;          // [f] (code offset, length)
  const int2* groups;        // [g] (first factor, count); a group's programs are contiguous
  const int32_t* wcol;       // [f] column of F (and of fnan) program f writes; NULL: column f
  const float* K;            // constant pool, double-float high parts
  const float* Klo;          // low parts
  int32_t chunk;             // rows per chunk, a multiple of kFacStep
  float2* F;                 // [column][n_pad] values (hi, lo); 0 on rows >= n.  Programs
                             // read columns of earlier levels from it
  float2* P;                 // [chunk][n_pairs] double-float partial sums
  int32_t n_pairs;
  unsigned long long* fnan;  // [column] first row with a NaN value
  uint32_t* status;
  // staging: 0 reads X and y from global memory (L2); 1 stages them.  The
  // features group g reads (of this launch's groups) are
  // gfeat[gfeat_off[g] .. gfeat_off[g + 1]), at most stage_slots of them.
  int32_t stage;
  int32_t stage_slots;
  const int32_t* gfeat_off;
  const int32_t* gfeat;
  CUtensorMap tm_xh, tm_xl, tm_yh, tm_yl;  // X hi / lo as [d][n_pad], y hi / lo as [1][n_pad]
};
// Shared memory of the staged evaluator for `slots` features of a chunk.
size_t fac_eval_smem_staged(int chunk, int slots);
// Encodes the four tensor maps of a dataset into a; false when the driver
// offers no tensor-map encoder or the layout is not copyable.
bool fac_stage_maps(FacEvalArgs& a, const DevData& ds);

struct PairArgs {
  const float2* F;
  int64_t n_pad;
  const int4* units;         // [u] (a, first cross pair, end cross pair, 0)
  int32_t n_units;
  const int32_t* partner;    // [cross pair] factor b (pairs of a unit share a)
  float2* P;                 // [row block][n_pairs]
  int32_t n_pairs, cross0;   // pair index of cross pair 0
};

struct ResidArgs {
  DevBatch b;
  DevData ds;
  const float2* F;
  const int32_t* mlist;      // mixed list: list index -> candidate
  const int32_t* list2;      // [i] list index of a candidate that needs the residual pass
  int32_t n2;                // entries of list2 the grid covers
  const int32_t* n2_dev;     // may be NULL: the device-decided length of list2 (<= n2)
  const int32_t* cand_col;   // [list index][kMixedMaxM] table column of each factor
  const MixedTerm* terms;    // [candidate]
  int32_t n_chunks;          // row blocks of pair_row_blocks(n_pad)
  double* sse;               // [candidate][row block]
};

// light: the groups' programs are short and shallow (4 rows per thread);
// otherwise 2 rows per thread
bool launch_fac_eval(const FacEvalArgs& a, int n_groups, int n_chunks, bool light, cudaStream_t st);
// The rows-per-thread class of a program (4 rows per thread when light).  A
// factor's class is taken from its own program, never from the table form
// that reads shared columns: the class fixes the order of its self sums.
inline bool fac_light(int code_len, int stack) { return stack <= 1 && code_len <= 16; }
size_t fac_eval_smem();
bool fac_allow_smem();
// Row blocks of the pair sums and the residual pass.
int pair_row_blocks(int64_t n_pad);
bool launch_pair_sum(const PairArgs& a, int n_row_blocks, cudaStream_t st);
// psum[p] for p in [p0, p1): FP64 sum over the first n_chunks rows of P.
// smap (may be NULL; self pairs): the sum of pair p goes to
// psum[3 * smap[p / 3] + p % 3] instead (program p / 3's column).
// omap (may be NULL): the sum of pair p goes to psum[omap[p]].
bool launch_pair_reduce(const float2* P, int32_t n_pairs, int32_t n_chunks, int32_t p0, int32_t p1, double* psum,
                        cudaStream_t st, const int32_t* smap = nullptr, const int32_t* omap = nullptr);
// dst[idx[i] * words + w] = v for i < n, w < words (per-slot records of a
// column arena)
bool launch_fill_slots(const int32_t* idx, int32_t n, unsigned long long* dst, int words, unsigned long long v,
                       cudaStream_t st);
// max_blocks > 0: at most that many blocks walk the items (the grid shape
// changes no result); otherwise one block per item.
bool launch_ftab_resid(const ResidArgs& a, cudaStream_t st, int max_blocks = 0);

}  // namespace rrd
