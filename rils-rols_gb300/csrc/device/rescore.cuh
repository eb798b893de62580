// Device-side bookkeeping of a mixed round's second half (rescore.cu): the
// list of candidates that need the residual pass and the FP64 re-scoring
// lane (which table columns to evaluate, which QR bucket each re-scored
// candidate falls in) are decided on the device from the solve's flags, so
// that a round needs no read-back before its results.
#pragma once
#include "common.cuh"

namespace rrd {

// QR column buckets of the re-scoring lane, as plain_qr_bucket: 4, 8, 16, RRG_MAX_TERMS + 1.
constexpr int kQrBuckets = 4;

// list2[0 .. *count2): the list positions li (ascending) of the mixed list
// whose candidate list[li] has pass2[list[li]] set.  One block.
bool launch_pass2_compact(const int32_t* list, int32_t cnt, const uint8_t* pass2, int32_t* list2, int32_t* count2,
                          cudaStream_t st);

// need[col] for every table column that the candidates fb[1 .. 1 + fb[0])
// read: their factor columns (cand_col[li_of[c] * kMixedMaxM + s]) and the
// shared-subexpression columns those programs read (deps[dep_off[col] ..
// dep_off[col + 1])): kNeedCopy when the column cache holds it (kept[col] >=
// 0, its slot; kept may be NULL), else kNeedEval.  cap bounds fb[0].
constexpr uint8_t kNeedEval = 1, kNeedCopy = 2;
bool launch_rescore_mark(const rrg_cand* cands, const int32_t* fb, int32_t cap, const int32_t* li_of,
                         const int32_t* cand_col, const int32_t* dep_off, const int32_t* deps, const int32_t* kept,
                         uint8_t* need, cudaStream_t st);
struct ColStat;
// The kNeedCopy columns (and their statistics) from the FP64 cache arena
// (slot kept[col]) into the round's FP64 table (column col).
bool launch_lane_copy(const uint8_t* need, const int32_t* kept, int32_t ncol, const double* arena,
                      const ColStat* arena_cs, double* table, ColStat* table_cs, int64_t n_pad, cudaStream_t st);
// pairs[2i] -> pairs[2i + 1]: FP64 table columns (and statistics) of a
// completed round into cache arena slots.
bool launch_cache_store(const int32_t* pairs, int32_t n_pairs, const double* table, const ColStat* table_cs,
                        double* arena, ColStat* arena_cs, int64_t n_pad, cudaStream_t st);

// Per level L (columns [level_end[L - 1], level_end[L])): the kNeedEval columns
// in ascending order at cols[level_end[L - 1] ..], their count in count[L].
// One block.
bool launch_rescore_levels(const uint8_t* need, const int32_t* level_end, int32_t n_levels, int32_t* cols,
                           int32_t* count, cudaStream_t st);

// The tuned candidates of fb[1 .. 1 + fb[0]) whose QR still runs (pc[c].pad
// bit 0 clear) by column bucket: bucket q's candidates at blist[q * cap ..],
// their count in bcount[q] (zero before the launch).
bool launch_rescore_buckets(const rrg_cand* cands, const int32_t* fb, int32_t cap, const PlainCand* pc,
                            int32_t* blist, int32_t* bcount, cudaStream_t st);

}  // namespace rrd
