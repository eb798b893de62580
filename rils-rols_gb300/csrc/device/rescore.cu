// Device-side lists of a mixed round's second half (declared in rescore.cuh).
#include <algorithm>

#include "mixed.cuh"
#include "plain.cuh"
#include "rescore.cuh"

namespace rrd {

namespace {

constexpr int kScanThreads = 1024;

// Exclusive prefix of `flag` over the block; *total gets the block's sum.
__device__ __forceinline__ int block_prefix(int flag, int* warp_tot, int* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const unsigned bal = __ballot_sync(0xffffffffu, flag);
  const int in_warp = __popc(bal & ((1u << lane) - 1u));
  if (lane == 0) warp_tot[wid] = __popc(bal);
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int w = 0; w < nw; ++w) {
      const int t = warp_tot[w];
      warp_tot[w] = s;
      s += t;
    }
    *total = s;
  }
  __syncthreads();
  const int out = warp_tot[wid] + in_warp;
  __syncthreads();  // warp_tot is rewritten by the next call
  return out;
}

__global__ void __launch_bounds__(kScanThreads) pass2_compact_kernel(const int32_t* list, int32_t cnt,
                                                                     const uint8_t* pass2, int32_t* list2,
                                                                     int32_t* count2) {
  __shared__ int warp_tot[kScanThreads / 32];
  __shared__ int total;
  int base = 0;
  for (int32_t c0 = 0; c0 < cnt; c0 += kScanThreads) {
    const int32_t li = c0 + (int32_t)threadIdx.x;
    const int flag = li < cnt && pass2[list[li]] ? 1 : 0;
    const int pos = block_prefix(flag, warp_tot, &total);
    if (flag) list2[base + pos] = li;
    base += total;
  }
  if (threadIdx.x == 0) *count2 = base;
}

__global__ void rescore_mark_kernel(const rrg_cand* cands, const int32_t* fb, int32_t cap, const int32_t* li_of,
                                    const int32_t* cand_col, const int32_t* dep_off, const int32_t* deps,
                                    const int32_t* kept, uint8_t* need) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int cnt = min(fb[0], cap);
  if (i >= cnt) return;
  const int c = fb[1 + i];
  const int li = li_of[c];
  if (li < 0) return;
  const rrg_cand cd = cands[c];
  const int m = cd.mode == RRG_TUNED ? cd.n_factors : 1;
  for (int s = 0; s < m && s < kMixedMaxM; ++s) {
    const int col = cand_col[(size_t)li * kMixedMaxM + s];
    need[col] = kept && kept[col] >= 0 ? kNeedCopy : kNeedEval;
    for (int j = dep_off[col]; j < dep_off[col + 1]; ++j) need[deps[j]] = kept && kept[deps[j]] >= 0 ? kNeedCopy : kNeedEval;
  }
}

__global__ void __launch_bounds__(kScanThreads) rescore_levels_kernel(const uint8_t* need, const int32_t* level_end,
                                                                      int32_t n_levels, int32_t* cols,
                                                                      int32_t* count) {
  __shared__ int warp_tot[kScanThreads / 32];
  __shared__ int total;
  for (int L = 0; L < n_levels; ++L) {
    const int32_t lo = L == 0 ? 0 : level_end[L - 1], hi = level_end[L];
    int base = 0;
    for (int32_t c0 = lo; c0 < hi; c0 += kScanThreads) {
      const int32_t col = c0 + (int32_t)threadIdx.x;
      const int flag = col < hi && need[col] == kNeedEval ? 1 : 0;
      const int pos = block_prefix(flag, warp_tot, &total);
      if (flag) cols[lo + base + pos] = col;
      base += total;
    }
    if (threadIdx.x == 0) count[L] = base;
  }
}

__global__ void rescore_buckets_kernel(const rrg_cand* cands, const int32_t* fb, int32_t cap, const PlainCand* pc,
                                       int32_t* blist, int32_t* bcount) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int cnt = min(fb[0], cap);
  if (i >= cnt) return;
  const int c = fb[1 + i];
  if (cands[c].mode != RRG_TUNED || (pc[c].pad & 1)) return;
  const int cols = pc[c].k + 1;
  const int q = cols <= 4 ? 0 : (cols <= 8 ? 1 : (cols <= 16 ? 2 : 3));
  const int slot = atomicAdd(bcount + q, 1);
  blist[(size_t)q * cap + slot] = c;
}

// Columns marked kNeedCopy: the column and its statistics from the cache
// arena (slot kept[col]) into the table (column col).  grid (x: row blocks of
// the column, y: columns in steps of gridDim.y).
__global__ void lane_copy_kernel(const uint8_t* need, const int32_t* kept, int32_t ncol, const double* arena,
                                 const ColStat* arena_cs, double* table, ColStat* table_cs, int64_t n_pad) {
  for (int32_t col = blockIdx.y; col < ncol; col += gridDim.y) {
    if (need[col] != kNeedCopy) continue;
    const double* src = arena + (int64_t)kept[col] * n_pad;
    double* dst = table + (int64_t)col * n_pad;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n_pad; r += (int64_t)gridDim.x * blockDim.x)
      dst[r] = src[r];
    if (blockIdx.x == 0 && threadIdx.x == 0) table_cs[col] = arena_cs[kept[col]];
  }
}

// Columns of a completed round's table into cache slots: pair i copies
// table column pairs[2i] to arena slot pairs[2i + 1], with its statistics.
__global__ void cache_store_kernel(const int32_t* pairs, int32_t n_pairs, const double* table, const ColStat* table_cs,
                                   double* arena, ColStat* arena_cs, int64_t n_pad) {
  for (int32_t i = blockIdx.y; i < n_pairs; i += gridDim.y) {
    const int32_t col = pairs[2 * i], slot = pairs[2 * i + 1];
    const double* src = table + (int64_t)col * n_pad;
    double* dst = arena + (int64_t)slot * n_pad;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n_pad; r += (int64_t)gridDim.x * blockDim.x)
      dst[r] = src[r];
    if (blockIdx.x == 0 && threadIdx.x == 0) arena_cs[slot] = table_cs[col];
  }
}

}  // namespace

bool launch_lane_copy(const uint8_t* need, const int32_t* kept, int32_t ncol, const double* arena,
                      const ColStat* arena_cs, double* table, ColStat* table_cs, int64_t n_pad, cudaStream_t st) {
  if (ncol <= 0) return true;
  const dim3 grid((unsigned)std::min<int64_t>(16, (n_pad + 4095) / 4096), (unsigned)std::min(ncol, 4096));
  lane_copy_kernel<<<grid, 256, 0, st>>>(need, kept, ncol, arena, arena_cs, table, table_cs, n_pad);
  return launch_ok("launch_lane_copy");
}

bool launch_cache_store(const int32_t* pairs, int32_t n_pairs, const double* table, const ColStat* table_cs,
                        double* arena, ColStat* arena_cs, int64_t n_pad, cudaStream_t st) {
  if (n_pairs <= 0) return true;
  const dim3 grid((unsigned)std::min<int64_t>(64, (n_pad + 4095) / 4096), (unsigned)std::min(n_pairs, 4096));
  cache_store_kernel<<<grid, 256, 0, st>>>(pairs, n_pairs, table, table_cs, arena, arena_cs, n_pad);
  return launch_ok("launch_cache_store");
}

bool launch_pass2_compact(const int32_t* list, int32_t cnt, const uint8_t* pass2, int32_t* list2, int32_t* count2,
                          cudaStream_t st) {
  pass2_compact_kernel<<<1, kScanThreads, 0, st>>>(list, cnt, pass2, list2, count2);
  return launch_ok("launch_pass2_compact");
}

bool launch_rescore_mark(const rrg_cand* cands, const int32_t* fb, int32_t cap, const int32_t* li_of,
                         const int32_t* cand_col, const int32_t* dep_off, const int32_t* deps, const int32_t* kept,
                         uint8_t* need, cudaStream_t st) {
  if (cap <= 0) return true;
  rescore_mark_kernel<<<(cap + 127) / 128, 128, 0, st>>>(cands, fb, cap, li_of, cand_col, dep_off, deps, kept, need);
  return launch_ok("launch_rescore_mark");
}

bool launch_rescore_levels(const uint8_t* need, const int32_t* level_end, int32_t n_levels, int32_t* cols,
                           int32_t* count, cudaStream_t st) {
  if (n_levels <= 0) return true;
  rescore_levels_kernel<<<1, kScanThreads, 0, st>>>(need, level_end, n_levels, cols, count);
  return launch_ok("launch_rescore_levels");
}

bool launch_rescore_buckets(const rrg_cand* cands, const int32_t* fb, int32_t cap, const PlainCand* pc,
                            int32_t* blist, int32_t* bcount, cudaStream_t st) {
  if (cap <= 0) return true;
  rescore_buckets_kernel<<<(cap + 127) / 128, 128, 0, st>>>(cands, fb, cap, pc, blist, bcount);
  return launch_ok("launch_rescore_buckets");
}

}  // namespace rrd
