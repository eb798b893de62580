// Device-side lists of a mixed round's second half (declared in rescore.cuh).
#include "mixed.cuh"
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
                                    uint8_t* need) {
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
    need[col] = 1;
    for (int j = dep_off[col]; j < dep_off[col + 1]; ++j) need[deps[j]] = 1;
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
      const int flag = col < hi && need[col] ? 1 : 0;
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

}  // namespace

bool launch_pass2_compact(const int32_t* list, int32_t cnt, const uint8_t* pass2, int32_t* list2, int32_t* count2,
                          cudaStream_t st) {
  pass2_compact_kernel<<<1, kScanThreads, 0, st>>>(list, cnt, pass2, list2, count2);
  return launch_ok("launch_pass2_compact");
}

bool launch_rescore_mark(const rrg_cand* cands, const int32_t* fb, int32_t cap, const int32_t* li_of,
                         const int32_t* cand_col, const int32_t* dep_off, const int32_t* deps, uint8_t* need,
                         cudaStream_t st) {
  if (cap <= 0) return true;
  rescore_mark_kernel<<<(cap + 127) / 128, 128, 0, st>>>(cands, fb, cap, li_of, cand_col, dep_off, deps, need);
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
