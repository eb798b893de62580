// Deterministic block reductions (fixed shuffle tree, then warps in order).
#pragma once
#include <cuda_runtime.h>

namespace rrd {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Sum of `v` over the block; every thread gets the same value.
// `red` is shared scratch of at least blockDim.x / 32 doubles.
__device__ __forceinline__ double block_sum(double v, double* red) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  for (int i = 0; i < nw; ++i) s = __dadd_rn(s, red[i]);
  return s;
}

// Element-wise block sum of part[0..cnt) (one vector per thread).  Result in
// out[0..cnt) (shared).  `red` needs (blockDim.x/32) * cnt doubles.
__device__ __forceinline__ void block_sum_vec(const double* part, int cnt, double* red, double* out) {
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  __syncthreads();
  for (int j = 0; j < cnt; ++j) {
    double v = warp_sum(part[j]);
    if (l == 0) red[w * cnt + j] = v;
  }
  __syncthreads();
  for (int j = threadIdx.x; j < cnt; j += blockDim.x) {
    double s = 0.0;
    for (int i = 0; i < nw; ++i) s = __dadd_rn(s, red[i * cnt + j]);
    out[j] = s;
  }
  __syncthreads();
}

}  // namespace rrd
