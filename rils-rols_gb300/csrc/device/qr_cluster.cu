// Direct column-pivoted QR of the plain FP64 path on 8-CTA clusters: the
// factorisation of ColPivHouseholderQR::computeInPlace
// (eigen/Eigen/src/QR/ColPivHouseholderQR.h:482-575) and the least-squares
// solve (:577-608) with makeHouseholder / applyHouseholderOnTheLeft
// (eigen/Eigen/src/Householder/Householder.h:67-133) semantics, every sum in
// the RR256 order of csrc/common/rr_sum.h.  Built for several warps-per-CTA
// shapes per column bucket; all give the same bits, the launch-shape tuner
// picks one.
#include <cooperative_groups.h>

#include <cfloat>
#include <cstdint>

#include "../common/error.h"
#include "../common/rr_sum.h"
#include "common.cuh"
#include "plain.cuh"
#include "qr_ops.cuh"
#include "reduce.cuh"

namespace rrd {

namespace {

constexpr int kMaxK = RRG_MAX_TERMS;

// ------------------------------------------------- cluster-wide direct QR --
// The same factorisation as plain_qr_kernel_t (direct, tsqr = 0), with the
// 256 lanes of every RR256 sum spread over a cluster of kQrCluster CTAs:
// CTA w runs lanes 32w .. 32w + 31.  A CTA has W warps over the same 32
// lanes; the columns of a pass are dealt to them (offset j to warp j mod W),
// so each column's lane sums are formed by one warp exactly as in the
// one-block kernel.  Each warp folds its columns and sends the totals to
// every CTA of the cluster through distributed shared memory; after the
// cluster barrier every CTA adds the eight totals of a column in order, so
// every sum is bit-identical to the one-block kernel's.  The scalar
// bookkeeping (norms, pivots, permutation) is replicated in every CTA from
// identical inputs; row kk of the working columns (the R entries) is written
// by CTA 0 only, after every CTA has read the old values.  A lane touches
// the rows kk + 1 + lane + 256 t within one step, which shift by one row per
// step, so a cluster barrier closes each step; working-column loads bypass
// L1 (ld.global.cg) since other SMs of the cluster wrote them.
namespace cg = cooperative_groups;
constexpr int kQrCluster = 8;

template <int KB>
struct ClRed {
  double buf[2][kQrCluster * KB];
  int parity;
};

// RR256 sums of the columns a warp holds: slot s of warp wi is column
// offset j = wi + s W (j < cnt); every lane of the warp gets out[s].
template <int KB, int W, int CPW>
__device__ __forceinline__ void cl_sum_cols(cg::cluster_group& cl, ClRed<KB>& r, const double (&part)[CPW], int cnt,
                                            double (&out)[CPW]) {
  const int w = (int)cl.block_rank(), lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
  double* buf = r.buf[r.parity];
#pragma unroll
  for (int s = 0; s < CPW; ++s) {
    const int j = wi + s * W;
    if (j < cnt) {
      const double v = __shfl_sync(0xffffffffu, warp_sum(part[s]), 0);  // lane 0's fold is the RR256 one
      if (lane < kQrCluster) cl.map_shared_rank(buf, lane)[w * KB + j] = v;
    }
  }
  cl.sync();
#pragma unroll
  for (int s = 0; s < CPW; ++s) {
    const int j = wi + s * W;
    double t = 0.0;
    if (j < cnt)
      for (int i = 0; i < kQrCluster; ++i) t = __dadd_rn(t, buf[i * KB + j]);
    out[s] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) r.parity ^= 1;
  __syncthreads();
}

// One RR256 sum formed by warp 0 (the other warps pass 0 and only take part
// in the barrier); every thread gets the total.
template <int KB, int W, int CPW>
__device__ __forceinline__ double cl_sum1(cg::cluster_group& cl, ClRed<KB>& r, double v) {
  double part[CPW], out[CPW];
#pragma unroll
  for (int s = 0; s < CPW; ++s) part[s] = s == 0 ? v : 0.0;
  cl_sum_cols<KB, W, CPW>(cl, r, part, 1, out);
  __shared__ double tot;
  if (threadIdx.x == 0) tot = out[0];
  __syncthreads();
  const double t = tot;
  __syncthreads();
  return t;
}

// One lane's share of an RR256 sum of squares over rows i0, i0 + 256, ...
// (in row order), with the loads of kRowBatch rows issued together.
constexpr int kRowBatch = 8;
__device__ __forceinline__ double lane_sumsq(const double* col, int64_t i0, int64_t rows) {
  double ps = 0.0;
  int64_t i = i0;
  for (; i + 256 * (kRowBatch - 1) < rows; i += 256 * kRowBatch) {
    double q[kRowBatch];
#pragma unroll
    for (int u = 0; u < kRowBatch; ++u) q[u] = __ldcg(col + i + 256 * u);
#pragma unroll
    for (int u = 0; u < kRowBatch; ++u) ps = __fma_rn(q[u], q[u], ps);
  }
  for (; i < rows; i += 256) {
    const double q = __ldcg(col + i);
    ps = __fma_rn(q, q, ps);
  }
  return ps;
}

// Columns per warp and rows per batch of the dot pass for W warps per CTA.
template <int KB, int W>
struct QrShape {
  static constexpr int CPW = (KB + W - 1) / W;
  static constexpr int U = CPW <= 4 ? 8 : (CPW <= 8 ? 4 : 2);
};

// The factorisation and solve of candidate c on this cluster, in the working
// columns Q (k + 1 columns of n_pad doubles).  Every CTA of the cluster calls
// it with the same c and takes the same exits.
template <int KB, int W>
__device__ __forceinline__ void qr_cluster_one(cg::cluster_group& cl, const DevBatch& b, const DevData& ds,
                                               const PlainCand* pc, int c, const double* A, double* Q, double* coefs,
                                               rrg_result* res, uint32_t* status, const int32_t* colmap,
                                               int count_bytes) {
  constexpr int CPW = QrShape<KB, W>::CPW, U = QrShape<KB, W>::U;
  const int w = (int)cl.block_rank();
  const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
  const int L = w * 32 + lane;  // RR256 lane
  const rrg_cand cd = b.cands[c];
  // uniform over the cluster: every CTA takes the same exits
  if (cd.mode != RRG_TUNED || (pc[c].pad & 1)) return;
  const int k = pc[c].k;
  if (k + 1 > KB || k > kMaxK) {
    if (w == 0 && threadIdx.x == 0) atomicOr(status, ST_TOO_LARGE);
    return;
  }
  __shared__ ClRed<KB> red;
  __shared__ double nupd[KB], ndir[KB];
  __shared__ int perm[KB], rec[KB];
  __shared__ double* colp[KB];
  __shared__ double ntmp[KB];
  __shared__ int s_nonzero;
  if (threadIdx.x == 0) red.parity = 0;
  cl.sync();  // every CTA of the cluster running before any distributed shared memory access
  const int64_t ld = ds.n_pad, rows = ds.n;
  for (int j = threadIdx.x; j <= k; j += blockDim.x) colp[j] = Q + (int64_t)j * ld;
  __syncthreads();
  // [A | 1 | y] into the working columns (column j by warp j mod W), the
  // initial norms on the way
  double part[CPW], out[CPW];
#pragma unroll
  for (int s = 0; s < CPW; ++s) {
    part[s] = 0.0;
    const int j = wi + s * W;
    if (j > k) continue;
    double* dst = Q + (int64_t)j * ld;
    if (j < k - 1) {
      const double* src = factor_column(A, ds.n_pad, pc[c].a_col, j, colmap);
      double acc = 0.0;
      int64_t r = L;
      for (; r + 256 * (kRowBatch - 1) < rows; r += 256 * kRowBatch) {
        double v[kRowBatch];
#pragma unroll
        for (int u = 0; u < kRowBatch; ++u) v[u] = src[r + 256 * u];
#pragma unroll
        for (int u = 0; u < kRowBatch; ++u) {
          __stcg(dst + r + 256 * u, v[u]);
          acc = __fma_rn(v[u], v[u], acc);
        }
      }
      for (; r < rows; r += 256) {
        const double v = src[r];
        __stcg(dst + r, v);
        acc = __fma_rn(v, v, acc);
      }
      part[s] = acc;
    } else if (j == k - 1) {
      double acc = 0.0;
      for (int64_t r = L; r < rows; r += 256) {
        __stcg(dst + r, 1.0);
        acc = __dadd_rn(acc, 1.0);
      }
      part[s] = acc;
    } else {
      for (int64_t r = L; r < rows; r += 256) __stcg(dst + r, ds.y64[r]);
    }
  }
  cl_sum_cols<KB, W, CPW>(cl, red, part, k, out);  // its barrier also publishes the copies
  const double rows_thr = (double)ds.n;
  const int size = (int)(rows < k ? rows : k);
  if (lane == 0) {
#pragma unroll
    for (int s = 0; s < CPW; ++s) {
      const int j = wi + s * W;
      if (j < k) {
        ndir[j] = __dsqrt_rn(out[s]);
        nupd[j] = ndir[j];
        perm[j] = j;
      }
    }
  }
  if (threadIdx.x == 0) s_nonzero = size;
  __syncthreads();
  double maxn = nupd[0];
  for (int j = 1; j < k; ++j)
    if (nupd[j] > maxn) maxn = nupd[j];
  const double thr_helper = __ddiv_rn(__dmul_rn(__dmul_rn(maxn, DBL_EPSILON), __dmul_rn(maxn, DBL_EPSILON)), rows_thr);
  const double downdate_thr = 1.4901161193847656e-08;  // sqrt(DBL_EPSILON)

  for (int kk = 0; kk < size; ++kk) {
    if (threadIdx.x == 0) {
      int big = kk;
      double bign = nupd[kk];
      for (int j = kk + 1; j < k; ++j)
        if (nupd[j] > bign) {
          bign = nupd[j];
          big = j;
        }
      if (s_nonzero == size && __dmul_rn(bign, bign) < __dmul_rn(thr_helper, rows_thr - kk)) s_nonzero = kk;
      if (big != kk) {
        double t = nupd[kk]; nupd[kk] = nupd[big]; nupd[big] = t;
        t = ndir[kk]; ndir[kk] = ndir[big]; ndir[big] = t;
        int p = perm[kk]; perm[kk] = perm[big]; perm[big] = p;
        double* cq = colp[kk]; colp[kk] = colp[big]; colp[big] = cq;
      }
    }
    __syncthreads();
    // Householder reflector of the pivot column (Householder.h:67-96)
    double* col = colp[kk];
    double tau;
    {
      // c0 is read before the barrier of the tail sum, after which CTA 0 overwrites it with beta
      const double c0 = __ldcg(col + kk);
      const double ps = wi == 0 ? lane_sumsq(col, kk + 1 + L, rows) : 0.0;
      const double tail_sq = (rows - kk == 1) ? 0.0 : cl_sum1<KB, W, CPW>(cl, red, ps);
      double beta;
      if (tail_sq <= DBL_MIN) {
        tau = 0.0;
        beta = c0;
        for (int64_t i = kk + 1 + L + 256 * (int64_t)wi; i < rows; i += 256 * W) __stcg(col + i, 0.0);
      } else {
        beta = __dsqrt_rn(__dadd_rn(__dmul_rn(c0, c0), tail_sq));
        if (c0 >= 0.0) beta = -beta;
        const double den = __dsub_rn(c0, beta);
        const double rden = __drcp_rn(den);
        // element-wise: the lane's rows are dealt to the CTA's warps
        int64_t i = kk + 1 + L + 256 * (int64_t)wi;
        for (; i + 256 * W * (kRowBatch - 1) < rows; i += 256 * W * kRowBatch) {
          double q[kRowBatch];
#pragma unroll
          for (int u = 0; u < kRowBatch; ++u) q[u] = __ldcg(col + i + 256 * W * u);
#pragma unroll
          for (int u = 0; u < kRowBatch; ++u) __stcg(col + i + 256 * W * u, div_by(q[u], den, rden));
        }
        for (; i < rows; i += 256 * W) __stcg(col + i, div_by(__ldcg(col + i), den, rden));
        tau = __ddiv_rn(__dsub_rn(beta, c0), beta);
      }
      if (w == 0 && threadIdx.x == 0) __stcg(col + kk, beta);
      // the division pass wrote rows that other warps of this CTA read next
      __syncthreads();
    }
    // apply H = I - tau v v^T to the columns after the pivot (Householder.h:116-133);
    // the right-hand side only while kk < rank
    const int c_lo = kk + 1, c_hi = s_nonzero == size ? k + 1 : k;
    const int cnt = c_hi - c_lo;
    if (cnt > 0) {
      if (rows - kk == 1) {
        if (w == 0)
          for (int j = threadIdx.x; j < cnt; j += blockDim.x) {
            double* q = colp[c_lo + j] + kk;
            __stcg(q, __dmul_rn(__ldcg(q), __dsub_rn(1.0, tau)));
          }
      } else if (tau != 0.0) {
        const double* v = col;
        double* cp[CPW];
        double qk[CPW];
#pragma unroll
        for (int s = 0; s < CPW; ++s) {
          const int j = wi + s * W;
          cp[s] = j < cnt ? colp[c_lo + j] : nullptr;
          qk[s] = j < cnt ? __ldcg(cp[s] + kk) : 0.0;  // row kk, read before CTA 0 rewrites it
          part[s] = 0.0;
        }
        if (cp[0]) {  // a warp without columns has no dot share
          int64_t i = kk + 1 + L;
          for (; i + 256 * (U - 1) < rows; i += 256 * U) {
            double vi[U], cv[U][CPW];
#pragma unroll
            for (int u = 0; u < U; ++u) {
              vi[u] = __ldcg(v + i + 256 * u);
#pragma unroll
              for (int s = 0; s < CPW; ++s) cv[u][s] = cp[s] ? __ldcg(cp[s] + i + 256 * u) : 0.0;
            }
#pragma unroll
            for (int u = 0; u < U; ++u)
#pragma unroll
              for (int s = 0; s < CPW; ++s)
                if (cp[s]) part[s] = __fma_rn(vi[u], cv[u][s], part[s]);
          }
          for (; i < rows; i += 256) {
            const double vi = __ldcg(v + i);
#pragma unroll
            for (int s = 0; s < CPW; ++s)
              if (cp[s]) part[s] = __fma_rn(vi, __ldcg(cp[s] + i), part[s]);
          }
        }
        cl_sum_cols<KB, W, CPW>(cl, red, part, cnt, out);
        // tmp_j += Q[kk, j]; Q[kk, j] -= tau * tmp_j; -tmp_j to every warp of the CTA
#pragma unroll
        for (int s = 0; s < CPW; ++s) {
          if (!cp[s]) continue;
          out[s] = __dadd_rn(out[s], qk[s]);
          if (w == 0 && lane == 0) __stcg(cp[s] + kk, __dsub_rn(qk[s], __dmul_rn(tau, out[s])));
          if (lane == 0) ntmp[wi + s * W] = -out[s];
        }
        __syncthreads();
        // element-wise Q[i, j] -= (tau v_i) tmp_j: the lane's rows are dealt to
        // the CTA's warps as in the division pass (the same thread wrote v_i),
        // each warp updating every column, so tau v_i is formed once per row
        {
          constexpr int UR = 4;
          int64_t i = kk + 1 + L + 256 * (int64_t)wi;
          for (; i + 256 * W * (UR - 1) < rows; i += 256 * W * UR) {
            double t[UR];
#pragma unroll
            for (int u = 0; u < UR; ++u) t[u] = __dmul_rn(tau, __ldcg(v + i + 256 * W * u));
            int j = 0;
            for (; j + 1 < cnt; j += 2) {
              double* q0 = colp[c_lo + j] + i;
              double* q1 = colp[c_lo + j + 1] + i;
              const double n0 = ntmp[j], n1 = ntmp[j + 1];
              double a0[UR], a1[UR];
#pragma unroll
              for (int u = 0; u < UR; ++u) {
                a0[u] = __ldcg(q0 + 256 * W * u);
                a1[u] = __ldcg(q1 + 256 * W * u);
              }
#pragma unroll
              for (int u = 0; u < UR; ++u) {
                __stcg(q0 + 256 * W * u, __fma_rn(t[u], n0, a0[u]));
                __stcg(q1 + 256 * W * u, __fma_rn(t[u], n1, a1[u]));
              }
            }
            if (j < cnt) {
              double* q0 = colp[c_lo + j] + i;
              const double n0 = ntmp[j];
              double a0[UR];
#pragma unroll
              for (int u = 0; u < UR; ++u) a0[u] = __ldcg(q0 + 256 * W * u);
#pragma unroll
              for (int u = 0; u < UR; ++u) __stcg(q0 + 256 * W * u, __fma_rn(t[u], n0, a0[u]));
            }
          }
          for (; i < rows; i += 256 * W) {
            const double t = __dmul_rn(tau, __ldcg(v + i));
            for (int j = 0; j < cnt; ++j) {
              double* q = colp[c_lo + j] + i;
              __stcg(q, __fma_rn(t, ntmp[j], __ldcg(q)));
            }
          }
        }
      }
    }
    cl.sync();  // the step's rows (and row kk) visible to every CTA
    // LAWN 176 norm down-dating (ColPivHouseholderQR.h:549-572)
    if (threadIdx.x == 0) {
      for (int j = kk + 1; j < k; ++j) {
        rec[j] = 0;
        if (nupd[j] != 0.0) {
          double temp = __ddiv_rn(fabs(__ldcg(colp[j] + kk)), nupd[j]);
          temp = __dmul_rn(__dadd_rn(1.0, temp), __dsub_rn(1.0, temp));
          temp = temp < 0.0 ? 0.0 : temp;
          const double ratio = __ddiv_rn(nupd[j], ndir[j]);
          const double temp2 = __dmul_rn(temp, __dmul_rn(ratio, ratio));
          if (temp2 <= downdate_thr) rec[j] = 1;
          else nupd[j] = __dmul_rn(nupd[j], __dsqrt_rn(temp));
        }
      }
    }
    __syncthreads();
    // direct recomputation of the flagged norms: one barrier for all of them
    // (column j by warp j mod W); every CTA takes the same branch
    int any_rec = 0;
    for (int j = kk + 1; j < k; ++j) any_rec |= rec[j];
    if (any_rec) {
#pragma unroll
      for (int s = 0; s < CPW; ++s) {
        const int j = wi + s * W;
        part[s] = (j > kk && j < k && rec[j]) ? lane_sumsq(colp[j], kk + 1 + L, rows) : 0.0;
      }
      cl_sum_cols<KB, W, CPW>(cl, red, part, k, out);
      if (lane == 0) {
#pragma unroll
        for (int s = 0; s < CPW; ++s) {
          const int j = wi + s * W;
          if (j > kk && j < k && rec[j]) {
            ndir[j] = __dsqrt_rn(out[s]);
            nupd[j] = ndir[j];
          }
        }
      }
      __syncthreads();
    }
  }
  if (w == 0 && threadIdx.x == 0) {
    const int r = s_nonzero;
    double cvec[kMaxK];
    for (int i = 0; i < r; ++i) cvec[i] = __ldcg(colp[k] + i);
    for (int kk = r - 1; kk >= 0; --kk) {
      cvec[kk] = __ddiv_rn(cvec[kk], __ldcg(colp[kk] + kk));
      for (int i = 0; i < kk; ++i) cvec[i] = __dsub_rn(cvec[i], __dmul_rn(cvec[kk], __ldcg(colp[kk] + i)));
    }
    double* outc = coefs + cd.coef_offset;
    for (int j = 0; j < k; ++j) outc[j] = 0.0;
    for (int i = 0; i < r; ++i) outc[perm[i]] = cvec[i];
    res[c].rank = r;
    // algorithmic bytes: the copy, then every remaining column (the right-hand
    // side while kk < rank) read and written once per step
    double cols = (double)(2 * k + 1);
    for (int kk = 0; kk < size; ++kk) cols += 2.0 * (double)((kk < r ? k + 1 : k) - kk);
    if (count_bytes)
      atomicAdd(reinterpret_cast<unsigned long long*>(status + kStatusQrBytes),
                (unsigned long long)(cols * 8.0 * (double)rows));
  }
  // no CTA leaves while another may still write into its shared memory
  cl.sync();
}

template <int KB, int W>
__global__ void __cluster_dims__(kQrCluster, 1, 1) __launch_bounds__(32 * W)
    plain_qr_cluster_kernel(DevBatch b, DevData ds, const PlainCand* pc, const int32_t* list, int cand0,
                            const double* A, double* M, double* coefs, rrg_result* res, uint32_t* status,
                            const int32_t* colmap, int count_bytes) {
  cg::cluster_group cl = cg::this_cluster();
  const int ci = blockIdx.x / kQrCluster;
  const int c = list ? list[cand0 + ci] : cand0 + ci;
  qr_cluster_one<KB, W>(cl, b, ds, pc, c, A, M + pc[c].m_col * ds.n_pad, coefs, res, status, colmap, count_bytes);
}

// Persistent form over a list whose length the device decided: the clusters
// of the grid take the candidates list[0 .. *count) one at a time from a
// shared counter (*next, zero before the launch), each factorising in its own
// working slot of slot_cols columns of M.  Same bits as the per-candidate
// kernel: only the placement of the working columns differs.
// Resident blocks the list form is compiled for: about the register
// footprint of the per-candidate form (72 registers a thread; 64 at 16 warps).
template <int W>
struct ListMinBlocks {
  static constexpr int value = W >= 16 ? 2 : 65536 / (32 * W * 72);
};

template <int KB, int W>
__global__ void __cluster_dims__(kQrCluster, 1, 1) __launch_bounds__(32 * W, ListMinBlocks<W>::value)
    plain_qr_cluster_list_kernel(DevBatch b, DevData ds, const PlainCand* pc, const int32_t* list,
                                 const int32_t* count, int32_t* next, const double* A, double* M, int slot_cols,
                                 double* coefs, rrg_result* res, uint32_t* status, const int32_t* colmap,
                                 int count_bytes) {
  cg::cluster_group cl = cg::this_cluster();
  __shared__ int s_take;
  const int slot = blockIdx.x / kQrCluster;
  double* Q = M + (int64_t)slot * slot_cols * ds.n_pad;
  const int cnt = *count;
  for (;;) {
    // CTA 0 takes the next candidate and every CTA reads it from CTA 0's
    // shared memory after the barrier; CTA 0 takes another only after the
    // factorisation's closing barrier, when every CTA has read this one
    if (cl.block_rank() == 0 && threadIdx.x == 0) s_take = atomicAdd(next, 1);
    cl.sync();
    const int t = *cl.map_shared_rank(&s_take, 0);
    if (t >= cnt) break;
    qr_cluster_one<KB, W>(cl, b, ds, pc, list[t], A, Q, coefs, res, status, colmap, count_bytes);
    cl.sync();
  }
  // no CTA leaves while CTA 0's counter slot may still be read
  cl.sync();
}

}  // namespace

int qr_warp_variants(int bucket, int* out) {
  switch (bucket) {
    case 4: out[0] = 2; out[1] = 1; out[2] = 4; return 3;
    case 8: out[0] = 4; out[1] = 2; out[2] = 8; return 3;
    case 16: out[0] = 8; out[1] = 4; out[2] = 16; return 3;
    case kMaxK + 1: out[0] = 8; out[1] = 16; return 2;
    default: return 0;
  }
}

bool launch_plain_qr_cluster(int max_cols, int warps, int n_cand, cudaStream_t st, DevBatch b, DevData ds,
                             const PlainCand* pc, const int32_t* list, int cand0, const double* A, double* M,
                             double* coefs, rrg_result* res, uint32_t* status, const int32_t* colmap,
                             bool count_bytes) {
  if (n_cand <= 0) return true;
  const int grid = n_cand * kQrCluster;
  const int bk = plain_qr_bucket(max_cols);
  int v[4];
  const int nv = qr_warp_variants(bk, v);
  if (warps == 0) warps = v[0];
  bool known = false;
  for (int i = 0; i < nv; ++i) known = known || v[i] == warps;
  if (!known) {
    rrc::set_error("QR launch: no kernel built for this column bucket and warps per CTA");
    return false;
  }
#define RRG_QR_CLUSTER(KB, W)                                                                               \
  if (bk == KB && warps == W) {                                                                             \
    plain_qr_cluster_kernel<KB, W><<<grid, 32 * W, 0, st>>>(b, ds, pc, list, cand0, A, M, coefs, res, status, \
                                                            colmap, count_bytes ? 1 : 0);                   \
    return launch_ok("launch_plain_qr_cluster");                                                               \
  }
  RRG_QR_CLUSTER(4, 1)
  RRG_QR_CLUSTER(4, 2)
  RRG_QR_CLUSTER(4, 4)
  RRG_QR_CLUSTER(8, 2)
  RRG_QR_CLUSTER(8, 4)
  RRG_QR_CLUSTER(8, 8)
  RRG_QR_CLUSTER(16, 4)
  RRG_QR_CLUSTER(16, 8)
  RRG_QR_CLUSTER(16, 16)
  RRG_QR_CLUSTER(kMaxK + 1, 8)
  RRG_QR_CLUSTER(kMaxK + 1, 16)
#undef RRG_QR_CLUSTER
  rrc::set_error("QR launch: no kernel built for this column bucket and warps per CTA");
  return false;
}

namespace {
// Kernel of a (bucket, warps) pair of the list form, or nullptr.
template <int KB, int W>
const void* list_kernel_of() {
  return reinterpret_cast<const void*>(&plain_qr_cluster_list_kernel<KB, W>);
}
bool list_kernel(int bk, int warps, const void** fn) {
#define RRG_QR_LIST(KB, W) \
  if (bk == KB && warps == W) { *fn = list_kernel_of<KB, W>(); return true; }
  RRG_QR_LIST(4, 1)
  RRG_QR_LIST(4, 2)
  RRG_QR_LIST(4, 4)
  RRG_QR_LIST(8, 2)
  RRG_QR_LIST(8, 4)
  RRG_QR_LIST(8, 8)
  RRG_QR_LIST(16, 4)
  RRG_QR_LIST(16, 8)
  RRG_QR_LIST(16, 16)
  RRG_QR_LIST(kMaxK + 1, 8)
  RRG_QR_LIST(kMaxK + 1, 16)
#undef RRG_QR_LIST
  return false;
}
}  // namespace

int qr_cluster_list_clusters(int bucket, int warps) {
  if (warps == 0) {
    int v[4];
    if (qr_warp_variants(bucket, v) == 0) return 0;
    warps = v[0];
  }
  const void* fn = nullptr;
  if (!list_kernel(bucket, warps, &fn)) return 0;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kQrCluster, 1, 1);
  cfg.blockDim = dim3(32 * warps, 1, 1);
  cfg.dynamicSmemBytes = 0;
  cudaLaunchAttribute attr;
  attr.id = cudaLaunchAttributeClusterDimension;
  attr.val.clusterDim.x = kQrCluster;
  attr.val.clusterDim.y = 1;
  attr.val.clusterDim.z = 1;
  cfg.attrs = &attr;
  cfg.numAttrs = 1;
  int clusters = 0;
  if (cudaOccupancyMaxActiveClusters(&clusters, fn, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return clusters;
}

bool launch_plain_qr_cluster_list(int bucket, int warps, int n_clusters, cudaStream_t st, DevBatch b, DevData ds,
                                  const PlainCand* pc, const int32_t* list, const int32_t* count, int32_t* next,
                                  const double* A, double* M, int slot_cols, double* coefs, rrg_result* res,
                                  uint32_t* status, const int32_t* colmap, bool count_bytes) {
  if (n_clusters <= 0) return true;
  int v[4];
  const int nv = qr_warp_variants(bucket, v);
  if (nv == 0) {
    rrc::set_error("QR launch: unknown column bucket");
    return false;
  }
  if (warps == 0) warps = v[0];
  const int grid = n_clusters * kQrCluster;
#define RRG_QR_LIST(KB, W)                                                                                 \
  if (bucket == KB && warps == W) {                                                                        \
    plain_qr_cluster_list_kernel<KB, W><<<grid, 32 * W, 0, st>>>(b, ds, pc, list, count, next, A, M,       \
                                                                 slot_cols, coefs, res, status, colmap,   \
                                                                 count_bytes ? 1 : 0);                    \
    return launch_ok("launch_plain_qr_cluster_list");                                                              \
  }
  RRG_QR_LIST(4, 1)
  RRG_QR_LIST(4, 2)
  RRG_QR_LIST(4, 4)
  RRG_QR_LIST(8, 2)
  RRG_QR_LIST(8, 4)
  RRG_QR_LIST(8, 8)
  RRG_QR_LIST(16, 4)
  RRG_QR_LIST(16, 8)
  RRG_QR_LIST(16, 16)
  RRG_QR_LIST(kMaxK + 1, 8)
  RRG_QR_LIST(kMaxK + 1, 16)
#undef RRG_QR_LIST
  rrc::set_error("QR launch: no list kernel built for this column bucket and warps per CTA");
  return false;
}

}  // namespace rrd
