// Column-pivoted QR least squares of the plain FP64 path over whole-GPU
// passes: the factorisation of ColPivHouseholderQR::computeInPlace
// (eigen/Eigen/src/QR/ColPivHouseholderQR.h:482-575) and its least-squares
// solve (:577-608), with makeHouseholder / applyHouseholderOnTheLeft semantics
// (eigen/Eigen/src/Householder/Householder.h:67-133), every sum in the QSUM
// order of csrc/common/rr_sum.h.
//
// A candidate's rows are cut into chunks of RR_CHUNK rows.  A pass is one
// launch over (candidate, chunk) items; an item is a 256-thread block whose
// thread t is QSUM lane t of the chunk (its rows i with i mod 256 = t, in
// increasing order), so the block folds its lanes into the chunk's totals.
// The last block of a candidate to finish a pass (a ticket counter) adds the
// chunk totals in chunk order and does the scalar work of the step (pivot
// choice, rank rule, Householder scalars, norm down-dating) for the next pass:
//
//   init   [factors | 1 | y] copied into the working columns; the norms over
//          rows >= 0 and the tails over rows >= 1; step 0's pivot and reflector
//   A(kk)  the pivot tail divided by (c0 - beta) (the Householder vector v)
//          and the dots v . a_j of the columns the reflector reaches; last
//          block: row kk, -tmp_j, down-dating, and the pivot of step kk + 1
//          when no norm must be recomputed
//   B(kk)  a_j -= (tau v_i) tmp_j, and the sums of squares of updated columns
//          step kk + 1 needs (recomputed norms over rows >= kk + 1, pivot
//          tails over rows >= kk + 2); last block: step kk + 1's pivot and
//          reflector
//   solve  back substitution with R and the transformed y
//
// A sum over rows >= kk + 2 differs from the one over rows >= kk + 1 only in
// the lane that owns row kk + 1, whose chain starts there: that lane forms
// the shorter chain too, and the chunk holding row kk + 1 is folded twice.
#include <cfloat>
#include <cstdint>

#include "../common/error.h"
#include "../common/rr_sum.h"
#include "common.cuh"
#include "qr_chunk.cuh"
#include "qr_ops.cuh"
#include "reduce.cuh"

namespace rrd {

namespace {

constexpr int kQC = RR_CHUNK;
constexpr int kLaneRows = kQC / 256;
constexpr double kDowndateThr = 1.4901161193847656e-08;  // sqrt(DBL_EPSILON)

__device__ __forceinline__ int job_count(const QrJob& j) {
  if (!j.dcount) return j.n_list;
  const int n = *j.dcount - j.list_off;
  return n < 0 ? 0 : (n > j.n_list ? j.n_list : n);
}

__device__ __forceinline__ double* wcol(const QrJob& j, int t, int c, int s) {
  const int64_t base = j.slot_cols > 0 ? (int64_t)t * j.slot_cols : j.pc[c].m_col;
  return j.M + (base + s) * j.ds.n_pad;
}

// chunk total of sum slot s; row nch holds the shorter-range variant
__device__ __forceinline__ double* part_at(const QrJob& j, int t, int row, int s) {
  return j.part + ((int64_t)t * (j.nch + 1) + row) * j.max_cols + s;
}

// QSUM of the chunk totals of slot s in chunk order from 0; chunk `sp` (if
// >= 0) contributes its variant instead
__device__ __forceinline__ double chunk_total(const QrJob& j, int t, int s, int sp) {
  double tot = 0.0;
  for (int ch = 0; ch < j.nch; ++ch) tot = __dadd_rn(tot, __ldcg(part_at(j, t, ch == sp ? j.nch : ch, s)));
  return tot;
}

// Lane fold of cnt values per thread (RR256's fold: halving strides inside
// each 32-lane group, then the eight group totals in order from 0) into
// out[0 .. cnt) (shared).  red: 8 * CG shared doubles.
template <int CG>
__device__ __forceinline__ void fold_lanes(const double (&v)[CG], int cnt, double* red, double* out) {
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
  for (int j = 0; j < CG; ++j)
    if (j < cnt) {
      const double s = warp_sum(v[j]);
      if (l == 0) red[w * CG + j] = s;
    }
  __syncthreads();
  if (threadIdx.x < cnt) {
    double s = 0.0;
    for (int i = 0; i < 8; ++i) s = __dadd_rn(s, red[i * CG + threadIdx.x]);
    out[threadIdx.x] = s;
  }
  __syncthreads();
}

// After an item's chunk totals are written: true in the block that finishes
// the candidate's pass last (every other block's writes are then visible)
__device__ __forceinline__ bool last_block(QrState* S, int nch, int* s_flag) {
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) *s_flag = atomicAdd(&S->ticket, 1u) == (unsigned)(nch - 1) ? 1 : 0;
  __syncthreads();
  const bool last = *s_flag != 0;
  if (last) __threadfence();
  return last;
}

// Businger-Golub pivot of step kk (largest down-dated norm, first index on
// ties), the rank rule of ColPivHouseholderQR.h:504-511, and the swap
__device__ void select_pivot(QrState* S, int kk, double rows) {
  int big = kk;
  double bign = S->nupd[kk];
  for (int j = kk + 1; j < S->k; ++j)
    if (S->nupd[j] > bign) {
      bign = S->nupd[j];
      big = j;
    }
  if (S->nonzero == S->size && __dmul_rn(bign, bign) < __dmul_rn(S->thr_helper, rows - kk)) S->nonzero = kk;
  if (big != kk) {
    double t = S->nupd[kk]; S->nupd[kk] = S->nupd[big]; S->nupd[big] = t;
    t = S->ndir[kk]; S->ndir[kk] = S->ndir[big]; S->ndir[big] = t;
    int p = S->perm[kk]; S->perm[kk] = S->perm[big]; S->perm[big] = p;
    p = S->pos2col[kk]; S->pos2col[kk] = S->pos2col[big]; S->pos2col[big] = p;
  }
}

// makeHouseholder of the pivot from its diagonal entry and tail sum of squares
__device__ void householder_scalars(QrState* S, double c0, double tail_sq) {
  if (tail_sq <= DBL_MIN) {
    S->tau = 0.0;
    S->beta = c0;
    S->den = 1.0;
    S->rden = 1.0;
    S->tau_zero = 1;
  } else {
    double beta = __dsqrt_rn(__dadd_rn(__dmul_rn(c0, c0), tail_sq));
    if (c0 >= 0.0) beta = -beta;
    const double den = __dsub_rn(c0, beta);
    S->den = den;
    S->rden = __drcp_rn(den);
    S->tau = __ddiv_rn(__dsub_rn(beta, c0), beta);
    S->beta = beta;
    S->tau_zero = 0;
  }
}

// Shared per-item view of a candidate's state.
struct ItemView {
  int t, c, active, k, nwork, nsum, upd, tau_zero;
  int piv;         // the pivot's storage column (step kk)
  int fastq;       // pass B: work index of the one summed column formed during the update, or -1
  int64_t lo, hi;  // rows of the item: [lo, hi)
  double tau, den, rden;
  int work[kQrMaxCols];   // storage columns the pass reads (and updates)
  int slot[kQrMaxCols];   // per storage column: its sum slot, or -1
  double ntmp[kQrMaxCols];
};

// Calls row(i) for the rows of this thread's lane in [lo, hi), in increasing
// order; a full chunk needs no bounds test.
template <class F>
__device__ __forceinline__ void lane_rows(int64_t r0, int64_t lo, int64_t hi, F&& row) {
  const int64_t base = r0 + threadIdx.x;
  if (lo == r0 && hi == r0 + kQC) {
#pragma unroll 2
    for (int u = 0; u < kLaneRows; ++u) row(base + 256 * u);
  } else {
    int64_t first = base;
    if (first < lo) first += (lo - first + 255) / 256 * 256;
#pragma unroll 1
    for (int64_t i = first; i < hi; i += 256) row(i);
  }
}

// Rows of this thread's lane in sub-chunks of kSub rows (kSubU per lane):
// body(s0, full) for each sub-chunk of the item in order; `full` when every
// row of the sub-chunk is in [lo, hi).
constexpr int kSub = 2048;
constexpr int kSubU = kSub / 256;
template <class F>
__device__ __forceinline__ void sub_chunks(int64_t r0, int64_t lo, int64_t hi, F&& body) {
  for (int64_t s0 = r0; s0 < r0 + kQC && s0 < hi; s0 += kSub) {
    if (s0 + kSub <= lo) continue;
    body(s0, s0 >= lo && s0 + kSub <= hi);
  }
}

// Reads the item's state into V (thread 0).  kk < 0: the copy pass.
__device__ void load_view(ItemView& V, const QrJob& j, int t, int ch, int kk, int pass_a) {
  QrState* S = j.state + t;
  const int64_t rows = j.ds.n;
  const int c = j.list[j.list_off + t];
  V.t = t;
  V.c = c;
  if (kk < 0) {
    const rrg_cand cd = j.b.cands[c];
    const int k = j.pc[c].k;
    V.active = cd.mode == RRG_TUNED && !(j.pc[c].pad & 1) && k >= 1;
    if (V.active && k + 1 > j.max_cols) {
      atomicOr(j.status, ST_TOO_LARGE);
      V.active = 0;
    }
    if (!V.active && ch == 0) S->active = 0;
    V.k = k;
    if (V.active) {
      V.nwork = k + 1;
      V.nsum = k;
      for (int s = 0; s <= k; ++s) {
        V.work[s] = s;
        V.slot[s] = s < k ? s : -1;
      }
    }
  } else {
    V.active = S->active && kk < S->size;
    if (V.active) {
      const int k = S->k;
      V.k = k;
      V.tau = S->tau;
      V.den = S->den;
      V.rden = S->rden;
      V.tau_zero = S->tau_zero;
      V.piv = S->pos2col[kk];
      V.upd = !S->tau_zero && rows - kk > 1;
      int nw = 0;
      if (V.upd) {
        for (int p = kk + 1; p < k; ++p) V.work[nw++] = S->pos2col[p];
        if (S->upd_y) V.work[nw++] = k;
      }
      if (pass_a) {
        V.nsum = 0;
      } else {
        V.nsum = S->nsum;
        for (int s = 0; s <= k; ++s) V.slot[s] = -1;
        for (int q = 0; q < V.nsum; ++q) V.slot[S->sum_store[q]] = q;
        V.fastq = -1;
        if (V.upd) {
          for (int q = 0; q < nw; ++q) {
            V.ntmp[q] = S->ntmp[V.work[q]];
            if (V.nsum == 1 && V.work[q] == S->sum_store[0]) V.fastq = q;
          }
        }
      }
      V.nwork = nw;
    }
  }
  const int64_t r0 = (int64_t)ch * kQC;
  V.lo = r0 > kk + 1 ? r0 : kk + 1;
  V.hi = r0 + kQC < rows ? r0 + kQC : rows;
}

// ------------------------------------------------------- init and B(kk) ----
// INIT: the copy pass (kk = -1).  Otherwise the rank-1 update of step kk and
// the sums step kk + 1 needs.
// Resident blocks the passes are compiled for (registers per thread <= 64K /
// (256 x blocks)): the step passes stream columns with little register
// state; the copy pass (run once) keeps a group's sources and sums.
template <int CG, bool INIT = false>
struct QrMinBlocks {
  static constexpr int value = CG <= 8 ? (INIT ? 3 : 4) : 2;
};

template <int CG, bool INIT>
__global__ void __launch_bounds__(256, (QrMinBlocks<CG, INIT>::value)) qr_sums_kernel(QrJob j, int kk) {
  __shared__ ItemView V;
  __shared__ double red[8 * CG], outA[CG], outB[CG];
  __shared__ int s_flag;
  __shared__ double s_norm[kQrMaxCols], s_tail[kQrMaxCols];
  __shared__ double sbuf[kSub];  // pass B: tau v_i of a sub-chunk (lane-owned entries)
  const int cnt = job_count(j);
  const int64_t items = (int64_t)cnt * j.nch;
  const int64_t rows = j.ds.n;
  const int64_t sp_row = kk + 1;  // the row only the longer sums include
  for (int64_t it = blockIdx.x; it < items; it += gridDim.x) {
    const int t = (int)(it / j.nch), ch = (int)(it % j.nch);
    QrState* S = j.state + t;
    if (threadIdx.x == 0) load_view(V, j, t, ch, kk, 0);
    __syncthreads();
    if (!V.active) {
      __syncthreads();
      continue;
    }
    if (INIT) {
      const int c = V.c, k = V.k;
      const int64_t r0 = (int64_t)ch * kQC;
      constexpr bool upd = false;
      const bool sp_chunk = sp_row >= r0 && sp_row < r0 + kQC;
      const bool sp_lane = sp_chunk && (int)(sp_row & 255) == (int)threadIdx.x;
      for (int g0 = 0; g0 < V.nwork; g0 += CG) {
        const int gc = V.nwork - g0 < CG ? V.nwork - g0 : CG;
        double* cp[CG];
        const double* src[CG];
        double nt[CG], sa[CG];
        bool sum[CG];
        bool any_sum = false;
  #pragma unroll
        for (int q = 0; q < CG; ++q) {
          const int s = q < gc ? V.work[g0 + q] : 0;
          cp[q] = q < gc ? wcol(j, t, c, s) : nullptr;
          sum[q] = q < gc && V.slot[s] >= 0;
          any_sum = any_sum || sum[q];
          nt[q] = 0.0;
          sa[q] = 0.0;
          src[q] = nullptr;
          if (q < gc && s != k - 1)
            src[q] = s < k - 1 ? factor_column(j.A, j.ds.n_pad, j.pc[c].a_col, s, j.colmap) : j.ds.y64;
        }
        // one row: every load first, then the arithmetic and the stores
        auto load = [&](int64_t i, double (&a)[CG], double& tv) {
  #pragma unroll
          for (int q = 0; q < CG; ++q)
            if (q < gc) a[q] = src[q] ? src[q][i] : 1.0;
          tv = 0.0;
        };
        auto finish = [&](int64_t i, double (&a)[CG], double tv) {
  #pragma unroll
          for (int q = 0; q < CG; ++q)
            if (q < gc) {
              cp[q][i] = a[q];
              if (sum[q]) sa[q] = __fma_rn(a[q], a[q], sa[q]);
            }
        };
        lane_rows(r0, V.lo, V.hi, [&](int64_t i) {
          double a[CG], tv;
          load(i, a, tv);
          finish(i, a, tv);
        });
        if (!any_sum) continue;  // uniform over the block
        double va[CG], vb[CG];
  #pragma unroll
        for (int q = 0; q < CG; ++q) va[q] = sum[q] ? sa[q] : 0.0;
        fold_lanes<CG>(va, gc, red, outA);
        if (sp_chunk) {
          // the lane owning row sp_row: its chain without that row
  #pragma unroll
          for (int q = 0; q < CG; ++q) vb[q] = va[q];
          if (sp_lane) {
  #pragma unroll
            for (int q = 0; q < CG; ++q) vb[q] = 0.0;
            for (int64_t i = sp_row + 256; i < V.hi; i += 256) {
  #pragma unroll
              for (int q = 0; q < CG; ++q)
                if (sum[q]) {
                  const double x = cp[q][i];
                  vb[q] = __fma_rn(x, x, vb[q]);
                }
            }
          }
          fold_lanes<CG>(vb, gc, red, outB);
        }
        if (threadIdx.x < gc) {
          const int sl = V.slot[V.work[g0 + threadIdx.x]];
          if (sl >= 0) {
            *part_at(j, t, ch, sl) = outA[threadIdx.x];
            if (sp_chunk) *part_at(j, t, j.nch, sl) = outB[threadIdx.x];
          }
        }
      }
    } else {
      const int c = V.c, k = V.k;
      (void)k;
      const int64_t r0 = (int64_t)ch * kQC;
      const int64_t np = j.ds.n_pad;
      double* Mb = j.M + (j.slot_cols > 0 ? (int64_t)t * j.slot_cols : j.pc[c].m_col) * np;
      const double* vcol = Mb + (int64_t)V.piv * np;
      const double tau = V.tau;
      const bool sp_chunk = sp_row >= r0 && sp_row < r0 + kQC;
      const bool sp_lane = sp_chunk && (int)(sp_row & 255) == (int)threadIdx.x;
      const int fq = V.fastq;
      double sf = 0.0;  // the summed column's chain, formed during the update
      if (V.upd) {
        // tau v_i of a sub-chunk's rows staged in shared memory (each thread
        // reads back only its own lane's entries), then each column streamed
        // on its own: its loads are independent of the other columns' stores
        for (int g0 = 0; g0 < V.nwork; g0 += CG) {
          const int gc = V.nwork - g0 < CG ? V.nwork - g0 : CG;
          sub_chunks(r0, V.lo, V.hi, [&](int64_t s0, bool full) {
#pragma unroll
            for (int u = 0; u < kSubU; ++u) {
              const int64_t i = s0 + threadIdx.x + 256 * u;
              sbuf[threadIdx.x + 256 * u] = (full || (i >= V.lo && i < V.hi)) ? __dmul_rn(tau, vcol[i]) : 0.0;
            }
#pragma unroll
            for (int q = 0; q < CG; ++q) {
              if (q >= gc) break;
              double* col = Mb + (int64_t)V.work[g0 + q] * np;
              const double nt = V.ntmp[g0 + q];
              const bool fsum = g0 + q == fq;
              if (full) {
#pragma unroll
                for (int u = 0; u < kSubU; ++u) {
                  const int64_t i = s0 + threadIdx.x + 256 * u;
                  const double a = __fma_rn(sbuf[threadIdx.x + 256 * u], nt, col[i]);
                  col[i] = a;
                  if (fsum) sf = __fma_rn(a, a, sf);
                }
              } else {
                for (int u = 0; u < kSubU; ++u) {
                  const int64_t i = s0 + threadIdx.x + 256 * u;
                  if (i < V.lo || i >= V.hi) continue;
                  const double a = __fma_rn(sbuf[threadIdx.x + 256 * u], nt, col[i]);
                  col[i] = a;
                  if (fsum) sf = __fma_rn(a, a, sf);
                }
              }
            }
          });
        }
      }
      // sums of squares of the summed columns (updated values): the one formed
      // above, or a pass over each (a norm recomputation, an identity reflector)
      for (int q0 = 0; q0 < V.nsum; ++q0) {
        const double* col;
        double pa;
        if (fq >= 0) {
          col = Mb + (int64_t)V.work[fq] * np;
          pa = sf;
        } else {
          col = nullptr;
          for (int s2 = 0; s2 <= V.k; ++s2)
            if (V.slot[s2] == q0) col = Mb + (int64_t)s2 * np;
          pa = 0.0;
          lane_rows(r0, V.lo, V.hi, [&](int64_t i) {
            const double x = col[i];
            pa = __fma_rn(x, x, pa);
          });
        }
        double va[1] = {pa}, vb[1];
        fold_lanes<1>(va, 1, red, outA);
        if (sp_chunk) {
          // the lane owning row sp_row: its chain without that row
          vb[0] = pa;
          if (sp_lane) {
            vb[0] = 0.0;
            for (int64_t i = sp_row + 256; i < V.hi; i += 256) vb[0] = __fma_rn(col[i], col[i], vb[0]);
          }
          fold_lanes<1>(vb, 1, red, outB);
        }
        if (threadIdx.x == 0) {
          const int sl = fq >= 0 ? 0 : q0;
          *part_at(j, t, ch, sl) = outA[0];
          if (sp_chunk) *part_at(j, t, j.nch, sl) = outB[0];
        }
        if (fq >= 0) break;
      }
    }
    if (!last_block(S, j.nch, &s_flag)) continue;
    // ---- the candidate's last block: totals, then step kk + 1's scalars
    const int nsum = V.nsum;
    const int sp = (int)(sp_row / kQC);
    for (int q = threadIdx.x; q < nsum; q += blockDim.x) {
      s_norm[q] = chunk_total(j, t, q, -1);
      s_tail[q] = chunk_total(j, t, q, sp);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      const int c = V.c, k = V.k;
      const double rows_d = (double)rows;
      const int next = kk + 1;
      bool choose = true;
      if (INIT) {
        S->active = 1;
        S->k = k;
        S->size = (int)(rows < k ? rows : k);
        S->nonzero = S->size;
        for (int s = 0; s < k; ++s) {
          S->ndir[s] = __dsqrt_rn(s_norm[s]);
          S->nupd[s] = S->ndir[s];
          S->perm[s] = s;
          S->pos2col[s] = s;
          S->sum_store[s] = s;
        }
        S->pos2col[k] = k;
        double maxn = S->nupd[0];
        for (int s = 1; s < k; ++s)
          if (S->nupd[s] > maxn) maxn = S->nupd[s];
        S->thr_helper = __ddiv_rn(__dmul_rn(__dmul_rn(maxn, DBL_EPSILON), __dmul_rn(maxn, DBL_EPSILON)), rows_d);
      } else {
        // recomputed norms (ColPivHouseholderQR.h:566-569)
        for (int q = 0; q < nsum; ++q)
          if (S->sum_norm[q]) {
            const int s = S->sum_store[q];
            for (int p = next; p < k; ++p)
              if (S->pos2col[p] == s) {
                S->ndir[p] = __dsqrt_rn(s_norm[q]);
                S->nupd[p] = S->ndir[p];
              }
          }
        choose = S->rec_any != 0;
      }
      if (next < S->size) {
        if (choose) {
          select_pivot(S, next, rows_d);
          S->upd_y = S->nonzero == S->size;
        } else {
          S->upd_y = S->upd_y_next;
        }
        const int ps = S->pos2col[next];
        int q = 0;
        while (q < nsum && S->sum_store[q] != ps) ++q;
        if (q == nsum) {
          atomicOr(j.status, ST_QR_STATE);
          S->active = 0;
        } else {
          const double tail_sq = rows - next == 1 ? 0.0 : s_tail[q];
          householder_scalars(S, __ldcg(wcol(j, t, c, ps) + next), tail_sq);
        }
      }
      S->kk = next;
      S->ticket = 0;
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------ A(kk) --
template <int CG>
__global__ void __launch_bounds__(256, QrMinBlocks<CG>::value) qr_passA_kernel(QrJob j, int kk) {
  __shared__ ItemView V;
  __shared__ double red[8 * CG], outA[CG];
  __shared__ int s_flag;
  __shared__ double sbuf[kSub];  // v_i of a sub-chunk (lane-owned entries)
  const int cnt = job_count(j);
  const int64_t items = (int64_t)cnt * j.nch;
  const int64_t rows = j.ds.n;
  for (int64_t it = blockIdx.x; it < items; it += gridDim.x) {
    const int t = (int)(it / j.nch), ch = (int)(it % j.nch);
    QrState* S = j.state + t;
    if (threadIdx.x == 0) load_view(V, j, t, ch, kk, 1);
    __syncthreads();
    if (!V.active) {
      __syncthreads();
      continue;
    }
    const int c = V.c;
    const int64_t r0 = (int64_t)ch * kQC;
    double* pcol = wcol(j, t, c, V.piv);
    const double den = V.den, rden = V.rden;
    // the Householder vector (Householder.h:83-90): the tail over c0 - beta,
    // or zeros when the reflector is the identity
    if (V.nwork == 0) {
      const bool tz = V.tau_zero != 0;
      lane_rows(r0, V.lo, V.hi, [&](int64_t i) { pcol[i] = tz ? 0.0 : div_by(pcol[i], den, rden); });
    }
    for (int g0 = 0; g0 < V.nwork; g0 += CG) {
      const int gc = V.nwork - g0 < CG ? V.nwork - g0 : CG;
      double pa[CG];
#pragma unroll
      for (int q = 0; q < CG; ++q) pa[q] = 0.0;
      const bool first = g0 == 0;
      sub_chunks(r0, V.lo, V.hi, [&](int64_t s0, bool full) {
        // the sub-chunk's v_i (divided once, by the first group) staged in
        // shared memory; then each column's dot chain on its own
#pragma unroll
        for (int u = 0; u < kSubU; ++u) {
          const int64_t i = s0 + threadIdx.x + 256 * u;
          double v = 0.0;
          if (full || (i >= V.lo && i < V.hi)) {
            v = pcol[i];
            if (first) {
              v = div_by(v, den, rden);
              pcol[i] = v;
            }
          }
          sbuf[threadIdx.x + 256 * u] = v;
        }
#pragma unroll
        for (int q = 0; q < CG; ++q) {
          if (q >= gc) break;
          const double* col = wcol(j, t, c, V.work[g0 + q]);
          double acc = pa[q];
          if (full) {
#pragma unroll
            for (int u = 0; u < kSubU; ++u)
              acc = __fma_rn(sbuf[threadIdx.x + 256 * u], col[s0 + threadIdx.x + 256 * u], acc);
          } else {
            for (int u = 0; u < kSubU; ++u) {
              const int64_t i = s0 + threadIdx.x + 256 * u;
              if (i >= V.lo && i < V.hi) acc = __fma_rn(sbuf[threadIdx.x + 256 * u], col[i], acc);
            }
          }
          pa[q] = acc;
        }
      });
      fold_lanes<CG>(pa, gc, red, outA);
      if (threadIdx.x < gc) *part_at(j, t, ch, g0 + threadIdx.x) = outA[threadIdx.x];
    }
    if (!last_block(S, j.nch, &s_flag)) continue;
    // ---- last block: row kk (Householder.h:121-126), then down-dating
    const int nw = V.nwork;
    const double tau = V.tau;
    for (int q = threadIdx.x; q < nw; q += blockDim.x) {
      const int s = V.work[q];
      double* a = wcol(j, t, c, s);
      const double w = chunk_total(j, t, q, -1);
      const double qk = __ldcg(a + kk);
      const double tmp = __dadd_rn(w, qk);
      a[kk] = __dsub_rn(qk, __dmul_rn(tau, tmp));
      S->ntmp[s] = -tmp;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      const int k = V.k;
      if (rows - kk == 1) {
        // a one-row tail: row kk of the other columns scaled by 1 - tau
        for (int p = kk + 1; p < k; ++p) {
          double* a = wcol(j, t, c, S->pos2col[p]);
          a[kk] = __dmul_rn(__ldcg(a + kk), __dsub_rn(1.0, tau));
        }
        if (S->upd_y) {
          double* a = wcol(j, t, c, k);
          a[kk] = __dmul_rn(__ldcg(a + kk), __dsub_rn(1.0, tau));
        }
      }
      pcol[kk] = S->beta;
      // LAWN 176 norm down-dating (ColPivHouseholderQR.h:549-572); the
      // recomputations happen in pass B, which sums the updated columns
      int rec_any = 0, nsum = 0;
      for (int p = kk + 1; p < k; ++p) {
        if (S->nupd[p] == 0.0) continue;
        double temp = __ddiv_rn(fabs(__ldcg(wcol(j, t, c, S->pos2col[p]) + kk)), S->nupd[p]);
        temp = __dmul_rn(__dadd_rn(1.0, temp), __dsub_rn(1.0, temp));
        temp = temp < 0.0 ? 0.0 : temp;
        const double ratio = __ddiv_rn(S->nupd[p], S->ndir[p]);
        const double temp2 = __dmul_rn(temp, __dmul_rn(ratio, ratio));
        if (temp2 <= kDowndateThr) {
          S->sum_store[nsum] = S->pos2col[p];
          S->sum_norm[nsum] = 1;
          ++nsum;
          rec_any = 1;
        } else {
          S->nupd[p] = __dmul_rn(S->nupd[p], __dsqrt_rn(temp));
        }
      }
      const int next = kk + 1;
      if (next >= S->size) {
        nsum = 0;  // no later step reads the norms
      } else if (rec_any) {
        // the pivot of step kk + 1 depends on the recomputed norms (and on
        // NaN norms through the scan's running maximum): the tails of every
        // remaining column, which a recomputation step can afford
        for (int p = next; p < k; ++p) {
          bool flagged = false;
          for (int q = 0; q < nsum && !flagged; ++q) flagged = S->sum_store[q] == S->pos2col[p];
          if (flagged) continue;
          S->sum_store[nsum] = S->pos2col[p];
          S->sum_norm[nsum] = 0;
          ++nsum;
        }
      } else {
        select_pivot(S, next, (double)rows);
        S->upd_y_next = S->nonzero == S->size;
        S->sum_store[0] = S->pos2col[next];
        S->sum_norm[0] = 0;
        nsum = 1;
      }
      S->rec_any = rec_any;
      S->nsum = nsum;
      S->ticket = 0;
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------ solve --
__global__ void qr_solve_kernel(QrJob j) {
  const int cnt = job_count(j);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < cnt; t += gridDim.x * blockDim.x) {
    const QrState* S = j.state + t;
    if (!S->active) continue;
    const int c = j.list[j.list_off + t];
    const rrg_cand cd = j.b.cands[c];
    const int k = S->k, r = S->nonzero, size = S->size;
    double cvec[kQrMaxCols];
    const double* yq = wcol(j, t, c, k);
    for (int i = 0; i < r; ++i) cvec[i] = yq[i];
    for (int kk = r - 1; kk >= 0; --kk) {
      const double* rc = wcol(j, t, c, S->pos2col[kk]);
      cvec[kk] = __ddiv_rn(cvec[kk], rc[kk]);
      for (int i = 0; i < kk; ++i) cvec[i] = __dsub_rn(cvec[i], __dmul_rn(cvec[kk], rc[i]));
    }
    double* out = j.coefs + cd.coef_offset;
    for (int q = 0; q < k; ++q) out[q] = 0.0;
    for (int i = 0; i < r; ++i) out[S->perm[i]] = cvec[i];
    j.res[c].rank = r;
    if (j.count_bytes) {
      // the copy, then every remaining column (y while kk < rank) read and
      // written once per step
      double cols = (double)(2 * k + 1);
      for (int kk = 0; kk < size; ++kk) cols += 2.0 * (double)((kk < r ? k + 1 : k) - kk);
      atomicAdd(reinterpret_cast<unsigned long long*>(j.status + kStatusQrBytes),
                (unsigned long long)(cols * 8.0 * (double)j.ds.n));
    }
  }
}

template <int CG>
bool launch_passes(const QrJob& job, int blocks, cudaStream_t st, int64_t* launches) {
  const int steps = job.max_steps > 0 && job.max_steps < job.max_cols ? job.max_steps : job.max_cols - 1;
  // tickets (and every other field) start at zero
  if (cudaMemsetAsync(job.state, 0, sizeof(QrState) * (size_t)job.n_list, st) != cudaSuccess) {
    cudaGetLastError();
    rrc::set_error("QR state reset failed");
    return false;
  }
  qr_sums_kernel<CG, true><<<blocks, 256, 0, st>>>(job, -1);
  if (!launch_ok("QR init pass")) return false;
  for (int kk = 0; kk < steps; ++kk) {
    qr_passA_kernel<CG><<<blocks, 256, 0, st>>>(job, kk);
    qr_sums_kernel<CG, false><<<blocks, 256, 0, st>>>(job, kk);
    if (!launch_ok("QR step passes")) return false;
  }
  const int sb = (int)((job.n_list + 127) / 128);
  qr_solve_kernel<<<sb < 1 ? 1 : sb, 128, 0, st>>>(job);
  if (!launch_ok("QR solve")) return false;
  if (launches) *launches += 2 + 2 * (int64_t)steps;
  return true;
}

}  // namespace

size_t qr_chunk_scratch_bytes(int64_t n_list, int64_t rows, int max_cols) {
  const int64_t nch = (rows + kQC - 1) / kQC;
  const size_t st = round_up(sizeof(QrState) * (size_t)n_list, 256);
  return st + sizeof(double) * (size_t)n_list * (size_t)(nch + 1) * (size_t)max_cols;
}

void qr_chunk_bind(QrJob& job, void* scratch) {
  job.nch = (int)((job.ds.n + kQC - 1) / kQC);
  const size_t st = round_up(sizeof(QrState) * (size_t)job.n_list, 256);
  job.state = static_cast<QrState*>(scratch);
  job.part = reinterpret_cast<double*>(static_cast<char*>(scratch) + st);
}

int qr_chunk_blocks_per_sm(int max_cols) {
  int a = 0, b = 0;
  cudaError_t e1, e2;
  if (max_cols <= 5) {
    e1 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, qr_sums_kernel<4, false>, 256, 0);
    e2 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, qr_passA_kernel<4>, 256, 0);
  } else if (max_cols <= 9) {
    e1 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, qr_sums_kernel<8, false>, 256, 0);
    e2 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, qr_passA_kernel<8>, 256, 0);
  } else {
    e1 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, qr_sums_kernel<16, false>, 256, 0);
    e2 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, qr_passA_kernel<16>, 256, 0);
  }
  if (e1 != cudaSuccess || e2 != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  const int m = a < b ? a : b;
  return m < 1 ? 1 : m;
}

bool launch_qr_chunked(const QrJob& job, int blocks, cudaStream_t st, int64_t* launches) {
  if (job.n_list <= 0) return true;
  if (job.max_cols > kQrMaxCols || job.max_cols < 2) {
    rrc::set_error("QR launch: column bound outside the kernel's range");
    return false;
  }
  if (blocks < 1) blocks = 1;
  // the work set of a pass: the columns after the pivot and y (at most k)
  const int w = job.max_cols - 1;
  if (w <= 4) return launch_passes<4>(job, blocks, st, launches);
  if (w <= 8) return launch_passes<8>(job, blocks, st, launches);
  return launch_passes<16>(job, blocks, st, launches);
}

}  // namespace rrd
