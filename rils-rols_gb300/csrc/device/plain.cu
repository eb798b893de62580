// Plain FP64 fitness path: the drop-in form of tune_constants + fitness
// (rils_rols_cpp/rils_rols_cpp.cpp:445-541).
//
//   plain_eval   evaluates every factor program of a candidate on every row
//                (node::evaluate_all, node.cpp:5-95) into the A arena;
//   plain_qr     column-pivoted Householder least squares with the pivot,
//                rank and norm-down-dating rules of Eigen's
//                ColPivHouseholderQR (eigen/Eigen/src/QR/ColPivHouseholderQR.h:482-608)
//                on [A | 1 | y], one block per candidate (small row counts
//                and the allocation-free entry; qr_chunk.cu spreads larger
//                ones over the GPU with the same bits);
//   plain_resid  the rebuilt sum  sum_i c_i * f_i  with the drop / snap rules
//                of rils_rols_cpp.cpp:488-517 and its squared residual;
//   finalize     R2, RMSE and the NaN sentinel (rils_rols_cpp.cpp:40-49, 520-541).
#include <cfloat>
#include <cstdint>

#include "../common/rr_math.h"
#include "../common/rr_sum.h"
#include "common.cuh"
#include "plain.cuh"
#include "qr_ops.cuh"
#include "reduce.cuh"

namespace rrd {

namespace {

constexpr int kMaxK = RRG_MAX_TERMS;

__device__ __forceinline__ double bin64(int base, double a, double b) {
  switch (base) {
    case RRG_ADD: return __dadd_rn(a, b);
    case RRG_SUB: return __dsub_rn(a, b);
    case RRG_MUL: return __dmul_rn(a, b);
    case RRG_DIV: return __ddiv_rn(a, b);
    case RRG_POW: return rr_pow(a, b);
    case RRG_LT: return a < b ? 1.0 : 0.0;
    case RRG_EQ: return a == b ? 1.0 : 0.0;
    case RRG_NE: return a != b ? 1.0 : 0.0;
    case RRG_MIN: return a < b ? a : b;
    case RRG_MAX: return a > b ? a : b;
    default: return __longlong_as_double(0x7ff8000000000000ll);
  }
}

// Runs the code of one candidate on `row`; factor slot s is written to
// out[s * n_pad + row].  Spill stack in shared memory, stride blockDim.x.
// Table programs also read columns of T (same rows, column stride n_pad).
__device__ __forceinline__ void run_row64(const uint32_t* code, int len, const double* consts, const DevData& ds,
                                          int64_t row, double* st, double* out, const double* T, uint32_t* status) {
  double tos = 0.0;
  int sp = 0;
  const int stride = blockDim.x;
  for (int pc = 0; pc < len; ++pc) {
    const uint32_t w = code[pc];
    const int op = (int)(w & 0xffu);
    const uint32_t arg = w >> 8;
    switch (op) {
      case RRG_OP_LDV: tos = ds.X64[(int64_t)arg * ds.n_pad + row]; break;
      case RRG_OP_LDC: tos = consts[arg]; break;
      case RRG_OP_PSV:
        if (sp >= RRG_MAX_STACK) { atomicOr(status, ST_STACK); return; }
        st[sp++ * stride] = tos;
        tos = ds.X64[(int64_t)arg * ds.n_pad + row];
        break;
      case RRG_OP_PSC:
        if (sp >= RRG_MAX_STACK) { atomicOr(status, ST_STACK); return; }
        st[sp++ * stride] = tos;
        tos = consts[arg];
        break;
      case RRG_OP_SIN: tos = rr_sin(tos); break;
      case RRG_OP_COS: tos = rr_cos(tos); break;
      case RRG_OP_LN: tos = rr_log(tos); break;
      case RRG_OP_EXP: tos = rr_exp(tos); break;
      case RRG_OP_SQRT: tos = __dsqrt_rn(tos); break;
      case RRG_OP_SQR: tos = __dmul_rn(tos, tos); break;
      case kOpLDT: tos = T[(int64_t)arg * ds.n_pad + row]; break;
      case kOpPST:
        if (sp >= RRG_MAX_STACK) { atomicOr(status, ST_STACK); return; }
        st[sp++ * stride] = tos;
        tos = T[(int64_t)arg * ds.n_pad + row];
        break;
      case RRG_OP_EMIT:
        out[(int64_t)arg * ds.n_pad + row] = tos;
        sp = 0;
        break;
      default: {
        const int kk = op - RRG_OP_BIN;
        if (kk < 0 || kk >= 8 * RRG_N_BASE) { atomicOr(status, ST_BAD_CODE); return; }
        const int base = kk >> 3, src = (kk & 7) >> 1, dir = kk & 1;
        double other;
        if (src == RRG_SRC_S) {
          if (sp <= 0) { atomicOr(status, ST_STACK); return; }
          other = st[--sp * stride];
        } else if (src == RRG_SRC_V) {
          other = ds.X64[(int64_t)arg * ds.n_pad + row];
        } else if (src == kSrcT) {
          other = T[(int64_t)arg * ds.n_pad + row];
        } else {
          other = consts[arg];
        }
        tos = dir == RRG_DIR_N ? bin64(base, other, tos) : bin64(base, tos, other);
      }
    }
  }
}

// One-column table program on rows [r0, r1) of this block, written to Ac;
// the column's statistics (NaN, infinite or overflowing square, non-trivial
// tail, largest finite magnitude) merged into *cs.
__device__ __forceinline__ void eval_column_stats(const uint32_t* code, int len, const double* consts,
                                                  const DevData& ds, int64_t r0, int64_t r1, double* st, double* Ac,
                                                  const double* T, uint32_t* status, ColStat* cs) {
  uint32_t f = 0;
  unsigned long long mx = 0;
  for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    run_row64(code, len, consts, ds, r, st, Ac, T, status);
    const double v = Ac[r];
    const double a = fabs(v);
    if (v != v) {
      f |= kCsNaN;
    } else if (!(a <= 1.35e154)) {  // infinite, or its square overflows
      f |= kCsBig;
    } else {
      const unsigned long long bits = (unsigned long long)__double_as_longlong(a);
      mx = bits > mx ? bits : mx;
    }
    if (r >= 1 && !(a <= 1e-150)) f |= kCsTail;
  }
  f = __reduce_or_sync(0xffffffffu, f);
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long t = __shfl_xor_sync(0xffffffffu, mx, o);
    mx = t > mx ? t : mx;
  }
  if ((threadIdx.x & 31) == 0) {
    if (f) atomicOr(&cs->flags, f);
    if (mx) atomicMax(&cs->maxabs, mx);
  }
}

}  // namespace

// ------------------------------------------------------------- kernels ----
__global__ void __launch_bounds__(256) table_eval_list_kernel(DevBatch b, DevData ds, const PlainCand* pc,
                                                               const int32_t* cols, const int32_t* count,
                                                               int max_nbc, double* A, uint32_t* status,
                                                               ColStat* cst) {
  extern __shared__ double smem[];
  const int cnt = *count;
  if (cnt <= 0) return;
  const int nbc = (int)max(1, min(max_nbc, (int)((gridDim.x + cnt - 1) / cnt)));
  const int64_t items = (int64_t)cnt * nbc;
  double* st = smem + threadIdx.x;
  uint32_t* code_s = reinterpret_cast<uint32_t*>(smem + RRG_MAX_STACK * blockDim.x);
  for (int64_t w = blockIdx.x; w < items; w += gridDim.x) {
    const int c = cols[w / nbc];
    const int bi = (int)(w % nbc);
    const rrg_cand cd = b.cands[c];
    const int64_t r0 = ds.n * (int64_t)bi / nbc, r1 = ds.n * (int64_t)(bi + 1) / nbc;
    const bool staged = cd.code_len <= kMaxCodeSmem;
    __syncthreads();  // the previous item's program is no longer read
    if (staged)
      for (int i = threadIdx.x; i < cd.code_len; i += blockDim.x) code_s[i] = b.code[cd.code_offset + i];
    __syncthreads();
    const uint32_t* code = staged ? code_s : b.code + cd.code_offset;
    eval_column_stats(code, cd.code_len, b.consts, ds, r0, r1, st, A + pc[c].a_col * ds.n_pad, A, status,
                      &cst[pc[c].a_col]);
  }
}

// grid (blocks per candidate, candidates); rows of block b: [b*n/nb, (b+1)*n/nb)
__global__ void __launch_bounds__(256) plain_eval_kernel(DevBatch b, DevData ds, const PlainCand* pc,
                                                          const int32_t* list, int cand0, double* A, uint32_t* status,
                                                          ColStat* cst) {
  extern __shared__ double smem[];
  const int c = list ? list[cand0 + blockIdx.y] : cand0 + blockIdx.y;
  const rrg_cand cd = b.cands[c];
  const int nb = gridDim.x;
  const int64_t r0 = ds.n * (int64_t)blockIdx.x / nb, r1 = ds.n * (int64_t)(blockIdx.x + 1) / nb;
  double* st = smem + threadIdx.x;  // spill stack, RRG_MAX_STACK * blockDim.x doubles
  uint32_t* code_s = reinterpret_cast<uint32_t*>(smem + RRG_MAX_STACK * blockDim.x);
  const bool staged = cd.code_len <= kMaxCodeSmem;
  if (staged)
    for (int i = threadIdx.x; i < cd.code_len; i += blockDim.x) code_s[i] = b.code[cd.code_offset + i];
  __syncthreads();
  const uint32_t* code = staged ? code_s : b.code + cd.code_offset;
  double* Ac = A + pc[c].a_col * ds.n_pad;
  if (cst) {
    eval_column_stats(code, cd.code_len, b.consts, ds, r0, r1, st, Ac, A, status, &cst[pc[c].a_col]);
    return;
  }
  for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x)
    run_row64(code, cd.code_len, b.consts, ds, r, st, Ac, A, status);
}

namespace {

// QSUM (csrc/common/rr_sum.h) of term(i, acc) over rows [start, rows) by the
// block's 256 threads, thread t being lane t: per chunk of RR_CHUNK rows the
// lanes' chains are folded as RR256, and the chunk totals are added in order
// from 0.  Every thread gets the total.
template <class F>
__device__ __forceinline__ double block_qsum(int64_t start, int64_t rows, double* red, F&& term) {
  double total = 0.0;
  for (int64_t c0 = start / RR_CHUNK * RR_CHUNK; c0 < rows; c0 += RR_CHUNK) {
    const int64_t hi = c0 + RR_CHUNK < rows ? c0 + RR_CHUNK : rows;
    double p = 0.0;
    for (int64_t i = c0 + threadIdx.x; i < hi; i += blockDim.x)
      if (i >= start) p = term(i, p);
    total = __dadd_rn(total, block_sum(p, red));
  }
  return total;
}

// The same for cnt columns at once: term(i, part) adds row i's terms to
// part[0 .. cnt); the totals land in tot[0 .. cnt) (shared).
template <int KB, class F>
__device__ __forceinline__ void block_qsum_vec(int64_t start, int64_t rows, int cnt, double* red, double* tmp,
                                               double* tot, F&& term) {
  for (int j = threadIdx.x; j < cnt; j += blockDim.x) tot[j] = 0.0;
  __syncthreads();
  for (int64_t c0 = start / RR_CHUNK * RR_CHUNK; c0 < rows; c0 += RR_CHUNK) {
    const int64_t hi = c0 + RR_CHUNK < rows ? c0 + RR_CHUNK : rows;
    double part[KB];
#pragma unroll
    for (int j = 0; j < KB; ++j) part[j] = 0.0;
    for (int64_t i = c0 + threadIdx.x; i < hi; i += blockDim.x)
      if (i >= start) term(i, part);
    // element-wise block fold (warps, then the eight warp totals in order)
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
#pragma unroll
    for (int j = 0; j < KB; ++j)
      if (j < cnt) {
        const double v = warp_sum(part[j]);
        if (l == 0) red[w * KB + j] = v;
      }
    __syncthreads();
    for (int j = threadIdx.x; j < cnt; j += blockDim.x) {
      double s = 0.0;
      for (int i = 0; i < nw; ++i) s = __dadd_rn(s, red[i * KB + j]);
      tot[j] = __dadd_rn(tot[j], s);
    }
    __syncthreads();
  }
  (void)tmp;
}

// Householder reflector of col[kk..rows) (Householder.h:67-96 semantics).
// Returns tau; writes beta to col[kk] and the essential part below it.
__device__ double make_householder_col(double* col, int64_t rows, int kk, double* red) {
  const double tail_sq =
      (rows - kk == 1) ? 0.0 : block_qsum(kk + 1, rows, red, [&](int64_t i, double p) { return __fma_rn(col[i], col[i], p); });
  const double c0 = col[kk];
  double tau, beta;
  __syncthreads();
  if (tail_sq <= DBL_MIN) {
    tau = 0.0;
    beta = c0;
    for (int64_t i = kk + 1 + threadIdx.x; i < rows; i += blockDim.x) col[i] = 0.0;
  } else {
    beta = __dsqrt_rn(__dadd_rn(__dmul_rn(c0, c0), tail_sq));
    if (c0 >= 0.0) beta = -beta;
    const double den = __dsub_rn(c0, beta);
    const double rden = __drcp_rn(den);
    for (int64_t i = kk + 1 + threadIdx.x; i < rows; i += blockDim.x) col[i] = div_by(col[i], den, rden);
    tau = __ddiv_rn(__dsub_rn(beta, c0), beta);
  }
  __syncthreads();
  if (threadIdx.x == 0) col[kk] = beta;
  __syncthreads();
  return tau;
}

// Applies H_kk = I - tau v v^T (v = [1, colp[kk][kk+1..]]) to the columns
// colp[c_lo..c_hi) (rows kk..rows-1).  Householder.h:116-133 semantics.
template <int KB>
__device__ void apply_householder_cols(double* const* colp, int64_t rows, int kk, double tau, int c_lo, int c_hi,
                                       double* red, double* sh_tmp) {
  const int cnt = c_hi - c_lo;
  if (cnt <= 0) return;
  if (rows - kk == 1) {
    for (int j = threadIdx.x; j < cnt; j += blockDim.x) {
      double* q = colp[c_lo + j] + kk;
      *q = __dmul_rn(*q, __dsub_rn(1.0, tau));
    }
    __syncthreads();
    return;
  }
  if (tau == 0.0) return;
  const double* v = colp[kk];
  double* cp[KB];
#pragma unroll
  for (int j = 0; j < KB; ++j) cp[j] = j < cnt ? colp[c_lo + j] : nullptr;
  block_qsum_vec<KB>(kk + 1, rows, cnt, red, nullptr, sh_tmp, [&](int64_t i, double (&part)[KB]) {
    const double vi = v[i];
#pragma unroll
    for (int j = 0; j < KB; ++j)
      if (j < cnt) part[j] = __fma_rn(vi, cp[j][i], part[j]);
  });
  // tmp_j += Q[kk, j]; Q[kk, j] -= tau * tmp_j
  if (threadIdx.x == 0) {
    for (int j = 0; j < cnt; ++j) {
      double* q = colp[c_lo + j] + kk;
      sh_tmp[j] = __dadd_rn(sh_tmp[j], *q);
      *q = __dsub_rn(*q, __dmul_rn(tau, sh_tmp[j]));
    }
  }
  __syncthreads();
  double t[KB];
#pragma unroll
  for (int j = 0; j < KB; ++j) t[j] = j < cnt ? sh_tmp[j] : 0.0;
  for (int64_t i = kk + 1 + threadIdx.x; i < rows; i += blockDim.x) {
    const double tv = __dmul_rn(tau, v[i]);
#pragma unroll
    for (int j = 0; j < KB; ++j)
      if (j < cnt) cp[j][i] = __fma_rn(-tv, t[j], cp[j][i]);
  }
  __syncthreads();
}

// One block per tuned candidate: column-pivoted QR least squares on
// [A | 1 | y] with every sum in QSUM order (bit-identical to the chunked
// passes of qr_chunk.cu).  KB bounds the columns (k + 1) so that per-column
// accumulators stay in registers.  Pivoting swaps column pointers, not data.
template <int KB>
__global__ void __launch_bounds__(256) plain_qr_kernel_t(DevBatch b, DevData ds, const PlainCand* pc,
                                                          const int32_t* list, int cand0, const double* A, double* M,
                                                          double* coefs, rrg_result* res, uint32_t* status,
                                                          const int32_t* colmap) {
  extern __shared__ double smem[];
  const int c = list ? list[cand0 + blockIdx.x] : cand0 + blockIdx.x;
  const rrg_cand cd = b.cands[c];
  if (cd.mode != RRG_TUNED || (pc[c].pad & 1)) return;  // pad bit 0: outcome already written
  const int k = pc[c].k;
  if (k + 1 > KB || k > kMaxK) {
    if (threadIdx.x == 0) atomicOr(status, ST_TOO_LARGE);
    return;
  }
  double* red = smem;                       // 8 * (kMaxK + 1)
  double* sh_tmp = red + 8 * (kMaxK + 1);   // kMaxK + 1
  double* nupd = sh_tmp + (kMaxK + 1);      // kMaxK
  double* ndir = nupd + kMaxK;              // kMaxK
  double* hc = ndir + kMaxK;                // kMaxK
  int* perm = reinterpret_cast<int*>(hc + kMaxK);
  int* misc = perm + kMaxK;                 // [0] pivot, [1] nonzero, [2..] recompute flags
  __shared__ double* colp[KB];              // current position -> column storage

  double* Q = M + pc[c].m_col * ds.n_pad;
  const int64_t ld = ds.n_pad, rows = ds.n;
  for (int j = threadIdx.x; j <= k; j += blockDim.x) colp[j] = Q + (int64_t)j * ld;
  // [A | 1 | y] into the working columns
  for (int j = 0; j <= k; ++j) {
    double* dst = Q + (int64_t)j * ld;
    if (j < k - 1) {
      const double* src = factor_column(A, ds.n_pad, pc[c].a_col, j, colmap);
      for (int64_t r = threadIdx.x; r < rows; r += blockDim.x) dst[r] = src[r];
    } else if (j == k - 1) {
      for (int64_t r = threadIdx.x; r < rows; r += blockDim.x) dst[r] = 1.0;
    } else {
      for (int64_t r = threadIdx.x; r < rows; r += blockDim.x) dst[r] = ds.y64[r];
    }
  }
  __syncthreads();
  // initial column norms
  block_qsum_vec<KB>(0, rows, k, red, nullptr, sh_tmp, [&](int64_t i, double (&part)[KB]) {
#pragma unroll
    for (int j = 0; j < KB; ++j)
      if (j < k) {
        const double q = colp[j][i];
        part[j] = __fma_rn(q, q, part[j]);
      }
  });
  const double rows_thr = (double)ds.n;
  const int size = (int)(rows < k ? rows : k);
  if (threadIdx.x == 0) {
    for (int j = 0; j < k; ++j) {
      ndir[j] = __dsqrt_rn(sh_tmp[j]);
      nupd[j] = ndir[j];
      perm[j] = j;
    }
    misc[1] = size;
  }
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
      if (misc[1] == size && __dmul_rn(bign, bign) < __dmul_rn(thr_helper, rows_thr - kk)) misc[1] = kk;
      misc[0] = big;
      if (big != kk) {
        double t = nupd[kk]; nupd[kk] = nupd[big]; nupd[big] = t;
        t = ndir[kk]; ndir[kk] = ndir[big]; ndir[big] = t;
        int p = perm[kk]; perm[kk] = perm[big]; perm[big] = p;
        double* cq = colp[kk]; colp[kk] = colp[big]; colp[big] = cq;
      }
    }
    __syncthreads();
    const double tau = make_householder_col(colp[kk], rows, kk, red);
    if (threadIdx.x == 0) hc[kk] = tau;
    // reflector kk reaches the right-hand side only while kk < rank
    const int c_hi = misc[1] == size ? k + 1 : k;
    apply_householder_cols<KB>(colp, rows, kk, tau, kk + 1, c_hi, red, sh_tmp);
    // LAWN 176 norm down-dating (ColPivHouseholderQR.h:549-572)
    int* rec = misc + 2;
    if (threadIdx.x == 0) {
      for (int j = kk + 1; j < k; ++j) {
        rec[j] = 0;
        if (nupd[j] != 0.0) {
          double temp = __ddiv_rn(fabs(colp[j][kk]), nupd[j]);
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
    for (int j = kk + 1; j < k; ++j) {
      if (!rec[j]) continue;  // uniform
      const double* cj = colp[j];
      const double s = block_qsum(kk + 1, rows, red, [&](int64_t i, double p) { return __fma_rn(cj[i], cj[i], p); });
      if (threadIdx.x == 0) {
        ndir[j] = __dsqrt_rn(s);
        nupd[j] = ndir[j];
      }
      __syncthreads();
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int r = misc[1];
    double cvec[kMaxK];
    for (int i = 0; i < r; ++i) cvec[i] = colp[k][i];
    for (int kk = r - 1; kk >= 0; --kk) {
      cvec[kk] = __ddiv_rn(cvec[kk], colp[kk][kk]);
      for (int i = 0; i < kk; ++i) cvec[i] = __dsub_rn(cvec[i], __dmul_rn(cvec[kk], colp[kk][i]));
    }
    double* out = coefs + cd.coef_offset;
    for (int j = 0; j < k; ++j) out[j] = 0.0;
    for (int i = 0; i < r; ++i) out[perm[i]] = cvec[i];
    res[c].rank = r;
  }
}

}  // namespace

int plain_qr_bucket(int cols) { return cols <= 4 ? 4 : (cols <= 8 ? 8 : (cols <= 16 ? 16 : kMaxK + 1)); }

bool launch_plain_qr(int max_cols, int grid, cudaStream_t st, DevBatch b, DevData ds, const PlainCand* pc,
                     const int32_t* list, int cand0, const double* A, double* M, double* coefs, rrg_result* res,
                     uint32_t* status, const int32_t* colmap) {
  if (grid <= 0) return true;
  const size_t sm = plain_qr_smem();
  if (max_cols <= 4)
    plain_qr_kernel_t<4><<<grid, 256, sm, st>>>(b, ds, pc, list, cand0, A, M, coefs, res, status, colmap);
  else if (max_cols <= 8)
    plain_qr_kernel_t<8><<<grid, 256, sm, st>>>(b, ds, pc, list, cand0, A, M, coefs, res, status, colmap);
  else if (max_cols <= 16)
    plain_qr_kernel_t<16><<<grid, 256, sm, st>>>(b, ds, pc, list, cand0, A, M, coefs, res, status, colmap);
  else
    plain_qr_kernel_t<kMaxK + 1><<<grid, 256, sm, st>>>(b, ds, pc, list, cand0, A, M, coefs, res, status, colmap);
  return launch_ok("launch_plain_qr");
}



// grid (ceil(n / RR_CHUNK), candidates): SSE of the rebuilt sum per chunk of
// RR_CHUNK rows in the fixed order of csrc/common/rr_sum.h
__global__ void __launch_bounds__(256) plain_resid_kernel(DevBatch b, DevData ds, const PlainCand* pc,
                                                           const int32_t* list, int cand0, const double* A,
                                                           const double* coefs, double* partial,
                                                           const int32_t* colmap, const int32_t* dcount) {
  if (dcount && cand0 + (int)blockIdx.y >= *dcount) return;
  __shared__ double red[32];
  __shared__ double cs[kMaxK];
  __shared__ int kind[kMaxK];  // 0 skip, 1 free term, 2 bare factor, 3 scaled factor
  __shared__ const double* colp[kMaxK];
  const int c = list ? list[cand0 + blockIdx.y] : cand0 + blockIdx.y;
  const rrg_cand cd = b.cands[c];
  const int nb = gridDim.x;
  const bool tuned = cd.mode == RRG_TUNED;
  if (tuned && (pc[c].pad & 1)) {
    // all-NaN coefficients: every row's rebuilt sum is NaN
    if (threadIdx.x == 0)
      partial[(int64_t)c * nb + blockIdx.x] = blockIdx.x == 0 ? __longlong_as_double(0x7ff8000000000000ll) : 0.0;
    return;
  }
  const int k = pc[c].k;
  const int m = tuned ? k - 1 : 1;
  if (tuned) {
    for (int i = threadIdx.x; i < k; i += blockDim.x) {
      const double ci = coefs[cd.coef_offset + i];
      cs[i] = ci;
      kind[i] = fabs(ci) < kEps12 ? 0 : (i == m ? 1 : (fabs(ci - 1) < kEps12 ? 2 : 3));
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < m; i += blockDim.x) colp[i] = factor_column(A, ds.n_pad, pc[c].a_col, i, colmap);
  __syncthreads();
  const int64_t r0 = (int64_t)blockIdx.x * RR_CHUNK, r1 = min(ds.n, r0 + (int64_t)RR_CHUNK);
  double acc = 0.0;
  for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    double yp;
    if (tuned) {
      yp = 0.0;
      bool have = false;
      for (int i = 0; i < k; ++i) {
        const int kd = kind[i];
        if (kd == 0) continue;
        const double term = kd == 1 ? __dmul_rn(cs[i], 1.0) : (kd == 2 ? colp[i][r] : __dmul_rn(cs[i], colp[i][r]));
        yp = have ? __dadd_rn(yp, term) : term;
        have = true;
      }
    } else {
      yp = colp[0][r];
    }
    const double e = __dsub_rn(ds.y64[r], yp);
    acc = __dadd_rn(acc, __dmul_rn(e, e));
  }
  const double s = block_sum(acc, red);
  if (threadIdx.x == 0) partial[(int64_t)c * nb + blockIdx.x] = s;
}

// one thread per candidate: R2, RMSE, sentinel, rebuilt size
__global__ void finalize_kernel(DevBatch b, DevData ds, const int32_t* list, int cand0, int cand1,
                                const double* partial, int nb, const double* coefs, rrg_result* res,
                                uint32_t flags_or, const double* sse_direct, const int32_t* dcount) {
  const int i = cand0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cand1 || (dcount && i >= *dcount)) return;
  const int c = list ? list[i] : i;
  const rrg_cand cd = b.cands[c];
  double ssr = 0.0;
  if (sse_direct && !(sse_direct[c] < 0.0)) {
    ssr = sse_direct[c];
  } else {
    for (int j = 0; j < nb; ++j) ssr = __dadd_rn(ssr, partial[(int64_t)c * nb + j]);
  }
  const double r2 = __dsub_rn(1.0, __ddiv_rn(ssr, ds.sst));
  const double rmse = __dsqrt_rn(__ddiv_rn(ssr, (double)ds.n));
  rrg_result out = res[c];
  out.flags |= flags_or;
  int size = 0;
  if (cd.mode == RRG_TUNED) {
    const int m = cd.n_factors;
    int kept = 0;
    for (int i = 0; i <= m; ++i) {
      const double ci = coefs[cd.coef_offset + i];
      if (fabs(ci) < kEps12) continue;
      ++kept;
      if (i == m) size += 1;
      else if (fabs(ci - 1) < kEps12) size += b.factors[cd.first_factor + i].n_nodes;
      else size += 2 + b.factors[cd.first_factor + i].n_nodes;
    }
    size = kept == 0 ? 1 : size + kept - 1;
    out.n_coef = m + 1;
    if (out.rank < m + 1) out.flags |= RRG_F_RANK_DEFICIENT;
  } else {
    size = b.factors[cd.first_factor].n_nodes;
    out.n_coef = 0;
    out.rank = 0;
  }
  if (r2 != r2 || rmse != rmse) {
    out.loss = 1000;
    out.rmse = 1000;
    out.size = 1000;
    out.flags |= RRG_F_NONFINITE;
  } else {
    out.loss = __dsub_rn(1.0, r2);
    out.rmse = rmse;
    out.size = size;
  }
  res[c] = out;
}

// ----------------------------------------------------------- launchers ----
// Result records of the listed candidates back to zero before a re-scoring.
__global__ void clear_results_kernel(const int32_t* list, int n, rrg_result* res, const int32_t* dcount) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && !(dcount && i >= *dcount)) res[list[i]] = rrg_result{};
}

// The outcome of the column-pivoted QR (ColPivHouseholderQR.h:482-608, as
// restated by the oracle) on [f_0 .. f_{m-1}, 1] when its first pivot has a
// non-finite norm.  Pivot selection keeps the first maximum under '>', so a
// NaN norm is chosen only when it heads the remaining columns and a +inf
// norm beats every finite one: the first pivot is non-finite when column 0's
// norm is NaN or some column's norm is +inf (an infinite value or an
// overflowing square, without NaN).  With a non-trivial tail in every column
// (some row after the first above 1e-150: the reflector is formed and every
// norm is non-zero), that pivot yields tau = NaN, which turns every other
// column and its norm NaN; no step cuts the rank (step 0 compares against an
// infinite or NaN threshold, later steps against NaN norms), so all
// coefficients are NaN at full rank.  A finite first pivot can leave a column
// with an exactly zero norm that a later step cuts, so NaN columns further
// on are left to the QR.
__global__ void sentinel_classify_kernel(DevBatch b, const int32_t* list, int cand0, int cnt, PlainCand* pc,
                                         const int32_t* colmap, const ColStat* cs, int64_t rows, double* coefs,
                                         rrg_result* res, uint32_t* decided, const int32_t* dcount) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cnt || (dcount && cand0 + i >= *dcount)) return;
  const int c = list[cand0 + i];
  const rrg_cand cd = b.cands[c];
  if (cd.mode != RRG_TUNED) return;
  const int k = pc[c].k;
  const int m = k - 1;
  if (m < 1 || rows < (int64_t)k + 2) return;
  bool tails = true, inf_norm = false, nan0 = false;
  for (int j = 0; j < m; ++j) {
    const ColStat st = cs[colmap[pc[c].a_col + j]];
    if (!(st.flags & kCsTail)) tails = false;
    if (st.flags & kCsNaN) {
      if (j == 0) nan0 = true;
    } else if (st.flags & kCsBig) {
      inf_norm = true;
    }
  }
  if (!tails) return;
  if (nan0 || inf_norm) {
    double* out = coefs + cd.coef_offset;
    for (int j = 0; j < k; ++j) out[j] = __longlong_as_double(0x7ff8000000000000ll);
    res[c].rank = k;
    pc[c].pad = 1;
    atomicAdd(decided, 1u);
    return;
  }
  // a NaN column further right: left to nan_gram_* (bit 1), which decides it
  // when the finite columns are well conditioned
  int nf = 0;
  bool any_nan = false;
  for (int j = 0; j < m; ++j) {
    if (cs[colmap[pc[c].a_col + j]].flags & kCsNaN) any_nan = true;
    else ++nf;
  }
  if (any_nan && nf + 1 <= kGramCols) pc[c].pad = 2;
}

// A NaN column at position q >= 1, column 0 finite, no infinite norm, every
// tail non-trivial: step 0 pivots on a finite column (NaN norms never win the
// '>' scan unless they head the remaining columns) with tau != 0, which turns
// every NaN-holding column entirely NaN; NaN columns do not move before step
// q, where the first of them heads the remaining columns and is chosen; its
// tau is NaN and every later norm and coefficient NaN, so the result is
// all-NaN coefficients at full rank, unless some step before q cut the rank.
// Steps before q factor finite columns only, so no cut is possible when the
// finite columns (the free term included) are well conditioned: every pivot
// of their pivoted Cholesky above 1e-8 of its column's squared norm and
// 1e-24 of the largest (the reference cuts at eps^2 ~ 5e-32 of the largest,
// and a remaining norm that far above it cannot be rounded down to it).
// nan_gram_kernel forms their FP64 Gram matrix (a certificate: any summation
// order), nan_gram_decide_kernel factors it.
constexpr int kGramE = kGramCols * (kGramCols + 1) / 2;

__device__ __forceinline__ int gram_finite_cols(const PlainCand& p, const int32_t* colmap, const ColStat* cs,
                                                const double* T, int64_t n_pad, const double* (&colp)[kGramCols]) {
  const int m = p.k - 1;
  int nf = 0;
  for (int j = 0; j < m && nf < kGramCols - 1; ++j) {
    const int32_t t = colmap[p.a_col + j];
    if (!(cs[t].flags & kCsNaN)) colp[nf++] = T + (int64_t)t * n_pad;
  }
  return nf;
}

__global__ void __launch_bounds__(256) nan_gram_kernel(const int32_t* list, int cnt, const PlainCand* pc,
                                                       const int32_t* colmap, const ColStat* cs, const double* T,
                                                       int64_t n, int64_t n_pad, double* gpart,
                                                       const int32_t* dcount) {
  __shared__ double red[8][kGramE];
  const int i = blockIdx.y;
  if (i >= cnt || (dcount && i >= *dcount)) return;
  const int c = list[i];
  const PlainCand p = pc[c];
  if (!(p.pad & 2)) return;
  const double* colp[kGramCols];
  const int nf = gram_finite_cols(p, colmap, cs, T, n_pad, colp);
  const int K = nf + 1;  // the free term last
  double part[kGramE];
#pragma unroll
  for (int e = 0; e < kGramE; ++e) part[e] = 0.0;
  const int64_t r0 = n * (int64_t)blockIdx.x / gridDim.x, r1 = n * (int64_t)(blockIdx.x + 1) / gridDim.x;
  for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    double v[kGramCols];
#pragma unroll
    for (int a = 0; a < kGramCols; ++a) v[a] = a < nf ? colp[a][r] : 1.0;
    int e = 0;
#pragma unroll
    for (int a = 0; a < kGramCols; ++a)
#pragma unroll
      for (int bb = a; bb < kGramCols; ++bb, ++e)
        if (bb < K) part[e] = fma(v[a], v[bb], part[e]);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
  for (int e = 0; e < kGramE; ++e) {
    const double t = warp_sum(part[e]);
    if (l == 0) red[w][e] = t;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < kGramE; e += blockDim.x) {
    double t = 0.0;
    for (int ww = 0; ww < 8; ++ww) t += red[ww][e];
    gpart[((int64_t)i * gridDim.x + blockIdx.x) * kGramE + e] = t;
  }
}

__global__ void nan_gram_decide_kernel(DevBatch b, const int32_t* list, int cnt, PlainCand* pc, const int32_t* colmap,
                                       const ColStat* cs, int nbx, const double* gpart, double* coefs,
                                       rrg_result* res, uint32_t* decided, const int32_t* dcount) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cnt || (dcount && i >= *dcount)) return;
  const int c = list[i];
  if (!(pc[c].pad & 2)) return;
  const int k = pc[c].k, m = k - 1;
  int nf = 0;
  for (int j = 0; j < m; ++j) nf += (cs[colmap[pc[c].a_col + j]].flags & kCsNaN) ? 0 : 1;
  const int K = nf + 1;
  double G[kGramCols][kGramCols];
  for (int a = 0, e = 0; a < kGramCols; ++a)
    for (int bb = a; bb < kGramCols; ++bb, ++e) {
      double t = 0.0;
      if (bb < K)
        for (int x = 0; x < nbx; ++x) t += gpart[((int64_t)i * nbx + x) * kGramE + e];
      G[a][bb] = t;
      G[bb][a] = t;
    }
  double d0[kGramCols], maxd = 0.0;
  for (int a = 0; a < K; ++a) {
    d0[a] = G[a][a];
    maxd = fmax(maxd, G[a][a]);
  }
  int piv[kGramCols];
  for (int a = 0; a < K; ++a) piv[a] = a;
  bool ok = maxd > 0.0 && maxd < 1e300;
  for (int s2 = 0; s2 < K && ok; ++s2) {
    int q = s2;
    for (int j = s2 + 1; j < K; ++j)
      if (G[j][j] > G[q][q]) q = j;
    const double dp = G[q][q];
    if (!(dp > 1e-8 * d0[piv[q]]) || !(dp > 1e-24 * maxd)) {
      ok = false;
      break;
    }
    if (q != s2) {
      for (int j = 0; j < K; ++j) { const double t = G[s2][j]; G[s2][j] = G[q][j]; G[q][j] = t; }
      for (int j = 0; j < K; ++j) { const double t = G[j][s2]; G[j][s2] = G[j][q]; G[j][q] = t; }
      const int t = piv[s2]; piv[s2] = piv[q]; piv[q] = t;
    }
    const double l = sqrt(dp);
    for (int a = s2 + 1; a < K; ++a) G[a][s2] /= l;
    for (int a = s2 + 1; a < K; ++a)
      for (int bb = s2 + 1; bb <= a; ++bb) {
        G[a][bb] -= G[a][s2] * G[bb][s2];
        G[bb][a] = G[a][bb];
      }
  }
  if (!ok) {
    pc[c].pad = 0;
    return;
  }
  double* out = coefs + b.cands[c].coef_offset;
  for (int j = 0; j < k; ++j) out[j] = __longlong_as_double(0x7ff8000000000000ll);
  res[c].rank = k;
  pc[c].pad = 1;
  atomicAdd(decided, 1u);
}

size_t plain_eval_smem() { return RRG_MAX_STACK * 256 * sizeof(double) + kMaxCodeSmem * sizeof(uint32_t); }
size_t plain_qr_smem() {
  return (8 * (kMaxK + 1) + (kMaxK + 1) + 3 * kMaxK) * sizeof(double) + (kMaxK + 2 + kMaxK) * sizeof(int);
}

}  // namespace rrd
