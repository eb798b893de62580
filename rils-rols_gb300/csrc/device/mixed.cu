// Mixed-precision fitness path: solve, probes and helpers.
//
// Same contract as the plain path (tune_constants + fitness of
// rils_rols_cpp.cpp:445-541 for every candidate of a round), different
// arithmetic.  The round's distinct factor programs are evaluated once in
// double-float arithmetic into a factor table and their Gram sums are formed
// per distinct pair
// (ftable.cu); here:
//   probe         double-float and FP64 interpreters on up to kProbeRows rows
//                 per distinct factor: the error estimate and non-finite
//                 patterns (certification input);
//   solve         one warp per candidate: gathers its Gram entries, runs a
//                 symmetric-pivoted Cholesky in FP64 (pivot = largest
//                 remaining column norm, as in column-pivoted QR) with one
//                 step of iterative refinement, applies the drop / snap rules
//                 of rils_rols_cpp.cpp:488-517 and gets the SSE from the Gram
//                 identity or flags the candidate for the residual pass;
//                 ambiguous or ill-conditioned systems are queued for the
//                 FP64 path.
#include <cfloat>
#include <cstdint>

#include "../common/df32.h"
#include "../common/rr_math.h"
#include "common.cuh"
#include "dfeval.cuh"
#include "mixed.cuh"
#include "plain.cuh"
#include "reduce.cuh"

namespace rrd {

// ------------------------------------------------------------- probe ----
// Scalar FP64 interpreter with the semantics of the plain path (rr_math
// functions); the double-float one is eval_row_df (dfeval.cuh).
template <int MM>
__device__ bool probe_eval64(const uint32_t* code, int len, const double* K, const DevData& ds, int64_t row,
                             double (&f)[MM]) {
  double st[RRG_MAX_STACK];
  double tos = 0.0;
  int sp = 0;
  for (int pc = 0; pc < len; ++pc) {
    const uint32_t w = code[pc];
    const int op = (int)(w & 0xffu);
    const uint32_t arg = w >> 8;
    switch (op) {
      case RRG_OP_LDV: tos = ds.X64[(int64_t)arg * ds.n_pad + row]; break;
      case RRG_OP_LDC: tos = K[arg]; break;
      case RRG_OP_PSV:
        if (sp >= RRG_MAX_STACK) return false;
        st[sp++] = tos;
        tos = ds.X64[(int64_t)arg * ds.n_pad + row];
        break;
      case RRG_OP_PSC:
        if (sp >= RRG_MAX_STACK) return false;
        st[sp++] = tos;
        tos = K[arg];
        break;
      case RRG_OP_SIN: tos = rr_sin(tos); break;
      case RRG_OP_COS: tos = rr_cos(tos); break;
      case RRG_OP_LN: tos = rr_log(tos); break;
      case RRG_OP_EXP: tos = rr_exp(tos); break;
      case RRG_OP_SQRT: tos = __dsqrt_rn(tos); break;
      case RRG_OP_SQR: tos = __dmul_rn(tos, tos); break;
      case RRG_OP_EMIT:
#pragma unroll
        for (int s = 0; s < MM; ++s)
          if ((int)arg == s) f[s] = tos;
        sp = 0;
        break;
      default: {
        const int kk = op - RRG_OP_BIN;
        const int base = kk >> 3, src = (kk & 7) >> 1, dir = kk & 1;
        double o;
        if (src == RRG_SRC_S) {
          if (sp <= 0) return false;
          o = st[--sp];
        } else if (src == RRG_SRC_V) {
          o = ds.X64[(int64_t)arg * ds.n_pad + row];
        } else {
          o = K[arg];
        }
        const double a = dir == RRG_DIR_N ? o : tos, b = dir == RRG_DIR_N ? tos : o;
        switch (base) {
          case RRG_ADD: tos = __dadd_rn(a, b); break;
          case RRG_SUB: tos = __dsub_rn(a, b); break;
          case RRG_MUL: tos = __dmul_rn(a, b); break;
          case RRG_DIV: tos = __ddiv_rn(a, b); break;
          case RRG_POW: tos = rr_pow(a, b); break;
          case RRG_LT: tos = a < b ? 1.0 : 0.0; break;
          case RRG_EQ: tos = a == b ? 1.0 : 0.0; break;
          case RRG_NE: tos = a != b ? 1.0 : 0.0; break;
          case RRG_MIN: tos = a < b ? a : b; break;
          default: tos = a > b ? a : b; break;
        }
      }
    }
  }
  return true;
}

// Certification: bound on the relative error of the penalised fitness
// (1 + loss)(1 + rmse)(1 + size * cp) caused by the table's evaluation, from
// the per-row bound E on the error of the rebuilt sum (independent of cp).
__device__ double cert_fitness_bound(double sse, double E, double n_d, double sst) {
  if (!(sse >= 0.0) || !(E >= 0.0)) return 1e300;
  const double dsse = 2.0 * sqrt(sse * n_d) * E + n_d * E * E;
  const double loss = sse / sst, rmse = sqrt(sse / n_d);
  const double rl = (dsse / sst) / (1.0 + loss);
  const double rr = (sqrt((sse + dsse) / n_d) - rmse) / (1.0 + rmse);
  return rl + rr;
}

// One warp per candidate: its Gram entries are gathered from the round's
// pair sums (FP64 totals of the double-float partials of the factor table);
// tuned candidates get a symmetric-pivoted Cholesky solve with one
// refinement step.  Every candidate then gets its SSE from the Gram identity
//     SSE = y'y - 2 c'b + c'Gc      (c: coefficients after the drop / snap rules)
// when its bound  u * (y'y + 2|c|'|b| + |c|'|G||c|)  is below pass2_tol * SSE;
// otherwise it is flagged for the residual pass.
// Entry layout per candidate (mmax = kMixedMaxM): G_ij for i <= j < mmax,
// then sum f_i, then sum f_i * y; pair index -1 reads 0.
__global__ void __launch_bounds__(128) mixed_solve_kernel(SolveArgs a) {
  __shared__ double red[4][GramSize<kMixedMaxM>::E];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int li = blockIdx.x * 4 + warp;
  if (li >= a.n_list) return;
  const int mmax = kMixedMaxM;
  const int Gn = mmax * (mmax + 1) / 2, E = Gn + 2 * mmax;
  const int32_t* po = a.pair_of + (size_t)li * E;
  for (int e = lane; e < E; e += 32) {
    const int32_t p = po[e];
    red[warp][e] = p >= 0 ? a.psum[p] : (p <= -2 ? a.pself[-2 - (int64_t)p] : 0.0);
  }
  __syncwarp();
  if (lane != 0) return;
  const int c = a.list[li];
  const rrg_cand cd = a.b.cands[c];
  const double* ent = red[warp];
  const double yy = a.ds.yy;
  // Relative accuracy of the double-float Gram sums with respect to the sums
  // of the absolute values of their terms: about 5u^2 per product and 3u^2
  // per double-float addition (u = 2^-24) over at most ~90 sequential
  // additions per sum, plus the FP64 sum of the chunk partials: about 4e-13.
  const double kU = 1e-12;
  // squared-norm ratio to the largest column below which the reference's
  // rank cut (eps^2 ~ 5e-32) cannot be ruled out
  const double kCutAbs = 1e-24;
  auto queue_fallback = [&](int why) {
    const int slot = atomicAdd(a.fallback, 1);
    if (slot < a.fallback_cap) a.fallback[1 + slot] = c;
    if (a.reasons) atomicAdd(a.reasons + why, 1u);
  };
  const ProbeOut pr = a.probe[c];
  const double n_d = (double)a.ds.n;
  auto cert_bound = [&](double sse, double E) { return cert_fitness_bound(sse, E, n_d, a.ds.sst); };
  // per-row error bound of factor i: the largest probed deviation with a
  // safety factor (exact maximum when every row was probed)
  const double safety = pr.all_rows ? 1.5 : 8.0;
  auto ferr = [&](int i) { return safety * (double)pr.dev[i] + 1e-12 * (double)pr.rms[i]; };
  if (cd.mode != RRG_TUNED) {
    // yp = f: SSE = y'y - 2 f'y + f'f
    const double ff = ent[0], fs = ent[Gn], fy = ent[Gn + mmax];
    const bool nan = ff != ff || fs != fs || fy != fy;
    const bool inf = !nan && (fabs(ff) > DBL_MAX || fabs(fs) > DBL_MAX || fabs(fy) > DBL_MAX);
    uint32_t confirmed = pr.nan64;
    if (nan && !(confirmed & 1u) && a.nanrow && a.nanrow[c] >= 0 && a.nanrow[c] < a.ds.n) {
      double f64[kMixedMaxM];
      for (int i = 0; i < kMixedMaxM; ++i) f64[i] = 0.0;
      if (probe_eval64<kMixedMaxM>(a.b.code + cd.code_offset, cd.code_len, a.b.consts, a.ds, a.nanrow[c], f64) &&
          f64[0] != f64[0])
        confirmed |= 1u;
    }
    uint8_t p2 = 0;
    double sse;
    if (pr.bad32 || pr.inf64 || inf || (nan && !(confirmed & 1u))) {
      // the table broke down, FP64 overflows, or a table NaN that the FP64 probe
      // does not confirm: the FP64 path scores it
      queue_fallback(pr.bad32 ? FB_PROBE_NONFINITE
                              : (pr.inf64 ? FB_FP64_INF : (inf ? FB_FP32_OVERFLOW : FB_OTHER_NAN)));
      sse = -1.0;
    } else if (nan || (pr.nan64 & 1u)) {
      sse = __longlong_as_double(0x7ff8000000000000ll);
    } else {
      sse = __dadd_rn(__dsub_rn(yy, __dmul_rn(2.0, fy)), ff);
      const double bound = kU * (yy + 2.0 * sqrt(fabs(ff) * yy) + ff);
      if (!(sse > 0.0 && bound <= a.pass2_tol * sse)) {
        // the residual pass gives the SSE; certified rounds check it after
        p2 = 1;
        if (a.certify) a.cert_e[c] = ferr(0);
        sse = -1.0;
      } else if (a.certify && cert_bound(sse, ferr(0)) > a.cert_tol) {
        queue_fallback(FB_CERT);
        sse = -1.0;
      }
    }
    a.sse1[c] = sse;
    a.pass2[c] = p2;
    a.res[c].rank = 0;
    return;
  }
  const int m = cd.n_factors, k = m + 1;
  double G[kMixedMaxM + 1][kMixedMaxM + 1], L[kMixedMaxM + 1][kMixedMaxM + 1], bvec[kMixedMaxM + 1];
  int e = 0;
  for (int i = 0; i < mmax; ++i)
    for (int j = i; j < mmax; ++j, ++e)
      if (i < m && j < m) G[i][j] = G[j][i] = ent[e];
  for (int i = 0; i < m; ++i) {
    G[i][m] = G[m][i] = ent[Gn + i];
    bvec[i] = ent[Gn + mmax + i];
  }
  G[m][m] = (double)a.ds.n;
  bvec[m] = a.ds.ysum;
  // Non-finite sums: NaN (a domain error in some factor) gives NaN
  // coefficients and so the fitness sentinel, as the reference's QR does;
  // +-inf without NaN (FP32 exponent overflow) is re-solved by the FP64 path.
  bool has_nan = false, has_inf = false;
  for (int i = 0; i < k; ++i) {
    for (int j = 0; j < k; ++j) {
      has_nan |= G[i][j] != G[i][j];
      has_inf |= fabs(G[i][j]) > DBL_MAX;
    }
    has_nan |= bvec[i] != bvec[i];
    has_inf |= fabs(bvec[i]) > DBL_MAX;
  }
  // factors whose own sums are NaN (a domain error on some row); the cross
  // sums of a NaN factor are NaN for every partner, so only the diagonal,
  // the factor sum and the factor-y sum identify it
  uint32_t nanmask = 0, infmask = 0;
  for (int i = 0; i < m; ++i) {
    const double d = G[i][i], sf = G[i][m], sy = bvec[i];
    if (d != d || sf != sf || sy != sy) nanmask |= 1u << i;
    else if (fabs(d) > DBL_MAX || fabs(sf) > DBL_MAX || fabs(sy) > DBL_MAX) infmask |= 1u << i;
  }
  const uint32_t fullmask = (m >= 32) ? 0xffffffffu : ((1u << m) - 1u);
  uint32_t confirmed = pr.nan64;
  if ((nanmask & ~confirmed) && a.nanrow && a.nanrow[c] >= 0 && a.nanrow[c] < a.ds.n) {
    // table NaN outside the probe rows: evaluate the first such row in FP64
    double f64[kMixedMaxM];
    for (int i = 0; i < kMixedMaxM; ++i) f64[i] = 0.0;
    if (probe_eval64<kMixedMaxM>(a.b.code + cd.code_offset, cd.code_len, a.b.consts, a.ds, a.nanrow[c], f64))
      for (int i = 0; i < m; ++i)
        if (f64[i] != f64[i]) confirmed |= 1u << i;
  }
  nanmask |= pr.nan64 & fullmask;
  if (pr.bad32 || pr.inf64 || infmask || (nanmask & ~confirmed) ||
      (!nanmask && (has_nan || has_inf))) {
    // the table broke down where FP64 did not, FP64 overflow, FP32 exponent
    // overflow, a table NaN the FP64 probe does not confirm, or a non-finite sum outside
    // the factor columns: the FP64 path scores it
    queue_fallback(pr.bad32 ? FB_PROBE_NONFINITE
                            : (pr.inf64 ? FB_FP64_INF : (infmask ? FB_FP32_OVERFLOW : FB_OTHER_NAN)));
    a.sse1[c] = -1.0;
    a.pass2[c] = 0;
    a.res[c].rank = 0;
    return;
  }
  if (nanmask) {
    // A NaN factor column makes the reference's QR return NaN coefficients
    // (the sentinel) unless a rank cut among the other columns happens before
    // the QR reaches it.  Full, well-conditioned rank of the other columns
    // rules that out; otherwise the FP64 path decides.
    int idx[kMixedMaxM + 1], kk2 = 0;
    for (int i = 0; i < k; ++i)
      if (i == m || !((nanmask >> i) & 1u)) idx[kk2++] = i;
    double H[kMixedMaxM + 1][kMixedMaxM + 1], hd0[kMixedMaxM + 1];
    int hp[kMixedMaxM + 1];
    for (int i = 0; i < kk2; ++i) {
      for (int j = 0; j < kk2; ++j) H[i][j] = G[idx[i]][idx[j]];
      hd0[i] = H[i][i];
      hp[i] = i;
    }
    bool full = true;
    double hmax = 0.0;
    for (int i = 0; i < kk2; ++i) hmax = fmax(hmax, H[i][i]);
    for (int s2 = 0; s2 < kk2 && full; ++s2) {
      int p = s2;
      for (int j = s2 + 1; j < kk2; ++j)
        if (H[j][j] > H[p][p]) p = j;
      // well away from a cut: relative to the column's own norm and to the largest
      if (!(H[p][p] > 1e-6 * hd0[hp[p]]) || !(H[p][p] > kCutAbs * hmax)) {
        full = false;
        break;
      }
      if (p != s2) {
        for (int j = 0; j < kk2; ++j) { const double t2 = H[s2][j]; H[s2][j] = H[p][j]; H[p][j] = t2; }
        for (int j = 0; j < kk2; ++j) { const double t2 = H[j][s2]; H[j][s2] = H[j][p]; H[j][p] = t2; }
        const int t3 = hp[s2]; hp[s2] = hp[p]; hp[p] = t3;
      }
      const double l = sqrt(H[s2][s2]);
      for (int i = s2 + 1; i < kk2; ++i) H[i][s2] /= l;
      for (int i = s2 + 1; i < kk2; ++i)
        for (int j = s2 + 1; j <= i; ++j) {
          H[i][j] -= H[i][s2] * H[j][s2];
          H[j][i] = H[i][j];
        }
    }
    double* out = a.coefs + cd.coef_offset;
    for (int i = 0; i < k; ++i) out[i] = __longlong_as_double(0x7ff8000000000000ll);
    if (full) {
      a.sse1[c] = __longlong_as_double(0x7ff8000000000000ll);
    } else {
      queue_fallback(FB_NAN_RANK);
      a.sse1[c] = -1.0;
    }
    a.pass2[c] = 0;
    a.res[c].rank = 0;
    return;
  }
  // symmetric pivoted Cholesky (pivot = largest remaining diagonal, i.e. the
  // largest remaining column norm of the design, as column-pivoted QR picks)
  int piv[kMixedMaxM + 1];
  double d0[kMixedMaxM + 1];
  double maxd = 0.0;
  for (int i = 0; i < k; ++i) {
    piv[i] = i;
    d0[i] = G[i][i];
    if (G[i][i] > maxd) maxd = G[i][i];
    for (int j = 0; j < k; ++j) L[i][j] = G[i][j];
  }
  int rank = k;
  double min_ratio = 1.0;
  const bool finite = !has_nan && !has_inf;
  for (int s2 = 0; s2 < k && finite; ++s2) {
    int p = s2;
    for (int j = s2 + 1; j < k; ++j)
      if (L[j][j] > L[p][p]) p = j;
    const double dp = L[p][p];
    // A pivot is cut when it is small against its own column's norm (the
    // Gram sums cannot resolve it) or so small against the largest column
    // that the reference's QR, whose cut is at eps^2 of the largest squared
    // norm, may cut it.  A badly scaled but independent column is kept.
    if (!(dp > a.rank_tol * d0[piv[p]]) || !(dp > kCutAbs * maxd)) {
      rank = s2;
      break;
    }
    if (p != s2) {
      for (int j = 0; j < k; ++j) { const double t2 = L[s2][j]; L[s2][j] = L[p][j]; L[p][j] = t2; }
      for (int j = 0; j < k; ++j) { const double t2 = L[j][s2]; L[j][s2] = L[j][p]; L[j][p] = t2; }
      const int t3 = piv[s2]; piv[s2] = piv[p]; piv[p] = t3;
    }
    const double ratio = dp / d0[piv[s2]];
    if (ratio < min_ratio) min_ratio = ratio;
    const double lss = sqrt(dp);
    L[s2][s2] = lss;
    for (int i = s2 + 1; i < k; ++i) L[i][s2] = L[i][s2] / lss;
    for (int i = s2 + 1; i < k; ++i)
      for (int j = s2 + 1; j <= i; ++j) {
        L[i][j] = L[i][j] - L[i][s2] * L[j][s2];
        L[j][i] = L[i][j];
      }
  }
  double coef[kMixedMaxM + 1];
  for (int i = 0; i < k; ++i) coef[i] = 0.0;
  uint32_t flags = 0;
  if (!finite) {
    for (int i = 0; i < k; ++i) coef[i] = __longlong_as_double(0x7ff8000000000000ll);
    rank = 0;
  } else if (rank > 0) {
    // solve L L^T z = P b on the leading `rank` block, then one refinement step
    double z[kMixedMaxM + 1], rhs[kMixedMaxM + 1];
    for (int i = 0; i < rank; ++i) rhs[i] = bvec[piv[i]];
    for (int pass = 0; pass < 2; ++pass) {
      for (int i = 0; i < rank; ++i) {
        double v = rhs[i];
        for (int j = 0; j < i; ++j) v -= L[i][j] * z[j];
        z[i] = v / L[i][i];
      }
      for (int i = rank - 1; i >= 0; --i) {
        double v = z[i];
        for (int j = i + 1; j < rank; ++j) v -= L[j][i] * z[j];
        z[i] = v / L[i][i];
      }
      for (int i = 0; i < rank; ++i) coef[piv[i]] += z[i];
      if (pass == 0) {
        for (int i = 0; i < rank; ++i) {
          const int pi = piv[i];
          double v = bvec[pi];
          for (int j = 0; j < k; ++j) v -= G[pi][j] * coef[j];
          rhs[i] = v;
        }
      }
    }
  }
  if (rank < k) flags |= RRG_F_RANK_DEFICIENT;
  // Decisions the FP64 path must take itself: a rank cut (the reference's
  // rule works at eps^2 of the column norms), ill-conditioning, and
  // coefficients inside the ambiguity band of the drop (|c| < 1e-12) and
  // snap (|c - 1| < 1e-12) rules of the rebuilt tree.
  int why = -1;
  if (!finite) why = FB_OTHER_NAN;
  else if (rank < k && a.certify) why = FB_RANK;
  else if (rank == k && min_ratio < a.fallback_tol) why = FB_ILL_COND;
  if (why < 0 && a.certify) {
    // Coefficient error of the Gram solve: with relative errors u of the
    // Gram entries (the sums, kU, and the table's evaluation, ferr / rms of
    // each column) and the smallest relative pivot as the scaled
    // conditioning,
    //   |dc_i| <= u (|y| + sum_j |c_j| |f_j|) sqrt(k) / (lam |f_i|),  lam = min_ratio / k.
    // The drop (|c| < 1e-12) and snap (|c - 1| < 1e-12) rules of the rebuilt
    // tree are left to the FP64 path when c lies within 8 |dc_i| of them.
    double u = kU, M = sqrt(yy);
    for (int i = 0; i < k; ++i) {
      M += fabs(coef[i]) * sqrt(fabs(G[i][i]));
      if (i < m) u = fmax(u, ferr(i) / fmax((double)pr.rms[i], 1e-300));
    }
    const double lam = fmax(min_ratio, 1e-300) / k;
    for (int i = 0; i < k && why < 0; ++i) {
      const double ci = coef[i];
      const double dc = 8.0 * u * M * sqrt((double)k) / (lam * fmax(sqrt(fabs(G[i][i])), 1e-300));
      if (i < m && !(fabs(fabs(ci - 1.0) - kEps12) > dc)) why = FB_SNAP;
      else if (!(fabs(fabs(ci) - kEps12) > dc)) why = FB_DROP;
    }
  }
  double* out = a.coefs + cd.coef_offset;
  MixedTerm& tm = a.terms[c];
  double ceff[kMixedMaxM + 1];
  for (int i = 0; i < k; ++i) {
    out[i] = coef[i];
    const double ci = coef[i];
    tm.hi[i] = (float)ci;
    tm.lo[i] = (float)(ci - (double)tm.hi[i]);
    const int kind = fabs(ci) < kEps12 ? 0 : (i == m ? 1 : (fabs(ci - 1) < kEps12 ? 2 : 3));
    tm.kind[i] = (int8_t)kind;
    ceff[i] = kind == 0 ? 0.0 : (kind == 2 ? 1.0 : ci);
  }
  double sse;
  uint8_t p2 = 0;
  if (has_nan || !finite) {
    sse = has_nan ? __longlong_as_double(0x7ff8000000000000ll) : -1.0;
  } else {
    // mag bounds the sums of |terms| behind every entry used (Cauchy-Schwarz:
    // sum |f_i f_j| <= sqrt(G_ii G_jj), sum |f_i y| <= sqrt(G_ii y'y))
    double lin = 0.0, quad = 0.0, mag = yy;
    for (int i = 0; i < k; ++i) {
      const double si = sqrt(fabs(G[i][i]));
      lin += ceff[i] * bvec[i];
      mag += 2.0 * fabs(ceff[i]) * si * sqrt(yy);
      for (int j = 0; j < k; ++j) {
        quad += ceff[i] * ceff[j] * G[i][j];
        mag += fabs(ceff[i] * ceff[j]) * si * sqrt(fabs(G[j][j]));
      }
    }
    sse = yy - 2.0 * lin + quad;
    double E = 0.0;
    for (int i = 0; i < m; ++i) E += fabs(ceff[i]) * ferr(i);
    if (why < 0 && !(sse > 0.0 && kU * mag <= a.pass2_tol * sse)) {
      // the residual pass gives the SSE; certified rounds check it after
      p2 = 1;
      if (a.certify) a.cert_e[c] = E;
    } else if (why < 0 && a.certify && cert_bound(sse, E) > a.cert_tol) {
      why = FB_CERT;
    }
  }
  const bool fallback = why >= 0;
  if (fallback) {
    queue_fallback(why);
    p2 = 0;
    sse = -1.0;
  } else if (p2) {
    sse = -1.0;
  }
  a.sse1[c] = sse;
  a.pass2[c] = p2;
  a.res[c].rank = rank;
  a.res[c].flags |= flags;
}


// One warp per distinct factor: both interpreters on kProbeRows rows spread
// evenly over the dataset (every row when n <= kProbeRows).
__global__ void __launch_bounds__(128) fac_probe_kernel(const uint32_t* code, const int2* meta, int32_t nf,
                                                        const double* K64, const float* K32, const float* K32lo,
                                                        DevData ds, FacProbe* out, const int32_t* omap) {
  const int lane = threadIdx.x & 31;
  const int f = blockIdx.x * 4 + (threadIdx.x >> 5);
  if (f >= nf) return;
  const int2 mt = meta[f];
  const uint32_t* fc = code + mt.x;
  const int P = ds.n < kProbeRows ? (int)ds.n : kProbeRows;
  float dev = 0.f;
  double ss = 0.0;
  int cnt = 0;
  uint32_t flags = 0;
  for (int p = lane; p < P; p += 32) {
    const int64_t row = ds.n < kProbeRows ? p : ((2 * (int64_t)p + 1) * ds.n) / (2 * kProbeRows);
    double f64[1] = {0.0};
    dfl fd = dfl_make(0.f, 0.f);
    if (!probe_eval64<1>(fc, mt.y, K64, ds, row, f64) || !eval_row_df(fc, mt.y, K32, K32lo, ds, row, fd)) {
      flags |= FP_FAIL;
      continue;
    }
    const double v = f64[0];
    const bool n64 = v != v, i64 = !n64 && fabs(v) > DBL_MAX;
    const bool n32 = fd.hi != fd.hi, i32 = !n32 && fabsf(fd.hi) > FLT_MAX;
    if (n64) flags |= FP_NAN64;
    if (i64) flags |= FP_INF64;
    if (n64 != n32 || (i32 && !i64) || (i64 && !i32)) flags |= FP_BAD32;
    if (!n64 && !i64 && !n32 && !i32) {
      dev = fmaxf(dev, (float)fabs(dfl_to_double(fd) - v));
      ss = __fma_rn(v, v, ss);
      cnt += 1;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    flags |= __shfl_xor_sync(0xffffffffu, flags, o);
    dev = fmaxf(dev, __shfl_xor_sync(0xffffffffu, dev, o));
    ss += __shfl_xor_sync(0xffffffffu, ss, o);
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  }
  if (lane == 0) {
    FacProbe r;
    r.dev = dev;
    r.rms = cnt > 0 ? (float)sqrt(ss / (double)cnt) : 0.f;
    r.flags = flags | (P == ds.n ? FP_ALL_ROWS : 0u);
    out[omap ? omap[f] : f] = r;
  }
}

// One thread per mixed candidate: its probe record and first NaN row from
// those of its factors.
__global__ void cand_probe_kernel(const rrg_cand* cands, const int32_t* list, int32_t n_list,
                                  const int32_t* cand_fac, const int32_t* fcol, const FacProbe* fp,
                                  const unsigned long long* fnan, ProbeOut* out, int64_t* nanrow) {
  const int li = blockIdx.x * blockDim.x + threadIdx.x;
  if (li >= n_list) return;
  const int c = list[li];
  const rrg_cand cd = cands[c];
  const int m = cd.mode == RRG_TUNED ? cd.n_factors : 1;
  ProbeOut r;
  r.nan64 = r.inf64 = r.bad32 = 0;
  r.all_rows = 0;
  unsigned long long first = 0x7f7f7f7f7f7f7f7full;
  for (int i = 0; i < kMixedMaxM; ++i) {
    r.dev[i] = 0.f;
    r.rms[i] = 0.f;
    if (i >= m) continue;
    const int f = cand_fac[(size_t)li * kMixedMaxM + i];
    const FacProbe p = fp[f];
    r.dev[i] = p.dev;
    r.rms[i] = p.rms;
    if (p.flags & FP_NAN64) r.nan64 |= 1u << i;
    if (p.flags & FP_INF64) r.inf64 |= 1u << i;
    if (p.flags & FP_BAD32) r.bad32 |= 1u << i;
    if (p.flags & FP_FAIL) r.bad32 = 0xffffffffu;
    if (p.flags & FP_ALL_ROWS) r.all_rows = 1u;
    const unsigned long long fr = fnan[fcol ? fcol[f] : f];
    first = fr < first ? fr : first;
  }
  out[c] = r;
  nanrow[c] = (int64_t)first;
}

// One thread per candidate of the residual pass of a certified round: the
// bound of cert_fitness_bound on its residual-pass SSE (partials summed in
// the order of finalize_kernel); above the tolerance it is queued for FP64.
__global__ void cert_resid_kernel(const int32_t* mlist, const int32_t* list2, int32_t n2, const double* sse_part,
                                  int nb, const double* cert_e, DevData ds, double cert_tol, int32_t* fallback,
                                  int32_t fallback_cap, uint32_t* reasons, const int32_t* n2_dev) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n2 || (n2_dev && i >= *n2_dev)) return;
  const int c = mlist[list2[i]];
  const double E = cert_e[c];
  if (!(E >= 0.0)) return;
  double sse = 0.0;
  for (int j = 0; j < nb; ++j) sse = __dadd_rn(sse, sse_part[(int64_t)c * nb + j]);
  if (cert_fitness_bound(sse, E, (double)ds.n, ds.sst) > cert_tol) {
    const int slot = atomicAdd(fallback, 1);
    if (slot < fallback_cap) fallback[1 + slot] = c;
    atomicAdd(reasons + FB_CERT, 1u);
  }
}

__global__ void to_f32_kernel(const double* src, float* dst, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (float)src[i];
}
__global__ void split_f32_kernel(const double* src, float* hi, float* lo, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const dfl v = dfl_from_double(src[i]);
    hi[i] = v.hi;
    lo[i] = v.lo;
  }
}

// ----------------------------------------------------------- launchers ----
bool launch_fac_probe(const uint32_t* code, const int2* meta, int32_t nf, const double* K64, const float* K32,
                      const float* K32lo, const DevData& ds, FacProbe* out, cudaStream_t st, const int32_t* omap) {
  if (nf <= 0) return true;
  fac_probe_kernel<<<(nf + 3) / 4, 128, 0, st>>>(code, meta, nf, K64, K32, K32lo, ds, out, omap);
  return launch_ok("launch_fac_probe");
}
bool launch_cand_probe(const rrg_cand* cands, const int32_t* list, int32_t n_list, const int32_t* cand_fac,
                       const int32_t* fcol, const FacProbe* fp, const unsigned long long* fnan, ProbeOut* out,
                       int64_t* nanrow, cudaStream_t st) {
  if (n_list <= 0) return true;
  cand_probe_kernel<<<(n_list + 127) / 128, 128, 0, st>>>(cands, list, n_list, cand_fac, fcol, fp, fnan, out,
                                                          nanrow);
  return launch_ok("launch_cand_probe");
}
bool launch_cert_resid(const int32_t* mlist, const int32_t* list2, int32_t n2, const double* sse_part, int nb,
                       const double* cert_e, const DevData& ds, double cert_tol, int32_t* fallback,
                       int32_t fallback_cap, uint32_t* reasons, cudaStream_t st, const int32_t* n2_dev) {
  if (n2 <= 0) return true;
  cert_resid_kernel<<<(n2 + 127) / 128, 128, 0, st>>>(mlist, list2, n2, sse_part, nb, cert_e, ds, cert_tol, fallback,
                                                      fallback_cap, reasons, n2_dev);
  return launch_ok("launch_cert_resid");
}
bool launch_solve(const SolveArgs& a, cudaStream_t st) {
  if (a.n_list <= 0) return true;
  mixed_solve_kernel<<<(a.n_list + 3) / 4, 128, 0, st>>>(a);
  return launch_ok("launch_solve");
}
bool launch_to_f32(const double* src, float* dst, int64_t n, cudaStream_t st) {
  to_f32_kernel<<<1024, 256, 0, st>>>(src, dst, n);
  return launch_ok("launch_to_f32");
}
bool launch_split_f32(const double* src, float* hi, float* lo, int64_t n, cudaStream_t st) {
  split_f32_kernel<<<1024, 256, 0, st>>>(src, hi, lo, n);
  return launch_ok("launch_split_f32");
}

}  // namespace rrd
