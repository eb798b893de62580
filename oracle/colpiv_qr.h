/*
 * ORACLE (test infrastructure only; never linked into the product path).
 *
 * Column-pivoted Householder least squares, restated from the published
 * algorithm that the reference's linear solve uses:
 *   - Businger & Golub column pivoting (largest remaining column norm, first
 *     index on ties),
 *   - LAPACK xGEQPF / LAWN 176 stable norm down-dating with direct
 *     recomputation once the down-dated norm loses sqrt(eps) of accuracy,
 *   - the rank rule of Eigen 3.4's ColPivHouseholderQR: pivot k is treated as
 *     zero once  |biggest|^2 < (max_initial_norm * eps)^2 / rows * (rows - k),
 *     coefficients beyond the rank are set to zero.
 *
 * Reference call site: rils_rols_cpp/rils_rols_cpp.cpp:484
 *   (A.colPivHouseholderQr().solve(b)).
 * Algorithm followed: rils_rols_cpp/eigen/Eigen/src/QR/ColPivHouseholderQR.h:482-608
 *   (computeInPlace, _solve_impl), eigen/Eigen/src/Householder/Householder.h:67-96
 *   (makeHouseholder) and :116-133 (applyHouseholderOnTheLeft).
 *
 * Reduction order (the one thing the vendored, incomplete Eigen cannot pin):
 * every sum, dot product and norm here follows the fixed QSUM order of
 * rils-rols_gb300/csrc/common/rr_sum.h (256 lanes by row index, chunks of
 * RR_CHUNK rows at absolute row multiples, chunk totals in order);
 * products are accumulated, and the rank-1 updates applied, with fused
 * multiply-adds, as Eigen's vectorised kernels do in the reference's
 * -O3 -march=native build on FMA hardware.
 * The Eigen-subset shim that compiles the reference sources uses this same
 * header, so the oracle and the compiled reference agree bit for bit.
 *
 * Plain C99, header-only, no allocation: the caller passes `work`.
 */
#ifndef RR_ORACLE_COLPIV_QR_H
#define RR_ORACLE_COLPIV_QR_H

#include <math.h>
#include <float.h>

#include "../rils-rols_gb300/csrc/common/rr_sum.h"

/* rank-1 update step c - (tau v_i) t: one fused multiply-add (a stock,
 * unvectorised build redefines it as a multiply and an add) */
#ifndef RRQ_UPDATE
#define RRQ_UPDATE(a, b, c) fma((a), (b), (c))
#endif

#ifdef __cplusplus
extern "C" {
#endif


/* Work space (doubles) needed by rrq_lstsq for a rows x cols problem. */
static inline long rrq_work_size(long rows, long cols) {
    return 4 * cols + rows + 8;
}

/*
 * Solve min ||A x - b|| for A (rows x cols, column-major, leading dimension
 * `lda`, overwritten by the factorisation).  Writes x[0..cols).  Returns the
 * number of non-zero pivots (the numerical rank by the rule above).
 */
static inline long rrq_lstsq(double* A, long lda, long rows, long cols,
                             const double* b, double* x, double* work) {
    const long size = rows < cols ? rows : cols;
    double* norm_upd = work;             /* cols */
    double* norm_dir = work + cols;      /* cols */
    double* hcoef    = work + 2 * cols;  /* cols (size used) */
    double* permf    = work + 3 * cols;  /* cols, permutation as doubles */
    double* c        = work + 4 * cols;  /* rows */
    long k, j, i;

    for (k = 0; k < cols; ++k) {
        norm_dir[k] = sqrt(rr_qsumsq(A + k * lda, 0, rows));
        norm_upd[k] = norm_dir[k];
        permf[k] = (double)k;
    }
    /* maxCoeff: sequential scan, strict '>' keeps the first maximum */
    double maxn = cols > 0 ? norm_upd[0] : 0.0;
    for (k = 1; k < cols; ++k) if (norm_upd[k] > maxn) maxn = norm_upd[k];
    const double thr_helper = (maxn * DBL_EPSILON) * (maxn * DBL_EPSILON) / (double)rows;
    const double downdate_thr = sqrt(DBL_EPSILON);

    long nonzero = size;
    for (k = 0; k < size; ++k) {
        long big = k;
        double bign = norm_upd[k];
        for (j = k + 1; j < cols; ++j) if (norm_upd[j] > bign) { bign = norm_upd[j]; big = j; }
        const double big_sq = bign * bign;
        if (nonzero == size && big_sq < thr_helper * (double)(rows - k)) nonzero = k;

        if (big != k) {
            double* ca = A + k * lda;
            double* cb = A + big * lda;
            for (i = 0; i < rows; ++i) { double t = ca[i]; ca[i] = cb[i]; cb[i] = t; }
            double t = norm_upd[k]; norm_upd[k] = norm_upd[big]; norm_upd[big] = t;
            t = norm_dir[k]; norm_dir[k] = norm_dir[big]; norm_dir[big] = t;
            t = permf[k]; permf[k] = permf[big]; permf[big] = t;
        }

        /* Householder reflector of A[k:rows, k] */
        double* col = A + k * lda;
        const long m = rows - k;
        const double tail_sq = (m == 1) ? 0.0 : rr_qsumsq(col, k + 1, rows);
        const double c0 = col[k];
        double tau, beta;
        if (tail_sq <= DBL_MIN) {
            tau = 0.0;
            beta = c0;
            for (i = k + 1; i < rows; ++i) col[i] = 0.0;
        } else {
            beta = sqrt(c0 * c0 + tail_sq);
            if (c0 >= 0.0) beta = -beta;
            const double den = c0 - beta;
            for (i = k + 1; i < rows; ++i) col[i] = col[i] / den;
            tau = (beta - c0) / beta;
        }
        col[k] = beta;
        hcoef[k] = tau;

        /* apply H = I - tau v v^T (v = [1, col[k+1:]]) to A[k:rows, k+1:cols] */
        if (cols - k - 1 > 0) {
            if (m == 1) {
                for (j = k + 1; j < cols; ++j) A[j * lda + k] *= (1.0 - tau);
            } else if (tau != 0.0) {
                for (j = k + 1; j < cols; ++j) {
                    double* cj = A + j * lda;
                    double tmp = rr_qdot(col, cj, k + 1, rows);
                    tmp += cj[k];
                    cj[k] -= tau * tmp;
                    for (i = k + 1; i < rows; ++i) cj[i] = RRQ_UPDATE(-(tau * col[i]), tmp, cj[i]);
                }
            }
        }

        /* LAWN 176 norm down-dating */
        for (j = k + 1; j < cols; ++j) {
            if (norm_upd[j] != 0.0) {
                double temp = fabs(A[j * lda + k]) / norm_upd[j];
                temp = (1.0 + temp) * (1.0 - temp);
                temp = temp < 0.0 ? 0.0 : temp;
                const double ratio = norm_upd[j] / norm_dir[j];
                const double temp2 = temp * (ratio * ratio);
                if (temp2 <= downdate_thr) {
                    norm_dir[j] = sqrt(rr_qsumsq(A + j * lda, k + 1, rows));
                    norm_upd[j] = norm_dir[j];
                } else {
                    norm_upd[j] *= sqrt(temp);
                }
            }
        }
    }

    for (j = 0; j < cols; ++j) x[j] = 0.0;
    if (nonzero == 0) return 0;

    /* c = Q^T b restricted to the first `nonzero` reflectors */
    for (i = 0; i < rows; ++i) c[i] = b[i];
    for (k = 0; k < nonzero; ++k) {
        const double* v = A + k * lda;
        const double tau = hcoef[k];
        const long m = rows - k;
        if (m == 1) {
            c[k] *= (1.0 - tau);
        } else if (tau != 0.0) {
            double tmp = rr_qdot(v, c, k + 1, rows);
            tmp += c[k];
            c[k] -= tau * tmp;
            for (i = k + 1; i < rows; ++i) c[i] = RRQ_UPDATE(-(tau * v[i]), tmp, c[i]);
        }
    }
    /* back substitution with R[0:r, 0:r], column sweep */
    for (k = nonzero - 1; k >= 0; --k) {
        c[k] /= A[k * lda + k];
        for (i = 0; i < k; ++i) c[i] -= c[k] * A[k * lda + i];
    }
    for (k = 0; k < nonzero; ++k) x[(long)permf[k]] = c[k];
    return nonzero;
}

#ifdef __cplusplus
}
#endif
#endif
