/*
 * flens_oracle.c -- CPU restatement of FLENS's generic dense level-3 / LU path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle the CUDA library is
 * checked against and the CPU baseline that bench.py times.  The product
 * (flens_gb300/csrc) never links or calls it.
 *
 * Each function restates the reference's generic C++ template for real double
 * precision, keeping its operation order (which element is scaled first, the
 * direction and start value of every dot product, reciprocal-multiply versus
 * divide), so that with -ffp-contract=off it is bitwise identical to the
 * reference's dgemm_/dtrsm_/dgetrf_/dgetrs_/dgesv_ compiled from source.
 * tests/test_oracle_pin.py checks that identity whenever oracle/_ref exists.
 * Citations are file:line inside the FLENS source tree.
 */
#define _GNU_SOURCE
#include "flens_oracle.h"

#include <float.h>
#include <stddef.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define IDX(i, j, ld) ((size_t)(i) + (size_t)(j) * (size_t)(ld))

static int is_notrans(char t) { return t == 'N' || t == 'n'; }

/*
 * GEMM.  cxxblas/level3/gemm.tcc:42-75 turns the column-major call into a
 * row-major one, scales C by beta first (gescal, :66; multiply, not assign,
 * cxxblas/level1/scal.tcc:40-49), returns when alpha==0 (:67-69) and then, per
 * row of C, calls gemv (:70-75) whose per-element result is a dot product
 * started at zero and summed in increasing k (cxxblas/level2/gemv.tcc:75-79,
 * cxxblas/level1/dot.tcc:48-51), added as C += alpha*dot.
 */
void oracle_dgemm(char transA, char transB, int m, int n, int k,
                  double alpha, const double *A, int ldA,
                  const double *B, int ldB,
                  double beta, double *C, int ldC)
{
    if (m == 0 || n == 0) {
        return;
    }
    for (int j = 0; j < n; ++j) {
        for (int i = 0; i < m; ++i) {
            C[IDX(i, j, ldC)] *= beta;
        }
    }
    if (alpha == 0.0) {
        return;
    }
    const int nA = is_notrans(transA), nB = is_notrans(transB);
    /* op(A)(i,p) and op(B)(p,j) as strides */
    const size_t aI = nA ? 1 : (size_t)ldA, aP = nA ? (size_t)ldA : 1;
    const size_t bP = nB ? 1 : (size_t)ldB, bJ = nB ? (size_t)ldB : 1;
    /* Loop nest as the reference: rows of C outermost (one gemv per row),
     * columns next, k innermost. */
    for (int i = 0; i < m; ++i) {
        for (int j = 0; j < n; ++j) {
            double dot = 0.0;
            const double *a = A + (size_t)i * aI;
            const double *b = B + (size_t)j * bJ;
            for (int p = 0; p < k; ++p) {
                dot += b[(size_t)p * bP] * a[(size_t)p * aP];
            }
            C[IDX(i, j, ldC)] += alpha * dot;
        }
    }
}

/*
 * TRSM.  cxxblas/level3/trsm.tcc:40-68: column-major is mapped to row-major,
 * every right-hand side is solved by trsv (dot-form substitution,
 * cxxblas/level2/trsv.tcc:48-200: x_i -= sum_p M(i,p) x_p with the sum started
 * at zero and taken in increasing p, then x_i /= M(i,i) for non-unit), and
 * alpha is applied AFTER the solve (:67, gescal).  For side=Left the effective
 * triangle is op(A) and the vectors are the columns of B; for side=Right it is
 * op(A)^T and the vectors are the rows of B.
 */
void oracle_dtrsm(char side, char upLo, char transA, char diag,
                  int m, int n, double alpha,
                  const double *A, int ldA, double *B, int ldB)
{
    const int left = (side == 'L' || side == 'l');
    const int lowerA = (upLo == 'L' || upLo == 'l');
    const int nT = is_notrans(transA);
    const int unit = (diag == 'U' || diag == 'u');
    const int ka = left ? m : n;
    const int nVec = left ? n : m;
    /* M(i,p) = A[i*mi + p*mp] */
    size_t mi, mp;
    int lowerM;
    if (left) {
        lowerM = lowerA ^ (!nT);
        mi = nT ? 1 : (size_t)ldA;
        mp = nT ? (size_t)ldA : 1;
    } else {
        lowerM = lowerA ^ nT;
        mi = nT ? (size_t)ldA : 1;
        mp = nT ? 1 : (size_t)ldA;
    }
    const size_t xs = left ? 1 : (size_t)ldB;      /* stride inside a vector */
    const size_t vs = left ? (size_t)ldB : 1;      /* stride between vectors */
    for (int v = 0; v < nVec; ++v) {
        double *x = B + (size_t)v * vs;
        if (lowerM) {
            for (int i = 0; i < ka; ++i) {
                double s = 0.0;
                for (int p = 0; p < i; ++p) {
                    s += A[(size_t)i * mi + (size_t)p * mp] * x[(size_t)p * xs];
                }
                x[(size_t)i * xs] -= s;
                if (!unit) {
                    x[(size_t)i * xs] /= A[(size_t)i * mi + (size_t)i * mp];
                }
            }
        } else {
            for (int i = ka - 1; i >= 0; --i) {
                double s = 0.0;
                for (int q = i + 1; q < ka; ++q) {
                    s += A[(size_t)i * mi + (size_t)q * mp] * x[(size_t)q * xs];
                }
                x[(size_t)i * xs] -= s;
                if (!unit) {
                    x[(size_t)i * xs] /= A[(size_t)i * mi + (size_t)i * mp];
                }
            }
        }
    }
    for (int j = 0; j < n; ++j) {
        for (int i = 0; i < m; ++i) {
            B[IDX(i, j, ldB)] *= alpha;
        }
    }
}

/*
 * IAMAX.  cxxblas/level1/iamax.tcc:42-58 and :80-92: start from element 0,
 * replace only on a strictly greater |x_i| (first maximum wins; a NaN never
 * wins unless it is element 0); n<=0 gives -1.
 */
int oracle_idamax(int n, const double *x, int incX)
{
    if (incX < 0) {
        x -= (ptrdiff_t)incX * (n - 1);
    }
    if (n <= 0) {
        return -1;
    }
    int iMax = 0;
    double absMax = fabs(x[0]);
    for (int i = 0; i < n; ++i) {
        const double a = fabs(x[(ptrdiff_t)i * incX]);
        if (a > absMax) {
            iMax = i;
            absMax = a;
        }
    }
    return iMax;
}

static void swap_row_segment(double *A, int ldA, int r1, int r2, int c0, int c1)
{
    for (int c = c0; c < c1; ++c) {
        const double t = A[IDX(r1, c, ldA)];
        A[IDX(r1, c, ldA)] = A[IDX(r2, c, ldA)];
        A[IDX(r2, c, ldA)] = t;
    }
}

/*
 * LASWP.  flens/lapack/la/laswp.tcc:54-93: columns in blocks of 32, inside a
 * block the interchanges i <-> piv(i) for i = k1..k2 (or k2..k1 when the pivot
 * view is reversed, as trs.tcc:106 does for the transposed solve).
 */
void oracle_dlaswp(int nCols, double *A, int ldA, int k1, int k2,
                   const int *piv, int inc)
{
    const int bs = 32;
    const int nbs = (nCols / bs) * bs;
    for (int c0 = 0; c0 < nCols; c0 += bs) {
        const int c1 = (c0 < nbs) ? c0 + bs : nCols;
        if (inc > 0) {
            for (int i = k1; i <= k2; ++i) {
                const int ip = piv[i - 1];
                if (ip != i) swap_row_segment(A, ldA, i - 1, ip - 1, c0, c1);
            }
        } else {
            for (int i = k2; i >= k1; --i) {
                const int ip = piv[i - 1];
                if (ip != i) swap_row_segment(A, ldA, i - 1, ip - 1, c0, c1);
            }
        }
    }
}

/*
 * TF2.  flens/lapack/ge/tf2.tcc:56-136.  Per column: iamax pivot (:101-102),
 * swap of the whole panel row (:108), scale by the reciprocal when
 * |pivot| >= SafeMin, else divide (:113-121), zero pivot sets info once
 * (:123-125), then the rank-1 update A22 += (-1*row_j) * col_j column by column
 * (:131 -> cxxblas/level2/ger.tcc:41-64 -> axpy).  SafeMin is DBL_MIN
 * (flens/lapack/la/lamch.tcc:73-81: 1/DBL_MAX < DBL_MIN).
 */
/*
 * Relative separation of the two largest |candidates| of one pivot search,
 * (|first| - |second|) / |first| (1 with a single candidate, 0 for an exact
 * tie or a zero column).  Test instrumentation only: it reads the column and
 * changes nothing, so the factorisation is the same with or without it.
 */
static double pivot_gap(int n, const double *x)
{
    double a1 = 0.0, a2 = 0.0;
    for (int i = 0; i < n; ++i) {
        const double a = fabs(x[i]);
        if (a > a1) {
            a2 = a1;
            a1 = a;
        } else if (a > a2) {
            a2 = a;
        }
    }
    if (n <= 1) return 1.0;
    return a1 > 0.0 ? (a1 - a2) / a1 : 0.0;
}

static int dgetf2_impl(int m, int n, double *A, int ldA, int *piv, double *gap)
{
    int info = 0;
    if (m == 0 || n == 0) {
        return info;
    }
    const double safeMin = DBL_MIN;
    const int mn = m < n ? m : n;
    for (int j = 0; j < mn; ++j) {
        if (gap) gap[j] = pivot_gap(m - j, &A[IDX(j, j, ldA)]);
        const int jp = j + oracle_idamax(m - j, &A[IDX(j, j, ldA)], 1);
        piv[j] = jp + 1;
        if (A[IDX(jp, j, ldA)] != 0.0) {
            if (jp != j) {
                swap_row_segment(A, ldA, j, jp, 0, n);
            }
            if (j < m - 1) {
                const double ajj = A[IDX(j, j, ldA)];
                if (fabs(ajj) >= safeMin) {
                    const double r = 1.0 / ajj;
                    for (int i = j + 1; i < m; ++i) A[IDX(i, j, ldA)] *= r;
                } else {
                    for (int i = j + 1; i < m; ++i) A[IDX(i, j, ldA)] /= ajj;
                }
            }
        } else if (info == 0) {
            info = j + 1;
        }
        if (j + 1 < mn) {
            for (int c = j + 1; c < n; ++c) {
                const double y = -1.0 * A[IDX(j, c, ldA)];
                for (int i = j + 1; i < m; ++i) {
                    A[IDX(i, c, ldA)] += y * A[IDX(i, j, ldA)];
                }
            }
        }
    }
    return info;
}

int oracle_dgetf2(int m, int n, double *A, int ldA, int *piv)
{
    return dgetf2_impl(m, n, A, ldA, piv, NULL);
}

/*
 * TRF.  flens/lapack/ge/trf.tcc:59-152 with bs = ilaenv(1,"GETRF") = 64
 * (flens/lapack/la/ilaenv.tcc:93-99); unblocked when bs<=1 or bs>=min(m,n)
 * (:87-91).  Per block: panel tf2 (:113), info/pivot offset (:117-122),
 * laswp left (:126) and right (:132), trsm for the U block row (:136-138),
 * trailing gemm with alpha=-1, beta=1 (:144-146).
 */
static int dgetrf_impl(int m, int n, double *A, int ldA, int *piv, int nb,
                       int maxBlocks, double *gap)
{
    int info = 0;
    if (m == 0 || n == 0) {
        return info;
    }
    const int mn = m < n ? m : n;
    if (nb <= 1 || nb >= mn) {
        return dgetf2_impl(m, n, A, ldA, piv, gap);
    }
    int blocks = 0;
    for (int j = 1; j <= mn; j += nb) {
        if (maxBlocks >= 0 && blocks++ >= maxBlocks) {
            break;
        }
        const int jb = (mn - j + 1 < nb) ? mn - j + 1 : nb;
        const int info_ = dgetf2_impl(m - j + 1, jb, &A[IDX(j - 1, j - 1, ldA)],
                                      ldA, &piv[j - 1], gap ? &gap[j - 1] : NULL);
        if (info == 0 && info_ > 0) {
            info = info_ + j - 1;
        }
        const int iEnd = (m < j + jb - 1) ? m : j + jb - 1;
        for (int i = j; i <= iEnd; ++i) {
            piv[i - 1] += j - 1;
        }
        oracle_dlaswp(j - 1, A, ldA, j, j + jb - 1, piv, 1);
        if (j + jb <= n) {
            oracle_dlaswp(n - j - jb + 1, &A[IDX(0, j + jb - 1, ldA)], ldA,
                          j, j + jb - 1, piv, 1);
            oracle_dtrsm('L', 'L', 'N', 'U', jb, n - j - jb + 1, 1.0,
                         &A[IDX(j - 1, j - 1, ldA)], ldA,
                         &A[IDX(j - 1, j + jb - 1, ldA)], ldA);
            if (j + jb <= m) {
                oracle_dgemm('N', 'N', m - j - jb + 1, n - j - jb + 1, jb,
                             -1.0, &A[IDX(j + jb - 1, j - 1, ldA)], ldA,
                             &A[IDX(j - 1, j + jb - 1, ldA)], ldA,
                             1.0, &A[IDX(j + jb - 1, j + jb - 1, ldA)], ldA);
            }
        }
    }
    return info;
}

int oracle_dgetrf_nb(int m, int n, double *A, int ldA, int *piv, int nb)
{
    return dgetrf_impl(m, n, A, ldA, piv, nb, -1, NULL);
}

int oracle_dgetrf(int m, int n, double *A, int ldA, int *piv)
{
    return dgetrf_impl(m, n, A, ldA, piv, 64, -1, NULL);
}

/* oracle_dgetrf that also records, per pivot search j, the relative gap
 * between the two largest |candidates| (gap[min(m,n)]). */
int oracle_dgetrf_gaps(int m, int n, double *A, int ldA, int *piv, double *gap)
{
    return dgetrf_impl(m, n, A, ldA, piv, 64, -1, gap);
}

int oracle_dgetrf_steps(int m, int n, double *A, int ldA, int *piv,
                        int nb, int nBlocks)
{
    return dgetrf_impl(m, n, A, ldA, piv, nb, nBlocks, NULL);
}

/*
 * TRS.  flens/lapack/ge/trs.tcc:59-109.  NoTrans: laswp forward, L (unit
 * lower) then U (non-unit upper).  Trans/ConjTrans: U^T, L^T, then laswp with
 * the pivot vector reversed.
 */
void oracle_dgetrs(char trans, int n, int nRhs, const double *A, int ldA,
                   const int *piv, double *B, int ldB)
{
    if (n == 0 || nRhs == 0) {
        return;
    }
    if (is_notrans(trans)) {
        oracle_dlaswp(nRhs, B, ldB, 1, n, piv, 1);
        oracle_dtrsm('L', 'L', 'N', 'U', n, nRhs, 1.0, A, ldA, B, ldB);
        oracle_dtrsm('L', 'U', 'N', 'N', n, nRhs, 1.0, A, ldA, B, ldB);
    } else {
        oracle_dtrsm('L', 'U', trans, 'N', n, nRhs, 1.0, A, ldA, B, ldB);
        oracle_dtrsm('L', 'L', trans, 'U', n, nRhs, 1.0, A, ldA, B, ldB);
        oracle_dlaswp(nRhs, B, ldB, 1, n, piv, -1);
    }
}

/* SV.  flens/lapack/ge/sv.tcc:58-77: trf, then trs only when info==0. */
int oracle_dgesv(int n, int nRhs, double *A, int ldA, int *piv,
                 double *B, int ldB)
{
    const int info = oracle_dgetrf(n, n, A, ldA, piv);
    if (info == 0) {
        oracle_dgetrs('N', n, nRhs, A, ldA, piv, B, ldB);
    }
    return info;
}

/* ---------------------------------------------------------------- timing -- */

/*
 * SYRK.  cxxblas/level3/syrk.tcc:42-90: column-major is mapped to row-major
 * with the triangle and the transposition flipped; the triangle is scaled by
 * beta unless beta == 1 (cxxblas/level1extensions/syscal.tcc:41-61, a
 * multiply); k == 0 returns; then one rank-1 update per l = 0..k-1
 * (cxxblas/level2/syr.tcc:42-70), each an axpy with the coefficient alpha*x_i
 * computed first: C(r, c) += (alpha*x_c)*x_r for the column c being updated.
 */
void oracle_dsyrk(char upLo, char trans, int n, int k, double alpha,
                  const double *A, int ldA, double beta, double *C, int ldC)
{
    const int lower = (upLo == 'L' || upLo == 'l');
    const int nT = is_notrans(trans);
    if (beta != 1.0) {
        for (int c = 0; c < n; ++c) {
            const int r0 = lower ? c : 0, r1 = lower ? n : c + 1;
            for (int r = r0; r < r1; ++r) {
                C[IDX(r, c, ldC)] *= beta;
            }
        }
    }
    if (k == 0) {
        return;
    }
    /* x_l(i) = op(A)(i, l): column l of A (trans N) or row l (trans T) */
    const size_t xi = nT ? 1 : (size_t)ldA, xl = nT ? (size_t)ldA : 1;
    for (int l = 0; l < k; ++l) {
        const double *x = A + (size_t)l * xl;
        for (int c = 0; c < n; ++c) {
            const double t = alpha * x[(size_t)c * xi];
            const int r0 = lower ? c : 0, r1 = lower ? n : c + 1;
            for (int r = r0; r < r1; ++r) {
                C[IDX(r, c, ldC)] += t * x[(size_t)r * xi];
            }
        }
    }
}

/*
 * TRMM.  cxxblas/level3/trmm.tcc:40-70: every vector (column of B for
 * side=Left, row for side=Right) is multiplied by the effective triangle M
 * (op(A), or op(A)^T for side=Right) with trmv (cxxblas/level2/trmv.tcc:
 * 42-200): x_i <- sum over the triangle row i of M(i,p) x_p, the dot started
 * at zero in increasing p, the diagonal term included unless unit, where
 * x_i + dot(off-diagonal) is taken; rows are visited so that only old values
 * are read.  alpha multiplies B at the end (gescal).
 */
void oracle_dtrmm(char side, char upLo, char transA, char diag, int m, int n,
                  double alpha, const double *A, int ldA, double *B, int ldB)
{
    if (m == 0 || n == 0) {
        return;
    }
    const int left = (side == 'L' || side == 'l');
    const int lowerA = (upLo == 'L' || upLo == 'l');
    const int nT = is_notrans(transA);
    const int unit = (diag == 'U' || diag == 'u');
    const int ka = left ? m : n;
    const int nVec = left ? n : m;
    size_t mi, mp;
    int lowerM;
    if (left) {
        lowerM = lowerA ^ (!nT);
        mi = nT ? 1 : (size_t)ldA;
        mp = nT ? (size_t)ldA : 1;
    } else {
        lowerM = lowerA ^ nT;
        mi = nT ? (size_t)ldA : 1;
        mp = nT ? 1 : (size_t)ldA;
    }
    const size_t xs = left ? 1 : (size_t)ldB;
    const size_t vs = left ? (size_t)ldB : 1;
    for (int v = 0; v < nVec; ++v) {
        double *x = B + (size_t)v * vs;
        if (lowerM) {
            for (int i = ka - 1; i >= 0; --i) {
                double s = 0.0;
                const int pe = unit ? i : i + 1;
                for (int p = 0; p < pe; ++p) {
                    s += A[(size_t)i * mi + (size_t)p * mp] * x[(size_t)p * xs];
                }
                x[(size_t)i * xs] = unit ? x[(size_t)i * xs] + s : s;
            }
        } else {
            for (int i = 0; i < ka; ++i) {
                double s = 0.0;
                for (int p = unit ? i + 1 : i; p < ka; ++p) {
                    s += A[(size_t)i * mi + (size_t)p * mp] * x[(size_t)p * xs];
                }
                x[(size_t)i * xs] = unit ? x[(size_t)i * xs] + s : s;
            }
        }
    }
    for (int j = 0; j < n; ++j) {
        for (int i = 0; i < m; ++i) {
            B[IDX(i, j, ldB)] *= alpha;
        }
    }
}

/*
 * SYMM.  cxxblas/level3/symm.tcc:40-70: C is scaled by beta first (gescal, a
 * multiply), then every vector (column of C for side=Left, row for
 * side=Right, with the matching vector x of B) gets symv with beta 1
 * (cxxblas/level2/symv.tcc:42-80): two passes over all i, y_i += alpha*s1_i
 * then y_i += alpha*s2_i, where with the lower triangle stored
 * s1_i = sum_{p>=i} A(p,i) x_p and s2_i = sum_{p<i} A(i,p) x_p, and with the
 * upper one s1_i = sum_{p<i} A(p,i) x_p and s2_i = sum_{p>=i} A(i,p) x_p;
 * every dot started at zero in increasing p.  No alpha == 0 shortcut.
 */
void oracle_dsymm(char side, char upLo, int m, int n, double alpha,
                  const double *A, int ldA, const double *B, int ldB,
                  double beta, double *C, int ldC)
{
    if (m == 0 || n == 0) {
        return;
    }
    const int left = (side == 'L' || side == 'l');
    const int lower = (upLo == 'L' || upLo == 'l');
    const int ka = left ? m : n;
    const int nVec = left ? n : m;
    const size_t xs = left ? 1 : (size_t)ldB, xv = left ? (size_t)ldB : 1;
    const size_t ys = left ? 1 : (size_t)ldC, yv = left ? (size_t)ldC : 1;
    for (int j = 0; j < n; ++j) {
        for (int i = 0; i < m; ++i) {
            C[IDX(i, j, ldC)] *= beta;
        }
    }
    for (int v = 0; v < nVec; ++v) {
        const double *x = B + (size_t)v * xv;
        double *y = C + (size_t)v * yv;
        for (int pass = 0; pass < 2; ++pass) {
            for (int i = 0; i < ka; ++i) {
                double s = 0.0;
                /* pass 0: the column of the stored triangle through A(i,i) for
                 * lower, above it for upper; pass 1: the row part */
                const int from_lower = (pass == 0) == (lower != 0);
                if (from_lower) {
                    if (pass == 0) {
                        for (int p = i; p < ka; ++p) s += A[IDX(p, i, ldA)] * x[(size_t)p * xs];
                    } else {
                        for (int p = i; p < ka; ++p) s += A[IDX(i, p, ldA)] * x[(size_t)p * xs];
                    }
                } else {
                    if (pass == 0) {
                        for (int p = 0; p < i; ++p) s += A[IDX(p, i, ldA)] * x[(size_t)p * xs];
                    } else {
                        for (int p = 0; p < i; ++p) s += A[IDX(i, p, ldA)] * x[(size_t)p * xs];
                    }
                }
                y[(size_t)i * ys] += alpha * s;
            }
        }
    }
}

/*
 * SYR2K.  cxxblas/level3/syr2k.tcc:42-95: the triangle is scaled by beta
 * unless beta == 1 (syscal); k == 0 returns; then for l = 0..k-1 one syr2
 * (cxxblas/level2/syr2.tcc:42-75) with x, y the l-th vectors of op(A), op(B):
 * per column c of the triangle, first C(r,c) += (alpha*x_c)*y_r for all its
 * rows r, then C(r,c) += (alpha*y_c)*x_r.
 */
void oracle_dsyr2k(char upLo, char trans, int n, int k, double alpha,
                   const double *A, int ldA, const double *B, int ldB,
                   double beta, double *C, int ldC)
{
    const int lower = (upLo == 'L' || upLo == 'l');
    const int nT = is_notrans(trans);
    if (beta != 1.0) {
        for (int c = 0; c < n; ++c) {
            const int r0 = lower ? c : 0, r1 = lower ? n : c + 1;
            for (int r = r0; r < r1; ++r) {
                C[IDX(r, c, ldC)] *= beta;
            }
        }
    }
    if (k == 0) {
        return;
    }
    const size_t ai = nT ? 1 : (size_t)ldA, al = nT ? (size_t)ldA : 1;
    const size_t bi = nT ? 1 : (size_t)ldB, bl = nT ? (size_t)ldB : 1;
    for (int l = 0; l < k; ++l) {
        const double *x = A + (size_t)l * al;
        const double *y = B + (size_t)l * bl;
        for (int c = 0; c < n; ++c) {
            const double t1 = alpha * x[(size_t)c * ai], t2 = alpha * y[(size_t)c * bi];
            const int r0 = lower ? c : 0, r1 = lower ? n : c + 1;
            for (int r = r0; r < r1; ++r) {
                C[IDX(r, c, ldC)] += t1 * y[(size_t)r * bi];
            }
            for (int r = r0; r < r1; ++r) {
                C[IDX(r, c, ldC)] += t2 * x[(size_t)r * ai];
            }
        }
    }
}

/*
 * GEMV.  cxxblas/level2/gemv.tcc:160-176 returns when m or n is 0 (before
 * any scaling); :42-130 maps column-major to row-major, scales y by beta
 * (scal, a multiply) and adds alpha*dot per element, the dot started at zero
 * in increasing index.
 */
void oracle_dgemv(char trans, int m, int n, double alpha, const double *A,
                  int ldA, const double *x, int incX, double beta, double *y,
                  int incY)
{
    if (m == 0 || n == 0) {
        return;
    }
    const int nT = is_notrans(trans);
    const int ny = nT ? m : n, nx = nT ? n : m;
    if (incX < 0) {
        x -= (ptrdiff_t)incX * (nx - 1);
    }
    if (incY < 0) {
        y -= (ptrdiff_t)incY * (ny - 1);
    }
    for (int i = 0; i < ny; ++i) {
        y[(ptrdiff_t)i * incY] *= beta;
    }
    for (int i = 0; i < ny; ++i) {
        double s = 0.0;
        for (int p = 0; p < nx; ++p) {
            const double a = nT ? A[IDX(i, p, ldA)] : A[IDX(p, i, ldA)];
            s += a * x[(ptrdiff_t)p * incX];
        }
        y[(ptrdiff_t)i * incY] += alpha * s;
    }
}

/*
 * TI2.  flens/lapack/tr/ti2.tcc (generic ti2_impl): upper: for j = 1..n,
 * A(j,j) = 1/A(j,j) and Ajj = -A(j,j) (or Ajj = -1 for a unit diagonal), then
 * u12 = A(1:j-1, j) <- U11 * u12 (trmv with the already inverted U11) and
 * u12 *= Ajj; lower: j = n..1 with l21 = A(j+1:n, j) and L22.
 */
int oracle_dtrti2(char upLo, char diag, int n, double *A, int ldA)
{
    const int upper = (upLo == 'U' || upLo == 'u');
    const int nonunit = (diag == 'N' || diag == 'n');
    if (upper) {
        for (int j = 0; j < n; ++j) {
            double ajj;
            if (nonunit) {
                A[IDX(j, j, ldA)] = 1.0 / A[IDX(j, j, ldA)];
                ajj = -A[IDX(j, j, ldA)];
            } else {
                ajj = -1.0;
            }
            if (j > 0) {
                oracle_dtrmm('L', 'U', 'N', nonunit ? 'N' : 'U', j, 1, 1.0, A, ldA,
                             &A[IDX(0, j, ldA)], ldA);
                for (int i = 0; i < j; ++i) {
                    A[IDX(i, j, ldA)] *= ajj;
                }
            }
        }
    } else {
        for (int j = n - 1; j >= 0; --j) {
            double ajj;
            if (nonunit) {
                A[IDX(j, j, ldA)] = 1.0 / A[IDX(j, j, ldA)];
                ajj = -A[IDX(j, j, ldA)];
            } else {
                ajj = -1.0;
            }
            if (j < n - 1) {
                const int r = n - 1 - j;
                oracle_dtrmm('L', 'L', 'N', nonunit ? 'N' : 'U', r, 1, 1.0,
                             &A[IDX(j + 1, j + 1, ldA)], ldA, &A[IDX(j + 1, j, ldA)], ldA);
                for (int i = 0; i < r; ++i) {
                    A[IDX(j + 1 + i, j, ldA)] *= ajj;
                }
            }
        }
    }
    return 0;
}

/*
 * TRTRI.  flens/lapack/tr/tri.tcc (generic tri_impl): a non-unit matrix with
 * an exactly zero diagonal element returns its index untouched; unblocked
 * (ti2) when nb <= 1 or nb >= n; else upper: for j = 1, 1+nb, ...:
 * U12 <- U11 U12 (trmm), U12 <- -U12 U22^-1 (trsm), ti2(U22); lower: j from
 * ((n-1)/nb)*nb+1 down: L21 <- L22 L21, L21 <- -L21 L11^-1, ti2(L11).
 */
int oracle_dtrtri_nb(char upLo, char diag, int n, double *A, int ldA, int nb)
{
    const int upper = (upLo == 'U' || upLo == 'u');
    const int nonunit = (diag == 'N' || diag == 'n');
    const char dg = nonunit ? 'N' : 'U';
    if (n == 0) {
        return 0;
    }
    if (nonunit) {
        for (int i = 0; i < n; ++i) {
            if (A[IDX(i, i, ldA)] == 0.0) {
                return i + 1;
            }
        }
    }
    if (nb <= 1 || nb >= n) {
        return oracle_dtrti2(upLo, diag, n, A, ldA);
    }
    if (upper) {
        for (int j = 0; j < n; j += nb) {
            const int jb = (nb < n - j) ? nb : n - j;
            if (j > 0) {
                oracle_dtrmm('L', 'U', 'N', dg, j, jb, 1.0, A, ldA, &A[IDX(0, j, ldA)], ldA);
                oracle_dtrsm('R', 'U', 'N', dg, j, jb, -1.0, &A[IDX(j, j, ldA)], ldA,
                             &A[IDX(0, j, ldA)], ldA);
            }
            oracle_dtrti2('U', dg, jb, &A[IDX(j, j, ldA)], ldA);
        }
    } else {
        const int nn = ((n - 1) / nb) * nb;
        for (int j = nn; j >= 0; j -= nb) {
            const int jb = (nb < n - j) ? nb : n - j;
            if (j + jb < n) {
                const int r = n - j - jb;
                oracle_dtrmm('L', 'L', 'N', dg, r, jb, 1.0, &A[IDX(j + jb, j + jb, ldA)], ldA,
                             &A[IDX(j + jb, j, ldA)], ldA);
                oracle_dtrsm('R', 'L', 'N', dg, r, jb, -1.0, &A[IDX(j, j, ldA)], ldA,
                             &A[IDX(j + jb, j, ldA)], ldA);
            }
            oracle_dtrti2('L', dg, jb, &A[IDX(j, j, ldA)], ldA);
        }
    }
    return 0;
}

int oracle_dtrtri(char upLo, char diag, int n, double *A, int ldA)
{
    return oracle_dtrtri_nb(upLo, diag, n, A, ldA, 64);
}

/*
 * GETRI.  flens/lapack/ge/tri.tcc (generic tri_impl) with the full workspace
 * (lwork = n*nb, nb = 64): trtri of U (return on a zero pivot); unblocked
 * when nb >= n: for j = n..1, work = A(j+1:n, j), A(j+1:n, j) = 0,
 * A(:, j) -= A(:, j+1:n) work (gemv); blocked: for j from nn down by nb, the
 * strictly lower part of the block column goes to Work and is zeroed,
 * A(:, J) -= A(:, j+jb:n) Work(j+jb:n, :) (gemm), A(:, J) <- A(:, J) Wunit^-1
 * (trsm, Work's unit lower block); last the column interchanges
 * j = n-1..1 with piv(j).
 */
int oracle_dgetri(int n, double *A, int ldA, const int *piv)
{
    const int nb = 64;
    if (n == 0) {
        return 0;
    }
    const int info = oracle_dtrtri('U', 'N', n, A, ldA);
    if (info > 0) {
        return info;
    }
    double *work = (double *)calloc((size_t)n * nb, sizeof(double));
    if (nb >= n) {
        for (int j = n - 1; j >= 0; --j) {
            for (int i = j + 1; i < n; ++i) {
                work[i] = A[IDX(i, j, ldA)];
                A[IDX(i, j, ldA)] = 0.0;
            }
            if (j < n - 1) {
                oracle_dgemv('N', n, n - j - 1, -1.0, &A[IDX(0, j + 1, ldA)], ldA, &work[j + 1], 1,
                             1.0, &A[IDX(0, j, ldA)], 1);
            }
        }
    } else {
        const int ldw = n;
        const int nn = ((n - 1) / nb) * nb;
        for (int j = nn; j >= 0; j -= nb) {
            const int jb = (nb < n - j) ? nb : n - j;
            for (int jj = j, JJ = 0; jj < j + jb; ++jj, ++JJ) {
                for (int i = jj + 1; i < n; ++i) {
                    work[IDX(i, JJ, ldw)] = A[IDX(i, jj, ldA)];
                    A[IDX(i, jj, ldA)] = 0.0;
                }
            }
            if (j + jb < n) {
                oracle_dgemm('N', 'N', n, jb, n - j - jb, -1.0, &A[IDX(0, j + jb, ldA)], ldA,
                             &work[IDX(j + jb, 0, ldw)], ldw, 1.0, &A[IDX(0, j, ldA)], ldA);
            }
            oracle_dtrsm('R', 'L', 'N', 'U', n, jb, 1.0, &work[IDX(j, 0, ldw)], ldw,
                         &A[IDX(0, j, ldA)], ldA);
        }
    }
    free(work);
    for (int j = n - 2; j >= 0; --j) {
        const int jp = piv[j] - 1;
        if (jp != j) {
            for (int i = 0; i < n; ++i) {
                const double t = A[IDX(i, j, ldA)];
                A[IDX(i, j, ldA)] = A[IDX(i, jp, ldA)];
                A[IDX(i, jp, ldA)] = t;
            }
        }
    }
    return 0;
}

/* ---------------------------------------------------------------------- */
/* FLENS's machine constants (flens/lapack/la/lamch.tcc: eps = epsilon/2,
 * SafeMin = DBL_MIN, Precision = eps*2), sign (flens/lapack/auxiliary/
 * sign.tcc: |x| with the sign bit of y) and nint (floor(x+1/2)). */
static const double kEps = DBL_EPSILON * 0.5;
static const double kSafeMin = DBL_MIN;
static const double kPrecision = DBL_EPSILON;

static double f_sign(double x, double y)
{
    if (y > 0.0) return fabs(x);
    if (y < 0.0) return -fabs(x);
    return signbit(y) ? -fabs(x) : fabs(x);
}

static double f_nint(double x) { return floor(x + 0.5); }

static double f_asum(int n, const double *x)
{
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += fabs(x[i]);
    return s;
}

/* std::max(a, b) / std::min(a, b): (a < b) ? b : a  /  (b < a) ? b : a */
static double f_max(double a, double b) { return (a < b) ? b : a; }
static double f_min(double a, double b) { return (b < a) ? b : a; }

/* LANGE.  flens/lapack/la/lan.tcc (GeMatrix): max |a_ij| in column order;
 * one-norm = max column sum (each sum in increasing i); infinity-norm = max
 * of the row sums accumulated column by column. */
double oracle_dlange(char norm, int m, int n, const double *A, int ldA)
{
    if (m == 0 || n == 0) return 0.0;
    double value = 0.0;
    if (norm == 'M' || norm == 'm') {
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < m; ++i) value = f_max(value, fabs(A[IDX(i, j, ldA)]));
    } else if (norm == 'I' || norm == 'i') {
        double *w = (double *)calloc((size_t)m, sizeof(double));
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < m; ++i) w[i] += fabs(A[IDX(i, j, ldA)]);
        for (int i = 0; i < m; ++i) value = f_max(value, w[i]);
        free(w);
    } else {
        for (int j = 0; j < n; ++j) {
            double sum = 0.0;
            for (int i = 0; i < m; ++i) sum += fabs(A[IDX(i, j, ldA)]);
            value = f_max(value, sum);
        }
    }
    return value;
}

/* LACN2.  flens/lapack/la/lacn2.tcc (real variant), the reference's
 * reverse-communication state machine step for step (isave[0..2] = its
 * iSave(1..3), indices 1-based as there). */
void oracle_dlacn2(int n, double *v, double *x, int *sgn, double *est, int *kase,
                   int *isave)
{
    const int itMax = 5;
    if (*kase == 0) {
        for (int i = 0; i < n; ++i) x[i] = 1.0 / (double)n;
        *kase = 1;
        isave[0] = 1;
        return;
    }
    int jlast, converged;
    double estold, altsgn, temp;
    switch (isave[0]) {
    case 1:
        if (n == 1) {
            v[0] = x[0];
            *est = fabs(v[0]);
            goto QUIT;
        }
        *est = f_asum(n, x);
        for (int i = 0; i < n; ++i) {
            x[i] = f_sign(1.0, x[i]);
            sgn[i] = (int)f_nint(x[i]);
        }
        *kase = 2;
        isave[0] = 2;
        return;
    case 2:
        isave[1] = oracle_idamax(n, x, 1) + 1;
        isave[2] = 2;
    MAIN:
        for (int i = 0; i < n; ++i) x[i] = 0.0;
        x[isave[1] - 1] = 1.0;
        *kase = 1;
        isave[0] = 3;
        return;
    case 3:
        for (int i = 0; i < n; ++i) v[i] = x[i];
        estold = *est;
        *est = f_asum(n, v);
        converged = 1;
        for (int i = 0; i < n; ++i) {
            if (f_nint(f_sign(1.0, x[i])) != (double)sgn[i]) {
                converged = 0;
                break;
            }
        }
        if (converged) goto ITERATION_COMPLETE;
        if (*est <= estold) goto ITERATION_COMPLETE;
        for (int i = 0; i < n; ++i) {
            x[i] = f_sign(1.0, x[i]);
            sgn[i] = (int)f_nint(x[i]);
        }
        *kase = 2;
        isave[0] = 4;
        return;
    case 4:
        jlast = isave[1];
        isave[1] = oracle_idamax(n, x, 1) + 1;
        if (x[jlast - 1] != fabs(x[isave[1] - 1]) && isave[2] < itMax) {
            ++isave[2];
            goto MAIN;
        }
    ITERATION_COMPLETE:
        altsgn = 1.0;
        for (int i = 0; i < n; ++i) {
            x[i] = altsgn * (1.0 + (double)i / (double)(n - 1));
            altsgn = -altsgn;
        }
        *kase = 1;
        isave[0] = 5;
        return;
    case 5:
        temp = 2.0 * (f_asum(n, x) / (double)(3 * n));
        if (temp > *est) {
            for (int i = 0; i < n; ++i) v[i] = x[i];
            *est = temp;
        }
    }
QUIT:
    *kase = 0;
}

/* LATRS.  flens/lapack/la/latrs.tcc (real variant), the part up to the
 * choice of path: column norms of the off-diagonal triangle (asum, unless
 * normIn), tscale from their max, xmax = |x(iamax)|, the growth bound grow
 * from the loop over the diagonal, and when grow*tscale > smallNum the plain
 * triangular solve blas::sv (the dot-form trsv of oracle_dtrsm).  The scaled
 * careful path is not restated: -1 is returned instead. */
int oracle_dlatrs(char upLo, char trans, char diag, int normIn, int n,
                  const double *A, int ldA, double *x, double *scale,
                  double *cnorm)
{
    const int upper = (upLo == 'U' || upLo == 'u');
    const int nT = is_notrans(trans);
    const int nonunit = (diag == 'N' || diag == 'n');
    *scale = 1.0;
    if (n == 0) return 0;
    const double smallNum = kSafeMin / kPrecision;
    const double bigNum = 1.0 / smallNum;
    if (!normIn) {
        if (upper) {
            for (int j = 0; j < n; ++j) cnorm[j] = f_asum(j, &A[IDX(0, j, ldA)]);
        } else {
            for (int j = 0; j < n - 1; ++j) cnorm[j] = f_asum(n - 1 - j, &A[IDX(j + 1, j, ldA)]);
            cnorm[n - 1] = 0.0;
        }
    }
    const int imax = oracle_idamax(n, cnorm, 1);
    const double tmax = cnorm[imax];
    double tscale;
    if (tmax <= bigNum) {
        tscale = 1.0;
    } else {
        return -1;
    }
    const int jx = oracle_idamax(n, x, 1);
    const double xmax = fabs(x[jx]);
    double xbound = xmax, grow;
    int jfirst, jlast, jinc;
    if (nT) {
        if (upper) { jfirst = n - 1; jlast = 0; jinc = -1; }
        else { jfirst = 0; jlast = n - 1; jinc = 1; }
    } else {
        if (upper) { jfirst = 0; jlast = n - 1; jinc = 1; }
        else { jfirst = n - 1; jlast = 0; jinc = -1; }
    }
    const int jend = jlast + jinc;
    if (tscale != 1.0) {
        grow = 0.0;
    } else if (nT) {
        if (nonunit) {
            grow = 1.0 / f_max(xbound, smallNum);
            xbound = grow;
            int too_small = 0;
            for (int j = jfirst; j != jend; j += jinc) {
                if (grow <= smallNum) { too_small = 1; break; }
                const double tjj = fabs(A[IDX(j, j, ldA)]);
                xbound = f_min(xbound, f_min(1.0, tjj) * grow);
                if (tjj + cnorm[j] >= smallNum) grow *= tjj / (tjj + cnorm[j]);
                else grow = 0.0;
            }
            if (!too_small) grow = xbound;
        } else {
            grow = f_min(1.0, 1.0 / f_max(xbound, smallNum));
            for (int j = jfirst; j != jend; j += jinc) {
                if (grow <= smallNum) break;
                grow *= 1.0 / (1.0 + cnorm[j]);
            }
        }
    } else {
        if (nonunit) {
            grow = 1.0 / f_max(xbound, smallNum);
            xbound = grow;
            for (int j = jfirst; j != jend; j += jinc) {
                if (grow <= smallNum) break;
                const double xj = 1.0 + cnorm[j];
                grow = f_min(grow, xbound / xj);
                const double tjj = fabs(A[IDX(j, j, ldA)]);
                if (xj > tjj) xbound *= tjj / xj;
            }
            grow = f_min(grow, xbound);
        } else {
            grow = f_min(1.0, 1.0 / f_max(xbound, smallNum));
            for (int j = jfirst; j != jend; j += jinc) {
                if (grow <= smallNum) break;
                grow /= 1.0 + cnorm[j];
            }
        }
    }
    if (grow * tscale > smallNum) {
        oracle_dtrsm('L', upper ? 'U' : 'L', nT ? 'N' : 'T', nonunit ? 'N' : 'U', n, 1, 1.0,
                     A, ldA, x, n);
        return 0;
    }
    return -1;
}

/* GECON.  flens/lapack/ge/cond.tcc (real variant): lacn2 drives solves with
 * the unit-lower L and upper U of the factors through latrs (L then U for
 * the chosen norm, U^T then L^T otherwise; column norms computed on the first
 * pair only); rcond = (1/estimate)/anorm. */
int oracle_dgecon(char norm, int n, const double *A, int ldA, double anorm,
                  double *rcond)
{
    *rcond = 0.0;
    if (n == 0) {
        *rcond = 1.0;
        return 0;
    } else if (anorm == 0.0) {
        return 0;
    }
    const int kase1 = (norm == '1' || norm == 'O' || norm == 'o') ? 1 : 2;
    double *work = (double *)calloc((size_t)4 * n, sizeof(double));
    int *iwork = (int *)calloc((size_t)n, sizeof(int));
    double *x = work, *v = work + n, *cnL = work + 2 * n, *cnU = work + 3 * n;
    int isave[3] = {0, 0, 0}, kase = 0, normIn = 0, status = 0;
    double ainvnm = 0.0;
    for (;;) {
        oracle_dlacn2(n, v, x, iwork, &ainvnm, &kase, isave);
        if (kase == 0) break;
        double sl, su;
        int r;
        if (kase == kase1) {
            r = oracle_dlatrs('L', 'N', 'U', normIn, n, A, ldA, x, &sl, cnL);
            if (r == 0) r = oracle_dlatrs('U', 'N', 'N', normIn, n, A, ldA, x, &su, cnU);
        } else {
            r = oracle_dlatrs('U', 'T', 'N', normIn, n, A, ldA, x, &su, cnU);
            if (r == 0) r = oracle_dlatrs('L', 'T', 'U', normIn, n, A, ldA, x, &sl, cnL);
        }
        if (r != 0) {
            status = -1;
            break;
        }
        normIn = 1;                       /* sl = su = 1 on the unscaled path */
    }
    if (status == 0 && ainvnm != 0.0) *rcond = (1.0 / ainvnm) / anorm;
    free(work);
    free(iwork);
    return status;
}

/* GERFS.  flens/lapack/ge/rfs.tcc (generic rfs_impl), per right-hand side:
 * r = b - op(A) x (gemv), w = |b| + |op(A)||x| (NoTrans accumulated column by
 * column, Trans as column dots), berr = max_i |r_i|/w_i (with safe1 added
 * where w_i <= safe2); while berr > eps, 2 berr <= last and at most 5 steps,
 * solve op(AF) dx = r and x += dx; then the forward error bound from lacn2
 * with w_i <- |r_i| + (n+1) eps w_i (+safe1), divided by max |x_i|. */
int oracle_dgerfs(char trans, int n, int nRhs, const double *A, int ldA,
                  const double *AF, int ldAF, const int *piv, const double *B,
                  int ldB, double *X, int ldX, double *ferr, double *berr)
{
    const int nT = is_notrans(trans);
    const char tr = nT ? 'N' : 'T', trT = nT ? 'T' : 'N';
    if (n == 0 || nRhs == 0) {
        for (int j = 0; j < nRhs; ++j) ferr[j] = berr[j] = 0.0;
        return 0;
    }
    const int nz = n + 1;
    const double eps = kEps, safeMin = kSafeMin;
    const double safe1 = nz * safeMin, safe2 = safe1 / eps;
    double *work = (double *)calloc((size_t)3 * n, sizeof(double));
    int *iwork = (int *)calloc((size_t)n, sizeof(int));
    double *w1 = work, *w2 = work + n, *w3 = work + 2 * n;
    for (int j = 0; j < nRhs; ++j) {
        int count = 1;
        double lastres = 3.0;
        double *x = &X[IDX(0, j, ldX)];
        const double *b = &B[IDX(0, j, ldB)];
        for (;;) {
            for (int i = 0; i < n; ++i) w2[i] = b[i];
            oracle_dgemv(tr, n, n, -1.0, A, ldA, x, 1, 1.0, w2, 1);
            for (int i = 0; i < n; ++i) w1[i] = fabs(b[i]);
            if (nT) {
                for (int k = 0; k < n; ++k) {
                    const double xk = fabs(x[k]);
                    for (int i = 0; i < n; ++i) w1[i] += fabs(A[IDX(i, k, ldA)]) * xk;
                }
            } else {
                for (int k = 0; k < n; ++k) {
                    double s = 0.0;
                    for (int i = 0; i < n; ++i) s += fabs(A[IDX(i, k, ldA)]) * fabs(x[i]);
                    w1[k] += s;
                }
            }
            double s = 0.0;
            for (int i = 0; i < n; ++i) {
                if (w1[i] > safe2) s = f_max(s, fabs(w2[i]) / w1[i]);
                else s = f_max(s, (fabs(w2[i]) + safe1) / (w1[i] + safe1));
            }
            berr[j] = s;
            if (berr[j] > eps && 2.0 * berr[j] <= lastres && count <= 5) {
                oracle_dgetrs(tr, n, 1, AF, ldAF, piv, w2, n);
                for (int i = 0; i < n; ++i) x[i] += w2[i];
                lastres = berr[j];
                ++count;
                continue;
            }
            break;
        }
        for (int i = 0; i < n; ++i) {
            if (w1[i] > safe2) w1[i] = fabs(w2[i]) + (double)nz * eps * w1[i];
            else w1[i] = fabs(w2[i]) + (double)nz * eps * w1[i] + safe1;
        }
        int kase = 0, isave[3] = {0, 0, 0};
        for (;;) {
            oracle_dlacn2(n, w3, w2, iwork, &ferr[j], &kase, isave);
            if (kase == 0) break;
            if (kase == 1) {
                oracle_dgetrs(trT, n, 1, AF, ldAF, piv, w2, n);
                for (int i = 0; i < n; ++i) w2[i] *= w1[i];
            } else {
                for (int i = 0; i < n; ++i) w2[i] *= w1[i];
                oracle_dgetrs(tr, n, 1, AF, ldAF, piv, w2, n);
            }
        }
        lastres = 0.0;
        for (int i = 0; i < n; ++i) lastres = f_max(lastres, fabs(x[i]));
        if (lastres != 0.0) ferr[j] /= lastres;
    }
    free(work);
    free(iwork);
    return 0;
}

/* GEEQU.  flens/lapack/ge/equ.tcc: r_i = 1/clamp(max_j |a_ij|), c_j =
 * 1/clamp(max_i |a_ij| r_i), the ratios rowcnd/colcnd and amax; info = i
 * (or m+j) for the first zero row (column). */
int oracle_dgeequ(int m, int n, const double *A, int ldA, double *r, double *c,
                  double *rowcnd, double *colcnd, double *amax)
{
    if (m == 0 || n == 0) {
        *rowcnd = 1.0;
        *colcnd = 1.0;
        *amax = 0.0;
        return 0;
    }
    const double smallNum = kSafeMin, bigNum = 1.0 / smallNum;
    for (int i = 0; i < m; ++i) r[i] = 0.0;
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < m; ++i) r[i] = f_max(r[i], fabs(A[IDX(i, j, ldA)]));
    double rcmin = bigNum, rcmax = 0.0;
    for (int i = 0; i < m; ++i) {
        rcmax = f_max(rcmax, r[i]);
        rcmin = f_min(rcmin, r[i]);
    }
    *amax = rcmax;
    if (rcmin == 0.0) {
        for (int i = 0; i < m; ++i)
            if (r[i] == 0.0) return i + 1;
    } else {
        for (int i = 0; i < m; ++i) r[i] = 1.0 / f_min(f_max(r[i], smallNum), bigNum);
        *rowcnd = f_max(rcmin, smallNum) / f_min(rcmax, bigNum);
    }
    for (int j = 0; j < n; ++j) c[j] = 0.0;
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < m; ++i) c[j] = f_max(c[j], fabs(A[IDX(i, j, ldA)]) * r[i]);
    rcmin = bigNum;
    rcmax = 0.0;
    for (int j = 0; j < n; ++j) {
        rcmin = f_min(rcmin, c[j]);
        rcmax = f_max(rcmax, c[j]);
    }
    if (rcmin == 0.0) {
        for (int j = 0; j < n; ++j)
            if (c[j] == 0.0) return m + j + 1;
    } else {
        for (int j = 0; j < n; ++j) c[j] = 1.0 / f_min(f_max(c[j], smallNum), bigNum);
        *colcnd = f_max(rcmin, smallNum) / f_min(rcmax, bigNum);
    }
    return 0;
}

/* LAQGE.  flens/lapack/la/laq.tcc: thresholds 0.1 and SafeMin/Precision. */
char oracle_dlaqge(int m, int n, double *A, int ldA, const double *r,
                   const double *c, double rowcnd, double colcnd, double amax)
{
    if (m == 0 || n == 0) return 'N';
    const double small = kSafeMin / kPrecision, large = 1.0 / small;
    if (rowcnd >= 0.1 && amax >= small && amax <= large) {
        if (colcnd >= 0.1) return 'N';
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < m; ++i) A[IDX(i, j, ldA)] *= c[j];
        return 'C';
    } else if (colcnd >= 0.1) {
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < m; ++i) A[IDX(i, j, ldA)] *= r[i];
        return 'R';
    }
    for (int j = 0; j < n; ++j) {
        const double cj = c[j];
        for (int i = 0; i < m; ++i) A[IDX(i, j, ldA)] *= cj * r[i];
    }
    return 'B';
}

/* maximum |a_ij| over the upper triangle (lan on a TrMatrix, max norm) */
static double upper_max(int m, int n, const double *A, int ldA)
{
    double v = 0.0;
    for (int j = 0; j < n; ++j)
        for (int i = 0; i <= j && i < m; ++i) v = f_max(v, fabs(A[IDX(i, j, ldA)]));
    return v;
}

/* GESVX.  flens/lapack/ge/svx.tcc (generic svx_impl). */
int oracle_dgesvx(char fact, char trans, int n, int nRhs, double *A, int ldA,
                  double *AF, int ldAF, int *piv, char *equed, double *r,
                  double *c, double *B, int ldB, double *X, int ldX,
                  double *rcond, double *ferr, double *berr, double *rpvgrw)
{
    const double smallNum = kSafeMin, bigNum = 1.0 / smallNum;
    const int nT = is_notrans(trans);
    int rowequ, colequ, info = 0;
    double rowcnd = 1.0, colcnd = 1.0;
    if (fact == 'N' || fact == 'E') {
        *equed = 'N';
        rowequ = colequ = 0;
    } else {
        rowequ = (*equed == 'R' || *equed == 'B');
        colequ = (*equed == 'C' || *equed == 'B');
    }
    if (rowequ) {
        double lo = bigNum, hi = 0.0;
        for (int j = 0; j < n; ++j) { lo = f_min(lo, r[j]); hi = f_max(hi, r[j]); }
        rowcnd = n > 0 ? f_max(lo, smallNum) / f_min(hi, bigNum) : 1.0;
    }
    if (colequ) {
        double lo = bigNum, hi = 0.0;
        for (int j = 0; j < n; ++j) { lo = f_min(lo, c[j]); hi = f_max(hi, c[j]); }
        colcnd = n > 0 ? f_max(lo, smallNum) / f_min(hi, bigNum) : 1.0;
    }
    if (fact == 'E') {
        double amax;
        if (oracle_dgeequ(n, n, A, ldA, r, c, &rowcnd, &colcnd, &amax) == 0) {
            *equed = oracle_dlaqge(n, n, A, ldA, r, c, rowcnd, colcnd, amax);
            rowequ = (*equed == 'R' || *equed == 'B');
            colequ = (*equed == 'C' || *equed == 'B');
        }
    }
    if (nT) {
        if (rowequ)
            for (int j = 0; j < nRhs; ++j)
                for (int i = 0; i < n; ++i) B[IDX(i, j, ldB)] *= r[i];
    } else if (colequ) {
        for (int j = 0; j < nRhs; ++j)
            for (int i = 0; i < n; ++i) B[IDX(i, j, ldB)] *= c[i];
    }
    if (fact == 'N' || fact == 'E') {
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) AF[IDX(i, j, ldAF)] = A[IDX(i, j, ldA)];
        info = oracle_dgetrf(n, n, AF, ldAF, piv);
        if (info > 0) {
            /* svx.tcc: max-norm of the whole A over that of U(1:info,1:info) */
            double g = upper_max(info, info, AF, ldAF);
            g = (g == 0.0) ? 1.0 : oracle_dlange('M', n, n, A, ldA) / g;
            *rpvgrw = g;
            *rcond = 0.0;
            return info;
        }
    }
    const double anorm = oracle_dlange(nT ? '1' : 'I', n, n, A, ldA);
    double g = upper_max(n, n, AF, ldAF);
    g = (g == 0.0) ? 1.0 : oracle_dlange('M', n, n, A, ldA) / g;
    if (oracle_dgecon(nT ? '1' : 'I', n, AF, ldAF, anorm, rcond) != 0) return -1;
    for (int j = 0; j < nRhs; ++j)
        for (int i = 0; i < n; ++i) X[IDX(i, j, ldX)] = B[IDX(i, j, ldB)];
    oracle_dgetrs(nT ? 'N' : 'T', n, nRhs, AF, ldAF, piv, X, ldX);
    oracle_dgerfs(trans, n, nRhs, A, ldA, AF, ldAF, piv, B, ldB, X, ldX, ferr, berr);
    if (nT) {
        if (colequ) {
            for (int j = 0; j < nRhs; ++j)
                for (int i = 0; i < n; ++i) X[IDX(i, j, ldX)] *= c[i];
            for (int j = 0; j < nRhs; ++j) ferr[j] /= colcnd;
        }
    } else if (rowequ) {
        for (int j = 0; j < nRhs; ++j)
            for (int i = 0; i < n; ++i) X[IDX(i, j, ldX)] *= r[i];
        for (int j = 0; j < nRhs; ++j) ferr[j] /= rowcnd;
    }
    *rpvgrw = g;
    if (*rcond < kEps) info = n + 1;
    return info;
}

/*
 * POTF2.  flens/lapack/po/potf2.tcc:56-140 (left-looking, dot form): for each
 * column j, ajj = A(j,j) - dot(a, a) over the finished part of row/column j;
 * ajj <= 0 or NaN stores ajj, sets info = j and stops; otherwise A(j,j) =
 * sqrt(ajj), the rest of column j (lower) or row j (upper) gets
 * gemv(-1, ., +1) and is multiplied by 1/ajj (reciprocal computed once).
 */
int oracle_dpotf2(char upLo, int n, double *A, int ldA)
{
    const int lower = (upLo == 'L' || upLo == 'l');
    for (int j = 0; j < n; ++j) {
        /* a = A(j, 0:j) (lower: row, stride ldA) or A(0:j, j) (upper: column) */
        const double *a = lower ? &A[IDX(j, 0, ldA)] : &A[IDX(0, j, ldA)];
        const size_t as = lower ? (size_t)ldA : 1;
        double dot = 0.0;
        for (int p = 0; p < j; ++p) {
            dot += a[(size_t)p * as] * a[(size_t)p * as];
        }
        double ajj = A[IDX(j, j, ldA)] - dot;
        if (ajj <= 0.0 || isnan(ajj)) {
            A[IDX(j, j, ldA)] = ajj;
            return j + 1;
        }
        ajj = sqrt(ajj);
        A[IDX(j, j, ldA)] = ajj;
        if (j + 1 < n) {
            const int rest = n - j - 1;
            if (lower) {
                /* a32 = a32 - A31 * a21^T ; a32 *= 1/ajj */
                oracle_dgemv('N', rest, j, -1.0, &A[IDX(j + 1, 0, ldA)], ldA,
                             &A[IDX(j, 0, ldA)], ldA, 1.0, &A[IDX(j + 1, j, ldA)], 1);
                const double r = 1.0 / ajj;
                for (int i = 0; i < rest; ++i) {
                    A[IDX(j + 1 + i, j, ldA)] *= r;
                }
            } else {
                /* a23 = a23 - A13^T * a12 ; a23 *= 1/ajj */
                oracle_dgemv('T', j, rest, -1.0, &A[IDX(0, j + 1, ldA)], ldA,
                             &A[IDX(0, j, ldA)], 1, 1.0, &A[IDX(j, j + 1, ldA)], ldA);
                const double r = 1.0 / ajj;
                for (int i = 0; i < rest; ++i) {
                    A[IDX(j, j + 1 + i, ldA)] *= r;
                }
            }
        }
    }
    return 0;
}

/*
 * POTRF.  flens/lapack/po/potrf.tcc:56-150: unblocked when nb <= 1 or
 * nb >= n; otherwise, per block column j (lower): A22 -= A21 A21^T (syrk),
 * potf2(A22) (info offset by j, stop on failure), A32 -= A31 A21^T (gemm),
 * A32 <- A32 L22^-T (trsm); upper mirrors it with A12, A13, A23.
 */
int oracle_dpotrf_nb(char upLo, int n, double *A, int ldA, int nb)
{
    const int lower = (upLo == 'L' || upLo == 'l');
    if (n == 0) {
        return 0;
    }
    if (nb <= 1 || nb >= n) {
        return oracle_dpotf2(upLo, n, A, ldA);
    }
    for (int j = 0; j < n; j += nb) {
        const int jb = (nb < n - j) ? nb : n - j;
        const int r3 = n - j - jb;
        double *A22 = &A[IDX(j, j, ldA)];
        if (lower) {
            oracle_dsyrk('L', 'N', jb, j, -1.0, &A[IDX(j, 0, ldA)], ldA, 1.0, A22, ldA);
            const int info = oracle_dpotf2('L', jb, A22, ldA);
            if (info != 0) {
                return info + j;
            }
            if (r3 > 0) {
                oracle_dgemm('N', 'T', r3, jb, j, -1.0, &A[IDX(j + jb, 0, ldA)], ldA,
                             &A[IDX(j, 0, ldA)], ldA, 1.0, &A[IDX(j + jb, j, ldA)], ldA);
                oracle_dtrsm('R', 'L', 'T', 'N', r3, jb, 1.0, A22, ldA,
                             &A[IDX(j + jb, j, ldA)], ldA);
            }
        } else {
            oracle_dsyrk('U', 'T', jb, j, -1.0, &A[IDX(0, j, ldA)], ldA, 1.0, A22, ldA);
            const int info = oracle_dpotf2('U', jb, A22, ldA);
            if (info != 0) {
                return info + j;
            }
            if (r3 > 0) {
                oracle_dgemm('T', 'N', jb, r3, j, -1.0, &A[IDX(0, j, ldA)], ldA,
                             &A[IDX(0, j + jb, ldA)], ldA, 1.0, &A[IDX(j, j + jb, ldA)], ldA);
                oracle_dtrsm('L', 'U', 'T', 'N', jb, r3, 1.0, A22, ldA,
                             &A[IDX(j, j + jb, ldA)], ldA);
            }
        }
    }
    return 0;
}

int oracle_dpotrf(char upLo, int n, double *A, int ldA)
{
    return oracle_dpotrf_nb(upLo, n, A, ldA, 64);
}

/*
 * POTRS.  flens/lapack/po/potrs.tcc:54-100: lower: L X = B then L^T X = B;
 * upper: U^T X = B then U X = B; both triangular solves non-unit, alpha 1.
 */
void oracle_dpotrs(char upLo, int n, int nRhs, const double *A, int ldA,
                   double *B, int ldB)
{
    const int lower = (upLo == 'L' || upLo == 'l');
    if (n == 0 || nRhs == 0) {
        return;
    }
    if (lower) {
        oracle_dtrsm('L', 'L', 'N', 'N', n, nRhs, 1.0, A, ldA, B, ldB);
        oracle_dtrsm('L', 'L', 'T', 'N', n, nRhs, 1.0, A, ldA, B, ldB);
    } else {
        oracle_dtrsm('L', 'U', 'T', 'N', n, nRhs, 1.0, A, ldA, B, ldB);
        oracle_dtrsm('L', 'U', 'N', 'N', n, nRhs, 1.0, A, ldA, B, ldB);
    }
}

int oracle_dposv(char upLo, int n, int nRhs, double *A, int ldA, double *B,
                 int ldB)
{
    const int info = oracle_dpotrf(upLo, n, A, ldA);
    if (info == 0) {
        oracle_dpotrs(upLo, n, nRhs, A, ldA, B, ldB);
    }
    return info;
}

static unsigned long long splitmix64(unsigned long long *s)
{
    unsigned long long z = (*s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static double uniform_pm1(unsigned long long *s)
{
    return 2.0 * ((double)(splitmix64(s) >> 11) * 0x1.0p-53) - 1.0;
}

static double now_seconds(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

typedef struct {
    int kind;            /* 0 = dgetrf steps, 1 = dgemm rows, 2 = one dgetrf step at block b */
    int m, n, k, rows, nBlocks;
    unsigned long long seed;
    pthread_barrier_t *barrier;
    double t0, t1, flops;
} job_t;

static void *run_job(void *arg)
{
    job_t *jb = (job_t *)arg;
    unsigned long long s = jb->seed;
    if (jb->kind == 0) {
        const int n = jb->n;
        double *A = (double *)malloc(sizeof(double) * (size_t)n * n);
        int *piv = (int *)malloc(sizeof(int) * (size_t)n);
        for (size_t i = 0; i < (size_t)n * n; ++i) A[i] = uniform_pm1(&s);
        for (int i = 0; i < n; ++i) A[IDX(i, i, n)] += 0.25 * n;
        pthread_barrier_wait(jb->barrier);
        jb->t0 = now_seconds();
        oracle_dgetrf_steps(n, n, A, n, piv, 64, jb->nBlocks);
        jb->t1 = now_seconds();
        double fl = 0.0;
        for (int b = 0, j = 0; b < jb->nBlocks && j < n; ++b, j += 64) {
            const double r = (double)(n - j), w = r < 64 ? r : 64;
            /* panel + trsm + trailing update of one block step */
            fl += r * w * w + w * w * (r - w) + 2.0 * (r - w) * (r - w) * w;
        }
        jb->flops = fl;
        free(A);
        free(piv);
    } else if (jb->kind == 2) {
        /* block step b of the n x n LU: the step on the trailing (n-j) x (n-j)
         * matrix at column j = 64 b, addressed with the full leading
         * dimension n as inside the factorisation */
        const int n = jb->n, j = 64 * jb->nBlocks, r = n - j;
        double *A = (double *)malloc(sizeof(double) * (size_t)n * n);
        int *piv = (int *)malloc(sizeof(int) * (size_t)n);
        for (size_t i = 0; i < (size_t)n * n; ++i) A[i] = uniform_pm1(&s);
        for (int i = 0; i < n; ++i) A[IDX(i, i, n)] += 0.25 * n;
        pthread_barrier_wait(jb->barrier);
        jb->t0 = now_seconds();
        dgetrf_impl(r, r, &A[IDX(j, j, n)], n, piv, 64, 1, NULL);
        jb->t1 = now_seconds();
        const double w = r < 64 ? r : 64;
        jb->flops = r * w * w + w * w * (r - w) + 2.0 * (r - w) * (r - w) * w;
        free(A);
        free(piv);
    } else {
        const int m = jb->m, n = jb->n, k = jb->k, rows = jb->rows;
        double *A = (double *)malloc(sizeof(double) * (size_t)m * k);
        double *B = (double *)malloc(sizeof(double) * (size_t)k * n);
        double *C = (double *)malloc(sizeof(double) * (size_t)m * n);
        for (size_t i = 0; i < (size_t)m * k; ++i) A[i] = uniform_pm1(&s);
        for (size_t i = 0; i < (size_t)k * n; ++i) B[i] = uniform_pm1(&s);
        for (size_t i = 0; i < (size_t)m * n; ++i) C[i] = uniform_pm1(&s);
        pthread_barrier_wait(jb->barrier);
        jb->t0 = now_seconds();
        oracle_dgemm('N', 'N', rows, n, k, 1.5, A, m, B, k, 0.5, C, m);
        jb->t1 = now_seconds();
        jb->flops = 2.0 * rows * (double)n * k;
        free(A);
        free(B);
        free(C);
    }
    return NULL;
}

static double run_jobs(job_t *proto, int nThreads, double *flops_out)
{
    pthread_t *th = (pthread_t *)calloc((size_t)nThreads, sizeof(pthread_t));
    job_t *jobs = (job_t *)calloc((size_t)nThreads, sizeof(job_t));
    pthread_barrier_t bar;
    pthread_barrier_init(&bar, NULL, (unsigned)nThreads);
    for (int t = 0; t < nThreads; ++t) {
        jobs[t] = *proto;
        jobs[t].seed = proto->seed + 1000003ULL * (unsigned long long)t;
        jobs[t].barrier = &bar;
        pthread_create(&th[t], NULL, run_job, &jobs[t]);
    }
    for (int t = 0; t < nThreads; ++t) pthread_join(th[t], NULL);
    double t0 = jobs[0].t0, t1 = jobs[0].t1;
    for (int t = 1; t < nThreads; ++t) {
        if (jobs[t].t0 < t0) t0 = jobs[t].t0;
        if (jobs[t].t1 > t1) t1 = jobs[t].t1;
    }
    if (flops_out) *flops_out = jobs[0].flops;
    pthread_barrier_destroy(&bar);
    free(jobs);
    free(th);
    return t1 - t0;
}

double oracle_time_dgetrf_steps(int n, int nBlocks, int nThreads,
                                unsigned long long seed, double *flops_out)
{
    job_t p;
    memset(&p, 0, sizeof p);
    p.kind = 0;
    p.n = n;
    p.nBlocks = nBlocks;
    p.seed = seed;
    return run_jobs(&p, nThreads < 1 ? 1 : nThreads, flops_out);
}

double oracle_time_dgetrf_step_at(int n, int block, int nThreads,
                                  unsigned long long seed, double *flops_out)
{
    job_t p;
    memset(&p, 0, sizeof p);
    p.kind = 2;
    p.n = n;
    p.nBlocks = block;
    p.seed = seed;
    return run_jobs(&p, nThreads < 1 ? 1 : nThreads, flops_out);
}

double oracle_time_dgemm_rows(int m, int n, int k, int rows, int nThreads,
                              unsigned long long seed)
{
    job_t p;
    memset(&p, 0, sizeof p);
    p.kind = 1;
    p.m = m;
    p.n = n;
    p.k = k;
    p.rows = rows;
    p.seed = seed;
    return run_jobs(&p, nThreads < 1 ? 1 : nThreads, NULL);
}
