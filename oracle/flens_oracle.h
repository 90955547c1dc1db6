/*
 * flens_oracle.h -- CPU restatement of FLENS's generic dense GEMM / TRSM / LU
 * path, used ONLY as test infrastructure (the reference results the CUDA library is tested against, and
 * the timed CPU baseline in bench.py).  Nothing in the product links this.
 *
 * Every routine follows the operation order of the reference's generic C++
 * templates (cited per function in flens_oracle.c) so that, compiled with
 * -ffp-contract=off, its results are bitwise identical to the reference's own
 * Fortran-ABI shims compiled from source (oracle/Makefile target `ref`).
 *
 * Conventions: column-major storage, leading dimensions in elements,
 * pivot vectors 1-based (LAPACK style), characters 'N','T','C','L','R','U'.
 */
#ifndef FLENS_ORACLE_H
#define FLENS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* C <- beta*C + alpha*op(A)*op(B)            cxxblas/level3/gemm.tcc:42-190 */
void oracle_dgemm(char transA, char transB, int m, int n, int k,
                  double alpha, const double *A, int ldA,
                  const double *B, int ldB,
                  double beta, double *C, int ldC);

/* B <- alpha*op(A)^-1*B  or  alpha*B*op(A)^-1  cxxblas/level3/trsm.tcc:40-82 */
void oracle_dtrsm(char side, char upLo, char transA, char diag,
                  int m, int n, double alpha,
                  const double *A, int ldA, double *B, int ldB);

/* 0-based index of the first max |x_i|; -1 if n<=0  cxxblas/level1/iamax.tcc:42-92 */
int oracle_idamax(int n, const double *x, int incX);

/* row interchanges, rows k1..k2 (1-based), inc>0 forward, inc<0 reverse
 *                                               flens/lapack/la/laswp.tcc:54-93 */
void oracle_dlaswp(int nCols, double *A, int ldA, int k1, int k2,
                   const int *piv, int inc);

/* unblocked LU of an m x n panel, piv 1-based local   flens/lapack/ge/tf2.tcc:56-136 */
int oracle_dgetf2(int m, int n, double *A, int ldA, int *piv);

/* blocked right-looking LU, block size nb (reference: 64)
 *                                               flens/lapack/ge/trf.tcc:59-152 */
int oracle_dgetrf_nb(int m, int n, double *A, int ldA, int *piv, int nb);
int oracle_dgetrf(int m, int n, double *A, int ldA, int *piv);
/* oracle_dgetrf plus, per pivot search j, (|first| - |second|) / |first| of
 * the two largest candidates (gap[min(m,n)]); same factors and pivots. */
int oracle_dgetrf_gaps(int m, int n, double *A, int ldA, int *piv, double *gap);

/* First `nBlocks` block steps of oracle_dgetrf_nb only (a bounded sample of
 * the full factorisation, for timing); returns info so far. */
int oracle_dgetrf_steps(int m, int n, double *A, int ldA, int *piv,
                        int nb, int nBlocks);

/* solve op(A) X = B from the LU factors          flens/lapack/ge/trs.tcc:59-109 */
void oracle_dgetrs(char trans, int n, int nRhs, const double *A, int ldA,
                   const int *piv, double *B, int ldB);

/* trf then trs(NoTrans) if info==0               flens/lapack/ge/sv.tcc:58-77 */
int oracle_dgesv(int n, int nRhs, double *A, int ldA, int *piv,
                 double *B, int ldB);

/* C <- beta*C + alpha*op(A)*op(A)^T on the uplo triangle of C
 *                                               cxxblas/level3/syrk.tcc:42-90 */
void oracle_dsyrk(char upLo, char trans, int n, int k, double alpha,
                  const double *A, int ldA, double beta, double *C, int ldC);

/* B <- alpha*op(A)*B or alpha*B*op(A), A triangular
 *                                               cxxblas/level3/trmm.tcc:40-70 */
void oracle_dtrmm(char side, char upLo, char transA, char diag, int m, int n,
                  double alpha, const double *A, int ldA, double *B, int ldB);

/* C <- beta*C + alpha*A*B or alpha*B*A, A symmetric (upLo triangle stored)
 *                                               cxxblas/level3/symm.tcc:40-70 */
void oracle_dsymm(char side, char upLo, int m, int n, double alpha,
                  const double *A, int ldA, const double *B, int ldB,
                  double beta, double *C, int ldC);

/* C <- beta*C + alpha*(op(A)op(B)^T + op(B)op(A)^T) on the upLo triangle
 *                                               cxxblas/level3/syr2k.tcc:42-95 */
void oracle_dsyr2k(char upLo, char trans, int n, int k, double alpha,
                   const double *A, int ldA, const double *B, int ldB,
                   double beta, double *C, int ldC);

/* inverse of a triangular matrix in place, unblocked  flens/lapack/tr/ti2.tcc */
int oracle_dtrti2(char upLo, char diag, int n, double *A, int ldA);

/* blocked triangular inverse (block 64, ilaenv TRTRI); info = first exactly
 * zero diagonal element (non-unit), nothing changed then
 *                                                flens/lapack/tr/tri.tcc */
int oracle_dtrtri_nb(char upLo, char diag, int n, double *A, int ldA, int nb);
int oracle_dtrtri(char upLo, char diag, int n, double *A, int ldA);

/* inverse from the LU factors of dgetrf (block 64, ilaenv GETRI; workspace
 * allocated inside); info as dtrtri of U         flens/lapack/ge/tri.tcc */
int oracle_dgetri(int n, double *A, int ldA, const int *piv);

/* ---- refinement, condition estimate, equilibration (expert driver) ---- */
/* norm '1'/'O' (max column sum), 'I' (max row sum), 'M' (max |a_ij|)
 *                                                flens/lapack/la/lan.tcc */
double oracle_dlange(char norm, int m, int n, const double *A, int ldA);

/* Hager/Higham 1-norm estimator, reverse communication (v, x, sgn length n;
 * isave[3]); kase = 0 on entry starts, on return 1: x <- A x, 2: x <- A^T x,
 * 0: done, est holds the estimate               flens/lapack/la/lacn2.tcc */
void oracle_dlacn2(int n, double *v, double *x, int *sgn, double *est, int *kase,
                   int *isave);

/* triangular solve with overflow protection: only the unscaled path
 * (blas::sv) is restated.  Returns 0 and *scale = 1 when the reference takes
 * it, -1 (x untouched) when the reference would scale
 *                                                flens/lapack/la/latrs.tcc */
int oracle_dlatrs(char upLo, char trans, char diag, int normIn, int n,
                  const double *A, int ldA, double *x, double *scale,
                  double *cnorm);

/* reciprocal condition number estimate from the LU factors; returns -1
 * where latrs would need its scaled path           flens/lapack/ge/cond.tcc */
int oracle_dgecon(char norm, int n, const double *A, int ldA, double anorm,
                  double *rcond);

/* iterative refinement with componentwise backward error and forward error
 * bound per right-hand side                        flens/lapack/ge/rfs.tcc */
int oracle_dgerfs(char trans, int n, int nRhs, const double *A, int ldA,
                  const double *AF, int ldAF, const int *piv, const double *B,
                  int ldB, double *X, int ldX, double *ferr, double *berr);

/* row/column equilibration scalings                flens/lapack/ge/equ.tcc */
int oracle_dgeequ(int m, int n, const double *A, int ldA, double *r, double *c,
                  double *rowcnd, double *colcnd, double *amax);

/* apply the scalings when worthwhile; returns 'N','R','C','B'
 *                                                   flens/lapack/la/laq.tcc */
char oracle_dlaqge(int m, int n, double *A, int ldA, const double *r,
                   const double *c, double rowcnd, double colcnd, double amax);

/* expert driver: fact 'N'/'E'/'F', *equed in/out, rpvgrw = reciprocal pivot
 * growth (WORK(1) of the reference)                 flens/lapack/ge/svx.tcc */
int oracle_dgesvx(char fact, char trans, int n, int nRhs, double *A, int ldA,
                  double *AF, int ldAF, int *piv, char *equed, double *r,
                  double *c, double *B, int ldB, double *X, int ldX,
                  double *rcond, double *ferr, double *berr, double *rpvgrw);

/* y <- beta*y + alpha*op(A)*x                  cxxblas/level2/gemv.tcc:42-200 */
void oracle_dgemv(char trans, int m, int n, double alpha, const double *A,
                  int ldA, const double *x, int incX, double beta, double *y,
                  int incY);

/* unblocked Cholesky of the uplo triangle       flens/lapack/po/potf2.tcc:56-140 */
int oracle_dpotf2(char upLo, int n, double *A, int ldA);

/* blocked Cholesky (reference block size 64: ilaenv PO TRF)
 *                                               flens/lapack/po/potrf.tcc:56-150 */
int oracle_dpotrf_nb(char upLo, int n, double *A, int ldA, int nb);
int oracle_dpotrf(char upLo, int n, double *A, int ldA);

/* solve A X = B from the Cholesky factor         flens/lapack/po/potrs.tcc:54-100 */
void oracle_dpotrs(char upLo, int n, int nRhs, const double *A, int ldA,
                   double *B, int ldB);

/* potrf then potrs if info==0                    flens/lapack/po/posv.tcc:55-70 */
int oracle_dposv(char upLo, int n, int nRhs, double *A, int ldA, double *B,
                 int ldB);

/*
 * Timing helper for the CPU baseline: nThreads independent copies of the
 * seeded n x n input (uniform[-1,1] + n/4 on the diagonal), each factorised
 * for the first nBlocks block steps with nb=64.  Returns the wall seconds of
 * the factorisation phase (all threads started together).  flops_out gets the
 * flops one thread performed (sum over the steps), so a caller can scale the
 * sample to a full factorisation.
 */
/* Wall time of block step `block` (nb = 64) of an n x n LU, run on the
 * trailing matrix at column 64*block with leading dimension n, by nThreads
 * threads each on its own copy; *flops_out = that step's flops. */
double oracle_time_dgetrf_step_at(int n, int block, int nThreads,
                                  unsigned long long seed, double *flops_out);
double oracle_time_dgetrf_steps(int n, int nBlocks, int nThreads,
                                unsigned long long seed, double *flops_out);

/* Same for GEMM: nThreads independent C = 1.5*A*B + 0.5*C on the first
 * `rows` rows of an m x n x k problem.  Returns wall seconds. */
double oracle_time_dgemm_rows(int m, int n, int k, int rows, int nThreads,
                              unsigned long long seed);

#ifdef __cplusplus
}
#endif

#endif
