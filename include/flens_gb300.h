/*
 * flens_gb300.h -- C ABI of the GB300 dense GEMM / TRSM / LU library.
 *
 * Two groups of entry points:
 *
 *  1. Fortran-ABI drop-ins.  Same symbols, signatures, argument checks and
 *     error convention as the reference's shims; HOST pointers (device or
 *     managed pointers are also accepted), column-major, 1-based IPIV.
 *     INTEGER is int and names carry one trailing underscore, as in
 *     flens/lapack/interface/include/config.h:11,29-31 and
 *     flens/blas/interface/blas/config.h:22-28.  Argument errors call
 *     xerbla_(name, &pos, 6) and return (LAPACK routines also set INFO=-pos).
 *     A CUDA failure sets INFO to a FLENS_GB300_ERR_* code (< -1000); the BLAS
 *     routines, which have no INFO, print it and record it for
 *     flens_gb300_last_error().
 *
 *  2. flens_gb300_* device-pointer entry points (extension; no counterpart in
 *     the reference).  All pointers are device pointers, work is queued on
 *     `stream` (a cudaStream_t, NULL = legacy default stream) and the call
 *     returns without waiting unless stated.  Return value: 0 on success,
 *     -pos for an illegal argument pos (1-based, LAPACK numbering), or a
 *     FLENS_GB300_ERR_* code.
 */
#ifndef FLENS_GB300_H
#define FLENS_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define FLENS_GB300_ERR_CUDA          (-1001)
#define FLENS_GB300_ERR_TIMEOUT       (-1002)
#define FLENS_GB300_ERR_NO_DEVICE     (-1003)
#define FLENS_GB300_ERR_ALLOC         (-1004)
#define FLENS_GB300_ERR_UNSUPPORTED   (-1005)
#define FLENS_GB300_ERR_NOT_CONVERGED (-1006)

/* ---------------------------------------------- Fortran-ABI drop-ins --- */

/* C <- beta*C + alpha*op(A)*op(B).
 * Replaces dgemm_ at flens/blas/interface/blas/gemm.cc:120-133 (checks :158-181,
 * then blas::mm :226 -> cxxblas::gemm cxxblas/level3/gemm.tcc:176-190). */
void dgemm_(const char *TRANSA, const char *TRANSB, const int *M, const int *N,
            const int *K, const double *ALPHA, const double *A, const int *LDA,
            const double *B, const int *LDB, const double *BETA, double *C,
            const int *LDC);

/* B <- alpha*op(A)^-1*B (SIDE='L') or alpha*B*op(A)^-1 (SIDE='R').
 * Replaces dtrsm_ at flens/blas/interface/blas/trsm.cc:90-102 (checks
 * :136-160, then blas::sm :166 -> cxxblas::trsm cxxblas/level3/trsm.tcc:70-82). */
void dtrsm_(const char *SIDE, const char *UPLO, const char *TRANSA,
            const char *DIAG, const int *M, const int *N, const double *ALPHA,
            const double *A, const int *LDA, double *B, const int *LDB);

/* A = P*L*U with partial pivoting; INFO>0: U(INFO,INFO) is exactly zero.
 * Replaces dgetrf_ at flens/lapack/interface/src/getrf.cc:10-45
 * (-> lapack::trf flens/lapack/ge/trf.tcc:187-261). */
void dgetrf_(const int *M, const int *N, double *A, const int *LDA, int *IPIV,
             int *INFO);

/* Solve op(A)*X = B from dgetrf_'s factors.
 * Replaces dgetrs_ at flens/lapack/interface/src/getrs.cc:13-53
 * (-> lapack::trs flens/lapack/ge/trs.tcc:151-223). */
void dgetrs_(const char *TRANS, const int *N, const int *NRHS, const double *A,
             const int *LDA, const int *IPIV, double *B, const int *LDB,
             int *INFO);

/* Factor and solve A*X = B (no solve when INFO>0).
 * Replaces dgesv_ at flens/lapack/interface/src/gesv.cc:13-49
 * (-> lapack::sv flens/lapack/ge/sv.tcc:115-219). */
void dgesv_(const int *N, const int *NRHS, double *A, const int *LDA, int *IPIV,
            double *B, const int *LDB, int *INFO);

/* C <- alpha*A*A^T + beta*C (TRANS='N') or alpha*A^T*A + beta*C ('T'/'C') on
 * the UPLO triangle of C.  Replaces dsyrk_ at
 * flens/blas/interface/blas/syrk.cc:104-160 (-> blas::rk ->
 * cxxblas::syrk, cxxblas/level3/syrk.tcc:42-90: the triangle is scaled by
 * beta unless beta == 1, then k rank-1 updates; no alpha == 0 shortcut). */
void dsyrk_(const char *UPLO, const char *TRANS, const int *N, const int *K,
            const double *ALPHA, const double *A, const int *LDA,
            const double *BETA, double *C, const int *LDC);

/* B <- alpha*op(A)*B (SIDE='L') or alpha*B*op(A) ('R'), A triangular.
 * Replaces dtrmm_ at flens/blas/interface/blas/trmm.cc:108-205 (-> blas::mm
 * -> cxxblas::trmm, cxxblas/level3/trmm.tcc:40-70: alpha applied after the
 * product). */
void dtrmm_(const char *SIDE, const char *UPLO, const char *TRANSA,
            const char *DIAG, const int *M, const int *N, const double *ALPHA,
            const double *A, const int *LDA, double *B, const int *LDB);

/* C <- beta*C + alpha*A*B (SIDE='L') or alpha*B*A ('R'), A symmetric with
 * the UPLO triangle stored.  Replaces dsymm_ at
 * flens/blas/interface/blas/symm.cc:93-174 (-> cxxblas::symm,
 * cxxblas/level3/symm.tcc:40-70). */
void dsymm_(const char *SIDE, const char *UPLO, const int *M, const int *N,
            const double *ALPHA, const double *A, const int *LDA,
            const double *B, const int *LDB, const double *BETA, double *C,
            const int *LDC);

/* C <- beta*C + alpha*(op(A)*op(B)^T + op(B)*op(A)^T) on the UPLO triangle.
 * Replaces dsyr2k_ at flens/blas/interface/blas/syr2k.cc:115-218
 * (-> cxxblas::syr2k, cxxblas/level3/syr2k.tcc:42-95). */
void dsyr2k_(const char *UPLO, const char *TRANS, const int *N, const int *K,
             const double *ALPHA, const double *A, const int *LDA,
             const double *B, const int *LDB, const double *BETA, double *C,
             const int *LDC);

/* Cholesky factorisation A = L*L^T (UPLO='L') or U^T*U ('U') of the UPLO
 * triangle in place; INFO=k>0: the leading minor of order k is not positive
 * definite.  UPLO must be exactly 'U' or 'L', as in the reference.
 * Replaces dpotrf_ at flens/lapack/interface/src/potrf.cc:11-41
 * (-> lapack::potrf flens/lapack/po/potrf.tcc:56-150). */
void dpotrf_(const char *UPLO, const int *N, double *A, const int *LDA,
             int *INFO);

/* Solve A*X = B from dpotrf_'s factor.
 * Replaces dpotrs_ at flens/lapack/interface/src/potrs.cc:13-49
 * (-> lapack::potrs flens/lapack/po/potrs.tcc:54-100). */
void dpotrs_(const char *UPLO, const int *N, const int *NRHS, const double *A,
             const int *LDA, double *B, const int *LDB, int *INFO);

/* Factor and solve a symmetric positive definite system (no solve when
 * INFO>0).  Replaces dposv_ at flens/lapack/interface/src/posv.cc:13-51
 * (-> lapack::posv flens/lapack/po/posv.tcc:55-70).  Unlike the reference's
 * shim, which discards posv's return value, INFO reports a failed
 * factorisation (LAPACK DPOSV semantics). */
void dposv_(const char *UPLO, const int *N, const int *NRHS, double *A,
            const int *LDA, double *B, const int *LDB, int *INFO);

/* Inverse of a triangular matrix in place (UPLO exactly 'U'/'L', DIAG
 * 'N'/'U', as in the reference); INFO=k>0: A(k,k) is exactly zero and A is
 * untouched.  Replaces dtrtri_ at flens/lapack/interface/src/trtri.cc:9-55
 * (-> lapack::tri flens/lapack/tr/tri.tcc).  The reference's shim discards
 * tri's return value; this one reports it (LAPACK DTRTRI semantics). */
void dtrtri_(const char *UPLO, const char *DIAG, const int *N, double *A,
             const int *LDA, int *INFO);

/* Inverse of A from dgetrf_'s factors and pivots, in place.  LWORK=-1 is a
 * workspace query (WORK(1) = N*64); otherwise LWORK >= max(1,N) and WORK(1)
 * receives the optimum on exit (the GPU path keeps its own workspace).
 * INFO=k>0: U(k,k) is exactly zero, A holds the factors.  Replaces dgetri_
 * at flens/lapack/interface/src/getri.cc:10-53 (-> lapack::tri
 * flens/lapack/ge/tri.tcc). */
void dgetri_(const int *N, double *A, const int *LDA, const int *IPIV,
             double *WORK, const int *LWORK, int *INFO);

/* Iterative refinement of X (op(A) X = B) with componentwise backward
 * error BERR and forward error bound FERR per right-hand side.  Replaces
 * dgerfs_ at flens/lapack/interface/src/gerfs.cc:13-66 (-> lapack::rfs
 * flens/lapack/ge/rfs.tcc).  WORK, IWORK are not used (device workspace). */
void dgerfs_(const char *TRANS, const int *N, const int *NRHS, const double *A,
             const int *LDA, const double *AF, const int *LDAF, const int *IPIV,
             const double *B, const int *LDB, double *X, const int *LDX,
             double *FERR, double *BERR, double *WORK, int *IWORK, int *INFO);

/* Reciprocal condition number estimate (1-norm for NORM '1'/'O', infinity
 * norm for 'I') from dgetrf_'s factors and the norm of A.  Replaces dgecon_
 * at flens/lapack/interface/src/gecon.cc:13-51 (-> lapack::con
 * flens/lapack/ge/cond.tcc).  Where the reference's latrs would switch to its
 * overflow-scaled solve (condition beyond about 1e290), RCOND is 0. */
void dgecon_(const char *NORM, const int *N, const double *A, const int *LDA,
             const double *ANORM, double *RCOND, double *WORK, int *IWORK,
             int *INFO);

/* Row and column scalings that equilibrate A.  Replaces dgeequ_ at
 * flens/lapack/interface/src/geequ.cc:10-40 (-> flens/lapack/ge/equ.tcc). */
void dgeequ_(const int *M, const int *N, const double *A, const int *LDA,
             double *R, double *C, double *ROWCND, double *COLCND, double *AMAX,
             int *INFO);

/* Apply them when worthwhile; EQUED 'N', 'R', 'C' or 'B'.  Replaces dlaqge_
 * at flens/lapack/interface/src/laqge.cc:10-27 (-> flens/lapack/la/laq.tcc). */
void dlaqge_(const int *M, const int *N, double *A, const int *LDA,
             const double *R, const double *C, const double *ROWCND,
             const double *COLCND, const double *AMAX, char *EQUED);

/* Expert driver: equilibrate (FACT='E'), factor (or use AF/IPIV, FACT='F'),
 * condition estimate, solve, refine, error bounds; WORK(1) = reciprocal
 * pivot growth.  INFO = N+1 when RCOND < eps.  Replaces dgesvx_ at
 * flens/lapack/interface/src/gesvx.cc:13-118 (-> lapack::svx
 * flens/lapack/ge/svx.tcc).  EQUED reports the scaling actually applied; the
 * reference's shim returns 'N' there (its svx takes EQUED by value). */
void dgesvx_(const char *FACT, const char *TRANS, const int *N, const int *NRHS,
             double *A, const int *LDA, double *AF, const int *LDAF, int *IPIV,
             char *EQUED, double *R, double *C, double *B, const int *LDB,
             double *X, const int *LDX, double *RCOND, double *FERR,
             double *BERR, double *WORK, int *IWORK, int *INFO);

/* Weak default error handler (prints, does not stop).  Link your own
 * xerbla_ to override it, as with Netlib BLAS/LAPACK. */
void xerbla_(const char *SRNAME, const int *INFO, int SRNAME_LEN);

/* ---------------------------------------- device-pointer entry points --- */

/* dgemm on device memory (same semantics as dgemm_: beta scaling first,
 * alpha==0 returns without reading A or B).  Async on stream. */
int flens_gb300_dgemm(char transA, char transB, int m, int n, int k,
                      double alpha, const double *A, int ldA,
                      const double *B, int ldB, double beta, double *C,
                      int ldC, void *stream);

/* dtrsm on device memory.  Async on stream. */
int flens_gb300_dtrsm(char side, char uplo, char transA, char diag, int m,
                      int n, double alpha, const double *A, int ldA,
                      double *B, int ldB, void *stream);

/* dgetrf on device memory: ipiv (min(m,n) ints, 1-based) and info (one int)
 * are device pointers, written asynchronously.  Async on stream. */
int flens_gb300_dgetrf(int m, int n, double *A, int ldA, int *ipiv, int *info,
                       void *stream);

/* Precision form of dgetrf on device memory: the same factorisation (FP64
 * storage, FP64 panels with the reference's pivot rule, FP64 interchanges and
 * triangular solves) with the trailing update beyond each outer block of
 * outer_nb columns (a multiple of 64; 0 = 512) computed by the split GEMM
 * (flens_gb300_dgemm_split) on the BF16 tensor cores.  The factors are
 * FP64-accurate, not bitwise those of flens_gb300_dgetrf; pivots can differ
 * where two candidates are within rounding of each other.  Synchronises on
 * stream once per outer block (the split GEMM's statistics).  Returns
 * -7 for a bad outer_nb. */
int flens_gb300_dgetrf_split(int m, int n, double *A, int ldA, int *ipiv,
                             int *info, int outer_nb, void *stream);

/* dgetrs on device memory (ipiv device, 1-based).  Async on stream. */
int flens_gb300_dgetrs(char trans, int n, int nrhs, const double *A, int ldA,
                       const int *ipiv, double *B, int ldB, void *stream);

/* dgesv on device memory.  Waits for the factorisation to read *info (a
 * device int) and solves only when it is 0; the solve is queued async. */
int flens_gb300_dgesv(int n, int nrhs, double *A, int ldA, int *ipiv, double *B,
                      int ldB, int *info, void *stream);

/* dsyrk on device memory (UPLO/TRANS in either case).  Async on stream. */
int flens_gb300_dsyrk(char uplo, char trans, int n, int k, double alpha,
                      const double *A, int ldA, double beta, double *C,
                      int ldC, void *stream);

/* dtrmm, dsymm, dsyr2k on device memory (characters in either case).  The
 * triangular / symmetric operand is expanded to a full matrix in the
 * workspace and the product runs on the FP64 GEMM.  Async on stream. */
int flens_gb300_dtrmm(char side, char uplo, char transA, char diag, int m,
                      int n, double alpha, const double *A, int ldA,
                      double *B, int ldB, void *stream);
int flens_gb300_dsymm(char side, char uplo, int m, int n, double alpha,
                      const double *A, int ldA, const double *B, int ldB,
                      double beta, double *C, int ldC, void *stream);
int flens_gb300_dsyr2k(char uplo, char trans, int n, int k, double alpha,
                       const double *A, int ldA, const double *B, int ldB,
                       double beta, double *C, int ldC, void *stream);

/* dtrtri / dgetri on device memory (ipiv device, 1-based; info a device
 * int).  Both wait for the stream once to read the zero-pivot check. */
int flens_gb300_dtrtri(char uplo, char diag, int n, double *A, int ldA,
                       int *info, void *stream);
int flens_gb300_dgetri(int n, double *A, int ldA, const int *ipiv, int *info,
                       void *stream);

/* Device forms of gecon, gerfs, geequ, laqge, gesvx: matrices, pivots and
 * the scaling vectors r, c in device memory; rcond, ferr, berr, rowcnd,
 * colcnd, amax, rpvgrw, info and equed are host scalars / arrays.  All
 * synchronise (their iterations branch on reductions).  gecon returns
 * FLENS_GB300_ERR_UNSUPPORTED (with *rcond = 0) where latrs would scale. */
int flens_gb300_dgecon(char norm, int n, const double *LU, int ldLU,
                       double anorm, double *rcond, void *stream);
int flens_gb300_dgerfs(char trans, int n, int nrhs, const double *A, int ldA,
                       const double *AF, int ldAF, const int *ipiv,
                       const double *B, int ldB, double *X, int ldX,
                       double *ferr, double *berr, void *stream);
int flens_gb300_dgeequ(int m, int n, const double *A, int ldA, double *r,
                       double *c, double *rowcnd, double *colcnd, double *amax,
                       int *info, void *stream);
int flens_gb300_dlaqge(int m, int n, double *A, int ldA, const double *r,
                       const double *c, double rowcnd, double colcnd,
                       double amax, char *equed, void *stream);
int flens_gb300_dgesvx(char fact, char trans, int n, int nrhs, double *A,
                       int ldA, double *AF, int ldAF, int *ipiv, char *equed,
                       double *r, double *c, double *B, int ldB, double *X,
                       int ldX, double *rcond, double *ferr, double *berr,
                       double *rpvgrw, int *info, void *stream);

/* dpotrf on device memory; info is a device int.  Blocked right-looking
 * (64-column steps: potf2 of the diagonal block, trsm, syrk of the trailing
 * triangle); waits for the stream once per step to stop at the first
 * non-positive pivot. */
int flens_gb300_dpotrf(char uplo, int n, double *A, int ldA, int *info,
                       void *stream);

/* dpotrs on device memory.  Async on stream. */
int flens_gb300_dpotrs(char uplo, int n, int nrhs, const double *A, int ldA,
                       double *B, int ldB, void *stream);

/* dposv on device memory: dpotrf, then dpotrs when *info (device) is 0. */
int flens_gb300_dposv(char uplo, int n, int nrhs, double *A, int ldA,
                      double *B, int ldB, int *info, void *stream);

/* ------------------------------------------- precision form (extension) --- */

/* C <- alpha*op(A)*op(B) + beta*C, FP32 operands in device memory, products
 * on the tcgen05 tensor cores in `precision` (0 = TF32, 1 = BF16, 2 = FP8
 * e4m3 with per-row / per-column scaling, 3 = FP32-accurate 3xTF32, 5 and 6 =
 * FP8 e4m3 as above with each scaled entry split into two or three e4m3
 * terms t0 + t1 (+ t2) and the products t_i t_j with i + j <= 1 or <= 2
 * taken, about 2^-8 or 2^-12 relative per entry; 4 is not a product
 * precision and returns -1) with FP32 accumulation.  Beta scales C by a multiply, as cxxblas gescal does.  No
 * reference counterpart: FLENS's float gemm is the generic loop
 * (cxxblas/level3/gemm.tcc:42-190).  Async on stream. */
int flens_gb300_sgemm_tc(int precision, char transA, char transB, int m, int n,
                         int k, float alpha, const float *A, int ldA,
                         const float *B, int ldB, float beta, float *C, int ldC,
                         void *stream);

/* LU with partial pivoting of an m x n FP32 matrix in device memory (column-
 * major, 1-based pivots), the factorisation of the precision form: panels
 * in FP32 arithmetic (the reference's tf2 for float: first-maximum pivot
 * search, scaling by the reciprocal above FLT_MIN; FLENS_GB300_PANEL32=0
 * runs them in FP64 arithmetic instead), U12 = L11^-1 A12 in FP32, and the
 * trailing updates A22 -= L21 U12 on the tensor cores in `precision`
 * (0, 1, 2, 3, 5 or 6 as
 * for flens_gb300_sgemm_tc) or, for precision -1, on the CUDA cores in
 * FP32.  *info (device) as dgetrf's.  The counterpart of FLENS's float trf
 * (flens/lapack/ge/trf.tcc:59-152).  Async on stream. */
int flens_gb300_sgetrf_tc(int precision, int m, int n, float *A, int ldA,
                          int *ipiv, int *info, void *stream);

/* FP64-accurate C <- beta*C + alpha*op(A)*op(B) on device memory without FP64
 * arithmetic units: every row of op(A) / column of op(B) is scaled by a power
 * of two and cut into `slices` balanced 7-bit integer digits (exact in BF16);
 * the digit products of slice pairs s+t <= slices+1 run on the tcgen05 tensor
 * cores in groups whose FP32 sums are provably exact (every partial sum an
 * integer <= 2^24), and are recombined in FP64.  slices = 0 picks the count
 * from the data (7*slices >= 53 + log2 max_i(2^e_i nnz_i / sum_k |a_ik|));
 * *slices_used receives it, or -1 when non-finite entries or exponents beyond
 * about 2^+-1000 sent the call to the plain FP64 kernel.  Argument positions
 * and semantics as dgemm_ (flens/blas/interface/blas/gemm.cc:158-181; beta
 * scaling by a multiply, alpha == 0 or k == 0 only scale C), slices at 14
 * (0..20).  The dgemm_ counterpart replaced for FP64-accurate products is
 * cxxblas::gemm (cxxblas/level3/gemm.tcc:176-190).  Reads its statistics back
 * to the host, so it synchronises on stream before the product is queued. */
int flens_gb300_dgemm_split(char transA, char transB, int m, int n, int k,
                            double alpha, const double *A, int ldA,
                            const double *B, int ldB, double beta, double *C,
                            int ldC, int slices, int *slices_used, void *stream);

/* Solve A X = B (device, column-major FP64; A and B untouched) to FP64
 * accuracy from an LU in FP32 storage whose trailing updates run on the
 * tensor cores in `precision` (0, 1, 2, 3, 5 or 6 as above), or, for precision 4, from the
 * FP64-accurate flens_gb300_dgetrf_split factors (FP64 storage and solves;
 * for systems too ill-conditioned for FP32 factors, kappa*u32 >> 1),
 * refined in FP64: solver 0 =
 * classical refinement (stops like the reference's rfs,
 * flens/lapack/ge/rfs.tcc:182-188), 1 = GMRES-IR, 2 = classical switching to
 * GMRES-IR per column when the backward error stops halving.  Stops when the
 * normwise backward error ||b-Ax||inf/(||A||inf||x||inf+||b||inf) <= tol
 * (tol <= 0: n*eps64) or after max_iter steps (<= 0: 30).  Outputs: refinement
 * steps (classical steps + GMRES iterations), final backward error, INFO of
 * the factorisation (>0: exactly singular pivot, no solve).  Returns
 * FLENS_GB300_ERR_NOT_CONVERGED if the tolerance was not reached (X holds the
 * last iterate).  Synchronises on stream. */
int flens_gb300_dgesv_mixed(int n, int nrhs, const double *A, int ldA,
                            const double *B, int ldB, double *X, int ldX,
                            int precision, int solver, int max_iter, double tol,
                            int *iters, double *berr, int *info, void *stream);

/* ---------------------------------------------- batched (extension) --- */

/* Plan for solving `count` independent systems A_i X_i = B_i (A_i n_i x n_i,
 * B_i n_i x nrhs_i, column-major FP64 in device memory), each as the
 * reference's dgesv (flens/lapack/ge/sv.tcc:58-77).  n, nrhs, lda, ldb and the
 * pointer arrays A, ipiv (n_i ints each, 1-based), B are HOST arrays read now;
 * info, iters, berr are DEVICE arrays of `count` entries written by every
 * execution.  precision 0 = FP64 (A_i <- LU factors); 1 = FP32 LU + FP64
 * refinement (A_i untouched, iters_i = refinement steps, berr_i = final
 * normwise backward error, max_iter bounds the steps) for every matrix with
 * nrhs_i <= 32: in the team's shared memory when its FP32 working set fits
 * there, otherwise on FP32 factors of a copy of A_i in a device pool that the
 * plan allocates (one slot per team, sized for the largest such matrix).
 * Matrices with more right-hand sides, or all of them if that pool cannot be
 * allocated, take the FP64 path (iters_i = -1, A_i <- LU factors).
 * precision 2 = per matrix: precision 1 where it is the faster of the two
 * (n_i >= 256 and nrhs_i <= n_i/64), the FP64 path otherwise.  B_i <- X_i
 * when INFO_i == 0, untouched otherwise.  Creating a plan autotunes the team
 * size and panel width of each size bucket (first use per device;
 * FLENS_GB300_BATCH_TUNE=0 disables it, FLENS_GB300_BATCH_TEAM=T and
 * FLENS_GB300_BATCH_PANEL=8|16 force them) and captures one persistent launch
 * in a CUDA graph.  Synchronises on stream. */
int flens_gb300_dgesv_batched_plan(int count, const int *n, const int *nrhs,
                                   double *const *A, const int *lda,
                                   int *const *ipiv, double *const *B,
                                   const int *ldb, int *info, int precision,
                                   int *iters, double *berr, int max_iter,
                                   void *stream, void **plan);

/* Run a plan: one graph launch.  Async on stream. */
int flens_gb300_batched_execute(void *plan, void *stream);

/* Release a plan. */
void flens_gb300_batched_destroy(void *plan);

/* Team size (threads per matrix) the plan uses for size bucket 0..9
 * (n <= 16, 32, 48, 64, 108, 216, 320, 432, 864, larger); -1 for any other
 * bucket index. */
int flens_gb300_batched_team(void *plan, int bucket);

/* Panel width (8 or 16 columns) of the blocked factorisation that the plan
 * uses for size bucket 0..9: matrices that do not fit their team's shared
 * memory are factored in place, one panel at a time.  Tuned together with the
 * team size; FLENS_GB300_BATCH_PANEL=8|16 forces it.  -1 for any other bucket
 * index.  No counterpart in the reference. */
int flens_gb300_batched_panel(void *plan, int bucket);

/* dgetrs on device memory for callers that must not allocate device memory
 * once running (a fixed, pre-reserved memory budget, a memory pool owned by
 * another framework, or a process that forbids cudaMalloc after start-up).
 * No counterpart in the reference.  Same arguments, results and return codes
 * as flens_gb300_dgetrs, but it calls no cudaMalloc/cudaFree, not even on a
 * stream it has never seen: all of its scratch (interchange buffers, and the
 * ready flags and status word of the chained solve used for nrhs <= 4) is a
 * fixed 8 MiB device array inside the library, held on every GPU that loads
 * the library until exit.  A call needs 33024 + round_up(4*n,256) +
 * 8*n*nrhs bytes of it (n=8192: nrhs <= 127); larger calls return
 * FLENS_GB300_ERR_UNSUPPORTED with a message.  Each call clears the parts
 * that must start at zero on its own stream.  All calls share that array:
 * calls that overlap on the GPU race, so serialise them.  The first call on a
 * device looks up the array's address (cudaGetSymbolAddress).  Use inside a
 * captured CUDA graph is not tested.  Async on stream. */
int flens_gb300_dgetrs_noalloc(char trans, int n, int nrhs, const double *A,
                               int ldA, const int *ipiv, double *B, int ldB,
                               void *stream);

/* Waits for `stream` and reports device-side failures (a bounded wait that
 * timed out) as FLENS_GB300_ERR_TIMEOUT. */
int flens_gb300_sync(void *stream);

/* Last error message of the calling thread ("" if none). */
const char *flens_gb300_last_error(void);

/* BLAS routines have no INFO: an internal failure (FLENS_GB300_ERR_*) of
 * dgemm_, dtrsm_, dsyrk_, dtrmm_, dsymm_, dsyr2k_ or dlaqge_ goes to `hook`
 * (routine name, status, message; called on the failing thread) instead of a
 * line on stderr; nullptr restores the stderr line.  The calling thread's last
 * such status (0 on success) is flens_gb300_blas_status().  The reference's
 * BLAS shims can fail only through xerbla_ (flens/blas/interface/blas/
 * gemm.cc:158-181); these have no counterpart there. */
void flens_gb300_set_blas_error_hook(void (*hook)(const char *routine, int status,
                                                  const char *message));
int flens_gb300_blas_status(void);

/* Diagnostics, no counterpart in the reference.  Device allocations
 * (cudaMalloc) the library has made since it was loaded. */
long long flens_gb300_device_alloc_count(void);

/* Test hook for the allocation-failure paths: the next `count` device
 * allocations of the library fail as an out-of-memory cudaMalloc would, so
 * the calls that needed them return FLENS_GB300_ERR_ALLOC (or INFO =
 * FLENS_GB300_ERR_ALLOC for the Fortran-ABI LAPACK symbols) with a message.
 * count <= 0 clears it. */
void flens_gb300_test_fail_device_allocs(int count);

/* Test hook: the mixed solve's chunked GEMVs on their own.  uplo 'L' or 'U':
 * the explicit-inverse preconditioner product, y = A x for an n x n FP64 A
 * whose other triangle (above the diagonal for 'L', below for 'U') holds
 * zeros; only the triangle and the zeros inside its 16 x 16 diagonal blocks
 * are read.  uplo 'G': the Arnoldi product y = A x over all of A.  Scratch
 * `part` (*part_elems doubles) and `cnt` (*cnt_elems counters, zero before
 * the first call; every call leaves them zero).  With part == NULL the call
 * only reports the two sizes.  Returns 0, -1/-2/-4 for uplo/n/ldA, or a
 * FLENS_GB300_ERR_* code.  Async on stream. */
int flens_gb300_test_trmv_zeros(char uplo, int n, const double *A, int ldA, const double *x,
                                double *y, double *part, unsigned *cnt, size_t *part_elems,
                                size_t *cnt_elems, void *stream);

/* Launch accounting: kernel launches issued since load; per-family CUDA-event
 * timing on the launching streams (enable clears the totals; read waits for
 * the recorded events and returns -1 for an unknown family); family names. */
long long flens_gb300_launch_count(void);
void flens_gb300_timing_enable(int on);
int flens_gb300_timing_read(int family, double *ms, long long *launches,
                            double *flops, double *bytes);
const char *flens_gb300_family_name(int family);

/* xerbla_ calls made by this library on the calling thread: count, the last
 * parameter position and routine name (for callers that cannot override
 * xerbla_). */
int flens_gb300_xerbla_calls(void);
int flens_gb300_xerbla_info(void);
const char *flens_gb300_xerbla_name(void);

/* Library version as an integer (major*100 + minor). */
int flens_gb300_version(void);

#ifdef __cplusplus
}
#endif

#endif /* FLENS_GB300_H */
