/* Test double for libflens_gb300.so: every Fortran-ABI entry point the C++
 * drop-in header calls prints its name and scalar arguments, so
 * tests/test_cpp_shim.py can check how FLENS's calls (including row-major
 * storage) are translated.  No computation. */
#include <stdio.h>

static void ok(int *info) { if (info) *info = 0; }

const char *flens_gb300_last_error(void) { return ""; }

void dgemm_(const char *ta, const char *tb, const int *m, const int *n, const int *k,
            const double *alpha, const double *A, const int *lda, const double *B, const int *ldb,
            const double *beta, double *C, const int *ldc)
{ printf("dgemm_ %c %c m=%d n=%d k=%d lda=%d ldb=%d ldc=%d alpha=%g beta=%g\n", *ta, *tb, *m, *n, *k,
         *lda, *ldb, *ldc, *alpha, *beta); (void)A; (void)B; (void)C; }

void dtrsm_(const char *s, const char *u, const char *t, const char *d, const int *m, const int *n,
            const double *alpha, const double *A, const int *lda, double *B, const int *ldb)
{ printf("dtrsm_ %c %c %c %c m=%d n=%d lda=%d ldb=%d\n", *s, *u, *t, *d, *m, *n, *lda, *ldb);
  (void)alpha; (void)A; (void)B; }

void dsyrk_(const char *u, const char *t, const int *n, const int *k, const double *alpha,
            const double *A, const int *lda, const double *beta, double *C, const int *ldc)
{ printf("dsyrk_ %c %c n=%d k=%d lda=%d ldc=%d\n", *u, *t, *n, *k, *lda, *ldc);
  (void)alpha; (void)A; (void)beta; (void)C; }

void dsyr2k_(const char *u, const char *t, const int *n, const int *k, const double *alpha,
             const double *A, const int *lda, const double *B, const int *ldb, const double *beta,
             double *C, const int *ldc)
{ printf("dsyr2k_ %c %c n=%d k=%d lda=%d ldb=%d ldc=%d\n", *u, *t, *n, *k, *lda, *ldb, *ldc);
  (void)alpha; (void)A; (void)B; (void)beta; (void)C; }

void dtrmm_(const char *s, const char *u, const char *t, const char *d, const int *m, const int *n,
            const double *alpha, const double *A, const int *lda, double *B, const int *ldb)
{ printf("dtrmm_ %c %c %c %c m=%d n=%d lda=%d ldb=%d\n", *s, *u, *t, *d, *m, *n, *lda, *ldb);
  (void)alpha; (void)A; (void)B; }

void dsymm_(const char *s, const char *u, const int *m, const int *n, const double *alpha,
            const double *A, const int *lda, const double *B, const int *ldb, const double *beta,
            double *C, const int *ldc)
{ printf("dsymm_ %c %c m=%d n=%d lda=%d ldb=%d ldc=%d\n", *s, *u, *m, *n, *lda, *ldb, *ldc);
  (void)alpha; (void)A; (void)B; (void)beta; (void)C; }

void dgetrf_(const int *m, const int *n, double *A, const int *lda, int *ipiv, int *info)
{ printf("dgetrf_ m=%d n=%d lda=%d\n", *m, *n, *lda); (void)A; (void)ipiv; ok(info); }

void dgetrs_(const char *t, const int *n, const int *nrhs, const double *A, const int *lda,
             const int *ipiv, double *B, const int *ldb, int *info)
{ printf("dgetrs_ %c n=%d nrhs=%d lda=%d ldb=%d\n", *t, *n, *nrhs, *lda, *ldb); (void)A; (void)ipiv;
  (void)B; ok(info); }

void dpotrf_(const char *u, const int *n, double *A, const int *lda, int *info)
{ printf("dpotrf_ %c n=%d lda=%d\n", *u, *n, *lda); (void)A; ok(info); }

void dpotrs_(const char *u, const int *n, const int *nrhs, const double *A, const int *lda,
             double *B, const int *ldb, int *info)
{ printf("dpotrs_ %c n=%d nrhs=%d lda=%d ldb=%d\n", *u, *n, *nrhs, *lda, *ldb); (void)A; (void)B;
  ok(info); }

void dgetri_(const int *n, double *A, const int *lda, const int *ipiv, double *work, const int *lwork,
             int *info)
{ printf("dgetri_ n=%d lda=%d lwork=%d\n", *n, *lda, *lwork); (void)A; (void)ipiv; (void)work;
  ok(info); }

void dtrtri_(const char *u, const char *d, const int *n, double *A, const int *lda, int *info)
{ printf("dtrtri_ %c %c n=%d lda=%d\n", *u, *d, *n, *lda); (void)A; ok(info); }

void dgerfs_(const char *t, const int *n, const int *nrhs, const double *A, const int *lda,
             const double *AF, const int *ldaf, const int *ipiv, const double *B, const int *ldb,
             double *X, const int *ldx, double *ferr, double *berr, double *work, int *iwork, int *info)
{ printf("dgerfs_ %c n=%d nrhs=%d lda=%d ldaf=%d ldb=%d ldx=%d\n", *t, *n, *nrhs, *lda, *ldaf, *ldb, *ldx);
  (void)A; (void)AF; (void)ipiv; (void)B; (void)X; (void)ferr; (void)berr; (void)work; (void)iwork;
  ok(info); }

void dgecon_(const char *norm, const int *n, const double *A, const int *lda, const double *anorm,
             double *rcond, double *work, int *iwork, int *info)
{ printf("dgecon_ %c n=%d lda=%d anorm=%g\n", *norm, *n, *lda, *anorm); (void)A; *rcond = 0.5;
  (void)work; (void)iwork; ok(info); }

void dgeequ_(const int *m, const int *n, const double *A, const int *lda, double *r, double *c,
             double *rowcnd, double *colcnd, double *amax, int *info)
{ printf("dgeequ_ m=%d n=%d lda=%d\n", *m, *n, *lda); (void)A; (void)r; (void)c; *rowcnd = 1;
  *colcnd = 1; *amax = 1; ok(info); }

void dlaqge_(const int *m, const int *n, double *A, const int *lda, const double *r, const double *c,
             const double *rowcnd, const double *colcnd, const double *amax, char *equed)
{ printf("dlaqge_ m=%d n=%d lda=%d\n", *m, *n, *lda); (void)A; (void)r; (void)c; (void)rowcnd;
  (void)colcnd; (void)amax; *equed = 'N'; }

void dgesvx_(const char *fact, const char *t, const int *n, const int *nrhs, double *A, const int *lda,
             double *AF, const int *ldaf, int *ipiv, char *equed, double *r, double *c, double *B,
             const int *ldb, double *X, const int *ldx, double *rcond, double *ferr, double *berr,
             double *work, int *iwork, int *info)
{ printf("dgesvx_ %c %c equed=%c n=%d nrhs=%d lda=%d ldaf=%d ldb=%d ldx=%d\n", *fact, *t, *equed, *n,
         *nrhs, *lda, *ldaf, *ldb, *ldx);
  (void)A; (void)AF; (void)ipiv; (void)r; (void)c; (void)B; (void)X; *rcond = 0.5; (void)ferr;
  (void)berr; work[0] = 1.0; (void)iwork; ok(info); }
