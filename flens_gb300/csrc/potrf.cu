// potrf.cu -- Cholesky factorisation and solve, FP64, column-major.
//
//   dpotrf: A = L L^T (uplo 'L') or U^T U ('U') in place, the other triangle
//           untouched; INFO = first column whose pivot is <= 0 or NaN.
//   dpotrs: A X = B from the factor (two triangular solves).
//
// Follows FLENS-LAPACK potrf (flens/lapack/po/potrf.tcc:56-150, block size 64
// from ilaenv PO/TRF, flens/lapack/la/ilaenv.tcc:126-132), potf2
// (flens/lapack/po/potf2.tcc:56-140: pivot test `ajj <= 0 || isnan(ajj)`,
// the failing pivot stored in A(j,j), column scaled by the reciprocal 1/ajj)
// and potrs (flens/lapack/po/potrs.tcc:54-100).  The reference updates
// left-looking (syrk of the diagonal block, gemm of the block column, then
// trsm); on the GPU the block steps are right-looking so that each step's
// trailing update is one large syrk over the whole remaining triangle:
//
//   for each 64-column block j:  potf2 of A(j,j) in one CTA (shared memory),
//                                A(j+,j) <- A(j+,j) L(j,j)^-T      (trsm),
//                                A(j+,j+) -= A(j+,j) A(j+,j)^T     (syrk, lower
//                                tiles only).
//
// Pivots, INFO and the factor agree with the reference to rounding; when
// INFO > 0 the columns after the failing block hold partially updated values
// (the reference leaves them as they were), as LAPACK leaves them undefined.
#include "common.cuh"

#include <cmath>

namespace fg {

namespace {

constexpr int POTRF_NB = 64;

// Unblocked right-looking Cholesky of the jb x jb (jb <= 64) diagonal block
// at A, whose lower-view element (i, c), i >= c, is A[i*rs + c*cs] (rs = 1,
// cs = ld for 'L'; rs = ld, cs = 1 for 'U').  On a pivot <= 0 or NaN in
// column f it stores that pivot, writes back columns < f only and sets
// *info = j0 + f + 1.
__global__ void __launch_bounds__(256)
potf2_kernel(int jb, double *__restrict__ A, size_t rs, size_t cs, int j0, int *__restrict__ info) {
    __shared__ double S[POTRF_NB][POTRF_NB + 1];
    __shared__ int s_fail;
    __shared__ double s_r;
    const int tid = threadIdx.x;
    for (int e = tid; e < jb * jb; e += blockDim.x) {
        const int i = e % jb, c = e / jb;
        if (i >= c) S[i][c] = A[(size_t)i * rs + (size_t)c * cs];
    }
    if (tid == 0) s_fail = 0;
    __syncthreads();
    int fail = 0;
    // thread (row, quarter) updates row `row`, columns c = quarter mod 4:
    // no index divisions, and the FP64 reciprocal is taken once per column
    // (the pipe issues 2 FP64 instructions per clock per SM)
    const int row = tid & (POTRF_NB - 1), quarter = tid / POTRF_NB;
    for (int j = 0; j < jb; ++j) {
        if (tid == 0) {
            const double a = S[j][j];
            if (a <= 0.0 || isnan(a)) {
                s_fail = j + 1;
            } else {
                const double d = sqrt(a);
                S[j][j] = d;
                s_r = 1.0 / d;
            }
        }
        __syncthreads();
        fail = s_fail;
        if (fail) break;
        const double r = s_r;
        for (int i = j + 1 + tid; i < jb; i += blockDim.x) S[i][j] *= r;
        __syncthreads();
        if (row > j && row < jb) {
            const double lij = S[row][j];
            for (int c = j + 1 + quarter; c <= row; c += 4) S[row][c] = fma(-lij, S[c][j], S[row][c]);
        }
        __syncthreads();
    }
    const int ncol = fail ? fail - 1 : jb;
    for (int e = tid; e < jb * jb; e += blockDim.x) {
        const int i = e % jb, c = e / jb;
        if (i >= c && c < ncol) A[(size_t)i * rs + (size_t)c * cs] = S[i][c];
    }
    if (fail && tid == 0) {
        const int f = fail - 1;
        A[(size_t)f * (rs + cs)] = S[f][f];
        *info = j0 + fail;
    }
}

int *pinned_info() {
    thread_local int *h = nullptr;
    if (!h && cudaMallocHost((void **)&h, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        h = nullptr;
    }
    return h;
}

}  // namespace

int dpotrf_launch(char uplo, int n, double *A, int ldA, int *info, cudaStream_t s) {
    FG_CUDA(cudaMemsetAsync(info, 0, sizeof(int), s));
    if (n == 0) return kOk;
    const bool lower = uplo == 'L' || uplo == 'l';
    const size_t rs = lower ? 1 : (size_t)ldA, cs = lower ? (size_t)ldA : 1;
    int *h = pinned_info();
    if (!h) {
        set_last_error("cudaMallocHost of the INFO readback failed");
        return kErrAlloc;
    }
    int st;
    for (int j = 0; j < n; j += POTRF_NB) {
        const int jb = n - j < POTRF_NB ? n - j : POTRF_NB;
        double *A22 = A + j + (size_t)j * ldA;
        {
            KTimer kt(kFamPanel, s, (double)jb * jb * jb / 3.0, 16.0 * jb * jb);
            potf2_kernel<<<1, 256, 0, s>>>(jb, A22, rs, cs, j, info);
            FG_CUDA(cudaGetLastError());
        }
        const int m2 = n - j - jb;
        if (m2 == 0) break;
        // stop at the first failing pivot, as potrf.tcc:104-107 does
        FG_CUDA(cudaMemcpyAsync(h, info, sizeof(int), cudaMemcpyDeviceToHost, s));
        FG_CUDA(cudaStreamSynchronize(s));
        if (*h != 0) break;
        double *A33 = A + (j + jb) + (size_t)(j + jb) * ldA;
        if (lower) {
            double *A32 = A + (j + jb) + (size_t)j * ldA;
            if ((st = dtrsm_launch('R', 'L', 'T', 'N', m2, jb, 1.0, A22, ldA, A32, ldA, s)) != kOk) return st;
            if ((st = dsyrk_launch('L', 'N', m2, jb, -1.0, A32, ldA, 1.0, A33, ldA, s)) != kOk) return st;
        } else {
            double *A23 = A + j + (size_t)(j + jb) * ldA;
            if ((st = dtrsm_launch('L', 'U', 'T', 'N', jb, m2, 1.0, A22, ldA, A23, ldA, s)) != kOk) return st;
            if ((st = dsyrk_launch('U', 'T', m2, jb, -1.0, A23, ldA, 1.0, A33, ldA, s)) != kOk) return st;
        }
    }
    trace("potrf %c n=%d", uplo, n);
    return kOk;
}

// flens/lapack/po/potrs.tcc:54-100: L X = B then L^T X = B (lower), or
// U^T X = B then U X = B (upper).
int dpotrs_launch(char uplo, int n, int nrhs, const double *A, int ldA, double *B, int ldB,
                  cudaStream_t s) {
    if (n == 0 || nrhs == 0) return kOk;
    const bool lower = uplo == 'L' || uplo == 'l';
    int st;
    if (lower) {
        if ((st = dtrsm_launch('L', 'L', 'N', 'N', n, nrhs, 1.0, A, ldA, B, ldB, s)) != kOk) return st;
        return dtrsm_launch('L', 'L', 'T', 'N', n, nrhs, 1.0, A, ldA, B, ldB, s);
    }
    if ((st = dtrsm_launch('L', 'U', 'T', 'N', n, nrhs, 1.0, A, ldA, B, ldB, s)) != kOk) return st;
    return dtrsm_launch('L', 'U', 'N', 'N', n, nrhs, 1.0, A, ldA, B, ldB, s);
}

}  // namespace fg
