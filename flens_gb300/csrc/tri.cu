// tri.cu -- triangular inverse (dtrtri) and inverse from the LU factors
// (dgetri), FP64, column-major, on the GEMM / TRSM / TRMM engine.
//
// Follows FLENS-LAPACK:
//   trtri  flens/lapack/tr/tri.tcc (generic tri_impl): a non-unit matrix with
//          an exactly zero diagonal element returns its 1-based index and is
//          left untouched; block size 64 (ilaenv TRTRI), here inside outer
//          blocks of 512 so that the trmm / trsm calls are wide; upper: for each
//          block column j (forward) U12 <- U11^-1 U12 (trmm with the already
//          inverted U11), U12 <- -U12 U22^-1 (trsm), then the diagonal block
//          is inverted (ti2, flens/lapack/tr/ti2.tcc); lower runs backward.
//   getri  flens/lapack/ge/tri.tcc (generic tri_impl): inv(U) by trtri, then
//          for each block column J from the last (512 columns here, 64 in
//          the reference; the same operations in exact arithmetic): the strictly lower part of
//          A(:,J) (the L factor) is moved to a workspace and zeroed,
//          A(:,J) -= A(:, after J) * Work(after J, :) (gemm),
//          A(:,J) <- A(:,J) * Wunit(J)^-1 (trsm with the unit lower block),
//          and finally the column interchanges j = n-1..1 with piv(j).
// Results agree with the reference to rounding (different summation order).
#include "common.cuh"

namespace fg {

namespace {

constexpr int TRI_NB = 64;       // diagonal blocks of the inner loop (trti2 size)
constexpr int TRI_OUTER = 512;   // outer block: the trmm / gemm / trsm calls get n >= 512 columns

// In-place inverse of the jb x jb (jb <= 64) triangular block at A (ti2):
// upper: for j = 0.., A(j,j) <- 1/A(j,j) (non-unit), u = A(0:j, j) <-
// -A(j,j) * U11inv * u; lower: for j = jb-1.., l = A(j+1:, j) <-
// -A(j,j) * L22inv * l.  One CTA, the block in shared memory.
__global__ void __launch_bounds__(256)
trti2_kernel(int jb, double *__restrict__ A, int ldA, int upper, int unit) {
    __shared__ double S[TRI_NB][TRI_NB + 1];
    __shared__ double t[TRI_NB];
    __shared__ double s_ajj;
    const int tid = threadIdx.x;
    for (int e = tid; e < jb * jb; e += blockDim.x) {
        const int i = e % jb, c = e / jb;
        if (upper ? i <= c : i >= c) S[i][c] = A[(size_t)i + (size_t)c * ldA];
    }
    __syncthreads();
    for (int s = 0; s < jb; ++s) {
        const int j = upper ? s : jb - 1 - s;
        if (tid == 0) {
            if (!unit) {
                S[j][j] = 1.0 / S[j][j];
                s_ajj = -S[j][j];
            } else {
                s_ajj = -1.0;
            }
        }
        __syncthreads();
        // t(i) = sum over the finished triangle row i of T(i,p) u(p), T with
        // a unit diagonal when unit (u = column j off the diagonal)
        if (upper) {
            if (tid < j) {
                double acc = 0.0;
                for (int p = tid; p < j; ++p) acc = fma(p == tid && unit ? 1.0 : S[tid][p], S[p][j], acc);
                t[tid] = acc;
            }
        } else {
            if (tid > j && tid < jb) {
                double acc = 0.0;
                for (int p = j + 1; p <= tid; ++p) acc = fma(p == tid && unit ? 1.0 : S[tid][p], S[p][j], acc);
                t[tid] = acc;
            }
        }
        __syncthreads();
        if (upper ? tid < j : (tid > j && tid < jb)) S[tid][j] = t[tid] * s_ajj;
        __syncthreads();
    }
    for (int e = tid; e < jb * jb; e += blockDim.x) {
        const int i = e % jb, c = e / jb;
        if (upper ? i <= c : i >= c) {
            if (!(unit && i == c)) A[(size_t)i + (size_t)c * ldA] = S[i][c];
        }
    }
}

// *info = 1-based index of the first exactly zero diagonal element, or 0.
__global__ void zero_diag_kernel(int n, const double *__restrict__ A, int ldA, int *info) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (A[(size_t)i * (ldA + 1)] == 0.0) atomicMin(info, i + 1);
}

__global__ void set_int_kernel(int *p, int v) { *p = v; }

// Work(i, c) = A(i, j0 + c) and A(i, j0 + c) = 0 for j0 + c < i < n
__global__ void __launch_bounds__(256)
take_lower_kernel(int n, int j0, int jb, double *__restrict__ A, int ldA, double *__restrict__ W,
                  int ldW) {
    const size_t total = (size_t)n * jb;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % n), c = (int)(e / n);
        double *a = &A[(size_t)i + (size_t)(j0 + c) * ldA];
        if (i > j0 + c) {
            W[(size_t)i + (size_t)c * ldW] = *a;
            *a = 0.0;
        } else {
            W[(size_t)i + (size_t)c * ldW] = 0.0;
        }
    }
}

// Column interchanges j = n-2..0 with piv(j) (1-based), one thread per row:
// every thread walks the whole sequence for its row, so the swaps compose in
// the reference's order and reads stay coalesced along the column.
__global__ void __launch_bounds__(256)
column_swaps_kernel(int n, double *__restrict__ A, int ldA, const int *__restrict__ piv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int j = n - 2; j >= 0; --j) {
        const int jp = piv[j] - 1;
        if (jp != j) {
            double *a = &A[(size_t)i + (size_t)j * ldA], *b = &A[(size_t)i + (size_t)jp * ldA];
            const double t = *a;
            *a = *b;
            *b = t;
        }
    }
}

int grid_for(size_t total) {
    const size_t g = (total + 255) / 256;
    const size_t cap = (size_t)num_sms() * 16;
    return (int)(g < cap ? (g > 0 ? g : 1) : cap);
}

int trti2(int jb, double *A, int ldA, bool upper, bool unit, cudaStream_t s) {
    KTimer kt(kFamPanel, s, (double)jb * jb * jb / 3.0, 16.0 * jb * jb);
    trti2_kernel<<<1, 256, 0, s>>>(jb, A, ldA, upper ? 1 : 0, unit ? 1 : 0);
    FG_CUDA(cudaGetLastError());
    return kOk;
}

int *pinned_int() {
    thread_local int *h = nullptr;
    if (!h && cudaMallocHost((void **)&h, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        h = nullptr;
    }
    return h;
}

}  // namespace

namespace {

// The blocked inverse of the k x k triangle at A in place (no zero check):
// block columns of `nb` (forward for upper, backward for lower), each
// U12 <- U11^-1 U12 (trmm with the part already inverted), U12 <- -U12 U22^-1
// (trsm), then the diagonal block -- by trti2 when nb is the inner size,
// else recursively with the inner size.
int trtri_blocked(bool upper, bool unit, int k, double *A, int ldA, int nb, cudaStream_t s) {
    const char dg = unit ? 'U' : 'N';
    int st;
    auto diag_block = [&](int jb, double *D) -> int {
        return nb == TRI_NB ? trti2(jb, D, ldA, upper, unit, s) : trtri_blocked(upper, unit, jb, D, ldA, TRI_NB, s);
    };
    if (k <= nb) return diag_block(k, A);
    if (upper) {
        for (int j = 0; j < k; j += nb) {
            const int jb = k - j < nb ? k - j : nb;
            double *A12 = A + (size_t)j * ldA, *A22 = A + j + (size_t)j * ldA;
            if (j > 0) {
                if ((st = dtrmm_launch('L', 'U', 'N', dg, j, jb, 1.0, A, ldA, A12, ldA, s)) != kOk) return st;
                if ((st = dtrsm_launch('R', 'U', 'N', dg, j, jb, -1.0, A22, ldA, A12, ldA, s)) != kOk) return st;
            }
            if ((st = diag_block(jb, A22)) != kOk) return st;
        }
    } else {
        const int nn = ((k - 1) / nb) * nb;
        for (int j = nn; j >= 0; j -= nb) {
            const int jb = k - j < nb ? k - j : nb;
            double *A11 = A + j + (size_t)j * ldA;
            if (j + jb < k) {
                const int r = k - j - jb;
                double *A21 = A + (j + jb) + (size_t)j * ldA;
                double *A22 = A + (j + jb) + (size_t)(j + jb) * ldA;
                if ((st = dtrmm_launch('L', 'L', 'N', dg, r, jb, 1.0, A22, ldA, A21, ldA, s)) != kOk) return st;
                if ((st = dtrsm_launch('R', 'L', 'N', dg, r, jb, -1.0, A11, ldA, A21, ldA, s)) != kOk) return st;
            }
            if ((st = diag_block(jb, A11)) != kOk) return st;
        }
    }
    return kOk;
}

}  // namespace

int dtrtri_launch(char uplo, char diag, int n, double *A, int ldA, int *info, cudaStream_t s) {
    const bool upper = uplo == 'U' || uplo == 'u';
    const bool unit = diag == 'U' || diag == 'u';
    set_int_kernel<<<1, 1, 0, s>>>(info, unit ? 0 : 0x7fffffff);
    FG_CUDA(cudaGetLastError());
    if (n == 0) return kOk;
    if (!unit) {
        zero_diag_kernel<<<grid_for((size_t)n), 256, 0, s>>>(n, A, ldA, info);
        FG_CUDA(cudaGetLastError());
        int *h = pinned_int();
        if (!h) {
            set_last_error("cudaMallocHost of the INFO readback failed");
            return kErrAlloc;
        }
        FG_CUDA(cudaMemcpyAsync(h, info, sizeof(int), cudaMemcpyDeviceToHost, s));
        FG_CUDA(cudaStreamSynchronize(s));
        if (*h != 0x7fffffff) return kOk;           // A untouched, *info = zero pivot
        set_int_kernel<<<1, 1, 0, s>>>(info, 0);
        FG_CUDA(cudaGetLastError());
    }
    // outer blocks of 512 (wide trmm/trsm calls), 64-column blocks inside
    const int st = trtri_blocked(upper, unit, n, A, ldA, n > TRI_OUTER ? TRI_OUTER : TRI_NB, s);
    if (st != kOk) return st;
    trace("trtri %c%c n=%d", uplo, diag, n);
    return kOk;
}

int dgetri_launch(int n, double *A, int ldA, const int *ipiv, int *info, cudaStream_t s) {
    int st = dtrtri_launch('U', 'N', n, A, ldA, info, s);
    if (st != kOk || n == 0) return st;
    int *h = pinned_int();
    if (!h) return kErrAlloc;
    FG_CUDA(cudaMemcpyAsync(h, info, sizeof(int), cudaMemcpyDeviceToHost, s));
    FG_CUDA(cudaStreamSynchronize(s));
    if (*h != 0) return kOk;                        // singular U: A holds the factors
    // block columns of 512: the gemm and trsm calls then have 512 columns
    // (the reference's 64-column blocks give 64-column calls with long k)
    const int nbg = n > TRI_OUTER ? TRI_OUTER : TRI_NB;
    const int jbmax = n < nbg ? n : nbg;
    double *W = (double *)workspace_slot(s, 1, (size_t)n * jbmax * sizeof(double));
    if (!W) return kErrAlloc;
    const int nn = ((n - 1) / nbg) * nbg;
    for (int j = nn; j >= 0; j -= nbg) {
        const int jb = n - j < nbg ? n - j : nbg;
        {
            KTimer kt(kFamAux, s, 0.0, 24.0 * n * (double)jb);
            take_lower_kernel<<<grid_for((size_t)n * jb), 256, 0, s>>>(n, j, jb, A, ldA, W, n);
            FG_CUDA(cudaGetLastError());
        }
        double *AJ = A + (size_t)j * ldA;
        if (j + jb < n) {
            if ((st = dgemm_launch('N', 'N', n, jb, n - j - jb, -1.0, A + (size_t)(j + jb) * ldA, ldA,
                                   W + (j + jb), n, 1.0, AJ, ldA, s)) != kOk) return st;
        }
        if ((st = dtrsm_launch('R', 'L', 'N', 'U', n, jb, 1.0, W + j, n, AJ, ldA, s)) != kOk) return st;
    }
    KTimer kt(kFamLaswp, s, 0.0, 32.0 * n * (double)n);
    column_swaps_kernel<<<ceil_div(n, 256), 256, 0, s>>>(n, A, ldA, ipiv);
    FG_CUDA(cudaGetLastError());
    trace("getri n=%d", n);
    return kOk;
}

}  // namespace fg
