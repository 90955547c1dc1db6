// blas3.cu -- the remaining level-3 BLAS for double on the FP64 GEMM engine.
//
//   dtrmm  B <- alpha*op(A)*B (side 'L') or alpha*B*op(A) ('R'), A triangular
//          (cxxblas/level3/trmm.tcc:40-70: trmv per vector, alpha applied at
//          the end);
//   dsymm  C <- beta*C + alpha*A*B ('L') or alpha*B*A ('R'), A symmetric with
//          one triangle stored (cxxblas/level3/symm.tcc:40-70);
//   dsyr2k C <- beta*C + alpha*(op(A)*op(B)^T + op(B)*op(A)^T) on one
//          triangle (cxxblas/level3/syr2k.tcc:42-95).
//
// The triangular or symmetric operand is first written out as a full ka x ka
// matrix in the workspace (zeros outside the triangle, ones on a unit
// diagonal; or both triangles from the stored one), so the product runs on
// the tiled FP64 GEMM.  trmm computes T*B (or B*T) into a workspace buffer and
// writes alpha*result back over B.  syr2k is two triangle-restricted GEMMs
// (tri_gemm_launch).  Results agree with the reference to rounding.
#include "common.cuh"

namespace fg {

namespace {

// mode 0: triangle (lower or upper) with zeros elsewhere, unit diagonal -> 1;
// mode 1: symmetric matrix from the stored (lower or upper) triangle.
__global__ void __launch_bounds__(256)
expand_kernel(int ka, const double *__restrict__ A, int ldA, double *__restrict__ T, int mode,
              int lower, int unit) {
    const size_t total = (size_t)ka * ka;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % ka), j = (int)(e / ka);
        double v;
        if (mode == 0) {
            const bool in = lower ? i >= j : i <= j;
            v = !in ? 0.0 : (unit && i == j) ? 1.0 : A[(size_t)i + (size_t)j * ldA];
        } else {
            const bool in = lower ? i >= j : i <= j;
            v = in ? A[(size_t)i + (size_t)j * ldA] : A[(size_t)j + (size_t)i * ldA];
        }
        T[e] = v;
    }
}

// B(i,j) = alpha * W(i,j), W with leading dimension m
__global__ void __launch_bounds__(256)
scale_copy_kernel(int m, int n, double alpha, const double *__restrict__ W, double *__restrict__ B,
                  int ldB) {
    const size_t total = (size_t)m * n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const size_t i = e % m, j = e / m;
        B[i + j * ldB] = alpha * W[e];
    }
}

int grid_for(size_t total) {
    const size_t g = (total + 255) / 256;
    const size_t cap = (size_t)num_sms() * 16;
    return (int)(g < cap ? (g > 0 ? g : 1) : cap);
}

}  // namespace

int dtrmm_launch(char side, char uplo, char transA, char diag, int m, int n, double alpha,
                 const double *A, int ldA, double *B, int ldB, cudaStream_t s) {
    if (m == 0 || n == 0) return kOk;
    const bool left = side == 'L' || side == 'l';
    const int ka = left ? m : n;
    double *T = (double *)workspace_slot(s, 2, (size_t)ka * ka * sizeof(double));
    double *W = (double *)workspace_slot(s, 3, (size_t)m * n * sizeof(double));
    if (!T || !W) return kErrAlloc;
    {
        KTimer kt(kFamAux, s, 0.0, 16.0 * ka * (double)ka);
        expand_kernel<<<grid_for((size_t)ka * ka), 256, 0, s>>>(ka, A, ldA, T, 0,
                                                               uplo == 'L' || uplo == 'l',
                                                               diag == 'U' || diag == 'u');
        FG_CUDA(cudaGetLastError());
    }
    FG_CUDA(cudaMemsetAsync(W, 0, (size_t)m * n * sizeof(double), s));
    const char ta = (transA == 'N' || transA == 'n') ? 'N' : 'T';
    // op(T) is upper when T is upper and not transposed, or lower and transposed
    const bool op_upper = (uplo == 'U' || uplo == 'u') == (ta == 'N');
    int st = left ? dgemm_kr_launch(ta, 'N', m, n, m, 1.0, T, ka, B, ldB, 0.0, W, m, op_upper ? 1 : 2, s)
                  : dgemm_kr_launch('N', ta, m, n, n, 1.0, B, ldB, T, ka, 0.0, W, m, op_upper ? 3 : 4, s);
    if (st != kOk) return st;
    KTimer kt(kFamAux, s, (double)m * n, 16.0 * m * (double)n);
    scale_copy_kernel<<<grid_for((size_t)m * n), 256, 0, s>>>(m, n, alpha, W, B, ldB);
    FG_CUDA(cudaGetLastError());
    trace("trmm %c%c%c%c m=%d n=%d", side, uplo, transA, diag, m, n);
    return kOk;
}

int dsymm_launch(char side, char uplo, int m, int n, double alpha, const double *A, int ldA,
                 const double *B, int ldB, double beta, double *C, int ldC, cudaStream_t s) {
    if (m == 0 || n == 0) return kOk;
    const bool left = side == 'L' || side == 'l';
    const int ka = left ? m : n;
    double *S = (double *)workspace_slot(s, 2, (size_t)ka * ka * sizeof(double));
    if (!S) return kErrAlloc;
    {
        KTimer kt(kFamAux, s, 0.0, 16.0 * ka * (double)ka);
        expand_kernel<<<grid_for((size_t)ka * ka), 256, 0, s>>>(ka, A, ldA, S, 1,
                                                               uplo == 'L' || uplo == 'l', 0);
        FG_CUDA(cudaGetLastError());
    }
    trace("symm %c%c m=%d n=%d", side, uplo, m, n);
    return left ? dgemm_launch('N', 'N', m, n, m, alpha, S, ka, B, ldB, beta, C, ldC, s)
                : dgemm_launch('N', 'N', m, n, n, alpha, B, ldB, S, ka, beta, C, ldC, s);
}

int dsyr2k_launch(char uplo, char trans, int n, int k, double alpha, const double *A, int ldA,
                  const double *B, int ldB, double beta, double *C, int ldC, cudaStream_t s) {
    trace("syr2k %c%c n=%d k=%d", uplo, trans, n, k);
    int st = tri_gemm_launch(uplo, trans, n, k, alpha, A, ldA, B, ldB, beta, C, ldC, s);
    if (st != kOk || k == 0 || n == 0) return st;
    return tri_gemm_launch(uplo, trans, n, k, alpha, B, ldB, A, ldA, 1.0, C, ldC, s);
}

}  // namespace fg
