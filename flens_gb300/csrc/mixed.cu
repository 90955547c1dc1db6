// mixed.cu -- the precision form of the solve: low-precision LU on the tensor
// cores, FP64 iterative refinement (classical, or GMRES-IR) to FP64 accuracy.
//
//   1. A32 = fp32(A); LU of A32 with partial pivoting (sgetrf_launch): the
//      panel's pivot search and scaling run in FP64 on FP32 storage, the
//      trailing updates A22 -= A21*U12 on the tensor cores in TF32, BF16,
//      FP8 e4m3 (per-row/column scaled) or FP32-accurate 3xTF32.
//   2. x0 = U^-1 L^-1 P b in FP32 (b scaled per column into FP32 range).
//   3. Refinement; everything that decides accuracy is FP64:
//        r = b - A x (FP64 GEMM/GEMV on the original A),
//        berr_j = ||r_j||_inf / (||A||_inf ||x_j||_inf + ||b_j||_inf),
//      classical: d = (LU)^-1 r (FP32 solve of the scaled residual), x += d;
//      GMRES-IR:  d from left-preconditioned GMRES on (LU)^-1 A d = (LU)^-1 r
//                 (Carson & Higham, SIAM J. Sci. Comput. 40(2), 2018): FP64
//                 Arnoldi, classical Gram-Schmidt applied twice, the
//                 preconditioner applied as FP64 triangular solves with the
//                 (FP32) factors, Givens rotations on the host; x += d.
//      Classical refinement stops like the reference's rfs
//      (flens/lapack/ge/rfs.tcc:182-188): on reaching the tolerance, when the
//      backward error stops halving, or after max_iter steps.  In the auto
//      mode a stall above the tolerance switches the column to GMRES-IR.
// The row interchanges of the LU are turned into one permutation after the
// factorisation and applied inside the FP64 -> FP32 conversion of each solve.
//
// Precision 4 (split) keeps FP64 storage and makes the LU itself FP64-accurate
// on the tensor cores: dgetrf_split_launch runs the trailing updates beyond
// each outer block through the split GEMM (exact BF16 products of
// exponent-aligned slices).  Its solves are FP64 triangular solves, so the
// refinement converges in one or two steps at any kappa*u64 < 1.
#include "common.cuh"

#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <vector>

namespace fg {

int laswp_perm_launch(int nrows, const int *ipiv, int *perm, cudaStream_t stream);

namespace {

// Y(:, j) = fp32(X(perm, j) / s_j)  (perm and colscale may be null)
__global__ void d2s_cols_kernel(int n, int ncols, const double *__restrict__ X, int ldx,
                                const int *__restrict__ perm, const double *__restrict__ colscale,
                                float *__restrict__ Y, int ldy) {
    const size_t total = (size_t)n * ncols;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const size_t j = e / n, i = e % n;
        const size_t src = perm ? (size_t)perm[i] : i;
        double v = X[src + j * ldx];
        if (colscale) {
            const double s = colscale[j];
            v = (s > 0.0 && isfinite(s)) ? v / s : 0.0;
        }
        Y[i + j * ldy] = (float)v;
    }
}

// X(:, j) (+)= s_j * fp64(D(:, j))
template <bool ADD>
__global__ void s2d_cols_kernel(int n, int ncols, const float *__restrict__ D, int ldd,
                                const double *__restrict__ colscale, double *__restrict__ X, int ldx) {
    const size_t total = (size_t)n * ncols;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const size_t j = e / n, i = e % n;
        const double s = colscale ? colscale[j] : 1.0;
        const double v = s * (double)D[i + j * ldd];
        if (ADD) X[i + j * ldx] += v;
        else X[i + j * ldx] = v;
    }
}

// D(:, j) = X(perm, j)
__global__ void gather_cols_kernel(int n, int ncols, const double *__restrict__ X, int ldx,
                                   const int *__restrict__ perm, double *__restrict__ D, int ldd) {
    const size_t total = (size_t)n * ncols;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const size_t j = e / n, i = e % n;
        D[i + j * ldd] = X[(size_t)perm[i] + j * ldx];
    }
}

// X(:, j) (+)= D(:, j)
template <bool ADD>
__global__ void put_cols_kernel(int n, int ncols, const double *__restrict__ D, int ldd,
                                double *__restrict__ X, int ldx) {
    const size_t total = (size_t)n * ncols;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const size_t j = e / n, i = e % n;
        if (ADD) X[i + j * ldx] += D[i + j * ldd];
        else X[i + j * ldx] = D[i + j * ldd];
    }
}

__global__ void copy_cols_kernel(int n, int ncols, const double *__restrict__ S, int lds,
                                 double *__restrict__ D, int ldd) {
    const size_t total = (size_t)n * ncols;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const size_t j = e / n, i = e % n;
        D[i + j * ldd] = S[i + j * lds];
    }
}

// out[j] = max_i |X(i, j)| (NaN wins), one CTA per column
__global__ void __launch_bounds__(256)
col_absmax_kernel(int n, const double *__restrict__ X, int ldx, double *__restrict__ out) {
    __shared__ double red[8];
    const int j = blockIdx.x;
    double m = 0.0;
    for (int i = threadIdx.x; i < n; i += 256) {
        const double a = fabs(X[i + (size_t)j * ldx]);
        m = (a > m || isnan(a)) ? a : m;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const double o = __shfl_xor_sync(0xffffffffu, m, off);
        m = (o > m || isnan(o)) ? o : m;
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = red[0];
        for (int w = 1; w < 8; ++w) r = (red[w] > r || isnan(red[w])) ? red[w] : r;
        out[j] = r;
    }
}

// ||A||_inf = max_i sum_j |A(i, j)|; non-negative doubles order like their bits
__global__ void __launch_bounds__(256)
inf_norm_kernel(int n, const double *__restrict__ A, int lda, unsigned long long *__restrict__ out) {
    const int i = blockIdx.x * 256 + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int j = 0; j < n; ++j) s += fabs(A[(size_t)i + (size_t)j * lda]);
    atomicMax(out, (unsigned long long)__double_as_longlong(s));
}

// h[c] += sum_r V(r, c) w(r), c < k (h zeroed by the caller); grid (chunks, k)
__global__ void __launch_bounds__(256)
multi_dot_kernel(int n, const double *__restrict__ V, int ldv, const double *__restrict__ w,
                 double *__restrict__ h) {
    __shared__ double red[8];
    const int c = blockIdx.y;
    double s = 0.0;
    for (int r = blockIdx.x * 256 + threadIdx.x; r < n; r += gridDim.x * 256)
        s = fma(V[(size_t)r + (size_t)c * ldv], w[r], s);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < 8; ++q) t += red[q];
        atomicAdd(&h[c], t);
    }
}

// w += sign * V(:, 0:k) * h
__global__ void __launch_bounds__(256)
combination_kernel(int n, int k, const double *__restrict__ V, int ldv, const double *__restrict__ h,
                   double sign, double *__restrict__ w) {
    for (int r = blockIdx.x * 256 + threadIdx.x; r < n; r += gridDim.x * 256) {
        double s = w[r];
        for (int c = 0; c < k; ++c) s = fma(sign * V[(size_t)r + (size_t)c * ldv], h[c], s);
        w[r] = s;
    }
}

__global__ void scale_into_kernel(int n, const double *__restrict__ a, const double *__restrict__ x,
                                  double *__restrict__ y) {
    const double s = 1.0 / *a;
    for (int r = blockIdx.x * 256 + threadIdx.x; r < n; r += gridDim.x * 256) y[r] = s * x[r];
}

__global__ void sqrt_kernel(double *v) { *v = sqrt(*v); }

// dst[i] = src[perm[i]]
__global__ void gather_perm_kernel(int n, const double *__restrict__ src, const int *__restrict__ perm,
                                   double *__restrict__ dst) {
    for (int r = blockIdx.x * 256 + threadIdx.x; r < n; r += gridDim.x * 256) dst[r] = src[perm[r]];
}

__global__ void s2d_matrix_kernel(int n, const float *__restrict__ S, int lds, double *__restrict__ D,
                                  int ldd) {
    const size_t total = (size_t)n * n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const size_t j = e / n, i = e % n;
        D[i + j * ldd] = (double)S[i + j * lds];
    }
}

int grid_for(size_t total) {
    int b = (int)ceil_div(total, (size_t)256);
    const int cap = num_sms() * 8;
    return (cap > 0 && b > cap) ? cap : (b < 1 ? 1 : b);
}

size_t a256(size_t b) { return (b + 255) / 256 * 256; }

constexpr int kGmresM = 100;      // restart length
constexpr int kPrecSplit = 4;     // FP64 storage, split-GEMM trailing updates

struct Solver {
    int n = 0, nrhs = 0;
    const double *A = nullptr;
    int ldA = 0;
    const double *B = nullptr;
    int ldB = 0;
    double *X = nullptr;
    int ldX = 0;
    int precision = 0;
    cudaStream_t s = nullptr;
    float *A32 = nullptr;
    int ld32 = 0;
    int *ipiv = nullptr;
    int *perm = nullptr;
    int *dinfo = nullptr;
    double *R = nullptr;        // n x nrhs residual
    float *D32 = nullptr;       // n x nrhs fp32 work
    double *colv = nullptr;     // [|r| | |x| | |b|] per column, plus GMRES scalars
    unsigned long long *anorm_bits = nullptr;
    double *V = nullptr;        // n x (M+1) Krylov basis (GMRES)
    double *w = nullptr;        // n
    double *t = nullptr;        // n
    double *LU64 = nullptr;     // FP64 copy of the FP32 factors (GMRES preconditioner),
                                // or the FP64 factors themselves (split)
    double *D64 = nullptr;      // n x nrhs fp64 work (split)
    double *h = nullptr;        // M+2 coefficients
    double *h2 = nullptr;       // M+2 (second Gram-Schmidt pass)
    double anorm = 0.0;
    std::vector<double> bnorm;
};

// out(:, 0:ncols) = (LU)^-1 X(:, 0:ncols), in FP32 on X scaled per column by
// `scale` (device, ncols); out may alias X.
int lu_solve(Solver &S, int ncols, const double *X, int ldx, const double *scale, double *out,
             int ldo, bool add) {
    if (S.precision == kPrecSplit) {
        // FP64 factors: P, L^-1, U^-1 in FP64 (no scaling needed)
        KTimer kt(kFamRefine, S.s, 2.0 * S.n * (double)S.n * ncols, 8.0 * S.n * (double)S.n);
        gather_cols_kernel<<<grid_for((size_t)S.n * ncols), 256, 0, S.s>>>(S.n, ncols, X, ldx, S.perm,
                                                                           S.D64, S.n);
        FG_CUDA(cudaGetLastError());
        int st = dtrsm_launch('L', 'L', 'N', 'U', S.n, ncols, 1.0, S.LU64, S.n, S.D64, S.n, S.s);
        if (st != kOk) return st;
        st = dtrsm_launch('L', 'U', 'N', 'N', S.n, ncols, 1.0, S.LU64, S.n, S.D64, S.n, S.s);
        if (st != kOk) return st;
        if (add)
            put_cols_kernel<true><<<grid_for((size_t)S.n * ncols), 256, 0, S.s>>>(S.n, ncols, S.D64,
                                                                                  S.n, out, ldo);
        else
            put_cols_kernel<false><<<grid_for((size_t)S.n * ncols), 256, 0, S.s>>>(S.n, ncols, S.D64,
                                                                                   S.n, out, ldo);
        FG_CUDA(cudaGetLastError());
        return kOk;
    }
    KTimer kt(kFamRefine, S.s, 2.0 * S.n * (double)S.n * ncols, 4.0 * S.n * (double)S.n);
    d2s_cols_kernel<<<grid_for((size_t)S.n * ncols), 256, 0, S.s>>>(S.n, ncols, X, ldx, S.perm,
                                                                      scale, S.D32, S.n);
    FG_CUDA(cudaGetLastError());
    int st = strsm_launch('L', 'L', 'N', 'U', S.n, ncols, 1.0f, S.A32, S.ld32, S.D32, S.n, S.s);
    if (st != kOk) return st;
    st = strsm_launch('L', 'U', 'N', 'N', S.n, ncols, 1.0f, S.A32, S.ld32, S.D32, S.n, S.s);
    if (st != kOk) return st;
    if (add)
        s2d_cols_kernel<true><<<grid_for((size_t)S.n * ncols), 256, 0, S.s>>>(S.n, ncols, S.D32, S.n,
                                                                               scale, out, ldo);
    else
        s2d_cols_kernel<false><<<grid_for((size_t)S.n * ncols), 256, 0, S.s>>>(S.n, ncols, S.D32,
                                                                                S.n, scale, out, ldo);
    FG_CUDA(cudaGetLastError());
    return kOk;
}

// dst = (L^ U^)^-1 P src with the FP32 factors applied in FP64 arithmetic:
// GMRES-IR needs the preconditioned operator (LU)^-1 A in the residual
// precision (Carson & Higham 2018, the u_r-precision matvec), an FP32 solve
// makes it inconsistent at the kappa*u32 level and Arnoldi stalls.
int precond64(Solver &S, const double *src, double *dst) {
    KTimer kt(kFamRefine, S.s, 2.0 * S.n * (double)S.n, 8.0 * S.n * (double)S.n);
    gather_perm_kernel<<<grid_for(S.n), 256, 0, S.s>>>(S.n, src, S.perm, dst);
    FG_CUDA(cudaGetLastError());
    int st = dtrsm_launch('L', 'L', 'N', 'U', S.n, 1, 1.0, S.LU64, S.n, dst, S.n, S.s);
    if (st != kOk) return st;
    return dtrsm_launch('L', 'U', 'N', 'N', S.n, 1, 1.0, S.LU64, S.n, dst, S.n, S.s);
}

// R = B - A X for columns [j0, j0+nc); berr[j] for those columns (host)
int residual(Solver &S, int j0, int nc, std::vector<double> &berr) {
    {
        KTimer kt(kFamRefine, S.s, 0.0, 16.0 * S.n * (double)nc);
        copy_cols_kernel<<<grid_for((size_t)S.n * nc), 256, 0, S.s>>>(
            S.n, nc, S.B + (size_t)j0 * S.ldB, S.ldB, S.R + (size_t)j0 * S.n, S.n);
        FG_CUDA(cudaGetLastError());
    }
    int st = dgemm_launch('N', 'N', S.n, nc, S.n, -1.0, S.A, S.ldA, S.X + (size_t)j0 * S.ldX, S.ldX,
                          1.0, S.R + (size_t)j0 * S.n, S.n, S.s);
    if (st != kOk) return st;
    col_absmax_kernel<<<nc, 256, 0, S.s>>>(S.n, S.R + (size_t)j0 * S.n, S.n, S.colv + j0);
    col_absmax_kernel<<<nc, 256, 0, S.s>>>(S.n, S.X + (size_t)j0 * S.ldX, S.ldX, S.colv + S.nrhs + j0);
    FG_CUDA(cudaGetLastError());
    std::vector<double> hr(nc), hx(nc);
    FG_CUDA(cudaMemcpyAsync(hr.data(), S.colv + j0, sizeof(double) * nc, cudaMemcpyDeviceToHost, S.s));
    FG_CUDA(cudaMemcpyAsync(hx.data(), S.colv + S.nrhs + j0, sizeof(double) * nc,
                            cudaMemcpyDeviceToHost, S.s));
    FG_CUDA(cudaStreamSynchronize(S.s));
    for (int q = 0; q < nc; ++q) {
        const double den = S.anorm * hx[q] + S.bnorm[j0 + q];
        double b = den > 0.0 ? hr[q] / den : (hr[q] > 0.0 ? INFINITY : 0.0);
        if (isnan(hr[q]) || isnan(hx[q])) b = INFINITY;
        berr[j0 + q] = b;
    }
    return kOk;
}

// one restarted GMRES(M) cycle for column j: x_j += d with (LU)^-1 A d ~ (LU)^-1 r_j
// (r_j already in R).  Returns the number of Arnoldi steps taken in *steps.
int gmres_cycle(Solver &S, int j, double rtol, int *steps) {
    const int n = S.n, M = kGmresM;
    double *r = S.R + (size_t)j * n;
    double *sc = S.colv + 3 * S.nrhs;     // device scalars: [scale, norm]
    *steps = 0;
    // z = (LU)^-1 r  -> V(:, 0) unnormalised
    int st = precond64(S, r, S.V);
    if (st != kOk) return st;
    auto norm2_into = [&](const double *v, double *dst) -> int {
        FG_CUDA(cudaMemsetAsync(dst, 0, sizeof(double), S.s));
        dim3 g(std::max(1, std::min(ceil_div(n, 256 * 8), num_sms() * 2)), 1);
        multi_dot_kernel<<<g, 256, 0, S.s>>>(n, v, n, v, dst);
        sqrt_kernel<<<1, 1, 0, S.s>>>(dst);
        FG_CUDA(cudaGetLastError());
        return kOk;
    };
    if ((st = norm2_into(S.V, sc + 1)) != kOk) return st;
    double beta = 0.0;
    FG_CUDA(cudaMemcpyAsync(&beta, sc + 1, sizeof(double), cudaMemcpyDeviceToHost, S.s));
    FG_CUDA(cudaStreamSynchronize(S.s));
    if (!(beta > 0.0) || !isfinite(beta)) return kOk;
    scale_into_kernel<<<grid_for(n), 256, 0, S.s>>>(n, sc + 1, S.V, S.V);
    FG_CUDA(cudaGetLastError());

    std::vector<double> H((size_t)(M + 1) * M, 0.0), cs(M), sn(M), g(M + 1, 0.0);
    g[0] = beta;
    int k = 0;
    for (; k < M; ++k) {
        double *vk = S.V + (size_t)k * n;
        // w = (LU)^-1 A v_k, all in FP64
        FG_CUDA(cudaMemsetAsync(S.t, 0, sizeof(double) * n, S.s));
        if ((st = dgemm_launch('N', 'N', n, 1, n, 1.0, S.A, S.ldA, vk, n, 0.0, S.t, n, S.s)) != kOk)
            return st;
        if ((st = precond64(S, S.t, S.w)) != kOk) return st;
        // classical Gram-Schmidt, twice
        dim3 gd(std::max(1, std::min(ceil_div(n, 256 * 8), num_sms() * 2)), k + 1);
        FG_CUDA(cudaMemsetAsync(S.h, 0, sizeof(double) * (k + 1), S.s));
        multi_dot_kernel<<<gd, 256, 0, S.s>>>(n, S.V, n, S.w, S.h);
        combination_kernel<<<grid_for(n), 256, 0, S.s>>>(n, k + 1, S.V, n, S.h, -1.0, S.w);
        FG_CUDA(cudaMemsetAsync(S.h2, 0, sizeof(double) * (k + 1), S.s));
        multi_dot_kernel<<<gd, 256, 0, S.s>>>(n, S.V, n, S.w, S.h2);
        combination_kernel<<<grid_for(n), 256, 0, S.s>>>(n, k + 1, S.V, n, S.h2, -1.0, S.w);
        FG_CUDA(cudaGetLastError());
        if ((st = norm2_into(S.w, S.h + k + 1)) != kOk) return st;
        std::vector<double> hh(k + 2), hh2(k + 1);
        FG_CUDA(cudaMemcpyAsync(hh.data(), S.h, sizeof(double) * (k + 2), cudaMemcpyDeviceToHost, S.s));
        FG_CUDA(cudaMemcpyAsync(hh2.data(), S.h2, sizeof(double) * (k + 1), cudaMemcpyDeviceToHost, S.s));
        FG_CUDA(cudaStreamSynchronize(S.s));
        for (int i = 0; i <= k; ++i) hh[i] += hh2[i];
        const double hk1 = hh[k + 1];
        if (k + 1 < M + 1 && hk1 > 0.0 && isfinite(hk1)) {
            scale_into_kernel<<<grid_for(n), 256, 0, S.s>>>(n, S.h + k + 1, S.w,
                                                            S.V + (size_t)(k + 1) * n);
            FG_CUDA(cudaGetLastError());
        }
        // apply the previous rotations to column k of H, then a new one
        for (int i = 0; i < k; ++i) {
            const double t = cs[i] * hh[i] + sn[i] * hh[i + 1];
            hh[i + 1] = -sn[i] * hh[i] + cs[i] * hh[i + 1];
            hh[i] = t;
        }
        const double den = hypot(hh[k], hh[k + 1]);
        cs[k] = den > 0.0 ? hh[k] / den : 1.0;
        sn[k] = den > 0.0 ? hh[k + 1] / den : 0.0;
        hh[k] = den;
        hh[k + 1] = 0.0;
        g[k + 1] = -sn[k] * g[k];
        g[k] = cs[k] * g[k];
        for (int i = 0; i <= k; ++i) H[(size_t)i * M + k] = hh[i];
        if (fabs(g[k + 1]) <= rtol * beta || !(hk1 > 0.0) || !isfinite(hk1)) {
            ++k;
            break;
        }
    }
    if (k > M) k = M;
    // y = H(0:k, 0:k)^-1 g(0:k); x_j += V(:, 0:k) y
    std::vector<double> y(k, 0.0);
    for (int i = k - 1; i >= 0; --i) {
        double t = g[i];
        for (int q = i + 1; q < k; ++q) t -= H[(size_t)i * M + q] * y[q];
        y[i] = H[(size_t)i * M + i] != 0.0 ? t / H[(size_t)i * M + i] : 0.0;
    }
    FG_CUDA(cudaMemcpyAsync(S.h, y.data(), sizeof(double) * k, cudaMemcpyHostToDevice, S.s));
    combination_kernel<<<grid_for(n), 256, 0, S.s>>>(n, k, S.V, n, S.h, 1.0, S.X + (size_t)j * S.ldX);
    FG_CUDA(cudaGetLastError());
    *steps = k;
    return kOk;
}

}  // namespace

int dgesv_mixed(int n, int nrhs, const double *A, int ldA, const double *B, int ldB, double *X,
                int ldX, int precision, int solver, int max_iter, double tol, int *iters,
                double *berr_out, int *info_out, cudaStream_t s) {
    Solver S;
    S.n = n;
    S.nrhs = nrhs;
    S.A = A;
    S.ldA = ldA;
    S.B = B;
    S.ldB = ldB;
    S.X = X;
    S.ldX = ldX;
    S.precision = precision;
    S.s = s;
    S.ld32 = (n + 3) / 4 * 4;
    *iters = 0;
    *berr_out = 0.0;
    *info_out = 0;
    if (n == 0 || nrhs == 0) return kOk;
    const double eps = 0x1.0p-53 * 2.0;           // DBL_EPSILON
    if (!(tol > 0.0)) tol = (double)n * eps;

    // slot 1: A32 | ipiv | perm | info | R | D32 | colv | anorm | h | h2
    // split: slot 3: LU64 | ipiv | perm | info | R | D64 | colv | anorm | h | h2
    // (slots 0-2 belong to the split GEMM while the LU runs)
    const bool split = precision == kPrecSplit;
    const int M = kGmresM;
    size_t off = 0;
    const size_t oA32 = off;
    off += split ? a256((size_t)n * n * sizeof(double)) : a256((size_t)S.ld32 * n * sizeof(float));
    const size_t oPiv = off; off += a256((size_t)n * sizeof(int));
    const size_t oPerm = off; off += a256((size_t)n * sizeof(int));
    const size_t oInfo = off; off += 256;
    const size_t oR = off; off += a256((size_t)n * nrhs * sizeof(double));
    const size_t oD = off; off += a256((size_t)n * nrhs * (split ? sizeof(double) : sizeof(float)));
    const size_t oCol = off; off += a256((size_t)(4 * nrhs + 4) * sizeof(double));
    const size_t oAn = off; off += 256;
    const size_t oH = off; off += a256((size_t)(M + 2) * sizeof(double));
    const size_t oH2 = off; off += a256((size_t)(M + 2) * sizeof(double));
    char *p = (char *)workspace_slot(s, split ? 3 : 1, off);
    if (!p) return kErrAlloc;
    if (split) {
        S.LU64 = (double *)(p + oA32);
        S.D64 = (double *)(p + oD);
    } else {
        S.A32 = (float *)(p + oA32);
        S.D32 = (float *)(p + oD);
    }
    S.ipiv = (int *)(p + oPiv);
    S.perm = (int *)(p + oPerm);
    S.dinfo = (int *)(p + oInfo);
    S.R = (double *)(p + oR);
    S.colv = (double *)(p + oCol);
    S.anorm_bits = (unsigned long long *)(p + oAn);
    S.h = (double *)(p + oH);
    S.h2 = (double *)(p + oH2);

    // 1. FP32 copy, norms, LU
    {
        KTimer kt(kFamAux, s, 0.0, 12.0 * n * (double)n);
        if (split)
            copy_cols_kernel<<<grid_for((size_t)n * n), 256, 0, s>>>(n, n, A, ldA, S.LU64, n);
        else
            d2s_cols_kernel<<<grid_for((size_t)n * n), 256, 0, s>>>(n, n, A, ldA, nullptr, nullptr,
                                                                    S.A32, S.ld32);
        FG_CUDA(cudaMemsetAsync(S.anorm_bits, 0, sizeof(unsigned long long), s));
        inf_norm_kernel<<<ceil_div(n, 256), 256, 0, s>>>(n, A, ldA, S.anorm_bits);
        col_absmax_kernel<<<nrhs, 256, 0, s>>>(n, B, ldB, S.colv + 2 * nrhs);
        FG_CUDA(cudaGetLastError());
    }
    int st = split ? dgetrf_split_launch(n, n, S.LU64, n, S.ipiv, S.dinfo, 0, s)
                   : sgetrf_launch(n, n, S.A32, S.ld32, S.ipiv, S.dinfo, precision, s);
    if (st != kOk) return st;
    if ((st = laswp_perm_launch(n, S.ipiv, S.perm, s)) != kOk) return st;
    int hinfo = 0;
    unsigned long long abits = 0;
    S.bnorm.resize(nrhs);
    FG_CUDA(cudaMemcpyAsync(&hinfo, S.dinfo, sizeof(int), cudaMemcpyDeviceToHost, s));
    FG_CUDA(cudaMemcpyAsync(&abits, S.anorm_bits, sizeof(abits), cudaMemcpyDeviceToHost, s));
    FG_CUDA(cudaMemcpyAsync(S.bnorm.data(), S.colv + 2 * nrhs, sizeof(double) * nrhs,
                            cudaMemcpyDeviceToHost, s));
    FG_CUDA(cudaStreamSynchronize(s));
    memcpy(&S.anorm, &abits, sizeof(double));
    *info_out = hinfo;
    if (hinfo != 0) return kOk;   // exactly singular in the working precision: no solve

    // 2. x0 = (LU)^-1 b
    if ((st = lu_solve(S, nrhs, B, ldB, S.colv + 2 * nrhs, X, ldX, false)) != kOk) return st;

    // 3. refinement
    std::vector<double> berr(nrhs, INFINITY), prev(nrhs, INFINITY);
    std::vector<char> use_gmres(nrhs, solver == 1 ? 1 : 0);
    if ((st = residual(S, 0, nrhs, berr)) != kOk) return st;
    int it = 0;
    const int maxit = max_iter > 0 ? max_iter : 30;
    std::vector<char> done(nrhs, 0);
    for (int step = 0; step < maxit; ++step) {
        // columns still above tolerance, by method; a column whose backward
        // error stopped halving switches to GMRES-IR (auto) or stops
        std::vector<int> classical, gmres;
        for (int j = 0; j < nrhs; ++j) {
            if (done[j]) continue;
            if (berr[j] <= tol) {
                done[j] = 1;
                continue;
            }
            // classical steps must halve the backward error (rfs.tcc:182); a
            // GMRES-IR cycle must improve it by at least 10%
            if (step > 0 && !(berr[j] <= (use_gmres[j] ? 0.9 : 0.5) * prev[j])) {
                if (!use_gmres[j] && solver == 2) {
                    use_gmres[j] = 1;
                } else {
                    done[j] = 1;
                    continue;
                }
            }
            (use_gmres[j] ? gmres : classical).push_back(j);
        }
        if (classical.empty() && gmres.empty()) break;
        for (int j = 0; j < nrhs; ++j) prev[j] = berr[j];
        if (!classical.empty()) {
            // one correction for every classical column (contiguous runs)
            size_t q = 0;
            while (q < classical.size()) {
                size_t e = q + 1;
                while (e < classical.size() && classical[e] == classical[e - 1] + 1) ++e;
                const int j0 = classical[q], nc = (int)(e - q);
                if ((st = lu_solve(S, nc, S.R + (size_t)j0 * n, n, S.colv + j0,
                                   X + (size_t)j0 * ldX, ldX, true)) != kOk)
                    return st;
                if ((st = residual(S, j0, nc, berr)) != kOk) return st;
                q = e;
            }
            ++it;
        }
        if (!gmres.empty()) {
            if (!S.V) {
                const size_t vB = a256((size_t)n * (M + 1) * sizeof(double));
                const size_t nB = a256((size_t)n * sizeof(double));
                char *p2 = (char *)workspace_slot(s, 2, vB + 2 * nB);
                if (!p2) return kErrAlloc;
                S.V = (double *)p2;
                S.w = (double *)(p2 + vB);
                S.t = (double *)(p2 + vB + nB);
                if (!split) {
                    S.LU64 = (double *)workspace_slot(s, 3, (size_t)n * n * sizeof(double));
                    if (!S.LU64) return kErrAlloc;
                    KTimer kt(kFamAux, s, 0.0, 12.0 * n * (double)n);
                    s2d_matrix_kernel<<<grid_for((size_t)n * n), 256, 0, s>>>(n, S.A32, S.ld32, S.LU64,
                                                                            n);
                    FG_CUDA(cudaGetLastError());
                }
            }
            for (int j : gmres) {
                int steps = 0;
                if ((st = gmres_cycle(S, j, 1e-10, &steps)) != kOk) return st;
                it += steps;
                if ((st = residual(S, j, 1, berr)) != kOk) return st;
            }
        }
    }
    double worst = 0.0;
    for (int j = 0; j < nrhs; ++j) worst = std::max(worst, berr[j]);
    *iters = it;
    *berr_out = worst;
    trace("dgesv_mixed n=%d nrhs=%d precision=%d solver=%d iters=%d berr=%.3e", n, nrhs, precision,
          solver, it, worst);
    if (!(worst <= tol)) {
        set_last_error("refinement stopped at backward error %.3e > %.3e after %d steps", worst, tol, it);
        return kErrNotConverged;
    }
    return check_device_status(s);
}

}  // namespace fg

// Solve A X = B to FP64 accuracy from a low-precision LU (see the header of
// this file).  A, B, X: device, column-major FP64; A and B are not modified.
FG_API int flens_gb300_dgesv_mixed(int n, int nrhs, const double *A, int ldA, const double *B,
                                   int ldB, double *X, int ldX, int precision, int solver,
                                   int max_iter, double tol, int *iters, double *berr, int *info,
                                   void *stream) {
    if (n < 0) return -1;
    if (nrhs < 0) return -2;
    if (ldA < (n > 1 ? n : 1)) return -4;
    if (ldB < (n > 1 ? n : 1)) return -6;
    if (ldX < (n > 1 ? n : 1)) return -8;
    if (precision < 0 || precision > 4) return -9;
    if (solver < 0 || solver > 2) return -10;
    int it = 0, inf = 0;
    double be = 0.0;
    const int st = fg::dgesv_mixed(n, nrhs, A, ldA, B, ldB, X, ldX, precision, solver, max_iter, tol,
                                   &it, &be, &inf, (cudaStream_t)stream);
    if (iters) *iters = it;
    if (berr) *berr = be;
    if (info) *info = inf;
    return st;
}
