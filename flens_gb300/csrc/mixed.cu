// mixed.cu -- the precision form of the solve: low-precision LU on the tensor
// cores, FP64 iterative refinement (classical, or GMRES-IR) to FP64 accuracy.
//
//   1. A32 = fp32(A); LU of A32 with partial pivoting (sgetrf_launch): the
//      panels in FP32 arithmetic (the reference's tf2 for float), the
//      trailing updates A22 -= A21*U12 on the tensor cores in TF32, BF16,
//      FP8 e4m3 (per-row/column scaled), FP32-accurate 3xTF32, or FP8 e4m3
//      with each scaled entry split into two or three e4m3 terms (precision
//      5 / 6: about 2^-8 / 2^-12 relative products from the FP8 kind).
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
#include <stdlib.h>
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

// ||A||_inf = max_i sum_j |A(i, j)|.  A CTA per 16 rows (one 128-byte line of
// each column) and 16 column groups, 8 loads in flight per thread, so the
// sweep streams A at HBM speed (a thread per row walking all columns with one
// load in flight took milliseconds at n = 16384).  The row sums are added in
// a fixed order and the maximum is an integer atomic: non-negative doubles
// order like their bit patterns, and a NaN sum wins.
__global__ void __launch_bounds__(256)
inf_norm_kernel(int n, const double *__restrict__ A, int lda, unsigned long long *__restrict__ out) {
    constexpr int LR = 16, G = 16, U = 8;
    __shared__ double red[G][LR];
    const int r = threadIdx.x % LR, g = threadIdx.x / LR;
    const int i = blockIdx.x * LR + r;
    double s = 0.0;
    if (i < n) {
        const double *a = A + i;
        int p = g;
        for (; p + (U - 1) * G < n; p += U * G) {
            double v[U];
#pragma unroll
            for (int u = 0; u < U; ++u) v[u] = __ldg(&a[(size_t)(p + u * G) * lda]);
#pragma unroll
            for (int u = 0; u < U; ++u) s += fabs(v[u]);
        }
        for (; p < n; p += G) s += fabs(__ldg(&a[(size_t)p * lda]));
    }
    red[g][r] = s;
    __syncthreads();
    if (threadIdx.x < LR) {
        const int ii = blockIdx.x * LR + threadIdx.x;
        if (ii < n) {
            double t = 0.0;
#pragma unroll
            for (int q = 0; q < G; ++q) t += red[q][threadIdx.x];
            atomicMax(out, (unsigned long long)__double_as_longlong(t));
        }
    }
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

// ---------------------------------------------------------------------------
// The GMRES preconditioner z = U^-1 L^-1 P v: the factors as stored (FP32, or
// FP64 for the split LU) applied in FP64 arithmetic, one vector.  A
// substitution solve is a chain of 64-row blocks, and GB300 issues FP64 at 2
// lanes per clock per SM, so a 64-step substitution inside each block (about
// 4 us in one warp) would dominate the chain.  Instead, per block b of the
// triangle (pred = the block solved just before b, b-1 for L and b+1 for U):
//   Dinv_b = inverse of the diagonal block (FP64, from the stored values),
//   P_b    = Dinv_b * M(b, pred),
//   x_b    = Dinv_b (v_b - sum over blocks before pred of M(b,k) x_k) - P_b x_pred.
// Everything but the last product is computed while the predecessor is still
// being solved, so the chain's critical path per block is one 64x64 FP64
// product (4096 FMAs, about 1 us on one SM) plus the flag hand-over.  The
// inverses make this a slightly different (equally fixed, linear) operator
// than substitution: its error is of order cond(diagonal block) * u64, far
// below the factors' own low-precision error, and GMRES only needs the
// preconditioner to be the same operator every time it is applied.
constexpr int PC_NB = 64;
constexpr int PC_THREADS = 256;
constexpr int PC_PREP_SMEM = 2 * PC_NB * (PC_NB + 1) * (int)sizeof(double);

// Dinv and P of every block, stored [block][p][r] (column-major 64 x 64);
// rows and columns beyond the matrix are identity (Dinv) and zero (P).
template <typename MT, bool LOWER>
__global__ void __launch_bounds__(PC_THREADS)
pc_prep_kernel(int n, const MT *__restrict__ F, int ldf, double *__restrict__ Dinv,
               double *__restrict__ P) {
    extern __shared__ double pc_sm[];
    double(*D)[PC_NB + 1] = (double(*)[PC_NB + 1])pc_sm;                       // D[i][j] = M(R0+i, j)
    double(*Y)[PC_NB + 1] = (double(*)[PC_NB + 1])(pc_sm + PC_NB * (PC_NB + 1));   // Y[i][c] = Dinv(i, c)
    const int nblk = gridDim.x, b = blockIdx.x, tid = threadIdx.x;
    const int R0 = b * PC_NB, kb = min(PC_NB, n - R0);
    for (int e = tid; e < PC_NB * PC_NB; e += PC_THREADS) {
        const int i = e % PC_NB, j = e / PC_NB;
        double v = (i == j) ? 1.0 : 0.0;
        if (i < kb && j < kb && (LOWER ? j < i : j >= i))
            v = (double)F[(size_t)(R0 + i) + (size_t)(R0 + j) * ldf];
        D[i][j] = v;
    }
    __syncthreads();
    if (tid < PC_NB) {          // column c of the inverse by substitution
        const int c = tid;
        if (LOWER) {
            for (int i = 0; i < c; ++i) Y[i][c] = 0.0;
            Y[c][c] = 1.0;
            for (int i = c + 1; i < PC_NB; ++i) {
                double s = 0.0;
                for (int j = c; j < i; ++j) s = fma(D[i][j], Y[j][c], s);
                Y[i][c] = -s;
            }
        } else {
            for (int i = c + 1; i < PC_NB; ++i) Y[i][c] = 0.0;
            Y[c][c] = 1.0 / D[c][c];
            for (int i = c - 1; i >= 0; --i) {
                double s = 0.0;
                for (int j = i + 1; j <= c; ++j) s = fma(D[i][j], Y[j][c], s);
                Y[i][c] = -s / D[i][i];
            }
        }
    }
    __syncthreads();
    double *dout = Dinv + (size_t)b * PC_NB * PC_NB;
    for (int e = tid; e < PC_NB * PC_NB; e += PC_THREADS) dout[e] = Y[e % PC_NB][e / PC_NB];
    const int pred = LOWER ? b - 1 : b + 1;
    if (pred < 0 || pred >= nblk) return;                 // uniform over the CTA
    const int K0 = pred * PC_NB, kk = min(PC_NB, n - K0);
    for (int e = tid; e < PC_NB * PC_NB; e += PC_THREADS) {   // D no longer read: reuse
        const int i = e % PC_NB, j = e / PC_NB;
        D[i][j] = (i < kb && j < kk) ? (double)F[(size_t)(R0 + i) + (size_t)(K0 + j) * ldf] : 0.0;
    }
    __syncthreads();
    double *pout = P + (size_t)b * PC_NB * PC_NB;
    for (int e = tid; e < PC_NB * PC_NB; e += PC_THREADS) {
        const int r = e % PC_NB, p = e / PC_NB;
        double s = 0.0;
        for (int t = 0; t < PC_NB; ++t) s = fma(Y[r][t], D[t][p], s);
        pout[e] = s;
    }
}

// A solved block is published as 128 tagged 64-bit words, (epoch << 32) |
// one 32-bit half of a double, written with single-copy-atomic 64-bit stores.
// A reader polls the words themselves until all carry the call's epoch: one
// L2 round trip per hand-off, where a ready flag costs the flag's round trip,
// then the data's, plus the writer's release fence.
__device__ __forceinline__ void pc_put(unsigned long long *p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long pc_get(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Thread (r, q) of a block's solve: row r, 16-column quarter q.  The stored
// block M(b, k) in registers: 16 values along row R0+r (coalesced over r).
template <typename MT>
__device__ __forceinline__ void pc_fetch(MT (&v)[16], const MT *__restrict__ F, int ldf, int n,
                                         int row, bool rok, int K0, int q) {
    const MT *src = F + (size_t)row + (size_t)(K0 + 16 * q) * ldf;
#pragma unroll
    for (int u = 0; u < 16; ++u) v[u] = (rok && K0 + 16 * q + u < n) ? src[(size_t)u * ldf] : MT(0);
}

// Reads the published block of x starting at row K0 into dst[0..63] (rows at
// or beyond n read as zero): threads 0..127 each poll one tagged word, bounded
// by kSpinLimit.  false on a timeout (status set), after which the CTA must
// return; ends with a block barrier either way.
__device__ __forceinline__ bool pc_take(const unsigned long long *tag, int K0, int n,
                                        unsigned epoch, double *dst, int *status, int *s_abort) {
    const int t = threadIdx.x;
    if (t < 2 * PC_NB) {
        const int p = t >> 1;
        unsigned half = 0;
        if (K0 + p < n) {
            const unsigned long long *w = tag + 2 * (size_t)K0 + t;
            unsigned long long v = pc_get(w);
            unsigned spins = 0;
            while ((unsigned)(v >> 32) != epoch) {
                if (++spins > kSpinLimit) {
                    atomicOr(status, kDevBarrierTimeout);
                    *s_abort = 1;
                    break;
                }
                if (spins > 64) __nanosleep(32);
                v = pc_get(w);
            }
            half = (unsigned)v;
        }
        reinterpret_cast<unsigned *>(dst + p)[t & 1] = half;
    }
    __syncthreads();
    return *s_abort == 0;
}

// One triangle of the preconditioner in place on X (n), in ONE cooperative
// launch: CTA s solves the s-th block in solve order (the first rows for L,
// the last for U) and publishes it into `tag` with the call's epoch.  The
// stored blocks before the predecessor are applied as they are published,
// the next one loaded into registers while waiting for the current one.
template <typename MT, bool LOWER>
__global__ void __launch_bounds__(PC_THREADS, 2)
pc_chain_kernel(int n, const MT *__restrict__ F, int ldf, const double *__restrict__ Dinv,
                const double *__restrict__ P, double *X, unsigned long long *tag, unsigned epoch,
                int *status) {
    __shared__ double xk[2][PC_NB];
    __shared__ double part[4][PC_NB];
    __shared__ double rhs[PC_NB];
    __shared__ int s_abort;
    const int nblk = gridDim.x, s = blockIdx.x, tid = threadIdx.x;
    const int b = LOWER ? s : nblk - 1 - s;
    const int R0 = b * PC_NB, kb = min(PC_NB, n - R0);
    const int r = tid & (PC_NB - 1), q = tid >> 6;
    const bool rok = r < kb;
    if (tid == 0) s_abort = 0;
    double di[16], pi[16];
    {
        const double *dsrc = Dinv + (size_t)b * PC_NB * PC_NB + (size_t)(16 * q) * PC_NB + r;
        const double *psrc = P + (size_t)b * PC_NB * PC_NB + (size_t)(16 * q) * PC_NB + r;
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            di[u] = dsrc[u * PC_NB];
            pi[u] = s > 0 ? psrc[u * PC_NB] : 0.0;
        }
    }
    __syncthreads();                 // s_abort initialised
    // blocks solved before the predecessor: solve-order indices 0 .. s-2
    const int npre = s - 1;
    double acc = 0.0;
    MT c0[16], c1[16];
    auto kblk = [&](int s2) { return (LOWER ? s2 : nblk - 1 - s2) * PC_NB; };
    auto apply = [&](MT(&v)[16], int s2, int buf) -> bool {
        if (!pc_take(tag, kblk(s2), n, epoch, xk[buf], status, &s_abort)) return false;
        // the block's 16 products summed on their own, then added
        double blk = 0.0;
#pragma unroll
        for (int u = 0; u < 16; ++u) blk = fma((double)v[u], xk[buf][16 * q + u], blk);
        acc += blk;
        return true;
    };
    if (npre > 0) pc_fetch(c0, F, ldf, n, R0 + r, rok, kblk(0), q);
    for (int s2 = 0; s2 < npre; s2 += 2) {
        if (s2 + 1 < npre) pc_fetch(c1, F, ldf, n, R0 + r, rok, kblk(s2 + 1), q);
        if (!apply(c0, s2, 0)) return;
        if (s2 + 1 >= npre) break;
        if (s2 + 2 < npre) pc_fetch(c0, F, ldf, n, R0 + r, rok, kblk(s2 + 2), q);
        if (!apply(c1, s2 + 1, 1)) return;
    }
    part[q][r] = acc;
    __syncthreads();
    if (q == 0) rhs[r] = rok ? X[R0 + r] - ((part[0][r] + part[1][r]) + (part[2][r] + part[3][r]))
                             : 0.0;
    __syncthreads();
    double cp = 0.0;
#pragma unroll
    for (int u = 0; u < 16; ++u) cp = fma(di[u], rhs[16 * q + u], cp);
    part[q][r] = cp;                 // every read of part above precedes the last barrier
    __syncthreads();
    double xr = (part[0][r] + part[1][r]) + (part[2][r] + part[3][r]);
    if (s > 0) {
        // xk[0] was last read before two barriers ago
        if (!pc_take(tag, (LOWER ? b - 1 : b + 1) * PC_NB, n, epoch, xk[0], status, &s_abort)) return;
        double pp = 0.0;
#pragma unroll
        for (int u = 0; u < 16; ++u) pp = fma(pi[u], xk[0][16 * q + u], pp);
        part[q][r] = pp;
        __syncthreads();
        xr -= (part[0][r] + part[1][r]) + (part[2][r] + part[3][r]);
    }
    if (q == 0 && rok) {
        X[R0 + r] = xr;
        const unsigned long long bits = (unsigned long long)__double_as_longlong(xr);
        const unsigned long long e = (unsigned long long)epoch << 32;
        unsigned long long *w = tag + 2 * (size_t)(R0 + r);
        pc_put(w, e | (bits & 0xffffffffull));
        pc_put(w + 1, e | (bits >> 32));
    }
}

// Blocks per SM of the chain kernel (0 if the query fails), per device.
template <typename MT>
int pc_chain_per_sm() {
    static int cached[64];
    const int d = device_id();
    if (d < 0 || d >= 64) return 0;
    if (cached[d] == 0) {
        int lo = 0, up = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&lo, pc_chain_kernel<MT, true>, PC_THREADS,
                                                          0) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&up, pc_chain_kernel<MT, false>, PC_THREADS,
                                                          0) != cudaSuccess) {
            cudaGetLastError();
            lo = up = 0;
        }
        const int bps = lo < up ? lo : up;
        cached[d] = bps > 0 ? bps : -1;
    }
    return cached[d] > 0 ? cached[d] : 0;
}

int grid_for(size_t total) {
    int b = (int)ceil_div(total, (size_t)256);
    const int cap = num_sms() * 8;
    return (cap > 0 && b > cap) ? cap : (b < 1 ? 1 : b);
}

size_t a256(size_t b) { return (b + 255) / 256 * 256; }

// GMRES restart length: 100, or FLENS_GB300_GMRES_RESTART (2..4000); the
// Krylov basis takes n x (restart+1) doubles
int gmres_restart() {
    static int m = [] {
        const char *e = getenv("FLENS_GB300_GMRES_RESTART");
        const int v = e ? atoi(e) : 0;
        return (v >= 2 && v <= 4000) ? v : 100;
    }();
    return m;
}
constexpr int kPrecBF16 = 1, kPrecFP8 = 2, kPrec3xTF32 = 3, kPrecFP8x2 = 5;   // = the tensor-core kinds
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
    // preconditioner blocks (pc_prep_kernel): Dinv and P of L, then of U
    double *pcDL = nullptr, *pcPL = nullptr, *pcDU = nullptr, *pcPU = nullptr;
    unsigned long long *pcTag = nullptr;   // 2n tagged words: the solved blocks of a call
    unsigned pc_epoch = 0;
    bool pc = false;            // chained block-inverse preconditioner in use
    // explicit-inverse preconditioner: L^-1 and U^-1 (FP64, n x n, zeros in
    // the other triangle) and an n-vector between the two products
    bool pcinv = false;
    double *Linv = nullptr, *Uinv = nullptr, *pcTmp = nullptr;
    // chunk sums and per-row-block counters of the chunked GEMVs (the
    // Arnoldi product A v and the explicit-inverse products)
    double *gvPart = nullptr;
    unsigned *gvCnt = nullptr;
};

// ---------------------------------------------------------------------------
// Explicit-inverse preconditioner, for factors that need hundreds of GMRES
// steps (BF16, FP8).  The chained solve above is bound by its 64-row
// hand-offs (about 4 us each, 1.1 ms per triangle at n = 16384); with L^-1
// and U^-1 formed once, each application is two triangle-aware FP64 GEMVs
// (n^2/2 DFMA each, spread over every SM).  The inverses are formed from the
// stored FP32 factors by 2 x 2 block recursion,
//   [A 0; B C]^-1 = [A^-1 0; -C^-1 B A^-1  C^-1]  (and likewise for U),
// with FP32-accurate products (3xTF32 on the tensor cores, FP32 FMAs for
// small blocks) over 64 x 64 diagonal inverses taken in FP64, and are kept in
// FP64.  Applying them is again a fixed linear operator -- an FP32-accurate
// approximation of (LU)^-1, far closer than the factors are to A -- which is
// what GMRES needs of its preconditioner.

// The inverse of each 64 x 64 diagonal block of the stored triangle (unit
// lower for LOWER, upper with its diagonal otherwise), in FP64 by
// substitution, written rounded to FP32 into the same block of Inv.
template <bool LOWER>
__global__ void __launch_bounds__(PC_THREADS)
inv_diag_kernel(int n, const float *__restrict__ F, int ldf, float *__restrict__ Inv, int ldi) {
    extern __shared__ double pc_sm[];
    double(*D)[PC_NB + 1] = (double(*)[PC_NB + 1])pc_sm;
    double(*Y)[PC_NB + 1] = (double(*)[PC_NB + 1])(pc_sm + PC_NB * (PC_NB + 1));
    const int b = blockIdx.x, tid = threadIdx.x;
    const int R0 = b * PC_NB, kb = min(PC_NB, n - R0);
    for (int e = tid; e < PC_NB * PC_NB; e += PC_THREADS) {
        const int i = e % PC_NB, j = e / PC_NB;
        double v = (i == j) ? 1.0 : 0.0;
        if (i < kb && j < kb && (LOWER ? j < i : j >= i))
            v = (double)F[(size_t)(R0 + i) + (size_t)(R0 + j) * ldf];
        D[i][j] = v;
    }
    __syncthreads();
    if (tid < PC_NB) {
        const int c = tid;
        if (LOWER) {
            for (int i = 0; i < c; ++i) Y[i][c] = 0.0;
            Y[c][c] = 1.0;
            for (int i = c + 1; i < PC_NB; ++i) {
                double s = 0.0;
                for (int j = c; j < i; ++j) s = fma(D[i][j], Y[j][c], s);
                Y[i][c] = -s;
            }
        } else {
            for (int i = c + 1; i < PC_NB; ++i) Y[i][c] = 0.0;
            Y[c][c] = 1.0 / D[c][c];
            for (int i = c - 1; i >= 0; --i) {
                double s = 0.0;
                for (int j = i + 1; j <= c; ++j) s = fma(D[i][j], Y[j][c], s);
                Y[i][c] = -s / D[i][i];
            }
        }
    }
    __syncthreads();
    for (int e = tid; e < kb * kb; e += PC_THREADS) {
        const int i = e % kb, j = e / kb;
        Inv[(size_t)(R0 + i) + (size_t)(R0 + j) * ldi] = (float)Y[i][j];
    }
}

// Whether the chained block-inverse preconditioner fits (every block of the
// triangle resident at once for the cooperative launch).
bool pc_fits(int n, bool fp64_factors) {
    const int nblk = ceil_div(n, PC_NB);
    const int per = fp64_factors ? pc_chain_per_sm<double>() : pc_chain_per_sm<float>();
    return per > 0 && (long long)per * num_sms() >= nblk && nblk <= 4096;
}

// bytes of Dinv or P of one triangle
size_t pc_block_bytes(int n) { return a256((size_t)ceil_div(n, PC_NB) * PC_NB * PC_NB * sizeof(double)); }

// Dinv and P of both triangles of the stored factors.
template <typename MT>
int pc_prepare(Solver &S, const MT *F, int ldf) {
    const int nblk = ceil_div(S.n, PC_NB);
    static DeviceOnce onceL, onceU;
    int st = set_smem_once(onceL, (const void *)pc_prep_kernel<MT, true>, PC_PREP_SMEM);
    if (st != kOk) return st;
    if ((st = set_smem_once(onceU, (const void *)pc_prep_kernel<MT, false>, PC_PREP_SMEM)) != kOk)
        return st;
    KTimer kt(kFamPrecond, S.s, 2.0 * nblk * 4.0 * PC_NB * PC_NB * PC_NB,
              2.0 * S.n * (double)S.n * sizeof(MT));
    pc_prep_kernel<MT, true><<<nblk, PC_THREADS, PC_PREP_SMEM, S.s>>>(S.n, F, ldf, S.pcDL, S.pcPL);
    pc_prep_kernel<MT, false><<<nblk, PC_THREADS, PC_PREP_SMEM, S.s>>>(S.n, F, ldf, S.pcDU, S.pcPU);
    FG_CUDA(cudaGetLastError());
    return kOk;
}

// One triangle of the preconditioner in place on x (device, n).
template <typename MT>
int pc_solve(Solver &S, const MT *F, int ldf, bool lower, double *x) {
    int n = S.n;
    const int nblk = ceil_div(n, PC_NB);
    Workspace *w = workspace_for(S.s, 0);
    if (!w) return kErrAlloc;
    int *status = w->status;
    // a fresh epoch per call; the tag words start at zero (epoch 0 is never used)
    unsigned epoch = ++S.pc_epoch;
    if (epoch == 0) {
        FG_CUDA(cudaMemsetAsync(S.pcTag, 0, 2 * sizeof(unsigned long long) * (size_t)n, S.s));
        epoch = S.pc_epoch = 1;
    }
    const double *Dv = lower ? S.pcDL : S.pcDU;
    const double *Pv = lower ? S.pcPL : S.pcPU;
    unsigned long long *tag = S.pcTag;
    void *args[] = {&n, &F, &ldf, &Dv, &Pv, &x, &tag, &epoch, &status};
    KTimer kt(kFamPrecond, S.s, (double)n * n, (double)n * n * sizeof(MT) / 2.0 + 16.0 * n * PC_NB);
    const void *fn = lower ? (const void *)pc_chain_kernel<MT, true> : (const void *)pc_chain_kernel<MT, false>;
    FG_CUDA(cudaLaunchCooperativeKernel(fn, dim3(nblk), dim3(PC_THREADS), args, 0, S.s));
    return kOk;
}

// ---- explicit-inverse preconditioner: build ---------------------------------
// Workspace of the build: the two FP32 inverses (ld ldi), the product
// scratch T, the 3xTF32 operand buffers, the FP64 inverses and an n-vector.
struct InvPlan {
    int n, ldi, half;
    size_t oL32, oU32, oT, oG, oL64, oU64, oTmp, total;
};

InvPlan inv_plan(int n) {
    InvPlan p;
    p.n = n;
    p.ldi = (n + 3) / 4 * 4;
    p.half = ((n + 1) / 2 + PC_NB - 1) / PC_NB * PC_NB;   // the largest block a product sees
    const int th = (p.half + 3) / 4 * 4;
    size_t o = 0;
    p.oL32 = o; o += a256((size_t)p.ldi * n * sizeof(float));
    p.oU32 = o; o += a256((size_t)p.ldi * n * sizeof(float));
    p.oT = o;   o += a256((size_t)th * p.half * sizeof(float));
    p.oG = o;   o += a256(tc_update_workspace_bytes(kPrec3xTF32, p.half, p.half, p.half));
    p.oL64 = o; o += a256((size_t)n * n * sizeof(double));
    p.oU64 = o; o += a256((size_t)n * n * sizeof(double));
    p.oTmp = o; o += a256((size_t)n * sizeof(double));
    p.total = o;
    return p;
}

// C (m x n) = alpha * A (m x k) * B (k x n), FP32 storage, FP32-accurate:
// 3xTF32 on the tensor cores, or FP32 FMAs on the CUDA cores for small blocks
int inv_product(int m, int n, int k, float alpha, const float *A, int lda, const float *B, int ldb,
                float *C, int ldc, void *gbuf, cudaStream_t s) {
    if ((double)m * n * k < 256.0 * 256.0 * 256.0)
        return sgemm_launch('N', 'N', m, n, k, alpha, A, lda, B, ldb, 0.0f, C, ldc, s);
    return tc_gemm_f32x3_nn(m, n, k, alpha, A, lda, B, ldb, 0.0f, C, ldc, gbuf, s);
}

// Inv(r0:r0+sz, r0:r0+sz) = inverse of the stored triangle's diagonal block,
// given the inverses of its 64 x 64 diagonal blocks already in place.
int inv_recurse(bool lower, int r0, int sz, const float *F, int ldf, float *Inv, int ldi, float *T,
                void *gbuf, cudaStream_t s) {
    if (sz <= PC_NB) return kOk;
    const int h = ((sz + 1) / 2 + PC_NB - 1) / PC_NB * PC_NB;   // h < sz, a multiple of 64
    const int h2 = sz - h;
    int st;
    if ((st = inv_recurse(lower, r0, h, F, ldf, Inv, ldi, T, gbuf, s)) != kOk) return st;
    if ((st = inv_recurse(lower, r0 + h, h2, F, ldf, Inv, ldi, T, gbuf, s)) != kOk) return st;
    float *I11 = Inv + r0 + (size_t)r0 * ldi;
    float *I22 = Inv + (r0 + h) + (size_t)(r0 + h) * ldi;
    if (lower) {
        // L^-1(21) = -L22^-1 L21 L11^-1
        const int ldt = (h2 + 3) / 4 * 4;
        const float *L21 = F + (r0 + h) + (size_t)r0 * ldf;
        if ((st = inv_product(h2, h, h2, 1.0f, I22, ldi, L21, ldf, T, ldt, gbuf, s)) != kOk) return st;
        return inv_product(h2, h, h, -1.0f, T, ldt, I11, ldi, Inv + (r0 + h) + (size_t)r0 * ldi, ldi,
                           gbuf, s);
    }
    // U^-1(12) = -U11^-1 U12 U22^-1
    const int ldt = (h + 3) / 4 * 4;
    const float *U12 = F + r0 + (size_t)(r0 + h) * ldf;
    if ((st = inv_product(h, h2, h, 1.0f, I11, ldi, U12, ldf, T, ldt, gbuf, s)) != kOk) return st;
    return inv_product(h, h2, h2, -1.0f, T, ldt, I22, ldi, Inv + r0 + (size_t)(r0 + h) * ldi, ldi,
                       gbuf, s);
}

// L^-1 and U^-1 of the FP32 factors into S.Linv / S.Uinv (FP64).
int pcinv_prepare(Solver &S) {
    const int n = S.n;
    const InvPlan p = inv_plan(n);
    char *base = (char *)workspace_slot(S.s, 3, p.total);
    if (!base) return kErrAlloc;
    float *L32 = (float *)(base + p.oL32), *U32 = (float *)(base + p.oU32), *T = (float *)(base + p.oT);
    void *gbuf = base + p.oG;
    S.Linv = (double *)(base + p.oL64);
    S.Uinv = (double *)(base + p.oU64);
    S.pcTmp = (double *)(base + p.oTmp);
    static DeviceOnce onceL, onceU;
    int st = set_smem_once(onceL, (const void *)inv_diag_kernel<true>, PC_PREP_SMEM);
    if (st != kOk) return st;
    if ((st = set_smem_once(onceU, (const void *)inv_diag_kernel<false>, PC_PREP_SMEM)) != kOk) return st;
    const int nblk = ceil_div(n, PC_NB);
    {
        KTimer kt(kFamPrecond, S.s, 2.0 * nblk * PC_NB * PC_NB * PC_NB / 3.0, 8.0 * n * (double)p.ldi);
        FG_CUDA(cudaMemsetAsync(L32, 0, (size_t)p.ldi * n * sizeof(float), S.s));
        FG_CUDA(cudaMemsetAsync(U32, 0, (size_t)p.ldi * n * sizeof(float), S.s));
        FG_CUDA(cudaMemsetAsync(T, 0, p.oG - p.oT, S.s));
        inv_diag_kernel<true><<<nblk, PC_THREADS, PC_PREP_SMEM, S.s>>>(n, S.A32, S.ld32, L32, p.ldi);
        inv_diag_kernel<false><<<nblk, PC_THREADS, PC_PREP_SMEM, S.s>>>(n, S.A32, S.ld32, U32, p.ldi);
        FG_CUDA(cudaGetLastError());
    }
    if ((st = inv_recurse(true, 0, n, S.A32, S.ld32, L32, p.ldi, T, gbuf, S.s)) != kOk) return st;
    if ((st = inv_recurse(false, 0, n, S.A32, S.ld32, U32, p.ldi, T, gbuf, S.s)) != kOk) return st;
    KTimer kt(kFamAux, S.s, 0.0, 24.0 * n * (double)n);
    s2d_matrix_kernel<<<grid_for((size_t)n * n), 256, 0, S.s>>>(n, L32, p.ldi, S.Linv, n);
    s2d_matrix_kernel<<<grid_for((size_t)n * n), 256, 0, S.s>>>(n, U32, p.ldi, S.Uinv, n);
    FG_CUDA(cudaGetLastError());
    return kOk;
}

// out(:, 0:ncols) = (LU)^-1 X(:, 0:ncols), in FP32 on X scaled per column by
// `scale` (device, ncols); out may alias X.
int lu_solve(Solver &S, int ncols, const double *X, int ldx, const double *scale, double *out,
             int ldo, bool add) {
    if (S.precision == kPrecSplit) {
        // FP64 factors: P, L^-1, U^-1 in FP64 (no scaling needed)
        {
            KTimer kt(kFamRefine, S.s, 0.0, 16.0 * S.n * (double)ncols);
            gather_cols_kernel<<<grid_for((size_t)S.n * ncols), 256, 0, S.s>>>(S.n, ncols, X, ldx,
                                                                               S.perm, S.D64, S.n);
            FG_CUDA(cudaGetLastError());
        }
        int st = dtrsm_launch('L', 'L', 'N', 'U', S.n, ncols, 1.0, S.LU64, S.n, S.D64, S.n, S.s);
        if (st != kOk) return st;
        st = dtrsm_launch('L', 'U', 'N', 'N', S.n, ncols, 1.0, S.LU64, S.n, S.D64, S.n, S.s);
        if (st != kOk) return st;
        KTimer kt(kFamRefine, S.s, 0.0, 24.0 * S.n * (double)ncols);
        if (add)
            put_cols_kernel<true><<<grid_for((size_t)S.n * ncols), 256, 0, S.s>>>(S.n, ncols, S.D64,
                                                                                  S.n, out, ldo);
        else
            put_cols_kernel<false><<<grid_for((size_t)S.n * ncols), 256, 0, S.s>>>(S.n, ncols, S.D64,
                                                                                   S.n, out, ldo);
        FG_CUDA(cudaGetLastError());
        return kOk;
    }
    {
        KTimer kt(kFamRefine, S.s, 0.0, 12.0 * S.n * (double)ncols);
        d2s_cols_kernel<<<grid_for((size_t)S.n * ncols), 256, 0, S.s>>>(S.n, ncols, X, ldx, S.perm,
                                                                          scale, S.D32, S.n);
        FG_CUDA(cudaGetLastError());
    }
    int st = strsm_launch('L', 'L', 'N', 'U', S.n, ncols, 1.0f, S.A32, S.ld32, S.D32, S.n, S.s);
    if (st != kOk) return st;
    st = strsm_launch('L', 'U', 'N', 'N', S.n, ncols, 1.0f, S.A32, S.ld32, S.D32, S.n, S.s);
    if (st != kOk) return st;
    KTimer kt(kFamRefine, S.s, 0.0, 20.0 * S.n * (double)ncols);
    if (add)
        s2d_cols_kernel<true><<<grid_for((size_t)S.n * ncols), 256, 0, S.s>>>(S.n, ncols, S.D32, S.n,
                                                                               scale, out, ldo);
    else
        s2d_cols_kernel<false><<<grid_for((size_t)S.n * ncols), 256, 0, S.s>>>(S.n, ncols, S.D32,
                                                                                S.n, scale, out, ldo);
    FG_CUDA(cudaGetLastError());
    return kOk;
}

// dst = (L^ U^)^-1 P src with the stored (FP32) factors applied in FP64
// arithmetic: GMRES-IR needs the preconditioned operator (LU)^-1 A in the
// residual precision (Carson & Higham 2018, the u_r-precision matvec); an FP32
// solve makes it inconsistent at the kappa*u32 level and Arnoldi stalls.  The
// chained block-inverse solves read the factors as stored; where they do not
// fit (n beyond what one cooperative launch holds) the FP64 copy LU64 goes
// through the blocked triangular solves.
int precond64(Solver &S, const double *src, double *dst) {
    {
        KTimer kt(kFamKrylov, S.s, 0.0, 20.0 * S.n);
        gather_perm_kernel<<<grid_for(S.n), 256, 0, S.s>>>(S.n, src, S.perm, dst);
        FG_CUDA(cudaGetLastError());
    }
    if (S.pcinv) {
        int st = dtrmv_zeros_launch('L', S.n, S.Linv, S.n, dst, S.pcTmp, S.gvPart, S.gvCnt, S.s);
        if (st != kOk) return st;
        return dtrmv_zeros_launch('U', S.n, S.Uinv, S.n, S.pcTmp, dst, S.gvPart, S.gvCnt, S.s);
    }
    if (S.pc) {
        int st;
        if (S.precision == kPrecSplit) {
            if ((st = pc_solve<double>(S, S.LU64, S.n, true, dst)) != kOk) return st;
            return pc_solve<double>(S, S.LU64, S.n, false, dst);
        }
        if ((st = pc_solve<float>(S, S.A32, S.ld32, true, dst)) != kOk) return st;
        return pc_solve<float>(S, S.A32, S.ld32, false, dst);
    }
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
    {
        KTimer kt(kFamRefine, S.s, 0.0, 16.0 * S.n * (double)nc);
        col_absmax_kernel<<<nc, 256, 0, S.s>>>(S.n, S.R + (size_t)j0 * S.n, S.n, S.colv + j0);
        col_absmax_kernel<<<nc, 256, 0, S.s>>>(S.n, S.X + (size_t)j0 * S.ldX, S.ldX,
                                               S.colv + S.nrhs + j0);
        FG_CUDA(cudaGetLastError());
    }
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
    const int n = S.n, M = gmres_restart();
    double *r = S.R + (size_t)j * n;
    double *sc = S.colv + 3 * S.nrhs;     // device scalars: [scale, norm]
    *steps = 0;
    // z = (LU)^-1 r  -> V(:, 0) unnormalised
    int st = precond64(S, r, S.V);
    if (st != kOk) return st;
    auto norm2_into = [&](const double *v, double *dst) -> int {
        KTimer kt(kFamKrylov, S.s, 2.0 * n, 8.0 * n);
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
    {
        KTimer kt(kFamKrylov, S.s, (double)n, 16.0 * n);
        scale_into_kernel<<<grid_for(n), 256, 0, S.s>>>(n, sc + 1, S.V, S.V);
        FG_CUDA(cudaGetLastError());
    }

    std::vector<double> H((size_t)(M + 1) * M, 0.0), cs(M), sn(M), g(M + 1, 0.0);
    g[0] = beta;
    int k = 0;
    for (; k < M; ++k) {
        double *vk = S.V + (size_t)k * n;
        // w = (LU)^-1 A v_k, all in FP64; A v_k in equal chunks per CTA
        if ((st = dgemv_chunk_launch(n, S.A, S.ldA, vk, S.t, S.gvPart, S.gvCnt, S.s)) != kOk)
            return st;
        if ((st = precond64(S, S.t, S.w)) != kOk) return st;
        // classical Gram-Schmidt, twice
        {
            KTimer kt(kFamKrylov, S.s, 8.0 * n * (k + 1), 32.0 * n * (k + 1));
            dim3 gd(std::max(1, std::min(ceil_div(n, 256 * 8), num_sms() * 2)), k + 1);
            FG_CUDA(cudaMemsetAsync(S.h, 0, sizeof(double) * (k + 1), S.s));
            multi_dot_kernel<<<gd, 256, 0, S.s>>>(n, S.V, n, S.w, S.h);
            combination_kernel<<<grid_for(n), 256, 0, S.s>>>(n, k + 1, S.V, n, S.h, -1.0, S.w);
            FG_CUDA(cudaMemsetAsync(S.h2, 0, sizeof(double) * (k + 1), S.s));
            multi_dot_kernel<<<gd, 256, 0, S.s>>>(n, S.V, n, S.w, S.h2);
            combination_kernel<<<grid_for(n), 256, 0, S.s>>>(n, k + 1, S.V, n, S.h2, -1.0, S.w);
            FG_CUDA(cudaGetLastError());
        }
        if ((st = norm2_into(S.w, S.h + k + 1)) != kOk) return st;
        std::vector<double> hh(k + 2), hh2(k + 1);
        FG_CUDA(cudaMemcpyAsync(hh.data(), S.h, sizeof(double) * (k + 2), cudaMemcpyDeviceToHost, S.s));
        FG_CUDA(cudaMemcpyAsync(hh2.data(), S.h2, sizeof(double) * (k + 1), cudaMemcpyDeviceToHost, S.s));
        FG_CUDA(cudaStreamSynchronize(S.s));
        for (int i = 0; i <= k; ++i) hh[i] += hh2[i];
        const double hk1 = hh[k + 1];
        if (k + 1 < M + 1 && hk1 > 0.0 && isfinite(hk1)) {
            KTimer kt(kFamKrylov, S.s, (double)n, 16.0 * n);
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
    KTimer kt(kFamKrylov, S.s, 2.0 * n * k, 8.0 * n * (k + 2));
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
    const int M = gmres_restart();
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
        inf_norm_kernel<<<ceil_div(n, 16), 256, 0, s>>>(n, A, ldA, S.anorm_bits);
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
                // BF16 and FP8 factors: hundreds of GMRES steps, so the
                // explicit inverses repay their formation (n >= 2048); their
                // workspace is taken first, and without it the chained
                // preconditioner serves instead
                S.pcinv = !split && n >= 2048 &&
                          (S.precision == kPrecBF16 || S.precision == kPrecFP8 || S.precision == kPrecFP8x2);
                if (S.pcinv && !workspace_slot(s, 3, inv_plan(n).total)) {
                    cudaGetLastError();
                    trace("dgesv_mixed: no memory for the explicit inverses, chained preconditioner");
                    S.pcinv = false;
                }
                S.pc = !S.pcinv && pc_fits(n, split);
                const size_t pB = S.pc ? pc_block_bytes(n) : 0;
                const size_t tB = S.pc ? a256(2 * sizeof(unsigned long long) * (size_t)n) : 0;
                const size_t gB = a256(dtrmv_zeros_part_elems(n) * sizeof(double));
                const size_t cB = a256(dtrmv_zeros_cnt_elems(n) * sizeof(unsigned));
                char *p2 = (char *)workspace_slot(s, 2, vB + 2 * nB + 4 * pB + tB + gB + cB);
                if (!p2) return kErrAlloc;
                S.V = (double *)p2;
                S.w = (double *)(p2 + vB);
                S.t = (double *)(p2 + vB + nB);
                S.gvPart = (double *)(p2 + vB + 2 * nB + 4 * pB + tB);
                S.gvCnt = (unsigned *)(p2 + vB + 2 * nB + 4 * pB + tB + gB);
                FG_CUDA(cudaMemsetAsync(S.gvCnt, 0, cB, s));
                if (S.pc) {
                    char *pp = p2 + vB + 2 * nB;
                    S.pcDL = (double *)pp;
                    S.pcPL = (double *)(pp + pB);
                    S.pcDU = (double *)(pp + 2 * pB);
                    S.pcPU = (double *)(pp + 3 * pB);
                    S.pcTag = (unsigned long long *)(pp + 4 * pB);
                    FG_CUDA(cudaMemsetAsync(S.pcTag, 0, tB, s));
                    st = split ? pc_prepare<double>(S, S.LU64, n) : pc_prepare<float>(S, S.A32, S.ld32);
                    if (st != kOk) return st;
                } else if (S.pcinv) {
                    if ((st = pcinv_prepare(S)) != kOk) return st;
                } else if (!split) {
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
    if (precision < 0 || precision > 6) return -9;
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
