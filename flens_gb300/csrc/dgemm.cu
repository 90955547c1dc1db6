// dgemm.cu -- FP64 GEMM, C <- beta*C + alpha*op(A)*op(B), column-major.
//
// Replaces cxxblas::gemm for double (cxxblas/level3/gemm.tcc:42-190, reached
// from flens::blas::mm flens/blas/level3/mm.tcc:379-479 and dgemm_
// flens/blas/interface/blas/gemm.cc:120-230).  Semantics kept from the
// reference: m==0 or n==0 returns at once; C is scaled by beta first (a
// multiply, so NaN/Inf in C propagate even when beta==0); alpha==0 returns
// after that scaling without reading A or B.
//
// GB300 has no FP64 tensor-core kind in tcgen05, so FP64 runs on the FP64
// pipe either as DFMA (dgemm_fma_kernel) or as the legacy FP64 mma.sync
// m8n8k4 (dgemm_dmma_kernel).  Both are register-tiled with shared-memory
// staging; the FP64 issue rate, not memory, bounds them.  Which one runs is
// picked by measured speed (FLENS_GB300_DGEMM=fma|dmma overrides).
#include "common.cuh"

#include <stdlib.h>
#include <string.h>

namespace fg {
namespace {

constexpr int BM = 64, BN = 64, BK = 16, PAD = 1;

// Load the ROWS x BK slab of op(X) starting at (r0, k0) into S[kk][r].
// CR: op(X) is contiguous along r in memory (else along kk).
template <typename T, bool CR, int ROWS, int NT>
struct SlabLoader {
    static constexpr int PER = ROWS * BK / NT;
    T v[PER];

    __device__ __forceinline__ void fetch(const T *__restrict__ X, int ld,
                                          int r0, int rTot, int k0, int kTot) {
#pragma unroll
        for (int t = 0; t < PER; ++t) {
            const int e = threadIdx.x + t * NT;
            int r, kk;
            if (CR) {
                r = e % ROWS;
                kk = e / ROWS;
            } else {
                kk = e % BK;
                r = e / BK;
            }
            const int gr = r0 + r, gk = k0 + kk;
            T x = T(0);
            if (gr < rTot && gk < kTot) {
                x = CR ? X[(size_t)gr + (size_t)gk * ld] : X[(size_t)gk + (size_t)gr * ld];
            }
            v[t] = x;
        }
    }
    __device__ __forceinline__ void store(T (*S)[ROWS + PAD]) {
#pragma unroll
        for (int t = 0; t < PER; ++t) {
            const int e = threadIdx.x + t * NT;
            int r, kk;
            if (CR) {
                r = e % ROWS;
                kk = e / ROWS;
            } else {
                kk = e % BK;
                r = e / BK;
            }
            S[kk][r] = v[t];
        }
    }
};

// ---------------------------------------------------------------- DFMA ----
// TM x TN CTA tile (64x64, or 32x32 for launches of few tiles), 256 threads as
// 16x16, each thread a (TM/16)x(TN/16) sub-tile strided by 16 so shared-memory
// reads are conflict-free broadcasts.  Every element is summed over k in the
// same order whatever the tile, so both tiles give the same bits.  TRI restricts the
// update to one triangle of a square C (syrk): 1 = lower (i >= j), 2 = upper
// (i <= j); tiles wholly outside it exit at once and diagonal tiles store only
// their part, so the other triangle of C is never written.
// KR restricts the k range of each tile to where a triangular operand can be
// nonzero (the skipped terms are exact zeros): 1 op(A) upper (k >= row),
// 2 op(A) lower (k <= row), 3 op(B) upper (k <= column), 4 op(B) lower
// (k >= column).
template <typename T, bool TA, bool TB, int TRI = 0, int KR = 0, int TM = BM, int TN = BN>
__global__ void __launch_bounds__(256)
dgemm_fma_kernel(int m, int n, int k, T alpha,
                 const T *__restrict__ A, int ldA,
                 const T *__restrict__ B, int ldB,
                 T beta, T *__restrict__ C, int ldC) {
    constexpr int RI = TM / 16, RJ = TN / 16;
    __shared__ T As[2][BK][TM + PAD];
    __shared__ T Bs[2][BK][TN + PAD];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int m0 = blockIdx.x * TM, n0 = blockIdx.y * TN;
    if (TRI == 1 && m0 + TM <= n0) return;       // tile strictly above the diagonal
    if (TRI == 2 && n0 + TN <= m0) return;       // tile strictly below the diagonal

    SlabLoader<T, !TA, TM, 256> la;
    SlabLoader<T, TB, TN, 256> lb;
    T acc[RI][RJ];
#pragma unroll
    for (int i = 0; i < RI; ++i)
#pragma unroll
        for (int j = 0; j < RJ; ++j) acc[i][j] = T(0);

    int kb0 = 0, nk = (k + BK - 1) / BK;
    if (KR == 1) kb0 = m0 / BK;
    if (KR == 2) nk = min(nk, (m0 + TM + BK - 1) / BK);
    if (KR == 3) nk = min(nk, (n0 + TN + BK - 1) / BK);
    if (KR == 4) kb0 = n0 / BK;
    if (kb0 < nk) {
        la.fetch(A, ldA, m0, m, kb0 * BK, k);
        lb.fetch(B, ldB, n0, n, kb0 * BK, k);
        la.store(As[0]);
        lb.store(Bs[0]);
        __syncthreads();
    }
    for (int kt = kb0; kt < nk; ++kt) {
        const int cur = (kt - kb0) & 1;
        if (kt + 1 < nk) {
            la.fetch(A, ldA, m0, m, (kt + 1) * BK, k);
            lb.fetch(B, ldB, n0, n, (kt + 1) * BK, k);
        }
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            T a[RI], b[RJ];
#pragma unroll
            for (int i = 0; i < RI; ++i) a[i] = As[cur][kk][tx + 16 * i];
#pragma unroll
            for (int j = 0; j < RJ; ++j) b[j] = Bs[cur][kk][ty + 16 * j];
#pragma unroll
            for (int i = 0; i < RI; ++i)
#pragma unroll
                for (int j = 0; j < RJ; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        if (kt + 1 < nk) {
            la.store(As[cur ^ 1]);
            lb.store(Bs[cur ^ 1]);
        }
        __syncthreads();
    }
    // beta == 1 (every trailing update): beta*C is C exactly, NaN and Inf
    // included, so the multiply is skipped -- one FP64 instruction fewer per
    // element on a pipe that bounds the kernel
    const bool beta1 = beta == T(1);
#pragma unroll
    for (int j = 0; j < RJ; ++j) {
        const int gj = n0 + ty + 16 * j;
        if (gj >= n) continue;
#pragma unroll
        for (int i = 0; i < RI; ++i) {
            const int gi = m0 + tx + 16 * i;
            if (gi >= m) continue;
            if (TRI == 1 && gi < gj) continue;
            if (TRI == 2 && gi > gj) continue;
            T *c = &C[(size_t)gi + (size_t)gj * ldC];
            *c = fma(alpha, acc[i][j], beta1 ? *c : beta * *c);
        }
    }
}

// ---------------------------------------------------------------- DMMA ----
// mma.sync.aligned.m8n8k4.row.col.f64: A frag a0 = A[lane/4][lane%4],
// B frag b0 = B[lane%4][lane/4], C frag {c0,c1} = C[lane/4][2*(lane%4)+{0,1}].
__device__ __forceinline__ void dmma_8x8x4(double &c0, double &c1, double a, double b) {
    asm volatile(
        "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
        : "+d"(c0), "+d"(c1)
        : "d"(a), "d"(b));
}

// 64x64 CTA tile, 4 warps as 2x2, each warp 32x32 = 4x4 tiles of 8x8.
template <bool TA, bool TB>
__global__ void __launch_bounds__(128)
dgemm_dmma_kernel(int m, int n, int k, double alpha,
                  const double *__restrict__ A, int ldA,
                  const double *__restrict__ B, int ldB,
                  double beta, double *__restrict__ C, int ldC) {
    __shared__ double As[2][BK][BM + PAD];
    __shared__ double Bs[2][BK][BN + PAD];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wm = warp & 1, wn = warp >> 1;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;

    SlabLoader<double, !TA, BM, 128> la;
    SlabLoader<double, TB, BN, 128> lb;
    double acc[4][4][2];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;

    const int nk = (k + BK - 1) / BK;
    if (nk > 0) {
        la.fetch(A, ldA, m0, m, 0, k);
        lb.fetch(B, ldB, n0, n, 0, k);
        la.store(As[0]);
        lb.store(Bs[0]);
        __syncthreads();
    }
    const int fr = lane >> 2, fk = lane & 3;
    for (int kt = 0; kt < nk; ++kt) {
        const int cur = kt & 1;
        if (kt + 1 < nk) {
            la.fetch(A, ldA, m0, m, (kt + 1) * BK, k);
            lb.fetch(B, ldB, n0, n, (kt + 1) * BK, k);
        }
#pragma unroll
        for (int ks = 0; ks < BK; ks += 4) {
            double a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[cur][ks + fk][wm * 32 + i * 8 + fr];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[cur][ks + fk][wn * 32 + j * 8 + fr];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) dmma_8x8x4(acc[i][j][0], acc[i][j][1], a[i], b[j]);
        }
        if (kt + 1 < nk) {
            la.store(As[cur ^ 1]);
            lb.store(Bs[cur ^ 1]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int gi = m0 + wm * 32 + i * 8 + fr;
        if (gi >= m) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int gj = n0 + wn * 32 + j * 8 + 2 * fk + h;
                if (gj >= n) continue;
                double *c = &C[(size_t)gi + (size_t)gj * ldC];
                *c = fma(alpha, acc[i][j][h], beta * *c);
            }
        }
    }
}

// ------------------------------------------------------------ skinny N ----
// n <= NC columns (the block updates of a solve with few right-hand sides):
// op(B) is staged in shared memory 64 rows of k at a time; op(A) is streamed
// once from memory, which bounds these launches (they are GEMV-like).
constexpr int SK_K = 64;

// op(A) = A (rows contiguous): one thread per row of C.
template <typename T, int NC, bool TB>
__global__ void __launch_bounds__(256)
dgemm_skinny_nn_kernel(int m, int n, int k, T alpha, const T *__restrict__ A, int ldA,
                       const T *__restrict__ B, int ldB, T beta,
                       T *__restrict__ C, int ldC) {
    __shared__ T Bs[SK_K][NC];
    const int i = blockIdx.x * 256 + threadIdx.x;
    T acc[NC];
#pragma unroll
    for (int j = 0; j < NC; ++j) acc[j] = T(0);
    for (int k0 = 0; k0 < k; k0 += SK_K) {
        const int kk = min(SK_K, k - k0);
        for (int e = threadIdx.x; e < SK_K * NC; e += 256) {
            const int p = e % SK_K, j = e / SK_K;
            T v = T(0);
            if (p < kk && j < n)
                v = TB ? B[(size_t)j + (size_t)(k0 + p) * ldB] : B[(size_t)(k0 + p) + (size_t)j * ldB];
            Bs[p][j] = v;
        }
        __syncthreads();
        if (i < m) {
            const T *a = A + i + (size_t)k0 * ldA;
            for (int p = 0; p < kk; ++p) {
                const T av = a[(size_t)p * ldA];
#pragma unroll
                for (int j = 0; j < NC; ++j) acc[j] = fma(av, Bs[p][j], acc[j]);
            }
        }
        __syncthreads();
    }
    if (i < m) {
#pragma unroll
        for (int j = 0; j < NC; ++j) {
            if (j < n) {
                T *c = &C[(size_t)i + (size_t)j * ldC];
                *c = fma(alpha, acc[j], beta * *c);
            }
        }
    }
}

// op(A) = A^T (each row of op(A) contiguous in memory): one warp per row of C.
template <typename T, int NC, bool TB>
__global__ void __launch_bounds__(256)
dgemm_skinny_tn_kernel(int m, int n, int k, T alpha, const T *__restrict__ A, int ldA,
                       const T *__restrict__ B, int ldB, T beta,
                       T *__restrict__ C, int ldC) {
    __shared__ T Bs[SK_K][NC];
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * 8 + (threadIdx.x >> 5);
    T acc[NC];
#pragma unroll
    for (int j = 0; j < NC; ++j) acc[j] = T(0);
    for (int k0 = 0; k0 < k; k0 += SK_K) {
        const int kk = min(SK_K, k - k0);
        for (int e = threadIdx.x; e < SK_K * NC; e += 256) {
            const int p = e % SK_K, j = e / SK_K;
            T v = T(0);
            if (p < kk && j < n)
                v = TB ? B[(size_t)j + (size_t)(k0 + p) * ldB] : B[(size_t)(k0 + p) + (size_t)j * ldB];
            Bs[p][j] = v;
        }
        __syncthreads();
        if (i < m) {
            const T *a = A + (size_t)i * ldA + k0;
            for (int p = lane; p < kk; p += 32) {
                const T av = a[p];
#pragma unroll
                for (int j = 0; j < NC; ++j) acc[j] = fma(av, Bs[p][j], acc[j]);
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < NC; ++j) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) acc[j] += __shfl_down_sync(0xffffffffu, acc[j], off);
    }
    if (i < m && lane == 0) {
#pragma unroll
        for (int j = 0; j < NC; ++j) {
            if (j < n) {
                T *c = &C[(size_t)i + (size_t)j * ldC];
                *c = fma(alpha, acc[j], beta * *c);
            }
        }
    }
}

// op(A) = A with a long k and at most 4 vectors (the residuals and Krylov
// products of the refinement, n x n times n x 1..4).  The kernel above gives
// a thread one row and walks k with one load in flight, so a 16384^2 GEMV
// streams A at a few percent of HBM.  Here a CTA owns one memory line of rows
// (128 bytes: 16 doubles or 32 floats); its 256 threads are G column groups
// of LR lanes, group g reading columns g, g+G, g+2G, ...  Each thread issues
// 8 column loads before their FMAs, and there are k/G of them per group, so
// the grid of m/LR CTAs keeps enough lines in flight to stream A at HBM
// speed.  The groups' partial sums are added in a fixed order at the end
// (deterministic).
constexpr int GV_UNROLL = 8;

template <typename T, int NC, bool TB>
__global__ void __launch_bounds__(256)
gemv_rows_kernel(int m, int n, int k, T alpha, const T *__restrict__ A, int ldA,
                 const T *__restrict__ B, int ldB, T beta, T *__restrict__ C, int ldC) {
    constexpr int LR = 128 / (int)sizeof(T);     // rows per CTA = lanes per column
    constexpr int G = 256 / LR;                  // column groups
    __shared__ T red[G][NC][LR];
    const int r = threadIdx.x % LR, g = threadIdx.x / LR;
    const int i = blockIdx.x * LR + r;
    T acc[NC];
#pragma unroll
    for (int j = 0; j < NC; ++j) acc[j] = T(0);
    if (i < m) {
        const T *a = A + i;
        auto xv = [&](int p, int j) -> T {
            return TB ? __ldg(&B[(size_t)j + (size_t)p * ldB]) : __ldg(&B[(size_t)p + (size_t)j * ldB]);
        };
        int p = g;
        for (; p + (GV_UNROLL - 1) * G < k; p += GV_UNROLL * G) {
            T av[GV_UNROLL];
#pragma unroll
            for (int u = 0; u < GV_UNROLL; ++u) av[u] = __ldg(&a[(size_t)(p + u * G) * ldA]);
#pragma unroll
            for (int u = 0; u < GV_UNROLL; ++u) {
#pragma unroll
                for (int j = 0; j < NC; ++j)
                    if (j < n) acc[j] = fma(av[u], xv(p + u * G, j), acc[j]);
            }
        }
        for (; p < k; p += G) {
            const T av = __ldg(&a[(size_t)p * ldA]);
#pragma unroll
            for (int j = 0; j < NC; ++j)
                if (j < n) acc[j] = fma(av, xv(p, j), acc[j]);
        }
    }
#pragma unroll
    for (int j = 0; j < NC; ++j) red[g][j][r] = acc[j];
    __syncthreads();
    if (threadIdx.x < LR * NC) {
        const int rr = threadIdx.x % LR, j = threadIdx.x / LR;
        const int ii = blockIdx.x * LR + rr;
        if (ii < m && j < n) {
            T s = T(0);
#pragma unroll
            for (int q = 0; q < G; ++q) s += red[q][j][rr];
            T *c = &C[(size_t)ii + (size_t)j * ldC];
            *c = fma(alpha, s, beta * *c);
        }
    }
}

// y = A x for a square FP64 A: SHAPE 1 reads the lower triangle (and its
// 16 x 16 diagonal blocks), the other triangle holding zeros; SHAPE 0 the
// upper triangle likewise; SHAPE 2 all of A.  The rows go in blocks of 16
// (one 128-byte line of each column); a row block's columns -- [0, i0 + 16)
// below the diagonal, [i0, n) above it -- are cut into chunks of `ch`
// columns (all n for SHAPE 2), and CTA (row block, chunk) sums its chunk with the row-tile
// GEMV's thread layout (16 column groups, 8 loads in flight per thread).
// Every CTA but a row block's last chunk has the same work, so the SMs
// finish together; with one CTA per whole row block the lengths run from 16
// to n columns and a quarter of the elapsed time the SMs idled in the
// ragged last wave.  A row block with one chunk stores y directly; with
// more, each chunk stores its 16 sums in part[c * n + i] and the CTA that
// finishes the row block last (a counter per row block, reset by that CTA)
// adds them in chunk order, so y does not depend on the CTAs' timing.
// A separate kernel, so that the general one keeps its registers (and
// residency).
template <int SHAPE>
__global__ void __launch_bounds__(256)
gemv_tri_kernel(int n, int ch, const double *__restrict__ A, int ldA, const double *__restrict__ x,
                double *__restrict__ y, double *__restrict__ part, unsigned *__restrict__ cnt) {
    constexpr int LR = 16;                       // rows per CTA = lanes per column
    constexpr int G = 256 / LR;                  // column groups
    __shared__ double red[G][LR];
    __shared__ int s_last;
    const int rb = blockIdx.x, c = blockIdx.y;
    const int i0 = rb * LR;
    const int kb = SHAPE == 0 ? i0 : 0;
    const int ke = SHAPE == 1 ? min(n, i0 + LR) : n;
    const int nch = (ke - kb + ch - 1) / ch;
    if (c >= nch) return;                        // uniform over the CTA
    const int cb = kb + c * ch, ce = min(ke, cb + ch);
    const int r = threadIdx.x % LR, g = threadIdx.x / LR;
    const int i = i0 + r;
    double acc = 0.0;
    if (i < n) {
        const double *a = A + i;
        int p = cb + g;
        for (; p + (GV_UNROLL - 1) * G < ce; p += GV_UNROLL * G) {
            double av[GV_UNROLL];
#pragma unroll
            for (int u = 0; u < GV_UNROLL; ++u) av[u] = __ldg(&a[(size_t)(p + u * G) * ldA]);
#pragma unroll
            for (int u = 0; u < GV_UNROLL; ++u) acc = fma(av[u], __ldg(&x[p + u * G]), acc);
        }
        for (; p < ce; p += G) acc = fma(__ldg(&a[(size_t)p * ldA]), __ldg(&x[p]), acc);
    }
    red[g][r] = acc;
    __syncthreads();
    const int ii = i0 + (int)threadIdx.x;
    if (threadIdx.x < LR && ii < n) {
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < G; ++q) s += red[q][threadIdx.x];
        if (nch == 1) {
            y[ii] = s;
        } else {
            part[(size_t)c * n + ii] = s;
            __threadfence();                     // before this chunk is counted
        }
    }
    if (nch == 1) return;
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(&cnt[rb], 1u) == (unsigned)(nch - 1);
    __syncthreads();
    if (s_last && threadIdx.x < LR) {
        __threadfence();
        if (ii < n) {
            double s = 0.0;
            for (int cc = 0; cc < nch; ++cc) s += __ldcg(&part[(size_t)cc * n + ii]);
            y[ii] = s;
        }
        if (threadIdx.x == 0) cnt[rb] = 0u;      // ready for the next launch
    }
}

template <typename T, int NC>
void launch_gemv_rows(bool tb, int m, int n, int k, T alpha, const T *A, int ldA, const T *B,
                      int ldB, T beta, T *C, int ldC, cudaStream_t s) {
    constexpr int LR = 128 / (int)sizeof(T);
    const int grid = ceil_div(m, LR);
    if (tb) gemv_rows_kernel<T, NC, true><<<grid, 256, 0, s>>>(m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC);
    else gemv_rows_kernel<T, NC, false><<<grid, 256, 0, s>>>(m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC);
}

}  // namespace

// y = A x for an n x n triangular FP64 A stored with zeros in its other
// triangle (uplo 'L' or 'U'); only the triangle and the zeros inside its
// 16 x 16 diagonal blocks are read, y is not.  The
// explicit-inverse preconditioner of the mixed solve.  `part` holds
// dtrmv_zeros_part_elems(n) doubles and `cnt` dtrmv_zeros_cnt_elems(n)
// counters, zero before the first call (each call leaves them zero).
static int dtrmv_zeros_chunk(int n, bool full = false) {
    // about 32 equal CTAs per SM over the n^2/2 triangle (n^2 for all of A),
    // at least 256 columns
    const int sms = num_sms() > 0 ? num_sms() : 1;
    const double per = (double)n * n / (full ? 1.0 : 2.0) / (16.0 * 32.0 * sms);
    int ch = ((int)per + 15) / 16 * 16;
    return ch < 256 ? 256 : ch;
}
size_t dtrmv_zeros_part_elems(int n) {
    return n <= 0 ? 0 : (size_t)ceil_div(n, dtrmv_zeros_chunk(n)) * n;
}
size_t dtrmv_zeros_cnt_elems(int n) { return n <= 0 ? 0 : (size_t)ceil_div(n, 16); }

int dtrmv_zeros_launch(char uplo, int n, const double *A, int lda, const double *x, double *y,
                       double *part, unsigned *cnt, cudaStream_t s) {
    if (n <= 0) return kOk;
    constexpr int LR = 16;
    const int ch = dtrmv_zeros_chunk(n);
    const dim3 grid(ceil_div(n, LR), ceil_div(n, ch));
    KTimer kt(kFamPrecond, s, (double)n * n, 4.0 * (double)n * n);
    if (uplo == 'L') gemv_tri_kernel<1><<<grid, 256, 0, s>>>(n, ch, A, lda, x, y, part, cnt);
    else gemv_tri_kernel<0><<<grid, 256, 0, s>>>(n, ch, A, lda, x, y, part, cnt);
    FG_CUDA(cudaGetLastError());
    return kOk;
}

// y = A x for a square n x n FP64 A in the same equal chunks (the Arnoldi
// product of GMRES); the scratch of dtrmv_zeros_launch serves (a row of A
// has at most as many chunks as the longest row of a triangle).
int dgemv_chunk_launch(int n, const double *A, int lda, const double *x, double *y, double *part,
                       unsigned *cnt, cudaStream_t s) {
    if (n <= 0) return kOk;
    constexpr int LR = 16;
    const int ch = dtrmv_zeros_chunk(n, true);
    const dim3 grid(ceil_div(n, LR), ceil_div(n, ch));
    KTimer kt(kFamGemm, s, 2.0 * (double)n * n, 8.0 * (double)n * n);
    gemv_tri_kernel<2><<<grid, 256, 0, s>>>(n, ch, A, lda, x, y, part, cnt);
    FG_CUDA(cudaGetLastError());
    return kOk;
}

namespace {

template <typename T, int NC>
void launch_skinny(bool ta, bool tb, int m, int n, int k, T alpha, const T *A, int ldA,
                   const T *B, int ldB, T beta, T *C, int ldC, cudaStream_t s) {
    if (!ta) {
        const int grid = ceil_div(m, 256);
        if (tb) dgemm_skinny_nn_kernel<T, NC, true><<<grid, 256, 0, s>>>(m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC);
        else dgemm_skinny_nn_kernel<T, NC, false><<<grid, 256, 0, s>>>(m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC);
    } else {
        const int grid = ceil_div(m, 8);
        if (tb) dgemm_skinny_tn_kernel<T, NC, true><<<grid, 256, 0, s>>>(m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC);
        else dgemm_skinny_tn_kernel<T, NC, false><<<grid, 256, 0, s>>>(m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC);
    }
}

template <typename T>
__global__ void scale_kernel(int m, int n, T alpha, T *__restrict__ X, int ld) {
    const size_t total = (size_t)m * n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const size_t j = e / m, i = e % m;
        X[i + j * ld] *= alpha;
    }
}

enum class Engine { Fma, Dmma };

Engine pick_engine() {
    static int mode = -1;
    if (mode < 0) {
        const char *s = getenv("FLENS_GB300_DGEMM");
        // DFMA is the default: on GB300 the FP64 mma.sync path measured no
        // faster than DFMA (see the dgemm profile); the override keeps both
        // reachable for measurement.
        mode = (s && strcmp(s, "dmma") == 0) ? 1 : 0;
    }
    return mode == 1 ? Engine::Dmma : Engine::Fma;
}

}  // namespace

template <typename T>
int scal_matrix_launch_t(int m, int n, T alpha, T *X, int ld, cudaStream_t stream) {
    if (m <= 0 || n <= 0) return kOk;
    const size_t total = (size_t)m * n;
    int blocks = (int)ceil_div(total, (size_t)256);
    const int cap = num_sms() * 8;
    if (cap > 0 && blocks > cap) blocks = cap;
    KTimer kt(kFamAux, stream, (double)m * n, 2.0 * sizeof(T) * m * n);
    scale_kernel<T><<<blocks, 256, 0, stream>>>(m, n, alpha, X, ld);
    FG_CUDA(cudaGetLastError());
    return kOk;
}

int dscal_matrix_launch(int m, int n, double alpha, double *X, int ld, cudaStream_t stream) {
    return scal_matrix_launch_t<double>(m, n, alpha, X, ld, stream);
}

int sscal_matrix_launch(int m, int n, float alpha, float *X, int ld, cudaStream_t stream) {
    return scal_matrix_launch_t<float>(m, n, alpha, X, ld, stream);
}

template <typename T>
int gemm_launch_t(char transA, char transB, int m, int n, int k, T alpha, const T *A, int ldA,
                  const T *B, int ldB, T beta, T *C, int ldC, cudaStream_t stream) {
    if (m == 0 || n == 0) return kOk;
    if (alpha == T(0)) return scal_matrix_launch_t<T>(m, n, beta, C, ldC, stream);
    const bool ta = !(transA == 'N' || transA == 'n');
    const bool tb = !(transB == 'N' || transB == 'n');
    const dim3 grid(ceil_div(m, BM), ceil_div(n, BN));
    if (grid.y > 65535) {
        set_last_error("gemm: n=%d too large for one launch", n);
        return kErrUnsupported;
    }
    KTimer kt(sizeof(T) == 8 ? kFamGemm : kFamAux, stream, 2.0 * m * n * (double)k,
              (double)sizeof(T) * ((double)m * k + (double)k * n + 2.0 * m * n));
    if (!ta && n <= 4 && k >= 256 && (size_t)m * k >= ((size_t)1 << 20)) {
        trace("gemm<%d> %c%c m=%d n=%d k=%d engine=gemv_rows", (int)sizeof(T), transA, transB, m, n, k);
        if (n <= 1) launch_gemv_rows<T, 1>(tb, m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC, stream);
        else if (n <= 2) launch_gemv_rows<T, 2>(tb, m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC, stream);
        else launch_gemv_rows<T, 4>(tb, m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC, stream);
        FG_CUDA(cudaGetLastError());
        return kOk;
    }
    if (n <= 16) {
        trace("gemm<%d> %c%c m=%d n=%d k=%d engine=skinny", (int)sizeof(T), transA, transB, m, n, k);
        if (n <= 1) launch_skinny<T, 1>(ta, tb, m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC, stream);
        else if (n <= 2) launch_skinny<T, 2>(ta, tb, m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC, stream);
        else if (n <= 4) launch_skinny<T, 4>(ta, tb, m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC, stream);
        else if (n <= 8) launch_skinny<T, 8>(ta, tb, m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC, stream);
        else launch_skinny<T, 16>(ta, tb, m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC, stream);
        FG_CUDA(cudaGetLastError());
        return kOk;
    }
    const Engine e = sizeof(T) == 8 ? pick_engine() : Engine::Fma;
    trace("gemm<%d> %c%c m=%d n=%d k=%d engine=%s", (int)sizeof(T), transA, transB, m, n, k,
          e == Engine::Dmma ? "dmma" : "fma");
    if (e == Engine::Dmma) {
        const double *Ad = (const double *)A, *Bd = (const double *)B;
        double *Cd = (double *)C;
        const double al = (double)alpha, be = (double)beta;
        if (!ta && !tb) dgemm_dmma_kernel<false, false><<<grid, 128, 0, stream>>>(m, n, k, al, Ad, ldA, Bd, ldB, be, Cd, ldC);
        else if (ta && !tb) dgemm_dmma_kernel<true, false><<<grid, 128, 0, stream>>>(m, n, k, al, Ad, ldA, Bd, ldB, be, Cd, ldC);
        else if (!ta && tb) dgemm_dmma_kernel<false, true><<<grid, 128, 0, stream>>>(m, n, k, al, Ad, ldA, Bd, ldB, be, Cd, ldC);
        else dgemm_dmma_kernel<true, true><<<grid, 128, 0, stream>>>(m, n, k, al, Ad, ldA, Bd, ldB, be, Cd, ldC);
    } else if ((long long)grid.x * grid.y < 4LL * num_sms()) {
        // few 64x64 tiles (the look-ahead update of the next panel's columns,
        // the last trailing updates): a 64x64x64 tile alone on an SM takes
        // 131k clocks of its FP64 pipe, so 32x32 tiles spread the same work
        // over four times as many SMs
        const dim3 g32(ceil_div(m, 32), ceil_div(n, 32));
#define FG_F32T(TA_, TB_) dgemm_fma_kernel<T, TA_, TB_, 0, 0, 32, 32><<<g32, 256, 0, stream>>>(m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC)
        if (!ta && !tb) FG_F32T(false, false);
        else if (ta && !tb) FG_F32T(true, false);
        else if (!ta && tb) FG_F32T(false, true);
        else FG_F32T(true, true);
#undef FG_F32T
    } else {
        if (!ta && !tb) dgemm_fma_kernel<T, false, false><<<grid, 256, 0, stream>>>(m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC);
        else if (ta && !tb) dgemm_fma_kernel<T, true, false><<<grid, 256, 0, stream>>>(m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC);
        else if (!ta && tb) dgemm_fma_kernel<T, false, true><<<grid, 256, 0, stream>>>(m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC);
        else dgemm_fma_kernel<T, true, true><<<grid, 256, 0, stream>>>(m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC);
    }
    FG_CUDA(cudaGetLastError());
    return kOk;
}

// C <- beta*C + alpha*op(A)*op(B) where one operand is a triangle stored as
// a full matrix with explicit zeros: kr (1..4, see dgemm_fma_kernel) skips
// the k blocks that only meet those zeros.  FMA engine, n > 16.
int dgemm_kr_launch(char transA, char transB, int m, int n, int k, double alpha, const double *A,
                    int ldA, const double *B, int ldB, double beta, double *C, int ldC, int kr,
                    cudaStream_t stream) {
    if (n <= 16 || kr < 1 || kr > 4 || pick_engine() != Engine::Fma)
        return gemm_launch_t<double>(transA, transB, m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC,
                                     stream);
    if (m == 0 || n == 0) return kOk;
    if (alpha == 0.0) return scal_matrix_launch_t<double>(m, n, beta, C, ldC, stream);
    const bool ta = !(transA == 'N' || transA == 'n');
    const bool tb = !(transB == 'N' || transB == 'n');
    const dim3 grid(ceil_div(m, BM), ceil_div(n, BN));
    if (grid.y > 65535) {
        set_last_error("gemm: n=%d too large for one launch", n);
        return kErrUnsupported;
    }
    // the triangle's half of the flops
    KTimer kt(kFamGemm, stream, 1.0 * m * n * (double)k,
              8.0 * ((double)m * k + (double)k * n + 2.0 * m * n));
    trace("gemm %c%c m=%d n=%d k=%d engine=fma k-range=%d", transA, transB, m, n, k, kr);
#define FG_KR(TA_, TB_, K_) dgemm_fma_kernel<double, TA_, TB_, 0, K_><<<grid, 256, 0, stream>>>(m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC)
#define FG_KR4(TA_, TB_) switch (kr) { case 1: FG_KR(TA_, TB_, 1); break; case 2: FG_KR(TA_, TB_, 2); break; \
                                       case 3: FG_KR(TA_, TB_, 3); break; default: FG_KR(TA_, TB_, 4); }
    if (!ta && !tb) { FG_KR4(false, false) }
    else if (ta && !tb) { FG_KR4(true, false) }
    else if (!ta && tb) { FG_KR4(false, true) }
    else { FG_KR4(true, true) }
#undef FG_KR4
#undef FG_KR
    FG_CUDA(cudaGetLastError());
    return kOk;
}

// C <- beta*C + alpha*op(A)*op(B)^T on the uplo triangle of the n x n C, op
// = identity (trans 'N': A, B n x k) or transpose ('T': A, B k x n); only the
// uplo triangle of C is read or written.  k == 0 only scales (unless beta ==
// 1).  No alpha == 0 shortcut: the reference's syrk/syr2k have none.
int tri_gemm_launch(char uplo, char trans, int n, int k, double alpha, const double *A, int ldA,
                    const double *B, int ldB, double beta, double *C, int ldC, cudaStream_t stream) {
    if (n == 0) return kOk;
    if (k == 0) {
        if (beta == 1.0) return kOk;
        alpha = 0.0;                              // acc == 0: C = beta*C on the triangle
    }
    const bool lower = uplo == 'L' || uplo == 'l';
    const bool nt = trans == 'N' || trans == 'n';
    const dim3 grid(ceil_div(n, BM), ceil_div(n, BN));
    if (grid.y > 65535) {
        set_last_error("syrk: n=%d too large for one launch", n);
        return kErrUnsupported;
    }
    KTimer kt(kFamGemm, stream, (double)n * (n + 1) * (double)k,
              8.0 * ((double)n * k * 2.0 + (double)n * (n + 1)));
    const double *Ak = k > 0 ? A : nullptr, *Bk = k > 0 ? B : nullptr;
    const int lda = k > 0 ? ldA : 1, ldb = k > 0 ? ldB : 1;
    // op(A) op(B)^T as gemm(op, op^T)
    if (lower) {
        if (nt) dgemm_fma_kernel<double, false, true, 1><<<grid, 256, 0, stream>>>(n, n, k, alpha, Ak, lda, Bk, ldb, beta, C, ldC);
        else dgemm_fma_kernel<double, true, false, 1><<<grid, 256, 0, stream>>>(n, n, k, alpha, Ak, lda, Bk, ldb, beta, C, ldC);
    } else {
        if (nt) dgemm_fma_kernel<double, false, true, 2><<<grid, 256, 0, stream>>>(n, n, k, alpha, Ak, lda, Bk, ldb, beta, C, ldC);
        else dgemm_fma_kernel<double, true, false, 2><<<grid, 256, 0, stream>>>(n, n, k, alpha, Ak, lda, Bk, ldb, beta, C, ldC);
    }
    FG_CUDA(cudaGetLastError());
    return kOk;
}

// C <- beta*C + alpha*op(A)*op(A)^T on the uplo triangle of the n x n C
// (cxxblas/level3/syrk.tcc:42-90): op(A) = A (n x k, trans 'N') or A^T.
int dsyrk_launch(char uplo, char trans, int n, int k, double alpha, const double *A, int ldA,
                 double beta, double *C, int ldC, cudaStream_t stream) {
    trace("syrk %c%c n=%d k=%d", uplo, trans, n, k);
    return tri_gemm_launch(uplo, trans, n, k, alpha, A, ldA, A, ldA, beta, C, ldC, stream);
}

int dgemm_launch(char transA, char transB, int m, int n, int k, double alpha,
                 const double *A, int ldA, const double *B, int ldB,
                 double beta, double *C, int ldC, cudaStream_t stream) {
    return gemm_launch_t<double>(transA, transB, m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC,
                                 stream);
}

int sgemm_launch(char transA, char transB, int m, int n, int k, float alpha, const float *A,
                 int ldA, const float *B, int ldB, float beta, float *C, int ldC,
                 cudaStream_t stream) {
    return gemm_launch_t<float>(transA, transB, m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC,
                                stream);
}

}  // namespace fg
