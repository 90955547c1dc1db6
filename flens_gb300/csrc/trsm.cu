// trsm.cu -- FP64 triangular solve with many right-hand sides.
//
// Replaces cxxblas::trsm for double (cxxblas/level3/trsm.tcc:40-82, reached
// from flens::blas::sm flens/blas/level3/sm.tcc:42-72 and dtrsm_
// flens/blas/interface/blas/trsm.cc:90-166).  As in the reference, alpha is
// applied AFTER the solve (trsm.tcc:67).
//
// All eight side/uplo/trans variants reduce to one description: an effective
// triangle M (op(A) for side=Left, op(A)^T for side=Right) addressed as
// M(i,p) = A[i*mi + p*mp], and a set of vectors (columns of B for Left, rows
// of B for Right).  The blocked, right-looking driver solves 64x64 diagonal
// blocks (trsm_diag_wide_kernel: a thread per vector; trsm_diag_narrow_kernel:
// a warp per vector, for few right-hand sides) and applies each solved block to the rest
// of B with the FP64 GEMM.  The diagonal solve uses the column-sweep (axpy)
// form rather than the reference's dot form; the result agrees to rounding.
#include "common.cuh"

namespace fg {
namespace {

constexpr int TRSM_NB = 64;      // diagonal block size
constexpr int TRSM_VEC = 64;     // vectors (threads) per CTA, wide kernel
constexpr int TRSM_WARPS = 8;    // vectors (warps) per CTA, narrow kernel
constexpr int TRSM_NARROW = 512; // below this many vectors use the warp kernel

// Wide kernel: one thread per vector, the vector held in 64 registers and
// solved column by column (x_r -= M(r,i) x_i for all r past i), so every step
// issues independent FMAs instead of one dependent dot-product chain.  The
// diagonal block of M is staged in shared memory and read as broadcasts.
template <typename T, bool LOWER, bool UNIT>
__global__ void __launch_bounds__(TRSM_VEC)
trsm_diag_wide_kernel(int nb, const T *__restrict__ M0, long long mi, long long mp,
                      T *__restrict__ X0, long long xs, long long vs, int nvec) {
    __shared__ T Ms[TRSM_NB * TRSM_NB];   // Ms[r*NB + i] = M(r, i)
    const int t = threadIdx.x;
    for (int e = t; e < nb * nb; e += TRSM_VEC) {
        int r, i;
        if (mi == 1) { r = e % nb; i = e / nb; }
        else { i = e % nb; r = e / nb; }
        Ms[r * TRSM_NB + i] = M0[r * mi + i * mp];
    }
    __syncthreads();
    const long long v = (long long)blockIdx.x * TRSM_VEC + t;
    if (v >= nvec) return;
    T *x = X0 + v * vs;
    T r_[TRSM_NB];
#pragma unroll
    for (int r = 0; r < TRSM_NB; ++r) r_[r] = (r < nb) ? x[r * xs] : T(0);
    if (LOWER) {
#pragma unroll
        for (int i = 0; i < TRSM_NB; ++i) {
            if (i < nb) {
                if (!UNIT) r_[i] = r_[i] / Ms[i * TRSM_NB + i];
                const T xi = r_[i];
#pragma unroll
                for (int r = i + 1; r < TRSM_NB; ++r)
                    if (r < nb) r_[r] = fma(-Ms[r * TRSM_NB + i], xi, r_[r]);
            }
        }
    } else {
#pragma unroll
        for (int i = TRSM_NB - 1; i >= 0; --i) {
            if (i < nb) {
                if (!UNIT) r_[i] = r_[i] / Ms[i * TRSM_NB + i];
                const T xi = r_[i];
#pragma unroll
                for (int r = 0; r < i; ++r) r_[r] = fma(-Ms[r * TRSM_NB + i], xi, r_[r]);
            }
        }
    }
#pragma unroll
    for (int r = 0; r < TRSM_NB; ++r)
        if (r < nb) x[r * xs] = r_[r];
}

// Narrow kernel: one warp per vector, lane l holding rows l and l+32; the
// finished x_i is broadcast with a shuffle and every lane updates its rows.
template <typename T, bool LOWER, bool UNIT>
__global__ void __launch_bounds__(32 * TRSM_WARPS)
trsm_diag_narrow_kernel(int nb, const T *__restrict__ M0, long long mi, long long mp,
                        T *__restrict__ X0, long long xs, long long vs, int nvec) {
    __shared__ T Ms[TRSM_NB * (TRSM_NB + 1)];   // Ms[i*(NB+1) + r] = M(r, i)
    for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
        int r, i;
        if (mi == 1) { r = e % nb; i = e / nb; }
        else { i = e % nb; r = e / nb; }
        Ms[i * (TRSM_NB + 1) + r] = M0[r * mi + i * mp];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const long long v = (long long)blockIdx.x * TRSM_WARPS + (threadIdx.x >> 5);
    if (v >= nvec) return;
    T *x = X0 + v * vs;
    const int r0 = lane, r1 = lane + 32;
    T x0 = (r0 < nb) ? x[r0 * xs] : T(0);
    T x1 = (r1 < nb) ? x[r1 * xs] : T(0);
    for (int s = 0; s < nb; ++s) {
        const int i = LOWER ? s : nb - 1 - s;
        const int owner = i & 31;
        T xi = __shfl_sync(0xffffffffu, (i < 32) ? x0 : x1, owner);
        if (!UNIT) xi = xi / Ms[i * (TRSM_NB + 1) + i];
        if (lane == owner) {
            if (i < 32) x0 = xi; else x1 = xi;
        }
        const T *col = &Ms[i * (TRSM_NB + 1)];
        if (LOWER) {
            if (r0 > i && r0 < nb) x0 = fma(-col[r0], xi, x0);
            if (r1 > i && r1 < nb) x1 = fma(-col[r1], xi, x1);
        } else {
            if (r0 < i) x0 = fma(-col[r0], xi, x0);
            if (r1 < i) x1 = fma(-col[r1], xi, x1);
        }
    }
    if (r0 < nb) x[r0 * xs] = x0;
    if (r1 < nb) x[r1 * xs] = x1;
}

template <typename T>
int launch_diag(int kb, const T *M0, long long mi, long long mp, bool lowerM, bool unit,
                T *X0, long long xs, long long vs, int nvec, cudaStream_t stream) {
    KTimer kt(kFamTrsm, stream, (double)kb * kb * nvec, 16.0 * (double)kb * nvec);
    if (nvec >= TRSM_NARROW) {
        const int grid = ceil_div(nvec, TRSM_VEC);
#define FG_WIDE(L, U) trsm_diag_wide_kernel<T, L, U><<<grid, TRSM_VEC, 0, stream>>>(kb, M0, mi, mp, X0, xs, vs, nvec)
        if (lowerM) { if (unit) FG_WIDE(true, true); else FG_WIDE(true, false); }
        else { if (unit) FG_WIDE(false, true); else FG_WIDE(false, false); }
#undef FG_WIDE
    } else {
        const int grid = ceil_div(nvec, TRSM_WARPS);
#define FG_NARROW(L, U) trsm_diag_narrow_kernel<T, L, U><<<grid, 32 * TRSM_WARPS, 0, stream>>>(kb, M0, mi, mp, X0, xs, vs, nvec)
        if (lowerM) { if (unit) FG_NARROW(true, true); else FG_NARROW(true, false); }
        else { if (unit) FG_NARROW(false, true); else FG_NARROW(false, false); }
#undef FG_NARROW
    }
    FG_CUDA(cudaGetLastError());
    return kOk;
}

template <typename T>
int gemm_t(char ta, char tb, int m, int n, int k, T alpha, const T *A, int ldA, const T *B,
           int ldB, T beta, T *C, int ldC, cudaStream_t s);
template <>
int gemm_t<double>(char ta, char tb, int m, int n, int k, double alpha, const double *A, int ldA,
                   const double *B, int ldB, double beta, double *C, int ldC, cudaStream_t s) {
    return dgemm_launch(ta, tb, m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC, s);
}
template <>
int gemm_t<float>(char ta, char tb, int m, int n, int k, float alpha, const float *A, int ldA,
                  const float *B, int ldB, float beta, float *C, int ldC, cudaStream_t s) {
    return sgemm_launch(ta, tb, m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC, s);
}

}  // namespace

template <typename T>
int trsm_launch_t(char side, char upLo, char transA, char diag, int m, int n,
                  T alpha, const T *A, int ldA, T *B, int ldB, cudaStream_t stream) {
    if (m == 0 || n == 0) return kOk;
    const bool left = (side == 'L' || side == 'l');
    const bool lowerA = (upLo == 'L' || upLo == 'l');
    const bool nT = (transA == 'N' || transA == 'n');
    const int unit = (diag == 'U' || diag == 'u') ? 1 : 0;
    const int ka = left ? m : n;
    const int nvec = left ? n : m;
    bool lowerM;
    long long mi, mp;
    if (left) {
        lowerM = lowerA ^ (!nT);
        mi = nT ? 1 : ldA;
        mp = nT ? ldA : 1;
    } else {
        lowerM = lowerA ^ nT;
        mi = nT ? ldA : 1;
        mp = nT ? 1 : ldA;
    }
    const long long xs = left ? 1 : ldB;
    const long long vs = left ? ldB : 1;
    trace("dtrsm %c%c%c%c m=%d n=%d (effective %s, %d vectors)", side, upLo, transA,
          diag, m, n, lowerM ? "lower" : "upper", nvec);

    const int nblk = ceil_div(ka, TRSM_NB);
    for (int s = 0; s < nblk; ++s) {
        const int bi = lowerM ? s : nblk - 1 - s;
        const int k0 = bi * TRSM_NB;
        const int kb = (ka - k0) < TRSM_NB ? (ka - k0) : TRSM_NB;
        int st0 = launch_diag<T>(kb, A + k0 * mi + k0 * mp, mi, mp, lowerM, unit != 0, B + k0 * xs, xs,
                              vs, nvec, stream);
        if (st0 != kOk) return st0;
        // rows still to solve: below the block (lower) or above it (upper)
        const int r0 = lowerM ? k0 + kb : 0;
        const int rn = lowerM ? ka - (k0 + kb) : k0;
        if (rn <= 0) continue;
        int st;
        if (left) {
            // B[R,:] -= M[R,blk] * B[blk,:];  M(r,p) = A[r*mi + p*mp]
            const char opA = (mi == 1) ? 'N' : 'T';
            const T *Ap = (mi == 1) ? A + r0 + (size_t)k0 * ldA : A + k0 + (size_t)r0 * ldA;
            st = gemm_t<T>(opA, 'N', rn, n, kb, T(-1), Ap, ldA, B + k0, ldB, T(1), B + r0, ldB,
                           stream);
        } else {
            // B[:,R] -= B[:,blk] * M[R,blk]^T;  M[R,blk]^T(p,r) = A[r*mi + p*mp]
            const char opA = (mp == 1) ? 'N' : 'T';
            const T *Ap = (mp == 1) ? A + k0 + (size_t)r0 * ldA : A + r0 + (size_t)k0 * ldA;
            st = gemm_t<T>('N', opA, m, rn, kb, T(-1), B + (size_t)k0 * ldB, ldB, Ap, ldA, T(1),
                           B + (size_t)r0 * ldB, ldB, stream);
        }
        if (st != kOk) return st;
    }
    if (alpha != T(1)) {
        if (sizeof(T) == 8) return dscal_matrix_launch(m, n, (double)alpha, (double *)B, ldB, stream);
        return sscal_matrix_launch(m, n, (float)alpha, (float *)B, ldB, stream);
    }
    return kOk;
}

int dtrsm_launch(char side, char upLo, char transA, char diag, int m, int n, double alpha,
                 const double *A, int ldA, double *B, int ldB, cudaStream_t stream) {
    return trsm_launch_t<double>(side, upLo, transA, diag, m, n, alpha, A, ldA, B, ldB, stream);
}

int strsm_launch(char side, char upLo, char transA, char diag, int m, int n, float alpha,
                 const float *A, int ldA, float *B, int ldB, cudaStream_t stream) {
    return trsm_launch_t<float>(side, upLo, transA, diag, m, n, alpha, A, ldA, B, ldB, stream);
}

}  // namespace fg
