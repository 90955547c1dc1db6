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
// blocks with trsm_diag_kernel (one thread per vector, the block of M and the
// vectors staged in shared memory) and applies each solved block to the rest
// of B with the FP64 GEMM.
#include "common.cuh"

namespace fg {
namespace {

constexpr int TRSM_NB = 64;      // diagonal block size
constexpr int TRSM_VEC = 128;    // vectors (threads) per CTA

__global__ void __launch_bounds__(TRSM_VEC)
trsm_diag_kernel(int nb, const double *__restrict__ M0, long long mi, long long mp,
                 int lowerM, int unit, double *__restrict__ X0, long long xs,
                 long long vs, int nvec) {
    extern __shared__ double smem[];
    double *Ms = smem;                                  // [TRSM_NB][TRSM_NB+1]: Ms[i*(NB+1)+p]
    double *Xs = smem + TRSM_NB * (TRSM_NB + 1);        // [TRSM_NB][TRSM_VEC]:  Xs[i*VEC+t]
    const int t = threadIdx.x;
    const long long v0 = (long long)blockIdx.x * TRSM_VEC;
    const int nv = (int)((nvec - v0) < TRSM_VEC ? (nvec - v0) : TRSM_VEC);

    for (int e = t; e < nb * nb; e += TRSM_VEC) {
        int i, p;
        if (mi == 1) { i = e % nb; p = e / nb; }
        else { p = e % nb; i = e / nb; }
        Ms[i * (TRSM_NB + 1) + p] = M0[i * mi + p * mp];
    }
    double *X = X0 + v0 * vs;
    if (xs == 1) {
        for (int e = t; e < nb * nv; e += TRSM_VEC) {
            const int i = e % nb, v = e / nb;
            Xs[i * TRSM_VEC + v] = X[(long long)v * vs + i];
        }
    } else {
        for (int e = t; e < nb * TRSM_VEC; e += TRSM_VEC) {
            const int v = e % TRSM_VEC, i = e / TRSM_VEC;
            if (v < nv) Xs[i * TRSM_VEC + v] = X[(long long)v * vs + (long long)i * xs];
        }
    }
    __syncthreads();
    if (t < nv) {
        if (lowerM) {
            for (int i = 0; i < nb; ++i) {
                double s = 0.0;
                for (int p = 0; p < i; ++p) s = fma(Ms[i * (TRSM_NB + 1) + p], Xs[p * TRSM_VEC + t], s);
                double x = Xs[i * TRSM_VEC + t] - s;
                if (!unit) x = x / Ms[i * (TRSM_NB + 1) + i];
                Xs[i * TRSM_VEC + t] = x;
            }
        } else {
            for (int i = nb - 1; i >= 0; --i) {
                double s = 0.0;
                for (int q = i + 1; q < nb; ++q) s = fma(Ms[i * (TRSM_NB + 1) + q], Xs[q * TRSM_VEC + t], s);
                double x = Xs[i * TRSM_VEC + t] - s;
                if (!unit) x = x / Ms[i * (TRSM_NB + 1) + i];
                Xs[i * TRSM_VEC + t] = x;
            }
        }
    }
    __syncthreads();
    if (xs == 1) {
        for (int e = t; e < nb * nv; e += TRSM_VEC) {
            const int i = e % nb, v = e / nb;
            X[(long long)v * vs + i] = Xs[i * TRSM_VEC + v];
        }
    } else {
        for (int e = t; e < nb * TRSM_VEC; e += TRSM_VEC) {
            const int v = e % TRSM_VEC, i = e / TRSM_VEC;
            if (v < nv) X[(long long)v * vs + (long long)i * xs] = Xs[i * TRSM_VEC + v];
        }
    }
}

constexpr size_t kDiagSmem = sizeof(double) * (TRSM_NB * (TRSM_NB + 1) + TRSM_NB * TRSM_VEC);

}  // namespace

int dtrsm_launch(char side, char upLo, char transA, char diag, int m, int n,
                 double alpha, const double *A, int ldA, double *B, int ldB,
                 cudaStream_t stream) {
    if (m == 0 || n == 0) return kOk;
    static bool attr_set = false;
    if (!attr_set) {
        FG_CUDA(cudaFuncSetAttribute(trsm_diag_kernel,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kDiagSmem));
        attr_set = true;
    }
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
    const int grid = ceil_div(nvec, TRSM_VEC);
    for (int s = 0; s < nblk; ++s) {
        const int bi = lowerM ? s : nblk - 1 - s;
        const int k0 = bi * TRSM_NB;
        const int kb = (ka - k0) < TRSM_NB ? (ka - k0) : TRSM_NB;
        {
            KTimer kt(kFamTrsm, stream, (double)kb * kb * nvec, 16.0 * (double)kb * nvec);
            trsm_diag_kernel<<<grid, TRSM_VEC, kDiagSmem, stream>>>(
                kb, A + k0 * mi + k0 * mp, mi, mp, lowerM ? 1 : 0, unit, B + k0 * xs, xs, vs, nvec);
            FG_CUDA(cudaGetLastError());
        }
        // rows still to solve: below the block (lower) or above it (upper)
        const int r0 = lowerM ? k0 + kb : 0;
        const int rn = lowerM ? ka - (k0 + kb) : k0;
        if (rn <= 0) continue;
        int st;
        if (left) {
            // B[R,:] -= M[R,blk] * B[blk,:];  M(r,p) = A[r*mi + p*mp]
            const char opA = (mi == 1) ? 'N' : 'T';
            const double *Ap = (mi == 1) ? A + r0 + (size_t)k0 * ldA : A + k0 + (size_t)r0 * ldA;
            st = dgemm_launch(opA, 'N', rn, n, kb, -1.0, Ap, ldA, B + k0, ldB, 1.0, B + r0, ldB,
                              stream);
        } else {
            // B[:,R] -= B[:,blk] * M[R,blk]^T;  M[R,blk]^T(p,r) = A[r*mi + p*mp]
            const char opA = (mp == 1) ? 'N' : 'T';
            const double *Ap = (mp == 1) ? A + k0 + (size_t)r0 * ldA : A + r0 + (size_t)k0 * ldA;
            st = dgemm_launch('N', opA, m, rn, kb, -1.0, B + (size_t)k0 * ldB, ldB, Ap, ldA, 1.0,
                              B + (size_t)r0 * ldB, ldB, stream);
        }
        if (st != kOk) return st;
    }
    if (alpha != 1.0) return dscal_matrix_launch(m, n, alpha, B, ldB, stream);
    return kOk;
}

}  // namespace fg
