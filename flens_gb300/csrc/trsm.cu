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
// blocks (trsm_diag_tile_kernel: 32 vectors per CTA, 8 rows per thread;
// trsm_diag_warp_kernel: a warp per vector for up to 32 vectors) and applies
// each solved block to the rest of B with the FP64 GEMM.  The
// diagonal solve uses the column-sweep (axpy) form rather than the
// reference's dot form, and multiplies by the reciprocal of the diagonal
// instead of dividing; the result agrees to rounding.
#include "common.cuh"

#include <stdlib.h>

#include <atomic>

namespace fg {
namespace {

constexpr int TRSM_NB = 64;      // diagonal block size
constexpr int TRSM_VPC = 32;     // vectors per CTA
constexpr int TRSM_THREADS = 256;
constexpr int TRSM_RPT = TRSM_NB * TRSM_VPC / TRSM_THREADS;   // rows per thread (8)

// Solves the kb x kb (kb <= 64) diagonal block M for 32 vectors per CTA.
// Lane l of every warp holds vector l; warp w holds the 8 consecutive rows
// of row block blk(w) in registers.  Column by column, the warp owning row i
// finishes x_i (times the precomputed 1/M(i,i) unless the diagonal is unit)
// and publishes it through a double-buffered shared slot; after one barrier
// the warps with rows still open below (lower) or above (upper) i update
// them.  A warp whose rows are all finished skips the step as a whole, so
// the FP64 instructions issued are about 1.1x the triangle's FMAs (the pipe
// issues 2 FP64 lanes per clock per SM, so this is the kernel's bound); the
// blocks are paired {0,7}, {1,6}, {2,5}, {3,4} on the warps that share a
// scheduler so the schedulers get equal work.  The 64 x 32 tile of X is
// staged through shared memory so that global loads and stores are
// coalesced whichever of the row or vector index is contiguous.
template <typename T, bool LOWER, bool UNIT>
__global__ void __launch_bounds__(TRSM_THREADS)
trsm_diag_tile_kernel(int nb, const T *__restrict__ M0, long long mi, long long mp,
                      T *__restrict__ X0, long long xs, long long vs, int nvec) {
    __shared__ T Ms[TRSM_NB][TRSM_NB + 1];     // Ms[i][r] = M(r, i)
    __shared__ T Xs[TRSM_NB][TRSM_VPC + 1];    // Xs[r][v]
    __shared__ T rinv[TRSM_NB];
    __shared__ T xb[2][TRSM_VPC];
    const int t = threadIdx.x;
    const long long v0 = (long long)blockIdx.x * TRSM_VPC;
    const int nv = (int)((nvec - v0) < TRSM_VPC ? (nvec - v0) : TRSM_VPC);
    for (int e = t; e < nb * nb; e += TRSM_THREADS) {
        int r, i;
        if (mi == 1) { r = e % nb; i = e / nb; }
        else { i = e % nb; r = e / nb; }
        Ms[i][r] = M0[r * mi + i * mp];
    }
    // X tile: lanes run along whichever index is contiguous in memory
    for (int e = t; e < TRSM_NB * TRSM_VPC; e += TRSM_THREADS) {
        int r, v;
        if (xs == 1) { r = e % TRSM_NB; v = e / TRSM_NB; }
        else { v = e % TRSM_VPC; r = e / TRSM_VPC; }
        Xs[r][v] = (r < nb && v < nv) ? X0[(v0 + v) * vs + r * xs] : T(0);
    }
    __syncthreads();
    if (!UNIT && t < nb) rinv[t] = T(1) / Ms[t][t];
    const int v = t & 31, w = t >> 5;
    const int r0 = 8 * (w < 4 ? w : 11 - w);        // this warp's row block
    T x[TRSM_RPT];
#pragma unroll
    for (int j = 0; j < TRSM_RPT; ++j) x[j] = Xs[r0 + j][v];
    __syncthreads();
    for (int s = 0; s < nb; ++s) {
        const int i = LOWER ? s : nb - 1 - s;
        if ((i >> 3) == (r0 >> 3)) {                  // warp-uniform: owner of row i
            // selects, not x[i & 7]: an indexed access would move x to local memory
            const int k = i & 7;
            T xi = x[0];
#pragma unroll
            for (int j = 1; j < TRSM_RPT; ++j) xi = (j == k) ? x[j] : xi;
            if (!UNIT) xi *= rinv[i];
#pragma unroll
            for (int j = 0; j < TRSM_RPT; ++j) x[j] = (j == k) ? xi : x[j];
            xb[s & 1][v] = xi;
        }
        __syncthreads();
        if (LOWER ? (r0 + 7 > i) : (r0 < i)) {          // warp-uniform: rows still open
            const T xi = xb[s & 1][v];
#pragma unroll
            for (int j = 0; j < TRSM_RPT; ++j) {
                const int r = r0 + j;
                if (LOWER ? (r > i && r < nb) : (r < i)) x[j] = fma(-Ms[i][r], xi, x[j]);
            }
        }
    }
#pragma unroll
    for (int j = 0; j < TRSM_RPT; ++j) Xs[r0 + j][v] = x[j];
    __syncthreads();
    for (int e = t; e < TRSM_NB * TRSM_VPC; e += TRSM_THREADS) {
        int r, vv;
        if (xs == 1) { r = e % TRSM_NB; vv = e / TRSM_NB; }
        else { vv = e % TRSM_VPC; r = e / TRSM_VPC; }
        if (r < nb && vv < nv) X0[(v0 + vv) * vs + r * xs] = Xs[r][vv];
    }
}

// Few vectors (the solves with one or a handful of right-hand sides): one warp
// per vector, lane l holding rows l and l + 32.  A step is a shuffle of the
// finished x_i, one multiply by the precomputed 1/M(i,i) and the FMAs of the
// rows still open -- no block barrier on the dependency chain.
constexpr int TRSM_WARP_VECS = 8;      // warps (vectors) per CTA

// The warp kernel is the lower-latency choice while the tile kernel would
// run at most one CTA per SM (each tile CTA is ~17 us of FP64 pipe time):
// up to FLENS_GB300_TRSM_WARP_MAX vectors, default 2560.
int trsm_warp_max() {
    static int v = [] {
        const char *e = getenv("FLENS_GB300_TRSM_WARP_MAX");
        const int x = e ? atoi(e) : 0;
        return x > 0 ? x : 2560;
    }();
    return v;
}

template <typename T, bool LOWER, bool UNIT>
__global__ void __launch_bounds__(32 * TRSM_WARP_VECS)
trsm_diag_warp_kernel(int nb, const T *__restrict__ M0, long long mi, long long mp,
                      T *__restrict__ X0, long long xs, long long vs, int nvec) {
    __shared__ T Ms[TRSM_NB][TRSM_NB + 1];     // Ms[i][r] = M(r, i)
    __shared__ T rinv[TRSM_NB];
    for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
        int r, i;
        if (mi == 1) { r = e % nb; i = e / nb; }
        else { i = e % nb; r = e / nb; }
        Ms[i][r] = M0[r * mi + i * mp];
    }
    __syncthreads();
    if (!UNIT && threadIdx.x < nb) rinv[threadIdx.x] = T(1) / Ms[threadIdx.x][threadIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const long long v = (long long)blockIdx.x * TRSM_WARP_VECS + (threadIdx.x >> 5);
    if (v >= nvec) return;
    T *x = X0 + v * vs;
    const int r0 = lane, r1 = lane + 32;
    T x0 = r0 < nb ? x[r0 * xs] : T(0);
    T x1 = r1 < nb ? x[r1 * xs] : T(0);
    for (int s = 0; s < nb; ++s) {
        const int i = LOWER ? s : nb - 1 - s;
        T xi = __shfl_sync(0xffffffffu, i < 32 ? x0 : x1, i & 31);
        if (!UNIT) xi *= rinv[i];
        if (lane == (i & 31)) {
            if (i < 32) x0 = xi;
            else x1 = xi;
        }
        if (LOWER) {
            if (r0 > i && r0 < nb) x0 = fma(-Ms[i][r0], xi, x0);
            if (r1 > i && r1 < nb) x1 = fma(-Ms[i][r1], xi, x1);
        } else {
            if (r0 < i) x0 = fma(-Ms[i][r0], xi, x0);
            if (r1 < i) x1 = fma(-Ms[i][r1], xi, x1);
        }
    }
    if (r0 < nb) x[r0 * xs] = x0;
    if (r1 < nb) x[r1 * xs] = x1;
}

// ------------------------------------------------------------------------
// Few vectors (<= 4) against a triangle of more than one block, in ONE launch:
// CTA s solves the s-th 64-row block in solve order (the first block for a
// lower triangle, the last for an upper one).  It applies the blocks solved
// before it as they are published -- staging each off-diagonal block of M
// before it waits, so the read overlaps the wait -- then solves its own
// diagonal block with one warp per vector and publishes it (release store of
// the call's epoch into its flag; acquire spins with an iteration limit).
// The launch is cooperative, so every CTA is resident and no wait can depend
// on a CTA that has not started.  This replaces the 2 x blocks launches of
// the blocked driver for the trs solves with one right-hand side.
constexpr int CH_NB = 64;
constexpr int CH_MAXV = 4;
constexpr int CH_THREADS = 256;

// spin limit of the next chained solve when it is made to stall (0: none)
std::atomic<unsigned> g_stall_next_chain{0};

__device__ __forceinline__ void ch_release(unsigned long long *p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ch_acquire(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// spin_limit bounds every wait (kSpinLimit when 0).  stall != 0 is the
// failure-detection test: block 0 first waits for a flag value that nothing
// publishes, so it gives up, sets the status word and returns, and every
// block after it gives up in turn.
template <typename T, bool LOWER, bool UNIT>
__global__ void __launch_bounds__(CH_THREADS)
trsv_chain_kernel(int ka, const T *__restrict__ M0, long long mi, long long mp, T *X0, long long xs,
                  long long vs, int nvec, unsigned long long *flags, unsigned long long epoch,
                  int *status, unsigned spin_limit, int stall) {
    __shared__ T Mb[CH_NB][CH_NB + 1];                 // Mb[p][r] = M(R0 + r, K0 + p)
    __shared__ T Md[CH_NB][CH_NB + 1];                 // the diagonal block, same layout
    __shared__ T xk[CH_MAXV][CH_NB];
    __shared__ T part[CH_THREADS / CH_NB][CH_MAXV][CH_NB];
    __shared__ T rinv[CH_NB];
    __shared__ int s_abort;
    const int nblk = gridDim.x, s = blockIdx.x, tid = threadIdx.x;
    const int b = LOWER ? s : nblk - 1 - s;
    const int R0 = b * CH_NB, kb = min(CH_NB, ka - R0);
    const int r = tid & (CH_NB - 1), q = tid / CH_NB;    // row; 16-column quarter
    const unsigned limit = spin_limit ? spin_limit : kSpinLimit;
    if (tid == 0) {
        s_abort = 0;
        if (stall && s == 0) {
            // its own flag never holds epoch + 1 during this launch
            unsigned spins = 0;
            while (ch_acquire(&flags[0]) != epoch + 1) {
                if (++spins > limit) {
                    atomicOr(status, kDevBarrierTimeout);
                    s_abort = 1;
                    break;
                }
                if (spins > 32) __nanosleep(64);
            }
        }
    }
    T acc[CH_MAXV];
#pragma unroll
    for (int v = 0; v < CH_MAXV; ++v) acc[v] = T(0);

    auto stage = [&](T (*D)[CH_NB + 1], int K0, int kk) {
        for (int e = tid; e < CH_NB * CH_NB; e += CH_THREADS) {
            int rr, pp;
            if (mi == 1) { rr = e % CH_NB; pp = e / CH_NB; }
            else { pp = e % CH_NB; rr = e / CH_NB; }
            D[pp][rr] = (rr < kb && pp < kk) ? M0[(R0 + rr) * mi + (K0 + pp) * mp] : T(0);
        }
    };
    // the diagonal block and its reciprocals do not depend on other blocks:
    // off the critical path, before any wait
    stage(Md, R0, kb);
    __syncthreads();
    if (s_abort) return;
    if (!UNIT && tid < kb) rinv[tid] = T(1) / Md[tid][tid];

    for (int s2 = 0; s2 < s; ++s2) {
        const int k = LOWER ? s2 : nblk - 1 - s2;
        const int K0 = k * CH_NB, kk = min(CH_NB, ka - K0);
        stage(Mb, K0, kk);
        if (tid == 0) {
            unsigned spins = 0;
            while (ch_acquire(&flags[s2]) != epoch) {
                if (++spins > limit) {
                    atomicOr(status, kDevBarrierTimeout);
                    s_abort = 1;
                    break;
                }
                if (spins > 32) __nanosleep(64);
            }
        }
        __syncthreads();
        if (s_abort) return;
        // block k of x, final (L2 reads: an L1 line could predate the solve)
        for (int e = tid; e < nvec * CH_NB; e += CH_THREADS) {
            const int v = e / CH_NB, p = e % CH_NB;
            xk[v][p] = p < kk ? __ldcg(&X0[v * vs + (K0 + p) * xs]) : T(0);
        }
        __syncthreads();
        // each block's 16 products summed on their own, then added to the
        // running sum: (16 + blocks) roundings per row instead of 16 * blocks
        // (this matters for the FP32 solves of the refinement)
#pragma unroll
        for (int v = 0; v < CH_MAXV; ++v) {
            if (v < nvec) {
                T blk = T(0);
#pragma unroll 4
                for (int p = q * 16; p < q * 16 + 16; ++p) blk = fma(Mb[p][r], xk[v][p], blk);
                acc[v] += blk;
            }
        }
        __syncthreads();                                   // Mb and xk are restaged next
    }
#pragma unroll
    for (int v = 0; v < CH_MAXV; ++v) part[q][v][r] = acc[v];
    __syncthreads();
    const int warp = tid >> 5, lane = tid & 31;
    if (warp < nvec) {
        const int v = warp;
        T *x = X0 + v * vs + (long long)R0 * xs;
        auto rhs = [&](int rr) -> T {
            if (rr >= kb) return T(0);
            return x[rr * xs] - ((part[0][v][rr] + part[1][v][rr]) + (part[2][v][rr] + part[3][v][rr]));
        };
        T x0 = rhs(lane), x1 = rhs(lane + 32);
        for (int st = 0; st < kb; ++st) {
            const int i = LOWER ? st : kb - 1 - st;
            T xi = __shfl_sync(0xffffffffu, i < 32 ? x0 : x1, i & 31);
            if (!UNIT) xi *= rinv[i];
            if (lane == (i & 31)) {
                if (i < 32) x0 = xi;
                else x1 = xi;
            }
            const int r1 = lane + 32;
            if (LOWER) {
                if (lane > i && lane < kb) x0 = fma(-Md[i][lane], xi, x0);
                if (r1 > i && r1 < kb) x1 = fma(-Md[i][r1], xi, x1);
            } else {
                if (lane < i) x0 = fma(-Md[i][lane], xi, x0);
                if (r1 < i) x1 = fma(-Md[i][r1], xi, x1);
            }
        }
        if (lane < kb) x[lane * xs] = x0;
        if (lane + 32 < kb) x[(lane + 32) * xs] = x1;
    }
    __syncthreads();
    if (tid == 0) ch_release(&flags[s], epoch);
}

// Returns kErrUnsupported when the chained solve does not apply (too many
// blocks to keep resident, or more than the flag array holds).
template <typename T>
int launch_chain(int ka, const T *M0, long long mi, long long mp, bool lowerM, bool unit, T *X0,
                 long long xs, long long vs, int nvec, cudaStream_t stream,
                 const ChainFixed *fx) {
    const int nblk = ceil_div(ka, CH_NB);
    static int per_sm = -1;
    if (per_sm < 0) {
        int bps = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, trsv_chain_kernel<T, true, false>,
                                                          CH_THREADS, 0) != cudaSuccess) {
            cudaGetLastError();
            bps = 0;
        }
        per_sm = bps;
    }
    if ((long long)per_sm * num_sms() < nblk) return kErrUnsupported;
    unsigned long long *flags = nullptr, epoch = 0;
    int *status = nullptr;
    if (fx) {
        // caller-supplied flags: cleared in stream order, one fixed epoch
        if (nblk > fx->cap) return kErrUnsupported;
        FG_CUDA(cudaMemsetAsync(fx->flags, 0, sizeof(unsigned long long) * nblk, stream));
        flags = fx->flags;
        epoch = 1;
        status = fx->status;
    } else {
        int st = workspace_flags(stream, nblk, &flags, &epoch);
        if (st != kOk) return st;
        Workspace *w = workspace_for(stream, 0);
        if (!w) return kErrAlloc;
        status = w->status;
    }
    // failure-detection test hook (flens_gb300_test_stall_next_chain)
    unsigned spin_limit = 0;
    int stall = 0;
    {
        const unsigned lim = g_stall_next_chain.exchange(0);
        if (lim) {
            spin_limit = lim;
            stall = 1;
        }
    }
    void *args[] = {&ka, &M0, &mi, &mp, &X0, &xs, &vs, &nvec, &flags, &epoch, &status,
                    &spin_limit, &stall};
    KTimer kt(kFamTrsv, stream, (double)ka * ka * nvec,
              (double)sizeof(T) * ka * (double)ka / 2.0 + 16.0 * ka * nvec);
    const void *fn;
    if (lowerM) fn = unit ? (const void *)trsv_chain_kernel<T, true, true>
                          : (const void *)trsv_chain_kernel<T, true, false>;
    else fn = unit ? (const void *)trsv_chain_kernel<T, false, true>
                   : (const void *)trsv_chain_kernel<T, false, false>;
    FG_CUDA(cudaLaunchCooperativeKernel(fn, dim3(nblk), dim3(CH_THREADS), args, 0, stream));
    return kOk;
}

// Chained solves on (FLENS_GB300_TRSV_CHAIN=0 turns them off).
bool chain_enabled() {
    static bool on = [] {
        const char *e = getenv("FLENS_GB300_TRSV_CHAIN");
        return !(e && atoi(e) == 0);
    }();
    return on;
}

template <typename T>
int launch_diag(int kb, const T *M0, long long mi, long long mp, bool lowerM, bool unit,
                T *X0, long long xs, long long vs, int nvec, cudaStream_t stream) {
    KTimer kt(kFamTrsm, stream, (double)kb * kb * nvec, 16.0 * (double)kb * nvec);
    if (nvec <= trsm_warp_max()) {
        const int grid = ceil_div(nvec, TRSM_WARP_VECS);
#define FG_WARP(L, U) trsm_diag_warp_kernel<T, L, U><<<grid, 32 * TRSM_WARP_VECS, 0, stream>>>(kb, M0, mi, mp, X0, xs, vs, nvec)
        if (lowerM) { if (unit) FG_WARP(true, true); else FG_WARP(true, false); }
        else { if (unit) FG_WARP(false, true); else FG_WARP(false, false); }
#undef FG_WARP
    } else {
        const int grid = ceil_div(nvec, TRSM_VPC);
#define FG_TILE(L, U) trsm_diag_tile_kernel<T, L, U><<<grid, TRSM_THREADS, 0, stream>>>(kb, M0, mi, mp, X0, xs, vs, nvec)
        if (lowerM) { if (unit) FG_TILE(true, true); else FG_TILE(true, false); }
        else { if (unit) FG_TILE(false, true); else FG_TILE(false, false); }
#undef FG_TILE
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
                  T alpha, const T *A, int ldA, T *B, int ldB, cudaStream_t stream,
                  const ChainFixed *fx = nullptr) {
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
    bool done = false;
    if (nvec <= CH_MAXV && nblk >= 2 && chain_enabled()) {
        const int st = launch_chain<T>(ka, A, mi, mp, lowerM, unit != 0, B, xs, vs, nvec, stream, fx);
        if (st == kOk) done = true;
        else if (st != kErrUnsupported) return st;
    }
    for (int s = 0; !done && s < nblk; ++s) {
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

int dtrsm_launch_fixed(char side, char upLo, char transA, char diag, int m, int n, double alpha,
                       const double *A, int ldA, double *B, int ldB, const ChainFixed &fx,
                       cudaStream_t stream) {
    return trsm_launch_t<double>(side, upLo, transA, diag, m, n, alpha, A, ldA, B, ldB, stream, &fx);
}

int strsm_launch(char side, char upLo, char transA, char diag, int m, int n, float alpha,
                 const float *A, int ldA, float *B, int ldB, cudaStream_t stream) {
    return trsm_launch_t<float>(side, upLo, transA, diag, m, n, alpha, A, ldA, B, ldB, stream);
}

}  // namespace fg

// Failure-detection test hook: the next chained triangular solve (trs and
// trsm with at most 4 right-hand sides against more than one 64-row block)
// makes its first block wait for a flag that nothing sets, bounded by
// `spin_limit` spins, so that every block gives up and the stream's status
// word reports FLENS_GB300_ERR_TIMEOUT at the next flens_gb300_sync.  No
// fault, trap or unbounded wait is involved: the kernel returns and the
// context stays usable.
FG_API void flens_gb300_test_stall_next_chain(unsigned spin_limit) {
    fg::g_stall_next_chain.store(spin_limit);
}
