// batched.cu -- thousands of independent, uneven-size LU factorisations and
// solves in one persistent launch, replayed through a CUDA graph.
//
// Per matrix the work is the reference's dgesv (flens/lapack/ge/sv.tcc:58-77:
// trf with partial pivoting -- first maximum wins, reciprocal scaling,
// INFO = first zero pivot -- then the row interchanges and the L and U
// solves of trs), done by a "team" of T threads of a persistent CTA:
//   * the plan sorts the matrices into size buckets, largest first; the
//     kernel walks the buckets in that order and, inside a bucket, the CTA
//     splits into 256/T teams that take matrices from the bucket's queue
//     (one atomic counter per bucket, no spin-waits);
//   * a matrix and its right-hand sides live in the team's share of shared
//     memory when they fit, otherwise the team works on them in place in
//     global memory (at these sizes, L2-resident);
//   * T per bucket comes from the autotuner below (candidates timed on
//     synthetic matrices of the bucket, cached per device);
//   * precision 0 = FP64; 1 = FP32 LU + FP64 iterative refinement (A
//     untouched; r = b - A x in FP64 from global A; stop at a normwise
//     backward error <= n*eps64, when a step fails to halve it
//     (flens/lapack/ge/rfs.tcc:182-188) or after max_iter steps).  The FP32
//     factors live in shared memory when they fit, otherwise in the plan's
//     pool (blocked LU); matrices with more than 32 right-hand sides are
//     solved in FP64 (iters = -1).  precision 2 = per matrix, precision 1
//     where it is faster than FP64 -- n >= 256 and nrhs <= n/64: the FP64
//     residuals of the refinement cost 3 n^2 nrhs FP64 FMAs, which the FP32
//     LU repays only for large n and few right-hand sides (measured on
//     homogeneous batches: n = 512, 1 rhs 16.6 against 23.6 ms; n = 300,
//     4 rhs 18.1 against 21.0 ms; n = 512, 16 rhs 28.7 against 26.1 ms;
//     n = 200, 4 rhs equal; n <= 100 up to 2.6x slower) -- and FP64
//     elsewhere (iters = -1).
#include "common.cuh"

#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <map>
#include <mutex>
#include <numeric>
#include <random>
#include <vector>

namespace fg {
namespace {

constexpr int BT_THREADS = 256;
constexpr size_t BT_SMEM = 216 * 1024;

// Size buckets (upper bounds of n).  108, 216, 432 and 864 are the largest n
// whose blocked factorisation fits a team's shared memory with 8, 4, 2 and 1
// teams per CTA (T = 32, 64, 128, 256), so a team size the tuner picks for a
// bucket keeps every matrix of the bucket off the unblocked global-memory path.
constexpr int BT_BUCKETS = 10;
constexpr int kBucketMax[BT_BUCKETS] = {16, 32, 48, 64, 108, 216, 320, 432, 864, INT_MAX};

inline int bucket_of(int n) {
    int b = 0;
    while (b < BT_BUCKETS - 1 && n > kBucketMax[b]) ++b;
    return b;
}

__host__ __device__ inline size_t team_share(int T) { return (BT_SMEM / (BT_THREADS / T)) / 16 * 16; }

struct BatchArgs {
    int beg[BT_BUCKETS], end[BT_BUCKETS];   // ranges of `order` per bucket
    int team[BT_BUCKETS];                   // threads per team per bucket
    int panel[BT_BUCKETS];                  // panel width of the blocked path (8 or 16)
    const int *order;
    const int *n, *nrhs, *lda, *ldb;
    double *const *A;
    double *const *B;
    int *const *ipiv;
    int *info;
    int *iters;
    double *berr;
    int *queue;                             // [BT_BUCKETS], zeroed before each launch
    int precision;
    int max_iter;
    // precision 1, matrices beyond the team's shared memory: FP32 factors and
    // FP64 refinement vectors in a plan-owned pool, one slot per team
    void *mx_pool;
    size_t mx_stride;                       // bytes per slot
    int mx_teams;                           // slots per CTA (CTA b owns b*mx_teams..)
};

__device__ __forceinline__ void team_sync(int id, int nthreads) {
    if (nthreads == 32) __syncwarp();
    else asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// Pivot keys as integers (|x| orders like its bits; NaN below every number,
// 0 = no candidate), so the search stays off the FP64 pipe.  (key, row)
// "better than": larger key, on equal keys the smaller row -- cxxblas
// iamax's first maximum (cxxblas/level1/iamax.tcc:52-56).
__device__ __forceinline__ unsigned long long pivot_key(double x) {
    const unsigned long long a = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
    return a > 0x7ff0000000000000ull ? 1ull : a + 2ull;
}

__device__ __forceinline__ bool better(unsigned long long k1, int i1, unsigned long long k2, int i2) {
    return k1 > k2 || (k1 == k2 && i1 < i2);
}

// argmax over the warp with redux.sync (all 32 lanes call it)
__device__ __forceinline__ void warp_argmax(unsigned long long &k, int &i) {
    const unsigned hi = (unsigned)(k >> 32), lo = (unsigned)k;
    const unsigned mhi = __reduce_max_sync(0xffffffffu, hi);
    const unsigned mlo = __reduce_max_sync(0xffffffffu, hi == mhi ? lo : 0u);
    const unsigned cand = (hi == mhi && lo == mlo) ? (unsigned)i : 0xffffffffu;
    i = (int)__reduce_min_sync(0xffffffffu, cand);
    k = ((unsigned long long)mhi << 32) | mlo;
}

// The pivot of column j (iamax's first maximum over the team's candidates,
// element j itself when it is NaN) with its value and, when |pivot| >=
// DBL_MIN, its reciprocal (tf2.tcc:101-121).  Warp 0 reduces the warps'
// candidates and divides once between the two team barriers, instead of
// every warp repeating the FP64 division.  col = column j, rows from 0.
// Reduction slots: red_k/red_v[0..7] candidates, red_v[8..9] pivot value
// and reciprocal, red_i[8] pivot row (red_k aliases red_v).
template <typename S>
__device__ void team_pivot(unsigned long long k, int i, const S *col, int j, int lt, int T, int bar,
                           unsigned long long *red_k, int *red_i, int &p, double &pv,
                           double &rinv) {
    double *red_v = (double *)red_k;
    warp_argmax(k, i);
    if (T == 32) {
        p = isnan((double)col[j]) ? j : i;
        pv = (double)col[p];
        rinv = fabs(pv) >= DBL_MIN ? 1.0 / pv : 0.0;
        return;
    }
    if ((lt & 31) == 0) { red_k[lt >> 5] = k; red_i[lt >> 5] = i; }
    team_sync(bar, T);
    if (lt < 32) {
        unsigned long long kk = lt < (T >> 5) ? red_k[lt] : 0ull;
        int ii = lt < (T >> 5) ? red_i[lt] : INT_MAX;
        warp_argmax(kk, ii);
        if (lt == 0) {
            const int pp = isnan((double)col[j]) ? j : ii;
            const double v = (double)col[pp];
            red_i[8] = pp;
            red_v[8] = v;
            red_v[9] = fabs(v) >= DBL_MIN ? 1.0 / v : 0.0;
        }
    }
    team_sync(bar, T);
    p = red_i[8];
    pv = red_v[8];
    rinv = red_v[9];
}

__device__ double team_max(double m, int lt, int T, int bar, double *red) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, off));
    if (T == 32) return m;
    if ((lt & 31) == 0) red[lt >> 5] = m;
    team_sync(bar, T);
    m = red[0];
    for (int q = 1; q < (T >> 5); ++q) m = fmax(m, red[q]);
    team_sync(bar, T);
    return m;
}

template <typename S>
__device__ void team_trs(int n, int k, const S *M, int ldm, S *X, int ldx, const int *piv, int lt,
                         int T, int bar);

// LU with partial pivoting of the n x n matrix M (storage S): pivot search
// and scaling in FP64, the rank-1 updates in S.  If INFO == 0 the k columns
// of X are then overwritten by U^-1 L^-1 P X; X is untouched otherwise.
template <typename S>
__device__ int team_gesv(int n, int k, S *M, int ldm, S *X, int ldx, int *piv, int lt, int T,
                         int bar, double *red_v, int *red_i) {
    unsigned long long *red_k = (unsigned long long *)red_v;
    int info = 0;
    for (int j = 0; j < n; ++j) {
        unsigned long long bv = 0ull;
        int bi = INT_MAX;
        for (int r = j + lt; r < n; r += T) {
            const unsigned long long key = pivot_key((double)M[r + (size_t)j * ldm]);
            if (better(key, r, bv, bi)) { bv = key; bi = r; }
        }
        int p;
        double pv, rinv;
        team_pivot<S>(bv, bi, M + (size_t)j * ldm, j, lt, T, bar, red_k, red_i, p, pv, rinv);
        if (lt == 0) piv[j] = p + 1;
        if (pv != 0.0) {
            if (p != j) {
                for (int c = lt; c < n; c += T) {
                    const S t = M[j + (size_t)c * ldm];
                    M[j + (size_t)c * ldm] = M[p + (size_t)c * ldm];
                    M[p + (size_t)c * ldm] = t;
                }
                team_sync(bar, T);
            }
            const bool recip = fabs(pv) >= DBL_MIN;
            for (int r = j + 1 + lt; r < n; r += T) {
                const double l = (double)M[r + (size_t)j * ldm];
                M[r + (size_t)j * ldm] = (S)(recip ? l * rinv : l / pv);
            }
        } else if (info == 0) {
            info = j + 1;
        }
        team_sync(bar, T);
        // rank-1 update of the R x R block below and right of (j, j)
        const int R = n - 1 - j;
        if (R > 0 && __isShared(M)) {
            // in shared memory: the team walks the block in column-major
            // element order (consecutive lanes on consecutive rows), so
            // lanes idle only in its last T elements -- lanes mapped to rows
            // 32 apart left up to 31 idle per column
            const int total = R * R, dr = T % R, dc = T / R;
            S *Mb = M + (j + 1) + (size_t)(j + 1) * ldm;
            const S *lcol = M + (j + 1) + (size_t)j * ldm;
            const S *urow = M + j + (size_t)(j + 1) * ldm;
            int r = lt % R, c = lt / R;
            for (int e = lt; e < total; e += T) {
                Mb[r + (size_t)c * ldm] = fma(-urow[(size_t)c * ldm], lcol[r], Mb[r + (size_t)c * ldm]);
                r += dr;
                c += dc;
                if (r >= R) { r -= R; ++c; }
            }
        } else {
            // in global memory: lane -> rows (32 apart), warp -> columns
            // (T/32 apart), the row's multiplier loaded once
            const int tr = lt & 31, tc = lt >> 5, TC = T >> 5;
            for (int r = j + 1 + tr; r < n; r += 32) {
                const S l = M[r + (size_t)j * ldm];
                for (int c = j + 1 + tc; c < n; c += TC)
                    M[r + (size_t)c * ldm] = fma(-M[j + (size_t)c * ldm], l, M[r + (size_t)c * ldm]);
            }
        }
        team_sync(bar, T);
    }
    if (info != 0) return info;
    team_trs<S>(n, k, M, ldm, X, ldx, piv, lt, T, bar);
    return 0;
}

// X <- U^-1 L^-1 P X with the factors and pivots of a team LU (trs.tcc:84
// interchanges, then the unit lower and the upper solve)
template <typename S>
__device__ void team_trs(int n, int k, const S *M, int ldm, S *X, int ldx, const int *piv, int lt,
                         int T, int bar) {
    for (int j = 0; j < n; ++j) {                          // interchanges (trs.tcc:84)
        const int p = piv[j] - 1;
        if (p != j) {
            for (int c = lt; c < k; c += T) {
                const S t = X[j + (size_t)c * ldx];
                X[j + (size_t)c * ldx] = X[p + (size_t)c * ldx];
                X[p + (size_t)c * ldx] = t;
            }
            team_sync(bar, T);
        }
    }
    for (int i = 0; i < n; ++i) {                          // unit lower
        for (int c = 0; c < k; ++c)
            for (int r = i + 1 + lt; r < n; r += T)
                X[r + (size_t)c * ldx] = fma(-M[r + (size_t)i * ldm], X[i + (size_t)c * ldx], X[r + (size_t)c * ldx]);
        team_sync(bar, T);
    }
    for (int i = n - 1; i >= 0; --i) {                     // upper
        for (int c = lt; c < k; c += T) X[i + (size_t)c * ldx] = X[i + (size_t)c * ldx] / M[i + (size_t)i * ldm];
        team_sync(bar, T);
        for (int c = 0; c < k; ++c)
            for (int r = lt; r < i; r += T)
                X[r + (size_t)c * ldx] = fma(-M[r + (size_t)i * ldm], X[i + (size_t)c * ldx], X[r + (size_t)c * ldx]);
        team_sync(bar, T);
    }
}

// Blocked form of team_gesv's factorisation for a matrix that stays in
// global memory: NB-column panels factored in shared memory, their
// interchanges applied to the other columns, U12 by forward substitution and
// the trailing matrix updated once per panel (instead of once per column).
// Every element receives the same FMAs in the same order as in the
// unblocked loop, so the factors and pivots are bitwise the same, whatever
// the panel width NB (8 or 16, picked per size bucket by the tuner; 4-column
// panels measured 10-17% slower than 8 at n = 200..480).
// Shared memory: P (n x NB) and U12 (NB x n) doubles.

// dst(0:rows, 0:cols) = src(0:rows, 0:cols), column-major, eight columns'
// loads issued before their stores (a load after a store through another
// pointer would otherwise wait for the previous load's round trip)
template <typename S>
__device__ __forceinline__ void team_copy_cols(int rows, int cols, const S *__restrict__ src,
                                               int lds, S *__restrict__ dst, int ldd, int lt,
                                               int T) {
    for (int c0 = 0; c0 < cols; c0 += 8)
        for (int r = lt; r < rows; r += T) {
            S v[8];
#pragma unroll
            for (int cc = 0; cc < 8; ++cc)
                if (c0 + cc < cols) v[cc] = src[r + (size_t)(c0 + cc) * lds];
#pragma unroll
            for (int cc = 0; cc < 8; ++cc)
                if (c0 + cc < cols) dst[r + (size_t)(c0 + cc) * ldd] = v[cc];
        }
}

__host__ __device__ inline size_t blocked_need(int n, int nb, size_t elem = sizeof(double)) {
    return (size_t)2 * n * nb * elem;
}

template <typename S, int BNB>
__device__ int team_lu_blocked(int n, S *M, int ldm, int *piv, int lt, int T, int bar,
                               double *red_v, int *red_i, S *sm) {
    unsigned long long *red_k = (unsigned long long *)red_v;
    S *P = sm, *U = sm + (size_t)n * BNB;
    int info = 0;
    for (int j0 = 0; j0 < n; j0 += BNB) {
        const int jb = min(BNB, n - j0), mp = n - j0;
        // panel rows j0.. of columns j0..j0+jb into P (ld mp)
        team_copy_cols(mp, jb, M + j0 + (size_t)j0 * ldm, ldm, P, mp, lt, T);
        team_sync(bar, T);
        // pivot keys of the panel's first column; later columns' keys come
        // out of the previous column's update, whose rows each thread owns
        unsigned long long bv = 0ull;
        int bi = INT_MAX;
        for (int r = lt; r < mp; r += T) {
            const unsigned long long key = pivot_key((double)P[r]);
            if (better(key, r, bv, bi)) { bv = key; bi = r; }
        }
        int *spiv = (int *)U;                   // the panel's pivots (U is free until U12)
        for (int jj = 0; jj < jb; ++jj) {
            int p;
            double pv, rinv;
            team_pivot<S>(bv, bi, P + jj * mp, jj, lt, T, bar, red_k, red_i, p, pv, rinv);
            if (lt == 0) {
                piv[j0 + jj] = j0 + p + 1;
                spiv[jj] = p;
            }
            const bool nz = pv != 0.0;
            if (nz && p != jj) {
                for (int c = lt; c < jb; c += T) {
                    const S t = P[jj + c * mp];
                    P[jj + c * mp] = P[p + c * mp];
                    P[p + c * mp] = t;
                }
                team_sync(bar, T);
            }
            if (!nz && info == 0) info = j0 + jj + 1;
            // scaling (a zero pivot leaves the column as it is), the rank-1
            // update and the next column's keys, row by row: the rows a
            // thread scales are the rows it updates
            const bool recip = fabs(pv) >= DBL_MIN;
            bv = 0ull;
            bi = INT_MAX;
            for (int r = jj + 1 + lt; r < mp; r += T) {
                S l = P[r + jj * mp];
                if (nz) {                       // scaled in FP64, stored in S
                    const double d = (double)l;
                    l = (S)(recip ? d * rinv : d / pv);
                    P[r + jj * mp] = l;
                }
                for (int c = jj + 1; c < jb; ++c) P[r + c * mp] = fma(-P[jj + c * mp], l, P[r + c * mp]);
                if (jj + 1 < jb) {
                    const unsigned long long key = pivot_key((double)P[r + (jj + 1) * mp]);
                    if (better(key, r, bv, bi)) { bv = key; bi = r; }
                }
            }
            team_sync(bar, T);
        }
        for (int c = 0; c < jb; ++c)
            for (int r = lt; r < mp; r += T) M[(j0 + r) + (size_t)(j0 + c) * ldm] = P[r + c * mp];
        // the panel's interchanges on the columns left and right of it: a
        // thread per column applies the jb swaps in order (no barrier
        // between swaps; pivots from shared memory)
        for (int c = lt; c < n - jb; c += T) {
            S *a = M + (size_t)(c < j0 ? c : c + jb) * ldm;
            for (int jj = 0; jj < jb; ++jj) {
                const int p = j0 + spiv[jj];
                if (p != j0 + jj) {
                    const S t = a[j0 + jj];
                    a[j0 + jj] = a[p];
                    a[p] = t;
                }
            }
        }
        team_sync(bar, T);
        const int nr = n - j0 - jb;
        if (nr > 0) {
            // U12 = L11^-1 A12, a thread per column, rows in the unblocked
            // loop's order; kept in U (ld BNB) and written back
            for (int c = lt; c < nr; c += T) {
                S u[BNB];
#pragma unroll
                for (int q = 0; q < BNB; ++q) u[q] = q < jb ? M[(j0 + q) + (size_t)(j0 + jb + c) * ldm] : S(0);
#pragma unroll
                for (int q = 0; q < BNB; ++q) {
#pragma unroll
                    for (int pp = q + 1; pp < BNB; ++pp)
                        if (pp < jb) u[pp] = fma(-u[q], P[pp + q * mp], u[pp]);
                }
#pragma unroll
                for (int q = 0; q < BNB; ++q) {
                    if (q < jb) {
                        U[q + (size_t)c * BNB] = u[q];
                        M[(j0 + q) + (size_t)(j0 + jb + c) * ldm] = u[q];
                    }
                }
            }
            team_sync(bar, T);
            // trailing update of the R x nr block in column-major element
            // order: thread lt takes elements lt, lt + T, ... (consecutive
            // lanes on consecutive rows), so lanes idle only in the block's
            // last T elements (lanes mapped to rows 32 apart left up to 31
            // of them idle in every column's last row group).  Two elements
            // (two independent FMA chains) per step; the next step's two are
            // loaded before this step's FMAs so that their L2 round trip
            // overlaps the FMA work.  nr > 0 implies jb == BNB.
            {
                const int R = mp - jb, total = R * nr;
                const int dr = T % R, dc = T / R;
                S *Mb = M + (j0 + jb) + (size_t)(j0 + jb) * ldm;
                const S *Pl = P + jb;
                int r0 = lt % R, c0 = lt / R;          // element e
                int r1 = r0 + dr, c1 = c0 + dc;        // element e + T
                if (r1 >= R) { r1 -= R; ++c1; }
                S n0 = lt < total ? Mb[r0 + (size_t)c0 * ldm] : S(0);
                S n1 = lt + T < total ? Mb[r1 + (size_t)c1 * ldm] : S(0);
                for (int e = lt; e < total; e += 2 * T) {
                    const int ra = r0, ca = c0, rb = r1, cb = c1;
                    S a0 = n0, a1 = n1;
                    r0 = r1 + dr;                      // elements e + 2T, e + 3T
                    c0 = c1 + dc;
                    if (r0 >= R) { r0 -= R; ++c0; }
                    r1 = r0 + dr;
                    c1 = c0 + dc;
                    if (r1 >= R) { r1 -= R; ++c1; }
                    if (e + 2 * T < total) n0 = Mb[r0 + (size_t)c0 * ldm];
                    if (e + 3 * T < total) n1 = Mb[r1 + (size_t)c1 * ldm];
                    if (e + T < total) {
#pragma unroll
                        for (int q = 0; q < BNB; ++q) {
                            a0 = fma(-U[q + (size_t)ca * BNB], Pl[ra + q * mp], a0);
                            a1 = fma(-U[q + (size_t)cb * BNB], Pl[rb + q * mp], a1);
                        }
                        Mb[ra + (size_t)ca * ldm] = a0;
                        Mb[rb + (size_t)cb * ldm] = a1;
                    } else {
#pragma unroll
                        for (int q = 0; q < BNB; ++q) a0 = fma(-U[q + (size_t)ca * BNB], Pl[ra + q * mp], a0);
                        Mb[ra + (size_t)ca * ldm] = a0;
                    }
                }
            }
            team_sync(bar, T);
        }
    }
    return info;
}

// X <- U^-1 L^-1 P X for FP64 factors that stay in global memory (the
// blocked path): the n x k right-hand sides are staged in shared memory and
// both triangles are solved in 32-row blocks -- the diagonal block by a warp
// per column (lane = row, shuffles instead of barriers), the rows beyond it by
// one coalesced pass over the block's columns of the factor.  Each element
// receives the same FMAs and divisions in the same order as in team_trs (the
// unit lower solve in ascending, the upper in descending column order), so
// the solutions are bitwise those of the row-at-a-time loop, which spent a
// team barrier and an L2 round trip per row.
// Shared memory: X (n x k) and one 32 x 32 block of the factor.
constexpr int SNB = 32;

__device__ size_t staged_need(int n, int k, size_t elem = sizeof(double)) {
    return ((size_t)n * k + SNB * SNB) * elem;
}

// rows [r0, r1) of X (ld n, columns c0..c0+KC) minus the factor's columns
// i0..i0+ib times the solved block rows of X, in ascending (lower) or
// descending (upper) column order
template <typename S, int KC, bool DESC>
__device__ __forceinline__ void staged_rows_update(int r0, int r1, int i0, int ib, int c0, int k,
                                                   const S *__restrict__ M, int ldm,
                                                   S *X, int n, int lt, int T) {
    for (int r = r0 + lt; r < r1; r += T) {
        S acc[KC];
#pragma unroll
        for (int cc = 0; cc < KC; ++cc) acc[cc] = c0 + cc < k ? X[r + (size_t)(c0 + cc) * n] : S(0);
        const S *mrow = M + r;
#pragma unroll 8
        for (int s = 0; s < ib; ++s) {
            const int q = DESC ? ib - 1 - s : s;
            const S l = mrow[(size_t)(i0 + q) * ldm];
#pragma unroll
            for (int cc = 0; cc < KC; ++cc)
                if (c0 + cc < k) acc[cc] = fma(-l, X[(i0 + q) + (size_t)(c0 + cc) * n], acc[cc]);
        }
#pragma unroll
        for (int cc = 0; cc < KC; ++cc)
            if (c0 + cc < k) X[r + (size_t)(c0 + cc) * n] = acc[cc];
    }
}

template <typename S, int KC>
__device__ void staged_update_all(bool upper, int r0, int r1, int i0, int ib, int k, const S *M,
                                  int ldm, S *X, int n, int lt, int T) {
    for (int c0 = 0; c0 < k; c0 += KC) {
        if (upper) staged_rows_update<S, KC, true>(r0, r1, i0, ib, c0, k, M, ldm, X, n, lt, T);
        else staged_rows_update<S, KC, false>(r0, r1, i0, ib, c0, k, M, ldm, X, n, lt, T);
    }
}

// x(0:ib) <- U^-1 x(0:ib) for the ib x ib upper block D (ld SNB), one
// column, rows from the bottom: per element the FMAs of the rows below in
// descending order, then the division (the order of team_trs's upper solve)
template <typename S>
__device__ __forceinline__ void upper_block_by_column(S *__restrict__ xc, const S *__restrict__ D,
                                                      int ib) {
    for (int q = ib - 1; q >= 0; --q) {
        const S xq = xc[q] / D[q + q * SNB];
        xc[q] = xq;
#pragma unroll 4
        for (int r = 0; r < q; ++r) xc[r] = fma(-D[r + q * SNB], xq, xc[r]);
    }
}

template <typename S>
__device__ void team_trs_staged(int n, int k, const S *M, int ldm, S *B, int ldb,
                                const int *piv, int lt, int T, int bar, S *sm) {
    S *X = sm, *Dg = sm + (size_t)n * k;
    const int lane = lt & 31, warp = lt >> 5, nw = T >> 5;
    team_copy_cols(n, k, B, ldb, X, n, lt, T);
    team_sync(bar, T);
    // interchanges in the order of trs.tcc:84: warp 0 reads 32 pivots at a
    // time and applies the swaps among them in order, a lane per column
    if (warp == 0) {
        for (int j0 = 0; j0 < n; j0 += 32) {
            const int j = j0 + lane;
            const int p = j < n ? piv[j] - 1 : j;
            unsigned m = __ballot_sync(0xffffffffu, p != j);
            while (m) {
                const int bit = __ffs(m) - 1;
                m &= m - 1;
                const int jj = j0 + bit, pj = __shfl_sync(0xffffffffu, p, bit);
                for (int c = lane; c < k; c += 32) {
                    S *x = X + (size_t)c * n;
                    const S t = x[jj];
                    x[jj] = x[pj];
                    x[pj] = t;
                }
            }
        }
    }
    for (int pass = 0; pass < 2; ++pass) {
        const bool upper = pass == 1;
        for (int b = 0; b < n; b += SNB) {
            // lower: blocks from the top; upper: from the bottom
            const int i0 = upper ? max(0, n - b - SNB) : b;
            const int ib = upper ? n - b - i0 : min(SNB, n - b);
            team_sync(bar, T);
            for (int e0 = lt; e0 < SNB * SNB; e0 += 4 * T) {
                S v[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int e = e0 + u * T, r = e & (SNB - 1), q = e >> 5;
                    v[u] = e < SNB * SNB && r < ib && q < ib ? M[(i0 + r) + (size_t)(i0 + q) * ldm] : S(0);
                }
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (e0 + u * T < SNB * SNB) Dg[e0 + u * T] = v[u];
            }
            team_sync(bar, T);
            if (upper && k >= 3) {
                // a thread per column: each row's division is one instruction
                // sequence for all k columns, where a warp per column spent a
                // whole warp's FP64 slots on every one-lane division
                for (int c = lt; c < k; c += T)
                    upper_block_by_column(X + (size_t)c * n + i0, Dg, ib);
            } else {
                for (int c = warp; c < k; c += nw) {
                    S *xc = X + (size_t)c * n + i0;
                    S x = lane < ib ? xc[lane] : S(0);
                    if (!upper) {
                        for (int q = 0; q < ib - 1; ++q) {
                            const S xq = __shfl_sync(0xffffffffu, x, q);
                            if (lane > q) x = fma(-Dg[lane + q * SNB], xq, x);
                        }
                    } else {
                        for (int q = ib - 1; q >= 0; --q) {
                            if (lane == q) x = x / Dg[q + q * SNB];
                            const S xq = __shfl_sync(0xffffffffu, x, q);
                            if (lane < q) x = fma(-Dg[lane + q * SNB], xq, x);
                        }
                    }
                    if (lane < ib) xc[lane] = x;
                }
            }
            team_sync(bar, T);
            const int r0 = upper ? 0 : i0 + ib, r1 = upper ? i0 : n;
            if (r0 < r1) {
                if (k == 1) staged_update_all<S, 1>(upper, r0, r1, i0, ib, k, M, ldm, X, n, lt, T);
                else if (k <= 4) staged_update_all<S, 4>(upper, r0, r1, i0, ib, k, M, ldm, X, n, lt, T);
                else staged_update_all<S, 8>(upper, r0, r1, i0, ib, k, M, ldm, X, n, lt, T);
            }
        }
    }
    team_sync(bar, T);
    team_copy_cols(n, k, X, n, B, ldb, lt, T);
    team_sync(bar, T);
}

// X <- U^-1 L^-1 P X with the FP32 factors in M (the pivots of team_gesv)
__device__ void team_lu_solve32(int n, int k, const float *M, const int *piv, float *X, int lt,
                                int T, int bar) {
    for (int j = 0; j < n; ++j) {
        const int p = piv[j] - 1;
        if (p != j) {
            for (int c = lt; c < k; c += T) {
                const float t = X[j + (size_t)c * n];
                X[j + (size_t)c * n] = X[p + (size_t)c * n];
                X[p + (size_t)c * n] = t;
            }
            team_sync(bar, T);
        }
    }
    for (int i = 0; i < n; ++i) {
        for (int c = 0; c < k; ++c)
            for (int r = i + 1 + lt; r < n; r += T) X[r + (size_t)c * n] -= M[r + (size_t)i * n] * X[i + (size_t)c * n];
        team_sync(bar, T);
    }
    for (int i = n - 1; i >= 0; --i) {
        for (int c = lt; c < k; c += T) X[i + (size_t)c * n] /= M[i + (size_t)i * n];
        team_sync(bar, T);
        for (int c = 0; c < k; ++c)
            for (int r = lt; r < i; r += T) X[r + (size_t)c * n] -= M[r + (size_t)i * n] * X[i + (size_t)c * n];
        team_sync(bar, T);
    }
}

__host__ __device__ inline size_t fp64_need(int n, int k) { return ((size_t)n * n + (size_t)n * k) * 8; }
// FP32 M and D, FP64 saved b and residual
__host__ __device__ inline size_t mixed_need(int n, int k) {
    return (size_t)n * n * 4 + (size_t)n * k * (4 + 8 + 8);
}
// pool slot of the blocked mixed path: FP32 factors, then saved b and the
// residual (FP64) and the FP32 corrections, n x k each
__host__ __device__ inline size_t mx_factor_bytes(int n) { return ((size_t)n * n * 4 + 255) / 256 * 256; }
__host__ __device__ inline size_t mx_need(int n, int k) {
    return mx_factor_bytes(n) + (size_t)n * k * (8 + 8 + 4);
}

__device__ void solve_fp64(const BatchArgs &a, int idx, unsigned char *sm, size_t share, int nb,
                           int lt, int T, int bar, double *rv, int *ri) {
    const int n = a.n[idx], k = a.nrhs[idx], lda = a.lda[idx], ldb = a.ldb[idx];
    double *A = a.A[idx], *B = a.B[idx];
    int info;
    if (fp64_need(n, k) <= share) {
        double *M = (double *)sm, *X = M + (size_t)n * n;
        for (int e = lt; e < n * n; e += T) M[e] = A[e % n + (size_t)(e / n) * lda];
        for (int e = lt; e < n * k; e += T) X[e] = B[e % n + (size_t)(e / n) * ldb];
        team_sync(bar, T);
        info = team_gesv<double>(n, k, M, n, X, n, a.ipiv[idx], lt, T, bar, rv, ri);
        for (int e = lt; e < n * n; e += T) A[e % n + (size_t)(e / n) * lda] = M[e];
        if (info == 0)
            for (int e = lt; e < n * k; e += T) B[e % n + (size_t)(e / n) * ldb] = X[e];
    } else if (blocked_need(n, nb) <= share) {
        // in place in global memory, blocked (panels in shared memory)
        double *ps = (double *)sm;
        info = nb == 8 ? team_lu_blocked<double, 8>(n, A, lda, a.ipiv[idx], lt, T, bar, rv, ri, ps)
                       : team_lu_blocked<double, 16>(n, A, lda, a.ipiv[idx], lt, T, bar, rv, ri, ps);
        if (info == 0) {
            if (staged_need(n, k) <= share)
                team_trs_staged<double>(n, k, A, lda, B, ldb, a.ipiv[idx], lt, T, bar, (double *)sm);
            else
                team_trs<double>(n, k, A, lda, B, ldb, a.ipiv[idx], lt, T, bar);
        }
    } else {
        info = team_gesv<double>(n, k, A, lda, B, ldb, a.ipiv[idx], lt, T, bar, rv, ri);
    }
    if (lt == 0) {
        a.info[idx] = info;
        if (a.iters) a.iters[idx] = -1;
        if (a.berr) a.berr[idx] = 0.0;
    }
    team_sync(bar, T);
}

// FP64 iterative refinement of the k solutions of A X = B (A, B in FP64,
// global): the first FP32 solution is in D (n x k, ld n); b is saved in Bs
// and the residuals go to Rr (FP64, ld n).  solve32() overwrites D with the
// FP32 factors' solution of D.  Stops per column at a normwise backward error
// <= n*eps64, when a step fails to halve it (flens/lapack/ge/rfs.tcc:182-188)
// or after max_iter steps.
template <typename Solve32>
__device__ void refine_fp64(const BatchArgs &a, int idx, const double *A, int lda, double *B,
                            int ldb, const double *Bs, double *Rr, float *D, int n, int k, int lt,
                            int T, int bar, double *rv, Solve32 solve32) {
    // x0 (FP64) lives in B from here on
    for (int e = lt; e < n * k; e += T) B[e % n + (size_t)(e / n) * ldb] = (double)D[e];
    double anorm = 0.0, worst = 0.0;
    for (int r = lt; r < n; r += T) {
        // eight loads in flight, summed in column order
        double s = 0.0;
        int c = 0;
        for (; c + 8 <= n; c += 8) {
            double v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) v[u] = A[r + (size_t)(c + u) * lda];
#pragma unroll
            for (int u = 0; u < 8; ++u) s += fabs(v[u]);
        }
        for (; c < n; ++c) s += fabs(A[r + (size_t)c * lda]);
        anorm = fmax(anorm, s);
    }
    anorm = team_max(anorm, lt, T, bar, rv);
    int steps = 0;
    unsigned done = 0;                  // bit c: column c finished (k <= 32)
    double prev[32];
    for (int c = 0; c < k && c < 32; ++c) prev[c] = INFINITY;
    for (int it = 0; it <= a.max_iter; ++it) {
        team_sync(bar, T);
        // r = b - A x, FP64: a thread takes one row and up to four columns,
        // so each element of A (from L2) is loaded once for four FMAs, with
        // eight loads in flight; every sum runs over q in order
        const int ng = (k + 3) / 4;
        for (int e = lt; e < n * ng; e += T) {
            const int r = e % n, c0 = (e / n) * 4, nc = min(4, k - c0);
            double s[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) s[u] = u < nc ? Bs[r + (size_t)(c0 + u) * n] : 0.0;
            int q = 0;
            for (; q + 8 <= n; q += 8) {
                double av[8];
#pragma unroll
                for (int v = 0; v < 8; ++v) av[v] = A[r + (size_t)(q + v) * lda];
#pragma unroll
                for (int v = 0; v < 8; ++v)
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        if (u < nc) s[u] = fma(-av[v], B[(q + v) + (size_t)(c0 + u) * ldb], s[u]);
            }
            for (; q < n; ++q) {
                const double a = A[r + (size_t)q * lda];
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (u < nc) s[u] = fma(-a, B[q + (size_t)(c0 + u) * ldb], s[u]);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (u < nc) Rr[r + (size_t)(c0 + u) * n] = s[u];
        }
        team_sync(bar, T);
        bool any = false;
        worst = 0.0;
        for (int c = 0; c < k; ++c) {
            double rm = 0.0, xm = 0.0, bm = 0.0;
            for (int r = lt; r < n; r += T) {
                rm = fmax(rm, fabs(Rr[r + (size_t)c * n]));
                xm = fmax(xm, fabs(B[r + (size_t)c * ldb]));
                bm = fmax(bm, fabs(Bs[r + (size_t)c * n]));
            }
            rm = team_max(rm, lt, T, bar, rv);
            xm = team_max(xm, lt, T, bar, rv);
            bm = team_max(bm, lt, T, bar, rv);
            const double den = anorm * xm + bm;
            const double be = den > 0.0 ? rm / den : (rm > 0.0 ? INFINITY : 0.0);
            worst = fmax(worst, be);
            const bool fin = (done >> c) & 1u;
            if (!fin && (be <= (double)n * DBL_EPSILON || !(be <= 0.5 * prev[c]) || it == a.max_iter))
                done |= 1u << c;
            prev[c] = be;
            // scaled residual into D (zero for finished columns)
            const bool go = !((done >> c) & 1u);
            any = any || go;
            const double sc = rm > 0.0 ? rm : 1.0;
            for (int r = lt; r < n; r += T) D[r + (size_t)c * n] = go ? (float)(Rr[r + (size_t)c * n] / sc) : 0.0f;
            if (lt == 0) Rr[(size_t)c * n] = go ? sc : 0.0;   // keep the scale in R(0, c)
        }
        team_sync(bar, T);
        if (!any) break;
        solve32();
        for (int e = lt; e < n * k; e += T) {
            const int c = e / n;
            const double sc = Rr[(size_t)c * n];
            if (sc != 0.0) B[e % n + (size_t)c * ldb] += sc * (double)D[e];
        }
        ++steps;
    }
    if (lt == 0) {
        a.info[idx] = 0;
        if (a.iters) a.iters[idx] = steps;
        if (a.berr) a.berr[idx] = worst;
    }
    team_sync(bar, T);
}

__device__ __noinline__ void solve_mixed(const BatchArgs &a, int idx, unsigned char *sm, int lt, int T, int bar,
                            double *rv, int *ri) {
    const int n = a.n[idx], k = a.nrhs[idx], lda = a.lda[idx], ldb = a.ldb[idx];
    const double *A = a.A[idx];
    double *B = a.B[idx];
    int *piv = a.ipiv[idx];
    double *Bs = (double *)sm;                         // n x k saved b (FP64)
    double *Rr = Bs + (size_t)n * k;                   // n x k residual (FP64)
    float *M = (float *)(Rr + (size_t)n * k);          // n x n FP32 factors
    float *D = M + (size_t)n * n;                      // n x k FP32 solves
    for (int e = lt; e < n * n; e += T) M[e] = (float)A[e % n + (size_t)(e / n) * lda];
    for (int e = lt; e < n * k; e += T) {
        const double v = B[e % n + (size_t)(e / n) * ldb];
        Bs[e] = v;
        D[e] = (float)v;
    }
    team_sync(bar, T);
    const int info = team_gesv<float>(n, k, M, n, D, n, piv, lt, T, bar, rv, ri);
    if (info != 0) {
        if (lt == 0) a.info[idx] = info;
        team_sync(bar, T);
        return;
    }
    refine_fp64(a, idx, A, lda, B, ldb, Bs, Rr, D, n, k, lt, T, bar, rv,
                [&]() { team_lu_solve32(n, k, M, piv, D, lt, T, bar); });
}

// The mixed variant for a matrix beyond the team's shared memory: FP32 copy
// of A factored in place in the team's pool slot by the blocked LU (FP32
// panels in shared memory, FP64 pivot search and scaling), the FP32 solves
// staged in shared memory, FP64 residuals from the untouched A.
// precision 2: the matrices for which FP32 LU + FP64 refinement is faster
__host__ __device__ inline bool mixed_pays(int n, int k) { return n >= 256 && 64 * k <= n; }

__device__ bool mixed_blocked_ok(const BatchArgs &a, int n, int k, int nb, int T, size_t share) {
    return a.mx_pool != nullptr && k <= 32 && BT_THREADS / T <= a.mx_teams &&
           mx_need(n, k) <= a.mx_stride && blocked_need(n, nb, sizeof(float)) <= share;
}

__device__ __noinline__ void solve_mixed_blocked(const BatchArgs &a, int idx, unsigned char *sm, size_t share,
                                    int nb, int slot, int lt, int T, int bar, double *rv,
                                    int *ri) {
    const int n = a.n[idx], k = a.nrhs[idx], lda = a.lda[idx], ldb = a.ldb[idx];
    const double *A = a.A[idx];
    double *B = a.B[idx];
    int *piv = a.ipiv[idx];
    char *base = (char *)a.mx_pool + (size_t)slot * a.mx_stride;
    float *F = (float *)base;                                  // n x n FP32 factors
    double *Bs = (double *)(base + mx_factor_bytes(n));        // n x k saved b
    double *Rr = Bs + (size_t)n * k;                           // n x k residual
    float *D = (float *)(Rr + (size_t)n * k);                  // n x k FP32 solves
    for (int c0 = 0; c0 < n; c0 += 8)                          // eight loads before their stores
        for (int r = lt; r < n; r += T) {
            double v[8];
#pragma unroll
            for (int cc = 0; cc < 8; ++cc)
                if (c0 + cc < n) v[cc] = A[r + (size_t)(c0 + cc) * lda];
#pragma unroll
            for (int cc = 0; cc < 8; ++cc)
                if (c0 + cc < n) F[r + (size_t)(c0 + cc) * n] = (float)v[cc];
        }
    for (int c = 0; c < k; ++c)
        for (int r = lt; r < n; r += T) {
            const double v = B[r + (size_t)c * ldb];
            Bs[r + (size_t)c * n] = v;
            D[r + (size_t)c * n] = (float)v;
        }
    team_sync(bar, T);
    float *ps = (float *)sm;
    const int info = nb == 8 ? team_lu_blocked<float, 8>(n, F, n, piv, lt, T, bar, rv, ri, ps)
                             : team_lu_blocked<float, 16>(n, F, n, piv, lt, T, bar, rv, ri, ps);
    if (info != 0) {
        if (lt == 0) a.info[idx] = info;
        team_sync(bar, T);
        return;
    }
    auto solve32 = [&]() {
        if (staged_need(n, k, sizeof(float)) <= share)
            team_trs_staged<float>(n, k, F, n, D, n, piv, lt, T, bar, ps);
        else
            team_trs<float>(n, k, F, n, D, n, piv, lt, T, bar);
    };
    solve32();
    refine_fp64(a, idx, A, lda, B, ldb, Bs, Rr, D, n, k, lt, T, bar, rv, solve32);
}

// MIXED: the precision-1 kernel (FP32 LU + FP64 refinement paths); the FP64
// kernel is compiled without them, so that their registers do not weigh on
// the FP64 paths.
template <bool MIXED>
__global__ void __launch_bounds__(BT_THREADS, 1)
batched_gesv_kernel(BatchArgs a) {
    extern __shared__ __align__(16) unsigned char bsm[];
    __shared__ double red_v[8][10];
    __shared__ int red_i[8][10];
    __shared__ int s_item[8];
    const int tid = threadIdx.x;
    for (int bk = BT_BUCKETS - 1; bk >= 0; --bk) {
        const int beg = a.beg[bk], end = a.end[bk];
        if (beg >= end) continue;
        const int T = a.team[bk], nb = a.panel[bk];
        const int tm = tid / T, lt = tid % T;
        const int bar = 1 + tm;
        const size_t share = team_share(T);
        unsigned char *sm = bsm + share * tm;
        // each pass takes one matrix; at most end-beg passes per team
        for (int pass = 0; pass <= end - beg; ++pass) {
            if (lt == 0) s_item[tm] = beg + atomicAdd(&a.queue[bk], 1);
            team_sync(bar, T);
            const int item = s_item[tm];
            team_sync(bar, T);
            if (item >= end) break;
            const int idx = a.order[item];
            const bool mix = MIXED && (a.precision != 2 || mixed_pays(a.n[idx], a.nrhs[idx]));
            if (mix && a.nrhs[idx] <= 32 && mixed_need(a.n[idx], a.nrhs[idx]) <= share)
                solve_mixed(a, idx, sm, lt, T, bar, red_v[tm], red_i[tm]);
            else if (mix && mixed_blocked_ok(a, a.n[idx], a.nrhs[idx], nb, T, share))
                // slots [blockIdx.x * mx_teams, +teams): the same for every
                // bucket, since CTAs move through the buckets independently
                solve_mixed_blocked(a, idx, sm, share, nb, blockIdx.x * a.mx_teams + tm, lt, T, bar,
                                    red_v[tm], red_i[tm]);
            else
                solve_fp64(a, idx, sm, share, nb, lt, T, bar, red_v[tm], red_i[tm]);
        }
        __syncthreads();
    }
}

}  // namespace

// ----------------------------------------------------------------- plan -----
struct BatchedPlan {
    int device = -1;
    int count = 0;
    BatchArgs args;
    int *d_meta = nullptr;          // order | n | nrhs | lda | ldb | queue
    void **d_ptrs = nullptr;        // A | B | ipiv
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int team[BT_BUCKETS];
    int panel[BT_BUCKETS];
    void *mx_pool = nullptr;        // precision 1: FP32 factors beyond shared memory
    std::vector<int> hn;
};

namespace {
std::mutex g_tune_mu;
// (device, bucket, precision) -> (team size, panel width)
std::map<std::tuple<int, int, int>, std::pair<int, int>> g_tuned;

int default_team(int bucket) {
    const int ub = kBucketMax[bucket];
    return ub <= 32 ? 32 : ub <= 216 ? 64 : ub <= 432 ? 128 : 256;
}

// T keeps an n x n matrix with k right-hand sides in shared memory
bool fits_shared(int T, int n, int k) { return fp64_need(n, k) <= team_share(T); }

// (T, nb) keeps it in shared memory or on the blocked path with nb-column
// panels (the unblocked global-memory path is several times slower).  The
// limits this gives for the blocked path, n <= 108 * 16/nb * T/32 (108, 216,
// 432, 864, or inside the last, unbounded bucket), are bucket bounds, so a
// choice feasible for a bucket's largest matrix is feasible for all of its
// matrices.
bool team_feasible(int T, int nb, int n, int k) {
    return fits_shared(T, n, k) || blocked_need(n, nb) <= team_share(T);
}

int env_panel() {
    const char *s = getenv("FLENS_GB300_BATCH_PANEL");
    const int v = s ? atoi(s) : 0;
    return (v == 8 || v == 16) ? v : 0;
}

int env_team() {
    const char *s = getenv("FLENS_GB300_BATCH_TEAM");
    if (!s) return 0;
    const int t = atoi(s);
    return (t == 32 || t == 64 || t == 128 || t == 256) ? t : 0;
}

bool tuning_enabled() {
    const char *s = getenv("FLENS_GB300_BATCH_TUNE");
    return !(s && s[0] == '0');
}

void fill_ranges(const std::vector<int> &hn, std::vector<int> &order, BatchArgs &a) {
    const int count = (int)hn.size();
    order.resize(count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        const int bx = bucket_of(hn[x]), by = bucket_of(hn[y]);
        if (bx != by) return bx > by;
        return hn[x] > hn[y];
    });
    int i = 0;
    for (int b = BT_BUCKETS - 1; b >= 0; --b) {
        a.beg[b] = i;
        while (i < count && bucket_of(hn[order[i]]) == b) ++i;
        a.end[b] = i;
    }
}

int set_attributes() {
    static DeviceOnce once64, once32;
    const int st = set_smem_once(once64, (const void *)batched_gesv_kernel<false>, (int)BT_SMEM);
    if (st != kOk) return st;
    return set_smem_once(once32, (const void *)batched_gesv_kernel<true>, (int)BT_SMEM);
}

// queue reset + the persistent kernel (also what a plan's graph holds)
int launch(const BatchArgs &a, cudaStream_t s) {
    int st = set_attributes();
    if (st != kOk) return st;
    FG_CUDA(cudaMemsetAsync(a.queue, 0, sizeof(int) * BT_BUCKETS, s));
    if (a.precision >= 1) batched_gesv_kernel<true><<<num_sms(), BT_THREADS, BT_SMEM, s>>>(a);
    else batched_gesv_kernel<false><<<num_sms(), BT_THREADS, BT_SMEM, s>>>(a);
    FG_CUDA(cudaGetLastError());
    return kOk;
}

// copies the pristine A | B at `master` over each of the tuner's `count`
// matrices (stride `per` bytes; `words` doubles each)
__global__ void tune_restore_kernel(char *buf, const char *master, size_t per, size_t words,
                                    int count) {
    const double *src = (const double *)master;
    const size_t total = words * (size_t)count;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const size_t i = e / words, w = e - i * words;
        ((double *)(buf + per * i))[w] = src[w];
    }
}

// Time each candidate team size on synthetic matrices of the bucket's largest
// size (diagonally dominant, uniform entries) and return the fastest.
std::pair<int, int> tune_bucket(int bucket, int nmax, int kmax, int precision, cudaStream_t s) {
    const int dev = device_id();
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        auto it = g_tuned.find(std::make_tuple(dev, bucket, precision));
        if (it != g_tuned.end()) return it->second;
    }
    const int sms = num_sms();
    const int n = nmax, k = kmax;
    const std::pair<int, int> fallback(default_team(bucket), 16);
    // candidates: (team size, panel width) pairs that keep the bucket's
    // largest matrix in shared memory or on the blocked path; the panel width
    // is only a choice where the blocked path runs
    std::vector<std::pair<int, int>> cand;
    for (int T : {32, 64, 128, 256}) {
        if (fits_shared(T, n, k)) {
            cand.emplace_back(T, 16);
            continue;
        }
        for (int nb : {16, 8})
            if (team_feasible(T, nb, n, k)) cand.emplace_back(T, nb);
    }
    if (cand.size() <= 1) {
        const std::pair<int, int> c = cand.empty() ? std::make_pair(256, 16) : cand[0];
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tuned[std::make_tuple(dev, bucket, precision)] = c;
        return c;
    }
    const size_t aBytes = (size_t)n * n * 8, bBytes = (size_t)n * k * 8, pBytes = (size_t)n * 4;
    const size_t per = (aBytes + bBytes + pBytes + 255) / 256 * 256;
    // four matrices for every team of the smallest candidate on every SM (a
    // smaller sample would leave SMs idle under the smaller teams and bias
    // the choice towards large ones), at most 1 GiB of them
    int count = 4 * sms * (BT_THREADS / cand[0].first);
    while (count > sms && per * (size_t)count > (1u << 30)) count /= 2;
    if (per * (size_t)count > (1u << 30)) return fallback;
    const size_t metaBytes = (size_t)count * 4 * 6 + 3 * (size_t)count * sizeof(void *) +
                             (size_t)count * (4 + 4 + 8) + 4096;
    char *buf = (char *)workspace_slot(s, 3, per * (count + 1) + metaBytes);
    if (!buf) return fallback;
    char *master = buf + per * count + metaBytes;       // one pristine A | B
    std::vector<double> hA((size_t)n * n), hB((size_t)n * k);
    std::mt19937_64 rng(1234 + bucket);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    for (auto &v : hA) v = U(rng);
    for (int i = 0; i < n; ++i) hA[i + (size_t)i * n] += n / 4.0;
    for (auto &v : hB) v = U(rng);
    std::vector<void *> pA(count), pB(count), pP(count);
    std::vector<int> hn(count, n), hk(count, k), hld(count, n);
    for (int i = 0; i < count; ++i) {
        pA[i] = buf + per * i;
        pB[i] = buf + per * i + aBytes;
        pP[i] = buf + per * i + aBytes + bBytes;
    }
    char *m = buf + per * count;
    int *d_order = (int *)m, *d_n = d_order + count, *d_k = d_n + count, *d_lda = d_k + count,
        *d_ldb = d_lda + count, *d_q = d_ldb + count;
    void **d_p = (void **)(((uintptr_t)(d_q + BT_BUCKETS) + 15) & ~(uintptr_t)15);
    int *d_info = (int *)(d_p + 3 * count), *d_it = d_info + count;
    double *d_be = (double *)(((uintptr_t)(d_it + count) + 15) & ~(uintptr_t)15);
    BatchArgs a;
    memset(&a, 0, sizeof a);
    std::vector<int> order;
    fill_ranges(hn, order, a);
    cudaMemcpyAsync(d_order, order.data(), 4 * count, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_n, hn.data(), 4 * count, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_k, hk.data(), 4 * count, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_lda, hld.data(), 4 * count, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_ldb, hld.data(), 4 * count, cudaMemcpyHostToDevice, s);
    std::vector<void *> hp(3 * count);
    for (int i = 0; i < count; ++i) {
        hp[i] = pA[i];
        hp[count + i] = pB[i];
        hp[2 * count + i] = pP[i];
    }
    cudaMemcpyAsync(d_p, hp.data(), sizeof(void *) * 3 * count, cudaMemcpyHostToDevice, s);
    a.order = d_order;
    a.n = d_n;
    a.nrhs = d_k;
    a.lda = d_lda;
    a.ldb = d_ldb;
    a.A = (double *const *)d_p;
    a.B = (double *const *)(d_p + count);
    a.ipiv = (int *const *)(d_p + 2 * count);
    a.info = d_info;
    a.iters = d_it;
    a.berr = d_be;
    a.queue = d_q;
    a.precision = precision;
    a.max_iter = 10;
    cudaMemcpyAsync(master, hA.data(), aBytes, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(master + aBytes, hB.data(), bBytes, cudaMemcpyHostToDevice, s);
    std::pair<int, int> best = fallback;
    float best_ms = 1e30f;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (const auto &c : cand) {
        for (int b = 0; b < BT_BUCKETS; ++b) {
            a.team[b] = c.first;
            a.panel[b] = c.second;
        }
        float tot = 0.0f;
        bool ok = true;
        for (int rep = 0; rep < 3; ++rep) {
            tune_restore_kernel<<<2 * sms, 256, 0, s>>>(buf, master, per, (aBytes + bBytes) / 8,
                                                       count);
            cudaEventRecord(e0, s);
            if (launch(a, s) != kOk) {
                ok = false;
                break;
            }
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep > 0) tot += ms;
        }
        if (ok && tot < best_ms) {
            best_ms = tot;
            best = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamSynchronize(s);
    trace("batched tune bucket=%d n=%d k=%d precision=%d -> team %d panel %d (%.3f ms)", bucket, n,
          k, precision, best.first, best.second, best_ms / 2);
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tuned[std::make_tuple(dev, bucket, precision)] = best;
    return best;
}

}  // namespace

int batched_plan_create(int count, const int *hn, const int *hk, double *const *hA, const int *hlda,
                        int *const *hipiv, double *const *hB, const int *hldb, int *d_info,
                        int precision, int *d_iters, double *d_berr, int max_iter,
                        cudaStream_t s, BatchedPlan **out) {
    *out = nullptr;
    int st0 = kOk;
    BatchedPlan *p = new BatchedPlan();
    p->device = device_id();
    p->count = count;
    p->hn.assign(hn, hn + count);
    BatchArgs &a = p->args;
    memset(&a, 0, sizeof a);
    std::vector<int> order;
    fill_ranges(p->hn, order, a);
    // team size and panel width per bucket
    const int forced = env_team(), forced_nb = env_panel();
    for (int b = 0; b < BT_BUCKETS; ++b) {
        std::pair<int, int> c(default_team(b), 16);
        if (forced || forced_nb) {
            if (forced) c.first = forced;
            if (forced_nb) c.second = forced_nb;
        } else if (tuning_enabled() && a.end[b] > a.beg[b]) {
            int nmax = 0, kmax = 0;
            for (int i = a.beg[b]; i < a.end[b]; ++i) {
                nmax = std::max(nmax, hn[order[i]]);
                kmax = std::max(kmax, hk[order[i]]);
            }
            c = tune_bucket(b, nmax, kmax, precision, s);
        }
        a.team[b] = p->team[b] = c.first;
        a.panel[b] = p->panel[b] = c.second;
    }
    const size_t intBytes = (size_t)count * 4;
    if (device_malloc((void **)&p->d_meta, 5 * intBytes + BT_BUCKETS * 4) != cudaSuccess ||
        device_malloc((void **)&p->d_ptrs, 3 * (size_t)count * sizeof(void *)) != cudaSuccess) {
        cudaGetLastError();
        set_last_error("batched plan: device allocation failed");
        if (p->d_meta) cudaFree(p->d_meta);
        delete p;
        return kErrAlloc;
    }
    int *d_order = p->d_meta, *d_n = d_order + count, *d_k = d_n + count, *d_lda = d_k + count,
        *d_ldb = d_lda + count, *d_q = d_ldb + count;
    FG_CUDA(cudaMemcpyAsync(d_order, order.data(), intBytes, cudaMemcpyHostToDevice, s));
    FG_CUDA(cudaMemcpyAsync(d_n, hn, intBytes, cudaMemcpyHostToDevice, s));
    FG_CUDA(cudaMemcpyAsync(d_k, hk, intBytes, cudaMemcpyHostToDevice, s));
    FG_CUDA(cudaMemcpyAsync(d_lda, hlda, intBytes, cudaMemcpyHostToDevice, s));
    FG_CUDA(cudaMemcpyAsync(d_ldb, hldb, intBytes, cudaMemcpyHostToDevice, s));
    std::vector<void *> hp(3 * (size_t)count);
    for (int i = 0; i < count; ++i) {
        hp[i] = hA[i];
        hp[count + i] = hB[i];
        hp[2 * (size_t)count + i] = hipiv[i];
    }
    FG_CUDA(cudaMemcpyAsync(p->d_ptrs, hp.data(), sizeof(void *) * 3 * (size_t)count,
                            cudaMemcpyHostToDevice, s));
    FG_CUDA(cudaStreamSynchronize(s));
    a.order = d_order;
    a.n = d_n;
    a.nrhs = d_k;
    a.lda = d_lda;
    a.ldb = d_ldb;
    a.A = (double *const *)p->d_ptrs;
    a.B = (double *const *)(p->d_ptrs + count);
    a.ipiv = (int *const *)(p->d_ptrs + 2 * (size_t)count);
    a.info = d_info;
    a.iters = d_iters;
    a.berr = d_berr;
    a.queue = d_q;
    a.precision = precision;
    a.max_iter = max_iter > 0 ? max_iter : 10;
    if (precision >= 1) {
        // pool for the matrices that take the blocked mixed path: a slot per
        // team of the CTAs, as large as the largest such matrix needs (if it
        // cannot be had, those matrices are solved in FP64 instead)
        size_t stride = 0;
        int teams = 0;
        for (int b = 0; b < BT_BUCKETS; ++b) {
            const int T = a.team[b];
            const size_t share = team_share(T);
            for (int i = a.beg[b]; i < a.end[b]; ++i) {
                const int ni = hn[order[i]], ki = hk[order[i]];
                if (ki > 32 || mixed_need(ni, ki) <= share) continue;
                if (precision == 2 && !mixed_pays(ni, ki)) continue;
                if (blocked_need(ni, a.panel[b], sizeof(float)) > share) continue;
                stride = std::max(stride, mx_need(ni, ki));
                teams = std::max(teams, BT_THREADS / T);
            }
        }
        if (stride > 0) {
            stride = (stride + 255) / 256 * 256;
            if (device_malloc(&p->mx_pool, stride * (size_t)num_sms() * teams) == cudaSuccess) {
                a.mx_pool = p->mx_pool;
                a.mx_stride = stride;
                a.mx_teams = teams;
            } else {
                cudaGetLastError();
                p->mx_pool = nullptr;
            }
        }
    }
    // capture the queue reset + persistent launch as one graph
    if ((st0 = set_attributes()) != kOk) return st0;
    cudaStream_t cap;
    FG_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    FG_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
    int st = launch(a, cap);
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(cap, &g);
    cudaStreamDestroy(cap);
    if (st != kOk || ce != cudaSuccess) {
        if (ce != cudaSuccess) cuda_fail(ce, "cudaStreamEndCapture");
        if (g) cudaGraphDestroy(g);
        cudaFree(p->d_meta);
        cudaFree(p->d_ptrs);
        if (p->mx_pool) cudaFree(p->mx_pool);
        delete p;
        return st != kOk ? st : kErrCuda;
    }
    p->graph = g;
    FG_CUDA(cudaGraphInstantiate(&p->exec, g, 0));
    *out = p;
    return kOk;
}

int batched_plan_execute(BatchedPlan *p, cudaStream_t s) {
    if (!p || !p->exec) return kErrUnsupported;
    KTimer kt(kFamBatched, s, 0.0, 0.0);
    FG_CUDA(cudaGraphLaunch(p->exec, s));
    return kOk;
}

void batched_plan_destroy(BatchedPlan *p) {
    if (!p) return;
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    if (p->d_meta) cudaFree(p->d_meta);
    if (p->d_ptrs) cudaFree(p->d_ptrs);
    if (p->mx_pool) cudaFree(p->mx_pool);
    delete p;
}

}  // namespace fg

// ----------------------------------------------------------------- C ABI ----
// A plan for solving `count` independent systems A_i X_i = B_i (n_i x n_i,
// n_i x nrhs_i, column-major FP64 in device memory).  The metadata arrays
// (n, nrhs, lda, ldb) and the pointer arrays (A, ipiv, B: device pointers)
// are HOST arrays read at creation; info / iters / berr are device arrays of
// `count` entries written by every execution.  Creating a plan autotunes the
// team size of each size bucket (first time per device and bucket; disable
// with FLENS_GB300_BATCH_TUNE=0) and captures one persistent launch in a
// CUDA graph.
FG_API int flens_gb300_dgesv_batched_plan(int count, const int *n, const int *nrhs,
                                          double *const *A, const int *lda, int *const *ipiv,
                                          double *const *B, const int *ldb, int *info,
                                          int precision, int *iters, double *berr, int max_iter,
                                          void *stream, void **plan) {
    if (count < 0) return -1;
    if (precision < 0 || precision > 2) return -10;
    if (!plan) return -15;
    for (int i = 0; i < count; ++i) {
        if (n[i] < 0 || nrhs[i] < 0 || lda[i] < (n[i] > 1 ? n[i] : 1) ||
            ldb[i] < (n[i] > 1 ? n[i] : 1)) {
            fg::set_last_error("batched: matrix %d has an illegal size or leading dimension", i);
            return -2;
        }
    }
    fg::BatchedPlan *p = nullptr;
    const int st = fg::batched_plan_create(count, n, nrhs, A, lda, ipiv, B, ldb, info, precision,
                                           iters, berr, max_iter, (cudaStream_t)stream, &p);
    *plan = p;
    return st;
}

// Run a plan (one graph launch: the persistent kernel); async on stream.
FG_API int flens_gb300_batched_execute(void *plan, void *stream) {
    return fg::batched_plan_execute((fg::BatchedPlan *)plan, (cudaStream_t)stream);
}

FG_API void flens_gb300_batched_destroy(void *plan) {
    fg::batched_plan_destroy((fg::BatchedPlan *)plan);
}

// Team size chosen for a size bucket of a plan (upper bounds of n: 16, 32, 48,
// 64, 108, 216, 320, 432, 864, unbounded); -1 past the last bucket.
FG_API int flens_gb300_batched_team(void *plan, int bucket) {
    if (!plan || bucket < 0 || bucket >= fg::BT_BUCKETS) return -1;
    return ((fg::BatchedPlan *)plan)->team[bucket];
}

// Panel width (8 or 16 columns) of the blocked factorisation the plan uses
// for a size bucket; -1 past the last bucket.
FG_API int flens_gb300_batched_panel(void *plan, int bucket) {
    if (!plan || bucket < 0 || bucket >= fg::BT_BUCKETS) return -1;
    return ((fg::BatchedPlan *)plan)->panel[bucket];
}
