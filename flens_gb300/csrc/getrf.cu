// getrf.cu -- blocked LU with partial pivoting (trf), its row interchanges
// (laswp) and solves (trs), FP64, column-major, 1-based pivots.
//
// Replaces, for double:
//   flens::lapack::trf  -> generic::trf_impl   flens/lapack/ge/trf.tcc:59-152
//   tf2 (panel)         -> generic::tf2_impl   flens/lapack/ge/tf2.tcc:56-136
//   laswp               -> generic::laswp_impl flens/lapack/la/laswp.tcc:54-93
//   trs                 -> generic::trs_impl   flens/lapack/ge/trs.tcc:59-109
//
// Structure (one stream, all asynchronous):
//   for each block column j (width jb <= 64, the reference's ilaenv GETRF
//   block size, flens/lapack/la/ilaenv.tcc:93-99):
//     panel_kernel      cooperative grid, up to one CTA per SM; the (m-j) x jb
//                       panel lives in shared memory split by rows.  Per
//                       column each CTA finds its best candidate (warp-shuffle
//                       argmax, first maximum wins), publishes it with the
//                       candidate row in its own slot (release store of a
//                       sequence number) and reads every CTA's slot (acquire,
//                       bounded wait), so all CTAs agree on the pivot without
//                       a separate barrier; then every CTA swaps, scales and
//                       applies the rank-1 update to its own rows.  At the end
//                       it turns the jb interchanges into a list of
//                       (destination row, source row) moves.  FP32 storage
//                       uses panel32_kernel: FP32 arithmetic, and the key
//                       published in one word with its sequence number.
//     laswp_pairs_kernel applies those moves to every column outside the
//                       panel, one warp per column (loads, then stores).
//     dtrsm_launch      U12 = L11^-1 A12
//     dgemm_launch      A22 -= A21 * U12
//
// Unlike the reference, the GPU path always uses the blocked algorithm (the
// reference switches to tf2 when nb >= min(m,n), trf.tcc:87-91); the pivots and
// factors are the same in exact arithmetic.
#include "common.cuh"

#include <float.h>
#include <limits.h>
#include <stdlib.h>

#include <algorithm>
#include <type_traits>
#include <mutex>

namespace fg {
namespace {

constexpr int PANEL_THREADS = 256;
constexpr int PANEL_NB = 64;           // max panel width
constexpr int PANEL_GMAX = 256;        // max CTAs in a panel grid
constexpr int PANEL_RMIN = 32;         // min rows per CTA
constexpr size_t PANEL_SMEM_MAX = 200 * 1024;

// One exchange slot per CTA and per step parity.  A CTA publishes its pivot
// candidate (|value|, row, the row's jb panel entries) and, if it owns panel
// row jj, that row; `seq` is written last with release semantics.
struct PanelSlot {
    unsigned long long seq;
    unsigned long long key;    // pivot key of the candidate (see pivot_key)
    int idx;
    int pad;
    double row[PANEL_NB];
    double rowjj[PANEL_NB];
};

struct PanelScratch {
    PanelSlot *slots;   // [2][GMAX]
    int *swap_cnt;      // [1]
    int *swap_dst;      // [2*NB]
    int *swap_src;      // [2*NB]
};

constexpr size_t kSlotBytes = 2 * (size_t)PANEL_GMAX * sizeof(PanelSlot);

size_t panel_scratch_bytes() { return kSlotBytes + 256 + 4 * PANEL_NB * sizeof(int) + 1024; }

PanelScratch carve_panel_scratch(void *base) {
    char *p = (char *)base;
    PanelScratch s;
    s.slots = (PanelSlot *)p;
    p += kSlotBytes;
    s.swap_cnt = (int *)p;
    p += 256;
    s.swap_dst = (int *)p;
    p += 2 * PANEL_NB * sizeof(int);
    s.swap_src = (int *)p;
    return s;
}

__device__ __forceinline__ void st_release(unsigned long long *p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Pivot keys are integers, so the pivot search never touches the FP64 pipe
// (2 instructions per clock per SM on this part): |x| of a double orders
// like its bit pattern with the sign cleared.  0 = no candidate, 1 = NaN
// (loses to every number: iamax's `>` is false for NaN), |x| bits + 2
// otherwise.  (key, row) "better than": larger key; on equal keys the
// smaller row, which is cxxblas iamax's first-maximum rule
// (cxxblas/level1/iamax.tcc:52-56).
constexpr unsigned long long kKeyNone = 0ull;

__device__ __forceinline__ unsigned long long pivot_key(double x) {
    const unsigned long long a = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
    return a > 0x7ff0000000000000ull ? 1ull : a + 2ull;
}

// Named barrier 1 over `count` threads: the producer warp arrives without
// waiting, the consumers wait until every participant has arrived.
__device__ __forceinline__ void named_bar_arrive(int id, int count) {
    asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(count) : "memory");
}
__device__ __forceinline__ void named_bar_sync(int id, int count) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

__device__ __forceinline__ bool better(unsigned long long k1, int i1, unsigned long long k2, int i2) {
    return k1 > k2 || (k1 == k2 && i1 < i2);
}

// Warp-wide argmax of (key, row) with three redux.sync: the largest high
// word, then the largest low word among those lanes, then the smallest row
// among the lanes holding that key.  Every lane gets the result; all 32
// lanes must call it.
__device__ __forceinline__ void warp_argmax(unsigned long long &k, int &i) {
    const unsigned hi = (unsigned)(k >> 32), lo = (unsigned)k;
    const unsigned mhi = __reduce_max_sync(0xffffffffu, hi);
    const unsigned mlo = __reduce_max_sync(0xffffffffu, hi == mhi ? lo : 0u);
    const unsigned cand = (hi == mhi && lo == mlo) ? (unsigned)i : 0xffffffffu;
    i = (int)__reduce_min_sync(0xffffffffu, cand);
    k = ((unsigned long long)mhi << 32) | mlo;
}

// Block 0, warp 0 of a panel (all 32 lanes): the jb interchanges of the
// panel at column j0 (ipiv, written by this warp's lane 0 during the panel)
// as a list of (destination row, source row) moves, compacted to the moves
// that change something, into ps.swap_dst / swap_src / swap_cnt.
__device__ __forceinline__ void panel_moves(int jb, int j0, const int *ipiv, PanelScratch ps,
                                            int *s_list_row, int *s_list_src, int lane) {
    for (int i = lane; i < jb; i += 32) {
        s_list_row[i] = j0 + i;
        s_list_src[i] = j0 + i;
    }
    __syncwarp();
    int cnt = jb;
    for (int i = 0; i < jb; ++i) {
        const int p = ipiv[j0 + i] - 1;
        int pos;
        if (p < j0 + jb) {
            pos = p - j0;
        } else {
            int found = -1;
            for (int base = jb; base < cnt; base += 32) {
                const int e = base + lane;
                const unsigned hit = __ballot_sync(0xffffffffu, e < cnt && s_list_row[e] == p);
                if (hit) { found = base + __ffs(hit) - 1; break; }
            }
            if (found < 0) {
                found = cnt;
                if (lane == 0) { s_list_row[cnt] = p; s_list_src[cnt] = p; }
                ++cnt;
            }
            pos = found;
        }
        __syncwarp();
        if (lane == 0 && pos != i) {
            const int t = s_list_src[i];
            s_list_src[i] = s_list_src[pos];
            s_list_src[pos] = t;
        }
        __syncwarp();
    }
    if (lane == 0) {
        int k = 0;
        for (int e = 0; e < cnt; ++e) {
            if (s_list_row[e] != s_list_src[e]) {
                ps.swap_dst[k] = s_list_row[e];
                ps.swap_src[k] = s_list_src[e];
                ++k;
            }
        }
        *ps.swap_cnt = k;
    }
}

// Panel factorisation, tf2 semantics (flens/lapack/ge/tf2.tcc:56-136).
// A points at the panel's top-left element A(j,j); the panel is mp x jb.
// CTA b owns panel rows [b*R, min(mp,(b+1)*R)), kept in shared memory as
// S[c*R + r].  With at most 128 rows a CTA gives each row W = 2, 4 or 8
// lanes (interleaved columns); with more rows thread t owns local rows t,
// t+256, ... and updates them at once.  Block barriers per column: one to
// collect the warps' candidates, one after the cross-CTA poll, one to hand
// the pivot to every thread.  Warp 0 does the cross-CTA exchange.
// Two builds: DEFER (lanes per row and most of each column's rank-1 update
// deferred past the next column's candidate search, see [E2] below; about
// 120 registers per thread) for panels that run alone or beside a small
// update, and the immediate update within 64 registers for panels beside a
// large look-ahead GEMM (74 registers, 256 threads per CTA): at 102
// registers only one GEMM CTA fitted beside the panel instead of two (the
// n = 8192 LU: 325.9 against 322.8 ms per solve), and capping the deferred
// build instead slowed the split-update LU's panels by 11%.
template <typename T, bool DEFER>
__global__ void __launch_bounds__(PANEL_THREADS, DEFER ? 1 : 4)
panel_kernel(T *__restrict__ A, int lda, int mp, int jb, int j0,
             int *__restrict__ ipiv, int *__restrict__ info, int *__restrict__ status,
             PanelScratch ps, int R, unsigned long long epoch) {
    extern __shared__ double S[];
    constexpr int NW = PANEL_THREADS / 32;
    __shared__ double prow[PANEL_NB], orow[PANEL_NB];
    __shared__ unsigned long long red_k[NW], red_k2[NW];
    __shared__ int red_i[NW], red_i2[NW];
    __shared__ int s_gs, s_abort;
    __shared__ double s_pv, s_rinv;
    __shared__ int s_list_row[2 * PANEL_NB], s_list_src[2 * PANEL_NB];

    const int b = blockIdx.x, G = gridDim.x, tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const int rb = b * R;
    const int re = min(mp, rb + R);
    const int nr = max(0, re - rb);
    // lanes per row in the update: 8, 4 or 2 while nr * W fits the CTA
    const int W = nr <= 32 ? 8 : nr <= 64 ? 4 : nr <= 128 ? 2 : 1;

    for (int e = tid; e < nr * jb; e += PANEL_THREADS) {
        const int r = e % nr, c = e / nr;
        S[c * R + r] = A[(size_t)(rb + r) + (size_t)c * lda];
    }
    if (tid == 0) s_abort = 0;
    __syncthreads();

    // pivot keys of column 0 over the owned rows (later columns: computed
    // during the update)
    unsigned long long nbk = kKeyNone;
    int nbi = INT_MAX;
    for (int r = tid; r < nr; r += PANEL_THREADS) {
        const unsigned long long key = pivot_key(S[r]);
        if (better(key, rb + r, nbk, nbi)) { nbk = key; nbi = rb + r; }
    }

    // Deferred update (DEFER and W > 1): after the pivot of column jj is
    // known, each
    // row gets its swap, its multiplier l and the update of column jj + 1
    // (whose pivot keys the next search needs); the update of columns
    // >= jj + 2 waits until the next column's candidates are published, so
    // it runs while the other CTAs publish and this CTA polls.  Warp 0
    // publishes the candidate rows with those columns computed on the fly,
    // by the same FMA the deferred update stores: the factors are bitwise
    // those of the undeferred order.
    const bool lanes = W > 1, defer = DEFER && lanes;
    const double *dP = nullptr;          // pivot row of the pending update
    int d_jj = -1, d_gs = -1;            // its column and pivot row (-1: none)
    bool d_swap = false;
    bool pend = false, pend_gs = false;  // this thread's row has a pending update
    double pend_l = 0.0;
    for (int jj = 0; jj < jb; ++jj) {
        const int par = jj & 1;
        const unsigned long long want = epoch * 128ull + (unsigned long long)jj + 1ull;
        // -- [A] this CTA's candidate among its rows g >= jj
        unsigned long long k = nbk;
        int i = nbi;
        warp_argmax(k, i);
        if (lane == 0) { red_k[warp] = k; red_i[warp] = i; }
        __syncthreads();                                             // B1
        if (warp == 0) {
            // -- [B] publish the candidate row (and row jj if owned); the
            // release store by lane 0 after __syncwarp orders the warp's slot
            // writes before the sequence number
            k = lane < NW ? red_k[lane] : kKeyNone;
            i = lane < NW ? red_i[lane] : INT_MAX;
            warp_argmax(k, i);
            PanelSlot *mine = &ps.slots[par * PANEL_GMAX + b];
            // entry c of local row x, final (the pending update applied)
            auto fin = [&](int x, int c) -> double {
                if (d_jj < 0 || c < d_jj + 2) return S[c * R + x];
                const double src = (d_swap && rb + x == d_gs) ? orow[c] : S[c * R + x];
                return fma(-dP[c], S[d_jj * R + x], src);
            };
            // both rows into registers (jb <= 64: two entries per lane)
            // before the other warps may store their pending updates
            const bool has_i = i != INT_MAX, has_jj = jj >= rb && jj < re;
            double vi[2] = {0.0, 0.0}, vj[2] = {0.0, 0.0};
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int c = lane + 32 * h;
                if (c < jb) {
                    if (has_i) vi[h] = fin(i - rb, c);
                    if (has_jj) vj[h] = fin(jj - rb, c);
                }
            }
            if (defer) named_bar_arrive(1, PANEL_THREADS);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int c = lane + 32 * h;
                if (c < jb) {
                    if (has_i) mine->row[c] = vi[h];
                    if (has_jj) mine->rowjj[c] = vj[h];
                }
            }
            if (lane == 0) {
                mine->key = k;
                mine->idx = i;
            }
            __syncwarp();
            if (lane == 0) st_release(&mine->seq, want);
        } else if (defer) {
            named_bar_sync(1, PANEL_THREADS);
        }
        // -- [E2] the pending update of column jj - 1: columns >= jj + 1
        if (pend) {
            const int r = tid / W, q = tid % W;
            const double *old = pend_gs ? orow : nullptr;
            int c = d_jj + 2 + q;
            for (; c + 3 * W < jb; c += 4 * W) {
                double v[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) v[u] = old ? old[c + u * W] : S[(c + u * W) * R + r];
#pragma unroll
                for (int u = 0; u < 4; ++u) S[(c + u * W) * R + r] = fma(-dP[c + u * W], pend_l, v[u]);
            }
            for (; c < jb; c += W) S[c * R + r] = fma(-dP[c], pend_l, old ? old[c] : S[c * R + r]);
            pend = false;
        }
        // -- [C] thread t < G waits for slot t of this step and reads it
        unsigned long long gk = kKeyNone;
        int gi = INT_MAX;
        if (tid < G) {
            const PanelSlot *sl = &ps.slots[par * PANEL_GMAX + tid];
            unsigned spins = 0;
            while (ld_acquire(&sl->seq) != want) {
                if (++spins > kSpinLimit) {
                    atomicOr(status, kDevBarrierTimeout);
                    s_abort = 1;
                    break;
                }
                if (spins > 32) __nanosleep(32);
            }
            gk = __ldcg(&sl->key);
            gi = __ldcg(&sl->idx);
        }
        if (warp * 32 < G) {                                          // warp-uniform
            warp_argmax(gk, gi);
            if (lane == 0) { red_k2[warp] = gk; red_i2[warp] = gi; }
        }
        __syncthreads();                                             // B2
        if (s_abort) return;
        if (warp == 0) {
            const int nw = (G + 31) / 32;
            gk = lane < nw ? red_k2[lane] : kKeyNone;
            gi = lane < nw ? red_i2[lane] : INT_MAX;
            warp_argmax(gk, gi);
            // -- [D] the old row jj and the winner's row, one round trip;
            // lane 0 settles the pivot (iamax starts from element jj: if it
            // is NaN nothing compares greater and jj is the pivot,
            // cxxblas/level1/iamax.tcc:50-57) and its reciprocal once
            const PanelSlot *sj = &ps.slots[par * PANEL_GMAX + jj / R];
            const PanelSlot *sw = &ps.slots[par * PANEL_GMAX + gi / R];
            for (int c = lane; c < jb; c += 32) {
                orow[c] = ld_cg(&sj->rowjj[c]);
                prow[c] = ld_cg(&sw->row[c]);
            }
            __syncwarp();
            if (lane == 0) {
                const double ajj = orow[jj];
                const int gs = isnan(ajj) ? jj : gi;
                const double pv = (gs == jj) ? ajj : prow[jj];
                s_gs = gs;
                s_pv = pv;
                s_rinv = (pv != 0.0 && fabs(pv) >= DBL_MIN) ? 1.0 / pv : 0.0;
                if (b == 0) {
                    ipiv[j0 + jj] = j0 + gs + 1;
                    if (pv == 0.0 && *info == 0) *info = j0 + jj + 1;
                }
            }
        }
        __syncthreads();                                             // B3
        const int gs = s_gs;
        const double pv = s_pv, rinv = s_rinv;
        const bool swap = (pv != 0.0) && (gs != jj);
        const double *P = (gs == jj) ? orow : prow;                  // new row jj

        // -- [E] per owned row: interchange, scaling, rank-1 update of the
        // columns > jj (deferred beyond jj + 1 when W > 1), and the pivot key
        // for column jj+1
        nbk = kKeyNone;
        nbi = INT_MAX;
        if (lanes) {
            // W lanes per row (nr * W <= 256: one row per lane group), lane q
            // of the group taking columns q, q + W, ...: the chain of
            // dependent shared-memory updates per thread is W times shorter.
            // The group's first lane reads the multiplier and broadcasts it
            // (all 32 lanes of every warp take part in the shuffle).
            const int r = tid / W, q = tid % W;
            const bool act = r < nr;
            const int g = rb + r;
            const bool to_jj = act && swap && g == jj, from_gs = act && swap && g == gs;
            double l0 = 0.0;
            if (act && q == 0) l0 = from_gs ? orow[jj] : S[jj * R + r];
            double l = __shfl_sync(0xffffffffu, l0, lane & ~(W - 1));
            if (to_jj) {
                for (int c = q; c < jb; c += W) S[c * R + r] = P[c];
            } else if (act && g > jj) {
                if (from_gs)
                    for (int c = q; c < jj; c += W) S[c * R + r] = orow[c];
                if (pv != 0.0) l = (rinv != 0.0) ? l * rinv : l / pv;
                if (q == 0 && pv != 0.0) S[jj * R + r] = l;
                const double *old = from_gs ? orow : nullptr;
                if (defer) {
                    // column jj + 1 and its key now, the rest in [E2]
                    if (q == 0 && jj + 1 < jb) {
                        const int c = jj + 1;
                        const double v = fma(-P[c], l, old ? old[c] : S[c * R + r]);
                        S[c * R + r] = v;
                        nbk = pivot_key(v);
                        nbi = g;
                    }
                    pend = jj + 2 + q < jb;
                    pend_gs = from_gs;
                    pend_l = l;
                } else {
                    int c = jj + 1 + q;
                    for (; c + 3 * W < jb; c += 4 * W) {
                        double v[4];
#pragma unroll
                        for (int u = 0; u < 4; ++u) v[u] = old ? old[c + u * W] : S[(c + u * W) * R + r];
#pragma unroll
                        for (int u = 0; u < 4; ++u) S[(c + u * W) * R + r] = fma(-P[c + u * W], l, v[u]);
                    }
                    for (; c < jb; c += W) S[c * R + r] = fma(-P[c], l, old ? old[c] : S[c * R + r]);
                    if (q == 0 && jj + 1 < jb) {
                        nbk = pivot_key(S[(jj + 1) * R + r]);
                        nbi = g;
                    }
                }
            }
            if (defer) {
                dP = P;
                d_jj = jj;
                d_gs = gs;
                d_swap = swap;
            }
        } else
        for (int r = tid; r < nr; r += PANEL_THREADS) {
            const int g = rb + r;
            if (swap && g == jj) {
                for (int c = 0; c < jb; ++c) S[c * R + r] = P[c];
            } else if (swap && g == gs) {
                for (int c = 0; c < jb; ++c) S[c * R + r] = orow[c];
            }
            if (g > jj) {
                double l = S[jj * R + r];
                if (pv != 0.0) {
                    l = (rinv != 0.0) ? l * rinv : l / pv;
                    S[jj * R + r] = l;
                }
                for (int c = jj + 1; c < jb; ++c) S[c * R + r] = fma(-P[c], l, S[c * R + r]);
                if (jj + 1 < jb) {
                    const unsigned long long key = pivot_key(S[(jj + 1) * R + r]);
                    if (better(key, g, nbk, nbi)) { nbk = key; nbi = g; }
                }
            }
        }
    }
    __syncthreads();

    for (int e = tid; e < nr * jb; e += PANEL_THREADS) {
        const int r = e % nr, c = e / nr;
        A[(size_t)(rb + r) + (size_t)c * lda] = (T)S[c * R + r];
    }

    // -- block 0, warp 0: the jb interchanges as (dst, src) row moves.
    if (b == 0 && tid < 32) panel_moves(jb, j0, ipiv, ps, s_list_row, s_list_src, lane);
}

// ---- the panel of the FP32-storage LU ---------------------------------------
// Same algorithm and thread layout as panel_kernel, in FP32 arithmetic (the
// reference's tf2 instantiated for float: slamch's safe minimum is FLT_MIN)
// and with a shorter exchange.  A float's pivot key fits in 32 bits, so each
// CTA publishes its candidate as ONE 64-bit word, (sequence << 32) | key,
// stored as soon as the CTA's argmax is known and before anything else; the
// load that finds a slot current also returns its key, so the pivot is
// settled after one round trip through L2 instead of a release store that
// waits for the rows, a sequence poll and a dependent key load.  The rows
// (candidate and row jj) and the candidate's index follow under their own
// release-stored sequence word, and only the two rows the pivot needs are
// waited for.  Equal keys go to the lower CTA, whose rows come first: with
// each CTA's own first maximum this is iamax's first-maximum rule.
struct PanelSlot32 {
    unsigned long long head;   // (sequence << 32) | pivot key (pivot_key32)
    unsigned long long rseq;   // sequence, release-stored after row/rowjj/idx
    int idx;
    int pad[3];
    float row[PANEL_NB];
    float rowjj[PANEL_NB];
};
static_assert(2 * PANEL_GMAX * sizeof(PanelSlot32) <= kSlotBytes, "FP32 slots fit the exchange area");

// 0 = no candidate, 1 = NaN, |x| bits + 2 otherwise (at most 0x7f800002)
__device__ __forceinline__ unsigned long long pivot_key32(float x) {
    const unsigned a = __float_as_uint(x) & 0x7fffffffu;
    return a > 0x7f800000u ? 1ull : (unsigned long long)a + 2ull;
}

__device__ __forceinline__ void st_relaxed(unsigned long long *p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

template <bool DEFER>
__global__ void __launch_bounds__(PANEL_THREADS, DEFER ? 1 : 4)
panel32_kernel(float *__restrict__ A, int lda, int mp, int jb, int j0,
               int *__restrict__ ipiv, int *__restrict__ info, int *__restrict__ status,
               PanelScratch ps, int R, unsigned long long epoch) {
    extern __shared__ double S32_raw[];
    float *S = reinterpret_cast<float *>(S32_raw);
    constexpr int NW = PANEL_THREADS / 32;
    __shared__ float prow[PANEL_NB], orow[PANEL_NB];
    __shared__ unsigned long long red_k[NW], red_k2[NW];
    __shared__ int red_i[NW], red_i2[NW];
    __shared__ int s_gs, s_abort;
    __shared__ float s_pv, s_rinv;
    __shared__ int s_list_row[2 * PANEL_NB], s_list_src[2 * PANEL_NB];
    PanelSlot32 *slots = reinterpret_cast<PanelSlot32 *>(ps.slots);

    const int b = blockIdx.x, G = gridDim.x, tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const int rb = b * R;
    const int re = min(mp, rb + R);
    const int nr = max(0, re - rb);
    const int W = nr <= 32 ? 8 : nr <= 64 ? 4 : nr <= 128 ? 2 : 1;

    for (int e = tid; e < nr * jb; e += PANEL_THREADS) {
        const int r = e % nr, c = e / nr;
        S[c * R + r] = A[(size_t)(rb + r) + (size_t)c * lda];
    }
    if (tid == 0) s_abort = 0;
    __syncthreads();

    unsigned long long nbk = kKeyNone;
    int nbi = INT_MAX;
    for (int r = tid; r < nr; r += PANEL_THREADS) {
        const unsigned long long key = pivot_key32(S[r]);
        if (better(key, rb + r, nbk, nbi)) { nbk = key; nbi = rb + r; }
    }

    const bool lanes = W > 1, defer = DEFER && lanes;
    const float *dP = nullptr;
    int d_jj = -1, d_gs = -1;
    bool d_swap = false;
    bool pend = false, pend_gs = false;
    float pend_l = 0.0f;
    for (int jj = 0; jj < jb; ++jj) {
        const int par = jj & 1;
        const unsigned long long want = epoch * 128ull + (unsigned long long)jj + 1ull;
        const unsigned want32 = (unsigned)want;
        // -- [A] this CTA's candidate among its rows g >= jj
        unsigned long long k = nbk;
        int i = nbi;
        warp_argmax(k, i);
        if (lane == 0) { red_k[warp] = k; red_i[warp] = i; }
        __syncthreads();                                             // B1
        if (warp == 0) {
            // -- [B] the key first, in one word with its sequence number;
            // then the rows under their own sequence word
            k = lane < NW ? red_k[lane] : kKeyNone;
            i = lane < NW ? red_i[lane] : INT_MAX;
            warp_argmax(k, i);
            PanelSlot32 *mine = &slots[par * PANEL_GMAX + b];
            if (lane == 0) st_relaxed(&mine->head, ((unsigned long long)want32 << 32) | k);
            auto fin = [&](int x, int c) -> float {
                if (d_jj < 0 || c < d_jj + 2) return S[c * R + x];
                const float src = (d_swap && rb + x == d_gs) ? orow[c] : S[c * R + x];
                return fmaf(-dP[c], S[d_jj * R + x], src);
            };
            const bool has_i = i != INT_MAX, has_jj = jj >= rb && jj < re;
            float vi[2] = {0.0f, 0.0f}, vj[2] = {0.0f, 0.0f};
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int c = lane + 32 * h;
                if (c < jb) {
                    if (has_i) vi[h] = fin(i - rb, c);
                    if (has_jj) vj[h] = fin(jj - rb, c);
                }
            }
            if (defer) named_bar_arrive(1, PANEL_THREADS);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int c = lane + 32 * h;
                if (c < jb) {
                    if (has_i) mine->row[c] = vi[h];
                    if (has_jj) mine->rowjj[c] = vj[h];
                }
            }
            if (lane == 0) mine->idx = i;
            __syncwarp();
            if (lane == 0) st_release(&mine->rseq, want);
        } else if (defer) {
            named_bar_sync(1, PANEL_THREADS);
        }
        // -- [E2] the pending update of column jj - 1: columns >= jj + 1
        if (pend) {
            const int r = tid / W, q = tid % W;
            const float *old = pend_gs ? orow : nullptr;
            int c = d_jj + 2 + q;
            for (; c + 3 * W < jb; c += 4 * W) {
                float v[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) v[u] = old ? old[c + u * W] : S[(c + u * W) * R + r];
#pragma unroll
                for (int u = 0; u < 4; ++u) S[(c + u * W) * R + r] = fmaf(-dP[c + u * W], pend_l, v[u]);
            }
            for (; c < jb; c += W) S[c * R + r] = fmaf(-dP[c], pend_l, old ? old[c] : S[c * R + r]);
            pend = false;
        }
        // -- [C] thread t < G waits for the key word of slot t; the winner is
        // the largest key, the lower CTA on equal keys
        unsigned long long gk = kKeyNone;
        int gc = INT_MAX;
        if (tid < G) {
            const PanelSlot32 *sl = &slots[par * PANEL_GMAX + tid];
            unsigned spins = 0;
            unsigned long long h;
            while (((h = ld_acquire(&sl->head)) >> 32) != (unsigned long long)want32) {
                if (++spins > kSpinLimit) {
                    atomicOr(status, kDevBarrierTimeout);
                    s_abort = 1;
                    break;
                }
                if (spins > 32) __nanosleep(32);
            }
            gk = h & 0xffffffffull;
            gc = tid;
        }
        if (warp * 32 < G) {                                          // warp-uniform
            warp_argmax(gk, gc);
            if (lane == 0) { red_k2[warp] = gk; red_i2[warp] = gc; }
        }
        __syncthreads();                                             // B2
        if (s_abort) return;
        if (warp == 0) {
            const int nw = (G + 31) / 32;
            gk = lane < nw ? red_k2[lane] : kKeyNone;
            gc = lane < nw ? red_i2[lane] : INT_MAX;
            warp_argmax(gk, gc);
            // -- [D] the winner's row and row jj, once their owners have
            // stored them (bounded waits, every lane)
            const PanelSlot32 *sj = &slots[par * PANEL_GMAX + jj / R];
            const PanelSlot32 *sw = &slots[par * PANEL_GMAX + gc];
            bool ok = true;
            {
                unsigned spins = 0;
                while (ld_acquire(&sw->rseq) != want || ld_acquire(&sj->rseq) != want) {
                    if (++spins > kSpinLimit) {
                        ok = false;
                        break;
                    }
                    if (spins > 32) __nanosleep(32);
                }
            }
            if (!__all_sync(0xffffffffu, ok)) {
                if (lane == 0) {
                    atomicOr(status, kDevBarrierTimeout);
                    s_abort = 1;
                }
            } else {
                for (int c = lane; c < jb; c += 32) {
                    orow[c] = __ldcg(&sj->rowjj[c]);
                    prow[c] = __ldcg(&sw->row[c]);
                }
                const int gi = __ldcg(&sw->idx);
                __syncwarp();
                if (lane == 0) {
                    const float ajj = orow[jj];
                    const int gs = isnan(ajj) ? jj : gi;
                    const float pv = (gs == jj) ? ajj : prow[jj];
                    s_gs = gs;
                    s_pv = pv;
                    s_rinv = (pv != 0.0f && fabsf(pv) >= FLT_MIN) ? 1.0f / pv : 0.0f;
                    if (b == 0) {
                        ipiv[j0 + jj] = j0 + gs + 1;
                        if (pv == 0.0f && *info == 0) *info = j0 + jj + 1;
                    }
                }
            }
        }
        __syncthreads();                                             // B3
        if (s_abort) return;
        const int gs = s_gs;
        const float pv = s_pv, rinv = s_rinv;
        const bool swap = (pv != 0.0f) && (gs != jj);
        const float *P = (gs == jj) ? orow : prow;                   // new row jj

        // -- [E] per owned row: interchange, scaling, rank-1 update of the
        // columns > jj (deferred beyond jj + 1 when W > 1), and the pivot key
        // for column jj+1
        nbk = kKeyNone;
        nbi = INT_MAX;
        if (lanes) {
            const int r = tid / W, q = tid % W;
            const bool act = r < nr;
            const int g = rb + r;
            const bool to_jj = act && swap && g == jj, from_gs = act && swap && g == gs;
            float l0 = 0.0f;
            if (act && q == 0) l0 = from_gs ? orow[jj] : S[jj * R + r];
            float l = __shfl_sync(0xffffffffu, l0, lane & ~(W - 1));
            if (to_jj) {
                for (int c = q; c < jb; c += W) S[c * R + r] = P[c];
            } else if (act && g > jj) {
                if (from_gs)
                    for (int c = q; c < jj; c += W) S[c * R + r] = orow[c];
                if (pv != 0.0f) l = (rinv != 0.0f) ? l * rinv : l / pv;
                if (q == 0 && pv != 0.0f) S[jj * R + r] = l;
                const float *old = from_gs ? orow : nullptr;
                if (defer) {
                    if (q == 0 && jj + 1 < jb) {
                        const int c = jj + 1;
                        const float v = fmaf(-P[c], l, old ? old[c] : S[c * R + r]);
                        S[c * R + r] = v;
                        nbk = pivot_key32(v);
                        nbi = g;
                    }
                    pend = jj + 2 + q < jb;
                    pend_gs = from_gs;
                    pend_l = l;
                } else {
                    int c = jj + 1 + q;
                    for (; c + 3 * W < jb; c += 4 * W) {
                        float v[4];
#pragma unroll
                        for (int u = 0; u < 4; ++u) v[u] = old ? old[c + u * W] : S[(c + u * W) * R + r];
#pragma unroll
                        for (int u = 0; u < 4; ++u) S[(c + u * W) * R + r] = fmaf(-P[c + u * W], l, v[u]);
                    }
                    for (; c < jb; c += W) S[c * R + r] = fmaf(-P[c], l, old ? old[c] : S[c * R + r]);
                    if (q == 0 && jj + 1 < jb) {
                        nbk = pivot_key32(S[(jj + 1) * R + r]);
                        nbi = g;
                    }
                }
            }
            if (defer) {
                dP = P;
                d_jj = jj;
                d_gs = gs;
                d_swap = swap;
            }
        } else
        for (int r = tid; r < nr; r += PANEL_THREADS) {
            const int g = rb + r;
            if (swap && g == jj) {
                for (int c = 0; c < jb; ++c) S[c * R + r] = P[c];
            } else if (swap && g == gs) {
                for (int c = 0; c < jb; ++c) S[c * R + r] = orow[c];
            }
            if (g > jj) {
                float l = S[jj * R + r];
                if (pv != 0.0f) {
                    l = (rinv != 0.0f) ? l * rinv : l / pv;
                    S[jj * R + r] = l;
                }
                for (int c = jj + 1; c < jb; ++c) S[c * R + r] = fmaf(-P[c], l, S[c * R + r]);
                if (jj + 1 < jb) {
                    const unsigned long long key = pivot_key32(S[(jj + 1) * R + r]);
                    if (better(key, g, nbk, nbi)) { nbk = key; nbi = g; }
                }
            }
        }
    }
    __syncthreads();

    for (int e = tid; e < nr * jb; e += PANEL_THREADS) {
        const int r = e % nr, c = e / nr;
        A[(size_t)(rb + r) + (size_t)c * lda] = S[c * R + r];
    }

    // -- block 0, warp 0: the jb interchanges as (dst, src) row moves.
    if (b == 0 && tid < 32) panel_moves(jb, j0, ipiv, ps, s_list_row, s_list_src, lane);
}

// Apply the panel's row moves to columns [0, cSplit) and [cSplit+skip, ...),
// ncols columns in total; one warp per column.
template <typename T>
__global__ void __launch_bounds__(256)
laswp_pairs_kernel(T *__restrict__ A, int lda, int ncols, int cSplit, int skip,
                   const int *__restrict__ cntp, const int *__restrict__ dst,
                   const int *__restrict__ src) {
    __shared__ int s_dst[2 * PANEL_NB], s_src[2 * PANEL_NB];
    const int cnt = *cntp;
    if (cnt == 0) return;
    for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
        s_dst[e] = dst[e];
        s_src[e] = src[e];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int q = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (q >= ncols) return;
    const int c = q < cSplit ? q : q + skip;
    T *col = A + (size_t)c * lda;
    T v[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        const int e = lane + 32 * t;
        if (e < cnt) v[t] = col[s_src[e]];
    }
    __syncwarp();
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        const int e = lane + 32 * t;
        if (e < cnt) col[s_dst[e]] = v[t];
    }
}

// ---- laswp with an arbitrary pivot range (used by trs) ----------------------
// perm[r] = source row of row r after the interchanges i <-> piv(i) for
// i = k1..k2 (inc > 0) or k2..k1 (inc < 0); one thread walks the pivots in
// order (the interchanges do not commute), the permutation lives in shared
// memory when it fits.
__global__ void laswp_perm_kernel(int nrows, int k1, int k2, const int *__restrict__ ipiv,
                                  int inc, int *__restrict__ perm_g, int use_smem) {
    extern __shared__ int perm_s[];
    int *perm = use_smem ? perm_s : perm_g;
    for (int r = threadIdx.x; r < nrows; r += blockDim.x) perm[r] = r;
    __syncthreads();
    if (threadIdx.x == 0) {
        if (inc > 0) {
            for (int i = k1; i <= k2; ++i) {
                const int p = ipiv[i - 1] - 1, a = i - 1;
                if (p != a && p >= 0 && p < nrows) { const int t = perm[a]; perm[a] = perm[p]; perm[p] = t; }
            }
        } else {
            for (int i = k2; i >= k1; --i) {
                const int p = ipiv[i - 1] - 1, a = i - 1;
                if (p != a && p >= 0 && p < nrows) { const int t = perm[a]; perm[a] = perm[p]; perm[p] = t; }
            }
        }
    }
    __syncthreads();
    if (use_smem)
        for (int r = threadIdx.x; r < nrows; r += blockDim.x) perm_g[r] = perm[r];
}

// tmp[:, c] = A[perm, c] for the first nrows rows
template <typename T>
__global__ void gather_rows_kernel(int nrows, int ncols, const T *__restrict__ A, int lda,
                                   const int *__restrict__ perm, T *__restrict__ tmp) {
    const size_t total = (size_t)nrows * ncols;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const size_t c = e / nrows, r = e % nrows;
        tmp[e] = A[(size_t)perm[r] + c * lda];
    }
}

template <typename T>
__global__ void copy_back_kernel(int nrows, int ncols, const T *__restrict__ tmp,
                                 T *__restrict__ A, int lda) {
    const size_t total = (size_t)nrows * ncols;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const size_t c = e / nrows, r = e % nrows;
        A[r + c * lda] = tmp[e];
    }
}

template <typename T>
int trsm_t(char side, char uplo, char ta, char diag, int m, int n, T alpha, const T *A, int ldA,
           T *B, int ldB, cudaStream_t s);
template <>
int trsm_t<double>(char side, char uplo, char ta, char diag, int m, int n, double alpha,
                   const double *A, int ldA, double *B, int ldB, cudaStream_t s) {
    return dtrsm_launch(side, uplo, ta, diag, m, n, alpha, A, ldA, B, ldB, s);
}
template <>
int trsm_t<float>(char side, char uplo, char ta, char diag, int m, int n, float alpha,
                  const float *A, int ldA, float *B, int ldB, cudaStream_t s) {
    return strsm_launch(side, uplo, ta, diag, m, n, alpha, A, ldA, B, ldB, s);
}
template <typename T>
int gemm_tt(char ta, char tb, int m, int n, int k, T alpha, const T *A, int ldA, const T *B,
            int ldB, T beta, T *C, int ldC, cudaStream_t s);
template <>
int gemm_tt<double>(char ta, char tb, int m, int n, int k, double alpha, const double *A, int ldA,
                    const double *B, int ldB, double beta, double *C, int ldC, cudaStream_t s) {
    return dgemm_launch(ta, tb, m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC, s);
}
template <>
int gemm_tt<float>(char ta, char tb, int m, int n, int k, float alpha, const float *A, int ldA,
                   const float *B, int ldB, float beta, float *C, int ldC, cudaStream_t s) {
    return sgemm_launch(ta, tb, m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC, s);
}

// The outer trailing update A22 -= L21 * U12 of the two-level LU: through the
// split GEMM for FP64 storage, on the tensor cores in `tc_kind` for FP32.
template <typename T>
int outer_update(int m, int n, int k, const T *L21, int ldL, const T *U12, int ldU, T *A22,
                 int ldA22, size_t ws0_off, int tc_kind, void *tc_buf, cudaStream_t s);
template <>
int outer_update<double>(int m, int n, int k, const double *L21, int ldL, const double *U12,
                         int ldU, double *A22, int ldA22, size_t ws0_off, int, void *,
                         cudaStream_t s) {
    return dgemm_split_launch_at('N', 'N', m, n, k, -1.0, L21, ldL, U12, ldU, 1.0, A22, ldA22, 0,
                                 nullptr, ws0_off, s);
}
template <>
int outer_update<float>(int m, int n, int k, const float *L21, int ldL, const float *U12, int ldU,
                        float *A22, int ldA22, size_t, int tc_kind, void *tc_buf, cudaStream_t s) {
    if (tc_kind < 0) {
        set_last_error("getrf: an FP32 outer update needs a tensor-core kind");
        return kErrUnsupported;
    }
    return tc_trailing_update(tc_kind, m, n, k, L21, ldL, U12, ldU, A22, ldA22, tc_buf, s);
}

// The FP32 panel (panel32_kernel) for FP32 storage: on unless
// FLENS_GB300_PANEL32=0, which factors FP32 panels with panel_kernel<float>
// (FP64 arithmetic on the FP32 values).
bool panel32_enabled() {
    static bool on = [] {
        const char *e = getenv("FLENS_GB300_PANEL32");
        return !(e && atoi(e) == 0);
    }();
    return on;
}

// Look-ahead in the blocked LU: on unless FLENS_GB300_LOOKAHEAD=0.
bool lookahead_enabled() {
    static bool on = [] {
        const char *e = getenv("FLENS_GB300_LOOKAHEAD");
        return !(e && atoi(e) == 0);
    }();
    return on;
}

// CTAs of a panel grid: at most one per SM and PANEL_GMAX, or
// FLENS_GB300_PANEL_CTAS when set (1..that bound).
int panel_ctas(int sms) {
    int cap = sms < PANEL_GMAX ? sms : PANEL_GMAX;
    static int env = [] {
        const char *e = getenv("FLENS_GB300_PANEL_CTAS");
        return e ? atoi(e) : 0;
    }();
    if (env >= 1 && env < cap) cap = env;
    return cap;
}

// Outer block of the split-update LU: FLENS_GB300_SPLIT_NB (a multiple of 64),
// else 512.
int split_outer_nb() {
    static int nb = [] {
        const char *e = getenv("FLENS_GB300_SPLIT_NB");
        const int v = e ? atoi(e) : 0;
        return (v >= 64 && v % 64 == 0) ? v : 512;
    }();
    return nb;
}

// Outer block of the tensor-core LU (FLENS_GB300_TC_NB, a multiple of 64; 64
// = one level): its trailing updates have this depth, so they read and write
// the FP32 C once per outer block instead of once per 64 columns.  At
// n = 16384 the updates took 49.8, 28.0 and 17.3 ms for 64, 128 and 256.
int tc_outer_nb() {
    static int nb = [] {
        const char *e = getenv("FLENS_GB300_TC_NB");
        const int v = e ? atoi(e) : 0;
        return (v >= 64 && v % 64 == 0) ? v : 256;
    }();
    return nb;
}

}  // namespace

template <typename T>
int laswp_launch_t(int nrows, int ncols, T *A, int ldA, int k1, int k2, const int *ipiv, int inc,
                   cudaStream_t stream) {
    if (nrows <= 0 || ncols <= 0 || k2 < k1) return kOk;
    const size_t permBytes = ((size_t)nrows * sizeof(int) + 255) / 256 * 256;
    const size_t tmpBytes = (size_t)nrows * ncols * sizeof(T);
    Workspace *w = workspace_for(stream, permBytes + tmpBytes);
    if (!w) return kErrAlloc;
    int *perm = (int *)w->buf;
    T *tmp = (T *)((char *)w->buf + permBytes);
    const int use_smem = (size_t)nrows * sizeof(int) <= 200 * 1024 ? 1 : 0;
    if (use_smem) {
        static DeviceOnce once;
        const int st0 = set_smem_once(once, (const void *)laswp_perm_kernel, 200 * 1024);
        if (st0 != kOk) return st0;
    }
    KTimer kt(kFamLaswp, stream, 0.0, 4.0 * sizeof(T) * (double)nrows * ncols);
    laswp_perm_kernel<<<1, 1024, use_smem ? (size_t)nrows * sizeof(int) : 0, stream>>>(
        nrows, k1, k2, ipiv, inc, perm, use_smem);
    FG_CUDA(cudaGetLastError());
    const size_t total = (size_t)nrows * ncols;
    int blocks = (int)ceil_div(total, (size_t)256);
    if (blocks > num_sms() * 16) blocks = num_sms() * 16;
    gather_rows_kernel<T><<<blocks, 256, 0, stream>>>(nrows, ncols, A, ldA, perm, tmp);
    FG_CUDA(cudaGetLastError());
    copy_back_kernel<T><<<blocks, 256, 0, stream>>>(nrows, ncols, tmp, A, ldA);
    FG_CUDA(cudaGetLastError());
    return kOk;
}

// perm[r] = source row of row r after the interchanges ipiv(1..nrows): the
// forward laswp as one gather (used by the solves of the precision form).
int laswp_perm_launch(int nrows, const int *ipiv, int *perm, cudaStream_t stream) {
    if (nrows <= 0) return kOk;
    const int use_smem = (size_t)nrows * sizeof(int) <= 200 * 1024 ? 1 : 0;
    if (use_smem) {
        static DeviceOnce once;
        const int st0 = set_smem_once(once, (const void *)laswp_perm_kernel, 200 * 1024);
        if (st0 != kOk) return st0;
    }
    KTimer kt(kFamLaswp, stream, 0.0, 8.0 * nrows);
    laswp_perm_kernel<<<1, 1024, use_smem ? (size_t)nrows * sizeof(int) : 0, stream>>>(
        nrows, 1, nrows, ipiv, 1, perm, use_smem);
    FG_CUDA(cudaGetLastError());
    return kOk;
}

int dlaswp_launch(int nrows, int ncols, double *A, int ldA, int k1, int k2, const int *ipiv,
                  int inc, cudaStream_t stream) {
    return laswp_launch_t<double>(nrows, ncols, A, ldA, k1, k2, ipiv, inc, stream);
}

int slaswp_launch(int nrows, int ncols, float *A, int ldA, int k1, int k2, const int *ipiv,
                  int inc, cudaStream_t stream) {
    return laswp_launch_t<float>(nrows, ncols, A, ldA, k1, k2, ipiv, inc, stream);
}

// Bytes of slot-0 workspace the blocked LU needs: the panel exchange area
// plus, for a tensor-core trailing update, its operand buffers.
size_t getrf_workspace_bytes(int m, int n, int tc_kind, int depth) {
    size_t b = (panel_scratch_bytes() + 255) / 256 * 256;
    if (tc_kind >= 0) b += tc_update_workspace_bytes(tc_kind, m, n, depth > PANEL_NB ? depth : PANEL_NB);
    return b;
}

// Blocked right-looking LU over storage T.  Panel, interchanges and the U12
// solve always run here; the trailing update A22 -= A21*U12 runs in T on the
// CUDA cores (tc_kind < 0) or, for T = float, on the tensor cores in the
// precision `tc_kind` (see tc_gemm.cu).
//
// split_nb > 0: two-level blocking.  The 64-column steps of an outer block
// of split_nb columns update only the columns of that block (their
// interchanges still reach every column); when the block is done,
// U12 = L11^-1 A12 for all columns to its right (trsm in T) and
// A22 -= L21 U12 with depth split_nb, through the split GEMM for T = double
// and on the tensor cores in `tc_kind` for T = float.  This is the order of
// LAPACK's dgetrf with a recursive panel; in exact arithmetic the factors
// and pivots are those of the right-looking loop.
template <typename T>
int getrf_t(int m, int n, T *A, int ldA, int *ipiv, int *info, int tc_kind, int split_nb,
            cudaStream_t stream) {
    FG_CUDA(cudaMemsetAsync(info, 0, sizeof(int), stream));
    if (m == 0 || n == 0) return kOk;
    const int mn = m < n ? m : n;
    const size_t ws0 = getrf_workspace_bytes(m, n, tc_kind, split_nb);
    // the split GEMM's slot-0 data goes after ours; sized for the largest
    // update now so that slot 0 never moves under the panel scratch
    const size_t split_off = (ws0 + 255) / 256 * 256;
    const bool fp64_split = split_nb > 0 && tc_kind < 0;
    Workspace *w = workspace_for(stream, fp64_split ? split_off + split_ws0_bytes(m, n) : ws0);
    if (!w) return kErrAlloc;
    PanelScratch ps = carve_panel_scratch(w->buf);
    void *tc_buf = (char *)w->buf + (panel_scratch_bytes() + 255) / 256 * 256;
    FG_CUDA(cudaMemsetAsync(ps.slots, 0, kSlotBytes, stream));
    unsigned long long epoch = 0;
    // FP32 storage: the FP32 panel (panel32_kernel); FP64: panel_kernel
    const bool f32 = std::is_same<T, float>::value && panel32_enabled();
    const void *panel_fn[2] = {
        f32 ? (const void *)panel32_kernel<false> : (const void *)panel_kernel<T, false>,
        f32 ? (const void *)panel32_kernel<true> : (const void *)panel_kernel<T, true>};
    {
        static DeviceOnce once, once_d, once_f, once_fd;
        int st0 = set_smem_once(f32 ? once_f : once, panel_fn[0], (int)PANEL_SMEM_MAX);
        if (st0 == kOk) st0 = set_smem_once(f32 ? once_fd : once_d, panel_fn[1], (int)PANEL_SMEM_MAX);
        if (st0 != kOk) return st0;
    }
    int sms = num_sms();
    if (sms <= 0) {
        set_last_error("no CUDA device");
        return kErrNoDevice;
    }
    const int gcap = panel_ctas(sms);
    // look-ahead (CUDA-core updates only: the tensor-core update is a
    // persistent kernel that leaves no SM free for a concurrent panel; with
    // its operand ring cut to 3 stages so that a panel CTA fits beside it, the
    // n = 16384 FP32 LU spent 114 ms in its updates instead of 49 and the
    // panels did not shorten)
    Workspace *wl = nullptr;
    if (tc_kind < 0 && lookahead_enabled()) {
        wl = workspace_side(stream);
        if (!wl) return kErrCuda;
    }
    trace("getrf<%d> m=%d n=%d lda=%d panel grid<=%d update=%d lookahead=%d", (int)sizeof(T), m, n,
          ldA, gcap, tc_kind, wl ? 1 : 0);

    // columns [ob_start, ob_end) are updated by the 64-column steps
    int ob_start = 0;
    int ob_end = (split_nb > 0 && split_nb < mn) ? split_nb : n;

    // Launches the panel at column j on stream s; *jb_out = its width.
    // `defer`: overlap the panel's own rank-1 updates with its exchanges --
    // asked for when nothing large runs beside the panel.  Beside a big
    // trailing update it measured slower overall (the n = 8192 LU: 325.3
    // against 322.8 ms per solve; the GEMM took 3 ms longer, the hidden
    // panels 6 ms less), since the panel's FP64 work then competes with the
    // GEMM's on the shared SMs.
    auto panel_at = [&](int j, cudaStream_t s, int *jb_out, bool defer) -> int {
        int mp = m - j;
        int R = ceil_div(mp, gcap);
        if (R < PANEL_RMIN) R = PANEL_RMIN;
        // panel width: the reference's 64, narrowed only if a CTA's rows
        // would not fit in shared memory (very tall matrices)
        // (panel_kernel holds the panel in FP64, panel32_kernel in FP32)
        const size_t es = f32 ? sizeof(float) : sizeof(double);
        int nb = PANEL_NB;
        while (nb > 1 && (size_t)R * nb * es > PANEL_SMEM_MAX) nb >>= 1;
        if ((size_t)R * nb * es > PANEL_SMEM_MAX) {
            set_last_error("getrf: m=%d too tall for the shared-memory panel", m);
            return kErrUnsupported;
        }
        int jb = (mn - j) < nb ? (mn - j) : nb;
        if (j + jb > ob_end) jb = ob_end - j;
        const int G = ceil_div(mp, R);
        T *Ap = A + j + (size_t)j * ldA;
        int *status = w->status;
        int j0 = j;
        size_t smem = (size_t)R * jb * es;
        ++epoch;
        void *args[] = {&Ap, &ldA, &mp, &jb, &j0, &ipiv, &info, &status, &ps, &R, &epoch};
        KTimer ktp(kFamPanel, s, (double)mp * jb * jb - (double)jb * jb * jb / 3.0,
                   2.0 * sizeof(T) * (double)mp * jb);
        const void *fn = panel_fn[defer ? 1 : 0];
        FG_CUDA(cudaLaunchCooperativeKernel(fn, dim3(G),
                                            dim3(PANEL_THREADS), args, smem, s));
        *jb_out = jb;
        return kOk;
    };
    auto update = [&](int j, int jb, int c0, int nc) -> int {
        // A(j+jb:m, c0:c0+nc) -= A(j+jb:m, j:j+jb) * A(j:j+jb, c0:c0+nc)
        T *A21 = A + (j + jb) + (size_t)j * ldA;
        T *U12 = A + j + (size_t)c0 * ldA;
        T *A22 = A + (j + jb) + (size_t)c0 * ldA;
        if (tc_kind >= 0)
            return tc_trailing_update(tc_kind, m - j - jb, nc, jb, (const float *)A21, ldA,
                                      (const float *)U12, ldA, (float *)A22, ldA, tc_buf, stream);
        return gemm_tt<T>('N', 'N', m - j - jb, nc, jb, T(-1), A21, ldA, U12, ldA, T(1), A22, ldA,
                          stream);
    };

    bool ahead = false;     // the panel at j was launched on the side stream
    auto body = [&]() -> int {
        int jb = 0, st;
        for (int j = 0; j < mn;) {
            if (ahead) {
                FG_CUDA(cudaStreamWaitEvent(stream, wl->ev_back, 0));
                ahead = false;
            } else if ((st = panel_at(j, stream, &jb, true)) != kOk) {
                return st;
            }
            // interchanges on the columns outside the panel
            const int ncols = n - jb;
            if (ncols > 0) {
                const int blocks = ceil_div(ncols, 256 / 32);
                KTimer ktl(kFamLaswp, stream, 0.0, 0.0);
                laswp_pairs_kernel<T><<<blocks, 256, 0, stream>>>(A, ldA, ncols, j, jb, ps.swap_cnt,
                                                                  ps.swap_dst, ps.swap_src);
                FG_CUDA(cudaGetLastError());
            }
            int next_jb = 0;
            if (j + jb < ob_end) {
                const int nr = ob_end - j - jb;
                if ((st = trsm_t<T>('L', 'L', 'N', 'U', jb, nr, T(1), A + j + (size_t)j * ldA, ldA,
                                    A + j + (size_t)(j + jb) * ldA, ldA, stream)) != kOk)
                    return st;
                if (j + jb < m) {
                    const int nx = j + jb;
                    if (wl && nx < mn) {
                        // the next panel's columns first, then that panel on
                        // the side stream while the rest of the update runs
                        const int w2 = std::min(std::min(PANEL_NB, mn - nx), nr);
                        if ((st = update(j, jb, nx, w2)) != kOk) return st;
                        FG_CUDA(cudaEventRecord(wl->ev_fwd, stream));
                        FG_CUDA(cudaStreamWaitEvent(wl->side, wl->ev_fwd, 0));
                        // defer when the update beside the panel is small
                        // (under ~4M elements: about the panel's own time)
                        const bool small = (double)(m - j - jb) * (double)(nr - w2) < 4.0e6;
                        if ((st = panel_at(nx, wl->side, &next_jb, small)) != kOk) return st;
                        FG_CUDA(cudaEventRecord(wl->ev_back, wl->side));
                        ahead = true;
                        if (next_jb > w2) {
                            set_last_error("getrf: look-ahead panel wider than its update");
                            return kErrUnsupported;
                        }
                        if (nr > w2 && (st = update(j, jb, nx + w2, nr - w2)) != kOk) return st;
                    } else if ((st = update(j, jb, j + jb, nr)) != kOk) {
                        return st;
                    }
                }
            }
            j += jb;
            if (ahead) jb = next_jb;
            if (j == ob_end && ob_end < n) {
                // outer block [ob_start, ob_end) done: its U12 and the trailing
                // update of everything to the right
                const int kb = ob_end - ob_start, nr = n - ob_end;
                if ((st = trsm_t<T>('L', 'L', 'N', 'U', kb, nr, T(1),
                                    A + ob_start + (size_t)ob_start * ldA, ldA,
                                    A + ob_start + (size_t)ob_end * ldA, ldA, stream)) != kOk)
                    return st;
                if (ob_end < m) {
                    st = outer_update(m - ob_end, nr, kb, A + ob_end + (size_t)ob_start * ldA, ldA,
                                      A + ob_start + (size_t)ob_end * ldA, ldA,
                                      A + ob_end + (size_t)ob_end * ldA, ldA, split_off, tc_kind,
                                      tc_buf, stream);
                    if (st != kOk) return st;
                }
                ob_start = ob_end;
                ob_end = (ob_start + split_nb < mn) ? ob_start + split_nb : n;
            }
        }
        return kOk;
    };
    const int st = body();
    // never leave side-stream work unjoined, also on an error path
    if (ahead) cudaStreamWaitEvent(stream, wl->ev_back, 0);
    return st;
}

int dgetrf_launch(int m, int n, double *A, int ldA, int *ipiv, int *info, cudaStream_t stream) {
    return getrf_t<double>(m, n, A, ldA, ipiv, info, -1, 0, stream);
}

int dgetrf_split_launch(int m, int n, double *A, int ldA, int *ipiv, int *info, int outer_nb,
                        cudaStream_t stream) {
    if (outer_nb <= 0) outer_nb = split_outer_nb();
    if (outer_nb % PANEL_NB != 0) {
        set_last_error("dgetrf_split: outer block %d is not a multiple of %d", outer_nb, PANEL_NB);
        return kErrUnsupported;
    }
    return getrf_t<double>(m, n, A, ldA, ipiv, info, -1, outer_nb, stream);
}

int sgetrf_launch(int m, int n, float *A, int ldA, int *ipiv, int *info, int tc_kind,
                  cudaStream_t stream) {
    const int onb = tc_kind >= 0 ? tc_outer_nb() : 0;
    return getrf_t<float>(m, n, A, ldA, ipiv, info, tc_kind, onb > PANEL_NB ? onb : 0, stream);
}

template <typename T>
int getrs_t(char trans, int n, int nrhs, const T *A, int ldA, const int *ipiv, T *B, int ldB,
            cudaStream_t stream) {
    if (n == 0 || nrhs == 0) return kOk;
    int st;
    if (trans == 'N' || trans == 'n') {
        if ((st = laswp_launch_t<T>(n, nrhs, B, ldB, 1, n, ipiv, 1, stream)) != kOk) return st;
        if ((st = trsm_t<T>('L', 'L', 'N', 'U', n, nrhs, T(1), A, ldA, B, ldB, stream)) != kOk) return st;
        return trsm_t<T>('L', 'U', 'N', 'N', n, nrhs, T(1), A, ldA, B, ldB, stream);
    }
    if ((st = trsm_t<T>('L', 'U', 'T', 'N', n, nrhs, T(1), A, ldA, B, ldB, stream)) != kOk) return st;
    if ((st = trsm_t<T>('L', 'L', 'T', 'U', n, nrhs, T(1), A, ldA, B, ldB, stream)) != kOk) return st;
    return laswp_launch_t<T>(n, nrhs, B, ldB, 1, n, ipiv, -1, stream);
}

int dgetrs_launch(char trans, int n, int nrhs, const double *A, int ldA, const int *ipiv,
                  double *B, int ldB, cudaStream_t stream) {
    return getrs_t<double>(trans, n, nrhs, A, ldA, ipiv, B, ldB, stream);
}

int sgetrs_launch(char trans, int n, int nrhs, const float *A, int ldA, const int *ipiv, float *B,
                  int ldB, cudaStream_t stream) {
    return getrs_t<float>(trans, n, nrhs, A, ldA, ipiv, B, ldB, stream);
}

}  // namespace fg

// ---------------------------------------------------------------------------
// Solve without allocating: flens_gb300_dgetrs_noalloc.
//
// Some callers cannot call cudaMalloc once they are running: a service that
// reserves all of its device memory up front and must not grow it on the
// request path, code that runs inside a pre-allocated memory pool owned by
// another framework, or a host that links this library into a process where
// device allocation is forbidden after start-up (a failed or blocking
// cudaMalloc there would stall or abort the caller).  flens_gb300_dgetrs
// takes its scratch (the row permutation and gathered right-hand sides of the
// row interchanges, and for up to 4 right-hand sides the ready flags and
// status word of the chained triangular solve) from a per-stream workspace
// that it creates with cudaMalloc on first use; this entry point takes all of
// it from the fixed file-scope array below instead and calls no allocating
// routine.
//
// Limits and rules:
//  * the array holds 8 MiB: 32 KiB of chain flags, a 256-byte status word,
//    and round_up(4*n, 256) + 8*n*nrhs bytes of interchange scratch per call
//    (n = 8192 allows nrhs <= 127); larger calls are rejected with
//    FLENS_GB300_ERR_UNSUPPORTED and a message in flens_gb300_last_error();
//  * every GPU that loads the library holds the array until the process exits;
//  * all calls on a device share the one array: calls whose work overlaps on
//    the GPU (different streams, or different host threads) race on it and
//    must be serialised by the caller;
//  * the first call on a device looks the array's device address up
//    (cudaGetSymbolAddress); use inside a captured CUDA graph is not tested.
// The array keeps the last call's contents.  What must start at zero is
// cleared on the call's stream by each call (cudaMemsetAsync, which does not
// allocate): the chain flags before every chained solve, and the status
// word.  The permutation is rebuilt from the identity and the gather buffer
// is fully written before it is read.  The chained solve's waits are bounded;
// a wait that gave up (not expected: every block of that cooperative launch is
// resident) leaves its bit in the array's status word, where this entry point
// does not report it.
namespace fg {
namespace {

constexpr size_t kNoAllocScratchBytes = 8u << 20;
constexpr int kNoAllocFlags = 4096;                                   // chain flags
constexpr size_t kNoAllocHead = kNoAllocFlags * sizeof(unsigned long long) + 256;   // + status word
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mu;
void *g_noalloc_ptr[64];

// Device address of g_noalloc_scratch on the current device, looked up once
// per device with that device current.
int noalloc_scratch(void **out) {
    int dev = -1;
    FG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_last_error("device ordinal %d out of range", dev);
        return kErrUnsupported;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr)
            return cuda_fail(e != cudaSuccess ? e : cudaErrorInvalidSymbol,
                             "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return kOk;
}

size_t noalloc_needed(int nrows, int ncols) {
    return ((size_t)nrows * sizeof(int) + 255) / 256 * 256 +
           (size_t)nrows * (size_t)ncols * sizeof(double);
}

// Same row interchanges as dlaswp_launch, scratch taken from `scratch`.
int laswp_fixed(int nrows, int ncols, double *A, int ldA, int k1, int k2, const int *ipiv,
                int inc, void *scratch, cudaStream_t stream) {
    if (nrows <= 0 || ncols <= 0 || k2 < k1) return kOk;
    const size_t permBytes = ((size_t)nrows * sizeof(int) + 255) / 256 * 256;
    int *perm = (int *)scratch;
    double *tmp = (double *)((char *)scratch + permBytes);
    const int use_smem = (size_t)nrows * sizeof(int) <= 200 * 1024 ? 1 : 0;
    if (use_smem) {
        static DeviceOnce once;
        const int st0 = set_smem_once(once, (const void *)laswp_perm_kernel, 200 * 1024);
        if (st0 != kOk) return st0;
    }
    KTimer kt(kFamLaswp, stream, 0.0, 2.0 * (double)nrows * ncols * 16.0);
    laswp_perm_kernel<<<1, 1024, use_smem ? (size_t)nrows * sizeof(int) : 0, stream>>>(
        nrows, k1, k2, ipiv, inc, perm, use_smem);
    FG_CUDA(cudaGetLastError());
    const size_t total = (size_t)nrows * ncols;
    int blocks = (int)ceil_div(total, (size_t)256);
    if (blocks > num_sms() * 16) blocks = num_sms() * 16;
    gather_rows_kernel<double><<<blocks, 256, 0, stream>>>(nrows, ncols, A, ldA, perm, tmp);
    FG_CUDA(cudaGetLastError());
    copy_back_kernel<double><<<blocks, 256, 0, stream>>>(nrows, ncols, tmp, A, ldA);
    FG_CUDA(cudaGetLastError());
    return kOk;
}

}  // namespace
}  // namespace fg

FG_API int flens_gb300_dgetrs_noalloc(char trans, int n, int nrhs, const double *A, int ldA,
                                      const int *ipiv, double *B, int ldB, void *stream) {
    using namespace fg;
    if (trans >= 'a' && trans <= 'z') trans = (char)(trans - 'a' + 'A');
    if (trans != 'N' && trans != 'T' && trans != 'C') return -1;
    if (n < 0) return -2;
    if (nrhs < 0) return -3;
    if (ldA < (n > 1 ? n : 1)) return -5;
    if (ldB < (n > 1 ? n : 1)) return -8;
    if (n == 0 || nrhs == 0) return kOk;
    const size_t need = kNoAllocHead + noalloc_needed(n, nrhs);
    if (need > kNoAllocScratchBytes) {
        set_last_error("flens_gb300_dgetrs_noalloc: n=%d nrhs=%d needs %zu bytes of scratch, "
                       "more than its fixed %zu-byte array; use flens_gb300_dgetrs or fewer "
                       "right-hand sides per call", n, nrhs, need, kNoAllocScratchBytes);
        return kErrUnsupported;
    }
    void *base = nullptr;
    int st = noalloc_scratch(&base);
    if (st != kOk) return st;
    cudaStream_t s = (cudaStream_t)stream;
    ChainFixed fx;
    fx.flags = (unsigned long long *)base;
    fx.cap = kNoAllocFlags;
    fx.status = (int *)((char *)base + kNoAllocFlags * sizeof(unsigned long long));
    void *scratch = (char *)base + kNoAllocHead;
    FG_CUDA(cudaMemsetAsync(fx.status, 0, sizeof(int), s));
    if (trans == 'N') {
        if ((st = laswp_fixed(n, nrhs, B, ldB, 1, n, ipiv, 1, scratch, s)) != kOk) return st;
        if ((st = dtrsm_launch_fixed('L', 'L', 'N', 'U', n, nrhs, 1.0, A, ldA, B, ldB, fx, s)) != kOk)
            return st;
        return dtrsm_launch_fixed('L', 'U', 'N', 'N', n, nrhs, 1.0, A, ldA, B, ldB, fx, s);
    }
    if ((st = dtrsm_launch_fixed('L', 'U', 'T', 'N', n, nrhs, 1.0, A, ldA, B, ldB, fx, s)) != kOk)
        return st;
    if ((st = dtrsm_launch_fixed('L', 'L', 'T', 'U', n, nrhs, 1.0, A, ldA, B, ldB, fx, s)) != kOk)
        return st;
    return laswp_fixed(n, nrhs, B, ldB, 1, n, ipiv, -1, scratch, s);
}
