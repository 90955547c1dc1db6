// split_gemm.cu -- FP64-accurate GEMM from exact low-precision tensor-core
// products (exponent-aligned slices).
//
// C <- beta*C + alpha*op(A)*op(B), FP64 in and out, with the same operand
// conventions and checks as dgemm_ (flens/blas/interface/blas/gemm.cc:120-181
// -> cxxblas::gemm, cxxblas/level3/gemm.tcc:176-190).  GB300 has no FP64
// tensor-core kind, so the product is rebuilt from BF16 tensor-core products
// that are exact:
//
//  1. stats: every row i of op(A) gets an exponent e_i with
//     max_k |a_ik| < 2^(e_i - 1), every column j of op(B) an f_j (and
//     2^e_i * nnz_i / sum_k |a_ik|, which bounds how far the slicing error
//     can exceed u*|A||B|, for the automatic slice count);
//  2. digits: a_ik = 2^e_i * sum_{s=1..S} d_s 2^(-beta s) + r with balanced
//     digits |d_s| <= 2^(beta-1) (exact in BF16) and |r| <= 2^(e_i-beta S-1),
//     obtained by repeated rint / subtract / scale, all exact in FP64.  Slices
//     are stored K-major and concatenated along K: slice s of op(A) at
//     [(s-1)*Kp, s*Kp), slice t of op(B) at [(S-t)*Kp, (S-t+1)*Kp);
//  3. products: for every diagonal dg = s + t <= S + 1 the pairs (s, dg-s)
//     are contiguous in both concatenations, so a run of pairs is one plain
//     GEMM over a longer K.  Runs ("groups") are cut so that (#pairs) * K_run
//     * 4^(beta-1) <= 2^24: every FP32 partial sum is then an integer of
//     magnitude <= 2^24, and the tensor-core sums are exact;
//  4. recombination: the persistent tcgen05 kernel (tcgen05.cuh) visits each
//     128 x 256 tile of C once and runs all groups into alternating TMEM
//     accumulators; its epilogue sums S = sum_groups acc*2^(e_i+f_j-beta dg)
//     in FP64, smallest weights first (the scaling is exact exponent
//     arithmetic, the sum one FP64 add per group), and the last group of a
//     tile writes C = (beta*C) + (alpha*S).
//
// Every step but the stats reduction runs on integer, BF16 tensor and a
// minimum of FP64 instructions: GB300 issues FP64 at a small fraction of its
// integer rate.
//
// The slice count S follows from the data (beta*S >= 53 + log2 of the worst
// ratio above) unless the caller fixes it.  Non-finite entries, or exponents
// outside about 2^+-1000, go to the plain FP64 GEMM kernel instead.
#include "tcgen05.cuh"

#include <cuda_bf16.h>

#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>

namespace fg {

namespace {

constexpr int kMaxSlices = 20;
constexpr int kDefaultBits = 7;               // digits |d| <= 64
constexpr int kTargetBits = 51;               // + 2 guard bits + log2(ratio)
constexpr int kBK = 64;                        // k-block of the BF16 kernel (128 bytes)
constexpr long long kAccLimit = 1ll << 24;     // exact FP32 integers

struct SplitStats {
    int emin, emax, bad, pad;
    unsigned long long ratio_bits;             // max 2^e*nnz/sum|x| (positive double bits)
};

__device__ __forceinline__ double pow2(int e) {  // exact 2^e for e in [-1022, 1023]
    return __longlong_as_double((long long)(e + 1023) << 52);
}

constexpr unsigned long long kInfBits = 0x7FF0000000000000ull;

// |v| as its IEEE bit pattern: for finite values the integer order is the
// order of the magnitudes (the statistics run on the integer pipes; GB300's
// FP64 rate is a small fraction of its integer rate)
__device__ __forceinline__ unsigned long long abs_bits(double v) {
    return (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
}

__global__ void stats_init_kernel(SplitStats *st) {
    if (threadIdx.x < 2) {
        st[threadIdx.x].emin = INT_MAX;
        st[threadIdx.x].emax = INT_MIN;
        st[threadIdx.x].bad = 0;
        st[threadIdx.x].pad = 0;
        st[threadIdx.x].ratio_bits = 0ull;
    }
}

__device__ void finish_row(int r, double amax, int nnz, double sum, int bad, int *__restrict__ e_out,
                           SplitStats *st) {
    int ex = 0;
    if (amax > 0.0) frexp(amax, &ex);          // amax = m 2^ex, m in [0.5, 1)
    const int e = amax > 0.0 ? ex + 1 : 0;
    e_out[r] = e;
    atomicMin(&st->emin, e);
    atomicMax(&st->emax, e);
    if (bad) atomicOr(&st->bad, 1);
    if (sum > 0.0) {
        const double ratio = ldexp((double)nnz, e) / sum;
        if (ratio > 0.0 && ratio <= 1.0e300)
            atomicMax(&st->ratio_bits, (unsigned long long)__double_as_longlong(ratio));
    }
}

// Row statistics of op(X) (R rows of length K).  RCONTIG: element (r, k) at
// X[r + k*ld] (32 rows x 8 k-lanes per block, coalesced along r); otherwise at
// X[k + r*ld] (one warp per row, coalesced along k).
template <bool RCONTIG>
__global__ void __launch_bounds__(256)
split_stats_kernel(int R, int K, const double *__restrict__ X, int ld, int *__restrict__ e_out,
                   SplitStats *st) {
    double amax = 0.0, sum = 0.0;
    int nnz = 0, bad = 0;
    if (RCONTIG) {
        __shared__ double s_max[8][32], s_sum[8][32];
        __shared__ int s_nnz[8][32], s_bad[8][32];
        const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
        const int r = blockIdx.x * 32 + tx;
        unsigned long long mb = 0ull;
        if (r < R) {
            for (int k = ty; k < K; k += 8) {
                const unsigned long long b = abs_bits(X[(size_t)r + (size_t)k * ld]);
                bad |= b >= kInfBits;
                mb = b > mb ? b : mb;
                sum += __longlong_as_double((long long)b);
                nnz += b != 0ull;
            }
        }
        amax = __longlong_as_double((long long)mb);
        s_max[ty][tx] = amax;
        s_sum[ty][tx] = sum;
        s_nnz[ty][tx] = nnz;
        s_bad[ty][tx] = bad;
        __syncthreads();
        if (ty == 0 && r < R) {
            for (int j = 1; j < 8; ++j) {
                amax = fmax(amax, s_max[j][tx]);
                sum += s_sum[j][tx];
                nnz += s_nnz[j][tx];
                bad |= s_bad[j][tx];
            }
            finish_row(r, amax, nnz, sum, bad, e_out, st);
        }
    } else {
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        const int r = blockIdx.x * 8 + warp;
        if (r >= R) return;
        const double *x = X + (size_t)r * ld;
        unsigned long long mb = 0ull;
        for (int k = lane; k < K; k += 32) {
            const unsigned long long b = abs_bits(x[k]);
            bad |= b >= kInfBits;
            mb = b > mb ? b : mb;
            sum += __longlong_as_double((long long)b);
            nnz += b != 0ull;
        }
        amax = __longlong_as_double((long long)mb);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, off));
            sum += __shfl_xor_sync(0xffffffffu, sum, off);
            nnz += __shfl_xor_sync(0xffffffffu, nnz, off);
            bad |= __shfl_xor_sync(0xffffffffu, bad, off);
        }
        if (lane == 0) finish_row(r, amax, nnz, sum, bad, e_out, st);
    }
}

// Balanced base-2^bits digits of x = v 2^(bits - e) (|x| < 2^(bits-1)),
// written by emit_digits as BF16 at out[slot(s) * Kp] (slot(s) = s, or S-1-s
// when REVERSE).  d_s = R_s - 2^bits R_{s-1} with R_s = rint(x 2^(bits (s-1)))
// (round half to even) -- the digits of repeated rint / subtract / scale,
// since 2^bits R_{s-1} is even -- computed exactly on the 53-bit significand
// with integer operations.  R_s is only needed modulo 2^32, as
// |d_s| <= 2^(bits-1).
__host__ __device__ __forceinline__ int trailing_zeros64(long long m) {
#ifdef __CUDA_ARCH__
    return m ? __ffsll(m) - 1 : 64;
#else
    return m ? __builtin_ctzll((unsigned long long)m) : 64;
#endif
}

// Digit s (0-based) is produced by calling next() S times.
struct DigitGen {
    long long m;                                  // signed significand of v
    int tz, D, bits;
    unsigned int Rprev;

    __host__ __device__ DigitGen(double v, int e, int bits_) : bits(bits_), Rprev(0u) {
        unsigned long long u;
        memcpy(&u, &v, sizeof(u));
        const int bexp = (int)((u >> 52) & 0x7FF);
        m = (long long)(u & 0xFFFFFFFFFFFFFull);
        if (bexp) m |= 1ll << 52;
        const int p = bexp ? bexp - 1075 : -1074;    // |v| = m 2^p
        if (u >> 63) m = -m;
        tz = trailing_zeros64(m);
        D = e - bits - p;                             // R_1 = rint(m / 2^D)
    }
    __host__ __device__ int next() {
        unsigned int R;
        if (m == 0 || D >= 55) {
            R = 0u;                                   // |m| / 2^D < 1/4
        } else if (D <= 0) {
            R = -D >= 32 ? 0u : (unsigned int)m << (-D);   // exact multiple, mod 2^32
        } else {
            const long long fl = m >> D;              // floor(m / 2^D)
            const unsigned int half = (unsigned int)(m >> (D - 1)) & 1u;
            const bool up = half && (tz < D - 1 || (fl & 1));
            R = (unsigned int)fl + (up ? 1u : 0u);
        }
        const int d = (int)(R - (Rprev << bits));
        Rprev = R;
        D -= bits;
        return d;
    }
};

template <bool REVERSE>
__device__ __forceinline__ void emit_digits(double v, int e, int S, int bits, size_t Kp,
                                            __nv_bfloat16 *__restrict__ out) {
    DigitGen gen(v, e, bits);
    for (int s = 0; s < S; ++s)
        out[(size_t)(REVERSE ? S - 1 - s : s) * Kp] = __float2bfloat16_rn((float)gen.next());
}

// Digits of op(X) (R x K) into a K-major BF16 buffer of R rows x (S*Kp);
// columns K..Kp-1 of every slice are zero.  Grid (ceil(R/32), Kp/32), 256
// threads.  RCONTIG as for the stats: a 32 x 32 tile is staged through shared
// memory so that both the FP64 reads and the BF16 writes are coalesced.
template <bool RCONTIG, bool REVERSE>
__global__ void __launch_bounds__(256)
split_digits_kernel(int R, int K, int Kp, int S, int bits, const double *__restrict__ X, int ld,
                    const int *__restrict__ e_row, __nv_bfloat16 *__restrict__ out) {
    __shared__ double tile[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int r0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
    const size_t ldS = (size_t)S * Kp;
    if (RCONTIG) {
        for (int kk = ty; kk < 32; kk += 8) {
            const int r = r0 + tx, k = k0 + kk;
            tile[kk][tx] = (r < R && k < K) ? X[(size_t)r + (size_t)k * ld] : 0.0;
        }
    } else {
        for (int rr = ty; rr < 32; rr += 8) {
            const int r = r0 + rr, k = k0 + tx;
            tile[tx][rr] = (r < R && k < K) ? X[(size_t)k + (size_t)r * ld] : 0.0;
        }
    }
    __syncthreads();
    for (int rr = ty; rr < 32; rr += 8) {
        const int r = r0 + rr, k = k0 + tx;
        if (r < R && k < Kp) {
            emit_digits<REVERSE>(tile[tx][rr], e_row[r], S, bits, (size_t)Kp,
                                 out + (size_t)r * ldS + k);
        }
    }
}

// Groups of slice pairs, in summation order (diagonal dg from S+1 down to 2):
//   nchunks == 1: runs of up to `per` pairs (s, dg-s), s = 1.. over the whole
//                 padded K (Kp);
//   nchunks  > 1: one pair per group, chunks of kc along K, chunk-major.
struct SplitGeom {
    int S, bits, Kp, kc, nchunks, per, ngroups;

    __host__ __device__ int count(int dg) const {
        return nchunks == 1 ? (dg - 1 + per - 1) / per : (dg - 1) * nchunks;
    }
    __host__ __device__ void decode(int g, int &dg, int &slo, int &shi, int &k0, int &k1) const {
        int gi, cnt;
        decode(g, dg, slo, shi, k0, k1, gi, cnt);
    }
    // also: gi = the group's index within its diagonal, cnt = count(dg)
    __host__ __device__ void decode(int g, int &dg, int &slo, int &shi, int &k0, int &k1, int &gi,
                                    int &cnt) const {
        for (dg = S + 1; dg > 2; --dg) {
            const int c = count(dg);
            if (g < c) break;
            g -= c;
        }
        gi = g;
        cnt = count(dg);
        if (nchunks == 1) {
            slo = 1 + g * per;
            shi = slo + per - 1 < dg - 1 ? slo + per - 1 : dg - 1;
            k0 = 0;
            k1 = Kp;
        } else {
            const int c = g / (dg - 1);
            slo = shi = 1 + g % (dg - 1);
            k0 = c * kc;
            k1 = k0 + kc < Kp ? k0 + kc : Kp;
        }
    }
};

// Recombination epilogue.  Every group sum acc is an exact integer of
// magnitude <= 2^24 held in FP32, and all groups of one diagonal dg share the
// scale 2^(e_i + f_j - bits*dg).  So the groups of a diagonal are summed
// exactly in int32, in segments of at most kSegGroups groups (127 * 2^24 <
// 2^31), in Wi; at the end of a segment the integer sum is converted to FP64
// (exact), scaled by moving its exponent field (exact) and added to the FP64
// sum Wd (one rounding per segment, largest dg first).  The last segment of
// the last diagonal finishes C = (beta*C) + (alpha*S).  Per group this is an
// int32 read-modify-write of the CTA's group-sum tile and no FP64 work; the
// FP64 add and its 8-byte traffic come once per diagonal.  (Summing every
// group into FP64 costs one FP64 add and a 16-byte read-modify-write per
// element and group, and that epilogue, not the MMAs, bounded the kernel.)
constexpr int kSegGroups = 127;

struct EpiSplit {
    static constexpr int kBN = 256;
    static constexpr int kTmemExtra = 0;
    SplitGeom geo;
    double alpha, beta;
    double *C;
    int ldc;
    double *Wd;                                  // FP64 sums: one BM x BN tile per CTA
    int *Wi;                                     // int32 segment sums: one BM x BN tile per CTA
    const int *ea, *eb;                          // row exponents of op(A), column exponents of op(B)

    __device__ int groups() const { return geo.ngroups; }
    __device__ void prefetch(int, int, int, int, int) const {}
    __device__ void group(int g, int &ka, int &kb, int &nk) const {
        int dg, slo, shi, k0, k1;
        geo.decode(g, dg, slo, shi, k0, k1);
        ka = (slo - 1) * geo.Kp + k0;
        kb = (geo.S - (dg - slo)) * geo.Kp + k0;
        nk = (shi - slo + 1) * ((k1 - k0) / kBK);
    }
    __device__ void apply(int g, int row, bool row_ok, int col, int ncol,
                          const uint32_t (&r)[32], uint32_t) const {
        int dg, slo, shi, k0, k1, gi, cnt;
        geo.decode(g, dg, slo, shi, k0, k1, gi, cnt);
        const bool seg_first = gi % kSegGroups == 0;
        const bool seg_last = gi % kSegGroups == kSegGroups - 1 || gi == cnt - 1;
        const bool first = dg == geo.S + 1 && gi < kSegGroups;          // first segment of all
        const bool last = dg == 2 && gi == cnt - 1;                     // last segment of all
        // these depend on g only: uniform over the warp, whose lanes all take
        // part in the shuffles below
        const int lane = threadIdx.x & 31;
        const int fl = lane < ncol ? eb[col + lane] : 0;
        const int erow = row_ok ? ea[row] - geo.bits * dg : 0;
        const size_t r0 = (size_t)(row_ok ? row : 0);
        // this CTA's own tiles of sums, reused for each of its tiles: they
        // stay in L2 (152 x 384 KB) instead of spanning m x n
        const size_t off = (size_t)blockIdx.x * (tc::BM * kBN) + (r0 & (tc::BM - 1)) +
                           (size_t)(col & (kBN - 1)) * tc::BM;
        int *wi = Wi + off;
        // the segment's integer sums: all 32 loads in flight before any use
        int iv[32];
#pragma unroll
        for (int j = 0; j < 32; ++j)
            iv[j] = (!seg_first && row_ok && j < ncol) ? __ldcg(wi + (size_t)j * tc::BM) : 0;
#pragma unroll
        for (int j = 0; j < 32; ++j) iv[j] += __float2int_rn(__uint_as_float(r[j]));   // exact
        if (!seg_last) {
            if (row_ok) {
#pragma unroll
                for (int j = 0; j < 32; ++j)
                    if (j < ncol) __stcg(wi + (size_t)j * tc::BM, iv[j]);
            }
            return;
        }
        // end of a segment: S = S + I * 2^(e_i + f_j - bits*dg)
        double *wd = Wd + off;
        double *crow = C + r0 + (size_t)col * ldc;
#pragma unroll
        for (int h = 0; h < 32; h += 16) {
            double sv[16];
#pragma unroll
            for (int j = 0; j < 16; ++j)
                sv[j] = (!first && row_ok && h + j < ncol) ? __ldcg(wd + (size_t)(h + j) * tc::BM) : 0.0;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int sh = erow + __shfl_sync(0xffffffffu, fl, h + j);
                double v = 0.0;
                if (iv[h + j] != 0) {
                    const long long bits = __double_as_longlong(__int2double_rn(iv[h + j]));
                    v = __longlong_as_double(bits + ((long long)sh << 52));
                }
                sv[j] = first ? v : __dadd_rn(sv[j], v);
            }
            if (row_ok && !last) {
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    if (h + j < ncol) __stcg(wd + (size_t)(h + j) * tc::BM, sv[j]);
            } else if (row_ok) {
                double cv[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) cv[j] = h + j < ncol ? __ldcs(crow + (size_t)(h + j) * ldc) : 0.0;
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    if (h + j < ncol)
                        __stcs(crow + (size_t)(h + j) * ldc,
                               __dadd_rn(__dmul_rn(beta, cv[j]), __dmul_rn(alpha, sv[j])));
            }
        }
    }
};

size_t round256(size_t b) { return (b + 255) / 256 * 256; }


// ceil(log2(x)) for x >= 1, exact (frexp based)
int ceil_log2(double x) {
    int ex = 0;
    const double m = std::frexp(x, &ex);       // x = m 2^ex, m in [0.5, 1)
    return m == 0.5 ? ex - 1 : ex;
}

int split_bits() {
    const char *e = std::getenv("FLENS_GB300_SPLIT_BITS");
    if (e && *e) {
        const int b = std::atoi(e);
        if (b >= 2 && b <= 8) return b;
    }
    return kDefaultBits;
}

}  // namespace

// Geometry of the pair groups for digit width `bits`, S slices, inner
// dimension k (host side of SplitGeom).
static SplitGeom split_geometry(int bits, int S, int k) {
    SplitGeom g{};
    g.S = S;
    g.bits = bits;
    g.Kp = (k + kBK - 1) / kBK * kBK;
    const long long P = 1ll << (2 * (bits - 1));
    long long kc = (kAccLimit / P) / kBK * kBK;
    if (kc > g.Kp) kc = g.Kp;
    g.kc = (int)kc;
    g.nchunks = (g.Kp + g.kc - 1) / g.kc;
    g.per = g.nchunks == 1 ? (int)(kAccLimit / (P * g.Kp)) : 1;
    g.ngroups = 0;
    for (int dg = 2; dg <= S + 1; ++dg) g.ngroups += g.count(dg);
    return g;
}

// Bytes of slot-0 workspace the split GEMM uses for an m x n product: the
// statistics and the per-row / per-column exponents.
size_t split_ws0_bytes(int m, int n) {
    return 256 + round256((size_t)m * sizeof(int)) + round256((size_t)n * sizeof(int));
}

// The split GEMM with its slot-0 data at byte offset ws0_off (callers that
// keep their own data at the start of slot 0, the blocked LU, pass its size).
int dgemm_split_launch_at(char transA, char transB, int m, int n, int k, double alpha,
                          const double *A, int ldA, const double *B, int ldB, double beta, double *C,
                          int ldC, int slices, int *slices_used, size_t ws0_off, cudaStream_t s) {
    if (slices_used) *slices_used = 0;
    if (m == 0 || n == 0) return kOk;
    if (k == 0 || alpha == 0.0) return dscal_matrix_launch(m, n, beta, C, ldC, s);
    const bool ta = !(transA == 'N' || transA == 'n');
    const bool tb = !(transB == 'N' || transB == 'n');
    const int bits = split_bits();

    // 1. exponents and slice-count statistics (slot 0: small)
    const size_t off_ea = 256, off_eb = off_ea + round256((size_t)m * sizeof(int));
    Workspace *w = workspace_for(s, ws0_off + split_ws0_bytes(m, n));
    if (!w) return kErrAlloc;
    char *ws = (char *)w->buf + ws0_off;
    SplitStats *st = (SplitStats *)ws;
    int *ea = (int *)(ws + off_ea), *eb = (int *)(ws + off_eb);
    {
        KTimer kt(kFamAux, s, 0.0, 8.0 * ((double)m * k + (double)n * k));
        stats_init_kernel<<<1, 32, 0, s>>>(st);
        // op(A)(i, k) = ta ? A[k + i ldA] : A[i + k ldA]; op(B)^T(j, k) = tb ? B[j + k ldB] : B[k + j ldB]
        if (!ta) split_stats_kernel<true><<<ceil_div(m, 32), 256, 0, s>>>(m, k, A, ldA, ea, st);
        else split_stats_kernel<false><<<ceil_div(m, 8), 256, 0, s>>>(m, k, A, ldA, ea, st);
        if (tb) split_stats_kernel<true><<<ceil_div(n, 32), 256, 0, s>>>(n, k, B, ldB, eb, st + 1);
        else split_stats_kernel<false><<<ceil_div(n, 8), 256, 0, s>>>(n, k, B, ldB, eb, st + 1);
        FG_CUDA(cudaGetLastError());
    }
    SplitStats hs[2];
    FG_CUDA(cudaMemcpyAsync(hs, st, sizeof(hs), cudaMemcpyDeviceToHost, s));
    FG_CUDA(cudaStreamSynchronize(s));

    // 2. slice count and range checks
    int S = slices;
    if (S <= 0) {
        double worst = 1.0;
        for (int i = 0; i < 2; ++i) {
            double r;
            const long long b = (long long)hs[i].ratio_bits;
            std::memcpy(&r, &b, sizeof(r));
            if (r > worst) worst = r;
        }
        const int need = kTargetBits + 2 + ceil_log2(worst);
        S = (need + bits - 1) / bits;
    }
    if (S > kMaxSlices) S = kMaxSlices;
    const int lo = bits * (S + 1);
    const bool in_range = !hs[0].bad && !hs[1].bad && hs[0].emax <= 1000 && hs[1].emax <= 1000 &&
                          hs[0].emax + hs[1].emax <= 1000 && hs[0].emin - lo >= -1000 &&
                          hs[1].emin >= -1000 && hs[0].emin + hs[1].emin - lo >= -1000;
    if (!in_range) {
        trace("dgemm_split: non-finite entries or exponents out of range -> FP64 kernel");
        if (slices_used) *slices_used = -1;
        return dgemm_launch(transA, transB, m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC, s);
    }

    // 3. digits (slot 1)
    const SplitGeom geo = split_geometry(bits, S, k);
    const size_t ldS = (size_t)S * geo.Kp;
    const size_t bytesA = round256((size_t)m * ldS * 2), bytesB = round256((size_t)n * ldS * 2);
    char *dig = (char *)workspace_slot(s, 1, bytesA + bytesB);
    if (!dig) return kErrAlloc;
    __nv_bfloat16 *Ad = (__nv_bfloat16 *)dig, *Bd = (__nv_bfloat16 *)(dig + bytesA);
    {
        KTimer kt(kFamAux, s, 0.0, (8.0 + 2.0 * S) * ((double)m + n) * geo.Kp);
        const dim3 ga(ceil_div(m, 32), geo.Kp / 32), gb(ceil_div(n, 32), geo.Kp / 32);
        if (!ta) split_digits_kernel<true, false><<<ga, 256, 0, s>>>(m, k, geo.Kp, S, bits, A, ldA, ea, Ad);
        else split_digits_kernel<false, false><<<ga, 256, 0, s>>>(m, k, geo.Kp, S, bits, A, ldA, ea, Ad);
        if (tb) split_digits_kernel<true, true><<<gb, 256, 0, s>>>(n, k, geo.Kp, S, bits, B, ldB, eb, Bd);
        else split_digits_kernel<false, true><<<gb, 256, 0, s>>>(n, k, geo.Kp, S, bits, B, ldB, eb, Bd);
        FG_CUDA(cudaGetLastError());
    }

    // 4. exact products and FP64 recombination
    CUtensorMap ma, mb;
    int rc = tc::make_kmajor_map(&ma, kTcBF16, Ad, m, (int)ldS, (int)ldS, tc::BM);
    if (rc != kOk) return rc;
    if ((rc = tc::make_kmajor_map(&mb, kTcBF16, Bd, n, (int)ldS, (int)ldS, EpiSplit::kBN)) != kOk) return rc;
    if ((rc = tc::prepare_kernel<kTcBF16, EpiSplit>()) != kOk) return rc;
    const int ntiles = ceil_div(m, tc::BM) * ceil_div(n, EpiSplit::kBN);
    const int grid = ntiles < num_sms() ? ntiles : num_sms();
    const size_t tileB = (size_t)tc::BM * EpiSplit::kBN;
    char *W = (char *)workspace_slot(s, 2, (size_t)grid * tileB * (sizeof(double) + sizeof(int)));
    if (!W) return kErrAlloc;
    const EpiSplit epi{geo, alpha, beta, C, ldC, (double *)W,
                       (int *)(W + (size_t)grid * tileB * sizeof(double)), ea, eb};
    const double pairs = (double)S * (S + 1) / 2;
    KTimer kt(kFamSplit, s, 2.0 * pairs * m * (double)n * geo.Kp,
              2.0 * ldS * ((double)m + n) + 16.0 * m * (double)n);   // digits in, C in + out
    tc::tc_kernel<kTcBF16, EpiSplit><<<grid, tc::THREADS, tc::Shape<EpiSplit>::SMEM, s>>>(
        ma, mb, m, n, epi, w->status);
    FG_CUDA(cudaGetLastError());
    trace("dgemm_split: m=%d n=%d k=%d bits=%d S=%d groups=%d", m, n, k, bits, S, geo.ngroups);
    if (slices_used) *slices_used = S;
    return kOk;
}

int dgemm_split_launch(char transA, char transB, int m, int n, int k, double alpha, const double *A,
                       int ldA, const double *B, int ldB, double beta, double *C, int ldC,
                       int slices, int *slices_used, cudaStream_t s) {
    return dgemm_split_launch_at(transA, transB, m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC, slices,
                                 slices_used, 0, s);
}

}  // namespace fg

// ----------------------------------------------------------------- C ABI ----
// FP64-accurate C <- beta*C + alpha*op(A)*op(B) on device memory from exact
// BF16 tensor-core products of exponent-aligned slices.  Argument positions
// as dgemm_ (flens/blas/interface/blas/gemm.cc:158-181), slices at 14.
FG_API int flens_gb300_dgemm_split(char transA, char transB, int m, int n, int k, double alpha,
                                   const double *A, int ldA, const double *B, int ldB, double beta,
                                   double *C, int ldC, int slices, int *slices_used, void *stream) {
    using namespace fg;
    const bool okA = transA == 'N' || transA == 'n' || transA == 'T' || transA == 't' ||
                     transA == 'C' || transA == 'c';
    const bool okB = transB == 'N' || transB == 'n' || transB == 'T' || transB == 't' ||
                     transB == 'C' || transB == 'c';
    if (!okA) return -1;
    if (!okB) return -2;
    if (m < 0) return -3;
    if (n < 0) return -4;
    if (k < 0) return -5;
    const bool ta = !(transA == 'N' || transA == 'n');
    const bool tb = !(transB == 'N' || transB == 'n');
    if (ldA < ((ta ? k : m) > 1 ? (ta ? k : m) : 1)) return -8;
    if (ldB < ((tb ? n : k) > 1 ? (tb ? n : k) : 1)) return -10;
    if (ldC < (m > 1 ? m : 1)) return -13;
    if (slices < 0 || slices > kMaxSlices) return -14;
    return dgemm_split_launch(transA, transB, m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC, slices,
                              slices_used, (cudaStream_t)stream);
}
