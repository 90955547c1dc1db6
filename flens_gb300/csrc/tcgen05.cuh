// tcgen05.cuh -- building blocks of the persistent tensor-core GEMM (TMA,
// mbarrier, tcgen05 MMA / TMEM in inline PTX) and the kernel template shared
// by the FP32-output GEMM (tc_gemm.cu) and the split-precision FP64 GEMM
// (split_gemm.cu).
//
// Kernel shape: persistent, one CTA per SM over 128 x BN output tiles (BN =
// 256, or 128 for a policy that keeps state in TMEM), 320 threads:
//   warp 0 lane 0  TMA producer: 128B-swizzled K-major tiles of A (128 rows)
//                  and B (256 rows) into a STAGES-deep shared-memory ring,
//                  one mbarrier (expect_tx) per stage;
//   warp 1         allocates 512 TMEM columns (two 128 x 256 FP32
//                  accumulators); lane 0 issues tcgen05.mma (M=128, N=256,
//                  32 bytes of K per instruction), commits each stage back to
//                  the producer and each finished work item to the epilogue;
//   warps 2-9      epilogue: tcgen05.ld 32x32b.x32 chunks of their TMEM lane
//                  quarter (= tile rows), handed to the Epi policy, then
//                  release the accumulator to the MMA warp.
// A work item is (output tile, group): each tile is visited once and its
// groups are accumulated one after the other, each into a fresh accumulator
// over its own k range of A and B (Epi::group), so the epilogue of one item
// overlaps the loads and MMAs of the next.  Tiles are walked in bands of 16
// tile rows so that the CTAs of one wave share A and B panels in L2.
// Every wait is bounded (kMbarSpinLimit); on a timeout the kernel sets the
// status word, lets in-flight copies land, frees its TMEM and returns.
#pragma once

#include "common.cuh"

#include <cuda.h>

namespace fg {

// Precisions of the tensor-core contraction.  kTcF32x3 is FP32-accurate: each
// operand is split into a TF32 head and a TF32 tail and three TF32 products
// (head*head + head*tail + tail*head) are accumulated.  kTcFP8x2 and kTcFP8x3
// do the same with e4m3: a scaled operand v is stored as t0 = e4m3(v),
// t1 = e4m3(v - t0) (and t2 = e4m3(v - t0 - t1)), and the products t_i t_j
// with i + j <= 1 (3 of them) or <= 2 (6 of them) are accumulated: about
// 2^-8 or 2^-12 relative per operand entry instead of e4m3's 2^-4.
// kTcTF32Lo, kTcFP8Lo (t1) and kTcFP8Lo2 (t2) are only conversion modes.
enum TcKind : int {
    kTcTF32 = 0,
    kTcBF16 = 1,
    kTcFP8 = 2,
    kTcF32x3 = 3,
    kTcTF32Lo = 4,
    kTcFP8x2 = 5,
    kTcFP8x3 = 6,
    kTcFP8Lo = 7,
    kTcFP8Lo2 = 8
};

namespace tc {

constexpr int BM = 128;
constexpr int BN = 256;                         // the default tile width
constexpr int THREADS = 320;                    // 10 warps: TMA, MMA, 8 epilogue
constexpr int EPI_WARPS = 8;
constexpr int BAND = 16;                        // tile rows per raster band
constexpr uint32_t kMbarSpinLimit = 1u << 20;
constexpr uint32_t A_BYTES = BM * 128;          // one stage of A: 128 rows x 128 B

// Per epilogue policy: the tile width Epi::kBN (128 or 256) and
// Epi::kTmemExtra TMEM columns the policy keeps beside the two accumulators.
template <class Epi>
struct Shape {
    static constexpr int BN = Epi::kBN;
    static constexpr int STAGES = BN >= 256 ? 4 : 6;      // ~192 KB of operand ring
    static constexpr uint32_t B_BYTES = BN * 128;          // one stage of B: BN rows x 128 B
    static constexpr size_t SMEM = 1024 + (size_t)STAGES * (A_BYTES + B_BYTES) + 256;
    static constexpr uint32_t TMEM_COLS = 2 * BN + Epi::kTmemExtra;
    static_assert(TMEM_COLS == 512 || TMEM_COLS == 256 || TMEM_COLS == 128,
                  "TMEM allocation must be a power of two <= 512 columns");
    static_assert(SMEM <= 227 * 1024, "shared memory per CTA");
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait on an mbarrier phase; false (and the status bit) on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int *status) {
    for (uint32_t i = 0; i < kMbarSpinLimit; ++i) {
        if (mbar_try_wait(bar, parity)) return true;
        if (i > 32) __nanosleep(64);
    }
    atomicOr(status, kDevMbarTimeout);
    return false;
}

__device__ __forceinline__ void tma_load_2d(const CUtensorMap *map, uint64_t *bar, void *dst,
                                            int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%3, %4}], [%2];" ::"r"(smem_u32(dst)),
        "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}

// UMMA shared-memory descriptor, K-major operand with 128-byte swizzle:
// rows of 128 B, 8-row (1024 B) swizzle atoms stacked along M/N (SBO = 1024),
// LBO unused for this layout, fixed 0b001 at bits 46-48, layout 2 = SW128.
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024u >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// Instruction descriptor: D = F32 (bits 4-5 = 1), A/B format at bits 7-9 and
// 10-12, both K-major (bits 15/16 = 0), N>>3 at bits 17-22, M>>4 at 24-28.
__host__ __device__ constexpr uint32_t idesc_for(int kind, int M, int N) {
    return (1u << 4) | ((uint32_t)(kind == kTcTF32 ? 2 : kind == kTcBF16 ? 1 : 0) << 7) |
           ((uint32_t)(kind == kTcTF32 ? 2 : kind == kTcBF16 ? 1 : 0) << 10) |
           ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

template <int KIND>
__device__ __forceinline__ void umma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                     uint32_t idesc, uint32_t accumulate) {
    if (KIND == kTcBF16) {
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
            "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
    } else if (KIND == kTcTF32) {
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
            "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
    } else {
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
            "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
    }
}

__device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// 32 lanes x 32 columns of 32-bit accumulators: thread i gets row (lane i)
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
          "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
          "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Output tile t -> (m0, n0): bands of BAND tile rows, tile rows fastest
// inside a band, so consecutive tiles (one wave of CTAs) cover a near-square
// block of C.
__device__ __forceinline__ void tile_origin(int t, int tiles_m, int tiles_n, int bn, int &m0, int &n0) {
    const int per_band = BAND * tiles_n;
    const int b = t / per_band, r = t - b * per_band;
    const int bm = min(BAND, tiles_m - b * BAND);
    m0 = (b * BAND + r % bm) * BM;
    n0 = (r / bm) * bn;
}

// Epi policy interface (all __device__, const):
//   int  groups() const                          work items per tile (>= 1)
//   void group(int g, int &ka, int &kb, int &nk) k offset (elements) of A and
//                                                of B, number of k-blocks
//   void apply(int g, int row, bool row_ok, int col, int ncol, const uint32_t (&r)[32],
//              uint32_t xt)
//        called by all 32 lanes of an epilogue warp for 32 accumulator
//        columns col..col+31 of tile row `row` (ncol of them inside C); xt is
//        the TMEM address of the policy's own kTmemExtra columns for this
//        warp's lane quarter (tile-local column 0).
//   void prefetch(int m0, int n0, int M, int N, int j) const
//        called by epilogue thread j (0..255) when its warps start a tile,
//        with the origin of the CTA's next tile: may bring column j of that
//        tile's output into L2 (a no-op for policies that read none)
//   static constexpr int kBN, kTmemExtra (see Shape)
template <int KIND, class Epi>
__global__ void __launch_bounds__(THREADS, 1)
tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int M,
          int N, const __grid_constant__ Epi epi, int *__restrict__ status) {
    constexpr int BN = Shape<Epi>::BN;
    constexpr int STAGES = Shape<Epi>::STAGES;
    constexpr uint32_t B_BYTES = Shape<Epi>::B_BYTES;
    constexpr uint32_t TMEM_COLS = Shape<Epi>::TMEM_COLS;
    constexpr int ELEM = KIND == kTcTF32 ? 4 : KIND == kTcBF16 ? 2 : 1;
    constexpr int BK = 128 / ELEM;               // elements per 128-byte row (one k-block)
    constexpr int KSTEPS = 4;                    // 32 bytes of K per MMA
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *sA = smem;
    uint8_t *sB = smem + STAGES * A_BYTES;
    uint64_t *full = (uint64_t *)(sB + STAGES * B_BYTES);
    uint64_t *empty = full + STAGES;
    uint64_t *tfull = empty + STAGES;            // [2] accumulator ready
    uint64_t *tempty = tfull + 2;                // [2] accumulator drained
    uint32_t *tmem_slot = (uint32_t *)(tempty + 2);
    __shared__ int s_abort;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tiles_m = (M + BM - 1) / BM, tiles_n = (N + BN - 1) / BN;
    const int ntiles = tiles_m * tiles_n;
    const int ngroups = epi.groups();

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], EPI_WARPS);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_abort = 0;
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            // ---- TMA producer
            int q = 0, issued = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
                int m0, n0;
                tile_origin(t, tiles_m, tiles_n, BN, m0, n0);
                for (int g = 0; g < ngroups && ok; ++g) {
                    int ka, kb, nk;
                    epi.group(g, ka, kb, nk);
                    for (int k = 0; k < nk; ++k, ++q) {
                        const int s = q % STAGES;
                        const uint32_t ph = (uint32_t)(q / STAGES) & 1u;
                        if (s_abort || !mbar_wait(&empty[s], ph ^ 1u, status)) {
                            s_abort = 1;
                            ok = false;
                            break;
                        }
                        mbar_expect_tx(&full[s], A_BYTES + B_BYTES);
                        tma_load_2d(&tmA, &full[s], sA + s * A_BYTES, ka + k * BK, m0);
                        tma_load_2d(&tmB, &full[s], sB + s * B_BYTES, kb + k * BK, n0);
                        ++issued;
                    }
                }
            }
            if (!ok) {
                // let the copies already issued land before the CTA can exit
                for (int r = (issued > STAGES ? issued - STAGES : 0); r < issued; ++r)
                    mbar_wait(&full[r % STAGES], (uint32_t)(r / STAGES) & 1u, status);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---- MMA issuer
            const uint32_t idesc = idesc_for(KIND, BM, BN);
            int q = 0, i = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
                for (int g = 0; g < ngroups && ok; ++g, ++i) {
                    const int b = i & 1;
                    const uint32_t acc = tmem + (uint32_t)(b * BN);
                    if (!mbar_wait(&tempty[b], ((uint32_t)(i >> 1) & 1u) ^ 1u, status)) {
                        s_abort = 1;
                        ok = false;
                        break;
                    }
                    fence_after();
                    int ka, kb, nk;
                    epi.group(g, ka, kb, nk);
                    for (int k = 0; k < nk; ++k, ++q) {
                        const int s = q % STAGES;
                        const uint32_t ph = (uint32_t)(q / STAGES) & 1u;
                        if (s_abort || !mbar_wait(&full[s], ph, status)) {
                            s_abort = 1;
                            ok = false;
                            break;
                        }
                        fence_after();
                        const uint32_t a0 = smem_u32(sA + s * A_BYTES);
                        const uint32_t b0 = smem_u32(sB + s * B_BYTES);
#pragma unroll
                        for (int kk = 0; kk < KSTEPS; ++kk)
                            umma<KIND>(acc, sdesc_sw128(a0 + kk * 32), sdesc_sw128(b0 + kk * 32),
                                       idesc, (k | kk) != 0 ? 1u : 0u);
                        umma_commit(&empty[s]);
                    }
                    if (ok) umma_commit(&tfull[b]);
                }
            }
        }
    } else {
        // ---- epilogue
        const int ew = warp - 2;                 // 0..7
        const int quarter = warp & 3;            // TMEM lane quarter this warp may access
        const int half = ew >> 2;                // column half
        int i = 0;
        bool live = true;
        for (int t = blockIdx.x; t < ntiles && live; t += gridDim.x) {
            int m0, n0;
            tile_origin(t, tiles_m, tiles_n, BN, m0, n0);
            const int row = m0 + quarter * 32 + lane;
            if (t + (int)gridDim.x < ntiles) {
                // the next tile's output, one tile ahead of its epilogue
                int m1, n1;
                tile_origin(t + (int)gridDim.x, tiles_m, tiles_n, BN, m1, n1);
                epi.prefetch(m1, n1, M, N, ew * 32 + lane);
            }
            for (int g = 0; g < ngroups; ++g, ++i) {
                const int b = i & 1;
                if (!mbar_wait(&tfull[b], (uint32_t)(i >> 1) & 1u, status)) {
                    s_abort = 1;
                    live = false;
                    break;
                }
                fence_after();
                const uint32_t lanes = (uint32_t)(quarter * 32) << 16;
                const uint32_t base = tmem + (uint32_t)(b * BN) + lanes;
                const uint32_t xt = tmem + (uint32_t)(2 * BN) + lanes;
                for (int c0 = half * (BN / 2); c0 < (half + 1) * (BN / 2); c0 += 32) {
                    if (n0 + c0 >= N) break;     // uniform across the warp
                    uint32_t r[32];
                    tmem_ld32(base + (uint32_t)c0, r);
                    epi.apply(g, row, row < M, n0 + c0, min(32, N - (n0 + c0)), r, xt);
                }
                fence_before();
                __syncwarp();
                if (lane == 0)
                    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&tempty[b]))
                                 : "memory");
                if (s_abort) {
                    live = false;
                    break;
                }
            }
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(TMEM_COLS)
                     : "memory");
    }
}

// 2-D TMA map over a K-major operand: inner dim = K (elements), outer = rows,
// 128-byte swizzle, box = one 128-byte k-block x box_rows.
int make_kmajor_map(CUtensorMap *map, int kind, const void *base, int rows, int K, int ldo,
                    int box_rows);

// Set the kernel's dynamic shared memory limit once per instantiation and device.
template <int KIND, class Epi>
int prepare_kernel() {
    static DeviceOnce once;               // per instantiation and device
    return set_smem_once(once, (const void *)tc_kernel<KIND, Epi>, (int)Shape<Epi>::SMEM);
}

}  // namespace tc
}  // namespace fg
