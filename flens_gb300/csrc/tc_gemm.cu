// tc_gemm.cu -- low-precision tensor-core GEMM (tcgen05 / TMEM / TMA), FP32
// accumulate, FP32 C in HBM.
//
// Used for the trailing-update contractions of the precision form of the LU
// (A22 -= A21 * A12 with A21, A12 rounded to TF32, BF16 or FP8 e4m3) and
// exposed as flens_gb300_sgemm_tc.  The reference has no low-precision path
// (its float gemm is the same generic loop as for double,
// cxxblas/level3/gemm.tcc:42-190); this is the contraction its FP32 `mm`
// would perform, carried out on the 5th-generation tensor cores.
//
// Kernel shape: persistent, one CTA per SM over 128 x BN output tiles
// (BN = 256), 320 threads:
//   warp 0 lane 0  TMA producer: 128B-swizzled K-major tiles of A (128 rows)
//                  and B (BN rows) into a STAGES-deep shared-memory ring,
//                  one mbarrier (expect_tx) per stage;
//   warp 1         allocates 2*BN TMEM columns (two accumulators); lane 0
//                  issues tcgen05.mma (M=128, N=BN, K=32 bytes per
//                  instruction), commits each stage back to the producer and
//                  each finished tile to the epilogue;
//   warps 2-9      epilogue: tcgen05.ld 32x32b.x32 chunks of their TMEM lane
//                  quarter (= tile rows), C = alpha*acc*(sa_i*sb_j) + beta*C,
//                  coalesced column-major stores, then release the
//                  accumulator to the MMA warp.
// Every wait is bounded (kMbarSpinLimit); on a timeout the kernel sets the
// status word, lets in-flight copies land, frees its TMEM and returns.
#include "common.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_fp8.h>

#include <mutex>

namespace fg {

// Precisions of the tensor-core contraction.  kTcF32x3 is FP32-accurate: each
// operand is split into a TF32 head and a TF32 tail and three TF32 products
// (head*head + head*tail + tail*head) are accumulated.  kTcTF32Lo is only a
// conversion mode (the tail of the split).
enum TcKind : int { kTcTF32 = 0, kTcBF16 = 1, kTcFP8 = 2, kTcF32x3 = 3, kTcTF32Lo = 4 };

namespace {

constexpr int TC_BM = 128;
constexpr int TC_BN = 256;
constexpr int TC_STAGES = 4;
constexpr int TC_THREADS = 320;                   // 10 warps: TMA, MMA, 8 epilogue
constexpr uint32_t kMbarSpinLimit = 1u << 20;
constexpr uint32_t TC_A_BYTES = TC_BM * 128;       // one stage of A: 128 rows x 128 B
constexpr uint32_t TC_B_BYTES = TC_BN * 128;       // one stage of B: BN rows x 128 B
constexpr size_t TC_SMEM = 1024 + (size_t)TC_STAGES * (TC_A_BYTES + TC_B_BYTES) + 256;

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

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
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

// Persistent kernel: one CTA per SM walks the output tiles
// (tile = blockIdx.x + i*gridDim.x, m fastest), two TMEM accumulators of
// TC_BN columns each, so the epilogue of one tile overlaps the TMA loads and
// MMAs of the next.  Roles:
//   warp 0 lane 0   TMA producer over (tile, k-block), STAGES-deep smem ring;
//   warp 1          TMEM allocation; lane 0 issues the MMAs of a tile into
//                   accumulator (tile & 1) once the epilogue has released it;
//   warps 2..9      epilogue: warp w drains TMEM lanes 32*(w%4).. (the lane
//                   quarter a warp may access) for column half (w-2)/4.
template <int KIND>
__global__ void __launch_bounds__(TC_THREADS, 1)
tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
               int M, int N, int K, float alpha, float beta, float *__restrict__ C, int ldc,
               const float *__restrict__ scale_a, const float *__restrict__ scale_b,
               int *__restrict__ status) {
    constexpr int ELEM = KIND == kTcTF32 ? 4 : KIND == kTcBF16 ? 2 : 1;
    constexpr int BK = 128 / ELEM;               // elements per 128-byte row (one k-block)
    constexpr int KSTEPS = 4;                    // 32 bytes of K per MMA
    constexpr int EPI_WARPS = 8;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *sA = smem;
    uint8_t *sB = smem + TC_STAGES * TC_A_BYTES;
    uint64_t *full = (uint64_t *)(sB + TC_STAGES * TC_B_BYTES);
    uint64_t *empty = full + TC_STAGES;
    uint64_t *tfull = empty + TC_STAGES;         // [2] accumulator ready
    uint64_t *tempty = tfull + 2;                // [2] accumulator drained
    uint32_t *tmem_slot = (uint32_t *)(tempty + 2);
    __shared__ int s_abort;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tiles_m = (M + TC_BM - 1) / TC_BM, tiles_n = (N + TC_BN - 1) / TC_BN;
    const int ntiles = tiles_m * tiles_n;
    const int nkb = (K + BK - 1) / BK;

    if (threadIdx.x == 0) {
        for (int s = 0; s < TC_STAGES; ++s) {
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
                     "r"((uint32_t)(2 * TC_BN))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            // ---- TMA producer
            int q = 0, issued = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
                const int m0 = (t % tiles_m) * TC_BM, n0 = (t / tiles_m) * TC_BN;
                for (int kb = 0; kb < nkb; ++kb, ++q) {
                    const int s = q % TC_STAGES;
                    const uint32_t ph = (uint32_t)(q / TC_STAGES) & 1u;
                    if (s_abort || !mbar_wait(&empty[s], ph ^ 1u, status)) {
                        s_abort = 1;
                        ok = false;
                        break;
                    }
                    mbar_expect_tx(&full[s], TC_A_BYTES + TC_B_BYTES);
                    tma_load_2d(&tmA, &full[s], sA + s * TC_A_BYTES, kb * BK, m0);
                    tma_load_2d(&tmB, &full[s], sB + s * TC_B_BYTES, kb * BK, n0);
                    ++issued;
                }
            }
            if (!ok) {
                // let the copies already issued land before the CTA can exit
                for (int r = (issued > TC_STAGES ? issued - TC_STAGES : 0); r < issued; ++r)
                    mbar_wait(&full[r % TC_STAGES], (uint32_t)(r / TC_STAGES) & 1u, status);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---- MMA issuer
            const uint32_t idesc = idesc_for(KIND, TC_BM, TC_BN);
            int q = 0, i = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++i) {
                const int b = i & 1;
                const uint32_t acc = tmem + (uint32_t)(b * TC_BN);
                if (!mbar_wait(&tempty[b], ((uint32_t)(i >> 1) & 1u) ^ 1u, status)) {
                    s_abort = 1;
                    break;
                }
                tc_fence_after();
                for (int kb = 0; kb < nkb; ++kb, ++q) {
                    const int s = q % TC_STAGES;
                    const uint32_t ph = (uint32_t)(q / TC_STAGES) & 1u;
                    if (s_abort || !mbar_wait(&full[s], ph, status)) {
                        s_abort = 1;
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t a0 = smem_u32(sA + s * TC_A_BYTES);
                    const uint32_t b0 = smem_u32(sB + s * TC_B_BYTES);
#pragma unroll
                    for (int kk = 0; kk < KSTEPS; ++kk)
                        umma<KIND>(acc, sdesc_sw128(a0 + kk * 32), sdesc_sw128(b0 + kk * 32), idesc,
                                   (kb | kk) != 0 ? 1u : 0u);
                    umma_commit(&empty[s]);
                }
                if (ok) umma_commit(&tfull[b]);
            }
        }
    } else {
        // ---- epilogue
        const int ew = warp - 2;                 // 0..7
        const int quarter = warp & 3;            // TMEM lane quarter this warp may access
        const int half = ew >> 2;                // column half
        int i = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++i) {
            const int b = i & 1;
            const int m0 = (t % tiles_m) * TC_BM, n0 = (t / tiles_m) * TC_BN;
            const bool have = mbar_wait(&tfull[b], (uint32_t)(i >> 1) & 1u, status);
            if (!have) {
                s_abort = 1;
                break;
            }
            tc_fence_after();
            const int row = m0 + quarter * 32 + lane;
            const float sa = (scale_a != nullptr && row < M) ? scale_a[row] : 1.0f;
            const uint32_t base = tmem + (uint32_t)(b * TC_BN) + ((uint32_t)(quarter * 32) << 16);
            for (int c0 = half * (TC_BN / 2); c0 < (half + 1) * (TC_BN / 2); c0 += 32) {
                if (n0 + c0 >= N) break;         // uniform across the warp
                uint32_t r[32];
                tmem_ld32(base + (uint32_t)c0, r);
                if (row < M) {
                    float *crow = C + (size_t)row + (size_t)(n0 + c0) * ldc;
                    const int ncol = min(32, N - (n0 + c0));
                    // all 32 loads of C in flight before any store
                    float cv[32];
#pragma unroll
                    for (int j = 0; j < 32; ++j) cv[j] = (j < ncol) ? __ldcs(crow + (size_t)j * ldc) : 0.0f;
#pragma unroll
                    for (int j = 0; j < 32; ++j) {
                        if (j < ncol) {
                            float accv = __uint_as_float(r[j]);
                            if (scale_b != nullptr) accv *= sa * scale_b[n0 + c0 + j];
                            __stcs(crow + (size_t)j * ldc, fmaf(alpha, accv, beta * cv[j]));
                        }
                    }
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&tempty[b])) : "memory");
            if (s_abort) break;
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"((uint32_t)(2 * TC_BN))
                     : "memory");
    }
}

// ------------------------------------------------------------ operands ----
// out(r, k) = round(in(r, k) * inv_scale[r]) with in(r, k) = in[r + k*ld]
// (TRANS = false: the op is stored r-contiguous, as A for op(A)=A) or
// in[k + r*ld] (TRANS = true).  out is K-major: out[r*ldo + k].  Columns
// k >= K up to ldo are zero-filled.
template <int KIND>
__device__ __forceinline__ void store_lp(void *out, size_t idx, float v);

template <>
__device__ __forceinline__ void store_lp<kTcBF16>(void *out, size_t idx, float v) {
    ((__nv_bfloat16 *)out)[idx] = __float2bfloat16_rn(v);
}
template <>
__device__ __forceinline__ void store_lp<kTcTF32>(void *out, size_t idx, float v) {
    uint32_t t;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(v));
    ((uint32_t *)out)[idx] = t;
}
template <>
__device__ __forceinline__ void store_lp<kTcTF32Lo>(void *out, size_t idx, float v) {
    uint32_t h, t;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(v));
    const float lo = v - __uint_as_float(h);
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(lo));
    ((uint32_t *)out)[idx] = t;
}
template <>
__device__ __forceinline__ void store_lp<kTcFP8>(void *out, size_t idx, float v) {
    ((__nv_fp8_storage_t *)out)[idx] = __nv_cvt_float_to_fp8(v, __NV_SATFINITE, __NV_E4M3);
}

template <int KIND, bool RCONTIG>
__global__ void __launch_bounds__(256)
to_kmajor_kernel(int R, int K, const float *__restrict__ in, int ld, void *__restrict__ out,
                 int ldo, const float *__restrict__ inv_scale) {
    __shared__ float tile[32][33];
    const int r0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 32 x 8
    if (RCONTIG) {
        for (int kk = ty; kk < 32; kk += 8) {
            const int r = r0 + tx, k = k0 + kk;
            tile[kk][tx] = (r < R && k < K) ? in[(size_t)r + (size_t)k * ld] : 0.0f;
        }
        __syncthreads();
        for (int rr = ty; rr < 32; rr += 8) {
            const int r = r0 + rr, k = k0 + tx;
            if (r < R && k < ldo) {
                float v = tile[tx][rr];
                if (inv_scale) v *= inv_scale[r];
                store_lp<KIND>(out, (size_t)r * ldo + k, v);
            }
        }
    } else {
        for (int rr = ty; rr < 32; rr += 8) {
            const int r = r0 + rr, k = k0 + tx;
            if (r < R && k < ldo) {
                float v = (k < K) ? in[(size_t)k + (size_t)r * ld] : 0.0f;
                if (inv_scale) v *= inv_scale[r];
                store_lp<KIND>(out, (size_t)r * ldo + k, v);
            }
        }
    }
}

// Per-row amax of op(X) (R rows, K columns) -> scale = amax/448 and 1/scale
// (FP8 e4m3 per-row scaling; a zero row keeps scale 1).
template <bool RCONTIG>
__global__ void __launch_bounds__(256)
row_scale_kernel(int R, int K, const float *__restrict__ in, int ld, float *__restrict__ scale,
                 float *__restrict__ inv_scale) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = blockIdx.x * 8 + warp;
    if (r >= R) return;
    float m = 0.0f;
    for (int k = lane; k < K; k += 32) {
        const float v = RCONTIG ? in[(size_t)r + (size_t)k * ld] : in[(size_t)k + (size_t)r * ld];
        m = fmaxf(m, fabsf(v));
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
    if (lane == 0) {
        const float s = (m > 0.0f && isfinite(m)) ? m / 448.0f : 1.0f;
        scale[r] = s;
        inv_scale[r] = 1.0f / s;
    }
}

__global__ void sscale_kernel(int m, int n, float beta, float *__restrict__ C, int ldc) {
    const size_t total = (size_t)m * n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const size_t j = e / m, i = e % m;
        C[i + j * ldc] *= beta;
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        cudaDriverEntryPointQueryResult q;
        void *p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    });
    return fn;
}

// 2-D map over a K-major operand: inner dim = K (elements), outer = rows.
int make_map(CUtensorMap *map, int kind, const void *base, int rows, int K, int ldo, int box_rows) {
    PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
    if (!fn) {
        set_last_error("cuTensorMapEncodeTiled is not available from the driver");
        return kErrCuda;
    }
    const int elem = kind == kTcTF32 ? 4 : kind == kTcBF16 ? 2 : 1;
    const CUtensorMapDataType dt = kind == kTcTF32   ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                   : kind == kTcBF16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16
                                                     : CU_TENSOR_MAP_DATA_TYPE_UINT8;
    cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)ldo * elem};
    cuuint32_t box[2] = {(cuuint32_t)(128 / elem), (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    const CUresult r = fn(map, dt, 2, const_cast<void *>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_last_error("cuTensorMapEncodeTiled failed (%d) rows=%d K=%d ld=%d", (int)r, rows, K, ldo);
        return kErrCuda;
    }
    return kOk;
}

}  // namespace

// K-major leading dimension (elements) for `kind`: K rounded up to 16 bytes.
static int gemm_kind(int kind) { return (kind == kTcF32x3 || kind == kTcTF32Lo) ? kTcTF32 : kind; }

int tc_kmajor_ld(int kind, int K) {
    kind = gemm_kind(kind);
    const int per16 = kind == kTcTF32 ? 4 : kind == kTcBF16 ? 8 : 16;
    return (K + per16 - 1) / per16 * per16;
}

size_t tc_elem_bytes(int kind) {
    kind = gemm_kind(kind);
    return kind == kTcTF32 ? 4 : kind == kTcBF16 ? 2 : 1;
}

// Convert op(X) (R x K, FP32, column-major storage, transposed or not) to a
// K-major low-precision operand.  For FP8, also computes per-row scales.
int tc_convert(int kind, bool trans, int R, int K, const float *X, int ldx, void *out, int ldo,
               float *scale, float *inv_scale, cudaStream_t stream) {
    if (R <= 0 || K <= 0) return kOk;
    KTimer kt(kFamAux, stream, 0.0, (4.0 + tc_elem_bytes(kind)) * R * (double)K);
    // op(X)(r, k): r-contiguous when X is stored R x K (no transpose)
    const bool rcontig = !trans;
    if (kind == kTcFP8) {
        const dim3 g(ceil_div(R, 8));
        if (rcontig) row_scale_kernel<true><<<g, 256, 0, stream>>>(R, K, X, ldx, scale, inv_scale);
        else row_scale_kernel<false><<<g, 256, 0, stream>>>(R, K, X, ldx, scale, inv_scale);
        FG_CUDA(cudaGetLastError());
    }
    const dim3 grid(ceil_div(R, 32), ceil_div(ldo, 32));
    const float *inv = kind == kTcFP8 ? inv_scale : nullptr;
#define FG_CONV(KD)                                                                          \
    do {                                                                                     \
        if (rcontig) to_kmajor_kernel<KD, true><<<grid, 256, 0, stream>>>(R, K, X, ldx, out, ldo, inv); \
        else to_kmajor_kernel<KD, false><<<grid, 256, 0, stream>>>(R, K, X, ldx, out, ldo, inv);        \
    } while (0)
    if (kind == kTcTF32) FG_CONV(kTcTF32);
    else if (kind == kTcTF32Lo) FG_CONV(kTcTF32Lo);
    else if (kind == kTcBF16) FG_CONV(kTcBF16);
    else FG_CONV(kTcFP8);
#undef FG_CONV
    FG_CUDA(cudaGetLastError());
    return kOk;
}

// C (M x N, FP32, col-major) = alpha * A_lp * B_lp^T (* sa_i sb_j) + beta * C
// A_lp: M x K K-major (lda), B_lp: N x K K-major (ldb), both 16-byte aligned.
int tc_gemm_launch(int kind, int M, int N, int K, float alpha, const void *A_lp, int lda,
                   const void *B_lp, int ldb, float beta, float *C, int ldc, const float *scale_a,
                   const float *scale_b, cudaStream_t stream) {
    if (M <= 0 || N <= 0) return kOk;
    Workspace *w = workspace_for(stream, 0);
    if (!w) return kErrAlloc;
    if (K <= 0) return kErrUnsupported;
    if (((uintptr_t)A_lp | (uintptr_t)B_lp) & 15) {
        set_last_error("tc_gemm: operands must be 16-byte aligned");
        return kErrUnsupported;
    }
    CUtensorMap ma, mb;
    int st = make_map(&ma, kind, A_lp, M, K, lda, TC_BM);
    if (st != kOk) return st;
    if ((st = make_map(&mb, kind, B_lp, N, K, ldb, TC_BN)) != kOk) return st;
    static bool attr[3] = {false, false, false};
    const int ntiles = ceil_div(M, TC_BM) * ceil_div(N, TC_BN);
    const int sms = num_sms();
    const dim3 grid(ntiles < sms ? ntiles : sms);
    KTimer kt(kFamTcGemm, stream, 2.0 * M * (double)N * K,
              tc_elem_bytes(kind) * ((double)M * K + (double)N * K) + 8.0 * M * (double)N);
#define FG_TC(KD)                                                                                 \
    do {                                                                                          \
        if (!attr[KD]) {                                                                          \
            FG_CUDA(cudaFuncSetAttribute(tc_gemm_kernel<KD>,                                      \
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM)); \
            attr[KD] = true;                                                                      \
        }                                                                                         \
        tc_gemm_kernel<KD><<<grid, TC_THREADS, TC_SMEM, stream>>>(ma, mb, M, N, K, alpha, beta, C,  \
                                                                 ldc, scale_a, scale_b, w->status); \
    } while (0)
    if (kind == kTcTF32) FG_TC(kTcTF32);
    else if (kind == kTcBF16) FG_TC(kTcBF16);
    else FG_TC(kTcFP8);
#undef FG_TC
    FG_CUDA(cudaGetLastError());
    return kOk;
}

static size_t round256(size_t b) { return (b + 255) / 256 * 256; }

size_t tc_update_workspace_bytes(int kind, int m, int n, int k) {
    const int ld = tc_kmajor_ld(kind, k);
    const size_t eb = tc_elem_bytes(kind);
    const size_t a = round256((size_t)m * ld * eb), b = round256((size_t)n * ld * eb);
    size_t total = a + b;
    if (kind == kTcF32x3) total *= 2;
    if (kind == kTcFP8) total += round256((size_t)(m + n) * 2 * sizeof(float));
    return total;
}

int tc_trailing_update(int kind, int m, int n, int k, const float *A21, int ldA21,
                       const float *U12, int ldU12, float *A22, int ldA22, void *buf,
                       cudaStream_t stream) {
    if (m <= 0 || n <= 0 || k <= 0) return kOk;
    const int ld = tc_kmajor_ld(kind, k);
    const size_t eb = tc_elem_bytes(kind);
    const size_t a = round256((size_t)m * ld * eb), b = round256((size_t)n * ld * eb);
    char *p = (char *)buf;
    void *Ahi = p, *Bhi = p + a;
    int st;
    if (kind == kTcF32x3) {
        void *Alo = p + a + b, *Blo = p + 2 * a + b;
        if ((st = tc_convert(kTcTF32, false, m, k, A21, ldA21, Ahi, ld, nullptr, nullptr, stream))) return st;
        if ((st = tc_convert(kTcTF32Lo, false, m, k, A21, ldA21, Alo, ld, nullptr, nullptr, stream))) return st;
        if ((st = tc_convert(kTcTF32, true, n, k, U12, ldU12, Bhi, ld, nullptr, nullptr, stream))) return st;
        if ((st = tc_convert(kTcTF32Lo, true, n, k, U12, ldU12, Blo, ld, nullptr, nullptr, stream))) return st;
        // small terms first, then the head product
        if ((st = tc_gemm_launch(kTcTF32, m, n, k, -1.0f, Alo, ld, Bhi, ld, 1.0f, A22, ldA22, nullptr, nullptr, stream))) return st;
        if ((st = tc_gemm_launch(kTcTF32, m, n, k, -1.0f, Ahi, ld, Blo, ld, 1.0f, A22, ldA22, nullptr, nullptr, stream))) return st;
        return tc_gemm_launch(kTcTF32, m, n, k, -1.0f, Ahi, ld, Bhi, ld, 1.0f, A22, ldA22, nullptr, nullptr, stream);
    }
    float *sa = nullptr, *sia = nullptr, *sb = nullptr, *sib = nullptr;
    if (kind == kTcFP8) {
        sa = (float *)(p + a + b);
        sia = sa + m;
        sb = sia + m;
        sib = sb + n;
    }
    if ((st = tc_convert(kind, false, m, k, A21, ldA21, Ahi, ld, sa, sia, stream))) return st;
    if ((st = tc_convert(kind, true, n, k, U12, ldU12, Bhi, ld, sb, sib, stream))) return st;
    return tc_gemm_launch(kind, m, n, k, -1.0f, Ahi, ld, Bhi, ld, 1.0f, A22, ldA22, sa, sb, stream);
}

}  // namespace fg

// ----------------------------------------------------------------- C ABI ----
// C = alpha*op(A)*op(B) + beta*C with FP32 operands in device memory, the
// products taken on the tensor cores in `precision` (0 = TF32, 1 = BF16,
// 2 = FP8 e4m3 with per-row/per-column scaling, 3 = FP32-accurate 3xTF32) and
// accumulated in FP32.
FG_API int flens_gb300_sgemm_tc(int precision, char transA, char transB, int m, int n, int k,
                                float alpha, const float *A, int ldA, const float *B, int ldB,
                                float beta, float *C, int ldC, void *stream) {
    using namespace fg;
    if (precision < 0 || precision > 3) return -1;
    const bool ta = !(transA == 'N' || transA == 'n');
    const bool tb = !(transB == 'N' || transB == 'n');
    if (!(transA == 'N' || transA == 'n' || transA == 'T' || transA == 't' || transA == 'C' || transA == 'c')) return -2;
    if (!(transB == 'N' || transB == 'n' || transB == 'T' || transB == 't' || transB == 'C' || transB == 'c')) return -3;
    if (m < 0) return -4;
    if (n < 0) return -5;
    if (k < 0) return -6;
    if (ldA < (ta ? (k > 1 ? k : 1) : (m > 1 ? m : 1))) return -9;
    if (ldB < (tb ? (n > 1 ? n : 1) : (k > 1 ? k : 1))) return -11;
    if (ldC < (m > 1 ? m : 1)) return -14;
    if (m == 0 || n == 0) return kOk;
    cudaStream_t s = (cudaStream_t)stream;
    if (k == 0 || alpha == 0.0f) {
        // C = beta*C (a multiply, as cxxblas gescal does) and nothing else
        KTimer kt(kFamAux, s, (double)m * n, 8.0 * m * (double)n);
        int blocks = (int)ceil_div((size_t)m * n, (size_t)256);
        if (blocks > num_sms() * 16) blocks = num_sms() * 16;
        sscale_kernel<<<blocks, 256, 0, s>>>(m, n, beta, C, ldC);
        FG_CUDA(cudaGetLastError());
        return kOk;
    }
    // op(A) (m x k) and op(B) (k x n) as the trailing-update shapes: A with
    // rows contiguous when not transposed, op(B)^T rows contiguous when B is.
    const size_t need = tc_update_workspace_bytes(precision, m, n, k);
    Workspace *w = workspace_for(s, need);
    if (!w) return kErrAlloc;
    const int ld = tc_kmajor_ld(precision, k);
    const size_t eb = tc_elem_bytes(precision);
    const size_t a = round256((size_t)m * ld * eb), b = round256((size_t)n * ld * eb);
    char *p = (char *)w->buf;
    int st;
    if (precision == kTcF32x3) {
        void *Ahi = p, *Bhi = p + a, *Alo = p + a + b, *Blo = p + 2 * a + b;
        if ((st = tc_convert(kTcTF32, ta, m, k, A, ldA, Ahi, ld, nullptr, nullptr, s))) return st;
        if ((st = tc_convert(kTcTF32Lo, ta, m, k, A, ldA, Alo, ld, nullptr, nullptr, s))) return st;
        if ((st = tc_convert(kTcTF32, !tb, n, k, B, ldB, Bhi, ld, nullptr, nullptr, s))) return st;
        if ((st = tc_convert(kTcTF32Lo, !tb, n, k, B, ldB, Blo, ld, nullptr, nullptr, s))) return st;
        if ((st = tc_gemm_launch(kTcTF32, m, n, k, alpha, Alo, ld, Bhi, ld, beta, C, ldC, nullptr, nullptr, s))) return st;
        if ((st = tc_gemm_launch(kTcTF32, m, n, k, alpha, Ahi, ld, Blo, ld, 1.0f, C, ldC, nullptr, nullptr, s))) return st;
        return tc_gemm_launch(kTcTF32, m, n, k, alpha, Ahi, ld, Bhi, ld, 1.0f, C, ldC, nullptr, nullptr, s);
    }
    void *Alp = p, *Blp = p + a;
    float *sa = nullptr, *sia = nullptr, *sb = nullptr, *sib = nullptr;
    if (precision == kTcFP8) {
        sa = (float *)(p + a + b);
        sia = sa + m;
        sb = sia + m;
        sib = sb + n;
    }
    if ((st = tc_convert(precision, ta, m, k, A, ldA, Alp, ld, sa, sia, s))) return st;
    // B^T(j, p) = op(B)(p, j): for op(B) = B (K x N col-major) row j of B^T is contiguous in p
    if ((st = tc_convert(precision, !tb, n, k, B, ldB, Blp, ld, sb, sib, s))) return st;
    return tc_gemm_launch(precision, m, n, k, alpha, Alp, ld, Blp, ld, beta, C, ldC, sa, sb, s);
}
