// tc_gemm.cu -- low-precision tensor-core GEMM (tcgen05 / TMEM / TMA), FP32
// accumulate, FP32 C in HBM.
//
// Used for the trailing-update contractions of the precision form of the LU
// (A22 -= A21 * A12 with A21, A12 rounded to TF32, BF16 or FP8 e4m3) and
// exposed as flens_gb300_sgemm_tc.  The reference has no low-precision path
// (its float gemm is the same generic loop as for double,
// cxxblas/level3/gemm.tcc:42-190); this is the contraction its FP32 `mm`
// would perform, carried out on the 5th-generation tensor cores.  The kernel
// (persistent, warp-specialised TMA / MMA / epilogue) is tc::tc_kernel of
// tcgen05.cuh with the FP32 epilogue below: one work item per tile over the
// whole K, C = alpha*acc*(sa_i*sb_j) + beta*C with coalesced column-major
// loads and stores.
#include "tcgen05.cuh"

#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_fp8.h>

#include <mutex>

namespace fg {

namespace {

using tc::BM;
using tc::BN;

// FP32 output: C = alpha * acc * (sa_i * sb_j) + beta * C, one group over K.
struct EpiF32 {
    static constexpr int kBN = 256;
    static constexpr int kTmemExtra = 0;
    float alpha, beta;
    float *C;
    int ldc;
    const float *scale_a, *scale_b;
    int nkb;                                     // k-blocks of the whole K
    int pf;                                      // C 16-byte aligned by column: prefetch it

    __device__ int groups() const { return 1; }
    // column j of the next tile's C into L2 (a contiguous run of its rows),
    // so that the epilogue's loads of it hit L2 instead of HBM
    __device__ void prefetch(int m0, int n0, int M, int N, int j) const {
        if (!pf || beta == 0.0f || j >= min(kBN, N - n0)) return;
        const int bytes = (min(BM, M - m0) * 4) & ~15;
        if (bytes <= 0) return;
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(
                         C + (size_t)m0 + (size_t)(n0 + j) * ldc),
                     "r"(bytes)
                     : "memory");
    }
    __device__ void group(int, int &ka, int &kb, int &nk) const {
        ka = 0;
        kb = 0;
        nk = nkb;
    }
    __device__ void apply(int, int row, bool row_ok, int col, int ncol,
                          const uint32_t (&r)[32], uint32_t) const {
        if (!row_ok) return;
        const float sa = scale_a != nullptr ? scale_a[row] : 1.0f;
        float *crow = C + (size_t)row + (size_t)col * ldc;
        // all 32 loads of C in flight before any store
        float cv[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) cv[j] = (j < ncol) ? __ldcs(crow + (size_t)j * ldc) : 0.0f;
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            if (j < ncol) {
                float accv = __uint_as_float(r[j]);
                if (scale_b != nullptr) accv *= sa * scale_b[col + j];
                __stcs(crow + (size_t)j * ldc, fmaf(alpha, accv, beta * cv[j]));
            }
        }
    }
};

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
// the terms of the e4m3 splits: t0 = e4m3(v), t1 = e4m3(v - t0),
// t2 = e4m3(v - t0 - t1).  Each difference is exact in FP32: a term has 4
// significant bits and is within half an e4m3 step of what it rounds.
__device__ __forceinline__ float fp8_round(float v, __nv_fp8_storage_t *q) {
    *q = __nv_cvt_float_to_fp8(v, __NV_SATFINITE, __NV_E4M3);
    return __half2float(__half(__nv_cvt_fp8_to_halfraw(*q, __NV_E4M3)));
}
template <>
__device__ __forceinline__ void store_lp<kTcFP8Lo>(void *out, size_t idx, float v) {
    __nv_fp8_storage_t q;
    const float t0 = fp8_round(v, &q);
    fp8_round(v - t0, &q);
    ((__nv_fp8_storage_t *)out)[idx] = q;
}
template <>
__device__ __forceinline__ void store_lp<kTcFP8Lo2>(void *out, size_t idx, float v) {
    __nv_fp8_storage_t q;
    const float t0 = fp8_round(v, &q);
    const float t1 = fp8_round(v - t0, &q);
    fp8_round(v - t0 - t1, &q);
    ((__nv_fp8_storage_t *)out)[idx] = q;
}

template <int KIND, bool RCONTIG>
__global__ void __launch_bounds__(256)
to_kmajor_kernel(int R, int K, const float *__restrict__ in, int ld, void *__restrict__ out,
                 int ldo, int width, const float *__restrict__ inv_scale) {
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
            if (r < R && k < width) {
                float v = tile[tx][rr];
                if (inv_scale) v *= inv_scale[r];
                store_lp<KIND>(out, (size_t)r * ldo + k, v);
            }
        }
    } else {
        for (int rr = ty; rr < 32; rr += 8) {
            const int r = r0 + rr, k = k0 + tx;
            if (r < R && k < width) {
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

// The split forms' operands in one pass: each entry of op(X) (R x K) is read
// once, split into its terms -- TF32: t0 = tf32(v), t1 = tf32(v - t0); e4m3
// (after the row scale): t0, t1, t2 as store_lp -- and segment q of the
// K-major output row (columns q*kp .. q*kp + kp - 1, zero beyond K) gets term
// seg[q].  Bitwise the terms of one tc_convert call per segment.
struct SegTerms {
    int nseg;
    int term[6];
};

template <bool FP8, bool RCONTIG>
__global__ void __launch_bounds__(256)
to_kmajor_terms_kernel(int R, int K, const float *__restrict__ in, int ld, void *__restrict__ out,
                       int ldo, int kp, SegTerms st, const float *__restrict__ inv_scale) {
    __shared__ float tile[32][33];
    const int r0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 32 x 8
    auto emit = [&](int r, int k, float v) {
        if (FP8 && inv_scale) v *= inv_scale[r];
        uint32_t w0, w1, w2 = 0u;
        if (FP8) {
            __nv_fp8_storage_t q;
            const float t0 = fp8_round(v, &q);
            w0 = q;
            const float t1 = fp8_round(v - t0, &q);
            w1 = q;
            fp8_round(v - t0 - t1, &q);
            w2 = q;
        } else {
            asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(w0) : "f"(v));
            asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(w1) : "f"(v - __uint_as_float(w0)));
        }
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            if (q >= st.nseg) break;
            const int tq = st.term[q];
            const uint32_t val = tq == 0 ? w0 : tq == 1 ? w1 : w2;
            const size_t idx = (size_t)r * ldo + (size_t)q * kp + k;
            if (FP8) ((__nv_fp8_storage_t *)out)[idx] = (__nv_fp8_storage_t)val;
            else ((uint32_t *)out)[idx] = val;
        }
    };
    if (RCONTIG) {
        for (int kk = ty; kk < 32; kk += 8) {
            const int r = r0 + tx, k = k0 + kk;
            tile[kk][tx] = (r < R && k < K) ? in[(size_t)r + (size_t)k * ld] : 0.0f;
        }
        __syncthreads();
        for (int rr = ty; rr < 32; rr += 8) {
            const int r = r0 + rr, k = k0 + tx;
            if (r < R && k < kp) emit(r, k, tile[tx][rr]);
        }
    } else {
        for (int rr = ty; rr < 32; rr += 8) {
            const int r = r0 + rr, k = k0 + tx;
            if (r < R && k < kp) emit(r, k, (k < K) ? in[(size_t)k + (size_t)r * ld] : 0.0f);
        }
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

}  // namespace

namespace tc {

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
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

int make_kmajor_map(CUtensorMap *map, int kind, const void *base, int rows, int K, int ldo, int box_rows) {
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

}  // namespace tc

// K-major leading dimension (elements) for `kind`: K rounded up to 16 bytes.
static int gemm_kind(int kind) {
    if (kind == kTcF32x3 || kind == kTcTF32Lo) return kTcTF32;
    if (kind == kTcFP8x2 || kind == kTcFP8x3 || kind == kTcFP8Lo || kind == kTcFP8Lo2) return kTcFP8;
    return kind;
}

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
// K-major low-precision operand: columns 0..width-1 of rows of stride ldo
// (zero beyond K).  For FP8, scales each row by inv_scale; when `scale` is
// given, first computes the per-row scales (else inv_scale holds them already).
int tc_convert(int kind, bool trans, int R, int K, const float *X, int ldx, void *out, int ldo,
               float *scale, float *inv_scale, cudaStream_t stream, int width = -1) {
    if (width < 0) width = ldo;
    if (R <= 0 || K <= 0) return kOk;
    KTimer kt(kFamAux, stream, 0.0, (4.0 + tc_elem_bytes(kind)) * R * (double)K);
    // op(X)(r, k): r-contiguous when X is stored R x K (no transpose)
    const bool rcontig = !trans;
    const bool fp8 = kind == kTcFP8 || kind == kTcFP8Lo || kind == kTcFP8Lo2;
    if (fp8 && scale != nullptr) {
        const dim3 g(ceil_div(R, 8));
        if (rcontig) row_scale_kernel<true><<<g, 256, 0, stream>>>(R, K, X, ldx, scale, inv_scale);
        else row_scale_kernel<false><<<g, 256, 0, stream>>>(R, K, X, ldx, scale, inv_scale);
        FG_CUDA(cudaGetLastError());
    }
    const dim3 grid(ceil_div(R, 32), ceil_div(width, 32));
    const float *inv = fp8 ? inv_scale : nullptr;
#define FG_CONV(KD)                                                                          \
    do {                                                                                     \
        if (rcontig) to_kmajor_kernel<KD, true><<<grid, 256, 0, stream>>>(R, K, X, ldx, out, ldo, width, inv); \
        else to_kmajor_kernel<KD, false><<<grid, 256, 0, stream>>>(R, K, X, ldx, out, ldo, width, inv);        \
    } while (0)
    if (kind == kTcTF32) FG_CONV(kTcTF32);
    else if (kind == kTcTF32Lo) FG_CONV(kTcTF32Lo);
    else if (kind == kTcBF16) FG_CONV(kTcBF16);
    else if (kind == kTcFP8Lo) FG_CONV(kTcFP8Lo);
    else if (kind == kTcFP8Lo2) FG_CONV(kTcFP8Lo2);
    else FG_CONV(kTcFP8);
#undef FG_CONV
    FG_CUDA(cudaGetLastError());
    return kOk;
}

// The split operand of op(X) (R x K) in one pass: segments st.term[q] at
// columns q*kp of the K-major rows (see to_kmajor_terms_kernel); for e4m3
// the per-row scales first (scale, inv_scale).
int tc_convert_terms(bool fp8, bool trans, int R, int K, const float *X, int ldx, void *out,
                     int ldo, int kp, const SegTerms &st, float *scale, float *inv_scale,
                     cudaStream_t stream) {
    if (R <= 0 || K <= 0) return kOk;
    KTimer kt(kFamAux, stream, 0.0, (4.0 + (fp8 ? 1.0 : 4.0) * st.nseg) * R * (double)K);
    const bool rcontig = !trans;
    if (fp8) {
        const dim3 g(ceil_div(R, 8));
        if (rcontig) row_scale_kernel<true><<<g, 256, 0, stream>>>(R, K, X, ldx, scale, inv_scale);
        else row_scale_kernel<false><<<g, 256, 0, stream>>>(R, K, X, ldx, scale, inv_scale);
    }
    const dim3 grid(ceil_div(R, 32), ceil_div(kp, 32));
    const float *inv = fp8 ? inv_scale : nullptr;
    if (fp8) {
        if (rcontig) to_kmajor_terms_kernel<true, true><<<grid, 256, 0, stream>>>(R, K, X, ldx, out, ldo, kp, st, inv);
        else to_kmajor_terms_kernel<true, false><<<grid, 256, 0, stream>>>(R, K, X, ldx, out, ldo, kp, st, inv);
    } else {
        if (rcontig) to_kmajor_terms_kernel<false, true><<<grid, 256, 0, stream>>>(R, K, X, ldx, out, ldo, kp, st, inv);
        else to_kmajor_terms_kernel<false, false><<<grid, 256, 0, stream>>>(R, K, X, ldx, out, ldo, kp, st, inv);
    }
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
    int st = tc::make_kmajor_map(&ma, kind, A_lp, M, K, lda, BM);
    if (st != kOk) return st;
    if ((st = tc::make_kmajor_map(&mb, kind, B_lp, N, K, ldb, BN)) != kOk) return st;
    const int ntiles = ceil_div(M, BM) * ceil_div(N, BN);
    const int sms = num_sms();
    const dim3 grid(ntiles < sms ? ntiles : sms);
    const int bk = 128 / (int)tc_elem_bytes(kind);
    const int pf = (((uintptr_t)C | ((uintptr_t)ldc * 4)) & 15) == 0 ? 1 : 0;
    const EpiF32 epi{alpha, beta, C, ldc, scale_a, scale_b, ceil_div(K, bk), pf};
    KTimer kt(kFamTcGemm, stream, 2.0 * M * (double)N * K,
              tc_elem_bytes(kind) * ((double)M * K + (double)N * K) + 8.0 * M * (double)N);
#define FG_TC(KD)                                                                               \
    do {                                                                                        \
        if ((st = tc::prepare_kernel<KD, EpiF32>()) != kOk) return st;                          \
        tc::tc_kernel<KD, EpiF32><<<grid, tc::THREADS, tc::Shape<EpiF32>::SMEM, stream>>>(      \
            ma, mb, M, N, epi,                                                                  \
                                                                         w->status);           \
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
    int ld = tc_kmajor_ld(kind, k);
    if (kind == kTcF32x3 || kind == kTcFP8x2) ld *= 3;   // three K segments, see f32x3_gemm
    if (kind == kTcFP8x3) ld *= 6;                       // six, see fp8_terms_gemm
    const size_t eb = tc_elem_bytes(kind);
    const size_t a = round256((size_t)m * ld * eb), b = round256((size_t)n * ld * eb);
    size_t total = a + b;
    if (kind == kTcFP8 || kind == kTcFP8x2 || kind == kTcFP8x3)
        total += round256((size_t)(m + n) * 2 * sizeof(float));
    return total;
}

namespace {

// FP32-accurate product as ONE TF32 GEMM over K' = 3 kp: op(A) is stored as
// [lo | hi | hi] and op(B)^T as [hi | lo | hi] along K, so the accumulator
// sums lo*hi + hi*lo + hi*hi (the small terms first) and C is read and
// written once (three separate products each read and wrote C).
int f32x3_gemm(bool ta_rows, bool tb_rows, int m, int n, int k, float alpha, const float *A, int ldA,
               const float *B, int ldB, float beta, float *C, int ldC, void *buf, cudaStream_t s) {
    const int kp = tc_kmajor_ld(kTcTF32, k), ld3 = 3 * kp;
    float *Ak = (float *)buf;
    float *Bk = (float *)((char *)buf + round256((size_t)m * ld3 * sizeof(float)));
    const SegTerms sa{3, {1, 0, 0}}, sb{3, {0, 1, 0}};     // [lo | hi | hi], [hi | lo | hi]
    int st;
    if ((st = tc_convert_terms(false, ta_rows, m, k, A, ldA, Ak, ld3, kp, sa, nullptr, nullptr, s))) return st;
    if ((st = tc_convert_terms(false, tb_rows, n, k, B, ldB, Bk, ld3, kp, sb, nullptr, nullptr, s))) return st;
    return tc_gemm_launch(kTcTF32, m, n, ld3, alpha, Ak, ld3, Bk, ld3, beta, C, ldC, nullptr, nullptr, s);
}

// The same segmented product in e4m3: op(A) row i is scaled by 1/sa_i
// (sa_i = amax/448 over its K entries) and op(B)^T row j by 1/sb_j; each
// scaled entry is split into `nterms` e4m3 terms t0 + t1 (+ t2), and the
// operands are laid out along K' = nseg kp so that segment q multiplies
// term ta[q] of op(A) by term tb[q] of op(B): for two terms t1*t0, t0*t1,
// t0*t0; for three terms t2*t0, t0*t2, t1*t1, t1*t0, t0*t1, t0*t0 (small
// terms first).  One FP32 accumulator sums them and the epilogue multiplies
// by sa_i sb_j, so C is read and written once.
int fp8_terms_gemm(int nterms, bool ta_rows, bool tb_rows, int m, int n, int k, float alpha,
                   const float *A, int ldA, const float *B, int ldB, float beta, float *C, int ldC,
                   void *buf, cudaStream_t s) {
    const SegTerms a2{3, {1, 0, 0}}, b2{3, {0, 1, 0}};
    const SegTerms a3{6, {2, 0, 1, 1, 0, 0}}, b3{6, {0, 2, 1, 0, 1, 0}};
    const SegTerms &tA = nterms == 3 ? a3 : a2, &tB = nterms == 3 ? b3 : b2;
    const int nseg = tA.nseg;
    const int kp = tc_kmajor_ld(kTcFP8, k), ldw = nseg * kp;
    const size_t a = round256((size_t)m * ldw), b = round256((size_t)n * ldw);
    uint8_t *Ak = (uint8_t *)buf, *Bk = (uint8_t *)buf + a;
    float *sa = (float *)((char *)buf + a + b), *sia = sa + m, *sb = sia + m, *sib = sb + n;
    int st;
    if ((st = tc_convert_terms(true, ta_rows, m, k, A, ldA, Ak, ldw, kp, tA, sa, sia, s))) return st;
    if ((st = tc_convert_terms(true, tb_rows, n, k, B, ldB, Bk, ldw, kp, tB, sb, sib, s))) return st;
    return tc_gemm_launch(kTcFP8, m, n, ldw, alpha, Ak, ldw, Bk, ldw, beta, C, ldC, sa, sb, s);
}

}  // namespace

int tc_gemm_f32x3_nn(int m, int n, int k, float alpha, const float *A, int ldA, const float *B,
                     int ldB, float beta, float *C, int ldC, void *buf, cudaStream_t stream) {
    if (m <= 0 || n <= 0 || k <= 0) return kOk;
    return f32x3_gemm(false, true, m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC, buf, stream);
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
    if (kind == kTcF32x3)
        return f32x3_gemm(false, true, m, n, k, -1.0f, A21, ldA21, U12, ldU12, 1.0f, A22, ldA22, buf, stream);
    if (kind == kTcFP8x2 || kind == kTcFP8x3)
        return fp8_terms_gemm(kind == kTcFP8x3 ? 3 : 2, false, true, m, n, k, -1.0f, A21, ldA21, U12,
                              ldU12, 1.0f, A22, ldA22, buf, stream);
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
// 2 = FP8 e4m3 with per-row/per-column scaling, 3 = FP32-accurate 3xTF32,
// 5 / 6 = two- / three-term e4m3 with the same scaling) and accumulated in
// FP32.
FG_API int flens_gb300_sgemm_tc(int precision, char transA, char transB, int m, int n, int k,
                                float alpha, const float *A, int ldA, const float *B, int ldB,
                                float beta, float *C, int ldC, void *stream) {
    using namespace fg;
    if (precision < 0 || precision > 6 || precision == 4) return -1;
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
    if (precision == kTcF32x3)
        return f32x3_gemm(ta, !tb, m, n, k, alpha, A, ldA, B, ldB, beta, C, ldC, p, s);
    if (precision == kTcFP8x2 || precision == kTcFP8x3)
        return fp8_terms_gemm(precision == kTcFP8x3 ? 3 : 2, ta, !tb, m, n, k, alpha, A, ldA, B, ldB,
                              beta, C, ldC, p, s);
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
