// common.cuh -- shared helpers for the GB300 dense LU / GEMM library.
//
// Everything in this directory is compiled for sm_103a only
// (-gencode arch=compute_103a,code=sm_103a).  Matrices are column-major with
// leading dimensions in elements, as in FLENS's FullStorage<T, ColMajor>
// (flens/storage/fullstorage/fullstorage.h:58-60) and the Fortran ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#define FG_API extern "C" __attribute__((visibility("default")))

namespace fg {

// ---------------------------------------------------------------- status --
// Library status codes (returned by the flens_gb300_* entry points).  Values
// below zero that are > -100 are LAPACK-style argument positions.
enum Status : int {
    kOk = 0,
    kErrCuda = -1001,        // a CUDA runtime call failed
    kErrTimeout = -1002,     // a bounded device-side wait gave up
    kErrNoDevice = -1003,    // no usable CUDA device
    kErrAlloc = -1004,       // device workspace allocation failed
    kErrUnsupported = -1005, // size/shape outside what this library supports
    kErrNotConverged = -1006 // iterative refinement did not reach tolerance
};

// Device-side status word bits (written by kernels, read by the host).
enum DeviceStatus : int {
    kDevOk = 0,
    kDevBarrierTimeout = 1,
    kDevMbarTimeout = 2,
};

void set_last_error(const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);

// Every device allocation of the library goes through here: it counts the
// allocations (flens_gb300_device_alloc_count) and honours the host-side
// failure hook flens_gb300_test_fail_device_allocs, which makes the next
// allocations fail as cudaMalloc does when the device is out of memory.
cudaError_t device_malloc(void **p, size_t bytes);

#define FG_CUDA(call)                                                     \
    do {                                                                  \
        cudaError_t _e = (call);                                          \
        if (_e != cudaSuccess) return ::fg::cuda_fail(_e, #call);         \
    } while (0)

inline int ceil_div(int a, int b) { return (a + b - 1) / b; }
inline size_t ceil_div(size_t a, size_t b) { return (a + b - 1) / b; }

// Per-(device, stream) workspace: scratch buffers kernels need beyond their
// inputs/outputs.  Grown on demand, never shrunk, freed at library unload.
struct Workspace {
    int device = -1;
    cudaStream_t stream = nullptr;
    void *buf = nullptr;         // general scratch (slot 0)
    size_t bytes = 0;
    void *slot_buf[4] = {nullptr, nullptr, nullptr, nullptr};   // slots 1..3
    size_t slot_bytes[4] = {0, 0, 0, 0};
    int *status = nullptr;       // device status word (DeviceStatus bits)
    int *info = nullptr;         // device INFO for host-pointer entry points
    // look-ahead: a high-priority side stream and two events that order it
    // against `stream` (created on first use)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fwd = nullptr, ev_back = nullptr;
    // ready flags of the chained triangular solve (flags_cap entries, never
    // moved once allocated) and the epoch the next call publishes
    unsigned long long *flags = nullptr;
    int flags_cap = 0;
    unsigned long long flag_epoch = 0;
};

// Returns the workspace bound to `stream` on the current device with at least
// `bytes` of scratch (nullptr on allocation failure; last error set).
Workspace *workspace_for(cudaStream_t stream, size_t bytes);

// Independent buffers 1..3 of the same workspace, for callers that hold
// pointers while calling routines that may grow slot 0.
void *workspace_slot(cudaStream_t stream, int slot, size_t bytes);

// The side stream and events of the workspace bound to `stream` (created
// on first use; nullptr on failure, last error set).
Workspace *workspace_side(cudaStream_t stream);

// The ready-flag array of the workspace bound to `stream` (at least n
// entries; allocated once with room for 4096) and a fresh epoch for one
// call.  Returns kOk, kErrUnsupported (n too large) or kErrAlloc.
int workspace_flags(cudaStream_t stream, int n, unsigned long long **flags,
                    unsigned long long *epoch);

int num_sms();                 // SM count of the current device
int device_id();               // current device ordinal

// Kernel attributes (the dynamic shared memory limit) belong to a device
// context: DeviceOnce remembers, per device, that one was set.
struct DeviceOnce {
    unsigned long long mask = 0;     // bit d: done on device d (benign race: setting twice is harmless)
    bool pending() const {
        const int d = device_id();
        return d < 0 || d >= 64 || !((__atomic_load_n(&mask, __ATOMIC_ACQUIRE) >> d) & 1ull);
    }
    void done() {
        const int d = device_id();
        if (d >= 0 && d < 64) __atomic_fetch_or(&mask, 1ull << d, __ATOMIC_ACQ_REL);
    }
};

// Sets the dynamic shared memory limit of `fn` to `bytes` once per device.
int set_smem_once(DeviceOnce &once, const void *fn, int bytes);

// Tracing: FLENS_GB300_TRACE=1 prints one line per kernel family chosen.
bool trace_enabled();
void trace(const char *fmt, ...);

// ------------------------------------------------- launch accounting --
// Every kernel launch of the library is wrapped in a KTimer: it counts the
// launch and, while timing is enabled (flens_gb300_timing_enable), records a
// CUDA event pair around it on the launching stream together with the
// launch's algorithmic flops and bytes.
enum Family : int {
    kFamGemm = 0,     // FP64 GEMM (trailing updates, trsm off-diagonal blocks)
    kFamPanel = 1,    // LU panel (pivot search, swap, scale, rank-1)
    kFamLaswp = 2,    // row interchanges
    kFamTrsm = 3,     // triangular diagonal-block solves
    kFamAux = 4,      // scaling, permutation helpers, conversions
    kFamTcGemm = 5,   // tcgen05 low-precision GEMM
    kFamRefine = 6,   // residual / refinement / Krylov helpers
    kFamBatched = 7,  // batched LU
    kFamSplit = 8,    // split-precision FP64 GEMM (slicing + tensor-core products)
    kFamTrsv = 9,     // chained triangular solves with few vectors (trs, refinement)
    kFamKrylov = 10,  // GMRES: permutation, Gram-Schmidt, norms, updates
    kFamPrecond = 11, // GMRES preconditioner: block inverses and chained solves
    kFamCount = 12
};

struct KTimer {
    KTimer(int family, cudaStream_t stream, double flops, double bytes);
    ~KTimer();
    int family;
    cudaStream_t stream;
    double flops, bytes;
    cudaEvent_t e0;
    bool on;
};

// ---------------------------------------------------------- device helpers --
__device__ __forceinline__ double ld_cg(const double *p) { return __ldcg(p); }
__device__ __forceinline__ int ld_cg(const int *p) { return __ldcg(p); }

// Bounded spin limit for every device-side wait (~1-2 s at GB300 clocks with
// the nanosleep back-off below).
constexpr unsigned kSpinLimit = 1u << 24;

// Grid-wide barrier for a cooperatively launched grid.  Every block must call
// it the same number of times.  Returns false (and sets *status) if the wait
// exceeded kSpinLimit; the caller must then return without further barriers.
struct GridBarrierState {
    unsigned int count;
    unsigned int generation;
};

__device__ __forceinline__ bool grid_barrier(GridBarrierState *bar,
                                             unsigned int nblocks,
                                             int *status) {
    __shared__ int s_ok;
    __syncthreads();
    if (nblocks == 1) return true;
    if (threadIdx.x == 0) {
        volatile unsigned int *vgen = &bar->generation;
        const unsigned int gen = *vgen;
        __threadfence();
        const unsigned int arrived = atomicAdd(&bar->count, 1u);
        int ok = 1;
        if (arrived == nblocks - 1) {
            atomicExch(&bar->count, 0u);
            __threadfence();
            atomicAdd(&bar->generation, 1u);
        } else {
            unsigned int spins = 0;
            while (*vgen == gen) {
                if (++spins > kSpinLimit) {
                    atomicOr(status, kDevBarrierTimeout);
                    ok = 0;
                    break;
                }
                if (spins > 64) __nanosleep(64);
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

}  // namespace fg

// ----------------------------------------------------- internal launchers --
// (host functions shared between translation units; all asynchronous on
// `stream`, returning a Status)
namespace fg {

int dgemm_launch(char transA, char transB, int m, int n, int k, double alpha,
                 const double *A, int ldA, const double *B, int ldB,
                 double beta, double *C, int ldC, cudaStream_t stream);

// dgemm with one triangular operand stored full (explicit zeros): kr 1/2 =
// op(A) upper/lower, 3/4 = op(B) upper/lower; the zero k blocks are skipped.
int dgemm_kr_launch(char transA, char transB, int m, int n, int k, double alpha,
                    const double *A, int ldA, const double *B, int ldB, double beta,
                    double *C, int ldC, int kr, cudaStream_t stream);

int dtrsm_launch(char side, char upLo, char transA, char diag, int m, int n,
                 double alpha, const double *A, int ldA, double *B, int ldB,
                 cudaStream_t stream);

// Scratch of the chained triangular solve supplied by the caller instead of
// the stream's workspace: `flags` holds `cap` ready flags, which the solve
// clears on its stream (cudaMemsetAsync) before each use, so every call
// publishes the same epoch; `status` receives the bounded-wait timeout bit.
struct ChainFixed {
    unsigned long long *flags;
    int cap;
    int *status;
};
int dtrsm_launch_fixed(char side, char upLo, char transA, char diag, int m, int n,
                       double alpha, const double *A, int ldA, double *B, int ldB,
                       const ChainFixed &fx, cudaStream_t stream);

int dscal_matrix_launch(int m, int n, double alpha, double *B, int ldB,
                        cudaStream_t stream);

// C <- beta*C + alpha*op(A)*op(A)^T on the uplo triangle ('L'/'U') of C,
// trans 'N' (A n x k) or 'T' (A k x n).
int dsyrk_launch(char uplo, char trans, int n, int k, double alpha,
                 const double *A, int ldA, double beta, double *C, int ldC,
                 cudaStream_t stream);

// C <- beta*C + alpha*op(A)*op(B)^T on the uplo triangle of C (trans 'N':
// A, B n x k; 'T': k x n).
int tri_gemm_launch(char uplo, char trans, int n, int k, double alpha,
                    const double *A, int ldA, const double *B, int ldB,
                    double beta, double *C, int ldC, cudaStream_t stream);

// Level-3 BLAS on the GEMM engine (blas3.cu): trmm (B <- alpha op(A) B or
// alpha B op(A), A triangular), symm (C <- beta C + alpha A B or alpha B A,
// A symmetric), syr2k (C <- beta C + alpha (op(A) op(B)^T + op(B) op(A)^T)).
int dtrmm_launch(char side, char uplo, char transA, char diag, int m, int n,
                 double alpha, const double *A, int ldA, double *B, int ldB,
                 cudaStream_t stream);
int dsymm_launch(char side, char uplo, int m, int n, double alpha,
                 const double *A, int ldA, const double *B, int ldB,
                 double beta, double *C, int ldC, cudaStream_t stream);
int dsyr2k_launch(char uplo, char trans, int n, int k, double alpha,
                  const double *A, int ldA, const double *B, int ldB,
                  double beta, double *C, int ldC, cudaStream_t stream);

// Triangular inverse in place (tri.cu); *info (device) = first exactly zero
// diagonal element (non-unit; A untouched then) or 0.  Synchronises to read
// it.
int dtrtri_launch(char uplo, char diag, int n, double *A, int ldA, int *info,
                  cudaStream_t stream);

// Inverse from dgetrf's factors and pivots (device ipiv, 1-based) in place;
// *info as dtrtri of U (A holds the factors when it is > 0).
int dgetri_launch(int n, double *A, int ldA, const int *ipiv, int *info,
                  cudaStream_t stream);

// Refinement, condition estimate, equilibration (refine.cu).  Matrices and
// vectors on the device; scalars (rcond, ferr, berr, ...) on the host; all
// synchronise.
int dgecon_launch(char norm, int n, const double *LU, int ldLU, double anorm,
                  double *rcond, cudaStream_t stream);
int dgerfs_launch(char trans, int n, int nrhs, const double *A, int ldA,
                  const double *AF, int ldAF, const int *ipiv, const double *B,
                  int ldB, double *X, int ldX, double *ferr, double *berr,
                  cudaStream_t stream);
int dgeequ_launch(int m, int n, const double *A, int ldA, double *r, double *c,
                  double *rowcnd, double *colcnd, double *amax, int *info,
                  cudaStream_t stream);
char dlaqge_launch(int m, int n, double *A, int ldA, const double *r,
                   const double *c, double rowcnd, double colcnd, double amax,
                   cudaStream_t stream);
int dgesvx_launch(char fact, char trans, int n, int nrhs, double *A, int ldA,
                  double *AF, int ldAF, int *ipiv, char *equed, double *r,
                  double *c, double *B, int ldB, double *X, int ldX,
                  double *rcond, double *ferr, double *berr, double *rpvgrw,
                  int *info, cudaStream_t stream);

// Cholesky (uplo 'L': A = L L^T, 'U': A = U^T U) of the n x n uplo triangle
// in place; *info (device) = first non-positive pivot (1-based) or 0.
// Synchronises once per 64-column block to stop at the first failure.
int dpotrf_launch(char uplo, int n, double *A, int ldA, int *info,
                  cudaStream_t stream);

// Solve A X = B with the Cholesky factor from dpotrf_launch.
int dpotrs_launch(char uplo, int n, int nrhs, const double *A, int ldA,
                  double *B, int ldB, cudaStream_t stream);

// FP32 counterparts (CUDA cores), used by the precision form's solves.
int sgemm_launch(char transA, char transB, int m, int n, int k, float alpha,
                 const float *A, int ldA, const float *B, int ldB,
                 float beta, float *C, int ldC, cudaStream_t stream);
int sscal_matrix_launch(int m, int n, float alpha, float *B, int ldB,
                        cudaStream_t stream);
int strsm_launch(char side, char upLo, char transA, char diag, int m, int n,
                 float alpha, const float *A, int ldA, float *B, int ldB,
                 cudaStream_t stream);

int dgetrf_launch(int m, int n, double *A, int ldA, int *ipiv, int *info,
                  cudaStream_t stream);
// FP64-accurate LU whose trailing updates beyond each outer block of
// `outer_nb` columns (a multiple of 64; <= 0: the default) run through the
// split GEMM; panels, interchanges, solves and the updates inside an outer
// block stay FP64.
int dgetrf_split_launch(int m, int n, double *A, int ldA, int *ipiv, int *info, int outer_nb,
                        cudaStream_t stream);

// FP64-accurate GEMM from exact BF16 products of exponent-aligned slices
// (split_gemm.cu); the _at form keeps its slot-0 data at byte offset
// ws0_off (split_ws0_bytes(m, n) bytes).
int dgemm_split_launch(char transA, char transB, int m, int n, int k, double alpha,
                       const double *A, int ldA, const double *B, int ldB, double beta,
                       double *C, int ldC, int slices, int *slices_used, cudaStream_t s);
int dgemm_split_launch_at(char transA, char transB, int m, int n, int k, double alpha,
                          const double *A, int ldA, const double *B, int ldB, double beta,
                          double *C, int ldC, int slices, int *slices_used, size_t ws0_off,
                          cudaStream_t s);
size_t split_ws0_bytes(int m, int n);

int dgetrs_launch(char trans, int n, int nrhs, const double *A, int ldA,
                  const int *ipiv, double *B, int ldB, cudaStream_t stream);

int dlaswp_launch(int nrows, int ncols, double *A, int ldA, int k1, int k2,
                  const int *ipiv, int inc, cudaStream_t stream);

int slaswp_launch(int nrows, int ncols, float *A, int ldA, int k1, int k2,
                  const int *ipiv, int inc, cudaStream_t stream);
// LU of FP32 storage (pivot search and scaling in FP64); the trailing update
// on the tensor cores in precision tc_kind (TcKind), or FP32 CUDA cores if < 0
int sgetrf_launch(int m, int n, float *A, int ldA, int *ipiv, int *info,
                  int tc_kind, cudaStream_t stream);
int sgetrs_launch(char trans, int n, int nrhs, const float *A, int ldA,
                  const int *ipiv, float *B, int ldB, cudaStream_t stream);

// Tensor-core trailing update C -= A21*U12 (m x n, depth k, FP32 storage)
// in precision `kind`, operand buffers at `buf`
// (tc_update_workspace_bytes(kind, m, n, k) bytes, 256-byte aligned).
size_t tc_update_workspace_bytes(int kind, int m, int n, int k);
int tc_trailing_update(int kind, int m, int n, int k, const float *A21, int ldA21,
                       const float *U12, int ldU12, float *A22, int ldA22, void *buf,
                       cudaStream_t stream);

// C = alpha * A * B + beta * C (FP32 storage, no transposes) as one
// FP32-accurate 3xTF32 tensor-core GEMM; `buf` holds
// tc_update_workspace_bytes(3, m, n, k) bytes.
int tc_gemm_f32x3_nn(int m, int n, int k, float alpha, const float *A, int ldA, const float *B,
                     int ldB, float beta, float *C, int ldC, void *buf, cudaStream_t stream);

// y = A x for an n x n triangular FP64 A whose other triangle holds zeros
// (uplo 'L' or 'U'): only the triangle and the zeros inside its 16 x 16
// diagonal blocks are read, y is only written.  Scratch:
// `part` of dtrmv_zeros_part_elems(n) doubles and `cnt` of
// dtrmv_zeros_cnt_elems(n) counters, zeroed once before the first call.
size_t dtrmv_zeros_part_elems(int n);
size_t dtrmv_zeros_cnt_elems(int n);
int dtrmv_zeros_launch(char uplo, int n, const double *A, int lda, const double *x, double *y,
                       double *part, unsigned *cnt, cudaStream_t s);
// y = A x for a square n x n FP64 A, same kernel and scratch.
int dgemv_chunk_launch(int n, const double *A, int lda, const double *x, double *y, double *part,
                       unsigned *cnt, cudaStream_t s);

// Reads and clears the workspace status word for `stream` (synchronises).
int check_device_status(cudaStream_t stream);

}  // namespace fg
