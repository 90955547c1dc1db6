// capi.cu -- the C ABI of the library.
//
// 1. Fortran-ABI drop-ins with the reference's argument checks and error
//    convention (xerbla_, then return; LAPACK routines also set INFO):
//      dgemm_   flens/blas/interface/blas/gemm.cc:120-230
//      dtrsm_   flens/blas/interface/blas/trsm.cc:90-166
//      dgetrf_  flens/lapack/interface/src/getrf.cc:10-45
//      dgetrs_  flens/lapack/interface/src/getrs.cc:13-53
//      dgesv_   flens/lapack/interface/src/gesv.cc:13-49
//      dsyrk_   flens/blas/interface/blas/syrk.cc:104-160
//      dtrmm_   flens/blas/interface/blas/trmm.cc:108-205
//      dsymm_   flens/blas/interface/blas/symm.cc:93-174
//      dsyr2k_  flens/blas/interface/blas/syr2k.cc:115-218
//      dpotrf_  flens/lapack/interface/src/potrf.cc:11-41
//      dpotrs_  flens/lapack/interface/src/potrs.cc:13-49
//      dposv_   flens/lapack/interface/src/posv.cc:13-51
//      dtrtri_  flens/lapack/interface/src/trtri.cc:9-55
//      dgetri_  flens/lapack/interface/src/getri.cc:10-53
//      dgerfs_, dgecon_, dgeequ_, dlaqge_, dgesvx_
//               flens/lapack/interface/src/{gerfs,gecon,geequ,laqge,gesvx}.cc
//    They take HOST pointers (as the reference does), copy the operands to
//    the device, run the GPU path and copy the results back before
//    returning.  Device (or managed) pointers are also accepted and used in
//    place.
// 2. flens_gb300_* device-pointer entry points, asynchronous on a caller
//    stream: the fast path for callers that keep matrices resident in HBM.
#include "common.cuh"

#include <cfloat>

#include <ctype.h>
#include <stdio.h>
#include <string.h>
#include <algorithm>

using namespace fg;

// ------------------------------------------------------------ xerbla ----
// Weak default: callers (or a Fortran runtime) may provide their own.  Like
// the Netlib routine it reports the routine name and the parameter position;
// unlike it, it does not stop the program.
static thread_local char g_xerbla_name[8];
static thread_local int g_xerbla_info;
static thread_local int g_xerbla_calls;

extern "C" __attribute__((weak, visibility("default"))) void xerbla_(const char *name,
                                                                    const int *info, int len) {
    (void)len;
    char buf[8] = {0};
    for (int i = 0; i < 6 && name[i]; ++i) buf[i] = name[i];
    fprintf(stderr, " ** On entry to %6s parameter number %2d had an illegal value\n", buf, *info);
}

// BLAS routines have no INFO argument: a failure inside the library (a CUDA
// error, a failed allocation, a device wait that timed out) goes to the
// caller's hook if one is set (flens_gb300_set_blas_error_hook), else to
// stderr, and is kept per thread for flens_gb300_blas_status().
FG_API const char *flens_gb300_last_error(void);
static thread_local int g_blas_status;
static void (*g_blas_hook)(const char *routine, int status, const char *message) = nullptr;

static void report_blas_failure(const char *routine, int st) {
    g_blas_status = st;
    if (st == kOk) return;
    void (*hook)(const char *, int, const char *) = __atomic_load_n(&g_blas_hook, __ATOMIC_ACQUIRE);
    if (hook) hook(routine, st, flens_gb300_last_error());
    else fprintf(stderr, "[flens_gb300] %s failed (%d): %s\n", routine, st, flens_gb300_last_error());
}

static void report_xerbla(const char *name, int info) {
    memset(g_xerbla_name, 0, sizeof g_xerbla_name);
    for (int i = 0; i < 6 && name[i]; ++i) g_xerbla_name[i] = name[i];
    g_xerbla_info = info;
    ++g_xerbla_calls;
    set_last_error("argument %d of %s had an illegal value", info, g_xerbla_name);
    xerbla_(name, &info, 6);
}

FG_API int flens_gb300_xerbla_calls(void) { return g_xerbla_calls; }
FG_API int flens_gb300_xerbla_info(void) { return g_xerbla_info; }
FG_API const char *flens_gb300_xerbla_name(void) { return g_xerbla_name; }

// --------------------------------------------------------- host staging --
namespace {

struct HostStage {
    cudaStream_t stream = nullptr;
    void *buf[4] = {nullptr, nullptr, nullptr, nullptr};
    size_t bytes[4] = {0, 0, 0, 0};
    ~HostStage() {
        for (int i = 0; i < 4; ++i)
            if (buf[i]) cudaFree(buf[i]);
        if (stream) cudaStreamDestroy(stream);
    }
};
thread_local HostStage t_stage;

int stage_stream(cudaStream_t *out) {
    if (!t_stage.stream) FG_CUDA(cudaStreamCreateWithFlags(&t_stage.stream, cudaStreamNonBlocking));
    *out = t_stage.stream;
    return kOk;
}

int stage_buf(int slot, size_t bytes, void **out) {
    if (t_stage.bytes[slot] < bytes) {
        if (t_stage.buf[slot]) {
            cudaStreamSynchronize(t_stage.stream);
            cudaFree(t_stage.buf[slot]);
            t_stage.buf[slot] = nullptr;
            t_stage.bytes[slot] = 0;
        }
        const cudaError_t e = device_malloc(&t_stage.buf[slot], bytes < 256 ? 256 : bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            t_stage.buf[slot] = nullptr;
            set_last_error("cudaMalloc of %zu bytes of host-call staging failed", bytes);
            return kErrAlloc;
        }
        t_stage.bytes[slot] = bytes;
    }
    *out = t_stage.buf[slot];
    return kOk;
}

bool is_device_ptr(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// A host rows x cols column-major matrix with leading dimension ld, viewed on
// the device: either the pointer itself (device/managed memory) or a staged
// copy with leading dimension `rows`.
struct DevView {
    double *p = nullptr;
    int ld = 1;
    bool staged = false;
};

// Copies between device memory and PINNED host memory can run as a kernel
// that loads or stores the host array through its device mapping (pinned
// memory is mapped into the GPU's address space), instead of a copy-engine
// DMA.  On this part a 512 MiB DMA to pinned host memory took either 2.8 ms
// or 22-45 ms from one call to the next (the LU beside it did not change); a
// kernel takes the same path every time.  FLENS_GB300_HOST_COPY=dma keeps the
// DMA.  Pageable host memory always goes through the DMA path.
__global__ void host_copy_kernel(int rows, int cols, const double *__restrict__ src, long long lds,
                                 double *__restrict__ dst, long long ldd) {
    if (lds == rows && ldd == rows && ((((uintptr_t)src) | ((uintptr_t)dst)) & 15) == 0) {
        const size_t total = (size_t)rows * cols, pairs = total / 2;
        const double2 *s2 = (const double2 *)src;
        double2 *d2 = (double2 *)dst;
        for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < pairs;
             e += (size_t)gridDim.x * blockDim.x)
            d2[e] = s2[e];
        if ((total & 1) && blockIdx.x == 0 && threadIdx.x == 0) dst[total - 1] = src[total - 1];
        return;
    }
    const size_t total = (size_t)rows * cols;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const size_t j = e / rows, i = e % rows;
        dst[i + j * ldd] = src[i + j * lds];
    }
}

bool host_copy_by_kernel() {
    static bool on = [] {
        const char *e = getenv("FLENS_GB300_HOST_COPY");
        return !(e && strcmp(e, "dma") == 0);
    }();
    return on;
}

// Device address of pinned (mapped) host memory, or nullptr for pageable
// memory and device memory.
void *mapped_host(const void *h) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

int host_copy_launch(int rows, int cols, const double *src, long long lds, double *dst, long long ldd,
                     cudaStream_t s) {
    const size_t total = (size_t)rows * cols;
    int blocks = (int)ceil_div(total, (size_t)512);
    if (blocks > num_sms() * 8) blocks = num_sms() * 8;
    if (blocks < 1) blocks = 1;
    KTimer kt(kFamAux, s, 0.0, 16.0 * (double)total);
    host_copy_kernel<<<blocks, 256, 0, s>>>(rows, cols, src, lds, dst, ldd);
    FG_CUDA(cudaGetLastError());
    return kOk;
}

int view_in(int slot, const double *h, int rows, int cols, int ld, bool copy, cudaStream_t s,
            DevView *v) {
    if (is_device_ptr(h)) {
        v->p = const_cast<double *>(h);
        v->ld = ld;
        v->staged = false;
        return kOk;
    }
    const int dld = rows > 0 ? rows : 1;
    void *d;
    int st = stage_buf(slot, (size_t)dld * (cols > 0 ? cols : 1) * sizeof(double), &d);
    if (st != kOk) return st;
    v->p = (double *)d;
    v->ld = dld;
    v->staged = true;
    if (copy && rows > 0 && cols > 0) {
        const void *hd = host_copy_by_kernel() ? mapped_host(h) : nullptr;
        if (hd) return host_copy_launch(rows, cols, (const double *)hd, ld, v->p, dld, s);
        if (ld == dld)      // one contiguous block: a plain copy
            FG_CUDA(cudaMemcpyAsync(v->p, h, (size_t)dld * cols * sizeof(double), cudaMemcpyHostToDevice, s));
        else
            FG_CUDA(cudaMemcpy2DAsync(v->p, (size_t)dld * sizeof(double), h, (size_t)ld * sizeof(double),
                                      (size_t)rows * sizeof(double), cols, cudaMemcpyHostToDevice, s));
    }
    return kOk;
}

int view_out(const DevView &v, double *h, int rows, int cols, int ld, cudaStream_t s) {
    if (!v.staged || rows <= 0 || cols <= 0) return kOk;
    void *hd = host_copy_by_kernel() ? mapped_host(h) : nullptr;
    if (hd) return host_copy_launch(rows, cols, v.p, v.ld, (double *)hd, ld, s);
    if (ld == v.ld)
        FG_CUDA(cudaMemcpyAsync(h, v.p, (size_t)v.ld * cols * sizeof(double), cudaMemcpyDeviceToHost, s));
    else
        FG_CUDA(cudaMemcpy2DAsync(h, (size_t)ld * sizeof(double), v.p, (size_t)v.ld * sizeof(double),
                                  (size_t)rows * sizeof(double), cols, cudaMemcpyDeviceToHost, s));
    return kOk;
}

int finish(cudaStream_t s) {
    FG_CUDA(cudaStreamSynchronize(s));
    return check_device_status(s);
}

}  // namespace

FG_API const char *flens_gb300_last_error(void);
// --------------------------------------------------------------- dgemm_ --
static int dgemm_host(char ta, char tb, int m, int n, int k, double alpha, const double *A,
                      int ldA, const double *B, int ldB, double beta, double *C, int ldC) {
    if (m == 0 || n == 0) return kOk;
    cudaStream_t s;
    int st = stage_stream(&s);
    if (st != kOk) return st;
    const bool nA = ta == 'N', nB = tb == 'N';
    DevView a, b, c;
    const bool need_ab = alpha != 0.0 && k > 0;
    if (need_ab) {
        if ((st = view_in(0, A, nA ? m : k, nA ? k : m, ldA, true, s, &a)) != kOk) return st;
        if ((st = view_in(1, B, nB ? k : n, nB ? n : k, ldB, true, s, &b)) != kOk) return st;
    }
    if ((st = view_in(2, C, m, n, ldC, true, s, &c)) != kOk) return st;
    if (need_ab)
        st = dgemm_launch(ta, tb, m, n, k, alpha, a.p, a.ld, b.p, b.ld, beta, c.p, c.ld, s);
    else
        st = dgemm_launch(ta, tb, m, n, 0, alpha, nullptr, 1, nullptr, 1, beta, c.p, c.ld, s);
    if (st != kOk) return st;
    if ((st = view_out(c, C, m, n, ldC, s)) != kOk) return st;
    return finish(s);
}

FG_API void dgemm_(const char *TRANSA, const char *TRANSB, const int *M, const int *N,
                   const int *K, const double *ALPHA, const double *A, const int *LDA,
                   const double *B, const int *LDB, const double *BETA, double *C,
                   const int *LDC) {
    const char ta = (char)toupper(*TRANSA), tb = (char)toupper(*TRANSB);
    const int nRowA = (ta == 'N') ? *M : *K;
    const int nRowB = (tb == 'N') ? *K : *N;
    int info = 0;
    if (ta != 'N' && ta != 'C' && ta != 'T') info = 1;
    else if (tb != 'N' && tb != 'C' && tb != 'T') info = 2;
    else if (*M < 0) info = 3;
    else if (*N < 0) info = 4;
    else if (*K < 0) info = 5;
    else if (*LDA < std::max(1, nRowA)) info = 8;
    else if (*LDB < std::max(1, nRowB)) info = 10;
    else if (*LDC < std::max(1, *M)) info = 13;
    if (info != 0) {
        report_xerbla("DGEMM ", info);
        return;
    }
    const int st = dgemm_host(ta == 'C' ? 'T' : ta, tb == 'C' ? 'T' : tb, *M, *N, *K, *ALPHA, A,
                              *LDA, B, *LDB, *BETA, C, *LDC);
    report_blas_failure("dgemm_", st);
}

// --------------------------------------------------------------- dtrsm_ --
FG_API void dtrsm_(const char *SIDE, const char *UPLO, const char *TRANSA, const char *DIAG,
                   const int *M, const int *N, const double *ALPHA, const double *A,
                   const int *LDA, double *B, const int *LDB) {
    const char side = (char)toupper(*SIDE), uplo = (char)toupper(*UPLO);
    const char ta = (char)toupper(*TRANSA), diag = (char)toupper(*DIAG);
    const int nRowA = (side == 'L') ? *M : *N;
    int info = 0;
    if (side != 'L' && side != 'R') info = 1;
    else if (uplo != 'U' && uplo != 'L') info = 2;
    else if (ta != 'N' && ta != 'T' && ta != 'C') info = 3;
    else if (diag != 'U' && diag != 'N') info = 4;
    else if (*M < 0) info = 5;
    else if (*N < 0) info = 6;
    else if (*LDA < std::max(1, nRowA)) info = 9;
    else if (*LDB < std::max(1, *M)) info = 11;
    if (info != 0) {
        report_xerbla("DTRSM ", info);
        return;
    }
    const int m = *M, n = *N;
    if (m == 0 || n == 0) return;
    cudaStream_t s;
    int st = stage_stream(&s);
    DevView a, b;
    const int ka = side == 'L' ? m : n;
    if (st == kOk) st = view_in(0, A, ka, ka, *LDA, true, s, &a);
    if (st == kOk) st = view_in(1, B, m, n, *LDB, true, s, &b);
    if (st == kOk)
        st = dtrsm_launch(side, uplo, ta == 'C' ? 'T' : ta, diag, m, n, *ALPHA, a.p, a.ld, b.p, b.ld, s);
    if (st == kOk) st = view_out(b, B, m, n, *LDB, s);
    if (st == kOk) st = finish(s);
    report_blas_failure("dtrsm_", st);
}

// ----------------------------------------------------------- LAPACK LU --
namespace {

// ipiv staging: device copy of an int vector
int ipiv_dev(int slot, int *h, int len, bool copy_in, cudaStream_t s, int **d, bool *staged) {
    if (is_device_ptr(h)) {
        *d = h;
        *staged = false;
        return kOk;
    }
    void *p;
    int st = stage_buf(slot, (size_t)(len > 0 ? len : 1) * sizeof(int), &p);
    if (st != kOk) return st;
    *d = (int *)p;
    *staged = true;
    if (copy_in && len > 0) FG_CUDA(cudaMemcpyAsync(*d, h, (size_t)len * sizeof(int), cudaMemcpyHostToDevice, s));
    return kOk;
}

int getrf_host(int m, int n, double *A, int ldA, int *IPIV, int *INFO) {
    *INFO = 0;
    if (m == 0 || n == 0) return kOk;
    cudaStream_t s;
    int st = stage_stream(&s);
    if (st != kOk) return st;
    DevView a;
    if ((st = view_in(0, A, m, n, ldA, true, s, &a)) != kOk) return st;
    const int mn = std::min(m, n);
    int *dpiv;
    bool pstaged;
    if ((st = ipiv_dev(3, IPIV, mn, false, s, &dpiv, &pstaged)) != kOk) return st;
    Workspace *w = workspace_for(s, 0);
    if (!w) return kErrAlloc;
    if ((st = dgetrf_launch(m, n, a.p, a.ld, dpiv, w->info, s)) != kOk) return st;
    if ((st = view_out(a, A, m, n, ldA, s)) != kOk) return st;
    if (pstaged) FG_CUDA(cudaMemcpyAsync(IPIV, dpiv, (size_t)mn * sizeof(int), cudaMemcpyDeviceToHost, s));
    FG_CUDA(cudaMemcpyAsync(INFO, w->info, sizeof(int), cudaMemcpyDeviceToHost, s));
    return finish(s);
}

int getrs_host(char trans, int n, int nrhs, const double *A, int ldA, const int *IPIV, double *B,
               int ldB) {
    if (n == 0 || nrhs == 0) return kOk;
    cudaStream_t s;
    int st = stage_stream(&s);
    if (st != kOk) return st;
    DevView a, b;
    if ((st = view_in(0, A, n, n, ldA, true, s, &a)) != kOk) return st;
    if ((st = view_in(1, B, n, nrhs, ldB, true, s, &b)) != kOk) return st;
    int *dpiv;
    bool pstaged;
    if ((st = ipiv_dev(3, const_cast<int *>(IPIV), n, true, s, &dpiv, &pstaged)) != kOk) return st;
    if ((st = dgetrs_launch(trans, n, nrhs, a.p, a.ld, dpiv, b.p, b.ld, s)) != kOk) return st;
    if ((st = view_out(b, B, n, nrhs, ldB, s)) != kOk) return st;
    return finish(s);
}

int gesv_host(int n, int nrhs, double *A, int ldA, int *IPIV, double *B, int ldB, int *INFO) {
    *INFO = 0;
    if (n == 0) return kOk;
    cudaStream_t s;
    int st = stage_stream(&s);
    if (st != kOk) return st;
    DevView a, b;
    if ((st = view_in(0, A, n, n, ldA, true, s, &a)) != kOk) return st;
    if ((st = view_in(1, B, n, nrhs, ldB, true, s, &b)) != kOk) return st;
    int *dpiv;
    bool pstaged;
    if ((st = ipiv_dev(3, IPIV, n, false, s, &dpiv, &pstaged)) != kOk) return st;
    Workspace *w = workspace_for(s, 0);
    if (!w) return kErrAlloc;
    if ((st = dgetrf_launch(n, n, a.p, a.ld, dpiv, w->info, s)) != kOk) return st;
    // the factors and pivots go back on the side stream while the solve runs
    // (both only read them)
    Workspace *ws = (a.staged || pstaged) ? workspace_side(s) : nullptr;
    cudaStream_t cs = ws ? ws->side : s;
    if (ws) {
        FG_CUDA(cudaEventRecord(ws->ev_fwd, s));
        FG_CUDA(cudaStreamWaitEvent(cs, ws->ev_fwd, 0));
    }
    if ((st = view_out(a, A, n, n, ldA, cs)) != kOk) return st;
    if (pstaged) FG_CUDA(cudaMemcpyAsync(IPIV, dpiv, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, cs));
    if (ws) FG_CUDA(cudaEventRecord(ws->ev_back, cs));
    FG_CUDA(cudaMemcpyAsync(INFO, w->info, sizeof(int), cudaMemcpyDeviceToHost, s));
    FG_CUDA(cudaStreamSynchronize(s));
    // flens/lapack/ge/sv.tcc:70-75: solve only if the factorisation succeeded
    if (*INFO == 0 && nrhs > 0) {
        if ((st = dgetrs_launch('N', n, nrhs, a.p, a.ld, dpiv, b.p, b.ld, s)) != kOk) return st;
        if ((st = view_out(b, B, n, nrhs, ldB, s)) != kOk) return st;
    }
    if (ws) FG_CUDA(cudaStreamWaitEvent(s, ws->ev_back, 0));
    return finish(s);
}

}  // namespace

FG_API void dgetrf_(const int *M, const int *N, double *A, const int *LDA, int *IPIV, int *INFO) {
    *INFO = 0;
    if (*M < 0) *INFO = -1;
    else if (*N < 0) *INFO = -2;
    else if (*LDA < std::max(1, *M)) *INFO = -4;
    if (*INFO != 0) {
        report_xerbla("DGETRF", -*INFO);
        return;
    }
    const int st = getrf_host(*M, *N, A, *LDA, IPIV, INFO);
    if (st != kOk) *INFO = st;
}

FG_API void dgetrs_(const char *TRANS, const int *N, const int *NRHS, const double *A,
                    const int *LDA, const int *IPIV, double *B, const int *LDB, int *INFO) {
    *INFO = 0;
    if (*TRANS != 'N' && *TRANS != 'T' && *TRANS != 'C') *INFO = -1;
    else if (*N < 0) *INFO = -2;
    else if (*NRHS < 0) *INFO = -3;
    else if (*LDA < std::max(1, *N)) *INFO = -5;
    else if (*LDB < std::max(1, *N)) *INFO = -8;
    if (*INFO != 0) {
        report_xerbla("DGETRS", -*INFO);
        return;
    }
    const int st = getrs_host(*TRANS == 'C' ? 'T' : *TRANS, *N, *NRHS, A, *LDA, IPIV, B, *LDB);
    if (st != kOk) *INFO = st;
}

FG_API void dgesv_(const int *N, const int *NRHS, double *A, const int *LDA, int *IPIV, double *B,
                   const int *LDB, int *INFO) {
    *INFO = 0;
    if (*N < 0) *INFO = -1;
    else if (*NRHS < 0) *INFO = -2;
    else if (*LDA < std::max(1, *N)) *INFO = -4;
    else if (*LDB < std::max(1, *N)) *INFO = -7;
    if (*INFO != 0) {
        report_xerbla("DGESV ", -*INFO);
        return;
    }
    int info = 0;
    const int st = gesv_host(*N, *NRHS, A, *LDA, IPIV, B, *LDB, &info);
    *INFO = (st != kOk) ? st : info;
}

// --------------------------------------------------------------- dsyrk_ --
// flens/blas/interface/blas/syrk.cc:104-160: UPLO and TRANS upper-cased, then
// checked in argument order (positions 1, 2, 3, 4, 7, 10).
FG_API void dsyrk_(const char *UPLO, const char *TRANS, const int *N, const int *K,
                   const double *ALPHA, const double *A, const int *LDA, const double *BETA,
                   double *C, const int *LDC) {
    const char uplo = (char)toupper(*UPLO), tr = (char)toupper(*TRANS);
    const int nRowA = (tr == 'N') ? *N : *K;
    int info = 0;
    if (uplo != 'U' && uplo != 'L') info = 1;
    else if (tr != 'N' && tr != 'T' && tr != 'C') info = 2;
    else if (*N < 0) info = 3;
    else if (*K < 0) info = 4;
    else if (*LDA < std::max(1, nRowA)) info = 7;
    else if (*LDC < std::max(1, *N)) info = 10;
    if (info != 0) {
        report_xerbla("DSYRK ", info);
        return;
    }
    const int n = *N, k = *K;
    if (n == 0) return;
    cudaStream_t s;
    int st = stage_stream(&s);
    DevView a, c;
    if (st == kOk && k > 0)
        st = view_in(0, A, tr == 'N' ? n : k, tr == 'N' ? k : n, *LDA, true, s, &a);
    if (st == kOk) st = view_in(1, C, n, n, *LDC, true, s, &c);
    if (st == kOk)
        st = dsyrk_launch(uplo, tr == 'N' ? 'N' : 'T', n, k, *ALPHA, a.p, a.ld, *BETA, c.p, c.ld, s);
    if (st == kOk) st = view_out(c, C, n, n, *LDC, s);
    if (st == kOk) st = finish(s);
    report_blas_failure("dsyrk_", st);
}

// ---------------------------------------------------------------- dtrmm_ --
// flens/blas/interface/blas/trmm.cc:108-205: upper-cased, checked 1, 2, 3, 4, 5, 6, 9, 11
FG_API void dtrmm_(const char *SIDE, const char *UPLO, const char *TRANSA, const char *DIAG,
                   const int *M, const int *N, const double *ALPHA, const double *A,
                   const int *LDA, double *B, const int *LDB) {
    const char side = (char)toupper(*SIDE), uplo = (char)toupper(*UPLO);
    const char ta = (char)toupper(*TRANSA), diag = (char)toupper(*DIAG);
    const int nRowA = (side == 'L') ? *M : *N;
    int info = 0;
    if (side != 'L' && side != 'R') info = 1;
    else if (uplo != 'U' && uplo != 'L') info = 2;
    else if (ta != 'N' && ta != 'T' && ta != 'C') info = 3;
    else if (diag != 'U' && diag != 'N') info = 4;
    else if (*M < 0) info = 5;
    else if (*N < 0) info = 6;
    else if (*LDA < std::max(1, nRowA)) info = 9;
    else if (*LDB < std::max(1, *M)) info = 11;
    if (info != 0) {
        report_xerbla("DTRMM ", info);
        return;
    }
    const int m = *M, n = *N;
    if (m == 0 || n == 0) return;
    cudaStream_t s;
    int st = stage_stream(&s);
    DevView a, b;
    const int ka = side == 'L' ? m : n;
    if (st == kOk) st = view_in(0, A, ka, ka, *LDA, true, s, &a);
    if (st == kOk) st = view_in(1, B, m, n, *LDB, true, s, &b);
    if (st == kOk) st = dtrmm_launch(side, uplo, ta == 'C' ? 'T' : ta, diag, m, n, *ALPHA, a.p, a.ld, b.p, b.ld, s);
    if (st == kOk) st = view_out(b, B, m, n, *LDB, s);
    if (st == kOk) st = finish(s);
    report_blas_failure("dtrmm_", st);
}

// ---------------------------------------------------------------- dsymm_ --
// flens/blas/interface/blas/symm.cc:93-174: upper-cased, checked 1, 2, 3, 4, 7, 9, 12
FG_API void dsymm_(const char *SIDE, const char *UPLO, const int *M, const int *N,
                   const double *ALPHA, const double *A, const int *LDA, const double *B,
                   const int *LDB, const double *BETA, double *C, const int *LDC) {
    const char side = (char)toupper(*SIDE), uplo = (char)toupper(*UPLO);
    const int nRowA = (side == 'L') ? *M : *N;
    int info = 0;
    if (side != 'L' && side != 'R') info = 1;
    else if (uplo != 'U' && uplo != 'L') info = 2;
    else if (*M < 0) info = 3;
    else if (*N < 0) info = 4;
    else if (*LDA < std::max(1, nRowA)) info = 7;
    else if (*LDB < std::max(1, *M)) info = 9;
    else if (*LDC < std::max(1, *M)) info = 12;
    if (info != 0) {
        report_xerbla("DSYMM ", info);
        return;
    }
    const int m = *M, n = *N;
    if (m == 0 || n == 0) return;
    cudaStream_t s;
    int st = stage_stream(&s);
    DevView a, b, c;
    const int ka = side == 'L' ? m : n;
    if (st == kOk) st = view_in(0, A, ka, ka, *LDA, true, s, &a);
    if (st == kOk) st = view_in(1, B, m, n, *LDB, true, s, &b);
    if (st == kOk) st = view_in(2, C, m, n, *LDC, true, s, &c);
    if (st == kOk) st = dsymm_launch(side, uplo, m, n, *ALPHA, a.p, a.ld, b.p, b.ld, *BETA, c.p, c.ld, s);
    if (st == kOk) st = view_out(c, C, m, n, *LDC, s);
    if (st == kOk) st = finish(s);
    report_blas_failure("dsymm_", st);
}

// --------------------------------------------------------------- dsyr2k_ --
// flens/blas/interface/blas/syr2k.cc:115-218: upper-cased, checked 1, 2, 3, 4, 7, 9, 12
FG_API void dsyr2k_(const char *UPLO, const char *TRANS, const int *N, const int *K,
                    const double *ALPHA, const double *A, const int *LDA, const double *B,
                    const int *LDB, const double *BETA, double *C, const int *LDC) {
    const char uplo = (char)toupper(*UPLO), tr = (char)toupper(*TRANS);
    const int nRowA = (tr == 'N') ? *N : *K;
    int info = 0;
    if (uplo != 'U' && uplo != 'L') info = 1;
    else if (tr != 'N' && tr != 'T' && tr != 'C') info = 2;
    else if (*N < 0) info = 3;
    else if (*K < 0) info = 4;
    else if (*LDA < std::max(1, nRowA)) info = 7;
    else if (*LDB < std::max(1, nRowA)) info = 9;
    else if (*LDC < std::max(1, *N)) info = 12;
    if (info != 0) {
        report_xerbla("DSYR2K", info);
        return;
    }
    const int n = *N, k = *K;
    if (n == 0) return;
    cudaStream_t s;
    int st = stage_stream(&s);
    DevView a, b, c;
    const int ra = tr == 'N' ? n : k, ca = tr == 'N' ? k : n;
    if (st == kOk && k > 0) st = view_in(0, A, ra, ca, *LDA, true, s, &a);
    if (st == kOk && k > 0) st = view_in(1, B, ra, ca, *LDB, true, s, &b);
    if (st == kOk) st = view_in(2, C, n, n, *LDC, true, s, &c);
    if (st == kOk)
        st = dsyr2k_launch(uplo, tr == 'N' ? 'N' : 'T', n, k, *ALPHA, a.p, a.ld, b.p, b.ld, *BETA, c.p, c.ld, s);
    if (st == kOk) st = view_out(c, C, n, n, *LDC, s);
    if (st == kOk) st = finish(s);
    report_blas_failure("dsyr2k_", st);
}

// ------------------------------------------------------ LAPACK Cholesky --
namespace {

int potrf_host(char uplo, int n, double *A, int ldA, int *INFO) {
    *INFO = 0;
    if (n == 0) return kOk;
    cudaStream_t s;
    int st = stage_stream(&s);
    if (st != kOk) return st;
    DevView a;
    if ((st = view_in(0, A, n, n, ldA, true, s, &a)) != kOk) return st;
    Workspace *w = workspace_for(s, 0);
    if (!w) return kErrAlloc;
    if ((st = dpotrf_launch(uplo, n, a.p, a.ld, w->info, s)) != kOk) return st;
    if ((st = view_out(a, A, n, n, ldA, s)) != kOk) return st;
    FG_CUDA(cudaMemcpyAsync(INFO, w->info, sizeof(int), cudaMemcpyDeviceToHost, s));
    return finish(s);
}

int potrs_host(char uplo, int n, int nrhs, const double *A, int ldA, double *B, int ldB) {
    if (n == 0 || nrhs == 0) return kOk;
    cudaStream_t s;
    int st = stage_stream(&s);
    if (st != kOk) return st;
    DevView a, b;
    if ((st = view_in(0, A, n, n, ldA, true, s, &a)) != kOk) return st;
    if ((st = view_in(1, B, n, nrhs, ldB, true, s, &b)) != kOk) return st;
    if ((st = dpotrs_launch(uplo, n, nrhs, a.p, a.ld, b.p, b.ld, s)) != kOk) return st;
    if ((st = view_out(b, B, n, nrhs, ldB, s)) != kOk) return st;
    return finish(s);
}

int posv_host(char uplo, int n, int nrhs, double *A, int ldA, double *B, int ldB, int *INFO) {
    *INFO = 0;
    if (n == 0) return kOk;
    cudaStream_t s;
    int st = stage_stream(&s);
    if (st != kOk) return st;
    DevView a, b;
    if ((st = view_in(0, A, n, n, ldA, true, s, &a)) != kOk) return st;
    if ((st = view_in(1, B, n, nrhs, ldB, true, s, &b)) != kOk) return st;
    Workspace *w = workspace_for(s, 0);
    if (!w) return kErrAlloc;
    if ((st = dpotrf_launch(uplo, n, a.p, a.ld, w->info, s)) != kOk) return st;
    FG_CUDA(cudaMemcpyAsync(INFO, w->info, sizeof(int), cudaMemcpyDeviceToHost, s));
    FG_CUDA(cudaStreamSynchronize(s));
    // flens/lapack/po/posv.tcc:58-64: solve only if the factorisation succeeded
    if (*INFO == 0 && nrhs > 0) {
        if ((st = dpotrs_launch(uplo, n, nrhs, a.p, a.ld, b.p, b.ld, s)) != kOk) return st;
        if ((st = view_out(b, B, n, nrhs, ldB, s)) != kOk) return st;
    }
    if ((st = view_out(a, A, n, n, ldA, s)) != kOk) return st;
    return finish(s);
}

}  // namespace

// flens/lapack/interface/src/potrf.cc:11-41: UPLO must be exactly 'U' or 'L'.
FG_API void dpotrf_(const char *UPLO, const int *N, double *A, const int *LDA, int *INFO) {
    *INFO = 0;
    if (*UPLO != 'U' && *UPLO != 'L') *INFO = -1;
    else if (*N < 0) *INFO = -2;
    else if (*LDA < std::max(1, *N)) *INFO = -4;
    if (*INFO != 0) {
        report_xerbla("DPOTRF", -*INFO);
        return;
    }
    int info = 0;
    const int st = potrf_host(*UPLO, *N, A, *LDA, &info);
    *INFO = (st != kOk) ? st : info;
}

// flens/lapack/interface/src/potrs.cc:13-49
FG_API void dpotrs_(const char *UPLO, const int *N, const int *NRHS, const double *A,
                    const int *LDA, double *B, const int *LDB, int *INFO) {
    *INFO = 0;
    if (*UPLO != 'U' && *UPLO != 'L') *INFO = -1;
    else if (*N < 0) *INFO = -2;
    else if (*NRHS < 0) *INFO = -3;
    else if (*LDA < std::max(1, *N)) *INFO = -5;
    else if (*LDB < std::max(1, *N)) *INFO = -7;
    if (*INFO != 0) {
        report_xerbla("DPOTRS", -*INFO);
        return;
    }
    const int st = potrs_host(*UPLO, *N, *NRHS, A, *LDA, B, *LDB);
    if (st != kOk) *INFO = st;
}

// flens/lapack/interface/src/posv.cc:13-51.  The reference's shim discards
// posv's return value (INFO stays 0 on a failed factorisation); this one
// returns it, as LAPACK's DPOSV and FLENS's own posv() do.
FG_API void dposv_(const char *UPLO, const int *N, const int *NRHS, double *A, const int *LDA,
                   double *B, const int *LDB, int *INFO) {
    *INFO = 0;
    if (*UPLO != 'U' && *UPLO != 'L') *INFO = -1;
    else if (*N < 0) *INFO = -2;
    else if (*NRHS < 0) *INFO = -3;
    else if (*LDA < std::max(1, *N)) *INFO = -5;
    else if (*LDB < std::max(1, *N)) *INFO = -7;
    if (*INFO != 0) {
        report_xerbla("DPOSV ", -*INFO);
        return;
    }
    int info = 0;
    const int st = posv_host(*UPLO, *N, *NRHS, A, *LDA, B, *LDB, &info);
    *INFO = (st != kOk) ? st : info;
}

// ------------------------------------------------------ LAPACK inverses --
namespace {

int trtri_host(char uplo, char diag, int n, double *A, int ldA, int *INFO) {
    *INFO = 0;
    if (n == 0) return kOk;
    cudaStream_t s;
    int st = stage_stream(&s);
    if (st != kOk) return st;
    DevView a;
    if ((st = view_in(0, A, n, n, ldA, true, s, &a)) != kOk) return st;
    Workspace *w = workspace_for(s, 0);
    if (!w) return kErrAlloc;
    if ((st = dtrtri_launch(uplo, diag, n, a.p, a.ld, w->info, s)) != kOk) return st;
    if ((st = view_out(a, A, n, n, ldA, s)) != kOk) return st;
    FG_CUDA(cudaMemcpyAsync(INFO, w->info, sizeof(int), cudaMemcpyDeviceToHost, s));
    return finish(s);
}

int getri_host(int n, double *A, int ldA, const int *IPIV, int *INFO) {
    *INFO = 0;
    if (n == 0) return kOk;
    cudaStream_t s;
    int st = stage_stream(&s);
    if (st != kOk) return st;
    DevView a;
    if ((st = view_in(0, A, n, n, ldA, true, s, &a)) != kOk) return st;
    int *dpiv;
    bool pstaged;
    if ((st = ipiv_dev(3, const_cast<int *>(IPIV), n, true, s, &dpiv, &pstaged)) != kOk) return st;
    Workspace *w = workspace_for(s, 0);
    if (!w) return kErrAlloc;
    if ((st = dgetri_launch(n, a.p, a.ld, dpiv, w->info, s)) != kOk) return st;
    if ((st = view_out(a, A, n, n, ldA, s)) != kOk) return st;
    FG_CUDA(cudaMemcpyAsync(INFO, w->info, sizeof(int), cudaMemcpyDeviceToHost, s));
    return finish(s);
}

}  // namespace

// flens/lapack/interface/src/trtri.cc:9-55: UPLO exactly 'U'/'L', DIAG 'N'/'U'.
// The reference's shim discards tri's return value; this one reports a zero
// diagonal element in INFO (LAPACK DTRTRI semantics, A untouched then).
FG_API void dtrtri_(const char *UPLO, const char *DIAG, const int *N, double *A, const int *LDA,
                    int *INFO) {
    *INFO = 0;
    if (*UPLO != 'U' && *UPLO != 'L') *INFO = -1;
    else if (*DIAG != 'N' && *DIAG != 'U') *INFO = -2;
    else if (*N < 0) *INFO = -3;
    else if (*LDA < std::max(1, *N)) *INFO = -5;
    if (*INFO != 0) {
        report_xerbla("DTRTRI", -*INFO);
        return;
    }
    int info = 0;
    const int st = trtri_host(*UPLO, *DIAG, *N, A, *LDA, &info);
    *INFO = (st != kOk) ? st : info;
}

// flens/lapack/interface/src/getri.cc:10-53 (checks N, LDA, LWORK >= max(1,N)
// unless LWORK == -1).  A workspace query returns WORK(1) = N*64 at once; the
// GPU path uses its own device workspace and reports the same optimum.  INFO
// reports an exactly zero U(i,i) (LAPACK DGETRI semantics; the reference's
// shim discards it).
FG_API void dgetri_(const int *N, double *A, const int *LDA, const int *IPIV, double *WORK,
                    const int *LWORK, int *INFO) {
    *INFO = 0;
    const bool query = *LWORK == -1;
    if (*N < 0) *INFO = -1;
    else if (*LDA < std::max(1, *N)) *INFO = -3;
    else if (*LWORK < std::max(1, *N) && !query) *INFO = -6;
    if (*INFO != 0) {
        report_xerbla("DGETRI", -*INFO);
        return;
    }
    const double opt = (double)std::max(1, *N * 64);
    if (query) {
        WORK[0] = opt;
        return;
    }
    int info = 0;
    const int st = getri_host(*N, A, *LDA, IPIV, &info);
    *INFO = (st != kOk) ? st : info;
    WORK[0] = opt;
}

// ------------------------------ refinement, condition, equilibration ----
namespace {

int dvec_in(int slot, const double *h, int n, cudaStream_t s, double **d, bool *staged) {
    if (is_device_ptr(h)) {
        *d = const_cast<double *>(h);
        *staged = false;
        return kOk;
    }
    void *p;
    int st = stage_buf(slot, (size_t)(n > 0 ? n : 1) * sizeof(double), &p);
    if (st != kOk) return st;
    *d = (double *)p;
    *staged = true;
    if (n > 0) FG_CUDA(cudaMemcpyAsync(*d, h, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, s));
    return kOk;
}

}  // namespace

// flens/lapack/interface/src/gerfs.cc:13-66 (checks 1, 2, 3, 5, 7, 10, 12)
FG_API void dgerfs_(const char *TRANS, const int *N, const int *NRHS, const double *A,
                    const int *LDA, const double *AF, const int *LDAF, const int *IPIV,
                    const double *B, const int *LDB, double *X, const int *LDX, double *FERR,
                    double *BERR, double *WORK, int *IWORK, int *INFO) {
    (void)WORK;
    (void)IWORK;
    *INFO = 0;
    if (*TRANS != 'N' && *TRANS != 'T' && *TRANS != 'C') *INFO = -1;
    else if (*N < 0) *INFO = -2;
    else if (*NRHS < 0) *INFO = -3;
    else if (*LDA < std::max(1, *N)) *INFO = -5;
    else if (*LDAF < std::max(1, *N)) *INFO = -7;
    else if (*LDB < std::max(1, *N)) *INFO = -10;
    else if (*LDX < std::max(1, *N)) *INFO = -12;
    if (*INFO != 0) {
        report_xerbla("DGERFS", -*INFO);
        return;
    }
    const int n = *N, nrhs = *NRHS;
    if (n == 0 || nrhs == 0) {
        for (int j = 0; j < nrhs; ++j) FERR[j] = BERR[j] = 0.0;
        return;
    }
    cudaStream_t s;
    int st = stage_stream(&s);
    DevView a, af, b, x;
    int *dpiv = nullptr;
    bool pst = false;
    if (st == kOk) st = view_in(0, A, n, n, *LDA, true, s, &a);
    if (st == kOk) st = view_in(1, AF, n, n, *LDAF, true, s, &af);
    if (st == kOk) st = view_in(2, B, n, nrhs, *LDB, true, s, &b);
    if (st == kOk) st = ipiv_dev(3, const_cast<int *>(IPIV), n, true, s, &dpiv, &pst);
    // X is staged through a buffer of its own (slots 0..3 hold A, AF, B, IPIV)
    double *dx = nullptr;
    if (st == kOk) {
        if (is_device_ptr(X)) {
            dx = X;
        } else {
            Workspace *w = workspace_for(s, 0);
            dx = w ? (double *)workspace_slot(s, 3, (size_t)n * nrhs * sizeof(double)) : nullptr;
            if (!dx) st = kErrAlloc;
            else if (cudaMemcpy2DAsync(dx, (size_t)n * sizeof(double), X, (size_t)*LDX * sizeof(double),
                                       (size_t)n * sizeof(double), nrhs, cudaMemcpyHostToDevice, s) != cudaSuccess)
                st = kErrCuda;
        }
    }
    const int ldx = is_device_ptr(X) ? *LDX : n;
    if (st == kOk)
        st = dgerfs_launch(*TRANS == 'C' ? 'T' : *TRANS, n, nrhs, a.p, a.ld, af.p, af.ld, dpiv, b.p, b.ld,
                           dx, ldx, FERR, BERR, s);
    if (st == kOk && dx != X &&
        cudaMemcpy2DAsync(X, (size_t)*LDX * sizeof(double), dx, (size_t)n * sizeof(double),
                          (size_t)n * sizeof(double), nrhs, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        st = kErrCuda;
    if (st == kOk) st = finish(s);
    if (st != kOk) *INFO = st;
}

// flens/lapack/interface/src/gecon.cc:13-51 (NORM '1', 'O' or 'I')
FG_API void dgecon_(const char *NORM, const int *N, const double *A, const int *LDA,
                    const double *ANORM, double *RCOND, double *WORK, int *IWORK, int *INFO) {
    (void)WORK;
    (void)IWORK;
    *INFO = 0;
    if (*NORM != '1' && *NORM != 'O' && *NORM != 'I') *INFO = -1;
    else if (*N < 0) *INFO = -2;
    else if (*LDA < std::max(1, *N)) *INFO = -4;
    else if (*ANORM < 0) *INFO = -5;
    if (*INFO != 0) {
        report_xerbla("DGECON", -*INFO);
        return;
    }
    cudaStream_t s;
    int st = stage_stream(&s);
    DevView a;
    if (st == kOk && *N > 0) st = view_in(0, A, *N, *N, *LDA, true, s, &a);
    if (st == kOk) st = dgecon_launch(*NORM, *N, a.p, a.ld, *ANORM, RCOND, s);
    if (st == kErrUnsupported) st = kOk;           // latrs would scale: RCOND = 0
    if (st == kOk) st = finish(s);
    if (st != kOk) *INFO = st;
}

// flens/lapack/interface/src/geequ.cc:10-40 (checks 1, 2, 4)
FG_API void dgeequ_(const int *M, const int *N, const double *A, const int *LDA, double *R,
                    double *C, double *ROWCND, double *COLCND, double *AMAX, int *INFO) {
    *INFO = 0;
    if (*M < 0) *INFO = -1;
    else if (*N < 0) *INFO = -2;
    else if (*LDA < std::max(1, *M)) *INFO = -4;
    if (*INFO != 0) {
        report_xerbla("DGEEQU", -*INFO);
        return;
    }
    const int m = *M, n = *N;
    cudaStream_t s;
    int st = stage_stream(&s);
    DevView a;
    double *dr = nullptr, *dc = nullptr;
    bool rs = false, cs = false;
    if (st == kOk && m > 0 && n > 0) st = view_in(0, A, m, n, *LDA, true, s, &a);
    if (st == kOk) st = dvec_in(1, R, m, s, &dr, &rs);
    if (st == kOk) st = dvec_in(2, C, n, s, &dc, &cs);
    int info = 0;
    if (st == kOk) st = dgeequ_launch(m, n, a.p, a.ld, dr, dc, ROWCND, COLCND, AMAX, &info, s);
    if (st == kOk && rs && m > 0) st = cudaMemcpyAsync(R, dr, (size_t)m * sizeof(double), cudaMemcpyDeviceToHost, s) == cudaSuccess ? kOk : kErrCuda;
    if (st == kOk && cs && n > 0) st = cudaMemcpyAsync(C, dc, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, s) == cudaSuccess ? kOk : kErrCuda;
    if (st == kOk) st = finish(s);
    *INFO = st != kOk ? st : info;
}

// flens/lapack/interface/src/laqge.cc:10-27 (no argument checks)
FG_API void dlaqge_(const int *M, const int *N, double *A, const int *LDA, const double *R,
                    const double *C, const double *ROWCND, const double *COLCND, const double *AMAX,
                    char *EQUED) {
    const int m = *M, n = *N;
    *EQUED = 'N';
    if (m <= 0 || n <= 0) return;
    cudaStream_t s;
    int st = stage_stream(&s);
    DevView a;
    double *dr = nullptr, *dc = nullptr;
    bool rs = false, cs = false;
    if (st == kOk) st = view_in(0, A, m, n, *LDA, true, s, &a);
    if (st == kOk) st = dvec_in(1, R, m, s, &dr, &rs);
    if (st == kOk) st = dvec_in(2, C, n, s, &dc, &cs);
    char eq = 'N';
    if (st == kOk) {
        eq = dlaqge_launch(m, n, a.p, a.ld, dr, dc, *ROWCND, *COLCND, *AMAX, s);
        if (eq == '?') st = kErrCuda;
    }
    if (st == kOk) st = view_out(a, A, m, n, *LDA, s);
    if (st == kOk) st = finish(s);
    report_blas_failure("dlaqge_", st);
    if (st == kOk) *EQUED = eq;
}

// flens/lapack/interface/src/gesvx.cc:13-118.  EQUED reports the scaling
// applied (the reference's svx takes it by value, so its shim returns 'N'
// after equilibrating); WORK(1) = reciprocal pivot growth.
FG_API void dgesvx_(const char *FACT, const char *TRANS, const int *N, const int *NRHS, double *A,
                    const int *LDA, double *AF, const int *LDAF, int *IPIV, char *EQUED, double *R,
                    double *C, double *B, const int *LDB, double *X, const int *LDX, double *RCOND,
                    double *FERR, double *BERR, double *WORK, int *IWORK, int *INFO) {
    (void)IWORK;
    const double bigNum = 1.0 / DBL_MIN;
    bool rowequ, colequ;
    if (*FACT == 'N' || *FACT == 'E') {
        *EQUED = 'N';
        rowequ = colequ = false;
    } else {
        rowequ = *EQUED == 'R' || *EQUED == 'B';
        colequ = *EQUED == 'C' || *EQUED == 'B';
    }
    *INFO = 0;
    if (*FACT != 'F' && *FACT != 'N' && *FACT != 'E') *INFO = -1;
    else if (*TRANS != 'N' && *TRANS != 'T' && *TRANS != 'C') *INFO = -2;
    else if (*N < 0) *INFO = -3;
    else if (*NRHS < 0) *INFO = -4;
    else if (*LDA < std::max(1, *N)) *INFO = -6;
    else if (*LDAF < std::max(1, *N)) *INFO = -8;
    else if (*FACT == 'F' && !(rowequ || colequ || *EQUED == 'N')) *INFO = -10;
    else {
        if (rowequ) {
            double lo = bigNum;
            for (int j = 0; j < *N; ++j) lo = std::min(lo, R[j]);
            if (lo <= 0.0) *INFO = -11;
        }
        if (colequ && *INFO == 0) {
            double lo = bigNum;
            for (int j = 0; j < *N; ++j) lo = std::min(lo, C[j]);
            if (lo <= 0.0) *INFO = -12;
        }
        if (*INFO == 0) {
            if (*LDB < std::max(1, *N)) *INFO = -14;
            else if (*LDX < std::max(1, *N)) *INFO = -16;
        }
    }
    if (*INFO != 0) {
        report_xerbla("DGESVX", -*INFO);
        return;
    }
    const int n = *N, nrhs = *NRHS;
    cudaStream_t s;
    int st = stage_stream(&s);
    // device copies: A, AF, B, X (n x n, n x n, n x nrhs, n x nrhs), IPIV, R, C
    const size_t nn = (size_t)(n > 0 ? n : 1), nr = (size_t)(nrhs > 0 ? nrhs : 1);
    const size_t bytes = sizeof(double) * (2 * nn * nn + 2 * nn * nr + 2 * nn) + sizeof(int) * nn + 256;
    char *buf = (char *)workspace_slot(s, 3, bytes);
    if (!buf) st = kErrAlloc;
    double *dA = (double *)buf, *dAF = dA + nn * nn, *dB = dAF + nn * nn, *dX = dB + nn * nr;
    double *dR = dX + nn * nr, *dC = dR + nn;
    int *dP = (int *)(dC + nn);
    auto up2 = [&](double *d, const double *h, int rows, int cols, int ld) {
        if (st != kOk || rows <= 0 || cols <= 0) return;
        if (cudaMemcpy2DAsync(d, (size_t)rows * sizeof(double), h, (size_t)ld * sizeof(double),
                              (size_t)rows * sizeof(double), cols, cudaMemcpyHostToDevice, s) != cudaSuccess)
            st = kErrCuda;
    };
    auto down2 = [&](double *h, const double *d, int rows, int cols, int ld) {
        if (st != kOk || rows <= 0 || cols <= 0) return;
        if (cudaMemcpy2DAsync(h, (size_t)ld * sizeof(double), d, (size_t)rows * sizeof(double),
                              (size_t)rows * sizeof(double), cols, cudaMemcpyDeviceToHost, s) != cudaSuccess)
            st = kErrCuda;
    };
    up2(dA, A, n, n, *LDA);
    up2(dB, B, n, nrhs, *LDB);
    if (*FACT == 'F') {
        up2(dAF, AF, n, n, *LDAF);
        if (st == kOk && n > 0 &&
            cudaMemcpyAsync(dP, IPIV, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, s) != cudaSuccess)
            st = kErrCuda;
    }
    up2(dR, R, n, 1, n);
    up2(dC, C, n, 1, n);
    int info = 0;
    double rpvgrw = 1.0;
    if (st == kOk)
        st = dgesvx_launch(*FACT, *TRANS == 'C' ? 'T' : *TRANS, n, nrhs, dA, std::max(1, n), dAF,
                           std::max(1, n), dP, EQUED, dR, dC, dB, std::max(1, n), dX, std::max(1, n),
                           RCOND, FERR, BERR, &rpvgrw, &info, s);
    down2(A, dA, n, n, *LDA);
    down2(AF, dAF, n, n, *LDAF);
    down2(B, dB, n, nrhs, *LDB);
    if (info == 0 || info == n + 1) down2(X, dX, n, nrhs, *LDX);
    down2(R, dR, n, 1, n);
    down2(C, dC, n, 1, n);
    if (st == kOk && n > 0 &&
        cudaMemcpyAsync(IPIV, dP, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess)
        st = kErrCuda;
    if (st == kOk) st = finish(s);
    WORK[0] = rpvgrw;
    *INFO = st != kOk ? st : info;
}

// ------------------------------------------------ device-pointer API ----
static inline cudaStream_t as_stream(void *s) { return (cudaStream_t)s; }

FG_API int flens_gb300_dsyrk(char uplo, char trans, int n, int k, double alpha, const double *A,
                             int ldA, double beta, double *C, int ldC, void *stream) {
    uplo = (char)toupper(uplo);
    trans = (char)toupper(trans);
    if (uplo != 'U' && uplo != 'L') return -1;
    if (trans != 'N' && trans != 'T' && trans != 'C') return -2;
    if (n < 0) return -3;
    if (k < 0) return -4;
    if (ldA < std::max(1, trans == 'N' ? n : k)) return -7;
    if (ldC < std::max(1, n)) return -10;
    return dsyrk_launch(uplo, trans == 'N' ? 'N' : 'T', n, k, alpha, A, ldA, beta, C, ldC,
                        as_stream(stream));
}

FG_API int flens_gb300_dtrmm(char side, char uplo, char transA, char diag, int m, int n,
                             double alpha, const double *A, int ldA, double *B, int ldB,
                             void *stream) {
    side = (char)toupper(side);
    uplo = (char)toupper(uplo);
    transA = (char)toupper(transA);
    diag = (char)toupper(diag);
    if (side != 'L' && side != 'R') return -1;
    if (uplo != 'U' && uplo != 'L') return -2;
    if (transA != 'N' && transA != 'T' && transA != 'C') return -3;
    if (diag != 'U' && diag != 'N') return -4;
    if (m < 0) return -5;
    if (n < 0) return -6;
    if (ldA < std::max(1, side == 'L' ? m : n)) return -9;
    if (ldB < std::max(1, m)) return -11;
    return dtrmm_launch(side, uplo, transA == 'C' ? 'T' : transA, diag, m, n, alpha, A, ldA, B,
                        ldB, as_stream(stream));
}

FG_API int flens_gb300_dsymm(char side, char uplo, int m, int n, double alpha, const double *A,
                             int ldA, const double *B, int ldB, double beta, double *C, int ldC,
                             void *stream) {
    side = (char)toupper(side);
    uplo = (char)toupper(uplo);
    if (side != 'L' && side != 'R') return -1;
    if (uplo != 'U' && uplo != 'L') return -2;
    if (m < 0) return -3;
    if (n < 0) return -4;
    if (ldA < std::max(1, side == 'L' ? m : n)) return -7;
    if (ldB < std::max(1, m)) return -9;
    if (ldC < std::max(1, m)) return -12;
    return dsymm_launch(side, uplo, m, n, alpha, A, ldA, B, ldB, beta, C, ldC, as_stream(stream));
}

FG_API int flens_gb300_dsyr2k(char uplo, char trans, int n, int k, double alpha, const double *A,
                              int ldA, const double *B, int ldB, double beta, double *C, int ldC,
                              void *stream) {
    uplo = (char)toupper(uplo);
    trans = (char)toupper(trans);
    if (uplo != 'U' && uplo != 'L') return -1;
    if (trans != 'N' && trans != 'T' && trans != 'C') return -2;
    if (n < 0) return -3;
    if (k < 0) return -4;
    if (ldA < std::max(1, trans == 'N' ? n : k)) return -7;
    if (ldB < std::max(1, trans == 'N' ? n : k)) return -9;
    if (ldC < std::max(1, n)) return -12;
    return dsyr2k_launch(uplo, trans == 'N' ? 'N' : 'T', n, k, alpha, A, ldA, B, ldB, beta, C, ldC,
                         as_stream(stream));
}

FG_API int flens_gb300_dtrtri(char uplo, char diag, int n, double *A, int ldA, int *info,
                              void *stream) {
    uplo = (char)toupper(uplo);
    diag = (char)toupper(diag);
    if (uplo != 'U' && uplo != 'L') return -1;
    if (diag != 'N' && diag != 'U') return -2;
    if (n < 0) return -3;
    if (ldA < std::max(1, n)) return -5;
    return dtrtri_launch(uplo, diag, n, A, ldA, info, as_stream(stream));
}

FG_API int flens_gb300_dgetri(int n, double *A, int ldA, const int *ipiv, int *info, void *stream) {
    if (n < 0) return -1;
    if (ldA < std::max(1, n)) return -3;
    return dgetri_launch(n, A, ldA, ipiv, info, as_stream(stream));
}

FG_API int flens_gb300_dgecon(char norm, int n, const double *LU, int ldLU, double anorm,
                              double *rcond, void *stream) {
    if (norm != '1' && norm != 'O' && norm != 'I' && norm != 'o' && norm != 'i') return -1;
    if (n < 0) return -2;
    if (ldLU < std::max(1, n)) return -4;
    if (anorm < 0) return -5;
    return dgecon_launch(norm, n, LU, ldLU, anorm, rcond, as_stream(stream));
}

FG_API int flens_gb300_dgerfs(char trans, int n, int nrhs, const double *A, int ldA, const double *AF,
                              int ldAF, const int *ipiv, const double *B, int ldB, double *X, int ldX,
                              double *ferr, double *berr, void *stream) {
    trans = (char)toupper(trans);
    if (trans != 'N' && trans != 'T' && trans != 'C') return -1;
    if (n < 0) return -2;
    if (nrhs < 0) return -3;
    if (ldA < std::max(1, n)) return -5;
    if (ldAF < std::max(1, n)) return -7;
    if (ldB < std::max(1, n)) return -10;
    if (ldX < std::max(1, n)) return -12;
    return dgerfs_launch(trans == 'C' ? 'T' : trans, n, nrhs, A, ldA, AF, ldAF, ipiv, B, ldB, X, ldX,
                         ferr, berr, as_stream(stream));
}

FG_API int flens_gb300_dgeequ(int m, int n, const double *A, int ldA, double *r, double *c,
                              double *rowcnd, double *colcnd, double *amax, int *info, void *stream) {
    if (m < 0) return -1;
    if (n < 0) return -2;
    if (ldA < std::max(1, m)) return -4;
    return dgeequ_launch(m, n, A, ldA, r, c, rowcnd, colcnd, amax, info, as_stream(stream));
}

FG_API int flens_gb300_dlaqge(int m, int n, double *A, int ldA, const double *r, const double *c,
                              double rowcnd, double colcnd, double amax, char *equed, void *stream) {
    if (m < 0) return -1;
    if (n < 0) return -2;
    if (ldA < std::max(1, m)) return -4;
    const char eq = dlaqge_launch(m, n, A, ldA, r, c, rowcnd, colcnd, amax, as_stream(stream));
    if (eq == '?') return kErrCuda;
    *equed = eq;
    return kOk;
}

FG_API int flens_gb300_dgesvx(char fact, char trans, int n, int nrhs, double *A, int ldA, double *AF,
                              int ldAF, int *ipiv, char *equed, double *r, double *c, double *B,
                              int ldB, double *X, int ldX, double *rcond, double *ferr, double *berr,
                              double *rpvgrw, int *info, void *stream) {
    fact = (char)toupper(fact);
    trans = (char)toupper(trans);
    if (fact != 'F' && fact != 'N' && fact != 'E') return -1;
    if (trans != 'N' && trans != 'T' && trans != 'C') return -2;
    if (n < 0) return -3;
    if (nrhs < 0) return -4;
    if (ldA < std::max(1, n)) return -6;
    if (ldAF < std::max(1, n)) return -8;
    if (fact == 'F' && *equed != 'N' && *equed != 'R' && *equed != 'C' && *equed != 'B') return -10;
    if (ldB < std::max(1, n)) return -14;
    if (ldX < std::max(1, n)) return -16;
    return dgesvx_launch(fact, trans == 'C' ? 'T' : trans, n, nrhs, A, ldA, AF, ldAF, ipiv, equed, r, c,
                         B, ldB, X, ldX, rcond, ferr, berr, rpvgrw, info, as_stream(stream));
}

FG_API int flens_gb300_dpotrf(char uplo, int n, double *A, int ldA, int *info, void *stream) {
    uplo = (char)toupper(uplo);
    if (uplo != 'U' && uplo != 'L') return -1;
    if (n < 0) return -2;
    if (ldA < std::max(1, n)) return -4;
    return dpotrf_launch(uplo, n, A, ldA, info, as_stream(stream));
}

FG_API int flens_gb300_dpotrs(char uplo, int n, int nrhs, const double *A, int ldA, double *B,
                              int ldB, void *stream) {
    uplo = (char)toupper(uplo);
    if (uplo != 'U' && uplo != 'L') return -1;
    if (n < 0) return -2;
    if (nrhs < 0) return -3;
    if (ldA < std::max(1, n)) return -5;
    if (ldB < std::max(1, n)) return -7;
    return dpotrs_launch(uplo, n, nrhs, A, ldA, B, ldB, as_stream(stream));
}

FG_API int flens_gb300_dposv(char uplo, int n, int nrhs, double *A, int ldA, double *B, int ldB,
                             int *info, void *stream) {
    uplo = (char)toupper(uplo);
    if (uplo != 'U' && uplo != 'L') return -1;
    if (n < 0) return -2;
    if (nrhs < 0) return -3;
    if (ldA < std::max(1, n)) return -5;
    if (ldB < std::max(1, n)) return -7;
    cudaStream_t s = as_stream(stream);
    int st = dpotrf_launch(uplo, n, A, ldA, info, s);
    if (st != kOk) return st;
    int h = 0;
    FG_CUDA(cudaMemcpyAsync(&h, info, sizeof(int), cudaMemcpyDeviceToHost, s));
    FG_CUDA(cudaStreamSynchronize(s));
    if (h != 0) return kOk;    // INFO>0 reported through *info; no solve (posv.tcc:58-64)
    return dpotrs_launch(uplo, n, nrhs, A, ldA, B, ldB, s);
}

FG_API int flens_gb300_dgemm(char transA, char transB, int m, int n, int k, double alpha,
                             const double *A, int ldA, const double *B, int ldB, double beta,
                             double *C, int ldC, void *stream) {
    const char ta = (char)toupper(transA), tb = (char)toupper(transB);
    if (ta != 'N' && ta != 'T' && ta != 'C') return -1;
    if (tb != 'N' && tb != 'T' && tb != 'C') return -2;
    if (m < 0) return -3;
    if (n < 0) return -4;
    if (k < 0) return -5;
    if (ldA < std::max(1, ta == 'N' ? m : k)) return -8;
    if (ldB < std::max(1, tb == 'N' ? k : n)) return -10;
    if (ldC < std::max(1, m)) return -13;
    return dgemm_launch(ta == 'C' ? 'T' : ta, tb == 'C' ? 'T' : tb, m, n, k, alpha, A, ldA, B,
                        ldB, beta, C, ldC, as_stream(stream));
}

FG_API int flens_gb300_dtrsm(char side, char uplo, char transA, char diag, int m, int n,
                             double alpha, const double *A, int ldA, double *B, int ldB,
                             void *stream) {
    side = (char)toupper(side);
    uplo = (char)toupper(uplo);
    transA = (char)toupper(transA);
    diag = (char)toupper(diag);
    if (side != 'L' && side != 'R') return -1;
    if (uplo != 'U' && uplo != 'L') return -2;
    if (transA != 'N' && transA != 'T' && transA != 'C') return -3;
    if (diag != 'U' && diag != 'N') return -4;
    if (m < 0) return -5;
    if (n < 0) return -6;
    if (ldA < std::max(1, side == 'L' ? m : n)) return -9;
    if (ldB < std::max(1, m)) return -11;
    return dtrsm_launch(side, uplo, transA == 'C' ? 'T' : transA, diag, m, n, alpha, A, ldA, B, ldB,
                        as_stream(stream));
}

FG_API int flens_gb300_dgetrf(int m, int n, double *A, int ldA, int *ipiv, int *info, void *stream) {
    if (m < 0) return -1;
    if (n < 0) return -2;
    if (ldA < std::max(1, m)) return -4;
    return dgetrf_launch(m, n, A, ldA, ipiv, info, as_stream(stream));
}

// FP64-accurate LU with the trailing updates beyond each outer block on the
// tensor cores (split GEMM).  Argument positions as flens_gb300_dgetrf, outer_nb 7.
FG_API int flens_gb300_dgetrf_split(int m, int n, double *A, int ldA, int *ipiv, int *info,
                                    int outer_nb, void *stream) {
    if (m < 0) return -1;
    if (n < 0) return -2;
    if (ldA < std::max(1, m)) return -4;
    if (outer_nb < 0 || outer_nb % 64 != 0) return -7;
    return dgetrf_split_launch(m, n, A, ldA, ipiv, info, outer_nb, as_stream(stream));
}

// LU of an FP32 matrix with tensor-core (or, precision -1, CUDA-core)
// trailing updates: the factorisation of flens_gb300_dgesv_mixed.
FG_API int flens_gb300_sgetrf_tc(int precision, int m, int n, float *A, int ldA, int *ipiv, int *info,
                                 void *stream) {
    if (precision < -1 || precision > 6 || precision == 4) return -1;
    if (m < 0) return -2;
    if (n < 0) return -3;
    if (ldA < std::max(1, m)) return -5;
    return sgetrf_launch(m, n, A, ldA, ipiv, info, precision, as_stream(stream));
}

// Test hook: the mixed solve's chunked GEMVs on their own: y = A x over one
// triangle of A, the other triangle holding zeros (uplo 'L' or 'U', the
// explicit-inverse preconditioner), or over all of A (uplo 'G', the Arnoldi
// product).  With part == NULL it only reports the scratch sizes.
FG_API int flens_gb300_test_trmv_zeros(char uplo, int n, const double *A, int ldA, const double *x,
                                       double *y, double *part, unsigned *cnt, size_t *part_elems,
                                       size_t *cnt_elems, void *stream) {
    uplo = (char)toupper(uplo);
    if (uplo != 'L' && uplo != 'U' && uplo != 'G') return -1;
    if (n < 0) return -2;
    if (ldA < std::max(1, n)) return -4;
    if (part_elems) *part_elems = dtrmv_zeros_part_elems(n);
    if (cnt_elems) *cnt_elems = dtrmv_zeros_cnt_elems(n);
    if (!part) return kOk;
    if (num_sms() <= 0) {
        set_last_error("no CUDA device");
        return kErrNoDevice;
    }
    if (uplo == 'G') return dgemv_chunk_launch(n, A, ldA, x, y, part, cnt, as_stream(stream));
    return dtrmv_zeros_launch(uplo, n, A, ldA, x, y, part, cnt, as_stream(stream));
}

FG_API int flens_gb300_dgetrs(char trans, int n, int nrhs, const double *A, int ldA,
                              const int *ipiv, double *B, int ldB, void *stream) {
    trans = (char)toupper(trans);
    if (trans != 'N' && trans != 'T' && trans != 'C') return -1;
    if (n < 0) return -2;
    if (nrhs < 0) return -3;
    if (ldA < std::max(1, n)) return -5;
    if (ldB < std::max(1, n)) return -8;
    return dgetrs_launch(trans == 'C' ? 'T' : trans, n, nrhs, A, ldA, ipiv, B, ldB, as_stream(stream));
}

FG_API int flens_gb300_dgesv(int n, int nrhs, double *A, int ldA, int *ipiv, double *B, int ldB,
                             int *info, void *stream) {
    if (n < 0) return -1;
    if (nrhs < 0) return -2;
    if (ldA < std::max(1, n)) return -4;
    if (ldB < std::max(1, n)) return -7;
    cudaStream_t s = as_stream(stream);
    int st = dgetrf_launch(n, n, A, ldA, ipiv, info, s);
    if (st != kOk) return st;
    int h = 0;
    FG_CUDA(cudaMemcpyAsync(&h, info, sizeof(int), cudaMemcpyDeviceToHost, s));
    FG_CUDA(cudaStreamSynchronize(s));
    if (h != 0) return kOk;    // INFO>0 reported through *info; no solve (sv.tcc:70-75)
    return dgetrs_launch('N', n, nrhs, A, ldA, ipiv, B, ldB, s);
}

FG_API int flens_gb300_sync(void *stream) {
    cudaStream_t s = as_stream(stream);
    FG_CUDA(cudaStreamSynchronize(s));
    return check_device_status(s);
}

FG_API int flens_gb300_version(void) { return 100; }

// Where failures of the BLAS routines (which have no INFO) are reported:
// hook(routine, status, message) on the calling thread instead of stderr;
// nullptr restores the stderr report.
FG_API void flens_gb300_set_blas_error_hook(void (*hook)(const char *routine, int status,
                                                         const char *message)) {
    __atomic_store_n(&g_blas_hook, hook, __ATOMIC_RELEASE);
}

// Status of the calling thread's last BLAS call (dgemm_, dtrsm_, dsyrk_,
// dtrmm_, dsymm_, dsyr2k_, dlaqge_): 0, or a FLENS_GB300_ERR_* code.
FG_API int flens_gb300_blas_status(void) { return g_blas_status; }
