// runtime.cu -- error state, per-stream device workspace, device queries,
// tracing.  The reference is stateless (every call allocates nothing the
// caller sees); this library keeps a small cache of device scratch per
// (device, stream) so repeated calls do not pay cudaMalloc, and frees it when
// the library is unloaded.
#include "common.cuh"

#include <atomic>
#include <mutex>
#include <vector>
#include <map>
#include <utility>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

namespace fg {

static thread_local char t_last_error[512] = "";

void set_last_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_last_error, sizeof t_last_error, fmt, ap);
    va_end(ap);
    if (trace_enabled()) fprintf(stderr, "[flens_gb300] error: %s\n", t_last_error);
}

int cuda_fail(cudaError_t e, const char *what) {
    set_last_error("%s failed: %s (%d)", what, cudaGetErrorString(e), (int)e);
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return kErrNoDevice;
    if (e == cudaErrorMemoryAllocation) return kErrAlloc;
    return kErrCuda;
}

namespace {
std::atomic<long long> g_dev_allocs{0};
std::atomic<int> g_fail_allocs{0};
}  // namespace

cudaError_t device_malloc(void **p, size_t bytes) {
    int k = g_fail_allocs.load();
    while (k > 0) {
        if (g_fail_allocs.compare_exchange_weak(k, k - 1)) {
            *p = nullptr;
            return cudaErrorMemoryAllocation;
        }
    }
    const cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) g_dev_allocs.fetch_add(1);
    return e;
}

bool trace_enabled() {
    static int flag = -1;
    if (flag < 0) {
        const char *s = getenv("FLENS_GB300_TRACE");
        flag = (s && *s && *s != '0') ? 1 : 0;
    }
    return flag == 1;
}

void trace(const char *fmt, ...) {
    if (!trace_enabled()) return;
    va_list ap;
    va_start(ap, fmt);
    fprintf(stderr, "[flens_gb300] ");
    vfprintf(stderr, fmt, ap);
    fprintf(stderr, "\n");
    va_end(ap);
}

int device_id() {
    int d = 0;
    if (cudaGetDevice(&d) != cudaSuccess) return -1;
    return d;
}

int num_sms() {
    static int cached[64];
    const int d = device_id();
    if (d < 0 || d >= 64) return 0;
    if (cached[d] == 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, d) != cudaSuccess) return 0;
        cached[d] = v;
    }
    return cached[d];
}

// ------------------------------------------------------------ workspace --
namespace {
struct Registry {
    std::mutex mu;
    std::map<std::pair<int, cudaStream_t>, Workspace *> map;
    ~Registry() {
        // Library unload: free what is still allocated.  Errors are ignored
        // (the CUDA runtime may already be shutting down).
        for (auto &kv : map) {
            Workspace *w = kv.second;
            if (w->buf) cudaFree(w->buf);
            for (int i = 0; i < 4; ++i)
                if (w->slot_buf[i]) cudaFree(w->slot_buf[i]);
            if (w->status) cudaFree(w->status);
            if (w->ev_fwd) cudaEventDestroy(w->ev_fwd);
            if (w->ev_back) cudaEventDestroy(w->ev_back);
            if (w->side) cudaStreamDestroy(w->side);
            if (w->flags) cudaFree(w->flags);
            delete w;
        }
        map.clear();
    }
};
Registry &registry() {
    static Registry r;
    return r;
}
}  // namespace

Workspace *workspace_for(cudaStream_t stream, size_t bytes) {
    const int dev = device_id();
    if (dev < 0) {
        set_last_error("no CUDA device");
        return nullptr;
    }
    Registry &r = registry();
    std::lock_guard<std::mutex> lock(r.mu);
    Workspace *&w = r.map[std::make_pair(dev, stream)];
    if (!w) {
        w = new Workspace();
        w->device = dev;
        w->stream = stream;
        // status word + info word, zeroed
        if (device_malloc((void **)&w->status, 2 * sizeof(int)) != cudaSuccess) {
            set_last_error("cudaMalloc of the status word failed");
            delete w;
            w = nullptr;
            return nullptr;
        }
        w->info = w->status + 1;
        if (cudaMemsetAsync(w->status, 0, 2 * sizeof(int), stream) != cudaSuccess) {
            set_last_error("cudaMemsetAsync of the status word failed");
            return nullptr;
        }
    }
    if (w->bytes < bytes) {
        // The old buffer may still be in use by work queued on this stream:
        // free it stream-ordered before growing.
        if (w->buf) {
            cudaStreamSynchronize(stream);
            cudaFree(w->buf);
            w->buf = nullptr;
            w->bytes = 0;
        }
        size_t want = bytes < (1u << 20) ? (1u << 20) : bytes;
        if (device_malloc(&w->buf, want) != cudaSuccess) {
            set_last_error("cudaMalloc of %zu bytes of workspace failed", want);
            return nullptr;
        }
        w->bytes = want;
    }
    return w;
}

Workspace *workspace_side(cudaStream_t stream) {
    Workspace *w = workspace_for(stream, 0);
    if (!w) return nullptr;
    Registry &r = registry();
    std::lock_guard<std::mutex> lock(r.mu);
    if (!w->side) {
        int least = 0, greatest = 0;
        if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess ||
            cudaStreamCreateWithPriority(&w->side, cudaStreamNonBlocking, greatest) != cudaSuccess ||
            cudaEventCreateWithFlags(&w->ev_fwd, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&w->ev_back, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            set_last_error("creating the look-ahead stream failed");
            return nullptr;
        }
    }
    return w;
}

int workspace_flags(cudaStream_t stream, int n, unsigned long long **flags,
                    unsigned long long *epoch) {
    constexpr int kCap = 4096;
    if (n > kCap) return kErrUnsupported;
    Workspace *w = workspace_for(stream, 0);
    if (!w) return kErrAlloc;
    Registry &r = registry();
    std::lock_guard<std::mutex> lock(r.mu);
    if (!w->flags) {
        if (device_malloc((void **)&w->flags, kCap * sizeof(unsigned long long)) != cudaSuccess) {
            cudaGetLastError();
            w->flags = nullptr;
            set_last_error("cudaMalloc of the solve flags failed");
            return kErrAlloc;
        }
        // epoch 0 is never published, so zeroed flags read as "not ready"
        if (cudaMemsetAsync(w->flags, 0, kCap * sizeof(unsigned long long), stream) != cudaSuccess) {
            cudaGetLastError();
            set_last_error("cudaMemsetAsync of the solve flags failed");
            return kErrCuda;
        }
        w->flags_cap = kCap;
    }
    *flags = w->flags;
    *epoch = ++w->flag_epoch;
    return kOk;
}

void *workspace_slot(cudaStream_t stream, int slot, size_t bytes) {
    if (slot < 1 || slot > 3) {
        set_last_error("workspace slot %d out of range", slot);
        return nullptr;
    }
    Workspace *w = workspace_for(stream, 0);
    if (!w) return nullptr;
    Registry &r = registry();
    std::lock_guard<std::mutex> lock(r.mu);
    if (w->slot_bytes[slot] < bytes) {
        if (w->slot_buf[slot]) {
            cudaStreamSynchronize(stream);
            cudaFree(w->slot_buf[slot]);
            w->slot_buf[slot] = nullptr;
            w->slot_bytes[slot] = 0;
        }
        const size_t want = bytes < 256 ? 256 : bytes;
        if (device_malloc(&w->slot_buf[slot], want) != cudaSuccess) {
            cudaGetLastError();
            set_last_error("cudaMalloc of %zu bytes (workspace slot %d) failed", want, slot);
            return nullptr;
        }
        w->slot_bytes[slot] = want;
    }
    return w->slot_buf[slot];
}

int set_smem_once(DeviceOnce &once, const void *fn, int bytes) {
    if (!once.pending()) return kOk;
    FG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    once.done();
    return kOk;
}

int check_device_status(cudaStream_t stream) {
    Workspace *w = workspace_for(stream, 0);
    if (!w) return kErrAlloc;
    int h = 0;
    FG_CUDA(cudaMemcpyAsync(&h, w->status, sizeof(int), cudaMemcpyDeviceToHost, stream));
    FG_CUDA(cudaStreamSynchronize(stream));
    if (h != kDevOk) {
        cudaMemsetAsync(w->status, 0, sizeof(int), stream);
        cudaStreamSynchronize(stream);
        set_last_error("device-side wait timed out (status bits 0x%x)", h);
        return kErrTimeout;
    }
    return kOk;
}

// ------------------------------------------------- launch accounting --
namespace {
struct TimingRec {
    int family;
    cudaEvent_t e0, e1;
    double flops, bytes;
};
std::atomic<long long> g_launches{0};
std::atomic<bool> g_timing{false};
std::mutex g_tmu;
std::vector<TimingRec> g_pending;
double g_ms[kFamCount], g_flops[kFamCount], g_bytes[kFamCount];
long long g_count[kFamCount];

void drain_pending_locked() {
    for (auto &r : g_pending) {
        float ms = 0.f;
        if (cudaEventSynchronize(r.e1) == cudaSuccess && cudaEventElapsedTime(&ms, r.e0, r.e1) == cudaSuccess) {
            g_ms[r.family] += ms;
            g_flops[r.family] += r.flops;
            g_bytes[r.family] += r.bytes;
            g_count[r.family] += 1;
        }
        cudaEventDestroy(r.e0);
        cudaEventDestroy(r.e1);
    }
    g_pending.clear();
}
}  // namespace

KTimer::KTimer(int fam, cudaStream_t s, double fl, double by)
    : family(fam), stream(s), flops(fl), bytes(by), e0(nullptr), on(false) {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if (g_timing.load(std::memory_order_relaxed)) {
        if (cudaEventCreate(&e0) == cudaSuccess && cudaEventRecord(e0, stream) == cudaSuccess) on = true;
    }
}

KTimer::~KTimer() {
    if (!on) return;
    cudaEvent_t e1;
    if (cudaEventCreate(&e1) != cudaSuccess) return;
    cudaEventRecord(e1, stream);
    std::lock_guard<std::mutex> lock(g_tmu);
    g_pending.push_back(TimingRec{family, e0, e1, flops, bytes});
    if (g_pending.size() > 4096) drain_pending_locked();
}

}  // namespace fg

FG_API const char *flens_gb300_last_error(void) { return fg::t_last_error; }

// Device allocations (cudaMalloc) the library has made since load.
FG_API long long flens_gb300_device_alloc_count(void) { return fg::g_dev_allocs.load(); }

// Test hook: the next `count` device allocations of the library fail as an
// out-of-memory cudaMalloc would (count <= 0 clears the hook).
FG_API void flens_gb300_test_fail_device_allocs(int count) {
    fg::g_fail_allocs.store(count > 0 ? count : 0);
}

// Number of kernel launches the library has issued since load.
FG_API long long flens_gb300_launch_count(void) { return fg::g_launches.load(); }

// Enable (1) or disable (0) per-launch event timing; enabling clears totals.
FG_API void flens_gb300_timing_enable(int on) {
    std::lock_guard<std::mutex> lock(fg::g_tmu);
    fg::drain_pending_locked();
    for (int f = 0; f < fg::kFamCount; ++f) {
        fg::g_ms[f] = fg::g_flops[f] = fg::g_bytes[f] = 0.0;
        fg::g_count[f] = 0;
    }
    fg::g_timing.store(on != 0);
}

// Totals for one kernel family since timing was enabled (waits for the
// recorded events).  Returns 0, or -1 for an unknown family.
FG_API int flens_gb300_timing_read(int family, double *ms, long long *launches, double *flops,
                                   double *bytes) {
    if (family < 0 || family >= fg::kFamCount) return -1;
    std::lock_guard<std::mutex> lock(fg::g_tmu);
    fg::drain_pending_locked();
    if (ms) *ms = fg::g_ms[family];
    if (launches) *launches = fg::g_count[family];
    if (flops) *flops = fg::g_flops[family];
    if (bytes) *bytes = fg::g_bytes[family];
    return 0;
}

FG_API const char *flens_gb300_family_name(int family) {
    static const char *names[fg::kFamCount] = {"dgemm_fp64", "lu_panel", "laswp", "trsm_diag",
                                               "aux", "tc_gemm", "refine", "batched_lu",
                                               "split_gemm", "trsv_chain", "krylov",
                                               "precond_chain"};
    return (family >= 0 && family < fg::kFamCount) ? names[family] : "";
}
