// refine.cu -- componentwise iterative refinement with error bounds (gerfs),
// condition estimate (gecon), equilibration (geequ / laqge) and the expert
// driver (gesvx), FP64, on the GPU.
//
// Follows FLENS-LAPACK:
//   gerfs  flens/lapack/ge/rfs.tcc: per right-hand side, r = b - op(A) x,
//          w = |b| + |op(A)||x|, berr = max_i |r_i| / w_i (safe1 added where
//          w_i <= safe2); while berr > eps, 2 berr <= the previous one and at
//          most 5 steps: solve op(AF) dx = r, x += dx; then the forward error
//          bound: lacn2 on diag(|r| + (n+1) eps w) op(A)^-1, over max |x_i|;
//   gecon  flens/lapack/ge/cond.tcc: lacn2 with triangular solves by L and U
//          through latrs (flens/lapack/la/latrs.tcc), rcond =
//          (1/estimate)/anorm;
//   geequ  flens/lapack/ge/equ.tcc, laqge flens/lapack/la/laq.tcc;
//   gesvx  flens/lapack/ge/svx.tcc.
// The O(n^2) work (residuals, |A||x|, the solves with the LU factors, the
// scalings) runs in CUDA kernels and the library's GEMM / TRSM / LU; the
// estimator's state machine (lacn2, flens/lapack/la/lacn2.tcc) keeps its few
// scalars on the host and reads each reduction it branches on back from the
// device.  latrs is used on its unscaled path only (its growth bound decides,
// as in the reference); where the reference would switch to its overflow-
// scaled solve, gecon reports rcond = 0 and returns FLENS_GB300_ERR_UNSUPPORTED
// from the device entry point (the Fortran one sets RCOND = 0).  Sums are
// parallel, so results agree with the reference to rounding.
#include "common.cuh"

#include <cfloat>
#include <climits>
#include <cmath>
#include <vector>

namespace fg {

namespace {

constexpr double kEps = DBL_EPSILON * 0.5;         // flens/lapack/la/lamch.tcc: Eps
constexpr double kSafeMin = DBL_MIN;               //                            SafeMin
constexpr double kPrecision = DBL_EPSILON;         //                            Precision
constexpr int RT = 1024;                           // threads of the one-CTA reductions

__device__ __forceinline__ double f_sign1(double y) {  // sign(1, y), sign bit of y
    return (y > 0.0) ? 1.0 : (y < 0.0) ? -1.0 : (signbit(y) ? -1.0 : 1.0);
}

template <int OP>
__device__ double block_reduce(double v) {          // OP 0: sum, 1: max
    __shared__ double sh[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const double o = __shfl_xor_sync(0xffffffffu, v, off);
        v = OP == 0 ? v + o : fmax(v, o);
    }
    if (lane == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        v = lane < (int)(blockDim.x >> 5) ? sh[lane] : (OP == 0 ? 0.0 : -DBL_MAX);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const double o = __shfl_xor_sync(0xffffffffu, v, off);
            v = OP == 0 ? v + o : fmax(v, o);
        }
    }
    return v;                                        // valid in thread 0
}

// out[0] = sum |x_i|, out[1] = max |x_i|, out[2] = first i with |x_i| = max
// (as a double), out[3] = min x_i, out[4] = first i with x_i == 0 (or -1).
__global__ void __launch_bounds__(RT) stats_kernel(int n, const double *__restrict__ x, int inc,
                                                   double *out) {
    __shared__ double s_max;
    __shared__ int s_idx, s_zero;
    double s = 0.0, m = 0.0, mn = 1.0e308;
    for (int i = threadIdx.x; i < n; i += RT) {
        const double a = fabs(x[(size_t)i * inc]);
        s += a;
        m = fmax(m, a);
        mn = fmin(mn, x[(size_t)i * inc]);
    }
    s = block_reduce<0>(s);
    if (threadIdx.x == 0) out[0] = s;
    __syncthreads();
    m = block_reduce<1>(m);
    if (threadIdx.x == 0) {
        s_max = m;
        s_idx = INT_MAX;
        s_zero = INT_MAX;
    }
    __syncthreads();
    mn = -block_reduce<1>(-mn);
    for (int i = threadIdx.x; i < n; i += RT) {
        const double xi = x[(size_t)i * inc];
        if (fabs(xi) == s_max) atomicMin(&s_idx, i);
        if (xi == 0.0) atomicMin(&s_zero, i);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        out[1] = s_max;
        out[2] = s_idx == INT_MAX ? 0.0 : (double)s_idx;
        out[3] = mn;
        out[4] = s_zero == INT_MAX ? -1.0 : (double)s_zero;
    }
}

// x_i = sign(1, x_i), sgn_i = nint(x_i)
__global__ void sign_kernel(int n, double *__restrict__ x, int *__restrict__ sgn) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double s = f_sign1(x[i]);
        x[i] = s;
        sgn[i] = (int)floor(s + 0.5);
    }
}

// *flag = 1 if nint(sign(1, x_i)) != sgn_i for some i
__global__ void sign_changed_kernel(int n, const double *__restrict__ x, const int *__restrict__ sgn,
                                    int *flag) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (floor(f_sign1(x[i]) + 0.5) != (double)sgn[i]) atomicOr(flag, 1);
}

__global__ void fill_kernel(int n, double *__restrict__ x, double v) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] = v;
}

__global__ void unit_kernel(int n, double *__restrict__ x, int j) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        x[i] = i == j ? 1.0 : 0.0;
}

// x_i = (-1)^i (1 + i/(n-1))
__global__ void altsgn_kernel(int n, double *__restrict__ x) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        x[i] = ((i & 1) ? -1.0 : 1.0) * (1.0 + (double)i / (double)(n - 1));
}

__global__ void mul_kernel(int n, double *__restrict__ x, const double *__restrict__ w) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] *= w[i];
}

__global__ void axpy1_kernel(int n, double *__restrict__ x, const double *__restrict__ d) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] += d[i];
}

// w = |b| + |op(A)||x|: NoTrans a thread per row (coalesced along the rows of
// each column), Trans a warp per column.
__global__ void __launch_bounds__(256)
abs_gemv_n_kernel(int n, const double *__restrict__ A, int ldA, const double *__restrict__ x,
                  const double *__restrict__ b, double *__restrict__ w) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = fabs(b[i]);
    for (int k = 0; k < n; ++k) s += fabs(A[(size_t)i + (size_t)k * ldA]) * fabs(x[k]);
    w[i] = s;
}

__global__ void __launch_bounds__(256)
abs_gemv_t_kernel(int n, const double *__restrict__ A, int ldA, const double *__restrict__ x,
                  const double *__restrict__ b, double *__restrict__ w) {
    const int k = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (k >= n) return;
    double s = 0.0;
    for (int i = lane; i < n; i += 32) s += fabs(A[(size_t)i + (size_t)k * ldA]) * fabs(x[i]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (lane == 0) w[k] = fabs(b[k]) + s;
}

// out[0] = max_i (|r_i| / w_i, or (|r_i| + safe1) / (w_i + safe1) if w_i <= safe2)
__global__ void __launch_bounds__(RT)
berr_kernel(int n, const double *__restrict__ w, const double *__restrict__ r, double safe1,
            double safe2, double *out) {
    double m = 0.0;
    for (int i = threadIdx.x; i < n; i += RT)
        m = fmax(m, w[i] > safe2 ? fabs(r[i]) / w[i] : (fabs(r[i]) + safe1) / (w[i] + safe1));
    m = block_reduce<1>(m);
    if (threadIdx.x == 0) out[0] = m;
}

// w_i = |r_i| + nzeps w_i (+ safe1 where w_i <= safe2)
__global__ void ferr_weights_kernel(int n, double *__restrict__ w, const double *__restrict__ r,
                                    double nzeps, double safe1, double safe2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        w[i] = w[i] > safe2 ? fabs(r[i]) + nzeps * w[i] : fabs(r[i]) + nzeps * w[i] + safe1;
}

// column sums of |A| strictly below (lower) or above (upper) the diagonal
__global__ void __launch_bounds__(256)
cnorm_kernel(int n, const double *__restrict__ A, int ldA, int upper, double *__restrict__ cn) {
    const int j = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (j >= n) return;
    const int i0 = upper ? 0 : j + 1, i1 = upper ? j : n;
    double s = 0.0;
    for (int i = i0 + lane; i < i1; i += 32) s += fabs(A[(size_t)i + (size_t)j * ldA]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (lane == 0) cn[j] = s;
}

__global__ void diag_kernel(int n, const double *__restrict__ A, int ldA, double *__restrict__ d) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        d[i] = A[(size_t)i * (ldA + 1)];
}

// geequ pieces: r_i = max_j |a_ij|; c_j = max_i |a_ij| r_i; v_i = 1/clamp(v_i)
__global__ void __launch_bounds__(256)
row_absmax_kernel(int m, int n, const double *__restrict__ A, int ldA, double *__restrict__ r) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    double v = 0.0;
    for (int j = 0; j < n; ++j) v = fmax(v, fabs(A[(size_t)i + (size_t)j * ldA]));
    r[i] = v;
}

__global__ void __launch_bounds__(256)
col_scaled_absmax_kernel(int m, int n, const double *__restrict__ A, int ldA,
                         const double *__restrict__ r, double *__restrict__ c) {
    const int j = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (j >= n) return;
    double v = 0.0;
    for (int i = lane; i < m; i += 32) v = fmax(v, fabs(A[(size_t)i + (size_t)j * ldA]) * r[i]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, off));
    if (lane == 0) c[j] = v;
}

__global__ void recip_clamp_kernel(int n, double *__restrict__ v, double lo, double hi) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        v[i] = 1.0 / fmin(fmax(v[i], lo), hi);
}

// A(i,j) *= mode 1: c_j; 2: r_i; 3: c_j * r_i (that product first)
__global__ void __launch_bounds__(256)
scale_matrix_kernel(int m, int n, double *__restrict__ A, int ldA, const double *__restrict__ r,
                    const double *__restrict__ c, int mode) {
    const size_t total = (size_t)m * n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % m), j = (int)(e / m);
        double &a = A[(size_t)i + (size_t)j * ldA];
        if (mode == 1) a *= c[j];
        else if (mode == 2) a *= r[i];
        else a *= c[j] * r[i];
    }
}

// max |a_ij| over the upper triangle of the leading k x k block (lan on a
// TrMatrix) and over the whole m x n matrix: out[0], out[1]
__global__ void __launch_bounds__(RT)
maxnorms_kernel(int k, const double *__restrict__ AF, int ldAF, int m, int n,
                const double *__restrict__ A, int ldA, double *out) {
    double u = 0.0, a = 0.0;
    for (size_t e = threadIdx.x; e < (size_t)k * k; e += RT) {
        const int i = (int)(e % k), j = (int)(e / k);
        if (i <= j) u = fmax(u, fabs(AF[(size_t)i + (size_t)j * ldAF]));
    }
    for (size_t e = threadIdx.x; e < (size_t)m * n; e += RT) {
        const int i = (int)(e % m), j = (int)(e / m);
        a = fmax(a, fabs(A[(size_t)i + (size_t)j * ldA]));
    }
    u = block_reduce<1>(u);
    if (threadIdx.x == 0) out[0] = u;
    __syncthreads();
    a = block_reduce<1>(a);
    if (threadIdx.x == 0) out[1] = a;
}

// one-norm (max column sum) or infinity-norm (max row sum): out[0]
__global__ void __launch_bounds__(256)
colsum_kernel(int m, int n, const double *__restrict__ A, int ldA, double *__restrict__ s) {
    const int j = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (j >= n) return;
    double v = 0.0;
    for (int i = lane; i < m; i += 32) v += fabs(A[(size_t)i + (size_t)j * ldA]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if (lane == 0) s[j] = v;
}

__global__ void __launch_bounds__(256)
rowsum_kernel(int m, int n, const double *__restrict__ A, int ldA, double *__restrict__ s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    double v = 0.0;
    for (int j = 0; j < n; ++j) v += fabs(A[(size_t)i + (size_t)j * ldA]);
    s[i] = v;
}

int grid_for(int n) {
    const int g = (n + 255) / 256;
    const int cap = num_sms() * 8;
    return g < 1 ? 1 : (g > cap ? cap : g);
}

// Device scratch for one call: vectors of n and the reduction outputs.
struct Scratch {
    double *x, *v, *w1, *w2, *cnL, *cnU, *dg, *red;
    int *sgn, *flag;
    double *h;                                     // pinned host mirror of red
};

int scratch_for(int n, cudaStream_t s, Scratch *S) {
    const size_t nn = (size_t)(n > 0 ? n : 1);
    char *p = (char *)workspace_slot(s, 1, 8 * (7 * nn + 16) + 4 * (nn + 4) + 256);
    if (!p) return kErrAlloc;
    double *d = (double *)p;
    S->x = d;
    S->v = d + nn;
    S->w1 = d + 2 * nn;
    S->w2 = d + 3 * nn;
    S->cnL = d + 4 * nn;
    S->cnU = d + 5 * nn;
    S->dg = d + 6 * nn;
    S->red = d + 7 * nn;
    S->sgn = (int *)(d + 7 * nn + 16);
    S->flag = S->sgn + nn;
    thread_local double *h = nullptr;
    if (!h && cudaMallocHost((void **)&h, 16 * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        h = nullptr;
    }
    if (!h) {
        set_last_error("cudaMallocHost of the reduction readback failed");
        return kErrAlloc;
    }
    S->h = h;
    return kOk;
}

// stats of x read back: h[0] asum, h[1] max|x|, h[2] first index of max|x|,
// h[3] min x, h[4] first index of an exact zero (or -1)
int stats(int n, const double *x, int inc, Scratch &S, cudaStream_t s) {
    stats_kernel<<<1, RT, 0, s>>>(n, x, inc, S.red);
    FG_CUDA(cudaGetLastError());
    FG_CUDA(cudaMemcpyAsync(S.h, S.red, 5 * sizeof(double), cudaMemcpyDeviceToHost, s));
    FG_CUDA(cudaStreamSynchronize(s));
    return kOk;
}

// One step of lacn2 (flens/lapack/la/lacn2.tcc, real variant) on device
// vectors x (the operand), v and sgn; isave[0..2] as the reference's
// iSave(1..3) with 1-based indices.
int lacn2_step(int n, Scratch &S, double *est, int *kase, int *isave, cudaStream_t s) {
    const int itMax = 5;
    const int g = grid_for(n);
    int st;
    if (*kase == 0) {
        fill_kernel<<<g, 256, 0, s>>>(n, S.x, 1.0 / (double)n);
        FG_CUDA(cudaGetLastError());
        *kase = 1;
        isave[0] = 1;
        return kOk;
    }
    int jlast;
    double estold;
    switch (isave[0]) {
    case 1:
        if (n == 1) {
            FG_CUDA(cudaMemcpyAsync(S.v, S.x, sizeof(double), cudaMemcpyDeviceToDevice, s));
            if ((st = stats(1, S.x, 1, S, s)) != kOk) return st;
            *est = S.h[0];
            *kase = 0;
            return kOk;
        }
        if ((st = stats(n, S.x, 1, S, s)) != kOk) return st;
        *est = S.h[0];
        sign_kernel<<<g, 256, 0, s>>>(n, S.x, S.sgn);
        FG_CUDA(cudaGetLastError());
        *kase = 2;
        isave[0] = 2;
        return kOk;
    case 2:
        if ((st = stats(n, S.x, 1, S, s)) != kOk) return st;
        isave[1] = (int)S.h[2] + 1;
        isave[2] = 2;
    main_step:
        unit_kernel<<<g, 256, 0, s>>>(n, S.x, isave[1] - 1);
        FG_CUDA(cudaGetLastError());
        *kase = 1;
        isave[0] = 3;
        return kOk;
    case 3: {
        FG_CUDA(cudaMemcpyAsync(S.v, S.x, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        estold = *est;
        FG_CUDA(cudaMemsetAsync(S.flag, 0, sizeof(int), s));
        sign_changed_kernel<<<g, 256, 0, s>>>(n, S.x, S.sgn, S.flag);
        FG_CUDA(cudaGetLastError());
        FG_CUDA(cudaMemcpyAsync(S.red + 8, S.flag, sizeof(int), cudaMemcpyDeviceToDevice, s));
        if ((st = stats(n, S.v, 1, S, s)) != kOk) return st;
        *est = S.h[0];
        int changed = 0;
        FG_CUDA(cudaMemcpyAsync(&changed, S.flag, sizeof(int), cudaMemcpyDeviceToHost, s));
        FG_CUDA(cudaStreamSynchronize(s));
        if (!changed || *est <= estold) goto iteration_complete;
        sign_kernel<<<g, 256, 0, s>>>(n, S.x, S.sgn);
        FG_CUDA(cudaGetLastError());
        *kase = 2;
        isave[0] = 4;
        return kOk;
    }
    case 4: {
        jlast = isave[1];
        if ((st = stats(n, S.x, 1, S, s)) != kOk) return st;
        isave[1] = (int)S.h[2] + 1;
        double xj = 0.0;
        FG_CUDA(cudaMemcpyAsync(&xj, S.x + (jlast - 1), sizeof(double), cudaMemcpyDeviceToHost, s));
        FG_CUDA(cudaStreamSynchronize(s));
        if (xj != S.h[1] && isave[2] < itMax) {
            ++isave[2];
            goto main_step;
        }
    }
    iteration_complete:
        altsgn_kernel<<<g, 256, 0, s>>>(n, S.x);
        FG_CUDA(cudaGetLastError());
        *kase = 1;
        isave[0] = 5;
        return kOk;
    case 5: {
        if ((st = stats(n, S.x, 1, S, s)) != kOk) return st;
        const double temp = 2.0 * (S.h[0] / (double)(3 * n));
        if (temp > *est) {
            FG_CUDA(cudaMemcpyAsync(S.v, S.x, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, s));
            *est = temp;
        }
    }
    }
    *kase = 0;
    return kOk;
}

// latrs on its unscaled path (flens/lapack/la/latrs.tcc): the growth bound
// from the column norms cn and the diagonal dg (host copies) and max |x|
// decides; solve op(T) x = b in place on the device, or return 1 where the
// reference would switch to its scaled solve.
int latrs_unscaled(bool upper, bool trans, bool unit, int n, const double *LU, int ldLU, Scratch &S,
                   const std::vector<double> &cn, const std::vector<double> &dg, int *needs_scaling,
                   cudaStream_t s) {
    const double smallNum = kSafeMin / kPrecision, bigNum = 1.0 / smallNum;
    double tmax = 0.0;
    for (int j = 0; j < n; ++j) tmax = cn[j] > tmax ? cn[j] : tmax;
    if (tmax > bigNum) {
        *needs_scaling = 1;
        return kOk;
    }
    int st;
    if ((st = stats(n, S.x, 1, S, s)) != kOk) return st;
    const double xmax = S.h[1];
    double xbound = xmax, grow;
    int jfirst, jlast, jinc;
    if (!trans) {
        if (upper) { jfirst = n - 1; jlast = 0; jinc = -1; }
        else { jfirst = 0; jlast = n - 1; jinc = 1; }
    } else {
        if (upper) { jfirst = 0; jlast = n - 1; jinc = 1; }
        else { jfirst = n - 1; jlast = 0; jinc = -1; }
    }
    const int jend = jlast + jinc;
    auto mx = [](double a, double b) { return a < b ? b : a; };
    auto mn = [](double a, double b) { return b < a ? b : a; };
    if (!trans) {
        if (!unit) {
            grow = 1.0 / mx(xbound, smallNum);
            xbound = grow;
            bool too_small = false;
            for (int j = jfirst; j != jend; j += jinc) {
                if (grow <= smallNum) { too_small = true; break; }
                const double tjj = std::fabs(dg[j]);
                xbound = mn(xbound, mn(1.0, tjj) * grow);
                if (tjj + cn[j] >= smallNum) grow *= tjj / (tjj + cn[j]);
                else grow = 0.0;
            }
            if (!too_small) grow = xbound;
        } else {
            grow = mn(1.0, 1.0 / mx(xbound, smallNum));
            for (int j = jfirst; j != jend; j += jinc) {
                if (grow <= smallNum) break;
                grow *= 1.0 / (1.0 + cn[j]);
            }
        }
    } else {
        if (!unit) {
            grow = 1.0 / mx(xbound, smallNum);
            xbound = grow;
            for (int j = jfirst; j != jend; j += jinc) {
                if (grow <= smallNum) break;
                const double xj = 1.0 + cn[j];
                grow = mn(grow, xbound / xj);
                const double tjj = std::fabs(dg[j]);
                if (xj > tjj) xbound *= tjj / xj;
            }
            grow = mn(grow, xbound);
        } else {
            grow = mn(1.0, 1.0 / mx(xbound, smallNum));
            for (int j = jfirst; j != jend; j += jinc) {
                if (grow <= smallNum) break;
                grow /= 1.0 + cn[j];
            }
        }
    }
    if (!(grow > smallNum)) {
        *needs_scaling = 1;
        return kOk;
    }
    return dtrsm_launch('L', upper ? 'U' : 'L', trans ? 'T' : 'N', unit ? 'U' : 'N', n, 1, 1.0, LU,
                        ldLU, S.x, n, s);
}

}  // namespace

int dgecon_launch(char norm, int n, const double *LU, int ldLU, double anorm, double *rcond,
                  cudaStream_t s) {
    *rcond = 0.0;
    if (n == 0) {
        *rcond = 1.0;
        return kOk;
    }
    if (anorm == 0.0) return kOk;
    Scratch S;
    int st = scratch_for(n, s, &S);
    if (st != kOk) return st;
    const int g = grid_for(n);
    std::vector<double> cnL(n), cnU(n), dg(n);
    cnorm_kernel<<<ceil_div(n, 8), 256, 0, s>>>(n, LU, ldLU, 0, S.cnL);
    cnorm_kernel<<<ceil_div(n, 8), 256, 0, s>>>(n, LU, ldLU, 1, S.cnU);
    diag_kernel<<<g, 256, 0, s>>>(n, LU, ldLU, S.dg);
    FG_CUDA(cudaGetLastError());
    FG_CUDA(cudaMemcpyAsync(cnL.data(), S.cnL, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, s));
    FG_CUDA(cudaMemcpyAsync(cnU.data(), S.cnU, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, s));
    FG_CUDA(cudaMemcpyAsync(dg.data(), S.dg, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, s));
    FG_CUDA(cudaStreamSynchronize(s));
    const int kase1 = (norm == '1' || norm == 'O' || norm == 'o') ? 1 : 2;
    int kase = 0, isave[3] = {0, 0, 0}, scaled = 0;
    double ainvnm = 0.0;
    for (;;) {
        if ((st = lacn2_step(n, S, &ainvnm, &kase, isave, s)) != kOk) return st;
        if (kase == 0) break;
        if (kase == kase1) {
            if ((st = latrs_unscaled(false, false, true, n, LU, ldLU, S, cnL, dg, &scaled, s)) != kOk) return st;
            if (!scaled && (st = latrs_unscaled(true, false, false, n, LU, ldLU, S, cnU, dg, &scaled, s)) != kOk) return st;
        } else {
            if ((st = latrs_unscaled(true, true, false, n, LU, ldLU, S, cnU, dg, &scaled, s)) != kOk) return st;
            if (!scaled && (st = latrs_unscaled(false, true, true, n, LU, ldLU, S, cnL, dg, &scaled, s)) != kOk) return st;
        }
        if (scaled) {
            set_last_error("gecon: latrs would need its scaled solve; rcond reported as 0");
            return kErrUnsupported;
        }
    }
    if (ainvnm != 0.0) *rcond = (1.0 / ainvnm) / anorm;
    trace("gecon %c n=%d rcond=%g", norm, n, *rcond);
    return kOk;
}

int dgerfs_launch(char trans, int n, int nrhs, const double *A, int ldA, const double *AF, int ldAF,
                  const int *ipiv, const double *B, int ldB, double *X, int ldX, double *ferr,
                  double *berr, cudaStream_t s) {
    const bool nt = trans == 'N' || trans == 'n';
    const char tr = nt ? 'N' : 'T', trT = nt ? 'T' : 'N';
    if (n == 0 || nrhs == 0) {
        for (int j = 0; j < nrhs; ++j) ferr[j] = berr[j] = 0.0;
        return kOk;
    }
    Scratch S;
    int st = scratch_for(n, s, &S);
    if (st != kOk) return st;
    const int g = grid_for(n);
    const int nz = n + 1;
    const double eps = kEps, safe1 = nz * kSafeMin, safe2 = safe1 / eps;
    for (int j = 0; j < nrhs; ++j) {
        double *x = X + (size_t)j * ldX;
        const double *b = B + (size_t)j * ldB;
        int count = 1;
        double lastres = 3.0;
        for (;;) {
            FG_CUDA(cudaMemcpyAsync(S.w2, b, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, s));
            if ((st = dgemm_launch(tr, 'N', n, 1, n, -1.0, A, ldA, x, ldX, 1.0, S.w2, n, s)) != kOk) return st;
            if (nt) abs_gemv_n_kernel<<<ceil_div(n, 256), 256, 0, s>>>(n, A, ldA, x, b, S.w1);
            else abs_gemv_t_kernel<<<ceil_div(n, 8), 256, 0, s>>>(n, A, ldA, x, b, S.w1);
            berr_kernel<<<1, RT, 0, s>>>(n, S.w1, S.w2, safe1, safe2, S.red);
            FG_CUDA(cudaGetLastError());
            FG_CUDA(cudaMemcpyAsync(S.h, S.red, sizeof(double), cudaMemcpyDeviceToHost, s));
            FG_CUDA(cudaStreamSynchronize(s));
            berr[j] = S.h[0];
            if (berr[j] > eps && 2.0 * berr[j] <= lastres && count <= 5) {
                if ((st = dgetrs_launch(tr, n, 1, AF, ldAF, ipiv, S.w2, n, s)) != kOk) return st;
                axpy1_kernel<<<g, 256, 0, s>>>(n, x, S.w2);
                FG_CUDA(cudaGetLastError());
                lastres = berr[j];
                ++count;
                continue;
            }
            break;
        }
        ferr_weights_kernel<<<g, 256, 0, s>>>(n, S.w1, S.w2, (double)nz * eps, safe1, safe2);
        FG_CUDA(cudaGetLastError());
        // lacn2 works on S.x (the operand) and S.v: start from r (S.w2)
        int kase = 0, isave[3] = {0, 0, 0};
        double est = 0.0;
        for (;;) {
            if ((st = lacn2_step(n, S, &est, &kase, isave, s)) != kOk) return st;
            if (kase == 0) break;
            if (kase == 1) {
                if ((st = dgetrs_launch(trT, n, 1, AF, ldAF, ipiv, S.x, n, s)) != kOk) return st;
                mul_kernel<<<g, 256, 0, s>>>(n, S.x, S.w1);
            } else {
                mul_kernel<<<g, 256, 0, s>>>(n, S.x, S.w1);
                if ((st = dgetrs_launch(tr, n, 1, AF, ldAF, ipiv, S.x, n, s)) != kOk) return st;
            }
            FG_CUDA(cudaGetLastError());
        }
        if ((st = stats(n, x, 1, S, s)) != kOk) return st;
        ferr[j] = S.h[1] != 0.0 ? est / S.h[1] : est;
    }
    trace("gerfs %c n=%d nrhs=%d", trans, n, nrhs);
    return kOk;
}

// geequ: r (m), c (n) device; scalars and info on the host.
int dgeequ_launch(int m, int n, const double *A, int ldA, double *r, double *c, double *rowcnd,
                  double *colcnd, double *amax, int *info, cudaStream_t s) {
    *info = 0;
    if (m == 0 || n == 0) {
        *rowcnd = 1.0;
        *colcnd = 1.0;
        *amax = 0.0;
        return kOk;
    }
    Scratch S;
    int st = scratch_for(m > n ? m : n, s, &S);
    if (st != kOk) return st;
    const double smallNum = kSafeMin, bigNum = 1.0 / smallNum;
    row_absmax_kernel<<<ceil_div(m, 256), 256, 0, s>>>(m, n, A, ldA, r);
    FG_CUDA(cudaGetLastError());
    if ((st = stats(m, r, 1, S, s)) != kOk) return st;       // r >= 0: min r = h[3]
    const double rmin = S.h[3], rmax = S.h[1];
    *amax = rmax;
    if (rmin == 0.0) {
        *info = (int)S.h[4] + 1;
        return kOk;
    }
    recip_clamp_kernel<<<grid_for(m), 256, 0, s>>>(m, r, smallNum, bigNum);
    *rowcnd = (rmin > smallNum ? rmin : smallNum) / (rmax < bigNum ? rmax : bigNum);
    col_scaled_absmax_kernel<<<ceil_div(n, 8), 256, 0, s>>>(m, n, A, ldA, r, c);
    FG_CUDA(cudaGetLastError());
    if ((st = stats(n, c, 1, S, s)) != kOk) return st;
    const double cmin = S.h[3], cmax = S.h[1];
    if (cmin == 0.0) {
        *info = m + (int)S.h[4] + 1;
        return kOk;
    }
    recip_clamp_kernel<<<grid_for(n), 256, 0, s>>>(n, c, smallNum, bigNum);
    FG_CUDA(cudaGetLastError());
    *colcnd = (cmin > smallNum ? cmin : smallNum) / (cmax < bigNum ? cmax : bigNum);
    return kOk;
}

// laqge: returns 'N', 'R', 'C' or 'B' (flens/lapack/la/laq.tcc thresholds).
char dlaqge_launch(int m, int n, double *A, int ldA, const double *r, const double *c, double rowcnd,
                   double colcnd, double amax, cudaStream_t s) {
    if (m == 0 || n == 0) return 'N';
    const double small = kSafeMin / kPrecision, large = 1.0 / small;
    int mode;
    char eq;
    if (rowcnd >= 0.1 && amax >= small && amax <= large) {
        if (colcnd >= 0.1) return 'N';
        mode = 1;
        eq = 'C';
    } else if (colcnd >= 0.1) {
        mode = 2;
        eq = 'R';
    } else {
        mode = 3;
        eq = 'B';
    }
    const size_t total = (size_t)m * n;
    const int g = (int)((total + 255) / 256 < (size_t)num_sms() * 16 ? (total + 255) / 256 : num_sms() * 16);
    scale_matrix_kernel<<<g, 256, 0, s>>>(m, n, A, ldA, r, c, mode);
    if (cudaGetLastError() != cudaSuccess) return '?';
    return eq;
}

namespace {
int norm_of(char norm, int m, int n, const double *A, int ldA, Scratch &S, double *out,
            cudaStream_t s) {
    const bool one = norm == '1' || norm == 'O' || norm == 'o';
    double *sums = S.w1;                            // n (one) or m (inf) entries
    if (one) colsum_kernel<<<ceil_div(n, 8), 256, 0, s>>>(m, n, A, ldA, sums);
    else rowsum_kernel<<<ceil_div(m, 256), 256, 0, s>>>(m, n, A, ldA, sums);
    FG_CUDA(cudaGetLastError());
    int st = stats(one ? n : m, sums, 1, S, s);
    *out = S.h[1];
    return st;
}
}  // namespace

int dgesvx_launch(char fact, char trans, int n, int nrhs, double *A, int ldA, double *AF, int ldAF,
                  int *ipiv, char *equed, double *r, double *c, double *B, int ldB, double *X,
                  int ldX, double *rcond, double *ferr, double *berr, double *rpvgrw, int *info,
                  cudaStream_t s) {
    const double smallNum = kSafeMin, bigNum = 1.0 / smallNum;
    const bool nt = trans == 'N' || trans == 'n';
    *info = 0;
    bool rowequ, colequ;
    double rowcnd = 1.0, colcnd = 1.0;
    if (fact == 'N' || fact == 'E') {
        *equed = 'N';
        rowequ = colequ = false;
    } else {
        rowequ = *equed == 'R' || *equed == 'B';
        colequ = *equed == 'C' || *equed == 'B';
    }
    Scratch S;
    int st = scratch_for(n > 0 ? n : 1, s, &S);
    if (st != kOk) return st;
    if (n > 0 && rowequ) {
        if ((st = stats(n, r, 1, S, s)) != kOk) return st;
        rowcnd = (S.h[3] > smallNum ? S.h[3] : smallNum) / (S.h[1] < bigNum ? S.h[1] : bigNum);
    }
    if (n > 0 && colequ) {
        if ((st = stats(n, c, 1, S, s)) != kOk) return st;
        colcnd = (S.h[3] > smallNum ? S.h[3] : smallNum) / (S.h[1] < bigNum ? S.h[1] : bigNum);
    }
    if (fact == 'E') {
        double amax;
        int einfo;
        if ((st = dgeequ_launch(n, n, A, ldA, r, c, &rowcnd, &colcnd, &amax, &einfo, s)) != kOk) return st;
        if (einfo == 0) {
            *equed = dlaqge_launch(n, n, A, ldA, r, c, rowcnd, colcnd, amax, s);
            if (*equed == '?') return kErrCuda;
            rowequ = *equed == 'R' || *equed == 'B';
            colequ = *equed == 'C' || *equed == 'B';
        }
    }
    if (nt ? rowequ : colequ) {
        scale_matrix_kernel<<<grid_for(n * (nrhs > 0 ? nrhs : 1)), 256, 0, s>>>(n, nrhs, B, ldB, nt ? r : c,
                                                                             nullptr, 2);
        FG_CUDA(cudaGetLastError());
    }
    Workspace *w = workspace_for(s, 0);
    if (!w) return kErrAlloc;
    if (fact == 'N' || fact == 'E') {
        if (n > 0)
            FG_CUDA(cudaMemcpy2DAsync(AF, (size_t)ldAF * sizeof(double), A, (size_t)ldA * sizeof(double),
                                      (size_t)n * sizeof(double), n, cudaMemcpyDeviceToDevice, s));
        if ((st = dgetrf_launch(n, n, AF, ldAF, ipiv, w->info, s)) != kOk) return st;
        int h = 0;
        FG_CUDA(cudaMemcpyAsync(&h, w->info, sizeof(int), cudaMemcpyDeviceToHost, s));
        FG_CUDA(cudaStreamSynchronize(s));
        if (h > 0) {
            maxnorms_kernel<<<1, RT, 0, s>>>(h, AF, ldAF, n, n, A, ldA, S.red);
            FG_CUDA(cudaGetLastError());
            FG_CUDA(cudaMemcpyAsync(S.h, S.red, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
            FG_CUDA(cudaStreamSynchronize(s));
            *rpvgrw = S.h[0] == 0.0 ? 1.0 : S.h[1] / S.h[0];
            *rcond = 0.0;
            *info = h;
            return kOk;
        }
    }
    double anorm = 0.0;
    if (n > 0 && (st = norm_of(nt ? '1' : 'I', n, n, A, ldA, S, &anorm, s)) != kOk) return st;
    if (n > 0) {
        maxnorms_kernel<<<1, RT, 0, s>>>(n, AF, ldAF, n, n, A, ldA, S.red);
        FG_CUDA(cudaGetLastError());
        FG_CUDA(cudaMemcpyAsync(S.h, S.red, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
        FG_CUDA(cudaStreamSynchronize(s));
    }
    const double g = (n == 0 || S.h[0] == 0.0) ? 1.0 : S.h[1] / S.h[0];
    st = dgecon_launch(nt ? '1' : 'I', n, AF, ldAF, anorm, rcond, s);
    if (st != kOk && st != kErrUnsupported) return st;
    if (n > 0 && nrhs > 0)
        FG_CUDA(cudaMemcpy2DAsync(X, (size_t)ldX * sizeof(double), B, (size_t)ldB * sizeof(double),
                                  (size_t)n * sizeof(double), nrhs, cudaMemcpyDeviceToDevice, s));
    if ((st = dgetrs_launch(nt ? 'N' : 'T', n, nrhs, AF, ldAF, ipiv, X, ldX, s)) != kOk) return st;
    if ((st = dgerfs_launch(trans, n, nrhs, A, ldA, AF, ldAF, ipiv, B, ldB, X, ldX, ferr, berr, s)) != kOk)
        return st;
    if (nt ? colequ : rowequ) {
        scale_matrix_kernel<<<grid_for(n * (nrhs > 0 ? nrhs : 1)), 256, 0, s>>>(n, nrhs, X, ldX, nt ? c : r,
                                                                             nullptr, 2);
        FG_CUDA(cudaGetLastError());
        for (int j = 0; j < nrhs; ++j) ferr[j] /= nt ? colcnd : rowcnd;
    }
    *rpvgrw = g;
    if (*rcond < kEps) *info = n + 1;
    return kOk;
}

}  // namespace fg
