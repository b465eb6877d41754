// Device-side Krylov arithmetic of restarted, left-preconditioned GMRES
// (the reference's gmres_restart, electrodrive/core/bem_solver.py:125-920).
//
// Vectors are in the working dtype T (float or double); every inner product,
// norm, Hessenberg entry, Givens rotation and the small triangular solve are
// carried in FP64 on the device, so the host reads nothing until the end of
// a restart cycle and a whole cycle can be replayed as one CUDA graph.
// Orthogonalisation is classical Gram-Schmidt applied twice (CGS2): per
// Arnoldi step two batched projections instead of the reference's j+1
// sequential modified-Gram-Schmidt passes; in exact arithmetic the basis is
// the same.  Reductions are deterministic: each block writes a partial sum
// and the last block to finish adds the partials in block order.
//
// Layout: V is (restart + 1, n) row-major in T; H is (restart + 1, restart)
// row-major FP64; g, cs, sn are FP64 vectors; `scal` (FP64) holds
//   [0] true residual norm at cycle start   [1] beta = |M r|
//   [2] first breakdown step or -1           [3] non-finite flag
//   [4 + j] |g_{j+1}| after Arnoldi step j.
#include <cmath>

#include "edfmm_internal.cuh"

namespace edfmm {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 4;
constexpr int kChunkN = kThreads * kItems;  // vector elements per block

inline unsigned nblocks(int64_t n) { return (unsigned)((n + kChunkN - 1) / kChunkN); }

// work area: [counter (uint, padded to 16 doubles)][h1 (R+1)][h2 (R+1)][y (R)][partials nb*(R+1)]
struct Work {
    unsigned *counter;
    double *h1, *h2, *y, *part;
};
__host__ __device__ inline Work work_view(void *base, int restart) {
    Work w;
    w.counter = static_cast<unsigned *>(base);
    double *d = static_cast<double *>(base) + 16;
    w.h1 = d;
    w.h2 = d + (restart + 1);
    w.y = d + 2 * (restart + 1);
    w.part = d + 3 * (restart + 1);
    return w;
}

__device__ __forceinline__ double block_sum(double v, double *sm) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) sm[wid] = v;
    __syncthreads();
    double t = 0;
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sm[k];
    return t;  // valid in thread 0
}

// true last-block election; returns true in every thread of the last block
__device__ __forceinline__ bool last_block(unsigned *counter) {
    __shared__ bool is_last;
    __threadfence();
    if (threadIdx.x == 0) {
        unsigned prev = atomicAdd(counter, 1u);
        is_last = prev == gridDim.x - 1;
    }
    __syncthreads();
    return is_last;
}

// r_true = b - ax; r = pinv * r_true (or r_true); V0 <- r (unscaled);
// scal[0] = |r_true|, scal[1] = |r|; resets g and the flags
template <typename T>
__global__ void __launch_bounds__(kThreads) k_start(int64_t n, const T *__restrict__ b, const T *__restrict__ ax,
                                                    const T *__restrict__ pinv, T *__restrict__ v0, double *g,
                                                    int restart, double *scal, void *work) {
    __shared__ double sm[32];
    Work W = work_view(work, restart);
    double s_true = 0, s_pre = 0;
    const int64_t base = (int64_t)blockIdx.x * kChunkN;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const int64_t i = base + (int64_t)k * kThreads + threadIdx.x;
        if (i < n) {
            const T rt = b[i] - ax[i];
            const T r = pinv ? pinv[i] * rt : rt;
            v0[i] = r;
            s_true += (double)rt * (double)rt;
            s_pre += (double)r * (double)r;
        }
    }
    double a = block_sum(s_true, sm);
    double c = block_sum(s_pre, sm);
    if (threadIdx.x == 0) {
        W.part[2 * blockIdx.x] = a;
        W.part[2 * blockIdx.x + 1] = c;
    }
    if (!last_block(W.counter)) return;
    if (threadIdx.x == 0) {
        double ta = 0, tc = 0;
        for (unsigned q = 0; q < gridDim.x; ++q) {
            ta += __ldcg(&W.part[2 * q]);
            tc += __ldcg(&W.part[2 * q + 1]);
        }
        scal[0] = sqrt(ta);
        scal[1] = sqrt(tc);
        scal[2] = -1.0;
        scal[3] = 0.0;
        for (int j = 0; j <= restart; ++j) g[j] = 0.0;
        g[0] = sqrt(tc);
        for (int j = 0; j < restart; ++j) scal[4 + j] = NAN;
        *W.counter = 0;
    }
}

// v <- v / scal[idx] (skipped when that value is 0 or not finite)
template <typename T>
__global__ void k_scale_by(int64_t n, T *v, const T *src, const double *scal, int idx) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double d = scal[idx];
    const T x = src[i];
    v[i] = (d > 0.0 && isfinite(d)) ? (T)((double)x / d) : x;
}

// h[i] = <V_i, w> for i <= j (w = pinv * av on the first pass, written back)
template <typename T>
__global__ void __launch_bounds__(kThreads) k_dots(int64_t n, int j, int restart, const T *__restrict__ V,
                                                   T *__restrict__ w, const T *__restrict__ av,
                                                   const T *__restrict__ pinv, void *work, int pass) {
    __shared__ double sm[32];
    Work W = work_view(work, restart);
    double *h = pass == 1 ? W.h1 : W.h2;
    const int64_t base = (int64_t)blockIdx.x * kChunkN;
    T wl[kItems];
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const int64_t i = base + (int64_t)k * kThreads + threadIdx.x;
        T x = 0;
        if (i < n) {
            if (av) {
                x = pinv ? pinv[i] * av[i] : av[i];
                w[i] = x;
            } else {
                x = w[i];
            }
        }
        wl[k] = x;
    }
    for (int r = 0; r <= j; ++r) {
        const T *vr = V + (int64_t)r * n;
        double s = 0;
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            const int64_t i = base + (int64_t)k * kThreads + threadIdx.x;
            if (i < n) s += (double)vr[i] * (double)wl[k];
        }
        s = block_sum(s, sm);
        if (threadIdx.x == 0) W.part[(int64_t)blockIdx.x * (restart + 1) + r] = s;
    }
    if (!last_block(W.counter)) return;
    for (int r = threadIdx.x; r <= j; r += blockDim.x) {
        double t = 0;
        for (unsigned q = 0; q < gridDim.x; ++q) t += __ldcg(&W.part[(int64_t)q * (restart + 1) + r]);
        h[r] = t;
    }
    __syncthreads();
    if (threadIdx.x == 0) *W.counter = 0;
}

// w -= sum_i h[i] V_i; on the second pass also |w| -> H[j+1, j] via scal
template <typename T>
__global__ void __launch_bounds__(kThreads) k_sub(int64_t n, int j, int restart, const T *__restrict__ V,
                                                  T *__restrict__ w, void *work, int pass, double *H) {
    __shared__ double sm[32];
    __shared__ double hs[257];
    Work W = work_view(work, restart);
    const double *h = pass == 1 ? W.h1 : W.h2;
    for (int r = threadIdx.x; r <= j; r += blockDim.x) hs[r] = h[r];
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kChunkN;
    double s2 = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const int64_t i = base + (int64_t)k * kThreads + threadIdx.x;
        if (i < n) {
            double x = (double)w[i];
            for (int r = 0; r <= j; ++r) x -= hs[r] * (double)V[(int64_t)r * n + i];
            const T xt = (T)x;
            w[i] = xt;
            s2 += (double)xt * (double)xt;
        }
    }
    if (pass == 1) return;
    s2 = block_sum(s2, sm);
    if (threadIdx.x == 0) W.part[blockIdx.x] = s2;
    if (!last_block(W.counter)) return;
    if (threadIdx.x == 0) {
        double t = 0;
        for (unsigned q = 0; q < gridDim.x; ++q) t += __ldcg(&W.part[q]);
        H[(int64_t)(j + 1) * restart + j] = sqrt(t);
        *W.counter = 0;
    }
}

// Hessenberg column j = h1 + h2, Givens rotations, g update, residual estimate.
// Mirrors bem_solver.py:590-616 (rotation with denom < 1e-14 -> identity).
__global__ void k_givens(int j, int restart, double *H, double *g, double *cs, double *sn, double *scal, void *work) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    Work W = work_view(work, restart);
    for (int i = 0; i <= j; ++i) H[(int64_t)i * restart + j] = W.h1[i] + W.h2[i];
    const double hn = H[(int64_t)(j + 1) * restart + j];
    if (!(isfinite(hn) && hn > 0.0)) {
        if (scal[2] < 0) scal[2] = (double)j;
    }
    for (int i = 0; i < j; ++i) {
        const double a = H[(int64_t)i * restart + j], b = H[(int64_t)(i + 1) * restart + j];
        H[(int64_t)i * restart + j] = cs[i] * a + sn[i] * b;
        H[(int64_t)(i + 1) * restart + j] = -sn[i] * a + cs[i] * b;
    }
    const double a = H[(int64_t)j * restart + j], b = H[(int64_t)(j + 1) * restart + j];
    const double den = sqrt(a * a + b * b);
    double c = 1.0, s = 0.0;
    if (den >= 1e-14 && isfinite(den)) {
        c = a / den;
        s = b / den;
    }
    cs[j] = c;
    sn[j] = s;
    H[(int64_t)j * restart + j] = c * a + s * b;
    H[(int64_t)(j + 1) * restart + j] = 0.0;
    const double gj = g[j];
    g[j] = c * gj;
    g[j + 1] = -s * gj;
    const double rn = fabs(g[j + 1]);
    scal[4 + j] = rn;
    if (!isfinite(rn)) scal[3] = 1.0;
    // keep the unrotated subdiagonal for the basis scaling
    scal[4 + restart] = hn;
}

// y = R^{-1} g[0:m] (upper triangular, FP64)
__global__ void k_trsv(int m, int restart, const double *H, const double *g, void *work) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    Work W = work_view(work, restart);
    for (int i = m - 1; i >= 0; --i) {
        double s = g[i];
        for (int k = i + 1; k < m; ++k) s -= H[(int64_t)i * restart + k] * W.y[k];
        const double d = H[(int64_t)i * restart + i];
        W.y[i] = (d != 0.0) ? s / d : 0.0;
    }
}

// x += V[0:m]^T y
template <typename T>
__global__ void k_update(int64_t n, int m, int restart, const T *__restrict__ V, T *__restrict__ x, void *work) {
    __shared__ double ys[256];
    Work W = work_view(work, restart);
    for (int r = threadIdx.x; r < m; r += blockDim.x) ys[r] = W.y[r];
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double acc = (double)x[i];
    for (int r = 0; r < m; ++r) acc += ys[r] * (double)V[(int64_t)r * n + i];
    x[i] = (T)acc;
}

}  // namespace

size_t gmres_work_bytes(int64_t n, int restart) {
    return sizeof(double) * (16 + 3 * (size_t)(restart + 1) + (size_t)nblocks(n) * (size_t)(restart + 1) + 2);
}

template <typename T>
int gmres_start(int64_t n, const void *b, const void *ax, const void *pinv, void *v0, void *g, int restart,
                void *scal, void *work, cudaStream_t s) {
    k_start<T><<<nblocks(n), kThreads, 0, s>>>(n, (const T *)b, (const T *)ax, (const T *)pinv, (T *)v0, (double *)g,
                                                restart, (double *)scal, work);
    EDFMM_LAUNCH_CHECK("k_start");
    k_scale_by<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, (T *)v0, (const T *)v0, (const double *)scal, 1);
    EDFMM_LAUNCH_CHECK("k_scale_by");
    return EDFMM_OK;
}

template <typename T>
int gmres_arnoldi(int64_t n, int j, int restart, void *V, const void *av, const void *pinv, void *H, void *g, void *cs,
                  void *sn, void *scal, void *w, void *work, cudaStream_t s) {
    const unsigned nb = nblocks(n);
    T *Vt = (T *)V;
    k_dots<T><<<nb, kThreads, 0, s>>>(n, j, restart, Vt, (T *)w, (const T *)av, (const T *)pinv, work, 1);
    EDFMM_LAUNCH_CHECK("k_dots");
    k_sub<T><<<nb, kThreads, 0, s>>>(n, j, restart, Vt, (T *)w, work, 1, (double *)H);
    EDFMM_LAUNCH_CHECK("k_sub");
    k_dots<T><<<nb, kThreads, 0, s>>>(n, j, restart, Vt, (T *)w, nullptr, nullptr, work, 2);
    EDFMM_LAUNCH_CHECK("k_dots");
    k_sub<T><<<nb, kThreads, 0, s>>>(n, j, restart, Vt, (T *)w, work, 2, (double *)H);
    EDFMM_LAUNCH_CHECK("k_sub");
    k_givens<<<1, 32, 0, s>>>(j, restart, (double *)H, (double *)g, (double *)cs, (double *)sn, (double *)scal, work);
    EDFMM_LAUNCH_CHECK("k_givens");
    k_scale_by<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, Vt + (int64_t)(j + 1) * n, (const T *)w,
                                                               (const double *)scal, 4 + restart);
    EDFMM_LAUNCH_CHECK("k_scale_by");
    return EDFMM_OK;
}

template <typename T>
int gmres_update(int64_t n, int m, int restart, const void *V, const void *H, const void *g, void *x, void *work,
                 cudaStream_t s) {
    k_trsv<<<1, 32, 0, s>>>(m, restart, (const double *)H, (const double *)g, work);
    EDFMM_LAUNCH_CHECK("k_trsv");
    k_update<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, m, restart, (const T *)V, (T *)x, work);
    EDFMM_LAUNCH_CHECK("k_update");
    return EDFMM_OK;
}

}  // namespace edfmm

using namespace edfmm;

static int check_common(int64_t n, int dtype, int restart) {
    if (n <= 0) return fail(EDFMM_ERR_ARG, "n must be positive");
    if (dtype != EDFMM_F32 && dtype != EDFMM_F64) return fail(EDFMM_ERR_ARG, "dtype must be EDFMM_F32 or EDFMM_F64");
    if (restart < 1 || restart > 256) return fail(EDFMM_ERR_ARG, "restart must be in [1, 256]");
    return EDFMM_OK;
}

extern "C" EDFMM_API size_t edfmm_gmres_work_bytes(int64_t n, int restart) { return gmres_work_bytes(n, restart); }

extern "C" EDFMM_API int edfmm_gmres_start(int64_t n, int dtype, int restart, const void *b, const void *ax,
                                           const void *pinv, void *v0, void *g, void *scal, void *work, void *stream) {
    if (int rc = check_common(n, dtype, restart)) return rc;
    if (!b || !ax || !v0 || !g || !scal || !work) return fail(EDFMM_ERR_ARG, "NULL argument");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    return dtype == EDFMM_F64 ? gmres_start<double>(n, b, ax, pinv, v0, g, restart, scal, work, s)
                              : gmres_start<float>(n, b, ax, pinv, v0, g, restart, scal, work, s);
}

extern "C" EDFMM_API int edfmm_gmres_arnoldi(int64_t n, int dtype, int restart, int j, void *V, const void *av,
                                             const void *pinv, void *H, void *g, void *cs, void *sn, void *scal,
                                             void *w, void *work, void *stream) {
    if (int rc = check_common(n, dtype, restart)) return rc;
    if (j < 0 || j >= restart) return fail(EDFMM_ERR_ARG, "j must be in [0, restart)");
    if (!V || !av || !H || !g || !cs || !sn || !scal || !w || !work) return fail(EDFMM_ERR_ARG, "NULL argument");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    return dtype == EDFMM_F64 ? gmres_arnoldi<double>(n, j, restart, V, av, pinv, H, g, cs, sn, scal, w, work, s)
                              : gmres_arnoldi<float>(n, j, restart, V, av, pinv, H, g, cs, sn, scal, w, work, s);
}

extern "C" EDFMM_API int edfmm_gmres_update(int64_t n, int dtype, int restart, int m, const void *V, const void *H,
                                            const void *g, void *x, void *work, void *stream) {
    if (int rc = check_common(n, dtype, restart)) return rc;
    if (m < 0 || m > restart) return fail(EDFMM_ERR_ARG, "m must be in [0, restart]");
    if (m == 0) return EDFMM_OK;
    if (!V || !H || !g || !x || !work) return fail(EDFMM_ERR_ARG, "NULL argument");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    return dtype == EDFMM_F64 ? gmres_update<double>(n, m, restart, V, H, g, x, work, s)
                              : gmres_update<float>(n, m, restart, V, H, g, x, work, s);
}
