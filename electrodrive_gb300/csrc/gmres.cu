// Device-side Krylov arithmetic of restarted, left-preconditioned GMRES
// (the reference's gmres_restart, electrodrive/core/bem_solver.py:125-920).
//
// Vectors are in the working dtype T (float or double).  Elementwise work
// (products, updates, the partial sums of a thread or lane) is done in T;
// the reductions across lanes and blocks, every Hessenberg entry, Givens
// rotation and the small triangular solve are carried in FP64 on the device
// (FP64 arithmetic is scarce on this GPU, so it is kept off the per-element
// path), so the host reads nothing until the end of a restart cycle and a
// whole cycle can be replayed as one CUDA graph.
// Orthogonalisation is classical Gram-Schmidt applied twice (CGS2): per
// Arnoldi step two batched projections instead of the reference's j+1
// sequential modified-Gram-Schmidt passes; in exact arithmetic the basis is
// the same.  Reductions are deterministic: each block writes a partial sum
// and the partials are added in a fixed order (by a separate kernel, or by
// the last block to finish).
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
    T s_true = 0, s_pre = 0;  // per-thread sums of kItems squares in T, then FP64
    const int64_t base = (int64_t)blockIdx.x * kChunkN;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const int64_t i = base + (int64_t)k * kThreads + threadIdx.x;
        if (i < n) {
            const T rt = b[i] - ax[i];
            const T r = pinv ? pinv[i] * rt : rt;
            v0[i] = r;
            s_true += rt * rt;
            s_pre += r * r;
        }
    }
    double a = block_sum((double)s_true, sm);
    double c = block_sum((double)s_pre, sm);
    if (threadIdx.x == 0) {
        W.part[2 * blockIdx.x] = a;
        W.part[2 * blockIdx.x + 1] = c;
    }
    if (!last_block(W.counter)) return;
    double ta = 0, tc = 0;
    for (unsigned q = threadIdx.x; q < gridDim.x; q += blockDim.x) {
        ta += __ldcg(&W.part[2 * q]);
        tc += __ldcg(&W.part[2 * q + 1]);
    }
    ta = block_sum(ta, sm);
    tc = block_sum(tc, sm);
    if (threadIdx.x == 0) {
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

// v <- v / scal[idx] (skipped when that value is 0 or not finite), as a
// multiplication by the reciprocal taken once per block in FP64
template <typename T>
__global__ void k_scale_by(int64_t n, T *v, const T *src, const double *scal, int idx) {
    __shared__ double inv;
    if (threadIdx.x == 0) {
        const double d = scal[idx];
        inv = (d > 0.0 && isfinite(d)) ? 1.0 / d : 1.0;
    }
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    v[i] = src[i] * (T)inv;
}

// Partial h[r] = <V_r, w> over one chunk of kChunkN rows per block, r <= j
// (w = pinv * av on the first pass, written back).  The chunk of w is staged
// in shared memory and each warp takes whole rows r, so a block needs no
// barrier per row; the partials are added by k_dots_fin.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_dots(int64_t n, int j, int restart, const T *__restrict__ V,
                                                   T *__restrict__ w, const T *__restrict__ av,
                                                   const T *__restrict__ pinv, void *work) {
    __shared__ T ws[kChunkN];
    Work W = work_view(work, restart);
    const int64_t base = (int64_t)blockIdx.x * kChunkN;
    const int cnt = (int)(n - base < kChunkN ? n - base : kChunkN);
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const int q = k * kThreads + threadIdx.x;
        const int64_t i = base + q;
        T x = 0;
        if (q < cnt) {
            if (av) {
                x = pinv ? pinv[i] * av[i] : av[i];
                w[i] = x;
            } else {
                x = w[i];
            }
        }
        ws[q] = x;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int r = wid; r <= j; r += kThreads / 32) {
        const T *vr = V + (int64_t)r * n + base;
        T sl = 0;  // a lane's 32 products in T, then FP64 across lanes and blocks
#pragma unroll 8
        for (int q = lane; q < cnt; q += 32) sl += vr[q] * ws[q];
        double s = (double)sl;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) W.part[(int64_t)blockIdx.x * (restart + 1) + r] = s;
    }
}

// h[r] = sum of the blocks' partials (fixed order: lane-strided sums, then a
// fixed shuffle tree); one warp per row r, one block of 32 warps
__global__ void __launch_bounds__(1024) k_dots_fin(int nb, int j, int restart, void *work, int pass) {
    Work W = work_view(work, restart);
    double *h = pass == 1 ? W.h1 : W.h2;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int r = wid; r <= j; r += 32) {
        double t = 0;
        for (int q = lane; q < nb; q += 32) t += W.part[(int64_t)q * (restart + 1) + r];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) h[r] = t;
    }
}

// w -= sum_i h[i] V_i; on the second pass also |w| -> H[j+1, j] via scal
template <typename T>
__global__ void __launch_bounds__(kThreads) k_sub(int64_t n, int j, int restart, const T *__restrict__ V,
                                                  T *__restrict__ w, void *work, int pass, double *H) {
    __shared__ double sm[32];
    __shared__ T hs[257];
    Work W = work_view(work, restart);
    const double *h = pass == 1 ? W.h1 : W.h2;
    for (int r = threadIdx.x; r <= j; r += blockDim.x) hs[r] = (T)h[r];
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kChunkN;
    T s2 = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const int64_t i = base + (int64_t)k * kThreads + threadIdx.x;
        if (i < n) {
            T x = w[i];
            for (int r = 0; r <= j; ++r) x -= hs[r] * V[(int64_t)r * n + i];
            w[i] = x;
            s2 += x * x;
        }
    }
    if (pass == 1) return;
    double s2d = block_sum((double)s2, sm);
    if (threadIdx.x == 0) W.part[blockIdx.x] = s2d;
    if (!last_block(W.counter)) return;
    double t = 0;
    for (unsigned q = threadIdx.x; q < gridDim.x; q += blockDim.x) t += __ldcg(&W.part[q]);
    t = block_sum(t, sm);
    if (threadIdx.x == 0) {
        H[(int64_t)(j + 1) * restart + j] = sqrt(t);
        *W.counter = 0;
    }
}

// Hessenberg column j = h1 + h2, Givens rotations, g update, residual estimate.
// Mirrors bem_solver.py:590-616 (rotation with denom < 1e-14 -> identity).
// The column is gathered into shared memory by the warp, rotated by one
// thread there (a dependent chain through shared memory, not global), and
// written back by the warp.
__global__ void k_givens(int j, int restart, double *H, double *g, double *cs, double *sn, double *scal, void *work) {
    __shared__ double col[258];
    if (blockIdx.x != 0) return;
    Work W = work_view(work, restart);
    for (int i = threadIdx.x; i <= j; i += blockDim.x) col[i] = W.h1[i] + W.h2[i];
    if (threadIdx.x == 0) col[j + 1] = H[(int64_t)(j + 1) * restart + j];
    __syncwarp();
    if (threadIdx.x == 0) {
        const double hn = col[j + 1];
        if (!(isfinite(hn) && hn > 0.0)) {
            if (scal[2] < 0) scal[2] = (double)j;
        }
        for (int i = 0; i < j; ++i) {
            const double a = col[i], b = col[i + 1];
            col[i] = cs[i] * a + sn[i] * b;
            col[i + 1] = -sn[i] * a + cs[i] * b;
        }
        const double a = col[j], b = col[j + 1];
        const double den = sqrt(a * a + b * b);
        double c = 1.0, s = 0.0;
        if (den >= 1e-14 && isfinite(den)) {
            c = a / den;
            s = b / den;
        }
        cs[j] = c;
        sn[j] = s;
        col[j] = c * a + s * b;
        col[j + 1] = 0.0;
        const double gj = g[j];
        g[j] = c * gj;
        g[j + 1] = -s * gj;
        const double rn = fabs(g[j + 1]);
        scal[4 + j] = rn;
        if (!isfinite(rn)) scal[3] = 1.0;
        // keep the unrotated subdiagonal for the basis scaling
        scal[4 + restart] = hn;
    }
    __syncwarp();
    for (int i = threadIdx.x; i <= j + 1; i += blockDim.x) H[(int64_t)i * restart + j] = col[i];
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
    __shared__ T ys[256];
    Work W = work_view(work, restart);
    for (int r = threadIdx.x; r < m; r += blockDim.x) ys[r] = (T)W.y[r];
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    T acc = x[i];
    for (int r = 0; r < m; ++r) acc += ys[r] * V[(int64_t)r * n + i];
    x[i] = acc;
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
    k_dots<T><<<nb, kThreads, 0, s>>>(n, j, restart, Vt, (T *)w, (const T *)av, (const T *)pinv, work);
    EDFMM_LAUNCH_CHECK("k_dots");
    k_dots_fin<<<1, 1024, 0, s>>>((int)nb, j, restart, work, 1);
    EDFMM_LAUNCH_CHECK("k_dots_fin");
    k_sub<T><<<nb, kThreads, 0, s>>>(n, j, restart, Vt, (T *)w, work, 1, (double *)H);
    EDFMM_LAUNCH_CHECK("k_sub");
    k_dots<T><<<nb, kThreads, 0, s>>>(n, j, restart, Vt, (T *)w, nullptr, nullptr, work);
    EDFMM_LAUNCH_CHECK("k_dots");
    k_dots_fin<<<1, 1024, 0, s>>>((int)nb, j, restart, work, 2);
    EDFMM_LAUNCH_CHECK("k_dots_fin");
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
