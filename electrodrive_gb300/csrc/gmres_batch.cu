// Batched restarted GMRES: K independent systems stored back to back in one
// vector (instance k owns rows soff[k] .. soff[k+1]-1), one Krylov space and
// one Hessenberg matrix per instance, one operator application per step for
// all of them.  The operator of a batched plan is block diagonal, so this is
// K runs of the single-instance algorithm (gmres.cu: left Jacobi
// preconditioning, CGS2, FP64 Hessenberg and Givens rotations) that share
// their kernel launches; each instance stops on its own residual estimate.
//
// An instance is active while its cycle runs.  It leaves the cycle at the
// step where its estimate |g_{j+1}| meets its threshold, when its Krylov
// space becomes invariant (a zero subdiagonal: that step is kept, unlike the
// single-instance solver, which drops it) or on a non-finite value.  Its
// later basis vectors are written as zeros, so the shared operator sees zero
// rows for it and its Hessenberg stays untouched.
//
// Per-instance state (FP64, K rows of kStateCols + restart):
//   [0] true residual norm at cycle start   [1] beta = |M r|
//   [2] first breakdown step or -1           [3] non-finite flag
//   [4] last unrotated subdiagonal           [5] estimate threshold
//   [6] true-residual threshold              [7] steps taken this cycle
//   [8] active flag                          [9] steps in all cycles
//   [10 + j] |g_{j+1}| after step j.
// Reductions are deterministic: every block writes one partial per
// instance and a second kernel adds them in block order.
#include <cmath>

#include "edfmm_internal.cuh"

namespace edfmm {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 4;
constexpr int kChunk = kThreads * kItems;
constexpr int kStateCols = 10;

enum { S_RTRUE = 0, S_BETA, S_BRK, S_NONFIN, S_HSUB, S_THR, S_TOLABS, S_STEPS, S_ACTIVE, S_TOTAL, S_EST };

struct BatchView {
    const int64_t *soff;
    int K, B, R;
    double *st;    // K x (kStateCols + R)
    double *part;  // K x B x (R + 1)
    double *h;     // 2 x K x (R + 1)
    double *H;     // K x (R + 1) x R
    double *g;     // K x (R + 1)
    double *cs;    // K x R
    double *sn;    // K x R
    double *y;     // K x R
    __device__ double *row(int k) const { return st + (int64_t)k * (kStateCols + R); }
};

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

// rows of block (bb, k): [lo, hi) within instance k's segment
__device__ __forceinline__ void chunk_of(const BatchView &W, int k, int bb, int64_t &lo, int64_t &hi) {
    const int64_t a = W.soff[k], e = W.soff[k + 1];
    lo = a + (int64_t)bb * kChunk;
    hi = lo + kChunk < e ? lo + kChunk : e;
}

// r_true = b - ax, r = pinv * r_true -> v0; partial |r_true|^2, |r|^2
template <typename T>
__global__ void __launch_bounds__(kThreads) k_bstart(BatchView W, const T *__restrict__ b, const T *__restrict__ ax,
                                                     const T *__restrict__ pinv, T *__restrict__ v0) {
    __shared__ double sm[32];
    const int k = blockIdx.y, bb = blockIdx.x;
    int64_t lo, hi;
    chunk_of(W, k, bb, lo, hi);
    T s_true = 0, s_pre = 0;  // per-thread sums in T, FP64 across threads and blocks
#pragma unroll
    for (int q = 0; q < kItems; ++q) {
        const int64_t i = lo + (int64_t)q * kThreads + threadIdx.x;
        if (i < hi) {
            const T rt = b[i] - ax[i];
            const T r = pinv ? pinv[i] * rt : rt;
            v0[i] = r;
            s_true += rt * rt;
            s_pre += r * r;
        }
    }
    const double a = block_sum((double)s_true, sm);
    const double c = block_sum((double)s_pre, sm);
    if (threadIdx.x == 0) {
        double *p = W.part + ((int64_t)k * W.B + bb) * (W.R + 1);
        p[0] = a;
        p[1] = c;
    }
}

// per instance: norms, thresholds (first cycle), active flag, cycle reset.
// tol[k] < 0 marks an instance that takes no part in this solve.
__global__ void k_bstart_fin(BatchView W, const double *tol, int first) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= W.K) return;
    double ta = 0, tc = 0;
    for (int bb = 0; bb < W.B; ++bb) {
        const double *p = W.part + ((int64_t)k * W.B + bb) * (W.R + 1);
        ta += p[0];
        tc += p[1];
    }
    double *S = W.row(k);
    const double rt = sqrt(ta), beta = sqrt(tc);
    S[S_RTRUE] = rt;
    S[S_BETA] = beta;
    if (first) {
        const double tk = tol[k];
        const double init = rt > 1e-16 ? rt : 1.0;
        S[S_TOLABS] = tk < 0 ? INFINITY : fmax(fmax(tk * init, tk * 1e-12), 1e-12);
        S[S_THR] = tk < 0 ? INFINITY : tk * beta;
        S[S_TOTAL] = 0.0;
    }
    S[S_BRK] = -1.0;
    S[S_NONFIN] = 0.0;
    S[S_STEPS] = 0.0;
    S[S_HSUB] = beta;
    const bool go = isfinite(rt) && isfinite(beta) && beta > 0.0 && rt > S[S_TOLABS];
    S[S_ACTIVE] = go ? 1.0 : 0.0;
    if (!isfinite(rt) || !isfinite(beta)) S[S_NONFIN] = 1.0;
    double *g = W.g + (int64_t)k * (W.R + 1);
    for (int j = 0; j <= W.R; ++j) g[j] = 0.0;
    g[0] = beta;
    for (int j = 0; j < W.R; ++j) S[S_EST + j] = NAN;
}

// v <- v / state[col] for active instances, 0 for the others
template <typename T>
__global__ void __launch_bounds__(kThreads) k_bscale(BatchView W, T *__restrict__ v, const T *__restrict__ src,
                                                     int col) {
    const int k = blockIdx.y, bb = blockIdx.x;
    int64_t lo, hi;
    chunk_of(W, k, bb, lo, hi);
    __shared__ double inv;  // the reciprocal once per block in FP64
    if (threadIdx.x == 0) {
        const double *S = W.row(k);
        const double d = S[col];
        inv = (S[S_ACTIVE] != 0.0 && d > 0.0 && isfinite(d)) ? 1.0 / d : 0.0;
    }
    __syncthreads();
    const T f = (T)inv;
#pragma unroll
    for (int q = 0; q < kItems; ++q) {
        const int64_t i = lo + (int64_t)q * kThreads + threadIdx.x;
        if (i < hi) v[i] = src[i] * f;
    }
}

// partial <V_r, w> for r <= j over the block's chunk (w = pinv * av on the
// first pass, written back); the chunk of w is staged in shared memory and
// each warp takes whole rows r (no barrier per row)
template <typename T>
__global__ void __launch_bounds__(kThreads) k_bdots(BatchView W, int j, int64_t n, const T *__restrict__ V,
                                                    T *__restrict__ w, const T *__restrict__ av,
                                                    const T *__restrict__ pinv) {
    __shared__ T ws[kChunk];
    const int k = blockIdx.y, bb = blockIdx.x;
    if (W.row(k)[S_ACTIVE] == 0.0) return;  // uniform over the block
    int64_t lo, hi;
    chunk_of(W, k, bb, lo, hi);
    const int cnt = hi > lo ? (int)(hi - lo) : 0;
#pragma unroll
    for (int q = 0; q < kItems; ++q) {
        const int o = q * kThreads + threadIdx.x;
        const int64_t i = lo + o;
        T x = 0;
        if (o < cnt) {
            if (av) {
                x = pinv ? pinv[i] * av[i] : av[i];
                w[i] = x;
            } else {
                x = w[i];
            }
        }
        ws[o] = x;
    }
    __syncthreads();
    double *p = W.part + ((int64_t)k * W.B + bb) * (W.R + 1);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int r = wid; r <= j; r += kThreads / 32) {
        const T *vr = V + (int64_t)r * n + lo;
        T sl = 0;  // a lane's products in T, then FP64 across lanes and blocks
#pragma unroll 8
        for (int q = lane; q < cnt; q += 32) sl += vr[q] * ws[q];
        double s = (double)sl;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) p[r] = s;
    }
}

// h[pass][k][r] = sum over blocks (block order), r <= j; one block per instance
__global__ void k_bdots_fin(BatchView W, int j, int pass) {
    const int k = blockIdx.x;
    if (W.row(k)[S_ACTIVE] == 0.0) return;
    double *h = W.h + ((int64_t)(pass - 1) * W.K + k) * (W.R + 1);
    for (int r = threadIdx.x; r <= j; r += blockDim.x) {
        double t = 0;
        for (int bb = 0; bb < W.B; ++bb) t += W.part[((int64_t)k * W.B + bb) * (W.R + 1) + r];
        h[r] = t;
    }
}

// w -= sum_r h[r] V_r; on the second pass also the partial |w|^2
template <typename T>
__global__ void __launch_bounds__(kThreads) k_bsub(BatchView W, int j, int64_t n, const T *__restrict__ V,
                                                   T *__restrict__ w, int pass) {
    __shared__ double sm[32];
    __shared__ T hs[257];
    const int k = blockIdx.y, bb = blockIdx.x;
    if (W.row(k)[S_ACTIVE] == 0.0) return;
    const double *h = W.h + ((int64_t)(pass - 1) * W.K + k) * (W.R + 1);
    for (int r = threadIdx.x; r <= j; r += blockDim.x) hs[r] = (T)h[r];
    __syncthreads();
    int64_t lo, hi;
    chunk_of(W, k, bb, lo, hi);
    T s2 = 0;
#pragma unroll
    for (int q = 0; q < kItems; ++q) {
        const int64_t i = lo + (int64_t)q * kThreads + threadIdx.x;
        if (i < hi) {
            T x = w[i];
            for (int r = 0; r <= j; ++r) x -= hs[r] * V[(int64_t)r * n + i];
            w[i] = x;
            s2 += x * x;
        }
    }
    if (pass == 1) return;
    const double s2d = block_sum((double)s2, sm);
    if (threadIdx.x == 0) W.part[((int64_t)k * W.B + bb) * (W.R + 1)] = s2d;
}

// Hessenberg column j, Givens rotations, estimate, and the instance's exit
// test; one thread per instance (mirrors gmres.cu:k_givens)
__global__ void k_bgivens(BatchView W, int j) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= W.K) return;
    double *S = W.row(k);
    if (S[S_ACTIVE] == 0.0) return;
    const int R = W.R;
    double *H = W.H + (int64_t)k * (R + 1) * R;
    double *g = W.g + (int64_t)k * (R + 1);
    double *cs = W.cs + (int64_t)k * R, *sn = W.sn + (int64_t)k * R;
    const double *h1 = W.h + (int64_t)k * (R + 1), *h2 = W.h + ((int64_t)W.K + k) * (R + 1);
    double t = 0;
    for (int bb = 0; bb < W.B; ++bb) t += W.part[((int64_t)k * W.B + bb) * (R + 1)];
    const double hn = sqrt(t);
    for (int i = 0; i <= j; ++i) H[(int64_t)i * R + j] = h1[i] + h2[i];
    H[(int64_t)(j + 1) * R + j] = hn;
    // hn == 0: the Krylov space is invariant and column j completes the
    // solution (a lucky breakdown, kept; the next basis vector is zero).  A
    // non-finite hn drops column j, as the single-instance solver does.
    bool stop = hn == 0.0;
    if (!isfinite(hn)) {
        if (S[S_BRK] < 0) S[S_BRK] = (double)j;
        stop = true;
    }
    for (int i = 0; i < j; ++i) {
        const double a = H[(int64_t)i * R + j], b = H[(int64_t)(i + 1) * R + j];
        H[(int64_t)i * R + j] = cs[i] * a + sn[i] * b;
        H[(int64_t)(i + 1) * R + j] = -sn[i] * a + cs[i] * b;
    }
    const double a = H[(int64_t)j * R + j], b = H[(int64_t)(j + 1) * R + j];
    const double den = sqrt(a * a + b * b);
    double c = 1.0, s = 0.0;
    if (den >= 1e-14 && isfinite(den)) {
        c = a / den;
        s = b / den;
    }
    cs[j] = c;
    sn[j] = s;
    H[(int64_t)j * R + j] = c * a + s * b;
    H[(int64_t)(j + 1) * R + j] = 0.0;
    const double gj = g[j];
    g[j] = c * gj;
    g[j + 1] = -s * gj;
    const double rn = fabs(g[j + 1]);
    S[S_EST + j] = rn;
    S[S_STEPS] = (double)(j + 1);
    S[S_HSUB] = hn;
    if (!isfinite(rn)) {
        S[S_NONFIN] = 1.0;
        stop = true;
    }
    if (rn <= S[S_THR] || j + 1 >= R) stop = true;
    if (stop) S[S_ACTIVE] = 0.0;
}

// per instance: y = R^{-1} g[0:m], m = the breakdown step when there was one
__global__ void k_btrsv(BatchView W) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= W.K) return;
    const double *S = W.row(k);
    const int R = W.R;
    const int steps = (int)S[S_STEPS], brk = (int)S[S_BRK];
    const int m = brk >= 0 && brk < steps ? brk : steps;
    const double *H = W.H + (int64_t)k * (R + 1) * R;
    const double *g = W.g + (int64_t)k * (R + 1);
    double *y = W.y + (int64_t)k * R;
    for (int i = 0; i < R; ++i) y[i] = 0.0;
    for (int i = m - 1; i >= 0; --i) {
        double s = g[i];
        for (int q = i + 1; q < m; ++q) s -= H[(int64_t)i * R + q] * y[q];
        const double d = H[(int64_t)i * R + i];
        y[i] = d != 0.0 ? s / d : 0.0;
    }
    W.row(k)[S_TOTAL] += (double)steps;
}

// x += V[0:m]^T y per instance (y is zero beyond each instance's m)
template <typename T>
__global__ void __launch_bounds__(kThreads) k_bupdate(BatchView W, int m, int64_t n, const T *__restrict__ V,
                                                      T *__restrict__ x) {
    __shared__ T ys[256];
    const int k = blockIdx.y, bb = blockIdx.x;
    const double *y = W.y + (int64_t)k * W.R;
    for (int r = threadIdx.x; r < m; r += blockDim.x) ys[r] = (T)y[r];
    __syncthreads();
    int64_t lo, hi;
    chunk_of(W, k, bb, lo, hi);
#pragma unroll
    for (int q = 0; q < kItems; ++q) {
        const int64_t i = lo + (int64_t)q * kThreads + threadIdx.x;
        if (i < hi) {
            T acc = x[i];
            for (int r = 0; r < m; ++r) acc += ys[r] * V[(int64_t)r * n + i];
            x[i] = acc;
        }
    }
}

struct Views {
    BatchView W;
    dim3 grid;
    unsigned kb;  // blocks of 128 threads over instances
};

Views make_views(const int64_t *soff, int K, int B, int R, void *state, void *work) {
    Views v;
    BatchView &W = v.W;
    W.soff = soff;
    W.K = K;
    W.B = B;
    W.R = R;
    W.st = static_cast<double *>(state);
    double *p = static_cast<double *>(work);
    W.part = p;
    p += (int64_t)K * B * (R + 1);
    W.h = p;
    p += 2 * (int64_t)K * (R + 1);
    W.H = p;
    p += (int64_t)K * (R + 1) * R;
    W.g = p;
    p += (int64_t)K * (R + 1);
    W.cs = p;
    p += (int64_t)K * R;
    W.sn = p;
    p += (int64_t)K * R;
    W.y = p;
    v.grid = dim3((unsigned)B, (unsigned)K);
    v.kb = (unsigned)((K + 127) / 128);
    return v;
}

template <typename T>
int bstart(const Views &v, const void *b, const void *ax, const void *pinv, void *v0, const double *tol, int first,
           cudaStream_t s) {
    k_bstart<T><<<v.grid, kThreads, 0, s>>>(v.W, (const T *)b, (const T *)ax, (const T *)pinv, (T *)v0);
    EDFMM_LAUNCH_CHECK("k_bstart");
    k_bstart_fin<<<v.kb, 128, 0, s>>>(v.W, tol, first);
    EDFMM_LAUNCH_CHECK("k_bstart_fin");
    k_bscale<T><<<v.grid, kThreads, 0, s>>>(v.W, (T *)v0, (const T *)v0, S_BETA);
    EDFMM_LAUNCH_CHECK("k_bscale");
    return EDFMM_OK;
}

template <typename T>
int barnoldi(const Views &v, int64_t n, int j, void *V, const void *av, const void *pinv, void *w, cudaStream_t s) {
    T *Vt = (T *)V;
    k_bdots<T><<<v.grid, kThreads, 0, s>>>(v.W, j, n, Vt, (T *)w, (const T *)av, (const T *)pinv);
    EDFMM_LAUNCH_CHECK("k_bdots");
    k_bdots_fin<<<(unsigned)v.W.K, 64, 0, s>>>(v.W, j, 1);
    EDFMM_LAUNCH_CHECK("k_bdots_fin");
    k_bsub<T><<<v.grid, kThreads, 0, s>>>(v.W, j, n, Vt, (T *)w, 1);
    EDFMM_LAUNCH_CHECK("k_bsub");
    k_bdots<T><<<v.grid, kThreads, 0, s>>>(v.W, j, n, Vt, (T *)w, nullptr, nullptr);
    EDFMM_LAUNCH_CHECK("k_bdots");
    k_bdots_fin<<<(unsigned)v.W.K, 64, 0, s>>>(v.W, j, 2);
    EDFMM_LAUNCH_CHECK("k_bdots_fin");
    k_bsub<T><<<v.grid, kThreads, 0, s>>>(v.W, j, n, Vt, (T *)w, 2);
    EDFMM_LAUNCH_CHECK("k_bsub");
    k_bgivens<<<v.kb, 128, 0, s>>>(v.W, j);
    EDFMM_LAUNCH_CHECK("k_bgivens");
    k_bscale<T><<<v.grid, kThreads, 0, s>>>(v.W, Vt + (int64_t)(j + 1) * n, (const T *)w, S_HSUB);
    EDFMM_LAUNCH_CHECK("k_bscale");
    return EDFMM_OK;
}

template <typename T>
int bupdate(const Views &v, int64_t n, int m, const void *V, void *x, cudaStream_t s) {
    k_btrsv<<<v.kb, 128, 0, s>>>(v.W);
    EDFMM_LAUNCH_CHECK("k_btrsv");
    if (m > 0) {
        k_bupdate<T><<<v.grid, kThreads, 0, s>>>(v.W, m, n, (const T *)V, (T *)x);
        EDFMM_LAUNCH_CHECK("k_bupdate");
    }
    return EDFMM_OK;
}

int check_batch(int64_t n, int dtype, int K, int max_seg, int restart) {
    if (n <= 0 || K <= 0) return fail(EDFMM_ERR_ARG, "n and the instance count must be positive");
    if (max_seg <= 0 || max_seg > n) return fail(EDFMM_ERR_ARG, "max_seg must be in [1, n]");
    if (K > 65535) return fail(EDFMM_ERR_ARG, "at most 65535 instances");
    if (dtype != EDFMM_F32 && dtype != EDFMM_F64) return fail(EDFMM_ERR_ARG, "dtype must be EDFMM_F32 or EDFMM_F64");
    if (restart < 1 || restart > 256) return fail(EDFMM_ERR_ARG, "restart must be in [1, 256]");
    return EDFMM_OK;
}

inline int blocks_per_seg(int max_seg) { return (max_seg + kChunk - 1) / kChunk; }

}  // namespace
}  // namespace edfmm

using namespace edfmm;

extern "C" EDFMM_API size_t edfmm_bgmres_state_cols(int restart) { return (size_t)(kStateCols + restart); }

extern "C" EDFMM_API size_t edfmm_bgmres_work_bytes(int K, int max_seg, int restart) {
    const int64_t B = blocks_per_seg(max_seg), R = restart;
    return sizeof(double) * (size_t)(K * B * (R + 1) + 2 * K * (R + 1) + K * (R + 1) * R + K * (R + 1) + 3 * K * R);
}

extern "C" EDFMM_API int edfmm_bgmres_start(int64_t n, int dtype, int K, const int64_t *soff, int max_seg, int restart,
                                            const void *b, const void *ax, const void *pinv, void *v0,
                                            const double *tol, int first, void *state, void *work, void *stream) {
    if (int rc = check_batch(n, dtype, K, max_seg, restart)) return rc;
    if (!soff || !b || !ax || !v0 || !tol || !state || !work) return fail(EDFMM_ERR_ARG, "NULL argument");
    const Views v = make_views(soff, K, blocks_per_seg(max_seg), restart, state, work);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    return dtype == EDFMM_F64 ? bstart<double>(v, b, ax, pinv, v0, tol, first, s)
                              : bstart<float>(v, b, ax, pinv, v0, tol, first, s);
}

extern "C" EDFMM_API int edfmm_bgmres_arnoldi(int64_t n, int dtype, int K, const int64_t *soff, int max_seg,
                                              int restart, int j, void *V, const void *av, const void *pinv, void *w,
                                              void *state, void *work, void *stream) {
    if (int rc = check_batch(n, dtype, K, max_seg, restart)) return rc;
    if (j < 0 || j >= restart) return fail(EDFMM_ERR_ARG, "j must be in [0, restart)");
    if (!soff || !V || !av || !w || !state || !work) return fail(EDFMM_ERR_ARG, "NULL argument");
    const Views v = make_views(soff, K, blocks_per_seg(max_seg), restart, state, work);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    return dtype == EDFMM_F64 ? barnoldi<double>(v, n, j, V, av, pinv, w, s)
                              : barnoldi<float>(v, n, j, V, av, pinv, w, s);
}

extern "C" EDFMM_API int edfmm_bgmres_update(int64_t n, int dtype, int K, const int64_t *soff, int max_seg,
                                             int restart, int m, const void *V, void *x, void *state, void *work,
                                             void *stream) {
    if (int rc = check_batch(n, dtype, K, max_seg, restart)) return rc;
    if (m < 0 || m > restart) return fail(EDFMM_ERR_ARG, "m must be in [0, restart]");
    if (!soff || !V || !x || !state || !work) return fail(EDFMM_ERR_ARG, "NULL argument");
    const Views v = make_views(soff, K, blocks_per_seg(max_seg), restart, state, work);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    return dtype == EDFMM_F64 ? bupdate<double>(v, n, m, V, x, s) : bupdate<float>(v, n, m, V, x, s);
}
