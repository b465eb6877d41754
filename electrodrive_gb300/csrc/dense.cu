// Dense single-layer operator (the reference's torch-tiled A(x),
// electrodrive/core/bem_kernel.py:157-230 and :341-381):
//   V_i = k_e sum_{j != i} sigma_j A_j / sqrt(max(|c_i - c_j|^2, 1e-24))
//         + self_integrals_i sigma_i A_i        (self term only if given)
//   non-finite V_i -> 0.
//
// The source index is split into chunks so that small N (5,120 panels) still
// fills every SM: block (row tile, chunk) accumulates its chunk's sources for
// 256 targets from (x, y, z, sigma A) tiles staged in shared memory and
// writes one partial sum per target; a second kernel adds the partials of a
// row in chunk order (deterministic) and applies k_e, the self term and the
// non-finite clamp.  With a single chunk the first kernel finishes the rows
// itself.
#include <algorithm>
#include <mutex>

#include "edfmm_internal.cuh"

namespace edfmm {

namespace {

constexpr int kRows = 256;  // targets per block (one per thread)
constexpr int kTile = 256;  // sources staged per shared-memory tile

__device__ __forceinline__ float inv_r(float r2) { return rsqrt_normal(fmaxf(r2, 1e-24f)); }
__device__ __forceinline__ double inv_r(double r2) { return rsqrt(fmax(r2, 1e-24)); }

template <typename T>
__device__ __forceinline__ T finish(T acc, int64_t i, T k_e, const T *self_int, const T *sigma, const T *areas) {
    T v = acc * k_e;
    if (self_int) v += self_int[i] * sigma[i] * areas[i];
    return isfinite(v) ? v : (T)0;
}

template <typename T>
__global__ void __launch_bounds__(kRows) k_dense_partial(const T *__restrict__ c, const T *__restrict__ sigma,
                                                         const T *__restrict__ areas, int64_t n, int64_t chunk,
                                                         T *__restrict__ partial, int finish_rows, T k_e,
                                                         const T *__restrict__ self_int, T *__restrict__ out) {
    using T4 = typename Vec4<T>::type;
    __shared__ T4 src[kTile];
    const int64_t i = (int64_t)blockIdx.x * kRows + threadIdx.x;
    const int64_t j0 = (int64_t)blockIdx.y * chunk;
    const int64_t j1 = min(n, j0 + chunk);
    T xi = 0, yi = 0, zi = 0;
    if (i < n) {
        xi = c[3 * i];
        yi = c[3 * i + 1];
        zi = c[3 * i + 2];
    }
    T acc = 0;
    for (int64_t jb = j0; jb < j1; jb += kTile) {
        const int64_t j = jb + threadIdx.x;
        T4 s;
        if (j < j1) {
            s.x = c[3 * j];
            s.y = c[3 * j + 1];
            s.z = c[3 * j + 2];
            s.w = sigma[j] * areas[j];
        } else {
            s.x = s.y = s.z = s.w = 0;
        }
        __syncthreads();
        src[threadIdx.x] = s;
        __syncthreads();
        const int cnt = (int)((j1 - jb) < (int64_t)kTile ? (j1 - jb) : (int64_t)kTile);
        const bool diag_here = i >= jb && i < jb + cnt;
        // two-level sum (tile, then chunk) bounds FP32 rounding growth
        T tacc = 0;
#pragma unroll 8
        for (int k = 0; k < cnt; ++k) {
            const T4 q = src[k];
            const T dx = xi - q.x, dy = yi - q.y, dz = zi - q.z;
            T w = q.w * inv_r(dx * dx + dy * dy + dz * dz);
            if (diag_here && jb + k == i) w = 0;
            tacc += w;
        }
        acc += tacc;
    }
    if (i >= n) return;
    if (finish_rows)
        out[i] = finish(acc, i, k_e, self_int, sigma, areas);
    else
        partial[(int64_t)blockIdx.y * n + i] = acc;
}

// induced potential at separate targets (no diagonal): bem_kernel.py:233-270
template <typename T>
__global__ void __launch_bounds__(kRows) k_targets_partial(const T *__restrict__ tgt, int64_t m,
                                                           const T *__restrict__ c, const T *__restrict__ sigma,
                                                           const T *__restrict__ areas, int64_t n, int64_t chunk,
                                                           T *__restrict__ partial, int finish_rows, T k_e,
                                                           T *__restrict__ out) {
    using T4 = typename Vec4<T>::type;
    __shared__ T4 src[kTile];
    const int64_t i = (int64_t)blockIdx.x * kRows + threadIdx.x;
    const int64_t j0 = (int64_t)blockIdx.y * chunk;
    const int64_t j1 = min(n, j0 + chunk);
    T xi = 0, yi = 0, zi = 0;
    if (i < m) {
        xi = tgt[3 * i];
        yi = tgt[3 * i + 1];
        zi = tgt[3 * i + 2];
    }
    T acc = 0;
    for (int64_t jb = j0; jb < j1; jb += kTile) {
        const int64_t j = jb + threadIdx.x;
        T4 s;
        if (j < j1) {
            s.x = c[3 * j];
            s.y = c[3 * j + 1];
            s.z = c[3 * j + 2];
            s.w = sigma[j] * areas[j];
        } else {
            s.x = s.y = s.z = s.w = 0;
        }
        __syncthreads();
        src[threadIdx.x] = s;
        __syncthreads();
        const int cnt = (int)((j1 - jb) < (int64_t)kTile ? (j1 - jb) : (int64_t)kTile);
        T tacc = 0;
#pragma unroll 8
        for (int k = 0; k < cnt; ++k) {
            const T4 q = src[k];
            const T dx = xi - q.x, dy = yi - q.y, dz = zi - q.z;
            tacc += q.w * inv_r(dx * dx + dy * dy + dz * dz);
        }
        acc += tacc;
    }
    if (i >= m) return;
    if (finish_rows)
        out[i] = acc * k_e;
    else
        partial[(int64_t)blockIdx.y * m + i] = acc;
}

// induced field at separate targets: E_i = sum_j (K_E / max(|x_i - r_j|^2,
// 1e-24)^(3/2)) (sigma_j A_j) (x_i - r_j)  (bem_kernel.py:280-335, Laplace
// fast path).  The weight is formed in the working dtype in the reference's
// order (K_E times 1/r^3, times sigma A), so a near-coincident pair overflows
// where the reference's does, and non-finite components become zero at the
// end (bem_kernel.py:990-997).
template <typename T>
__global__ void __launch_bounds__(kRows) k_field_partial(const T *__restrict__ tgt, int64_t m,
                                                         const T *__restrict__ c, const T *__restrict__ sigma,
                                                         const T *__restrict__ areas, int64_t n, int64_t chunk,
                                                         T *__restrict__ partial, int finish_rows, T k_e,
                                                         T *__restrict__ out) {
    using T4 = typename Vec4<T>::type;
    __shared__ T4 src[kTile];
    const int64_t i = (int64_t)blockIdx.x * kRows + threadIdx.x;
    const int64_t j0 = (int64_t)blockIdx.y * chunk;
    const int64_t j1 = min(n, j0 + chunk);
    T xi = 0, yi = 0, zi = 0;
    if (i < m) {
        xi = tgt[3 * i];
        yi = tgt[3 * i + 1];
        zi = tgt[3 * i + 2];
    }
    T ex = 0, ey = 0, ez = 0;
    for (int64_t jb = j0; jb < j1; jb += kTile) {
        const int64_t j = jb + threadIdx.x;
        T4 s;
        if (j < j1) {
            s.x = c[3 * j];
            s.y = c[3 * j + 1];
            s.z = c[3 * j + 2];
            s.w = sigma[j] * areas[j];
        } else {
            s.x = s.y = s.z = s.w = 0;
        }
        __syncthreads();
        src[threadIdx.x] = s;
        __syncthreads();
        const int cnt = (int)((j1 - jb) < (int64_t)kTile ? (j1 - jb) : (int64_t)kTile);
        T tx = 0, ty = 0, tz = 0;
#pragma unroll 8
        for (int k = 0; k < cnt; ++k) {
            const T4 q = src[k];
            const T dx = xi - q.x, dy = yi - q.y, dz = zi - q.z;
            const T ir = inv_r(dx * dx + dy * dy + dz * dz);
            const T w = (k_e * (ir * ir * ir)) * q.w;
            tx += w * dx;
            ty += w * dy;
            tz += w * dz;
        }
        ex += tx;
        ey += ty;
        ez += tz;
    }
    if (i >= m) return;
    if (finish_rows) {
        out[3 * i] = isfinite(ex) ? ex : (T)0;
        out[3 * i + 1] = isfinite(ey) ? ey : (T)0;
        out[3 * i + 2] = isfinite(ez) ? ez : (T)0;
    } else {
        T *p = partial + ((int64_t)blockIdx.y * m + i) * 3;
        p[0] = ex;
        p[1] = ey;
        p[2] = ez;
    }
}

template <typename T>
__global__ void k_field_reduce(const T *__restrict__ partial, int chunks, int64_t m, T *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    T ex = 0, ey = 0, ez = 0;
    for (int c = 0; c < chunks; ++c) {
        const T *p = partial + ((int64_t)c * m + i) * 3;
        ex += p[0];
        ey += p[1];
        ez += p[2];
    }
    out[3 * i] = isfinite(ex) ? ex : (T)0;
    out[3 * i + 1] = isfinite(ey) ? ey : (T)0;
    out[3 * i + 2] = isfinite(ez) ? ez : (T)0;
}

template <typename T>
__global__ void k_targets_reduce(const T *__restrict__ partial, int chunks, int64_t m, T k_e, T *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    T acc = 0;
    for (int c = 0; c < chunks; ++c) acc += partial[(int64_t)c * m + i];
    out[i] = acc * k_e;
}

template <typename T>
__global__ void k_dense_reduce(const T *__restrict__ partial, int chunks, int64_t n, T k_e,
                               const T *__restrict__ self_int, const T *__restrict__ sigma,
                               const T *__restrict__ areas, T *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    T acc = 0;
    for (int c = 0; c < chunks; ++c) acc += partial[(int64_t)c * n + i];
    out[i] = finish(acc, i, k_e, self_int, sigma, areas);
}

int sm_count() {
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 152;
    if (dev < 64 && cached[dev]) return cached[dev];
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (dev < 64) cached[dev] = sms;
    return sms;
}

}  // namespace

// Source chunking: enough blocks for ~8 per SM, at most 64 chunks, chunks a
// multiple of the shared-memory tile.
void dense_plan(int64_t n, int &chunks, int64_t &chunk) {
    const int64_t rows = (n + kRows - 1) / kRows;
    const int64_t want = 8LL * sm_count();
    int64_t c = rows >= want ? 1 : (want + rows - 1) / rows;
    c = std::min<int64_t>(std::max<int64_t>(c, 1), 64);
    chunk = ((n + c - 1) / c + kTile - 1) / kTile * kTile;
    if (chunk <= 0) chunk = kTile;
    chunks = (int)((n + chunk - 1) / chunk);
    if (chunks < 1) chunks = 1;
}

size_t dense_scratch_bytes(int64_t n, int dtype) {
    int chunks;
    int64_t chunk;
    dense_plan(n, chunks, chunk);
    if (chunks <= 1) return 0;
    return (size_t)chunks * (size_t)n * (dtype == EDFMM_F64 ? 8 : 4);
}

template <typename T>
int dense_run(const T *c, const T *sigma, const T *areas, const T *self_int, int64_t n, T k_e, T *out, T *partial,
              cudaStream_t s) {
    int chunks;
    int64_t chunk;
    dense_plan(n, chunks, chunk);
    dim3 grid((unsigned)((n + kRows - 1) / kRows), (unsigned)chunks);
    k_dense_partial<T><<<grid, kRows, 0, s>>>(c, sigma, areas, n, chunk, partial, chunks == 1, k_e, self_int, out);
    EDFMM_LAUNCH_CHECK("k_dense_partial");
    if (chunks > 1) {
        k_dense_reduce<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(partial, chunks, n, k_e, self_int, sigma, areas,
                                                                     out);
        EDFMM_LAUNCH_CHECK("k_dense_reduce");
    }
    return EDFMM_OK;
}

int dense_matvec(const void *c, const void *sigma, const void *areas, const void *self_int, int64_t n, int dtype,
                 double k_e, void *out, void *scratch, cudaStream_t s) {
    if (dtype == EDFMM_F64)
        return dense_run<double>(static_cast<const double *>(c), static_cast<const double *>(sigma),
                                 static_cast<const double *>(areas), static_cast<const double *>(self_int), n, k_e,
                                 static_cast<double *>(out), static_cast<double *>(scratch), s);
    return dense_run<float>(static_cast<const float *>(c), static_cast<const float *>(sigma),
                            static_cast<const float *>(areas), static_cast<const float *>(self_int), n, (float)k_e,
                            static_cast<float *>(out), static_cast<float *>(scratch), s);
}

}  // namespace edfmm

using namespace edfmm;

// ---------------------------------------------------------------------------
// Allocation-free variant.
//
// Some callers cannot allocate device memory while they apply the operator:
// an application whose framework allocator has already reserved the GPU's
// free memory (so a cudaMalloc/cudaMallocAsync from this library would fail
// or fragment that pool), or a host language binding that exposes no CUDA
// allocator and cannot release device memory it did not create.  For them,
// the partial sums live in one fixed, file-scope device array instead of
// stream-ordered scratch.  The array (8 MiB) is part of the library's
// device image: every GPU that loads the library holds it until the process
// exits.  Host code must not pass the array's name to a kernel (on the host
// it is only a stand-in symbol); its device address is looked up once per
// device with cudaGetSymbolAddress, with that device current, and kept for
// the life of the process (a cudaDeviceReset would make it stale, so the
// entry point is not for use after one).
// ---------------------------------------------------------------------------
#define EDFMM_DENSE_NOALLOC_SCRATCH_BYTES (8u << 20)
#define EDFMM_DENSE_NOALLOC_MAX_N 262144

static __device__ __align__(256) unsigned char g_dense_noalloc_scratch[EDFMM_DENSE_NOALLOC_SCRATCH_BYTES];

namespace {
std::mutex g_noalloc_mu;
constexpr int kMaxDevices = 64;
void *g_noalloc_addr[kMaxDevices] = {nullptr};

// Device address of g_dense_noalloc_scratch on the current device (looked up
// on the first call per device).
int noalloc_scratch(void **addr) {
    int dev = 0;
    EDFMM_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(EDFMM_ERR_ARG, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_dense_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(EDFMM_ERR_CUDA,
                        std::string("cudaGetSymbolAddress(g_dense_noalloc_scratch) failed: ") + cudaGetErrorString(e));
        g_noalloc_addr[dev] = p;
    }
    *addr = g_noalloc_addr[dev];
    return EDFMM_OK;
}
}  // namespace

extern "C" EDFMM_API int edfmm_dense_matvec_noalloc(const void *centroids, const void *sigma, const void *areas,
                                                    const void *self_integrals, int64_t n, int dtype, double k_e,
                                                    void *out, void *stream) {
    if (n < 0) return fail(EDFMM_ERR_ARG, "n must be >= 0");
    if (dtype != EDFMM_F32 && dtype != EDFMM_F64) return fail(EDFMM_ERR_ARG, "dtype must be EDFMM_F32 or EDFMM_F64");
    if (n > EDFMM_DENSE_NOALLOC_MAX_N)
        return fail(EDFMM_ERR_ARG, "edfmm_dense_matvec_noalloc: n = " + std::to_string(n) + " exceeds its limit of " +
                                       std::to_string(EDFMM_DENSE_NOALLOC_MAX_N) +
                                       " panels (fixed 8 MiB device scratch); use edfmm_dense_matvec");
    if (n == 0) return EDFMM_OK;
    if (!centroids || !sigma || !areas || !out) return fail(EDFMM_ERR_ARG, "centroids, sigma, areas, out must be non-NULL");
    const size_t bytes = dense_scratch_bytes(n, dtype);
    if (bytes > EDFMM_DENSE_NOALLOC_SCRATCH_BYTES)
        return fail(EDFMM_ERR_ARG, "edfmm_dense_matvec_noalloc: this device needs " + std::to_string(bytes) +
                                       " bytes of partial sums, above the fixed 8 MiB scratch; use edfmm_dense_matvec");
    void *scratch = nullptr;
    if (bytes) {
        if (int rc = noalloc_scratch(&scratch)) return rc;
    }
    // every partial-sum slot the reduction reads is written by this call, so
    // nothing left by an earlier call needs clearing
    return dense_matvec(centroids, sigma, areas, self_integrals, n, dtype, k_e, out, scratch,
                        static_cast<cudaStream_t>(stream));
}

namespace {
template <typename T>
int targets_run(const T *tgt, int64_t m, const T *c, const T *sigma, const T *areas, int64_t n, T k_e, T *out,
                cudaStream_t s) {
    // target rows of 256, source chunks so that there are ~8 blocks per SM
    const int64_t rows = (m + kRows - 1) / kRows;
    const int64_t want = 8LL * sm_count();
    int64_t nch = rows >= want ? 1 : (want + rows - 1) / rows;
    nch = std::min<int64_t>(std::max<int64_t>(nch, 1), 64);
    int64_t chunk = ((n + nch - 1) / nch + kTile - 1) / kTile * kTile;
    if (chunk <= 0) chunk = kTile;
    int chunks = (int)((n + chunk - 1) / chunk);
    if (chunks < 1) chunks = 1;
    T *partial = nullptr;
    if (chunks > 1) EDFMM_CUDA_TRY(cudaMallocAsync((void **)&partial, sizeof(T) * (size_t)chunks * (size_t)m, s));
    dim3 grid((unsigned)((m + kRows - 1) / kRows), (unsigned)chunks);
    k_targets_partial<T><<<grid, kRows, 0, s>>>(tgt, m, c, sigma, areas, n, chunk, partial, chunks == 1, k_e, out);
    int rc = EDFMM_OK;
    {
        count_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = fail(EDFMM_ERR_CUDA, std::string("k_targets_partial: ") + cudaGetErrorString(e));
    }
    if (!rc && chunks > 1) {
        k_targets_reduce<T><<<(unsigned)((m + 255) / 256), 256, 0, s>>>(partial, chunks, m, k_e, out);
        count_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = fail(EDFMM_ERR_CUDA, std::string("k_targets_reduce: ") + cudaGetErrorString(e));
    }
    if (partial) cudaFreeAsync(partial, s);
    return rc;
}
template <typename T>
int field_run(const T *tgt, int64_t m, const T *c, const T *sigma, const T *areas, int64_t n, T k_e, T *out,
              cudaStream_t s) {
    const int64_t rows = (m + kRows - 1) / kRows;
    const int64_t want = 8LL * sm_count();
    int64_t nch = rows >= want ? 1 : (want + rows - 1) / rows;
    nch = std::min<int64_t>(std::max<int64_t>(nch, 1), 64);
    int64_t chunk = ((n + nch - 1) / nch + kTile - 1) / kTile * kTile;
    if (chunk <= 0) chunk = kTile;
    int chunks = (int)((n + chunk - 1) / chunk);
    if (chunks < 1) chunks = 1;
    T *partial = nullptr;
    if (chunks > 1)
        EDFMM_CUDA_TRY(cudaMallocAsync((void **)&partial, sizeof(T) * 3 * (size_t)chunks * (size_t)m, s));
    dim3 grid((unsigned)((m + kRows - 1) / kRows), (unsigned)chunks);
    k_field_partial<T><<<grid, kRows, 0, s>>>(tgt, m, c, sigma, areas, n, chunk, partial, chunks == 1, k_e, out);
    int rc = EDFMM_OK;
    {
        count_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = fail(EDFMM_ERR_CUDA, std::string("k_field_partial: ") + cudaGetErrorString(e));
    }
    if (!rc && chunks > 1) {
        k_field_reduce<T><<<(unsigned)((m + 255) / 256), 256, 0, s>>>(partial, chunks, m, out);
        count_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = fail(EDFMM_ERR_CUDA, std::string("k_field_reduce: ") + cudaGetErrorString(e));
    }
    if (partial) cudaFreeAsync(partial, s);
    return rc;
}
}  // namespace

extern "C" EDFMM_API int edfmm_dense_field_targets(const void *targets, int64_t m, const void *centroids,
                                                   const void *sigma, const void *areas, int64_t n, int dtype,
                                                   double k_e, void *out, void *stream) {
    if (m < 0 || n < 0) return fail(EDFMM_ERR_ARG, "sizes must be >= 0");
    if (dtype != EDFMM_F32 && dtype != EDFMM_F64) return fail(EDFMM_ERR_ARG, "bad dtype");
    if (m == 0) return EDFMM_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (n == 0) {
        EDFMM_CUDA_TRY(cudaMemsetAsync(out, 0, (size_t)m * 3 * (dtype == EDFMM_F64 ? 8 : 4), s));
        return EDFMM_OK;
    }
    if (!targets || !centroids || !sigma || !areas || !out) return fail(EDFMM_ERR_ARG, "NULL argument");
    if (dtype == EDFMM_F64)
        return field_run<double>((const double *)targets, m, (const double *)centroids, (const double *)sigma,
                                 (const double *)areas, n, k_e, (double *)out, s);
    return field_run<float>((const float *)targets, m, (const float *)centroids, (const float *)sigma,
                            (const float *)areas, n, (float)k_e, (float *)out, s);
}

extern "C" EDFMM_API int edfmm_dense_potential_targets(const void *targets, int64_t m, const void *centroids,
                                                       const void *sigma, const void *areas, int64_t n, int dtype,
                                                       double k_e, void *out, void *stream) {
    if (m < 0 || n < 0) return fail(EDFMM_ERR_ARG, "sizes must be >= 0");
    if (dtype != EDFMM_F32 && dtype != EDFMM_F64) return fail(EDFMM_ERR_ARG, "bad dtype");
    if (m == 0) return EDFMM_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (n == 0) {
        EDFMM_CUDA_TRY(cudaMemsetAsync(out, 0, (size_t)m * (dtype == EDFMM_F64 ? 8 : 4), s));
        return EDFMM_OK;
    }
    if (!targets || !centroids || !sigma || !areas || !out) return fail(EDFMM_ERR_ARG, "NULL argument");
    if (dtype == EDFMM_F64)
        return targets_run<double>((const double *)targets, m, (const double *)centroids, (const double *)sigma,
                                   (const double *)areas, n, k_e, (double *)out, s);
    return targets_run<float>((const float *)targets, m, (const float *)centroids, (const float *)sigma,
                              (const float *)areas, n, (float)k_e, (float *)out, s);
}

extern "C" EDFMM_API size_t edfmm_dense_workspace_bytes(int64_t n, int dtype) {
    return n > 0 ? dense_scratch_bytes(n, dtype) : 0;
}

extern "C" EDFMM_API int edfmm_dense_matvec_ws(const void *centroids, const void *sigma, const void *areas,
                                               const void *self_integrals, int64_t n, int dtype, double k_e, void *out,
                                               void *workspace, size_t workspace_bytes, void *stream) {
    if (n < 0) return fail(EDFMM_ERR_ARG, "n must be >= 0");
    if (dtype != EDFMM_F32 && dtype != EDFMM_F64) return fail(EDFMM_ERR_ARG, "dtype must be EDFMM_F32 or EDFMM_F64");
    if (n == 0) return EDFMM_OK;
    if (!centroids || !sigma || !areas || !out) return fail(EDFMM_ERR_ARG, "centroids, sigma, areas, out must be non-NULL");
    const size_t bytes = dense_scratch_bytes(n, dtype);
    if (bytes && (!workspace || workspace_bytes < bytes))
        return fail(EDFMM_ERR_ARG, "workspace smaller than edfmm_dense_workspace_bytes(n, dtype)");
    return dense_matvec(centroids, sigma, areas, self_integrals, n, dtype, k_e, out, workspace,
                        static_cast<cudaStream_t>(stream));
}

extern "C" EDFMM_API int edfmm_dense_matvec(const void *centroids, const void *sigma, const void *areas,
                                            const void *self_integrals, int64_t n, int dtype, double k_e, void *out,
                                            void *stream) {
    if (n < 0) return fail(EDFMM_ERR_ARG, "n must be >= 0");
    if (dtype != EDFMM_F32 && dtype != EDFMM_F64) return fail(EDFMM_ERR_ARG, "dtype must be EDFMM_F32 or EDFMM_F64");
    if (n == 0) return EDFMM_OK;
    if (!centroids || !sigma || !areas || !out) return fail(EDFMM_ERR_ARG, "centroids, sigma, areas, out must be non-NULL");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t bytes = dense_scratch_bytes(n, dtype);
    void *scratch = nullptr;
    if (bytes) EDFMM_CUDA_TRY(cudaMallocAsync(&scratch, bytes, s));
    int rc = dense_matvec(centroids, sigma, areas, self_integrals, n, dtype, k_e, out, scratch, s);
    if (scratch) {
        cudaError_t e = cudaFreeAsync(scratch, s);
        if (!rc && e != cudaSuccess) rc = fail(EDFMM_ERR_CUDA, std::string("cudaFreeAsync: ") + cudaGetErrorString(e));
    }
    return rc;
}
