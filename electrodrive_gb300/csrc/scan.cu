// Device-wide exclusive prefix sum and per-row sort of CSR value arrays.
#include <climits>

#include "edfmm_internal.cuh"

namespace edfmm {

namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int64_t block_exclusive_scan(int64_t v, int64_t *smem_warp, int64_t *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) smem_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int64_t w = lane < (int)(blockDim.x >> 5) ? smem_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int64_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        smem_warp[lane] = w;  // inclusive warp totals
    }
    __syncthreads();
    int64_t warp_base = warp ? smem_warp[warp - 1] : 0;
    if (total) *total = smem_warp[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warp_base + x - v;
}

__global__ void __launch_bounds__(kScanThreads) k_tile_sums(const int32_t *in, int64_t n, int64_t *sums) {
    __shared__ int64_t sw[32];
    int64_t base = (int64_t)blockIdx.x * kScanTile;
    int64_t acc = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        int64_t i = base + (int64_t)k * kScanThreads + threadIdx.x;
        if (i < n) acc += in[i];
    }
    int64_t tot;
    block_exclusive_scan(acc, sw, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// single block: exclusive scan of the tile sums (in place), writes grand total
__global__ void __launch_bounds__(kScanThreads) k_scan_sums(int64_t *sums, int64_t nt, int64_t *total) {
    __shared__ int64_t sw[32];
    int64_t carry = 0;
    for (int64_t base = 0; base < nt; base += kScanThreads) {
        int64_t i = base + threadIdx.x;
        int64_t v = i < nt ? sums[i] : 0;
        int64_t tot;
        int64_t ex = block_exclusive_scan(v, sw, &tot);
        if (i < nt) sums[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0 && total) *total = carry;
}

__global__ void __launch_bounds__(kScanThreads) k_tile_scan(const int32_t *in, int32_t *out, int64_t n,
                                                            const int64_t *sums) {
    __shared__ int64_t sw[32];
    int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int64_t v[kScanItems];
    int64_t acc = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        int64_t i = base + k;
        v[k] = i < n ? in[i] : 0;
        acc += v[k];
    }
    int64_t ex = block_exclusive_scan(acc, sw, nullptr) + sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        int64_t i = base + k;
        if (i < n) out[i] = (int32_t)ex;
        ex += v[k];
    }
}

// n <= one tile: the whole scan and its total in a single launch (most scans
// of the per-level tree and list builds are this small)
__global__ void __launch_bounds__(kScanThreads) k_scan_one_tile(const int32_t *in, int32_t *out, int64_t n,
                                                                int64_t *total) {
    __shared__ int64_t sw[32];
    const int64_t base = (int64_t)threadIdx.x * kScanItems;
    int64_t v[kScanItems];
    int64_t acc = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t i = base + k;
        v[k] = i < n ? in[i] : 0;
        acc += v[k];
    }
    int64_t tot;
    int64_t ex = block_exclusive_scan(acc, sw, &tot);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t i = base + k;
        if (i < n) out[i] = (int32_t)ex;
        ex += v[k];
    }
    if (threadIdx.x == 0 && total) *total = tot;
}

}  // namespace

size_t scan_tmp_bytes(int64_t n) {
    int64_t nt = (n + kScanTile - 1) / kScanTile;
    return sizeof(int64_t) * (size_t)(nt + 2);
}

int scan_exclusive(const int32_t *in, int32_t *out, int64_t n, int64_t *total_dev, void *tmp, cudaStream_t s) {
    if (n <= 0) {
        if (total_dev) EDFMM_CUDA_TRY(cudaMemsetAsync(total_dev, 0, sizeof(int64_t), s));
        return EDFMM_OK;
    }
    int64_t nt = (n + kScanTile - 1) / kScanTile;
    if (nt == 1) {
        k_scan_one_tile<<<1, kScanThreads, 0, s>>>(in, out, n, total_dev);
        EDFMM_LAUNCH_CHECK("k_scan_one_tile");
        return EDFMM_OK;
    }
    int64_t *sums = static_cast<int64_t *>(tmp);
    k_tile_sums<<<(unsigned)nt, kScanThreads, 0, s>>>(in, n, sums);
    EDFMM_LAUNCH_CHECK("k_tile_sums");
    k_scan_sums<<<1, kScanThreads, 0, s>>>(sums, nt, total_dev);
    EDFMM_LAUNCH_CHECK("k_scan_sums");
    k_tile_scan<<<(unsigned)nt, kScanThreads, 0, s>>>(in, out, n, sums);
    EDFMM_LAUNCH_CHECK("k_tile_scan");
    return EDFMM_OK;
}

// ---------------------------------------------------------------------------
// per-row bitonic sort
// ---------------------------------------------------------------------------
namespace {

constexpr int kRowCap = 4096;

__device__ __forceinline__ void bitonic_sort(int32_t *a, int len) {
    for (int k = 2; k <= len; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < len; i += blockDim.x) {
                int ixj = i ^ j;
                if (ixj > i) {
                    int32_t x = a[i], y = a[ixj];
                    bool up = (i & k) == 0;
                    if ((x > y) == up) {
                        a[i] = y;
                        a[ixj] = x;
                    }
                }
            }
            __syncthreads();
        }
    }
}

__global__ void __launch_bounds__(1024) k_sort_rows_smem(const int32_t *off, int32_t *vals, int64_t rows) {
    __shared__ int32_t buf[kRowCap];
    int64_t r = blockIdx.x;
    if (r >= rows) return;
    int32_t b = off[r], e = off[r + 1];
    int len = e - b;
    if (len <= 1 || len > kRowCap) return;
    int p2 = 1;
    while (p2 < len) p2 <<= 1;
    for (int i = threadIdx.x; i < p2; i += blockDim.x) buf[i] = i < len ? vals[b + i] : INT_MAX;
    __syncthreads();
    bitonic_sort(buf, p2);
    for (int i = threadIdx.x; i < len; i += blockDim.x) vals[b + i] = buf[i];
}

__global__ void __launch_bounds__(1024) k_sort_long_row(int32_t *row, int len, int32_t *scratch, int p2) {
    for (int i = threadIdx.x; i < p2; i += blockDim.x) scratch[i] = i < len ? row[i] : INT_MAX;
    __syncthreads();
    bitonic_sort(scratch, p2);
    for (int i = threadIdx.x; i < len; i += blockDim.x) row[i] = scratch[i];
}

}  // namespace

int sort_csr_rows(const int32_t *offsets, int32_t *vals, int64_t rows, int64_t max_row_len, cudaStream_t s) {
    if (rows <= 0 || max_row_len <= 1) return EDFMM_OK;
    k_sort_rows_smem<<<(unsigned)rows, 1024, 0, s>>>(offsets, vals, rows);
    EDFMM_LAUNCH_CHECK("k_sort_rows_smem");
    if (max_row_len <= kRowCap) return EDFMM_OK;
    // rows longer than the shared-memory capacity: one block each, global scratch
    std::vector<int32_t> h(rows + 1);
    EDFMM_CUDA_TRY(cudaMemcpyAsync(h.data(), offsets, sizeof(int32_t) * (rows + 1), cudaMemcpyDeviceToHost, s));
    EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
    int p2max = 1;
    while (p2max < max_row_len) p2max <<= 1;
    DevBuf scratch;
    int rc = scratch.reserve(sizeof(int32_t) * (size_t)p2max);
    if (rc) return rc;
    for (int64_t r = 0; r < rows; ++r) {
        int len = h[r + 1] - h[r];
        if (len <= kRowCap) continue;
        int p2 = 1;
        while (p2 < len) p2 <<= 1;
        k_sort_long_row<<<1, 1024, 0, s>>>(vals + h[r], len, dptr<int32_t>(scratch), p2);
        EDFMM_LAUNCH_CHECK("k_sort_long_row");
    }
    EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
    return EDFMM_OK;
}

}  // namespace edfmm
