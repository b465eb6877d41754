// Point-cloud warm-start network: per-panel features -> initial surface charge
// density for the GMRES start.  Inference and training kernels.
//
// Network (width 128, BF16 weights and activations, FP32 accumulation):
//   x_i  = 16 features of panel i (8 used, zero padded)
//   h1_i = relu(W1 x_i + b1)                          16 -> 128
//   g    = mean_i h1_i                                global context
//   h2_i = relu(W2 h1_i + V2 g + b2)                  128 -> 128
//   h3_i = relu(W3 h2_i + b3)                         128 -> 128
//   y_i  = w4 . h3_i + b4                             128 -> 1
// The three per-panel GEMMs and the weight gradients' partial products run
// on the tensor cores (mma.sync m16n8k16, BF16 inputs, FP32 accumulators);
// the context, output and bias reductions run on the FP32 pipe, and every
// reduction has a fixed order, so forward and backward are deterministic.
#include <cuda_bf16.h>

#include <algorithm>

#include "edfmm_internal.cuh"

namespace edfmm {
namespace {

constexpr int W = EDFMM_PCN_WIDTH;  // 128
constexpr int NIN = EDFMM_PCN_INPUTS;  // 16

// parameter block offsets (FP32)
constexpr int64_t O_W1 = 0;
constexpr int64_t O_B1 = O_W1 + W * NIN;
constexpr int64_t O_W2 = O_B1 + W;
constexpr int64_t O_V2 = O_W2 + W * W;
constexpr int64_t O_B2 = O_V2 + W * W;
constexpr int64_t O_W3 = O_B2 + W;
constexpr int64_t O_B3 = O_W3 + W * W;
constexpr int64_t O_W4 = O_B3 + W;
constexpr int64_t O_B4 = O_W4 + W;
constexpr int64_t NPARAM = O_B4 + 1;

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }
inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// workspace layout for n panels
struct Ws {
    __nv_bfloat16 *x0, *h1, *h2, *h3, *dz, *dz2;  // activations / gradients (n x K)
    __nv_bfloat16 *w1b, *w2b, *w3b;          // weights (out x in)
    __nv_bfloat16 *w2t, *w3t;                // transposed (in x out) for the data gradients
    float *g, *c2, *dc, *dg, *part;          // context vectors, partial sums
    double *stats;
    size_t bytes;
};

constexpr int kPartRows = 1024;  // rows per weight-gradient partial

inline int64_t n_parts(int64_t n) { return std::max<int64_t>(1, (n + kPartRows - 1) / kPartRows); }

Ws carve(void *base, int64_t n) {
    Ws w{};
    size_t o = 0;
    auto take = [&](size_t b) {
        size_t at = o;
        o = align256(o + b);
        return at;
    };
    const size_t bf = sizeof(__nv_bfloat16);
    size_t a_x0 = take(n * NIN * bf), a_h1 = take(n * W * bf), a_h2 = take(n * W * bf), a_h3 = take(n * W * bf),
           a_dz = take(n * W * bf), a_dz2 = take(n * W * bf), a_w1 = take(W * NIN * bf), a_w2 = take(W * W * bf), a_w3 = take(W * W * bf),
           a_w2t = take(W * W * bf), a_w3t = take(W * W * bf), a_g = take(W * 4), a_c2 = take(W * 4), a_dc = take(W * 4),
           a_dg = take(W * 4), a_part = take((size_t)n_parts(n) * (W * W + W) * 4), a_st = take(16 * 8);
    w.bytes = o;
    if (base) {
        char *b = static_cast<char *>(base);
        w.x0 = (__nv_bfloat16 *)(b + a_x0);
        w.h1 = (__nv_bfloat16 *)(b + a_h1);
        w.h2 = (__nv_bfloat16 *)(b + a_h2);
        w.h3 = (__nv_bfloat16 *)(b + a_h3);
        w.dz = (__nv_bfloat16 *)(b + a_dz);
        w.dz2 = (__nv_bfloat16 *)(b + a_dz2);
        w.w1b = (__nv_bfloat16 *)(b + a_w1);
        w.w2b = (__nv_bfloat16 *)(b + a_w2);
        w.w3b = (__nv_bfloat16 *)(b + a_w3);
        w.w2t = (__nv_bfloat16 *)(b + a_w2t);
        w.w3t = (__nv_bfloat16 *)(b + a_w3t);
        w.g = (float *)(b + a_g);
        w.c2 = (float *)(b + a_c2);
        w.dc = (float *)(b + a_dc);
        w.dg = (float *)(b + a_dg);
        w.part = (float *)(b + a_part);
        w.stats = (double *)(b + a_st);
    }
    return w;
}

// ---------------------------------------------------------------------------
// features
// ---------------------------------------------------------------------------
// stats: [0..2] mean centroid, [3] mean area, [4] rms rhs, [5] rms radius.
// Two passes of kStatBlocks blocks (grid-stride partial sums, then one small
// kernel that adds the blocks' partials in block order): the second pass
// needs the mean centroid of the first.  The partition is fixed, so the
// sums are deterministic.
constexpr int kStatBlocks = 152;

__global__ void __launch_bounds__(256) k_pcn_stats_part(const double *__restrict__ c, const double *__restrict__ a,
                                                        const double *__restrict__ b, int64_t n,
                                                        const double *__restrict__ mean, double *__restrict__ part) {
    __shared__ double red[5][8];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    double s[5] = {0, 0, 0, 0, 0};
    for (int64_t i = (int64_t)blockIdx.x * 256 + tid; i < n; i += (int64_t)gridDim.x * 256) {
        if (mean) {
            const double dx = c[3 * i] - mean[0], dy = c[3 * i + 1] - mean[1], dz = c[3 * i + 2] - mean[2];
            s[0] += dx * dx + dy * dy + dz * dz;
        } else {
            s[0] += c[3 * i];
            s[1] += c[3 * i + 1];
            s[2] += c[3 * i + 2];
            s[3] += a[i];
            s[4] += b[i] * b[i];
        }
    }
#pragma unroll
    for (int q = 0; q < 5; ++q) {
        for (int o = 16; o > 0; o >>= 1) s[q] += __shfl_xor_sync(0xffffffffu, s[q], o);
        if (lane == 0) red[q][wid] = s[q];
    }
    __syncthreads();
    if (tid < 5) {
        double t = 0;
        for (int w = 0; w < 8; ++w) t += red[tid][w];
        part[(int64_t)blockIdx.x * 8 + tid] = t;
    }
}

// pass 0: stats[0..4] from the first partials; pass 1: stats[5]
__global__ void k_pcn_stats_fin(const double *__restrict__ part, int nb, int64_t n, int pass, double *stats) {
    const int q = threadIdx.x;
    if (pass == 0 && q < 5) {
        double t = 0;
        for (int k = 0; k < nb; ++k) t += part[(int64_t)k * 8 + q];
        const double inv = n > 0 ? 1.0 / (double)n : 0.0;
        stats[q] = q < 4 ? t * inv : sqrt(t * inv);
    } else if (pass == 1 && q == 0) {
        double t = 0;
        for (int k = 0; k < nb; ++k) t += part[(int64_t)k * 8];
        stats[5] = sqrt(t / (double)(n > 0 ? n : 1));
    }
}

__global__ void k_pcn_features(const double *__restrict__ c, const double *__restrict__ nrm,
                               const double *__restrict__ a, const double *__restrict__ b, int64_t n,
                               const double *__restrict__ stats, float *__restrict__ f) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double R = stats[5] > 0 ? stats[5] : 1.0, rb = stats[4] > 0 ? stats[4] : 1.0;
    float *o = f + i * NIN;
    o[0] = (float)((c[3 * i] - stats[0]) / R);
    o[1] = (float)((c[3 * i + 1] - stats[1]) / R);
    o[2] = (float)((c[3 * i + 2] - stats[2]) / R);
    o[3] = (float)nrm[3 * i];
    o[4] = (float)nrm[3 * i + 1];
    o[5] = (float)nrm[3 * i + 2];
    o[6] = (float)(a[i] > 0 ? log(a[i] / (R * R)) : 0.0);
    o[7] = (float)(b[i] / rb);
    for (int q = 8; q < NIN; ++q) o[q] = 0.0f;
}

// ---------------------------------------------------------------------------
// weights: FP32 master -> BF16 (and transposed BF16 for the data gradients)
// ---------------------------------------------------------------------------
__global__ void k_pcn_cast(const float *__restrict__ prm, __nv_bfloat16 *w1b, __nv_bfloat16 *w2b,
                           __nv_bfloat16 *w3b, __nv_bfloat16 *w2t, __nv_bfloat16 *w3t) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < W * NIN) w1b[i] = __float2bfloat16_rn(prm[O_W1 + i]);
    if (i < W * W) {
        const int r = i / W, c = i % W;
        const __nv_bfloat16 x2 = __float2bfloat16_rn(prm[O_W2 + i]), x3 = __float2bfloat16_rn(prm[O_W3 + i]);
        w2b[i] = x2;
        w3b[i] = x3;
        w2t[c * W + r] = x2;
        w3t[c * W + r] = x3;
    }
}

__global__ void k_pcn_cast_x(const float *__restrict__ f, int64_t n, __nv_bfloat16 *__restrict__ x0) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n * NIN) x0[i] = __float2bfloat16_rn(f[i]);
}

// ---------------------------------------------------------------------------
// tensor-core linear layer: out[r][n] = epi(sum_k X[r][k] Wt[n][k])
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16 *p) { return *reinterpret_cast<const uint32_t *>(p); }

enum Epi { EPI_RELU = 0, EPI_MASK = 1 };

// One warp computes 16 rows x 128 columns.  Wt (128 x K, K contiguous) is
// staged in shared memory with a padded row stride (conflict-free fragment
// loads).  EPI_RELU: out = relu(acc + bias[n]) and optionally y = w4 . out + b4;
// EPI_MASK: out = mask[r][n] > 0 ? acc + bias[n] : 0 (ReLU backward).
template <int K, int EPI, bool HEAD>
__global__ void __launch_bounds__(128) k_pcn_linear(const __nv_bfloat16 *__restrict__ X, const __nv_bfloat16 *__restrict__ Wt,
                                                    const float *__restrict__ bias, const __nv_bfloat16 *__restrict__ mask,
                                                    int64_t n, __nv_bfloat16 *__restrict__ out,
                                                    const float *__restrict__ prm, float *__restrict__ y) {
    constexpr int LD = K + 8;  // padded row stride (bf16 elements)
    __shared__ __align__(16) __nv_bfloat16 sw[W * LD];
    for (int i = threadIdx.x; i < W * K / 2; i += blockDim.x) {
        const int r = (2 * i) / K, c = (2 * i) % K;
        *reinterpret_cast<uint32_t *>(&sw[r * LD + c]) = ld32(Wt + 2 * i);
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int64_t r0 = ((int64_t)blockIdx.x * 4 + warp) * 16;
    if (r0 >= n) return;
    const int64_t ra = r0 + g, rb = r0 + g + 8;
    const bool va = ra < n, vb = rb < n;
    float acc[16][4];
#pragma unroll
    for (int j = 0; j < 16; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
#pragma unroll
    for (int k0 = 0; k0 < K; k0 += 16) {
        uint32_t a[4];
        a[0] = va ? ld32(X + ra * K + k0 + 2 * t) : 0u;
        a[1] = vb ? ld32(X + rb * K + k0 + 2 * t) : 0u;
        a[2] = va ? ld32(X + ra * K + k0 + 2 * t + 8) : 0u;
        a[3] = vb ? ld32(X + rb * K + k0 + 2 * t + 8) : 0u;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const __nv_bfloat16 *wr = sw + (8 * j + g) * LD + k0 + 2 * t;
            mma_bf16(acc[j], a, ld32(wr), ld32(wr + 8));
        }
    }
    float ya = 0.0f, yb = 0.0f;
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        const int col = 8 * j + 2 * t;
        const float b0 = bias ? bias[col] : 0.0f, b1 = bias ? bias[col + 1] : 0.0f;
        float v[4] = {acc[j][0] + b0, acc[j][1] + b1, acc[j][2] + b0, acc[j][3] + b1};
        if (EPI == EPI_RELU) {
#pragma unroll
            for (int q = 0; q < 4; ++q) v[q] = fmaxf(v[q], 0.0f);
        } else {
            if (va) {
                const __nv_bfloat162 m = *reinterpret_cast<const __nv_bfloat162 *>(mask + ra * W + col);
                if (!(__bfloat162float(m.x) > 0.0f)) v[0] = 0.0f;
                if (!(__bfloat162float(m.y) > 0.0f)) v[1] = 0.0f;
            }
            if (vb) {
                const __nv_bfloat162 m = *reinterpret_cast<const __nv_bfloat162 *>(mask + rb * W + col);
                if (!(__bfloat162float(m.x) > 0.0f)) v[2] = 0.0f;
                if (!(__bfloat162float(m.y) > 0.0f)) v[3] = 0.0f;
            }
        }
        const __nv_bfloat162 oa = __floats2bfloat162_rn(v[0], v[1]), ob = __floats2bfloat162_rn(v[2], v[3]);
        if (va) *reinterpret_cast<__nv_bfloat162 *>(out + ra * W + col) = oa;
        if (vb) *reinterpret_cast<__nv_bfloat162 *>(out + rb * W + col) = ob;
        if (HEAD) {  // the head reads the stored (BF16-rounded) activations
            const float w0 = prm[O_W4 + col], w1 = prm[O_W4 + col + 1];
            ya += __bfloat162float(oa.x) * w0 + __bfloat162float(oa.y) * w1;
            yb += __bfloat162float(ob.x) * w0 + __bfloat162float(ob.y) * w1;
        }
    }
    if (HEAD) {
#pragma unroll
        for (int o = 1; o < 4; o <<= 1) {
            ya += __shfl_xor_sync(0xffffffffu, ya, o);
            yb += __shfl_xor_sync(0xffffffffu, yb, o);
        }
        if (t == 0) {
            const float b4 = prm[O_B4];
            if (va) y[ra] = ya + b4;
            if (vb) y[rb] = yb + b4;
        }
    }
}

// ---------------------------------------------------------------------------
// context: g = mean_i h1_i;  c2 = V2 g + b2
// ---------------------------------------------------------------------------
// per-part column sums of a BF16 (n x 128) matrix, optionally weighted by w[r]
__global__ void __launch_bounds__(W) k_pcn_colsum_part(const __nv_bfloat16 *__restrict__ h, const float *__restrict__ w,
                                                       int64_t n, float *__restrict__ part) {
    const int c = threadIdx.x;
    const int64_t r0 = (int64_t)blockIdx.x * kPartRows, r1 = (n < r0 + kPartRows) ? n : r0 + kPartRows;
    float s = 0.0f;
    for (int64_t r = r0; r < r1; ++r) {
        const float v = __bfloat162float(h[r * W + c]);
        s += w ? w[r] * v : v;
    }
    part[(int64_t)blockIdx.x * W + c] = s;
}

// out[c] = scale * sum_p part[p][c]  (fixed order)
__global__ void __launch_bounds__(W) k_pcn_reduce_cols(const float *__restrict__ part, int64_t np, float scale,
                                                       float *__restrict__ out) {
    const int c = threadIdx.x;
    float s = 0.0f;
    for (int64_t p = 0; p < np; ++p) s += part[p * W + c];
    out[c] = s * scale;
}

__global__ void __launch_bounds__(W) k_pcn_context(const float *__restrict__ prm, const float *__restrict__ g,
                                                   float *__restrict__ c2) {
    const int r = threadIdx.x;
    float s = prm[O_B2 + r];
    for (int k = 0; k < W; ++k) s += prm[O_V2 + r * W + k] * g[k];
    c2[r] = s;
}

// ---------------------------------------------------------------------------
// backward
// ---------------------------------------------------------------------------
// dz3[r][c] = (h3 > 0) ? dy[r] w4[c] : 0
__global__ void k_pcn_head_grad(const __nv_bfloat16 *__restrict__ h3, const float *__restrict__ dy,
                                const float *__restrict__ prm, int64_t n, __nv_bfloat16 *__restrict__ dz) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * W) return;
    const int64_t r = i / W;
    const int c = (int)(i % W);
    const float v = __bfloat162float(h3[i]) > 0.0f ? dy[r] * prm[O_W4 + c] : 0.0f;
    dz[i] = __float2bfloat16_rn(v);
}

// partial weight gradients over a block of rows, on the tensor cores:
//   part[p][o][k] = sum_{r in block p} D[r][o] X[r][k]     (o < 128, k < K)
//   part[p][128*K + o] = sum_r D[r][o]                   (bias gradient)
// The product D^T X has the rows r as its reduction dimension, so each stage
// of RT rows is staged transposed in shared memory (Dt[o][r], Xt[k][r], padded
// rows: conflict-free fragment loads) and warp w computes output rows
// 16w..16w+15 against all K columns with mma.sync m16n8k16 (BF16 in, FP32
// accumulate; the order of the additions is fixed, so the sums are
// deterministic).  The bias sums run on the FP32 pipe in row order.
template <int K>
__global__ void __launch_bounds__(256) k_pcn_wgrad_part(const __nv_bfloat16 *__restrict__ D,
                                                        const __nv_bfloat16 *__restrict__ X, int64_t n,
                                                        float *__restrict__ part) {
    constexpr int RT = 32;       // rows per stage (two MMA k-steps)
    constexpr int LD = RT + 8;   // padded row stride of the transposed tiles (bf16 elements)
    constexpr int NT = K / 8;    // n-tiles of 8 columns
    __shared__ __align__(16) __nv_bfloat16 Dt[W * LD];
    __shared__ __align__(16) __nv_bfloat16 Xt[K * LD];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int o0 = 16 * warp;
    float acc[NT][4];
#pragma unroll
    for (int j = 0; j < NT; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
    float bsum = 0.0f;
    const int64_t r0 = (int64_t)blockIdx.x * kPartRows, r1 = (n < r0 + kPartRows) ? n : r0 + kPartRows;
    for (int64_t rt = r0; rt < r1; rt += RT) {
        const int rows = (int)((r1 - rt < RT) ? r1 - rt : RT);
        __syncthreads();
        // transpose RT x 128 of D and RT x K of X into Dt / Xt (pairs of
        // columns per 32-bit global load; rows past the end are zeros)
        for (int i = tid; i < RT * (W / 2); i += 256) {
            const int r = i / (W / 2), c = 2 * (i % (W / 2));
            __nv_bfloat162 v = __floats2bfloat162_rn(0.0f, 0.0f);
            if (r < rows) v = *reinterpret_cast<const __nv_bfloat162 *>(D + (rt + r) * W + c);
            Dt[c * LD + r] = v.x;
            Dt[(c + 1) * LD + r] = v.y;
        }
        for (int i = tid; i < RT * (K / 2); i += 256) {
            const int r = i / (K / 2), c = 2 * (i % (K / 2));
            __nv_bfloat162 v = __floats2bfloat162_rn(0.0f, 0.0f);
            if (r < rows) v = *reinterpret_cast<const __nv_bfloat162 *>(X + (rt + r) * K + c);
            Xt[c * LD + r] = v.x;
            Xt[(c + 1) * LD + r] = v.y;
        }
        __syncthreads();
#pragma unroll
        for (int k0 = 0; k0 < RT; k0 += 16) {
            uint32_t a[4];
            a[0] = ld32(Dt + (o0 + g) * LD + k0 + 2 * t);
            a[1] = ld32(Dt + (o0 + g + 8) * LD + k0 + 2 * t);
            a[2] = ld32(Dt + (o0 + g) * LD + k0 + 2 * t + 8);
            a[3] = ld32(Dt + (o0 + g + 8) * LD + k0 + 2 * t + 8);
#pragma unroll
            for (int j = 0; j < NT; ++j) {
                const __nv_bfloat16 *xr = Xt + (8 * j + g) * LD + k0 + 2 * t;
                mma_bf16(acc[j], a, ld32(xr), ld32(xr + 8));
            }
        }
        if (tid < W)
            for (int r = 0; r < rows; ++r) bsum += __bfloat162float(Dt[tid * LD + r]);
    }
    float *pp = part + (int64_t)blockIdx.x * (W * K + W);
#pragma unroll
    for (int j = 0; j < NT; ++j) {
        const int col = 8 * j + 2 * t;
        pp[(o0 + g) * K + col] = acc[j][0];
        pp[(o0 + g) * K + col + 1] = acc[j][1];
        pp[(o0 + g + 8) * K + col] = acc[j][2];
        pp[(o0 + g + 8) * K + col + 1] = acc[j][3];
    }
    if (tid < W) pp[W * K + tid] = bsum;
}

// grads[off + i] = sum_p part[p][i] (i < W*K), grads[boff + o] = sum_p part[p][W*K + o]
__global__ void k_pcn_wgrad_reduce(const float *__restrict__ part, int64_t np, int K, float *__restrict__ grads,
                                   int64_t off, int64_t boff) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int stride = W * K + W;
    if (i >= stride) return;
    float s = 0.0f;
    for (int64_t p = 0; p < np; ++p) s += part[p * stride + i];
    if (i < W * K)
        grads[off + i] = s;
    else
        grads[boff + (i - W * K)] = s;
}

// head: dw4[c] = sum_r dy[r] h3[r][c] (from colsum partials), db4 = sum dy
__global__ void __launch_bounds__(256) k_pcn_sum(const float *__restrict__ v, int64_t n, float *__restrict__ out) {
    __shared__ float red[8];
    float s = 0.0f;
    for (int64_t i = threadIdx.x; i < n; i += 256) s += v[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.0f;
        for (int w = 0; w < 8; ++w) t += red[w];
        *out = t;
    }
}

// context backward: dV2 = dc2 g^T, db2 = dc2, dg = V2^T dc2 / n  (dc2 = column sum of dz2)
__global__ void __launch_bounds__(W) k_pcn_context_grad(const float *__restrict__ prm, const float *__restrict__ g,
                                                        const float *__restrict__ dc, int64_t n, float *__restrict__ grads,
                                                        float *__restrict__ dg) {
    const int r = threadIdx.x;
    for (int k = 0; k < W; ++k) grads[O_V2 + r * W + k] = dc[r] * g[k];
    float s = 0.0f;
    for (int o = 0; o < W; ++o) s += prm[O_V2 + o * W + r] * dc[o];
    dg[r] = s / (float)(n > 0 ? n : 1);
}

// ---------------------------------------------------------------------------
// loss: L = sum A (s (1 + y) - sigma)^2 / sum A sigma^2, dL/dy
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_pcn_loss(const float *__restrict__ y, const double *__restrict__ s,
                                                   const double *__restrict__ sigma, const double *__restrict__ a,
                                                   int64_t n, float *__restrict__ dy, double *__restrict__ loss) {
    __shared__ double red[2][32];
    __shared__ double den_s;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    double num = 0, den = 0;
    for (int64_t i = tid; i < n; i += blockDim.x) {
        const double e = s[i] * (1.0 + (double)y[i]) - sigma[i];
        num += a[i] * e * e;
        den += a[i] * sigma[i] * sigma[i];
    }
    for (int o = 16; o > 0; o >>= 1) {
        num += __shfl_xor_sync(0xffffffffu, num, o);
        den += __shfl_xor_sync(0xffffffffu, den, o);
    }
    if (lane == 0) {
        red[0][wid] = num;
        red[1][wid] = den;
    }
    __syncthreads();
    if (tid == 0) {
        double tn = 0, td = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            tn += red[0][w];
            td += red[1][w];
        }
        den_s = td > 0 ? td : 1.0;
        *loss = tn / den_s;
    }
    __syncthreads();
    const double d = den_s;
    for (int64_t i = tid; i < n; i += blockDim.x) {
        const double e = s[i] * (1.0 + (double)y[i]) - sigma[i];
        dy[i] = (float)(2.0 * a[i] * e * s[i] / d);
    }
}

__global__ void k_pcn_adam(float *__restrict__ p, const float *__restrict__ gr, float *__restrict__ m,
                           float *__restrict__ v, int64_t count, float lr, float b1, float b2, float eps, float c1,
                           float c2) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float gi = gr[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

}  // namespace
}  // namespace edfmm

using namespace edfmm;

extern "C" EDFMM_API int64_t edfmm_pcn_num_params(void) { return NPARAM; }

extern "C" EDFMM_API size_t edfmm_pcn_workspace_bytes(int64_t n) { return carve(nullptr, std::max<int64_t>(n, 1)).bytes; }

extern "C" EDFMM_API int edfmm_pcn_features(const double *centroids_dev, const double *normals_dev,
                                            const double *areas_dev, const double *rhs_dev, int64_t n,
                                            float *features_dev, void *ws_dev, size_t ws_bytes, void *stream) {
    if (n <= 0 || !centroids_dev || !normals_dev || !areas_dev || !rhs_dev || !features_dev || !ws_dev)
        return fail(EDFMM_ERR_ARG, "edfmm_pcn_features: bad arguments");
    Ws w = carve(ws_dev, n);
    if (ws_bytes < w.bytes) return fail(EDFMM_ERR_ARG, "edfmm_pcn_features: workspace too small");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the stats partials borrow the weight-gradient partial buffer (at least
    // W * W + W floats, far more than kStatBlocks * 8 doubles; not in use here)
    double *sp = reinterpret_cast<double *>(w.part);
    k_pcn_stats_part<<<kStatBlocks, 256, 0, s>>>(centroids_dev, areas_dev, rhs_dev, n, nullptr, sp);
    EDFMM_LAUNCH_CHECK("k_pcn_stats_part");
    k_pcn_stats_fin<<<1, 32, 0, s>>>(sp, kStatBlocks, n, 0, w.stats);
    EDFMM_LAUNCH_CHECK("k_pcn_stats_fin");
    k_pcn_stats_part<<<kStatBlocks, 256, 0, s>>>(centroids_dev, areas_dev, rhs_dev, n, w.stats, sp);
    EDFMM_LAUNCH_CHECK("k_pcn_stats_part");
    k_pcn_stats_fin<<<1, 32, 0, s>>>(sp, kStatBlocks, n, 1, w.stats);
    EDFMM_LAUNCH_CHECK("k_pcn_stats_fin");
    k_pcn_features<<<nblk(n, 256), 256, 0, s>>>(centroids_dev, normals_dev, areas_dev, rhs_dev, n, w.stats,
                                                 features_dev);
    EDFMM_LAUNCH_CHECK("k_pcn_features");
    return EDFMM_OK;
}

extern "C" EDFMM_API int edfmm_pcn_forward(const float *params_dev, const float *features_dev, int64_t n,
                                           float *y_dev, void *ws_dev, size_t ws_bytes, void *stream) {
    if (n <= 0 || !params_dev || !features_dev || !y_dev || !ws_dev)
        return fail(EDFMM_ERR_ARG, "edfmm_pcn_forward: bad arguments");
    Ws w = carve(ws_dev, n);
    if (ws_bytes < w.bytes) return fail(EDFMM_ERR_ARG, "edfmm_pcn_forward: workspace too small");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int64_t np = n_parts(n);
    k_pcn_cast<<<nblk(W * W, 256), 256, 0, s>>>(params_dev, w.w1b, w.w2b, w.w3b, w.w2t, w.w3t);
    EDFMM_LAUNCH_CHECK("k_pcn_cast");
    k_pcn_cast_x<<<nblk(n * NIN, 256), 256, 0, s>>>(features_dev, n, w.x0);
    EDFMM_LAUNCH_CHECK("k_pcn_cast_x");
    const unsigned grid = nblk(n, 64);
    k_pcn_linear<NIN, EPI_RELU, false><<<grid, 128, 0, s>>>(w.x0, w.w1b, params_dev + O_B1, nullptr, n, w.h1, params_dev,
                                                             nullptr);
    EDFMM_LAUNCH_CHECK("k_pcn_linear");
    k_pcn_colsum_part<<<(unsigned)np, W, 0, s>>>(w.h1, nullptr, n, w.part);
    EDFMM_LAUNCH_CHECK("k_pcn_colsum_part");
    k_pcn_reduce_cols<<<1, W, 0, s>>>(w.part, np, 1.0f / (float)n, w.g);
    EDFMM_LAUNCH_CHECK("k_pcn_reduce_cols");
    k_pcn_context<<<1, W, 0, s>>>(params_dev, w.g, w.c2);
    EDFMM_LAUNCH_CHECK("k_pcn_context");
    k_pcn_linear<W, EPI_RELU, false><<<grid, 128, 0, s>>>(w.h1, w.w2b, w.c2, nullptr, n, w.h2, params_dev, nullptr);
    EDFMM_LAUNCH_CHECK("k_pcn_linear");
    k_pcn_linear<W, EPI_RELU, true><<<grid, 128, 0, s>>>(w.h2, w.w3b, params_dev + O_B3, nullptr, n, w.h3, params_dev,
                                                          y_dev);
    EDFMM_LAUNCH_CHECK("k_pcn_linear");
    return EDFMM_OK;
}

extern "C" EDFMM_API int edfmm_pcn_backward(const float *params_dev, int64_t n, const float *dy_dev, float *grads_dev,
                                            void *ws_dev, size_t ws_bytes, void *stream) {
    if (n <= 0 || !params_dev || !dy_dev || !grads_dev || !ws_dev)
        return fail(EDFMM_ERR_ARG, "edfmm_pcn_backward: bad arguments");
    Ws w = carve(ws_dev, n);
    if (ws_bytes < w.bytes) return fail(EDFMM_ERR_ARG, "edfmm_pcn_backward: workspace too small");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int64_t np = n_parts(n);
    const unsigned grid = nblk(n, 64);
    // head: dw4 = sum_r dy_r h3_r, db4 = sum dy
    k_pcn_colsum_part<<<(unsigned)np, W, 0, s>>>(w.h3, dy_dev, n, w.part);
    EDFMM_LAUNCH_CHECK("k_pcn_colsum_part");
    k_pcn_reduce_cols<<<1, W, 0, s>>>(w.part, np, 1.0f, grads_dev + O_W4);
    EDFMM_LAUNCH_CHECK("k_pcn_reduce_cols");
    k_pcn_sum<<<1, 256, 0, s>>>(dy_dev, n, grads_dev + O_B4);
    EDFMM_LAUNCH_CHECK("k_pcn_sum");
    // layer 3: dz3 = (h3 > 0) dy w4;  dW3 = dz3^T h2;  dz2 = (h2 > 0) dz3 W3
    k_pcn_head_grad<<<nblk(n * W, 256), 256, 0, s>>>(w.h3, dy_dev, params_dev, n, w.dz);
    EDFMM_LAUNCH_CHECK("k_pcn_head_grad");
    k_pcn_wgrad_part<W><<<(unsigned)np, 256, 0, s>>>(w.dz, w.h2, n, w.part);
    EDFMM_LAUNCH_CHECK("k_pcn_wgrad_part");
    k_pcn_wgrad_reduce<<<nblk(W * W + W, 256), 256, 0, s>>>(w.part, np, W, grads_dev, O_W3, O_B3);
    EDFMM_LAUNCH_CHECK("k_pcn_wgrad_reduce");
    k_pcn_linear<W, EPI_MASK, false><<<grid, 128, 0, s>>>(w.dz, w.w3t, nullptr, w.h2, n, w.dz2, params_dev, nullptr);
    EDFMM_LAUNCH_CHECK("k_pcn_linear");
    // layer 2: dW2 = dz2^T h1, dc2 = colsum(dz2) -> dV2, db2, dg
    k_pcn_wgrad_part<W><<<(unsigned)np, 256, 0, s>>>(w.dz2, w.h1, n, w.part);
    EDFMM_LAUNCH_CHECK("k_pcn_wgrad_part");
    k_pcn_wgrad_reduce<<<nblk(W * W + W, 256), 256, 0, s>>>(w.part, np, W, grads_dev, O_W2, O_B2);
    EDFMM_LAUNCH_CHECK("k_pcn_wgrad_reduce");
    k_pcn_context_grad<<<1, W, 0, s>>>(params_dev, w.g, grads_dev + O_B2, n, grads_dev, w.dg);
    EDFMM_LAUNCH_CHECK("k_pcn_context_grad");
    // layer 1: dz1 = (h1 > 0) (dz2 W2 + dg / n);  dW1 = dz1^T x0
    k_pcn_linear<W, EPI_MASK, false><<<grid, 128, 0, s>>>(w.dz2, w.w2t, w.dg, w.h1, n, w.dz, params_dev, nullptr);
    EDFMM_LAUNCH_CHECK("k_pcn_linear");
    k_pcn_wgrad_part<NIN><<<(unsigned)np, 256, 0, s>>>(w.dz, w.x0, n, w.part);
    EDFMM_LAUNCH_CHECK("k_pcn_wgrad_part");
    k_pcn_wgrad_reduce<<<nblk(W * NIN + W, 256), 256, 0, s>>>(w.part, np, NIN, grads_dev, O_W1, O_B1);
    EDFMM_LAUNCH_CHECK("k_pcn_wgrad_reduce");
    return EDFMM_OK;
}

extern "C" EDFMM_API int edfmm_pcn_loss(const float *y_dev, const double *scale_dev, const double *sigma_dev,
                                        const double *areas_dev, int64_t n, float *dy_dev, double *loss_dev,
                                        void *stream) {
    if (n <= 0 || !y_dev || !scale_dev || !sigma_dev || !areas_dev || !dy_dev || !loss_dev)
        return fail(EDFMM_ERR_ARG, "edfmm_pcn_loss: bad arguments");
    k_pcn_loss<<<1, 1024, 0, static_cast<cudaStream_t>(stream)>>>(y_dev, scale_dev, sigma_dev, areas_dev, n, dy_dev,
                                                                   loss_dev);
    EDFMM_LAUNCH_CHECK("k_pcn_loss");
    return EDFMM_OK;
}

extern "C" EDFMM_API int edfmm_pcn_adam(float *params_dev, const float *grads_dev, float *m_dev, float *v_dev,
                                        int64_t count, float lr, float beta1, float beta2, float eps, int step,
                                        void *stream) {
    if (count <= 0 || step <= 0 || !params_dev || !grads_dev || !m_dev || !v_dev)
        return fail(EDFMM_ERR_ARG, "edfmm_pcn_adam: bad arguments");
    const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
    k_pcn_adam<<<nblk(count, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(params_dev, grads_dev, m_dev, v_dev,
                                                                                 count, lr, beta1, beta2, eps, c1, c2);
    EDFMM_LAUNCH_CHECK("k_pcn_adam");
    return EDFMM_OK;
}
