// Near field (P2P) fused with the local-expansion evaluation (L2P) and the
// matvec epilogue.
//
// One warp owns one target leaf.  Source leaves of the target's P2P row are
// staged in shared memory 64 points at a time (the next chunk loaded while
// the current one is computed) and read by broadcast.  The leaf's targets
// are split into slots that each fill the warp (32 targets with one lane
// each, 16 with two, 8 with four, 4 with eight); FP32 runs the distances as
// packed pairs.  The kernel is the reference's kernels_cpu.py:83-153
// contribution
//     q_s / max(|x_t - x_s|, eps)   (eps = machine epsilon of the dtype)
// evaluated as q_s * rsqrt(max(r^2, eps^2)), with the diagonal dropped only
// inside the self leaf pair.  The same warp then evaluates the leaf's local
// expansion at its points and, for a full matvec, applies the epilogue of
// bem_fmm.py:718-749 (K_E, original order, self term, non-finite -> 0), so
// each output is written exactly once.
#include <cfloat>
#include <type_traits>

#include "edfmm_internal.cuh"
#include "harmonics.cuh"
#include "twofloat.cuh"

namespace edfmm {

namespace {

__constant__ float c_rdiv_f[kPMax + 1][kPMax + 1];
__constant__ double c_rdiv_d[kPMax + 1][kPMax + 1];
__constant__ float2 c_rdiv_tf[kPMax + 1][kPMax + 1];  // (hi, lo) of the FP64 table

template <typename T> __device__ __forceinline__ T rdiv(int n, int m);
template <> __device__ __forceinline__ float rdiv<float>(int n, int m) { return c_rdiv_f[n][m]; }
template <> __device__ __forceinline__ double rdiv<double>(int n, int m) { return c_rdiv_d[n][m]; }

__device__ __forceinline__ double inv_dist(double r2, double eps2) { return rsqrt(fmax(r2, eps2)); }


// Re sum_{n,m} L_n^m R_n^m(x, y, z) over m in [-n, n]
template <typename T>
__device__ __forceinline__ T l2p_point(const Cplx<T> *L, int p, T x, T y, T z) {
    const T r2 = x * x + y * y + z * z;
    T acc = (T)0, dr = (T)1, di = (T)0;
    for (int m = 0; m <= p; ++m) {
        if (m > 0) {
            const T s = -(T)0.5 * rdiv<T>(m, 0) * (T)m;  // -1 / (2m): rdiv(m, 0) = 1 / m^2
            const T nr = s * (x * dr - y * di), ni = s * (x * di + y * dr);
            dr = nr;
            di = ni;
        }
        const T w = m == 0 ? (T)1 : (T)2;
        T pr = dr, pi = di, qr = (T)0, qi = (T)0;
        Cplx<T> lv = L[tri(m, m)];
        T col = lv.re * pr - lv.im * pi;
        for (int n = m + 1; n <= p; ++n) {
            const T d = rdiv<T>(n, m);
            const T c1 = (T)(2 * n - 1) * z;
            const T nr = (c1 * pr - r2 * qr) * d, ni = (c1 * pi - r2 * qi) * d;
            lv = L[tri(n, m)];
            col += lv.re * nr - lv.im * ni;
            qr = pr;
            qi = pi;
            pr = nr;
            pi = ni;
        }
        acc += w * col;
    }
    return acc;
}

// l2p_point in two-float arithmetic, on two-float locals
__device__ __forceinline__ tf32x2 l2p_point_tf(const tf32x2c *L, int p, tf32x2 x, tf32x2 y, tf32x2 z) {
    using T = tf32x2;
    const T r2 = fma(z, z, fma(y, y, x * x));
    T acc = T(0), dr = T(1), di = T(0);
    for (int m = 0; m <= p; ++m) {
        if (m > 0) {
            const float2 rd = c_rdiv_tf[m][0];
            const T sc = T(rd.x, rd.y) * T(-m) * T(0.5);  // -1 / (2m)
            const T nr = sc * (x * dr - y * di), ni = sc * (x * di + y * dr);
            dr = nr;
            di = ni;
        }
        T pr = dr, pi = di, qr = T(0), qi = T(0);
        tf32x2c lv = L[tri(m, m)];
        T col = lv.x * pr - lv.y * pi;
        for (int n = m + 1; n <= p; ++n) {
            const float2 rd = c_rdiv_tf[n][m];
            const T d(rd.x, rd.y);
            const T c1 = T(2 * n - 1) * z;
            const T nr = (c1 * pr - r2 * qr) * d, ni = (c1 * pi - r2 * qi) * d;
            lv = L[tri(n, m)];
            col = col + (lv.x * nr - lv.y * ni);
            qr = pr;
            qi = pi;
            pr = nr;
            pi = ni;
        }
        acc = m == 0 ? acc + col : acc + T(2) * col;
    }
    return acc;
}

template <typename T> struct NearParams {
    const int32_t *leaves;
    int64_t n_leaves;
    const int32_t *off;
    const int32_t *src;
    const typename Vec4<T>::type *pts;   // targets
    const int2 *range;                   // target leaves' point ranges
    const typename Vec4<T>::type *spts;  // sources (== pts for one tree)
    const float4 *spts_tf;               // two-float mode: sources as (xh, xl, yh, yl), (zh, zl, qh, ql)
    const int2 *srange;
    int same;                            // one tree: drop i == j in self pairs
    const typename Vec4<T>::type *center;
    const typename Vec4<T>::type *half;
    const Cplx<T> *Lexp;
    int p;
    int nc_pad;
    T eps2;
    int near;
    int far;
    const T *add_in;  // tree-order near sums computed by an earlier pass (nullable)
    InstMask mask;    // batched plans: leaves of inactive instances are skipped
    // epilogue
    int scatter;
    const int32_t *index_map;
    const T *sigma;
    const T *areas;
    const T *self_int;
    T k_e;
    T *out;
};

// Target slots.  A block of nt <= 64 targets of a leaf is split by the
// binary digits of nt rounded up to a multiple of 4: up to two slots of 32
// targets with one lane each, then 16 targets with 2 lanes each, 8 with 4
// and 4 with 8.  Every slot fills the warp, so the lanes stay busy whatever
// the leaf size; the lanes of a target take every G-th source (FP32: source
// pair) of a chunk and a fixed shuffle tree combines them.
template <typename T> struct Slot;
template <> struct Slot<float> {
    float2 nx, ny, nz;  // -x of the lane's target, in both halves
    float2 ps;          // packed partial sums
    int ti;             // target point index, -1 for a padding lane
};
template <> struct Slot<double> {
    double x, y, z;
    double ps;
    int ti;
};
template <> struct Slot<tf32x2> {
    tf32x2 x, y, z;
    tf32x2 ps;
    int ti;
};

// FP32: sources two at a time as packed pairs (FADD2 / FMUL2 / FFMA2); only
// the reciprocal square roots and the eps clamp are scalar.  An odd chunk is
// padded with a zero-charge source.
template <int G, bool SELF>
__device__ __forceinline__ void accumulate_slot(const float *sx, int cnt, int sbase, int part, Slot<float> &S,
                                                float eps2) {
    const float *sy = sx + 64, *sz = sx + 128, *sw = sx + 192;
    const int np = (cnt + 1) >> 1;
    float2 ps = S.ps;
#pragma unroll 2  // measured: 2.31 ms against 2.39 (unroll 4) at 1M uniform points
    for (int j = part; j < np; j += G) {
        const float2 qx = *reinterpret_cast<const float2 *>(sx + 2 * j);
        const float2 qy = *reinterpret_cast<const float2 *>(sy + 2 * j);
        const float2 qz = *reinterpret_cast<const float2 *>(sz + 2 * j);
        const float2 qw = *reinterpret_cast<const float2 *>(sw + 2 * j);
        const float2 dx = __fadd2_rn(qx, S.nx), dy = __fadd2_rn(qy, S.ny), dz = __fadd2_rn(qz, S.nz);
        const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
        float i0 = rsqrt_normal(fmaxf(r2.x, eps2)), i1 = rsqrt_normal(fmaxf(r2.y, eps2));
        if (SELF) {
            if (sbase + 2 * j == S.ti) i0 = 0.0f;
            if (sbase + 2 * j + 1 == S.ti) i1 = 0.0f;
        }
        ps = __ffma2_rn(qw, make_float2(i0, i1), ps);
    }
    S.ps = ps;
}

// FP64: one source per step from the staged (x, y, z, q) chunk
template <int G, bool SELF>
__device__ __forceinline__ void accumulate_slot(const double4 *sp, int cnt, int sbase, int part, Slot<double> &S,
                                                double eps2) {
    double ps = 0.0;
#pragma unroll 4
    for (int j = part; j < cnt; j += G) {
        const double4 q = sp[j];
        const double dx = S.x - q.x, dy = S.y - q.y, dz = S.z - q.z;
        double inv = inv_dist(dx * dx + dy * dy + dz * dz, eps2);
        if (SELF && sbase + j == S.ti) inv = 0.0;
        ps += q.w * inv;
    }
    S.ps += ps;  // per-chunk partial, then one add: two-level summation
}

// Two-float: one source per step from the staged split points
// (s4[2j] = (xh, xl, yh, yl), s4[2j + 1] = (zh, zl, qh, ql): two 16-byte
// shared loads).  The coordinate differences are formed from the split
// parts, so the cancellation of nearby points loses nothing; 1 / r takes one
// Newton step from the FP32 estimate.
template <int G, bool SELF>
__device__ __forceinline__ void accumulate_slot(const float4 *s4, int cnt, int sbase, int part, Slot<tf32x2> &S,
                                                float eps2) {
    tf32x2 ps = tf32x2(0);
#pragma unroll 2
    for (int j = part; j < cnt; j += G) {
        const float4 a = s4[2 * j], b = s4[2 * j + 1];
        const tf32x2 dx = S.x - tf32x2(a.x, a.y);
        const tf32x2 dy = S.y - tf32x2(a.z, a.w);
        const tf32x2 dz = S.z - tf32x2(b.x, b.y);
        tf32x2 r2 = fma(dz, dz, fma(dy, dy, dx * dx));
        if (!(r2.hi >= eps2)) r2 = tf32x2(eps2, 0.0f);
        tf32x2 inv = tf_rsqrt(r2, rsqrt_normal(r2.hi));
        if (SELF && sbase + j == S.ti) inv = tf32x2(0);
        ps = fma(tf32x2(b.z, b.w), inv, ps);
    }
    S.ps = S.ps + ps;  // per-chunk partial, then one add: two-level summation
}

template <typename T, int G>
__device__ __forceinline__ void slot_init(const NearParams<T> &P, int tb, int te, int base, int lane, Slot<T> &S) {
    const int ti = tb + base + lane / G;
    S.ti = ti < te ? ti : -1;
    const typename Vec4<T>::type x = P.pts[ti < te ? ti : tb];
    if constexpr (sizeof(T) == 4) {
        S.nx = make_float2(-x.x, -x.x);
        S.ny = make_float2(-x.y, -x.y);
        S.nz = make_float2(-x.z, -x.z);
        S.ps = make_float2(0.0f, 0.0f);
    } else {
        S.x = x.x;
        S.y = x.y;
        S.z = x.z;
        S.ps = 0.0;
    }
}

template <int G>
__device__ __forceinline__ void slot_init(const NearParams<double> &P, int tb, int te, int base, int lane,
                                          Slot<tf32x2> &S) {
    const int ti = tb + base + lane / G;
    S.ti = ti < te ? ti : -1;
    const double4 x = P.pts[ti < te ? ti : tb];
    S.x = tf_from_double(x.x);
    S.y = tf_from_double(x.y);
    S.z = tf_from_double(x.z);
    S.ps = tf32x2(0);
}

template <int G>
__device__ __forceinline__ void slot_finish(Slot<tf32x2> &S, int lane, int tb, double *pot) {
    tf32x2 a = S.ps;
#pragma unroll
    for (int o = 1; o < G; o <<= 1) a = a + tf_shfl_xor(a, o);
    if (lane % G == 0 && S.ti >= 0) pot[S.ti - tb] = tf_to_double(a);
}

template <typename T, int G>
__device__ __forceinline__ void slot_finish(Slot<T> &S, int lane, int tb, T *pot) {
    T a;
    if constexpr (sizeof(T) == 4)
        a = S.ps.x + S.ps.y;
    else
        a = S.ps;
#pragma unroll
    for (int o = 1; o < G; o <<= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane % G == 0 && S.ti >= 0) pot[S.ti - tb] = a;
}

template <typename T, bool SELF, typename C, typename E>
__device__ __forceinline__ void accumulate_slots(const C *chunk, int cnt, int sb, int lane, const bool (&on)[5],
                                                 Slot<T> (&S)[5], E eps2) {
    if (on[0]) accumulate_slot<1, SELF>(chunk, cnt, sb, 0, S[0], eps2);
    if (on[1]) accumulate_slot<1, SELF>(chunk, cnt, sb, 0, S[1], eps2);
    if (on[2]) accumulate_slot<2, SELF>(chunk, cnt, sb, lane % 2, S[2], eps2);
    if (on[3]) accumulate_slot<4, SELF>(chunk, cnt, sb, lane % 4, S[3], eps2);
    if (on[4]) accumulate_slot<8, SELF>(chunk, cnt, sb, lane % 8, S[4], eps2);
}

// Targets tb..te-1 (at most 64) of leaf t: near field by slots, then the
// local expansion and the epilogue with one lane per target.  Source chunks
// of up to 64 points (one leaf, or a 64-point piece of a larger one) are
// staged in shared memory (FP32 as x / y / z / q arrays, two-float as split
// points, FP64 as points).
// The leaf ids and ranges of the row are read 32 entries at a time (one per
// lane) and broadcast by shuffles, and the next chunk's points are loaded
// before the current chunk is computed, so the dependent global loads
// overlap the arithmetic.
struct SplitPt {  // two-float source point: (xh, xl, yh, yl), (zh, zl, qh, ql)
    float4 a, b;
};

template <typename T, bool TF>
__device__ __forceinline__ void leaf_slots(const NearParams<T> &P, int t, int tb, int te,
                                           typename Vec4<T>::type *sp, T *pot, const Cplx<T> *sL) {
    using T4 = typename Vec4<T>::type;
    using ST = std::conditional_t<TF, tf32x2, T>;      // slot arithmetic
    using Pre = std::conditional_t<TF, SplitPt, T4>;  // prefetched source point
    constexpr bool F32 = !TF && sizeof(T) == 4;
    const int lane = threadIdx.x & 31;
    const int nt = te - tb;
    bool on[5];
    int base[5];
    {
        int rem = (nt + 3) & ~3, o = 0;
        on[0] = rem >= 32;
        base[0] = o;
        if (on[0]) o += 32, rem -= 32;
        on[1] = rem >= 32;
        base[1] = o;
        if (on[1]) o += 32, rem -= 32;
        on[2] = (rem & 16) != 0;
        base[2] = o;
        if (on[2]) o += 16;
        on[3] = (rem & 8) != 0;
        base[3] = o;
        if (on[3]) o += 8;
        on[4] = (rem & 4) != 0;
        base[4] = o;
    }
    Slot<ST> S[5];
    if constexpr (TF) {
        slot_init<1>(P, tb, te, base[0], lane, S[0]);
        slot_init<1>(P, tb, te, base[1], lane, S[1]);
        slot_init<2>(P, tb, te, base[2], lane, S[2]);
        slot_init<4>(P, tb, te, base[3], lane, S[3]);
        slot_init<8>(P, tb, te, base[4], lane, S[4]);
    } else {
        slot_init<T, 1>(P, tb, te, base[0], lane, S[0]);
        slot_init<T, 1>(P, tb, te, base[1], lane, S[1]);
        slot_init<T, 2>(P, tb, te, base[2], lane, S[2]);
        slot_init<T, 4>(P, tb, te, base[3], lane, S[3]);
        slot_init<T, 8>(P, tb, te, base[4], lane, S[4]);
    }
    if (P.near) {
        const T eps2 = P.eps2;
        const int kbeg = P.off[t], kend = P.off[t + 1];
        int kb = kbeg, s_l = 0, sa_l = 0, se_l = 0;
        auto load_batch = [&](int b0) {
            kb = b0;
            const int k = b0 + lane;
            s_l = k < kend ? P.src[k] : 0;
            const int2 r = k < kend ? P.srange[s_l] : make_int2(0, 0);
            sa_l = r.x;
            se_l = r.y;
        };
        auto fetch = [&](int sb, int se, int i) -> Pre {
            if constexpr (TF) {
                if (i < se - sb) return SplitPt{P.spts_tf[2 * (sb + i)], P.spts_tf[2 * (sb + i) + 1]};
                return SplitPt{make_float4(0, 0, 0, 0), make_float4(0, 0, 0, 0)};
            } else {
                return i < se - sb ? P.spts[sb + i] : T4{0, 0, 0, 0};
            }
        };
        if (kbeg < kend) {
            load_batch(kbeg);
            int k = kbeg;
            int s = __shfl_sync(0xffffffffu, s_l, 0), sb = __shfl_sync(0xffffffffu, sa_l, 0),
                se = __shfl_sync(0xffffffffu, se_l, 0);
            Pre qa = fetch(sb, se, lane), qb = fetch(sb, se, lane + 32);
            while (true) {
                const int cs = s, csb = sb, cnt = min(64, se - sb);
                __syncwarp();
                if constexpr (TF) {
                    float4 *s4 = reinterpret_cast<float4 *>(sp);
                    s4[2 * lane] = qa.a;
                    s4[2 * lane + 1] = qa.b;
                    s4[2 * lane + 64] = qb.a;
                    s4[2 * lane + 65] = qb.b;
                } else if constexpr (F32) {
                    float *sx = reinterpret_cast<float *>(sp);
                    sx[lane] = qa.x;
                    sx[64 + lane] = qa.y;
                    sx[128 + lane] = qa.z;
                    sx[192 + lane] = qa.w;
                    sx[lane + 32] = qb.x;
                    sx[64 + lane + 32] = qb.y;
                    sx[128 + lane + 32] = qb.z;
                    sx[192 + lane + 32] = qb.w;
                } else {
                    sp[lane] = qa;
                    sp[lane + 32] = qb;
                }
                __syncwarp();
                bool more = true;
                if (sb + 64 < se) {
                    sb += 64;
                } else if (++k >= kend) {
                    more = false;
                } else {
                    if (k >= kb + 32) load_batch(k);
                    s = __shfl_sync(0xffffffffu, s_l, k - kb);
                    sb = __shfl_sync(0xffffffffu, sa_l, k - kb);
                    se = __shfl_sync(0xffffffffu, se_l, k - kb);
                }
                if (more) {
                    qa = fetch(sb, se, lane);
                    qb = fetch(sb, se, lane + 32);
                }
                if constexpr (TF) {
                    const float4 *s4 = reinterpret_cast<const float4 *>(sp);
                    if (P.same && cs == t)
                        accumulate_slots<tf32x2, true>(s4, cnt, csb, lane, on, S, (float)eps2);
                    else
                        accumulate_slots<tf32x2, false>(s4, cnt, csb, lane, on, S, (float)eps2);
                } else if constexpr (F32) {
                    const float *sx = reinterpret_cast<const float *>(sp);
                    if (P.same && cs == t)
                        accumulate_slots<T, true>(sx, cnt, csb, lane, on, S, eps2);
                    else
                        accumulate_slots<T, false>(sx, cnt, csb, lane, on, S, eps2);
                } else {
                    if (P.same && cs == t)
                        accumulate_slots<T, true>(sp, cnt, csb, lane, on, S, eps2);
                    else
                        accumulate_slots<T, false>(sp, cnt, csb, lane, on, S, eps2);
                }
                if (!more) break;
            }
        }
    }
    if constexpr (TF) {
        slot_finish<1>(S[0], lane, tb, pot);
        slot_finish<1>(S[1], lane, tb, pot);
        slot_finish<2>(S[2], lane, tb, pot);
        slot_finish<4>(S[3], lane, tb, pot);
        slot_finish<8>(S[4], lane, tb, pot);
    } else {
        slot_finish<T, 1>(S[0], lane, tb, pot);
        slot_finish<T, 1>(S[1], lane, tb, pot);
        slot_finish<T, 2>(S[2], lane, tb, pot);
        slot_finish<T, 4>(S[3], lane, tb, pot);
        slot_finish<T, 8>(S[4], lane, tb, pot);
    }
    __syncwarp();
    T4 c;
    T ia = (T)1;
    if (P.far) {
        c = P.center[t];
        ia = (T)1 / P.half[t].w;
    }
    for (int i = lane; i < nt; i += 32) {
        const int ti = tb + i;
        const T4 x = P.pts[ti];
        T v = P.near ? pot[i] : (T)0;
        if (P.add_in) v += P.add_in[ti];
        if (P.far) {
            if constexpr (TF)
                v += tf_to_double(l2p_point_tf(reinterpret_cast<const tf32x2c *>(sL), P.p,
                                               tf_from_double((x.x - c.x) * ia), tf_from_double((x.y - c.y) * ia),
                                               tf_from_double((x.z - c.z) * ia)));
            else
                v += l2p_point<T>(sL, P.p, (x.x - c.x) * ia, (x.y - c.y) * ia, (x.z - c.z) * ia);
        }
        if (P.scatter) {
            const int o = P.index_map[ti];
            v = v * P.k_e;
            if (P.self_int) v += P.self_int[o] * P.sigma[o] * P.areas[o];
            if (!isfinite(v)) v = (T)0;
            P.out[o] = v;
        } else {
            P.out[ti] = v;
        }
    }
    __syncwarp();
}

template <typename T, bool TF>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 6 : 4) k_p2p_l2p(const NearParams<T> P) {
    using T4 = typename Vec4<T>::type;
    __shared__ T4 sp[4][64];  // a staged chunk of up to 64 sources
    __shared__ Cplx<T> sL[4][ncoef(kPMax)];
    __shared__ T spot[4][64];  // the near-field sums of a block of targets
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t w = (int64_t)blockIdx.x * 4 + wl;
    if (w >= P.n_leaves) return;
    const int t = P.leaves[w];
    if (!inst_active(P.mask, t)) return;  // uniform over the warp; the kernel has no block barrier
    if (P.far) {
        const int nc = ncoef(P.p);
        for (int k = lane; k < nc; k += 32) {
            const Cplx<T> c = P.Lexp[(int64_t)t * P.nc_pad + k];
            if constexpr (TF)  // staged as two-float (the same 16 bytes per coefficient)
                reinterpret_cast<tf32x2c *>(sL[wl])[k] = tf32x2c{tf_from_double(c.re), tf_from_double(c.im)};
            else
                sL[wl][k] = c;
        }
        __syncwarp();
    }
    const int2 rg = P.range[t];
    for (int tb = rg.x; tb < rg.y; tb += 64)
        leaf_slots<T, TF>(P, t, tb, min(rg.y, tb + 64), sp[wl], spot[wl], sL[wl]);
}

}  // namespace

// 1 / ((n + m)(n - m)) tables (1 / n^2 at m = 0); __constant__ data lives in
// each device context, so every plan creation uploads it on its device.
int upload_tables() {
    float hf[kPMax + 1][kPMax + 1];
    double hd[kPMax + 1][kPMax + 1];
    for (int n = 0; n <= kPMax; ++n)
        for (int m = 0; m <= kPMax; ++m) {
            int d = (n + m) * (n - m);
            if (m == 0 && n > 0) d = n * n;
            hd[n][m] = d != 0 ? 1.0 / d : 0.0;
            hf[n][m] = (float)hd[n][m];
        }
    float2 ht[kPMax + 1][kPMax + 1];
    for (int n = 0; n <= kPMax; ++n)
        for (int m = 0; m <= kPMax; ++m) {
            ht[n][m].x = (float)hd[n][m];
            ht[n][m].y = (float)(hd[n][m] - (double)ht[n][m].x);
        }
    EDFMM_CUDA_TRY(cudaMemcpyToSymbol(c_rdiv_f, hf, sizeof(hf)));
    EDFMM_CUDA_TRY(cudaMemcpyToSymbol(c_rdiv_d, hd, sizeof(hd)));
    EDFMM_CUDA_TRY(cudaMemcpyToSymbol(c_rdiv_tf, ht, sizeof(ht)));
    return EDFMM_OK;
}

namespace {

template <typename T>
int near_impl(const DevTree &tree, const DevLists &lists, const FmmBuffers &buf, const NearArgs &a, cudaStream_t s) {
    using T4 = typename Vec4<T>::type;
    if (tree.n_leaves == 0) return EDFMM_OK;
    NearParams<T> P;
    P.leaves = lists.p2p_leaves.p ? dptr<int32_t>(lists.p2p_leaves) : dptr<int32_t>(tree.leaves);
    P.n_leaves = tree.n_leaves;
    P.off = dptr<int32_t>(lists.p2p_off);
    P.src = dptr<int32_t>(lists.p2p_src);
    P.pts = dptr<T4>(tree.pts);
    P.range = dptr<int2>(tree.range);
    P.spts = a.src_tree ? dptr<T4>(a.src_tree->pts) : P.pts;
    // two-float near field: an FP64 plan (one tree) whose split points exist
    const bool tf = sizeof(T) == 8 && !a.src_tree && buf.arith == EDFMM_ARITH_TWO_FLOAT && tree.pts_tf.p;
    P.spts_tf = tf ? dptr<float4>(tree.pts_tf) : nullptr;
    P.srange = a.src_tree ? dptr<int2>(a.src_tree->range) : P.range;
    P.same = a.src_tree ? 0 : 1;
    P.center = dptr<T4>(tree.center);
    P.half = dptr<T4>(tree.half);
    P.Lexp = dptr<Cplx<T>>(buf.locals);
    P.p = buf.p;
    P.nc_pad = buf.nc_pad;
    const T eps = sizeof(T) == 8 ? (T)DBL_EPSILON : (T)FLT_EPSILON;
    P.eps2 = eps * eps;
    P.near = a.near ? 1 : 0;
    P.far = a.far ? 1 : 0;
    P.add_in = static_cast<const T *>(a.add_in);
    P.mask = a.src_tree ? InstMask{} : buf.mask;
    P.scatter = a.scatter ? 1 : 0;
    P.index_map = dptr<int32_t>(tree.index_map);
    P.sigma = static_cast<const T *>(a.sigma);
    P.areas = static_cast<const T *>(a.areas);
    P.self_int = static_cast<const T *>(a.self_int);
    P.k_e = (T)a.k_e;
    P.out = static_cast<T *>(a.out);
    if constexpr (sizeof(T) == 8) {
        if (tf) {
            k_p2p_l2p<T, true><<<(unsigned)((tree.n_leaves + 3) / 4), 128, 0, s>>>(P);
            EDFMM_LAUNCH_CHECK("k_p2p_l2p (two-float)");
            return EDFMM_OK;
        }
    }
    k_p2p_l2p<T, false><<<(unsigned)((tree.n_leaves + 3) / 4), 128, 0, s>>>(P);
    EDFMM_LAUNCH_CHECK("k_p2p_l2p");
    return EDFMM_OK;
}

}  // namespace

int run_p2p_l2p(const DevTree &tree, const DevLists &lists, const FmmBuffers &buf, const NearArgs &args,
                cudaStream_t s) {
    return tree.dtype == EDFMM_F64 ? near_impl<double>(tree, lists, buf, args, s)
                                   : near_impl<float>(tree, lists, buf, args, s);
}

namespace {

// Gradient of the local expansion sum_{n,m} w_m Re(L_n^m R_n^m(x, y, z))
// (w_0 = 1, w_m = 2) in the node's scaled frame, from
//   d/dz R_n^m = R_{n-1}^m,  (d/dx + i d/dy) R_n^m = R_{n-1}^{m+1},
//   (d/dx - i d/dy) R_n^m = -R_{n-1}^{m-1}
// (negative orders through R^{-m} = (-1)^m conj(R^m)).
template <typename T>
__device__ void l2p_gradient(const Cplx<T> *L, int p, T x, T y, T z, T &gx, T &gy, T &gz) {
    Cplx<T> R[ncoef(kPMax - 1)];
    gx = gy = gz = (T)0;
    if (p < 1) return;
    regular_harmonics_rt<T>(x, y, z, p - 1, R);
    for (int n = 1; n <= p; ++n) {
        for (int m = 0; m <= n; ++m) {
            const Cplx<T> l = L[tri(n, m)];
            const Cplx<T> zero{(T)0, (T)0};
            const Cplx<T> dp = m + 1 <= n - 1 ? R[tri(n - 1, m + 1)] : zero;
            Cplx<T> dm = zero;
            if (m - 1 >= -(n - 1) && m - 1 <= n - 1) {
                const Cplx<T> h = harm_at<T>(R, n - 1, m - 1);
                dm = Cplx<T>{-h.re, -h.im};
            }
            const Cplx<T> dz = m <= n - 1 ? R[tri(n - 1, m)] : zero;
            const T w = m == 0 ? (T)1 : (T)2;
            const Cplx<T> sp = cmul(l, Cplx<T>{dp.re + dm.re, dp.im + dm.im});
            const Cplx<T> sm = cmul(l, Cplx<T>{dp.re - dm.re, dp.im - dm.im});
            gx += w * (T)0.5 * sp.re;
            gy += w * (T)0.5 * sm.im;
            gz += w * cmul(l, dz).re;
        }
    }
}

// Field at the points of a target tree from a source plan: one warp per
// target leaf, one lane per target.  Near part: sum_j q_j (x - y_j) / r^3
// over the leaf's P2P row (the gradient of the potential kernel
// q / max(r, eps), zero where r <= eps); far part: minus the gradient of the
// leaf's local expansion.  out[3 * index_map[i] + c] = k_e * E_c.
template <typename T>
__global__ void __launch_bounds__(128) k_targets_field(
    const int32_t *__restrict__ leaves, int64_t n_leaves, const int32_t *__restrict__ off,
    const int32_t *__restrict__ src, const typename Vec4<T>::type *__restrict__ pts, const int2 *__restrict__ range,
    const typename Vec4<T>::type *__restrict__ spts, const int2 *__restrict__ srange,
    const typename Vec4<T>::type *__restrict__ center, const typename Vec4<T>::type *__restrict__ half,
    const Cplx<T> *__restrict__ Lexp, int p, int nc_pad, T eps2, int near, int far,
    const int32_t *__restrict__ index_map, T k_e, T *__restrict__ out) {
    using T4 = typename Vec4<T>::type;
    __shared__ T4 sp[4][32];
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t w = (int64_t)blockIdx.x * 4 + wl;
    if (w >= n_leaves) return;
    const int t = leaves[w];
    const int2 rg = range[t];
    T4 c{};
    T ia = (T)1;
    if (far) {
        c = center[t];
        ia = (T)1 / half[t].w;
    }
    for (int tb = rg.x; tb < rg.y; tb += 32) {
        const int ti = tb + lane;
        const bool valid = ti < rg.y;
        const T4 x = pts[valid ? ti : rg.x];
        T ex = 0, ey = 0, ez = 0;
        if (near) {
            for (int k = off[t]; k < off[t + 1]; ++k) {
                const int2 sr = srange[src[k]];
                for (int sb = sr.x; sb < sr.y; sb += 32) {
                    const int cnt = min(32, sr.y - sb);
                    __syncwarp();
                    if (lane < cnt) sp[wl][lane] = spts[sb + lane];
                    __syncwarp();
                    for (int j = 0; j < cnt; ++j) {
                        const T4 q = sp[wl][j];
                        const T dx = x.x - q.x, dy = x.y - q.y, dz = x.z - q.z;
                        const T r2 = dx * dx + dy * dy + dz * dz;
                        if (r2 > eps2) {
                            const T ir = (T)1 / sqrt(r2);
                            const T wq = q.w * ir * ir * ir;
                            ex += wq * dx;
                            ey += wq * dy;
                            ez += wq * dz;
                        }
                    }
                }
            }
        }
        if (far && valid) {
            T gx, gy, gz;
            l2p_gradient<T>(Lexp + (int64_t)t * nc_pad, p, (x.x - c.x) * ia, (x.y - c.y) * ia, (x.z - c.z) * ia, gx, gy,
                            gz);
            ex -= gx * ia;
            ey -= gy * ia;
            ez -= gz * ia;
        }
        if (valid) {
            const int o = index_map[ti];
            out[3 * o] = k_e * ex;
            out[3 * o + 1] = k_e * ey;
            out[3 * o + 2] = k_e * ez;
        }
    }
}

template <typename T>
int field_impl(const DevTree &tree, const DevLists &lists, const FmmBuffers &buf, const DevTree &stree, double k_e,
               bool near, bool far, void *out, cudaStream_t s) {
    using T4 = typename Vec4<T>::type;
    if (tree.n_leaves == 0) return EDFMM_OK;
    const T eps = sizeof(T) == 8 ? (T)DBL_EPSILON : (T)FLT_EPSILON;
    k_targets_field<T><<<(unsigned)((tree.n_leaves + 3) / 4), 128, 0, s>>>(
        dptr<int32_t>(tree.leaves), tree.n_leaves, dptr<int32_t>(lists.p2p_off), dptr<int32_t>(lists.p2p_src),
        dptr<T4>(tree.pts), dptr<int2>(tree.range), dptr<T4>(stree.pts), dptr<int2>(stree.range),
        dptr<T4>(tree.center), dptr<T4>(tree.half), dptr<Cplx<T>>(buf.locals), buf.p, buf.nc_pad, eps * eps,
        near ? 1 : 0, far ? 1 : 0, dptr<int32_t>(tree.index_map), (T)k_e, static_cast<T *>(out));
    EDFMM_LAUNCH_CHECK("k_targets_field");
    return EDFMM_OK;
}

}  // namespace

int run_targets_field(const DevTree &tree, const DevLists &lists, const FmmBuffers &buf, const DevTree &stree,
                      double k_e, bool near, bool far, void *out, cudaStream_t s) {
    return tree.dtype == EDFMM_F64 ? field_impl<double>(tree, lists, buf, stree, k_e, near, far, out, s)
                                   : field_impl<float>(tree, lists, buf, stree, k_e, near, far, out, s);
}

}  // namespace edfmm
