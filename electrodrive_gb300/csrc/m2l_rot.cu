// Rotation-based M2L ("point and shoot").
//
// With d = (c_L - c_M) / a_L at polar angle theta and azimuth phi, rotate the
// frame so that d lies on +z, translate along z, rotate back:
//   M' = conj T(Q) M,   L' = axial(M', |d|),   L = T(Q)^T L',
//   Q = R_y(-theta) R_z(-phi),
// where T(Q) maps the solid harmonics under the rotation,
// R_n^m(Q v) = sum_m' T^n_{m m'}(Q) R_n^m'(v).  A z rotation is diagonal
// (e^{i m a}), and a y rotation is R_y(b) = Q_m R_z(b) Q_p with the fixed
// quarter turns Q_p, Q_m about x.  Their exact matrices (rotation_tables.h,
// real block basis [Re X0, Re X1, Im X1, ...] per degree, about 25% non-zero)
// are compile-time constants, so the zero entries cost nothing.  Along z,
// I_j^mu(0, 0, rho) = delta_mu0 j! / rho^(j+1), so
//   L'_n^m = (-1)^(n+m) sum_{k >= m} M'_k^m (n+k)! / rho^(n+k+1).
// Per pair this is about 2,300 multiply-adds at p = 8, against 7,300 for the
// azimuth-factored contraction.  One lane per (target, source) pair, one
// warp per target row; each lane accumulates its translated locals in
// private shared-memory slots, reduced over the warp at the end (fixed order).
#include <type_traits>

#include "edfmm_internal.cuh"
#include "harmonics.cuh"
#include "rotation_tables.h"
#include "twofloat.cuh"

namespace edfmm {
namespace {

constexpr float kRotExtremeRatio = 256.0f;  // FP32: beyond this (a_M/a_L)^k may overflow
constexpr int kRotThreads = 128;             // 4 warps; FP32: 3 blocks per SM at <= 168 registers

template <int TAB> __host__ __device__ constexpr double rot_entry(int i) {
    return TAB == 0 ? kRotFwdP[i] : TAB == 1 ? kRotFwdM[i] : TAB == 2 ? kRotBwdP[i] : kRotBwdM[i];
}

// y[I] = sum_J G[I][J] x[J] over the non-zero entries of table TAB, degree block at OFF
template <typename T, int TAB, int N, int OFF, int I, int J>
__device__ __forceinline__ void rot_dot(const T (&x)[N], T &acc) {
    constexpr double g = rot_entry<TAB>(OFF + I * N + J);
    if constexpr (g != 0.0) {
        if constexpr (std::is_same<T, tf32x2>::value) {
            // the table entries are dyadic rationals: nearly all exact in FP32
            constexpr float ghi = (float)g;
            constexpr float glo = (float)(g - (double)ghi);
            acc = tf_fma_const<glo == 0.0f>(ghi, glo, x[J], acc);
        } else {
            acc = fma((T)g, x[J], acc);
        }
    }
    if constexpr (J + 1 < N) rot_dot<T, TAB, N, OFF, I, J + 1>(x, acc);
}
template <typename T, int TAB, int N, int OFF, int I>
__device__ __forceinline__ void rot_apply(const T (&x)[N], T (&y)[N]) {
    T acc = T(0);
    rot_dot<T, TAB, N, OFF, I, 0>(x, acc);
    y[I] = acc;
    if constexpr (I + 1 < N) rot_apply<T, TAB, N, OFF, I + 1>(x, y);
}

// X_m <- X_m e^{i m a} on a degree block: (c[m], s[m]) = (cos m a, sin m a)
template <typename T, int N, int P>
__device__ __forceinline__ void zrot(T (&b)[N], const T (&c)[P + 1], const T (&s)[P + 1], T sign) {
#pragma unroll
    for (int m = 1; 2 * m < N; ++m) {
        const T re = b[2 * m - 1], im = b[2 * m], cm = c[m], sm = sign * s[m];
        b[2 * m - 1] = re * cm - im * sm;
        b[2 * m] = re * sm + im * cm;
    }
}

template <typename T, int P> struct Frame {
    T cp[P + 1], sp[P + 1];  // cos / sin (m phi)
    T ct[P + 1], st[P + 1];  // cos / sin (m theta)
};

template <typename T, int P>
__device__ __forceinline__ void powers(T c, T s, T (&cm)[P + 1], T (&sm)[P + 1]) {
    cm[0] = T(1);
    sm[0] = T(0);
#pragma unroll
    for (int m = 1; m <= P; ++m) {
        cm[m] = cm[m - 1] * c - sm[m - 1] * s;
        sm[m] = cm[m - 1] * s + sm[m - 1] * c;
    }
}

// register store of the (P+1)^2 real coefficients, or private shared-memory slots
template <typename T, int NV> struct RegV {
    T v[NV];
    __device__ __forceinline__ T get(int i) const { return v[i]; }
    __device__ __forceinline__ void set(int i, T x) { v[i] = x; }
};
// Shared-memory loads the compiler may not hoist or merge, so the FP64 kernel
// re-reads each coefficient where it is used instead of keeping them all in
// registers (FP64 FMAs are the cost there; shared-memory traffic is free).
__device__ __forceinline__ float lds_keep(const float *p) {
    float v;
    asm volatile("ld.volatile.shared.f32 %0, [%1];" : "=f"(v) : "r"((unsigned)__cvta_generic_to_shared(p)));
    return v;
}
__device__ __forceinline__ double lds_keep(const double *p) {
    double v;
    asm volatile("ld.volatile.shared.f64 %0, [%1];" : "=d"(v) : "r"((unsigned)__cvta_generic_to_shared(p)));
    return v;
}
// The matching stores are volatile too: volatile accesses keep their program
// order, which a plain store next to an asm load would not be guaranteed.
__device__ __forceinline__ void sts_keep(float *p, float v) {
    asm volatile("st.volatile.shared.f32 [%0], %1;" ::"r"((unsigned)__cvta_generic_to_shared(p)), "f"(v));
}
__device__ __forceinline__ void sts_keep(double *p, double v) {
    asm volatile("st.volatile.shared.f64 [%0], %1;" ::"r"((unsigned)__cvta_generic_to_shared(p)), "d"(v));
}
__device__ __forceinline__ tf32x2 lds_keep(const tf32x2 *p) {
    tf32x2 v;
    asm volatile("ld.volatile.shared.v2.f32 {%0, %1}, [%2];"
                 : "=f"(v.hi), "=f"(v.lo)
                 : "r"((unsigned)__cvta_generic_to_shared(p)));
    return v;
}
__device__ __forceinline__ void sts_keep(tf32x2 *p, tf32x2 v) {
    asm volatile("st.volatile.shared.v2.f32 [%0], {%1, %2};" ::"r"((unsigned)__cvta_generic_to_shared(p)), "f"(v.hi),
                 "f"(v.lo));
}
template <typename T, int STRIDE> struct SmemV {
    T *base;  // this lane's slot 0; slot i at base[i * STRIDE]
    __device__ __forceinline__ T get(int i) const { return lds_keep(base + i * STRIDE); }
    __device__ __forceinline__ void set(int i, T x) { sts_keep(base + i * STRIDE, x); }
};

template <typename T> struct Vec2 {};
template <> struct Vec2<float> { using type = float2; };
template <> struct Vec2<double> { using type = double2; };

__device__ __forceinline__ float2 lds_keep(const float2 *p) {
    float2 v;
    asm volatile("ld.volatile.shared.v2.f32 {%0, %1}, [%2];"
                 : "=f"(v.x), "=f"(v.y)
                 : "r"((unsigned)__cvta_generic_to_shared(p)));
    return v;
}
__device__ __forceinline__ double2 lds_keep(const double2 *p) {
    double2 v;
    asm volatile("ld.volatile.shared.v2.f64 {%0, %1}, [%2];"
                 : "=d"(v.x), "=d"(v.y)
                 : "r"((unsigned)__cvta_generic_to_shared(p)));
    return v;
}
__device__ __forceinline__ void sts_keep(float2 *p, float2 v) {
    asm volatile("st.volatile.shared.v2.f32 [%0], {%1, %2};" ::"r"((unsigned)__cvta_generic_to_shared(p)), "f"(v.x),
                 "f"(v.y));
}
__device__ __forceinline__ void sts_keep(double2 *p, double2 v) {
    asm volatile("st.volatile.shared.v2.f64 [%0], {%1, %2};" ::"r"((unsigned)__cvta_generic_to_shared(p)), "d"(v.x),
                 "d"(v.y));
}
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ double2 add2(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }

// Per-lane accumulator of the translated locals: complex slot tri(n, m) at
// base[tri(n, m) * STRIDE] (one 8- or 16-byte word per lane, so a warp's
// access is conflict-free and each coefficient pair is one load and one store).
// FP32 uses plain accesses (the compiler keeps the slots in shared memory at
// 167 registers; volatile stores measured 5% slower); FP64 uses volatile ones
// so that its 45 complex slots are not pulled into registers.
template <typename T, int STRIDE> struct AccC {
    using T2 = typename Vec2<T>::type;
    T2 *base;
    __device__ __forceinline__ T2 get(int q) const {
        if constexpr (sizeof(T) == 8)
            return lds_keep(base + q * STRIDE);
        else
            return base[q * STRIDE];
    }
    __device__ __forceinline__ void set(int q, T2 x) {
        if constexpr (sizeof(T) == 8)
            sts_keep(base + q * STRIDE, x);
        else
            base[q * STRIDE] = x;
    }
};

// forward rotation of degree n: scale by f^n, R_z(+phi), Q_p, R_z(+theta), Q_m
template <typename T, int P, int n, typename V>
__device__ __forceinline__ void forward(V &v, T f, T fn, const Frame<T, P> &F) {
    constexpr int N = 2 * n + 1, OV = n * n, OFF = kRotOff[n];
    T b[N], o[N];
#pragma unroll
    for (int i = 0; i < N; ++i) b[i] = v.get(OV + i) * fn;
    zrot<T, N, P>(b, F.cp, F.sp, T(1));
    rot_apply<T, 0, N, OFF, 0>(b, o);
    zrot<T, N, P>(o, F.ct, F.st, T(1));
    rot_apply<T, 1, N, OFF, 0>(o, b);
#pragma unroll
    for (int i = 0; i < N; ++i) v.set(OV + i, b[i]);
    if constexpr (n < P) forward<T, P, n + 1>(v, f, fn * f, F);
}

// backward rotation of degree n (transposes in reverse order), added to acc
template <typename T, int P, int n, typename V, typename A>
__device__ __forceinline__ void backward(V &v, A &acc, const Frame<T, P> &F) {
    constexpr int N = 2 * n + 1, OV = n * n, OFF = kRotOff[n];
    T b[N], o[N];
#pragma unroll
    for (int i = 0; i < N; ++i) b[i] = v.get(OV + i);
    rot_apply<T, 3, N, OFF, 0>(b, o);
    zrot<T, N, P>(o, F.ct, F.st, T(-1));
    rot_apply<T, 2, N, OFF, 0>(o, b);
    zrot<T, N, P>(b, F.cp, F.sp, T(-1));
    using T2 = typename Vec2<T>::type;
    {
        T2 a = acc.get(tri(n, 0));
        a.x += b[0];
        acc.set(tri(n, 0), a);
    }
#pragma unroll
    for (int m = 1; m <= n; ++m) {
        T2 x;
        x.x = b[2 * m - 1];
        x.y = b[2 * m];
        acc.set(tri(n, m), add2(acc.get(tri(n, m)), x));
    }
    if constexpr (n < P) backward<T, P, n + 1>(v, acc, F);
}

// L'_n^m = (-1)^(n+m) sum_{k=m..P} M'_k^m (n+k)! / rho^(n+k+1), in place.
// FP32 runs the complex (m >= 1) terms as packed pairs: f2[j] = (f[j], f[j]).
template <typename T, int P, int m, typename V>
__device__ __forceinline__ void axial(V &v, const T (&f)[2 * P + 1], const float2 (&f2)[2 * P + 1]) {
    if constexpr (m > 0 && sizeof(T) == 4) {
        float2 u[P + 1];
#pragma unroll
        for (int k = m; k <= P; ++k) u[k] = make_float2(v.get(k * k + 2 * m - 1), v.get(k * k + 2 * m));
#pragma unroll
        for (int n = m; n <= P; ++n) {
            float2 sum = make_float2(0.0f, 0.0f);
#pragma unroll
            for (int k = m; k <= P; ++k) sum = __ffma2_rn(u[k], f2[n + k], sum);
            const float sg = ((n + m) & 1) ? -1.0f : 1.0f;
            v.set(n * n + 2 * m - 1, sg * sum.x);
            v.set(n * n + 2 * m, sg * sum.y);
        }
    } else {
        T ur[P + 1], ui[P + 1], wr[P + 1], wi[P + 1];
#pragma unroll
        for (int k = m; k <= P; ++k) {
            ur[k] = v.get(k * k + (m == 0 ? 0 : 2 * m - 1));
            ui[k] = m == 0 ? T(0) : v.get(k * k + 2 * m);
        }
#pragma unroll
        for (int n = m; n <= P; ++n) {
            T sr = T(0), si = T(0);
#pragma unroll
            for (int k = m; k <= P; ++k) {
                sr = fma(ur[k], f[n + k], sr);
                if (m > 0) si = fma(ui[k], f[n + k], si);
            }
            wr[n] = ((n + m) & 1) ? -sr : sr;
            wi[n] = ((n + m) & 1) ? -si : si;
        }
#pragma unroll
        for (int n = m; n <= P; ++n) {
            v.set(n * n + (m == 0 ? 0 : 2 * m - 1), wr[n]);
            if (m > 0) v.set(n * n + 2 * m, wi[n]);
        }
    }
    if constexpr (m < P) axial<T, P, m + 1>(v, f, f2);
}

// One pair: translated locals of source s added to acc.
template <typename T, int P, typename V, typename A>
__device__ __forceinline__ void rot_pair(V &v, A &acc, const typename Vec2<T>::type *__restrict__ Mrow, T c, T dx, T dy,
                                         T dz) {
#pragma unroll
    for (int n = 0; n <= P; ++n) {
#pragma unroll
        for (int m = 0; m <= n; ++m) {
            const typename Vec2<T>::type x = Mrow[tri(n, m)];
            if (m == 0) {
                v.set(n * n, x.x);
            } else {
                v.set(n * n + 2 * m - 1, x.x);
                v.set(n * n + 2 * m, x.y);
            }
        }
    }
    const T s2 = dx * dx + dy * dy, r2 = s2 + dz * dz;
    const T s = sqrt(s2), rho = sqrt(r2), irho = T(1) / rho;
    Frame<T, P> F;
    T cphi = T(1), sphi = T(0);
    if (s2 > T(0)) {
        const T is = T(1) / s;
        cphi = dx * is;
        sphi = dy * is;
    }
    powers<T, P>(cphi, sphi, F.cp, F.sp);
    powers<T, P>(dz * irho, s * irho, F.ct, F.st);
    forward<T, P, 0>(v, c, T(1), F);
    T f[2 * P + 1];
    f[0] = irho;
#pragma unroll
    for (int j = 1; j <= 2 * P; ++j) f[j] = f[j - 1] * (T)j * irho;
    float2 f2[2 * P + 1];
    if constexpr (sizeof(T) == 4) {
#pragma unroll
        for (int j = 0; j <= 2 * P; ++j) f2[j] = make_float2((float)f[j], (float)f[j]);
    }
    axial<T, P, 0>(v, f, f2);
    backward<T, P, 0>(v, acc, F);
}

// One warp per target row, one lane per (target, source) pair.  The warps of
// a block run the same number of rounds of pairs, with a barrier between
// rounds, so that the warps of an SM walk the long straight-line pair code
// close together and share its instruction fetches.
template <typename T, int P, bool V_IN_SMEM>
__global__ void __launch_bounds__(kRotThreads, sizeof(T) == 4 ? 3 : 1)
    k_m2l_rot(int64_t n_nodes, const int32_t *__restrict__ off, const int32_t *__restrict__ src,
              const typename Vec4<T>::type *__restrict__ tcenter, const typename Vec4<T>::type *__restrict__ thalf,
              const typename Vec4<T>::type *__restrict__ center, const typename Vec4<T>::type *__restrict__ half,
              const typename Vec2<T>::type *__restrict__ Mexp, typename Vec2<T>::type *__restrict__ Lexp,
              int nc_pad, const InstMask mask) {
    using T2 = typename Vec2<T>::type;
    constexpr int NV = (P + 1) * (P + 1), NQ = (P + 1) * (P + 2) / 2, NT = kRotThreads;
    extern __shared__ __align__(16) unsigned char rot_smem[];
    __shared__ int max_rounds;
    T2 *sq = reinterpret_cast<T2 *>(rot_smem);
    AccC<T, NT> acc{sq + threadIdx.x};
    const int64_t t = ((int64_t)blockIdx.x * NT + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const bool live = t < n_nodes && inst_active(mask, (int)t);
    typename Vec4<T>::type ct{};
    T iaL = T(1);
    int b = 0, e = 0;
    if (live) {
        ct = tcenter[t];
        iaL = T(1) / thalf[t].w;
        b = off[t];
        e = off[t + 1];
    }
#pragma unroll
    for (int q = 0; q < NQ; ++q) acc.set(q, T2{});
    if (threadIdx.x == 0) max_rounds = 0;
    __syncthreads();
    if (lane == 0) atomicMax(&max_rounds, (e - b + 31) >> 5);
    __syncthreads();
    const int rounds = max_rounds;
    for (int r = 0; r < rounds; ++r) {
        __syncthreads();
        const int k = b + r * 32 + lane;
        if (k >= e) continue;
        const int s = __ldg(src + k);
        const typename Vec4<T>::type cs = center[s];
        const T c = half[s].w * iaL;
        if (sizeof(T) == 4 && c > (T)kRotExtremeRatio) continue;  // translated by k_m2l_generic
        const T2 *Mrow = Mexp + (int64_t)s * nc_pad;
        if constexpr (V_IN_SMEM) {
            SmemV<T, NT> v{reinterpret_cast<T *>(sq + NQ * NT) + threadIdx.x};
            rot_pair<T, P>(v, acc, Mrow, c, (ct.x - cs.x) * iaL, (ct.y - cs.y) * iaL, (ct.z - cs.z) * iaL);
        } else {
            RegV<T, NV> v;
            rot_pair<T, P>(v, acc, Mrow, c, (ct.x - cs.x) * iaL, (ct.y - cs.y) * iaL, (ct.z - cs.z) * iaL);
        }
    }
    if (!live) return;
    T2 *out = Lexp + t * nc_pad;
#pragma unroll
    for (int n = 0; n <= P; ++n) {
#pragma unroll
        for (int m = 0; m <= n; ++m) {
            const int q = tri(n, m);
            const T2 a = acc.get(q);
            T re = a.x, im = a.y;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                re += __shfl_xor_sync(0xffffffffu, re, o);
                im += __shfl_xor_sync(0xffffffffu, im, o);
            }
            if ((q & 31) == lane) {
                T2 r;
                r.x = re * iaL;
                r.y = im * iaL;
                out[q] = r;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Two-float M2L for FP64 plans.  The same rotation algorithm on the FP32 pipe
// in two-float arithmetic (about 48 significant bits; twofloat.cuh).  The
// source multipoles and the node geometry arrive already split into (hi, lo)
// FP32 pairs (split once per node, not once per pair: a pair-time split
// costs hundreds of FP64-pipe conversions), the pair geometry is formed in
// two-float, and the locals are written back as FP64.  Each lane's
// translated locals go back into its own coefficient slots (81 two-float
// values at p = 8), and after every round of 32 pairs the warp adds the
// slots of its lanes, lane i owning coefficients i, i + 32, i + 64 in
// registers; so a block needs 81 KB of shared memory and two blocks share an
// SM (the FP64 kernel's per-lane accumulators allow one).  Pairs whose source
// scale exceeds 256x the target's are left to the caller (FP32 exponent
// range), as in the FP32 kernel.
// ---------------------------------------------------------------------------
template <int P, int n, typename V>
__device__ __forceinline__ void backward_tf(V &v, const Frame<tf32x2, P> &F) {
    constexpr int N = 2 * n + 1, OV = n * n, OFF = kRotOff[n];
    tf32x2 b[N], o[N];
#pragma unroll
    for (int i = 0; i < N; ++i) b[i] = v.get(OV + i);
    rot_apply<tf32x2, 3, N, OFF, 0>(b, o);
    zrot<tf32x2, N, P>(o, F.ct, F.st, tf32x2(-1));
    rot_apply<tf32x2, 2, N, OFF, 0>(o, b);
    zrot<tf32x2, N, P>(b, F.cp, F.sp, tf32x2(-1));
#pragma unroll
    for (int i = 0; i < N; ++i) v.set(OV + i, b[i]);
    if constexpr (n < P) backward_tf<P, n + 1>(v, F);
}

// One pair: v <- the translated locals (real block basis) of source row Mrow
// (split multipoles: (re hi, re lo, im hi, im lo) per coefficient).
template <int P, typename V>
__device__ __forceinline__ void rot_pair_tf(V &v, const float4 *__restrict__ Mrow, tf32x2 c, tf32x2 dx, tf32x2 dy,
                                            tf32x2 dz) {
    using T = tf32x2;
#pragma unroll
    for (int n = 0; n <= P; ++n) {
#pragma unroll
        for (int m = 0; m <= n; ++m) {
            const float4 x = Mrow[tri(n, m)];
            if (m == 0) {
                v.set(n * n, T(x.x, x.y));
            } else {
                v.set(n * n + 2 * m - 1, T(x.x, x.y));
                v.set(n * n + 2 * m, T(x.z, x.w));
            }
        }
    }
    const T s2 = fma(dy, dy, dx * dx), r2 = fma(dz, dz, s2);
    const T s = sqrt(s2), rho = sqrt(r2), irho = tf_recip(rho);
    Frame<T, P> F;
    T cphi = T(1), sphi = T(0);
    if (s2.hi > 0.0f) {
        const T is = tf_recip(s);
        cphi = dx * is;
        sphi = dy * is;
    }
    powers<T, P>(cphi, sphi, F.cp, F.sp);
    powers<T, P>(dz * irho, s * irho, F.ct, F.st);
    forward<T, P, 0>(v, c, T(1), F);
    T f[2 * P + 1];
    f[0] = irho;
#pragma unroll
    for (int j = 1; j <= 2 * P; ++j) f[j] = f[j - 1] * T(j) * irho;
    float2 f2[2 * P + 1];
    axial<T, P, 0>(v, f, f2);
    backward_tf<P, 0>(v, F);
}

// tnodes / snodes: per node (cx hi, cx lo, cy hi, cy lo), (cz hi, cz lo, a hi, a lo).
// NT = 128 (two blocks per SM) or 256 (one block of 8 warps per SM: one
// instruction-fetch stream per SM for the long pair code).
template <int P, int NT>
__global__ void __launch_bounds__(NT, 256 / NT)
    k_m2l_rot_tf(int64_t n_nodes, const int32_t *__restrict__ off, const int32_t *__restrict__ src,
                 const float4 *__restrict__ tnodes, const double4 *__restrict__ thalf,
                 const float4 *__restrict__ snodes, const double4 *__restrict__ half,
                 const float4 *__restrict__ Mexp, double2 *__restrict__ Lexp, int nc_pad, const InstMask mask) {
    using T = tf32x2;
    constexpr int NV = (P + 1) * (P + 1), NR = (NV + 31) / 32;
    extern __shared__ __align__(16) unsigned char rot_smem[];
    __shared__ int max_rounds;
    T *slots = reinterpret_cast<T *>(rot_smem);  // slot i of thread u at slots[i * NT + u]
    SmemV<T, NT> v{slots + threadIdx.x};
    const int64_t t = ((int64_t)blockIdx.x * NT + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int wbase = threadIdx.x & ~31;
    const bool live = t < n_nodes && inst_active(mask, (int)t);
    T ctx = T(0), cty = T(0), ctz = T(0), iaT = T(1);
    double iaL = 1.0;  // FP64, for the extreme-pair test (the same test as the pair lists of the FP64 kernel)
    int b = 0, e = 0;
    if (live) {
        const float4 u = tnodes[2 * t], w = tnodes[2 * t + 1];
        ctx = T(u.x, u.y);
        cty = T(u.z, u.w);
        ctz = T(w.x, w.y);
        iaT = tf_recip(T(w.z, w.w));
        iaL = 1.0 / thalf[t].w;
        b = off[t];
        e = off[t + 1];
    }
    T acc[NR];
#pragma unroll
    for (int j = 0; j < NR; ++j) acc[j] = T(0);
    if (threadIdx.x == 0) max_rounds = 0;
    __syncthreads();
    if (lane == 0) atomicMax(&max_rounds, (e - b + 31) >> 5);
    __syncthreads();
    const int rounds = max_rounds;
    for (int r = 0; r < rounds; ++r) {
        // the block's warps walk the (long, straight-line) pair code together
        // and share its instruction fetches; every thread runs `rounds` rounds
        __syncthreads();
        const int k = b + r * 32 + lane;
        bool have = false;
        if (k < e) {
            const int s = __ldg(src + k);
            if (!(half[s].w * iaL > (double)kRotExtremeRatio)) {
                have = true;
                const float4 u = snodes[2 * s], w = snodes[2 * s + 1];
                rot_pair_tf<P>(v, Mexp + (int64_t)s * nc_pad, T(w.z, w.w) * iaT, (ctx - T(u.x, u.y)) * iaT,
                               (cty - T(u.z, u.w)) * iaT, (ctz - T(w.x, w.y)) * iaT);
            }
        }
        if (!have) {
#pragma unroll
            for (int i = 0; i < NV; ++i) v.set(i, T(0));
        }
        __syncwarp();
        // coefficient i = lane + 32 j summed over the warp's lanes, starting at
        // this lane (conflict-free shared-memory reads; a fixed order per i)
#pragma unroll
        for (int j = 0; j < NR; ++j) {
            const int i = lane + 32 * j;
            if (i < NV) {
                T sum = acc[j];
                const T *row = slots + i * NT + wbase;
#pragma unroll 8
                for (int l = 0; l < 32; ++l) sum = sum + lds_keep(row + ((l + lane) & 31));
                acc[j] = sum;
            }
        }
        __syncwarp();
    }
    if (!live) return;
    double *out = reinterpret_cast<double *>(Lexp + t * nc_pad);
#pragma unroll
    for (int j = 0; j < NR; ++j) {
        const int i = lane + 32 * j;
        if (i < NV) {
            int n = 0;
            while ((n + 1) * (n + 1) <= i) ++n;
            const int q = i - n * n;  // 0: Re X0; 2m - 1: Re Xm; 2m: Im Xm
            const double val = tf_to_double(acc[j] * iaT);
            if (q == 0) {
                out[2 * tri(n, 0)] = val;
                out[2 * tri(n, 0) + 1] = 0.0;
            } else {
                out[2 * tri(n, (q + 1) >> 1) + ((q & 1) ? 0 : 1)] = val;
            }
        }
    }
}

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

template <int P, int NT>
int launch_rot_tf(int64_t M, const int32_t *off, const int32_t *src, const void *tnodes, const void *thal,
                  const void *snodes, const void *hal, const void *Mx, void *Lx, int nc_pad, const InstMask &mask,
                  cudaStream_t s) {
    constexpr int NV = (P + 1) * (P + 1);
    constexpr size_t smem = (size_t)NV * NT * sizeof(tf32x2);
    static const cudaError_t attr =
        cudaFuncSetAttribute(k_m2l_rot_tf<P, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (attr != cudaSuccess)
        return fail(EDFMM_ERR_CUDA, std::string("k_m2l_rot_tf shared memory attribute: ") + cudaGetErrorString(attr));
    k_m2l_rot_tf<P, NT><<<nblk(M * 32, NT), NT, smem, s>>>(
        M, off, src, static_cast<const float4 *>(tnodes), static_cast<const double4 *>(thal),
        static_cast<const float4 *>(snodes), static_cast<const double4 *>(hal), static_cast<const float4 *>(Mx),
        static_cast<double2 *>(Lx), nc_pad, mask);
    EDFMM_LAUNCH_CHECK("k_m2l_rot_tf");
    return EDFMM_OK;
}

template <typename T, int P, bool V_IN_SMEM>
int launch_rot(int64_t M, const int32_t *off, const int32_t *src, const void *tcen, const void *thal, const void *cen,
               const void *hal, const void *Mx, void *Lx, int nc_pad, const InstMask &mask, cudaStream_t s) {
    using T4 = typename Vec4<T>::type;
    using T2 = typename Vec2<T>::type;
    constexpr int NV = (P + 1) * (P + 1), NQ = (P + 1) * (P + 2) / 2, NT = kRotThreads;
    constexpr size_t smem = (size_t)NQ * NT * sizeof(T2) + (V_IN_SMEM ? (size_t)NV * NT * sizeof(T) : 0);
    static const cudaError_t attr =
        cudaFuncSetAttribute(k_m2l_rot<T, P, V_IN_SMEM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (attr != cudaSuccess)
        return fail(EDFMM_ERR_CUDA, std::string("k_m2l_rot shared memory attribute: ") + cudaGetErrorString(attr));
    k_m2l_rot<T, P, V_IN_SMEM><<<nblk(M * 32, NT), NT, smem, s>>>(
        M, off, src, static_cast<const T4 *>(tcen), static_cast<const T4 *>(thal), static_cast<const T4 *>(cen),
        static_cast<const T4 *>(hal), static_cast<const T2 *>(Mx), static_cast<T2 *>(Lx), nc_pad, mask);
    EDFMM_LAUNCH_CHECK("k_m2l_rot");
    return EDFMM_OK;
}

}  // namespace

// Rotation-based M2L for expansion orders 1..8 (FP32: pairs with a source
// scale above 256x the target's are left to the caller's generic kernel).
// Rows of instances inactive under ``mask`` are skipped (their locals are
// left as they were).
int launch_m2l_rot(int dtype, int p, int64_t M, const int32_t *off, const int32_t *src, const void *tcen,
                   const void *thal, const void *cen, const void *hal, const void *Mx, void *Lx, int nc_pad,
                   const InstMask &mask, cudaStream_t s) {
    if (M <= 0) return EDFMM_OK;
#define EDFMM_ROT_CASE(PP)                                                                                    \
    case PP:                                                                                                  \
        return dtype == EDFMM_F64                                                                             \
                   ? launch_rot<double, PP, true>(M, off, src, tcen, thal, cen, hal, Mx, Lx, nc_pad, mask, s) \
                   : launch_rot<float, PP, false>(M, off, src, tcen, thal, cen, hal, Mx, Lx, nc_pad, mask, s);
    switch (p) {
        EDFMM_ROT_CASE(1)
        EDFMM_ROT_CASE(2)
        EDFMM_ROT_CASE(3)
        EDFMM_ROT_CASE(4)
        EDFMM_ROT_CASE(5)
        EDFMM_ROT_CASE(6)
        EDFMM_ROT_CASE(7)
        EDFMM_ROT_CASE(8)
        default:
            return fail(EDFMM_ERR_UNSUPPORTED, "rotation M2L supports orders 1..8");
    }
#undef EDFMM_ROT_CASE
}

// Two-float M2L of an FP64 plan (orders 6..8); returns EDFMM_ERR_UNSUPPORTED
// for other orders (the caller then runs the FP64 kernel).
int launch_m2l_rot_tf(int p, int64_t M, const int32_t *off, const int32_t *src, const void *tnodes, const void *thal,
                      const void *snodes, const void *hal, const void *Mx, void *Lx, int nc_pad, const InstMask &mask,
                      int block, cudaStream_t s) {
    if (M <= 0) return EDFMM_OK;
    if (p == 8 && block == 256)
        return launch_rot_tf<8, 256>(M, off, src, tnodes, thal, snodes, hal, Mx, Lx, nc_pad, mask, s);
    switch (p) {
        case 6: return launch_rot_tf<6, 128>(M, off, src, tnodes, thal, snodes, hal, Mx, Lx, nc_pad, mask, s);
        case 7: return launch_rot_tf<7, 128>(M, off, src, tnodes, thal, snodes, hal, Mx, Lx, nc_pad, mask, s);
        case 8: return launch_rot_tf<8, 128>(M, off, src, tnodes, thal, snodes, hal, Mx, Lx, nc_pad, mask, s);
        default: return EDFMM_ERR_UNSUPPORTED;
    }
}

}  // namespace edfmm
