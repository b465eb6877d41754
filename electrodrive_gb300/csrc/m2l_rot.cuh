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
#pragma once

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
// x * h + a on both halves
__device__ __forceinline__ float2 fma2(float2 x, float h, float2 a) { return __ffma2_rn(x, make_float2(h, h), a); }
__device__ __forceinline__ double2 fma2(double2 x, double h, double2 a) {
    return make_double2(fma(x.x, h, a.x), fma(x.y, h, a.y));
}

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

// forward rotation of degree n: scale by fn, R_z(+phi), Q_p, R_z(+theta), Q_m.
// BINOM: fn = c^n n! / rho^n (cr = c / rho); else fn = c^n (cr = c).
template <typename T, int P, bool BINOM, int n, typename V>
__device__ __forceinline__ void forward(V &v, T cr, T fn, const Frame<T, P> &F) {
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
    if constexpr (n < P) forward<T, P, BINOM, n + 1>(v, cr, BINOM ? fn * cr * T(n + 1) : fn * cr, F);
}

// backward rotation of degree n (transposes in reverse order), added to acc;
// BINOM: scaled by hn = n! / rho^(n+1) as it is added
template <typename T, int P, bool BINOM, int n, typename V, typename A>
__device__ __forceinline__ void backward(V &v, A &acc, const Frame<T, P> &F, T hn, T irho) {
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
        a.x = BINOM ? fma(b[0], hn, a.x) : a.x + b[0];
        acc.set(tri(n, 0), a);
    }
#pragma unroll
    for (int m = 1; m <= n; ++m) {
        T2 x;
        x.x = b[2 * m - 1];
        x.y = b[2 * m];
        acc.set(tri(n, m), BINOM ? fma2(x, hn, acc.get(tri(n, m))) : add2(acc.get(tri(n, m)), x));
    }
    if constexpr (n < P) backward<T, P, BINOM, n + 1>(v, acc, F, hn * T(n + 1) * irho, irho);
}

// The axial translation with the factor table f[j] = j! / rho^(j+1):
// L'_n^m = (-1)^(n+m) sum_{k=m..P} M'_k^m f[n+k], in place.  FP32 runs the
// complex (m >= 1) terms as packed pairs: f2[j] = (f[j], f[j]).
template <typename T, int P, int m, typename V>
__device__ __forceinline__ void axial_table(V &v, const T (&f)[2 * P + 1], const float2 (&f2)[2 * P + 1]) {
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
    if constexpr (m < P) axial_table<T, P, m + 1>(v, f, f2);
}

// The axial translation in binomial form (the FP32 kernel at p <= 7 and the
// two-float kernel; the FP32 kernel at p = 8 keeps the factor table, whose
// packed m >= 1 sums issue fewer instructions).  Along z,
//   L'_n^m = (-1)^(n+m) sum_{k=m..P} M'_k^m (n+k)! / rho^(n+k+1)
//          = h_n (-1)^(n+m) sum_k C(n+k, k) u_k^m,
// with u_k = M'_k k! / rho^k and h_n = n! / rho^(n+1).  The forward pass folds
// k! / rho^k into its scaling by c^k and the backward pass folds h_n into its
// accumulation, so the sums here have exact integer coefficients (at most
// C(16, 8) = 12,870), compile-time constants: no per-pair factor table.
__host__ __device__ constexpr double binom(int n, int k) {
    double r = 1.0;
    for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
    return r;
}

// s = sum_{k=K..P} C(N+k, k) u[k] (K = the first term: a product)
template <typename T, int P, int N, int K, bool FIRST>
__device__ __forceinline__ void binom_dot(const T (&u)[P + 1], T &s) {
    constexpr double cb = binom(N + K, K);
    if constexpr (std::is_same<T, tf32x2>::value) {
        if constexpr (FIRST) {  // u * cb, cb exact in FP32
            const tf32x2 pr = tf_two_prod(u[K].hi, (float)cb);
            s = tf_fast_two_sum(pr.hi, __fmaf_rn(u[K].lo, (float)cb, pr.lo));
        } else {
            s = tf_fma_const<true>((float)cb, 0.0f, u[K], s);
        }
    } else if constexpr (FIRST) {
        s = u[K] * (T)cb;
    } else {
        s = fma((T)cb, u[K], s);
    }
    if constexpr (K < P) binom_dot<T, P, N, K + 1, false>(u, s);
}

template <typename T, int P, int m, int N, bool SCALE_OUT>
__device__ __forceinline__ void binom_rows(const T (&ur)[P + 1], const T (&ui)[P + 1], T (&wr)[P + 1],
                                           T (&wi)[P + 1], const T (&h)[P + 1]) {
    T sr, si = T(0);
    binom_dot<T, P, N, m, true>(ur, sr);
    if constexpr (m > 0) binom_dot<T, P, N, m, true>(ui, si);
    if constexpr (SCALE_OUT) {
        sr = sr * h[N];
        if constexpr (m > 0) si = si * h[N];
    }
    wr[N] = ((N + m) & 1) ? -sr : sr;
    wi[N] = ((N + m) & 1) ? -si : si;
    if constexpr (N < P) binom_rows<T, P, m, N + 1, SCALE_OUT>(ur, ui, wr, wi, h);
}

// u -> (-1)^(n+m) sum_k C(n+k, k) u_k^m in place (times h_n when SCALE_OUT)
template <typename T, int P, int m, bool SCALE_OUT, typename V>
__device__ __forceinline__ void axial(V &v, const T (&h)[P + 1]) {
    T ur[P + 1], ui[P + 1], wr[P + 1], wi[P + 1];
#pragma unroll
    for (int k = m; k <= P; ++k) {
        ur[k] = v.get(k * k + (m == 0 ? 0 : 2 * m - 1));
        ui[k] = m == 0 ? T(0) : v.get(k * k + 2 * m);
    }
    binom_rows<T, P, m, m, SCALE_OUT>(ur, ui, wr, wi, h);
#pragma unroll
    for (int n = m; n <= P; ++n) {
        v.set(n * n + (m == 0 ? 0 : 2 * m - 1), wr[n]);
        if (m > 0) v.set(n * n + 2 * m, wi[n]);
    }
    if constexpr (m < P) axial<T, P, m + 1, SCALE_OUT>(v, h);
}

// Which axial form the FP32 / FP64 kernel of order P runs (measured on the
// GB300: binomial 2.05 against 2.14 ms per M2L at p = 6, table 3.59 against
// 3.82 ms at p = 8)
template <typename T, int P> __host__ __device__ constexpr bool rot_binomial() { return !(sizeof(T) == 4 && P >= 8); }

// One pair: translated locals of source s added to acc.
template <typename T, int P, typename V, typename A>
__device__ __forceinline__ void rot_pair(V &v, A &acc, const typename Vec2<T>::type *__restrict__ Mrow, T c, T dx, T dy,
                                         T dz) {
    // FP32 rows are read two coefficients per 16-byte load (rows of an even
    // number of coefficients, 16-byte aligned): half the scattered loads
    float4 x4{};
#pragma unroll
    for (int n = 0; n <= P; ++n) {
#pragma unroll
        for (int m = 0; m <= n; ++m) {
            const int q = tri(n, m);
            typename Vec2<T>::type x;
            if constexpr (sizeof(T) == 4) {
                if ((q & 1) == 0) {
                    x4 = reinterpret_cast<const float4 *>(Mrow)[q >> 1];
                    x = make_float2(x4.x, x4.y);
                } else {
                    x = make_float2(x4.z, x4.w);
                }
            } else {
                x = Mrow[q];
            }
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
    constexpr bool BINOM = rot_binomial<T, P>();
    forward<T, P, BINOM, 0>(v, BINOM ? c * irho : c, T(1), F);
    if constexpr (BINOM) {
        const T none[P + 1] = {};
        axial<T, P, 0, false>(v, none);
    } else {
        T f[2 * P + 1];
        f[0] = irho;
#pragma unroll
        for (int j = 1; j <= 2 * P; ++j) f[j] = f[j - 1] * (T)j * irho;
        float2 f2[2 * P + 1];
        if constexpr (sizeof(T) == 4) {
#pragma unroll
            for (int j = 0; j <= 2 * P; ++j) f2[j] = make_float2((float)f[j], (float)f[j]);
        }
        axial_table<T, P, 0>(v, f, f2);
    }
    backward<T, P, BINOM, 0>(v, acc, F, irho, irho);
}

// ---------------------------------------------------------------------------
// Packed layouts of the quarter-turn matrices.  In the real block basis each
// matrix of degree n is the direct sum of four dense blocks: an output
// coefficient reads only inputs of one class (real or imaginary part, m even
// or odd), and the four classes map to one another in pairs.  Pairing Re X_j
// with Im X_{j+1} (j = 0..n-1; Re X_n stays alone) puts two rows of
// different blocks into one packed FP32x2 operation whose operand is one
// input pair, for every input pair: 145 instead of 247 multiply-adds per
// matrix at p = 8, no cross terms.  Two layouts of a degree block are used:
//   RI: pair j = (Re X_j, Im X_{j+1});
//   XN: the same pairs with the halves swapped where j + n is odd;
// a forward matrix maps XN to RI, a backward one RI to XN.  The two-float
// kernel runs its matrices in this form (below).  (For the FP32 kernel the
// packed form measured slower: 4.43 against 3.59 ms per M2L at p = 8.)
// ---------------------------------------------------------------------------
__host__ __device__ constexpr int ix_re(int m) { return m == 0 ? 0 : 2 * m - 1; }

// block index of half h of pair j of a degree-n block in layout L (0: RI, 1: XN)
template <int n, int L>
__host__ __device__ constexpr int pk_ix(int j, int h) {
    return ((L == 1 && ((j + n) & 1)) ? 1 - h : h) == 0 ? ix_re(j) : 2 * (j + 1);
}

// matrix entry (a, c) of table TAB, degree n
template <int TAB, int n>
__host__ __device__ constexpr double pk_g(int a, int c) {
    return rot_entry<TAB>(kRotOff[n] + a * (2 * n + 1) + c);
}

// does input pair i < I hold a non-zero for row A (half x) or row B (half y)?
template <int TAB, int n, int LIN, int A, int B>
__host__ __device__ constexpr bool pk_started(int I) {
    for (int i = 0; i < I; ++i)
        if (pk_g<TAB, n>(A, pk_ix<n, LIN>(i, 0)) != 0.0 || pk_g<TAB, n>(B, pk_ix<n, LIN>(i, 1)) != 0.0) return true;
    return false;
}

// One warp per target row, one lane per (target, source) pair.  The warps of
// a block run the same number of rounds of pairs, with a barrier between
// rounds, so that the warps of an SM walk the long straight-line pair code
// close together and share its instruction fetches.
template <typename T, int P, bool V_IN_SMEM>
__global__ void __launch_bounds__(kRotThreads, sizeof(T) == 4 ? (rot_binomial<T, P>() ? 4 : 3) : 1)
    k_m2l_rot(int64_t n_nodes, const int32_t *__restrict__ off, const int32_t *__restrict__ src,
              const int32_t *__restrict__ rows,
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
    // warp w takes target row rows[w] (rows by decreasing pair count), or row w
    const int64_t w = ((int64_t)blockIdx.x * NT + threadIdx.x) >> 5;
    const int64_t t = rows && w < n_nodes ? (int64_t)rows[w] : w;
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

// --- the two-float matrices on packed FP32x2 instructions ---
// Two two-float values of the rows of one packed pair: (hi.x, lo.x) and
// (hi.y, lo.y).  Each operation is the scalar two-float one (twofloat.cuh)
// on both halves at once; negations are folded into the constants or taken
// as fma(b, -1, a) = a - b, which rounds exactly like the subtraction, so
// the results are bit-identical to the scalar two-float matrices.
struct tfp {
    float2 hi, lo;
};
__device__ __forceinline__ float2 f2_sub(float2 a, float2 b) {
    return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);
}
// x * g + c, g = (ghi + glo) per half; ng = -ghi, nglo = -glo (EXACT: glo = 0)
template <bool EXACT>
__device__ __forceinline__ tfp tfp_fma_const(float2 g, float2 ng, float2 nglo, const tfp &x, const tfp &c) {
    const float2 p = __fmul2_rn(x.hi, g);
    float2 ne = __ffma2_rn(x.hi, ng, p);  // -(x.hi g - p), the product's rounding error negated
    ne = __ffma2_rn(x.lo, ng, ne);        // -(error + x.lo g)
    if constexpr (!EXACT) ne = __ffma2_rn(x.hi, nglo, ne);
    const float2 s = __fadd2_rn(p, c.hi);  // two-sum of p and c.hi
    const float2 bb = f2_sub(s, p);
    const float2 es = __fadd2_rn(f2_sub(p, f2_sub(s, bb)), f2_sub(c.hi, bb));
    const float2 t = __fadd2_rn(es, f2_sub(c.lo, ne));
    const float2 h = __fadd2_rn(s, t);  // fast two-sum
    return tfp{h, f2_sub(t, f2_sub(h, s))};
}
// x * g (the first term of a row: the fma above with c = 0)
template <bool EXACT>
__device__ __forceinline__ tfp tfp_mul_const(float2 g, float2 ng, float2 nglo, const tfp &x) {
    const float2 p = __fmul2_rn(x.hi, g);
    float2 ne = __ffma2_rn(x.hi, ng, p);
    ne = __ffma2_rn(x.lo, ng, ne);
    if constexpr (!EXACT) ne = __ffma2_rn(x.hi, nglo, ne);
    const float2 h = f2_sub(p, ne);
    return tfp{h, f2_sub(f2_sub(p, h), ne)};
}

template <int n> struct PkT {  // one degree block of two-float values in a packed layout
    tfp p[n > 0 ? n : 1];
    tf32x2 r;  // Re X_n
};
template <int n, int L, int J>
__device__ __forceinline__ tf32x2 pkt_get(const PkT<n> &v) {
    if constexpr (J == ix_re(n)) {
        return v.r;
    } else {
        constexpr bool re = J == 0 || (J & 1);
        constexpr int j = re ? (J + 1) >> 1 : J / 2 - 1;
        constexpr bool y = re == (L == 1 && ((j + n) & 1));
        if constexpr (y) return tf32x2(v.p[j].hi.y, v.p[j].lo.y);
        else return tf32x2(v.p[j].hi.x, v.p[j].lo.x);
    }
}
template <int n, int L, int J>
__device__ __forceinline__ void pkt_set(PkT<n> &v, tf32x2 a) {
    if constexpr (J == ix_re(n)) {
        v.r = a;
    } else {
        constexpr bool re = J == 0 || (J & 1);
        constexpr int j = re ? (J + 1) >> 1 : J / 2 - 1;
        constexpr bool y = re == (L == 1 && ((j + n) & 1));
        if constexpr (y) {
            v.p[j].hi.y = a.hi;
            v.p[j].lo.y = a.lo;
        } else {
            v.p[j].hi.x = a.hi;
            v.p[j].lo.x = a.lo;
        }
    }
}

__host__ __device__ constexpr float tf_hi(double g) { return (float)g; }
__host__ __device__ constexpr float tf_lo(double g) { return (float)(g - (double)(float)g); }

template <int TAB, int n, int LIN, int A, int B, int I>
__device__ __forceinline__ void pkt_rows(const PkT<n> &x, tfp &acc) {
    if constexpr (I < n) {
        constexpr int C = pk_ix<n, LIN>(I, 0), D = pk_ix<n, LIN>(I, 1);
        constexpr double ga = pk_g<TAB, n>(A, C), gb = pk_g<TAB, n>(B, D);
        static_assert(pk_g<TAB, n>(A, D) == 0.0 && pk_g<TAB, n>(B, C) == 0.0,
                      "packed rotation layouts must leave no cross terms");
        if constexpr (ga != 0.0 || gb != 0.0) {
            constexpr bool exact = tf_lo(ga) == 0.0f && tf_lo(gb) == 0.0f;
            const float2 g = make_float2(tf_hi(ga), tf_hi(gb)), ng = make_float2(-tf_hi(ga), -tf_hi(gb));
            const float2 nglo = make_float2(-tf_lo(ga), -tf_lo(gb));
            if constexpr (pk_started<TAB, n, LIN, A, B>(I)) acc = tfp_fma_const<exact>(g, ng, nglo, x.p[I], acc);
            else acc = tfp_mul_const<exact>(g, ng, nglo, x.p[I]);
        }
        pkt_rows<TAB, n, LIN, A, B, I + 1>(x, acc);
    }
}

template <int TAB, int n, int LIN, int I, bool STARTED>
__device__ __forceinline__ void pkt_left_row(const PkT<n> &x, tf32x2 &acc) {
    constexpr int L = ix_re(n);
    if constexpr (I < n) {
        constexpr double ga = pk_g<TAB, n>(L, pk_ix<n, LIN>(I, 0));
        constexpr double gb = pk_g<TAB, n>(L, pk_ix<n, LIN>(I, 1));
        static_assert(ga == 0.0 || gb == 0.0, "one input class per row");
        if constexpr (ga != 0.0) {
            const tf32x2 v(x.p[I].hi.x, x.p[I].lo.x);
            acc = tf_fma_const<tf_lo(ga) == 0.0f>(tf_hi(ga), tf_lo(ga), v, STARTED ? acc : tf32x2(0.0f, 0.0f));
        }
        if constexpr (gb != 0.0) {
            const tf32x2 v(x.p[I].hi.y, x.p[I].lo.y);
            acc = tf_fma_const<tf_lo(gb) == 0.0f>(tf_hi(gb), tf_lo(gb), v, STARTED ? acc : tf32x2(0.0f, 0.0f));
        }
        pkt_left_row<TAB, n, LIN, I + 1, STARTED || ga != 0.0 || gb != 0.0>(x, acc);
    } else {
        constexpr double g = pk_g<TAB, n>(L, L);
        if constexpr (g != 0.0)
            acc = tf_fma_const<tf_lo(g) == 0.0f>(tf_hi(g), tf_lo(g), x.r, STARTED ? acc : tf32x2(0.0f, 0.0f));
        else if constexpr (!STARTED)
            acc = tf32x2(0.0f, 0.0f);
    }
}

template <int TAB, int n, int LIN, int LOUT, int J>
__device__ __forceinline__ void pkt_out_pairs(const PkT<n> &x, PkT<n> &y) {
    if constexpr (J < n) {
        constexpr int A = pk_ix<n, LOUT>(J, 0), B = pk_ix<n, LOUT>(J, 1), L = ix_re(n);
        constexpr double la = pk_g<TAB, n>(A, L), lb = pk_g<TAB, n>(B, L);
        tfp acc{make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f)};
        if constexpr (pk_started<TAB, n, LIN, A, B>(n)) pkt_rows<TAB, n, LIN, A, B, 0>(x, acc);
        if constexpr (la != 0.0) {
            const tf32x2 r = tf_fma_const<tf_lo(la) == 0.0f>(tf_hi(la), tf_lo(la), x.r, tf32x2(acc.hi.x, acc.lo.x));
            acc.hi.x = r.hi;
            acc.lo.x = r.lo;
        }
        if constexpr (lb != 0.0) {
            const tf32x2 r = tf_fma_const<tf_lo(lb) == 0.0f>(tf_hi(lb), tf_lo(lb), x.r, tf32x2(acc.hi.y, acc.lo.y));
            acc.hi.y = r.hi;
            acc.lo.y = r.lo;
        }
        y.p[J] = acc;
        pkt_out_pairs<TAB, n, LIN, LOUT, J + 1>(x, y);
    }
}

template <int TAB, int n, int LIN, int LOUT>
__device__ __forceinline__ void pkt_apply(const PkT<n> &x, PkT<n> &y) {
    pkt_out_pairs<TAB, n, LIN, LOUT, 0>(x, y);
    pkt_left_row<TAB, n, LIN, 0, false>(x, y.r);
}

// X_m <- X_m e^{+-i m a} in two-float, x in layout LA, y in layout LB
template <int n, int LA, int LB, int P, int m>
__device__ __forceinline__ void pkt_zrot(const PkT<n> &x, PkT<n> &y, const tf32x2 (&c)[P + 1],
                                         const tf32x2 (&s)[P + 1], bool neg) {
    if constexpr (m == 0) {
        pkt_set<n, LB, 0>(y, pkt_get<n, LA, 0>(x));
    } else {
        const tf32x2 re = pkt_get<n, LA, 2 * m - 1>(x), im = pkt_get<n, LA, 2 * m>(x), cm = c[m];
        const tf32x2 sm = neg ? -s[m] : s[m];
        pkt_set<n, LB, 2 * m - 1>(y, re * cm - im * sm);
        pkt_set<n, LB, 2 * m>(y, re * sm + im * cm);
    }
    if constexpr (m < n) pkt_zrot<n, LA, LB, P, m + 1>(x, y, c, s, neg);
}

// all 2n + 1 values of a packed block to / from the slots of v (block index order)
template <int n, int L, int J, typename V>
__device__ __forceinline__ void pkt_store(V &v, const PkT<n> &x) {
    v.set(n * n + J, pkt_get<n, L, J>(x));
    if constexpr (J < 2 * n) pkt_store<n, L, J + 1>(v, x);
}
template <int n, int L, int J, typename V>
__device__ __forceinline__ void pkt_load(const V &v, PkT<n> &x) {
    pkt_set<n, L, J>(x, v.get(n * n + J));
    if constexpr (J < 2 * n) pkt_load<n, L, J + 1>(v, x);
}

// forward of degree n on the slots of v: scale by fn = c^n n! / rho^n,
// R_z(+phi), Q_p, R_z(+theta), Q_m
template <int P, int n, typename V>
__device__ __forceinline__ void forward_tf_pk(V &v, tf32x2 cr, tf32x2 fn, const Frame<tf32x2, P> &F) {
    constexpr int OV = n * n;
    PkT<n> a, b;
    pkt_set<n, 0, 0>(b, v.get(OV) * fn);
#pragma unroll
    for (int m = 1; m <= n; ++m) {
        // scaled row into layout RI (compile-time indices after unrolling)
        const tf32x2 re = v.get(OV + 2 * m - 1) * fn, im = v.get(OV + 2 * m) * fn;
        if (m < n) {
            b.p[m].hi.x = re.hi;
            b.p[m].lo.x = re.lo;
        } else {
            b.r = re;
        }
        b.p[m - 1].hi.y = im.hi;
        b.p[m - 1].lo.y = im.lo;
    }
    pkt_zrot<n, 0, 1, P, 0>(b, a, F.cp, F.sp, false);
    pkt_apply<0, n, 1, 0>(a, b);
    pkt_zrot<n, 0, 1, P, 0>(b, a, F.ct, F.st, false);
    pkt_apply<1, n, 1, 0>(a, b);
    pkt_store<n, 0, 0>(v, b);
    if constexpr (n < P) forward_tf_pk<P, n + 1>(v, cr, fn * cr * tf32x2(n + 1), F);
}

// backward of degree n on the slots of v (transposes in reverse order)
template <int P, int n, typename V>
__device__ __forceinline__ void backward_tf_pk(V &v, const Frame<tf32x2, P> &F) {
    PkT<n> a, b;
    pkt_load<n, 0, 0>(v, a);
    pkt_apply<3, n, 0, 1>(a, b);
    pkt_zrot<n, 1, 0, P, 0>(b, a, F.ct, F.st, true);
    pkt_apply<2, n, 0, 1>(a, b);
    pkt_zrot<n, 1, 0, P, 0>(b, a, F.cp, F.sp, true);
    pkt_store<n, 0, 0>(v, a);
    if constexpr (n < P) backward_tf_pk<P, n + 1>(v, F);
}

// two-float slots split into a hi and a lo array (slot i of this thread at
// [i * STRIDE]), so that single values load straight into packed pairs
template <int STRIDE> struct SmemSplit {
    float *hi, *lo;
    __device__ __forceinline__ tf32x2 get(int i) const {
        return tf32x2(lds_keep(hi + i * STRIDE), lds_keep(lo + i * STRIDE));
    }
    __device__ __forceinline__ void set(int i, tf32x2 x) {
        sts_keep(hi + i * STRIDE, x.hi);
        sts_keep(lo + i * STRIDE, x.lo);
    }
};

// One pair: v <- the translated locals (real block basis) of source row Mrow
// (split multipoles: (re hi, re lo, im hi, im lo) per coefficient).
template <int P, bool PK, typename V>
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
    const T cr = c * irho;
    if constexpr (PK) forward_tf_pk<P, 0>(v, cr, T(1), F);
    else forward<T, P, true, 0>(v, cr, T(1), F);
    T h[P + 1];
    h[0] = irho;
#pragma unroll
    for (int j = 1; j <= P; ++j) h[j] = h[j - 1] * T(j) * irho;
    axial<T, P, 0, true>(v, h);
    if constexpr (PK) backward_tf_pk<P, 0>(v, F);
    else backward_tf<P, 0>(v, F);
}

// tnodes / snodes: per node (cx hi, cx lo, cy hi, cy lo), (cz hi, cz lo, a hi, a lo).
// NT = 128 (two blocks per SM) or 256 (one block of 8 warps per SM: one
// instruction-fetch stream per SM for the long pair code).  PK: the four
// matrices on packed FP32x2 instructions, with the slots split into hi and
// lo arrays (the same shared memory).
template <int P, int NT, bool PK>
__global__ void __launch_bounds__(NT, 256 / NT)
    k_m2l_rot_tf(int64_t n_nodes, const int32_t *__restrict__ off, const int32_t *__restrict__ src,
                 const int32_t *__restrict__ rows,
                 const float4 *__restrict__ tnodes, const double4 *__restrict__ thalf,
                 const float4 *__restrict__ snodes, const double4 *__restrict__ half,
                 const float4 *__restrict__ Mexp, double2 *__restrict__ Lexp, int nc_pad, const InstMask mask) {
    using T = tf32x2;
    constexpr int NV = (P + 1) * (P + 1), NR = (NV + 31) / 32;
    extern __shared__ __align__(16) unsigned char rot_smem[];
    __shared__ int max_rounds;
    T *slots = reinterpret_cast<T *>(rot_smem);  // slot i of thread u at slots[i * NT + u]
    float *slots_hi = reinterpret_cast<float *>(rot_smem), *slots_lo = slots_hi + NV * NT;  // PK
    using VS = typename std::conditional<PK, SmemSplit<NT>, SmemV<T, NT>>::type;
    VS v;
    if constexpr (PK) v = VS{slots_hi + threadIdx.x, slots_lo + threadIdx.x};
    else v = VS{slots + threadIdx.x};
    // warp w takes target row rows[w] (rows by decreasing pair count), or row w
    const int64_t w = ((int64_t)blockIdx.x * NT + threadIdx.x) >> 5;
    const int64_t t = rows && w < n_nodes ? (int64_t)rows[w] : w;
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
                rot_pair_tf<P, PK>(v, Mexp + (int64_t)s * nc_pad, T(w.z, w.w) * iaT, (ctx - T(u.x, u.y)) * iaT,
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
                if constexpr (PK) {
                    const float *rh = slots_hi + i * NT + wbase, *rl = slots_lo + i * NT + wbase;
#pragma unroll 8
                    for (int l = 0; l < 32; ++l) {
                        const int o = (l + lane) & 31;
                        sum = sum + T(lds_keep(rh + o), lds_keep(rl + o));
                    }
                } else {
                    const T *row = slots + i * NT + wbase;
#pragma unroll 8
                    for (int l = 0; l < 32; ++l) sum = sum + lds_keep(row + ((l + lane) & 31));
                }
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

template <int P, int NT, bool PK>
int launch_rot_tf(int64_t M, const int32_t *off, const int32_t *src, const int32_t *rows, const void *tnodes,
                  const void *thal,
                  const void *snodes, const void *hal, const void *Mx, void *Lx, int nc_pad, const InstMask &mask,
                  cudaStream_t s) {
    constexpr int NV = (P + 1) * (P + 1);
    constexpr size_t smem = (size_t)NV * NT * sizeof(tf32x2);
    static const cudaError_t attr =
        cudaFuncSetAttribute(k_m2l_rot_tf<P, NT, PK>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (attr != cudaSuccess)
        return fail(EDFMM_ERR_CUDA, std::string("k_m2l_rot_tf shared memory attribute: ") + cudaGetErrorString(attr));
    k_m2l_rot_tf<P, NT, PK><<<nblk(M * 32, NT), NT, smem, s>>>(
        M, off, src, rows, static_cast<const float4 *>(tnodes), static_cast<const double4 *>(thal),
        static_cast<const float4 *>(snodes), static_cast<const double4 *>(hal), static_cast<const float4 *>(Mx),
        static_cast<double2 *>(Lx), nc_pad, mask);
    EDFMM_LAUNCH_CHECK("k_m2l_rot_tf");
    return EDFMM_OK;
}

template <typename T, int P, bool V_IN_SMEM>
int launch_rot(int64_t M, const int32_t *off, const int32_t *src, const int32_t *rows, const void *tcen,
               const void *thal, const void *cen,
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
        M, off, src, rows, static_cast<const T4 *>(tcen), static_cast<const T4 *>(thal), static_cast<const T4 *>(cen),
        static_cast<const T4 *>(hal), static_cast<const T2 *>(Mx), static_cast<T2 *>(Lx), nc_pad, mask);
    EDFMM_LAUNCH_CHECK("k_m2l_rot");
    return EDFMM_OK;
}

}  // namespace

// Entry points of the translation units that instantiate the kernels (they
// compile in parallel): FP32 and FP64 orders 1..8 (m2l_rot_f32.cu,
// m2l_rot_f64.cu; a..d = target centres, target halves, source centres,
// source halves) and two-float orders 6, 7 and 8 with 128 or 256 threads
// (m2l_rot_tf*.cu; a..d = target nodes, target halves, source nodes, source
// halves).
int m2l_rot_f32(int p, int64_t M, const int32_t *off, const int32_t *src, const int32_t *rows, const void *a, const void *b,
                const void *c, const void *d, const void *Mx, void *Lx, int nc_pad, const InstMask &mask,
                cudaStream_t s);
int m2l_rot_f64(int p, int64_t M, const int32_t *off, const int32_t *src, const int32_t *rows, const void *a, const void *b,
                const void *c, const void *d, const void *Mx, void *Lx, int nc_pad, const InstMask &mask,
                cudaStream_t s);
int m2l_rot_tf6(bool packed, int64_t M, const int32_t *off, const int32_t *src, const int32_t *rows, const void *a, const void *b,
                const void *c, const void *d, const void *Mx, void *Lx, int nc_pad, const InstMask &mask,
                cudaStream_t s);
int m2l_rot_tf7(bool packed, int64_t M, const int32_t *off, const int32_t *src, const int32_t *rows, const void *a, const void *b,
                const void *c, const void *d, const void *Mx, void *Lx, int nc_pad, const InstMask &mask,
                cudaStream_t s);
int m2l_rot_tf8(bool packed, int64_t M, const int32_t *off, const int32_t *src, const int32_t *rows, const void *a, const void *b,
                const void *c, const void *d, const void *Mx, void *Lx, int nc_pad, const InstMask &mask,
                cudaStream_t s);
int m2l_rot_tf8w(bool packed, int64_t M, const int32_t *off, const int32_t *src, const int32_t *rows, const void *a, const void *b,
                const void *c, const void *d, const void *Mx, void *Lx, int nc_pad, const InstMask &mask,
                cudaStream_t s);

}  // namespace edfmm
