// Far-field stages of the FMM: P2M, M2M, M2L, L2L.
//
// Coefficients are stored per node as (p+1)(p+2)/2 complex numbers (m >= 0),
// scaled by the node's expansion radius a (the tight-box radius, but at least
// 1/8 of the parent's a and 2^-40 of the root radius):
//   Mhat_n^m = M_n^m / a^n,  Lhat_n^m = L_n^m a^n.
// This keeps every coefficient O(1) in FP32 at any tree depth.
//
// M2L (the dominant stage) is organised so that one lane owns one
// (target, source) pair at a time and keeps the whole translation in
// registers: the source multipole (scaled by (a_M/a_L)^k), the accumulator
// for the 45 target coefficients (p = 8) and one column of irregular
// harmonics of v = (c_L - c_M) / a_L, generated by recurrence.  A warp walks
// one target's row of the interaction list; the 32 partial sums are reduced
// with shuffles, so the result is deterministic.  With this scaling
//   Lhat_n^m = (-1)^(n+m) / a_L  sum_pairs sum_{k,l} Mhat_k^l (a_M/a_L)^k I_{n+k}^{l-m}(v),
// which is exact algebra; pairs whose source scale exceeds 256x the target's
// (only in strongly adaptive trees) would overflow (a_M/a_L)^k in FP32 and are
// instead translated by a shared-memory kernel using
//   Lhat_n^m = (-1)^(n+m) / a_L  (a_L/a_M)^(n+1) sum_{k,l} Mhat_k^l I_{n+k}^{l-m}((c_L - c_M)/a_M).
// FP64 plans (p <= 8) translate every pair with an FP64 form of the fast
// kernel; orders above 8 use the shared-memory kernel.
#include <algorithm>

#include "edfmm_internal.cuh"
#include "harmonics.cuh"
#include "twofloat.cuh"

namespace edfmm {

namespace {

constexpr float kExtremeRatio = 256.0f;
constexpr int kRotPMaxUsed = 8;  // rotation-based M2L (m2l_rot.cuh) for p <= 8

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

__device__ __forceinline__ void coef_nm(int c, int &n, int &m) {
    n = 0;
    while ((n + 1) * (n + 2) / 2 <= c) ++n;
    m = c - n * (n + 1) / 2;
}

// ---------------------------------------------------------------------------
// charges
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_set_charges(typename Vec4<T>::type *pts, const int32_t *__restrict__ idx, int64_t n,
                              const T *__restrict__ a, const T *__restrict__ b) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int o = idx[i];
    pts[i].w = b ? a[o] * b[o] : a[o];
}

// two-float mode: node geometry (cx, cy, cz, a) and FP64 complex
// coefficients split into (hi, lo) FP32 pairs
__global__ void k_split_nodes(const double4 *__restrict__ center, const double4 *__restrict__ half, int64_t n,
                              float4 *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double4 c = center[i];
    const tf32x2 x = tf_from_double(c.x), y = tf_from_double(c.y), z = tf_from_double(c.z),
                 a = tf_from_double(half[i].w);
    out[2 * i] = make_float4(x.hi, x.lo, y.hi, y.lo);
    out[2 * i + 1] = make_float4(z.hi, z.lo, a.hi, a.lo);
}
__global__ void k_split_coeffs(const double2 *__restrict__ in, int64_t n, float4 *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double2 c = in[i];
    const tf32x2 re = tf_from_double(c.x), im = tf_from_double(c.y);
    out[i] = make_float4(re.hi, re.lo, im.hi, im.lo);
}

// FP64 trees in two-float mode: the charges as above (a == NULL keeps them)
// and every point split into (hi, lo) FP32 pairs, 8 floats per point
__global__ void k_set_charges_split(double4 *pts, float4 *pts_tf, const int32_t *__restrict__ idx, int64_t n,
                                    const double *__restrict__ a, const double *__restrict__ b) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double4 x = pts[i];
    if (a) {
        const int o = idx[i];
        x.w = b ? a[o] * b[o] : a[o];
        pts[i].w = x.w;
    }
    const tf32x2 sx = tf_from_double(x.x), sy = tf_from_double(x.y), sz = tf_from_double(x.z),
                 sq = tf_from_double(x.w);
    pts_tf[2 * i] = make_float4(sx.hi, sx.lo, sy.hi, sy.lo);
    pts_tf[2 * i + 1] = make_float4(sz.hi, sz.lo, sq.hi, sq.lo);
}

// ---------------------------------------------------------------------------
// P2M: warp per leaf, lanes over points
// ---------------------------------------------------------------------------
template <typename T, int P>
__global__ void __launch_bounds__(128) k_p2m(const int32_t *__restrict__ leaves, int64_t n_leaves,
                                             const typename Vec4<T>::type *__restrict__ pts,
                                             const typename Vec4<T>::type *__restrict__ center,
                                             const typename Vec4<T>::type *__restrict__ half, const int2 *range,
                                             Cplx<T> *Mexp, int nc_pad) {
    constexpr int NC = ncoef(P);
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= n_leaves) return;
    const int leaf = leaves[w];
    const typename Vec4<T>::type c = center[leaf];
    const T ia = (T)1 / half[leaf].w;
    const int2 rg = range[leaf];
    T accr[NC], acci[NC];
#pragma unroll
    for (int k = 0; k < NC; ++k) accr[k] = acci[k] = (T)0;
    for (int i = rg.x + lane; i < rg.y; i += 32) {
        const typename Vec4<T>::type p = pts[i];
        T Rr[NC], Ri[NC];
        regular_harmonics<T, P>((p.x - c.x) * ia, (p.y - c.y) * ia, (p.z - c.z) * ia, Rr, Ri);
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            accr[k] += p.w * Rr[k];
            acci[k] -= p.w * Ri[k];
        }
    }
#pragma unroll
    for (int k = 0; k < NC; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            accr[k] += __shfl_xor_sync(0xffffffffu, accr[k], o);
            acci[k] += __shfl_xor_sync(0xffffffffu, acci[k], o);
        }
    }
    Cplx<T> *out = Mexp + (int64_t)leaf * nc_pad;
#pragma unroll
    for (int k = 0; k < NC; ++k)
        if ((k & 31) == lane) out[k] = Cplx<T>{accr[k], acci[k]};
}

// ---------------------------------------------------------------------------
// M2M: warp per internal node of one level, lanes over output coefficients
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(128) k_m2m(const int32_t *__restrict__ nodes, int n_nodes,
                                             const uint8_t *__restrict__ is_leaf, const int32_t *__restrict__ children,
                                             const typename Vec4<T>::type *__restrict__ center,
                                             const typename Vec4<T>::type *__restrict__ half, Cplx<T> *Mexp, int p,
                                             int nc_pad) {
    __shared__ Cplx<T> sR[4][ncoef(kPMax)], sM[4][ncoef(kPMax)];
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = blockIdx.x * 4 + wl;
    if (w >= n_nodes) return;
    const int node = nodes[w];
    if (is_leaf[node]) return;
    const int nc = ncoef(p);
    const typename Vec4<T>::type cp = center[node];
    const T aP = half[node].w, iaP = (T)1 / aP;
    Cplx<T> acc[3] = {{0, 0}, {0, 0}, {0, 0}};
    for (int o = 0; o < 8; ++o) {
        const int ch = children[8 * node + o];
        if (ch < 0) continue;
        const typename Vec4<T>::type cc = center[ch];
        const T ratio = half[ch].w * iaP;
        if (lane == 0) regular_harmonics_rt<T>((cc.x - cp.x) * iaP, (cc.y - cp.y) * iaP, (cc.z - cp.z) * iaP, p, sR[wl]);
        for (int k = lane; k < nc; k += 32) {
            int n, m;
            coef_nm(k, n, m);
            T sc = (T)1;
            for (int e = 0; e < n; ++e) sc *= ratio;
            Cplx<T> v = Mexp[(int64_t)ch * nc_pad + k];
            sM[wl][k] = Cplx<T>{v.re * sc, v.im * sc};
        }
        __syncwarp();
        for (int q = 0; q < 3; ++q) {
            const int k = lane + 32 * q;
            if (k >= nc) break;
            int n, m;
            coef_nm(k, n, m);
            Cplx<T> a = acc[q];
            for (int kk = 0; kk <= n; ++kk) {
                const int j = n - kk;
                for (int l = -kk; l <= kk; ++l) {
                    const int u = m - l;
                    if (u < -j || u > j) continue;
                    Cplx<T> r = harm_at(sR[wl], kk, l);
                    Cplx<T> mm = harm_at(sM[wl], j, u);
                    // conj(r) * mm
                    a.re += r.re * mm.re + r.im * mm.im;
                    a.im += r.re * mm.im - r.im * mm.re;
                }
            }
            acc[q] = a;
        }
        __syncwarp();
    }
    for (int q = 0; q < 3; ++q) {
        const int k = lane + 32 * q;
        if (k < nc) Mexp[(int64_t)node * nc_pad + k] = acc[q];
    }
}

// ---------------------------------------------------------------------------
// pair helpers: (sr, si) += (xr, xi) * (c0, c1) on coefficients held in
// separate re / im arrays; FP32 as one packed FMA (FFMA2), FP64 as two
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
template <typename T> struct Pair {};
template <> struct Pair<float> { using type = float2; };
template <> struct Pair<double> { using type = double2; };
__device__ __forceinline__ float2 mk2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ double2 mk2(double a, double b) { return make_double2(a, b); }
__device__ __forceinline__ void fma2_into(float &sr, float &si, float xr, float xi, float2 c) {
    const float2 r = __ffma2_rn(f2(xr, xi), c, f2(sr, si));
    sr = r.x;
    si = r.y;
}
__device__ __forceinline__ void fma2_into(double &sr, double &si, double xr, double xi, double2 c) {
    sr = fma(xr, c.x, sr);
    si = fma(xi, c.y, si);
}

// FP64 coefficient arrays in the thread's shared-memory slots (element i at
// b[i * STRIDE]: one word per thread per coefficient, conflict-free): the
// 180 doubles of a translation do not fit in registers.  Elements are read
// and written with volatile shared-memory accesses, which the compiler keeps
// in program order and may neither hoist into registers nor merge, so the
// arrays stay in shared memory (FP64 FMAs are the cost here, not the loads).
__device__ __forceinline__ double lds_vol(const double *p) {
    double v;
    asm volatile("ld.volatile.shared.f64 %0, [%1];" : "=d"(v) : "r"((unsigned)__cvta_generic_to_shared(p)));
    return v;
}
__device__ __forceinline__ void sts_vol(double *p, double v) {
    asm volatile("st.volatile.shared.f64 [%0], %1;" ::"r"((unsigned)__cvta_generic_to_shared(p)), "d"(v));
}
struct DRef {
    double *p;
    __device__ __forceinline__ operator double() const { return lds_vol(p); }
    __device__ __forceinline__ DRef &operator=(double v) {
        sts_vol(p, v);
        return *this;
    }
    __device__ __forceinline__ DRef &operator=(const DRef &o) { return *this = (double)o; }
    __device__ __forceinline__ DRef &operator+=(double v) { return *this = lds_vol(p) + v; }
};
template <int STRIDE> struct DArr {
    double *b;
    __device__ __forceinline__ DRef operator[](int i) const { return DRef{b + i * STRIDE}; }
};
__device__ __forceinline__ void fma2_into(DRef sr, DRef si, double xr, double xi, double2 c) {
    sr = fma(xr, c.x, (double)sr);
    si = fma(xi, c.y, (double)si);
}

// ---------------------------------------------------------------------------
// M2M / L2L fast paths (compile-time order): one thread per node of a level,
// FP32 in registers with packed FMAs, FP64 in shared-memory slots.  Both
// translations factor the azimuth out like the M2L.  With
// d = (c_C - c_P) / a_P = (s cos phi, s sin phi, z) and the real regular
// harmonics rho_k^l := R_k^l(s, 0, z) (R_k^l(d) = e^{i l phi} rho_k^l,
// rho_k^{-l} = (-1)^l rho_k^l):
//   M2M  Mhat_P,n^m = sum_C e^{-i m phi} sum_{k,l} rho_k^l Mt_{n-k}^{m-l},
//        Mt_j^u = e^{i u phi} (a_C/a_P)^j Mhat_C,j^u
//   L2L  Lhat_C,j^u += (a_C/a_P)^j e^{-i u phi} sum_{k,l} rho_k^l Lt_{j+k}^{u+l},
//        Lt_n^m = e^{i m phi} Lhat_P,n^m
// with negative orders through X^{-m} = (-1)^m conj(X^m).  The M2M runs from
// the deepest level up: a node first sums its children's translated
// multipoles (fixed order: deterministic), stores its own multipole, then
// writes its translation to the parent's centre for the next level up.
// ---------------------------------------------------------------------------
template <typename T, int MU, int K>
__device__ __forceinline__ T rho_coef(T z, T r2, T diag, T cm1, T cm2) {
    if constexpr (K == MU) {
        return diag;
    } else if constexpr (K == MU + 1) {
        return ((T)(2 * K - 1) / (T)((K + MU) * (K - MU))) * z * cm1;
    } else {
        return ((T)(2 * K - 1) * z * cm1 - r2 * cm2) * ((T)1 / (T)((K + MU) * (K - MU)));
    }
}

template <typename T, int P, int MU, int K, typename AR>
__device__ __forceinline__ void m2m_degree(AR &mr, AR &mi, T z, T r2, T diag, T cm1, T cm2, AR &Sr, AR &Si) {
    const T c = rho_coef<T, MU, K>(z, r2, diag, cm1, cm2);
    const auto cpp = mk2(c, c), cnn = mk2(-c, -c), cpn = mk2(c, -c), cnp = mk2(-c, c);
#pragma unroll
    for (int n = 0; n <= P; ++n) {
        if (n < K) continue;
        const int j = n - K;
#pragma unroll
        for (int m = 0; m <= P; ++m) {
            if (m > n) continue;
            {  // l = +mu, u = m - mu
                const int u = m - MU, au = u < 0 ? -u : u;
                if (au <= j) {
                    if (u >= 0)
                        fma2_into(Sr[tri(n, m)], Si[tri(n, m)], mr[tri(j, u)], mi[tri(j, u)], cpp);
                    else  // (-1)^|u| conj(Mt_j^|u|)
                        fma2_into(Sr[tri(n, m)], Si[tri(n, m)], mr[tri(j, au)], mi[tri(j, au)], (au & 1) ? cnp : cpn);
                }
            }
            if (MU > 0) {  // l = -mu: (-1)^mu rho, u = m + mu
                const int u = m + MU;
                if (u <= j) fma2_into(Sr[tri(n, m)], Si[tri(n, m)], mr[tri(j, u)], mi[tri(j, u)], (MU & 1) ? cnn : cpp);
            }
        }
    }
    if constexpr (K < P) m2m_degree<T, P, MU, K + 1>(mr, mi, z, r2, diag, c, cm1, Sr, Si);
}

template <typename T, int P, int MU, int K, typename AR>
__device__ __forceinline__ void l2l_degree(AR &lr, AR &li, T z, T r2, T diag, T cm1, T cm2, AR &Sr, AR &Si) {
    const T c = rho_coef<T, MU, K>(z, r2, diag, cm1, cm2);
    const auto cpp = mk2(c, c), cnn = mk2(-c, -c), cpn = mk2(c, -c), cnp = mk2(-c, c);
#pragma unroll
    for (int j = 0; j <= P; ++j) {
        if (j + K > P) continue;
        const int n = j + K;
#pragma unroll
        for (int u = 0; u <= P; ++u) {
            if (u > j) continue;
            {  // l = +mu, m' = u + mu
                const int mp = u + MU;
                if (mp <= n) fma2_into(Sr[tri(j, u)], Si[tri(j, u)], lr[tri(n, mp)], li[tri(n, mp)], cpp);
            }
            if (MU > 0) {  // l = -mu: (-1)^mu rho, m' = u - mu
                const int mp = u - MU;
                if (mp >= 0) {
                    fma2_into(Sr[tri(j, u)], Si[tri(j, u)], lr[tri(n, mp)], li[tri(n, mp)], (MU & 1) ? cnn : cpp);
                } else {  // (-1)^(mu + |m'|) conj(Lt_n^|m'|)
                    const int am = -mp;
                    if (am <= n)
                        fma2_into(Sr[tri(j, u)], Si[tri(j, u)], lr[tri(n, am)], li[tri(n, am)],
                                  ((MU + am) & 1) ? cnp : cpn);
                }
            }
        }
    }
    if constexpr (K < P) l2l_degree<T, P, MU, K + 1>(lr, li, z, r2, diag, c, cm1, Sr, Si);
}

// columns mu = 0..P of rho; diag carries rho_mu^mu = -s / (2 mu) rho_{mu-1}^{mu-1}
template <typename T, int P, bool L2L, int MU, typename AR>
__device__ __forceinline__ void shift_column(AR &xr, AR &xi, T s, T z, T r2, T &diag, AR &Sr, AR &Si) {
    if constexpr (MU > 0) diag *= -s * ((T)1 / (T)(2 * MU));
    if constexpr (L2L)
        l2l_degree<T, P, MU, MU>(xr, xi, z, r2, diag, (T)0, (T)0, Sr, Si);
    else
        m2m_degree<T, P, MU, MU>(xr, xi, z, r2, diag, (T)0, (T)0, Sr, Si);
    if constexpr (MU < P) shift_column<T, P, L2L, MU + 1>(xr, xi, s, z, r2, diag, Sr, Si);
}

// Load a coefficient row (16-byte aligned, nc_pad complex) into re / im arrays.
template <int P, typename AR>
__device__ __forceinline__ void load_row(const float2 *row, AR &xr, AR &xi) {
    constexpr int NC = ncoef(P);
    const float4 *r4 = reinterpret_cast<const float4 *>(row);
#pragma unroll
    for (int q = 0; q < (NC + 1) / 2; ++q) {
        const float4 v = r4[q];
        xr[2 * q] = v.x;
        xi[2 * q] = v.y;
        if (2 * q + 1 < NC) {
            xr[2 * q + 1] = v.z;
            xi[2 * q + 1] = v.w;
        }
    }
}
template <int P, typename AR>
__device__ __forceinline__ void load_row(const double2 *row, AR &xr, AR &xi) {
#pragma unroll
    for (int q = 0; q < ncoef(P); ++q) {
        const double2 v = row[q];
        xr[q] = v.x;
        xi[q] = v.y;
    }
}
template <int P, typename AR>
__device__ __forceinline__ void store_row(float2 *row, AR &xr, AR &xi) {
    constexpr int NC = ncoef(P);
    float4 *o4 = reinterpret_cast<float4 *>(row);
#pragma unroll
    for (int q = 0; q < (NC + 1) / 2; ++q)
        o4[q] = make_float4(xr[2 * q], xi[2 * q], 2 * q + 1 < NC ? xr[2 * q + 1] : 0.0f,
                            2 * q + 1 < NC ? xi[2 * q + 1] : 0.0f);
}
template <int P, typename AR>
__device__ __forceinline__ void store_row(double2 *row, AR &xr, AR &xi) {
#pragma unroll
    for (int q = 0; q < ncoef(P); ++q) row[q] = make_double2(xr[q], xi[q]);
}

// x_n^m <- e^{i m phi} f^n x_n^m  (f = 1 for the L2L)
template <typename T, int P, typename AR>
__device__ __forceinline__ void rotate_scale(AR &xr, AR &xi, T ec, T es, T f) {
    T wr = 1, wi = 0;
#pragma unroll
    for (int m = 0; m <= P; ++m) {
        if (m > 0) {
            const T nr = wr * ec - wi * es, ni = wr * es + wi * ec;
            wr = nr;
            wi = ni;
        }
        T fk = 1;
#pragma unroll
        for (int n = 0; n <= P; ++n) {
            if (n >= m) {
                const T fr = wr * fk, fi = wi * fk;
                if constexpr (sizeof(T) == 4) {
                    const float2 x = f2(xr[tri(n, m)], xi[tri(n, m)]);
                    const float2 y = __ffma2_rn(f2(x.y, x.x), f2(-fi, fi), __fmul2_rn(x, f2(fr, fr)));
                    xr[tri(n, m)] = y.x;
                    xi[tri(n, m)] = y.y;
                } else {
                    const T a = xr[tri(n, m)], b = xi[tri(n, m)];
                    xr[tri(n, m)] = a * fr - b * fi;
                    xi[tri(n, m)] = a * fi + b * fr;
                }
            }
            fk *= f;
        }
    }
}

// frame of the translation child -> parent: d = (c_C - c_P) / a_P
template <typename T> struct Shift {
    T ratio, s, z, r2, ec, es;
};
template <typename T>
__device__ __forceinline__ Shift<T> shift_of(typename Vec4<T>::type cc, typename Vec4<T>::type cp, T a_child,
                                             T a_par) {
    Shift<T> f;
    const T iaP = (T)1 / a_par;
    f.ratio = a_child * iaP;
    const T dx = (cc.x - cp.x) * iaP, dy = (cc.y - cp.y) * iaP;
    f.z = (cc.z - cp.z) * iaP;
    const T s2 = dx * dx + dy * dy;
    f.s = sqrt(s2);
    f.r2 = s2 + f.z * f.z;
    f.ec = 1;
    f.es = 0;
    if (s2 > (T)0) {
        const T is = (T)1 / f.s;
        f.ec = dx * is;
        f.es = dy * is;
    }
    return f;
}

template <typename T, int P, typename AR>
__device__ __forceinline__ void m2m_node(int node, const uint8_t *__restrict__ is_leaf,
                                         const int32_t *__restrict__ children, const int32_t *__restrict__ parent,
                                         const typename Vec4<T>::type *__restrict__ center,
                                         const typename Vec4<T>::type *__restrict__ half,
                                         typename Pair<T>::type *__restrict__ Mexp,
                                         typename Pair<T>::type *__restrict__ moved, int nc_pad, AR &xr, AR &xi,
                                         AR &Sr, AR &Si) {
    constexpr int NC = ncoef(P);
    if (is_leaf[node]) {
        load_row<P>(Mexp + (int64_t)node * nc_pad, xr, xi);
    } else {
#pragma unroll
        for (int q = 0; q < NC; ++q) xr[q] = xi[q] = (T)0;
        for (int o = 0; o < 8; ++o) {
            const int ch = children[8 * node + o];
            if (ch < 0) continue;
            load_row<P>(moved + (int64_t)ch * nc_pad, Sr, Si);
#pragma unroll
            for (int q = 0; q < NC; ++q) {
                xr[q] += Sr[q];
                xi[q] += Si[q];
            }
        }
        store_row<P>(Mexp + (int64_t)node * nc_pad, xr, xi);
    }
    const int par = parent[node];
    if (par < 0) return;
    const Shift<T> f = shift_of<T>(center[node], center[par], half[node].w, half[par].w);
    rotate_scale<T, P>(xr, xi, f.ec, f.es, f.ratio);
#pragma unroll
    for (int q = 0; q < NC; ++q) Sr[q] = Si[q] = (T)0;
    T diag = 1;
    shift_column<T, P, false, 0>(xr, xi, f.s, f.z, f.r2, diag, Sr, Si);
    rotate_scale<T, P>(Sr, Si, f.ec, -f.es, (T)1);  // e^{-i m phi}
    store_row<P>(moved + (int64_t)node * nc_pad, Sr, Si);
}

template <typename T, int P, typename AR>
__device__ __forceinline__ void l2l_node(int node, const int32_t *__restrict__ parent,
                                         const typename Vec4<T>::type *__restrict__ center,
                                         const typename Vec4<T>::type *__restrict__ half,
                                         typename Pair<T>::type *__restrict__ Lexp, int nc_pad, AR &xr, AR &xi,
                                         AR &Sr, AR &Si) {
    constexpr int NC = ncoef(P);
    const int par = parent[node];
    if (par < 0) return;
    const Shift<T> f = shift_of<T>(center[node], center[par], half[node].w, half[par].w);
    load_row<P>(Lexp + (int64_t)par * nc_pad, xr, xi);
    rotate_scale<T, P>(xr, xi, f.ec, f.es, (T)1);
#pragma unroll
    for (int q = 0; q < NC; ++q) Sr[q] = Si[q] = (T)0;
    T diag = 1;
    shift_column<T, P, true, 0>(xr, xi, f.s, f.z, f.r2, diag, Sr, Si);
    rotate_scale<T, P>(Sr, Si, f.ec, -f.es, f.ratio);  // (a_C/a_P)^j e^{-i u phi}
    load_row<P>(Lexp + (int64_t)node * nc_pad, xr, xi);
#pragma unroll
    for (int q = 0; q < NC; ++q) {
        xr[q] += Sr[q];
        xi[q] += Si[q];
    }
    store_row<P>(Lexp + (int64_t)node * nc_pad, xr, xi);
}

constexpr int kFastThreads32 = 128, kFastThreads64 = 64;

template <typename T> constexpr int fast_threads() { return sizeof(T) == 4 ? kFastThreads32 : kFastThreads64; }
template <typename T, int P> constexpr size_t fast_smem() {
    return sizeof(T) == 4 ? 0 : (size_t)4 * ncoef(P) * kFastThreads64 * sizeof(double);
}

template <typename T, int P>
__global__ void __launch_bounds__(fast_threads<T>()) k_m2m_fast(
    const int32_t *__restrict__ nodes, int count, const uint8_t *__restrict__ is_leaf,
    const int32_t *__restrict__ children, const int32_t *__restrict__ parent,
    const typename Vec4<T>::type *__restrict__ center, const typename Vec4<T>::type *__restrict__ half,
    typename Pair<T>::type *__restrict__ Mexp, typename Pair<T>::type *__restrict__ moved, int nc_pad) {
    constexpr int NC = ncoef(P);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int node = nodes[i];
    if constexpr (sizeof(T) == 4) {
        float xr[NC], xi[NC], Sr[NC], Si[NC];
        m2m_node<T, P>(node, is_leaf, children, parent, center, half, Mexp, moved, nc_pad, xr, xi, Sr, Si);
    } else {
        extern __shared__ double fast_dsm[];
        constexpr int S = kFastThreads64;
        DArr<S> xr{fast_dsm + threadIdx.x}, xi{fast_dsm + NC * S + threadIdx.x}, Sr{fast_dsm + 2 * NC * S + threadIdx.x},
            Si{fast_dsm + 3 * NC * S + threadIdx.x};
        m2m_node<T, P>(node, is_leaf, children, parent, center, half, Mexp, moved, nc_pad, xr, xi, Sr, Si);
    }
}

template <typename T, int P>
__global__ void __launch_bounds__(fast_threads<T>()) k_l2l_fast(const int32_t *__restrict__ nodes, int count,
                                                                 const int32_t *__restrict__ parent,
                                                                 const typename Vec4<T>::type *__restrict__ center,
                                                                 const typename Vec4<T>::type *__restrict__ half,
                                                                 typename Pair<T>::type *__restrict__ Lexp,
                                                                 int nc_pad) {
    constexpr int NC = ncoef(P);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int node = nodes[i];
    if constexpr (sizeof(T) == 4) {
        float xr[NC], xi[NC], Sr[NC], Si[NC];
        l2l_node<T, P>(node, parent, center, half, Lexp, nc_pad, xr, xi, Sr, Si);
    } else {
        extern __shared__ double fast_dsm[];
        constexpr int S = kFastThreads64;
        DArr<S> xr{fast_dsm + threadIdx.x}, xi{fast_dsm + NC * S + threadIdx.x}, Sr{fast_dsm + 2 * NC * S + threadIdx.x},
            Si{fast_dsm + 3 * NC * S + threadIdx.x};
        l2l_node<T, P>(node, parent, center, half, Lexp, nc_pad, xr, xi, Sr, Si);
    }
}

// ---------------------------------------------------------------------------
// M2L generic path: any precision / order; warp per target row, lanes over
// harmonics columns and output coefficients, operands in shared memory.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(128) k_m2l_generic(int64_t n_rows, const int32_t *__restrict__ row_ids,
                                                     const int32_t *__restrict__ off, const int32_t *__restrict__ src,
                                                     const typename Vec4<T>::type *__restrict__ tcenter,
                                                     const typename Vec4<T>::type *__restrict__ thalf,
                                                     const typename Vec4<T>::type *__restrict__ center,
                                                     const typename Vec4<T>::type *__restrict__ half,
                                                     const Cplx<T> *__restrict__ Mexp, Cplx<T> *Lexp, int p, int nc_pad,
                                                     int accumulate) {
    __shared__ Cplx<T> sI[4][ncoef(2 * kPMax)];
    __shared__ Cplx<T> sM[4][ncoef(kPMax)];
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t w = (int64_t)blockIdx.x * 4 + wl;
    if (w >= n_rows) return;
    const int t = row_ids ? row_ids[w] : (int)w;
    const int nc = ncoef(p);
    const typename Vec4<T>::type ct = tcenter[t];
    const T aL = thalf[t].w;
    Cplx<T> acc[3] = {{0, 0}, {0, 0}, {0, 0}};
    for (int k = off[t]; k < off[t + 1]; ++k) {
        const int s = src[k];
        const typename Vec4<T>::type cs = center[s];
        // Scale by the larger of the two radii so that every ratio is <= 1:
        //  source scale: A_n += (a_L/a_M)^(n+1) sum Mhat_k I_{n+k}(t / a_M)
        //  target scale: A_n += sum Mhat_k (a_M/a_L)^k I_{n+k}(t / a_L)
        const T aM = half[s].w;
        const bool by_src = aM >= aL;
        const T ia = (T)1 / (by_src ? aM : aL);
        const T f = by_src ? aL / aM : aM / aL;
        const T vx = (ct.x - cs.x) * ia, vy = (ct.y - cs.y) * ia, vz = (ct.z - cs.z) * ia;
        const T r2 = vx * vx + vy * vy + vz * vz, ir2 = (T)1 / r2;
        if (lane <= 2 * p) {
            const int mu = lane;
            T dr = (T)1 / sqrt(r2), di = (T)0;
            for (int i = 1; i <= mu; ++i) {
                const T sc = -(T)(2 * i - 1) * ir2;
                const T nr = sc * (vx * dr - vy * di), ni = sc * (vx * di + vy * dr);
                dr = nr;
                di = ni;
            }
            sI[wl][tri(mu, mu)] = Cplx<T>{dr, di};
            T pr = dr, pi = di, qr = 0, qi = 0;
            for (int j = mu + 1; j <= 2 * p; ++j) {
                const T a = (T)(2 * j - 1) * vz, b = (T)((j - 1 + mu) * (j - 1 - mu));
                const T nr = (a * pr - b * qr) * ir2, ni = (a * pi - b * qi) * ir2;
                sI[wl][tri(j, mu)] = Cplx<T>{nr, ni};
                qr = pr;
                qi = pi;
                pr = nr;
                pi = ni;
            }
        }
        for (int c = lane; c < nc; c += 32) {
            Cplx<T> mv = Mexp[(int64_t)s * nc_pad + c];
            if (!by_src) {
                int n, m;
                coef_nm(c, n, m);
                T fk = (T)1;
                for (int e = 0; e < n; ++e) fk *= f;
                mv.re *= fk;
                mv.im *= fk;
            }
            sM[wl][c] = mv;
        }
        __syncwarp();
        for (int q = 0; q < 3; ++q) {
            const int c = lane + 32 * q;
            if (c >= nc) break;
            int n, m;
            coef_nm(c, n, m);
            Cplx<T> sacc{0, 0};
            for (int kk = 0; kk <= p; ++kk)
                for (int l = -kk; l <= kk; ++l) {
                    Cplx<T> v = cmul(harm_at(sM[wl], kk, l), harm_at(sI[wl], n + kk, l - m));
                    sacc.re += v.re;
                    sacc.im += v.im;
                }
            T fn = (T)1;
            if (by_src) {
                fn = f;
                for (int e = 0; e < n; ++e) fn *= f;
            }
            acc[q].re += fn * sacc.re;
            acc[q].im += fn * sacc.im;
        }
        __syncwarp();
    }
    const T iaL = (T)1 / aL;
    for (int q = 0; q < 3; ++q) {
        const int c = lane + 32 * q;
        if (c >= nc) break;
        int n, m;
        coef_nm(c, n, m);
        const T sg = ((n + m) & 1) ? -iaL : iaL;
        Cplx<T> v{sg * acc[q].re, sg * acc[q].im};
        Cplx<T> *o = Lexp + (int64_t)t * nc_pad + c;
        if (accumulate) {
            v.re += o->re;
            v.im += o->im;
        }
        *o = v;
    }
}

// extreme pairs (source radius > 256x target radius) as a CSR by target
template <typename T4>
__global__ void k_extreme_flags(int64_t n_nodes, const int32_t *off, const int32_t *src, const T4 *thalf,
                                const T4 *half, int32_t *row_cnt) {
    using T = decltype(thalf->w);
    const int64_t t = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (t >= n_nodes) return;
    const T iaL = (T)1 / thalf[t].w;
    int c = 0;
    for (int k = off[t] + lane; k < off[t + 1]; k += 32) c += (half[src[k]].w * iaL > (T)kExtremeRatio) ? 1 : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0) row_cnt[t] = c;
}
template <typename T4>
__global__ void k_extreme_fill(int64_t n_nodes, const int32_t *off, const int32_t *src, const T4 *thalf,
                               const T4 *half, const int32_t *eoff, int32_t *esrc) {
    using T = decltype(thalf->w);
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_nodes) return;
    const T iaL = (T)1 / thalf[t].w;
    int j = eoff[t];
    for (int k = off[t]; k < off[t + 1]; ++k)
        if (half[src[k]].w * iaL > (T)kExtremeRatio) esrc[j++] = src[k];
}
__global__ void k_set_last(int32_t *off, int64_t rows, const int64_t *total) { off[rows] = (int32_t)*total; }
__global__ void k_nonempty_rows(int64_t n_nodes, const int32_t *cnt, const int32_t *pos, int32_t *rows) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n_nodes && cnt[t] > 0) rows[pos[t]] = (int32_t)t;
}
__global__ void k_flag_nonzero(int64_t n, const int32_t *cnt, int32_t *flag) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) flag[t] = cnt[t] > 0;
}

// ---------------------------------------------------------------------------
// L2L: warp per node of one level (level >= 1)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(128) k_l2l(const int32_t *__restrict__ nodes, int n_nodes,
                                             const int32_t *__restrict__ parent,
                                             const typename Vec4<T>::type *__restrict__ center,
                                             const typename Vec4<T>::type *__restrict__ half, Cplx<T> *Lexp, int p,
                                             int nc_pad) {
    __shared__ Cplx<T> sR[4][ncoef(kPMax)], sL[4][ncoef(kPMax)];
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = blockIdx.x * 4 + wl;
    if (w >= n_nodes) return;
    const int node = nodes[w];
    const int par = parent[node];
    const int nc = ncoef(p);
    const typename Vec4<T>::type cc = center[node], cp = center[par];
    const T aP = half[par].w, iaP = (T)1 / aP, ratio = half[node].w * iaP;
    if (lane == 0) regular_harmonics_rt<T>((cc.x - cp.x) * iaP, (cc.y - cp.y) * iaP, (cc.z - cp.z) * iaP, p, sR[wl]);
    for (int k = lane; k < nc; k += 32) sL[wl][k] = Lexp[(int64_t)par * nc_pad + k];
    __syncwarp();
    for (int q = 0; q < 3; ++q) {
        const int c = lane + 32 * q;
        if (c >= nc) break;
        int j, u;
        coef_nm(c, j, u);
        Cplx<T> a{0, 0};
        for (int kk = 0; kk + j <= p; ++kk)
            for (int l = -kk; l <= kk; ++l) {
                const int nn = j + kk, mm = u + l;
                if (mm < -nn || mm > nn) continue;
                Cplx<T> v = cmul(harm_at(sL[wl], nn, mm), harm_at(sR[wl], kk, l));
                a.re += v.re;
                a.im += v.im;
            }
        T sc = (T)1;
        for (int e = 0; e < j; ++e) sc *= ratio;
        Cplx<T> *o = Lexp + (int64_t)node * nc_pad + c;
        o->re += sc * a.re;
        o->im += sc * a.im;
    }
}

template <typename T> int p2m_impl(const DevTree &tree, FmmBuffers &buf, cudaStream_t s) {
    using T4 = typename Vec4<T>::type;
    if (tree.n_leaves == 0) return EDFMM_OK;
    const unsigned grid = nblk(tree.n_leaves * 32, 128);
#define EDFMM_P2M_CASE(PP)                                                                                          \
    case PP:                                                                                                        \
        k_p2m<T, PP><<<grid, 128, 0, s>>>(dptr<int32_t>(tree.leaves), tree.n_leaves, dptr<T4>(tree.pts),              \
                                          dptr<T4>(tree.center), dptr<T4>(tree.half), dptr<int2>(tree.range),          \
                                          dptr<Cplx<T>>(buf.multipoles), buf.nc_pad);                                \
        break;
    switch (buf.p) {
        EDFMM_P2M_CASE(1)
        EDFMM_P2M_CASE(2)
        EDFMM_P2M_CASE(3)
        EDFMM_P2M_CASE(4)
        EDFMM_P2M_CASE(5)
        EDFMM_P2M_CASE(6)
        EDFMM_P2M_CASE(7)
        EDFMM_P2M_CASE(8)
        EDFMM_P2M_CASE(9)
        EDFMM_P2M_CASE(10)
        default:
            return fail(EDFMM_ERR_UNSUPPORTED, "expansion order out of range");
    }
#undef EDFMM_P2M_CASE
    EDFMM_LAUNCH_CHECK("k_p2m");
    return EDFMM_OK;
}

template <typename T, int P> int fast_smem_attr(const void *fn) {
    if (fast_smem<T, P>() <= 48 * 1024) return EDFMM_OK;
    const cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fast_smem<T, P>());
    return e == cudaSuccess ? EDFMM_OK : fail(EDFMM_ERR_CUDA, std::string("fast M2M/L2L shared memory: ") +
                                                                   cudaGetErrorString(e));
}

template <typename T, int P> int launch_m2m_fast(const DevTree &tree, FmmBuffers &buf, cudaStream_t s) {
    using T4 = typename Vec4<T>::type;
    using T2 = typename Pair<T>::type;
    static const int attr = fast_smem_attr<T, P>((const void *)k_m2m_fast<T, P>);
    if (attr) return attr;
    constexpr int NT = fast_threads<T>();
    for (int lev = tree.max_level; lev >= 0; --lev) {
        const int lo = tree.level_offsets[lev], hi = tree.level_offsets[lev + 1];
        if (hi <= lo) continue;
        k_m2m_fast<T, P><<<nblk(hi - lo, NT), NT, fast_smem<T, P>(), s>>>(
            dptr<int32_t>(tree.level_nodes) + lo, hi - lo, dptr<uint8_t>(tree.is_leaf), dptr<int32_t>(tree.children),
            dptr<int32_t>(tree.parent), dptr<T4>(tree.center), dptr<T4>(tree.half), dptr<T2>(buf.multipoles),
            dptr<T2>(buf.translated), buf.nc_pad);
        if (lev > 0) count_launch();
    }
    return EDFMM_OK;
}

template <typename T, int P> int launch_l2l_fast(const DevTree &tree, FmmBuffers &buf, cudaStream_t s) {
    using T4 = typename Vec4<T>::type;
    using T2 = typename Pair<T>::type;
    static const int attr = fast_smem_attr<T, P>((const void *)k_l2l_fast<T, P>);
    if (attr) return attr;
    constexpr int NT = fast_threads<T>();
    for (int lev = 1; lev <= tree.max_level; ++lev) {
        const int lo = tree.level_offsets[lev], hi = tree.level_offsets[lev + 1];
        if (hi <= lo) continue;
        k_l2l_fast<T, P><<<nblk(hi - lo, NT), NT, fast_smem<T, P>(), s>>>(
            dptr<int32_t>(tree.level_nodes) + lo, hi - lo, dptr<int32_t>(tree.parent), dptr<T4>(tree.center),
            dptr<T4>(tree.half), dptr<T2>(buf.locals), buf.nc_pad);
        if (lev < tree.max_level) count_launch();
    }
    return EDFMM_OK;
}

template <typename T> int m2m_impl(const DevTree &tree, FmmBuffers &buf, cudaStream_t s) {
    using T4 = typename Vec4<T>::type;
    if (buf.p <= 8 && tree.n_nodes > 0) {
        int rc;
        switch (buf.p) {
            case 1: rc = launch_m2m_fast<T, 1>(tree, buf, s); break;
            case 2: rc = launch_m2m_fast<T, 2>(tree, buf, s); break;
            case 3: rc = launch_m2m_fast<T, 3>(tree, buf, s); break;
            case 4: rc = launch_m2m_fast<T, 4>(tree, buf, s); break;
            case 5: rc = launch_m2m_fast<T, 5>(tree, buf, s); break;
            case 6: rc = launch_m2m_fast<T, 6>(tree, buf, s); break;
            case 7: rc = launch_m2m_fast<T, 7>(tree, buf, s); break;
            default: rc = launch_m2m_fast<T, 8>(tree, buf, s); break;
        }
        if (rc) return rc;
        EDFMM_LAUNCH_CHECK("k_m2m_fast");
        return EDFMM_OK;
    }
    for (int lev = tree.max_level - 1; lev >= 0; --lev) {
        const int lo = tree.level_offsets[lev], hi = tree.level_offsets[lev + 1];
        if (hi <= lo) continue;
        k_m2m<T><<<nblk(hi - lo, 4), 128, 0, s>>>(dptr<int32_t>(tree.level_nodes) + lo, hi - lo, dptr<uint8_t>(tree.is_leaf),
                                                  dptr<int32_t>(tree.children), dptr<T4>(tree.center), dptr<T4>(tree.half),
                                                  dptr<Cplx<T>>(buf.multipoles), buf.p, buf.nc_pad);
        EDFMM_LAUNCH_CHECK("k_m2m");
    }
    return EDFMM_OK;
}

template <typename T> int l2l_impl(const DevTree &tree, FmmBuffers &buf, cudaStream_t s) {
    using T4 = typename Vec4<T>::type;
    if (buf.p <= 8) {
        if (tree.max_level < 1) return EDFMM_OK;
        int rc;
        switch (buf.p) {
            case 1: rc = launch_l2l_fast<T, 1>(tree, buf, s); break;
            case 2: rc = launch_l2l_fast<T, 2>(tree, buf, s); break;
            case 3: rc = launch_l2l_fast<T, 3>(tree, buf, s); break;
            case 4: rc = launch_l2l_fast<T, 4>(tree, buf, s); break;
            case 5: rc = launch_l2l_fast<T, 5>(tree, buf, s); break;
            case 6: rc = launch_l2l_fast<T, 6>(tree, buf, s); break;
            case 7: rc = launch_l2l_fast<T, 7>(tree, buf, s); break;
            default: rc = launch_l2l_fast<T, 8>(tree, buf, s); break;
        }
        if (rc) return rc;
        EDFMM_LAUNCH_CHECK("k_l2l_fast");
        return EDFMM_OK;
    }
    for (int lev = 1; lev <= tree.max_level; ++lev) {
        const int lo = tree.level_offsets[lev], hi = tree.level_offsets[lev + 1];
        if (hi <= lo) continue;
        k_l2l<T><<<nblk(hi - lo, 4), 128, 0, s>>>(dptr<int32_t>(tree.level_nodes) + lo, hi - lo, dptr<int32_t>(tree.parent),
                                                  dptr<T4>(tree.center), dptr<T4>(tree.half), dptr<Cplx<T>>(buf.locals),
                                                  buf.p, buf.nc_pad);
        EDFMM_LAUNCH_CHECK("k_l2l");
    }
    return EDFMM_OK;
}

// extreme-pair CSR for one orientation (float plans only)
template <typename T4>
int build_extreme(const DevTree &tree, const DevTree &stree, const int32_t *off, const int32_t *src, ExtremeRows &ext,
                  cudaStream_t s) {
    int rc;
    const int64_t M = tree.n_nodes;
    DevBuf cnt, tmp, total, flag, pos;
    if ((rc = cnt.reserve(sizeof(int32_t) * M)) || (rc = ext.off.reserve(sizeof(int32_t) * (M + 1))) ||
        (rc = tmp.reserve(scan_tmp_bytes(M))) || (rc = total.reserve(sizeof(int64_t))))
        return rc;
    k_extreme_flags<T4><<<nblk(M * 32, 128), 128, 0, s>>>(M, off, src, dptr<T4>(tree.half), dptr<T4>(stree.half),
                                                      dptr<int32_t>(cnt));
    EDFMM_LAUNCH_CHECK("k_extreme_flags");
    if ((rc = scan_exclusive(dptr<int32_t>(cnt), dptr<int32_t>(ext.off), M, dptr<int64_t>(total), tmp.p, s))) return rc;
    k_set_last<<<1, 1, 0, s>>>(dptr<int32_t>(ext.off), M, dptr<int64_t>(total));
    EDFMM_LAUNCH_CHECK("k_set_last");
    int64_t n_ext = 0;
    EDFMM_CUDA_TRY(cudaMemcpyAsync(&n_ext, total.p, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
    ext.n_pairs = n_ext;
    ext.n_rows = 0;
    ext.built = true;
    if (n_ext == 0) return EDFMM_OK;
    if ((rc = ext.src.reserve(sizeof(int32_t) * n_ext)) || (rc = flag.reserve(sizeof(int32_t) * M)) ||
        (rc = pos.reserve(sizeof(int32_t) * M)) || (rc = ext.rows.reserve(sizeof(int32_t) * M)))
        return rc;
    k_extreme_fill<T4><<<nblk(M, 128), 128, 0, s>>>(M, off, src, dptr<T4>(tree.half), dptr<T4>(stree.half),
                                                 dptr<int32_t>(ext.off), dptr<int32_t>(ext.src));
    EDFMM_LAUNCH_CHECK("k_extreme_fill");
    k_flag_nonzero<<<nblk(M, 256), 256, 0, s>>>(M, dptr<int32_t>(cnt), dptr<int32_t>(flag));
    EDFMM_LAUNCH_CHECK("k_flag_nonzero");
    if ((rc = scan_exclusive(dptr<int32_t>(flag), dptr<int32_t>(pos), M, dptr<int64_t>(total), tmp.p, s))) return rc;
    k_nonempty_rows<<<nblk(M, 256), 256, 0, s>>>(M, dptr<int32_t>(cnt), dptr<int32_t>(pos), dptr<int32_t>(ext.rows));
    EDFMM_LAUNCH_CHECK("k_nonempty_rows");
    int64_t nr = 0;
    EDFMM_CUDA_TRY(cudaMemcpyAsync(&nr, total.p, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    EDFMM_CUDA_TRY(cudaStreamSynchronize(s));
    ext.n_rows = nr;
    return EDFMM_OK;
}

// M2L from the source tree's multipoles (sbuf) into the target tree's locals
// (tbuf); for one tree, tree == stree and sbuf == tbuf.
template <typename T>
int m2l_impl(const DevTree &tree, const DevTree &stree, const DevLists &lists, const FmmBuffers &sbuf,
             FmmBuffers &buf, bool swapped, cudaStream_t s) {
    using T4 = typename Vec4<T>::type;
    const int64_t M = tree.n_nodes;
    if (M == 0 || stree.n_nodes == 0) return EDFMM_OK;
    const int32_t *off = swapped ? dptr<int32_t>(lists.m2l_swapped_off) : dptr<int32_t>(lists.m2l_off);
    const int32_t *src = swapped ? dptr<int32_t>(lists.m2l_swapped_src) : dptr<int32_t>(lists.m2l_src);
    const int32_t *rows = swapped ? nullptr : dptr<int32_t>(lists.m2l_rows);
    if (buf.p > kRotPMaxUsed) {
        // orders above 8: the shared-memory kernel (scales by the larger radius)
        k_m2l_generic<T><<<nblk(M, 4), 128, 0, s>>>(M, nullptr, off, src, dptr<T4>(tree.center), dptr<T4>(tree.half),
                                                    dptr<T4>(stree.center), dptr<T4>(stree.half),
                                                    dptr<Cplx<T>>(sbuf.multipoles), dptr<Cplx<T>>(buf.locals), buf.p,
                                                    buf.nc_pad, 0);
        EDFMM_LAUNCH_CHECK("k_m2l_generic");
        return EDFMM_OK;
    }
    // FP64 plans in two-float mode: the rotation kernel on the FP32 pipe
    // (orders 6..8), which leaves extreme pairs like the FP32 kernel does
    bool two_float = false;
    if (sizeof(T) == 8 && buf.arith == EDFMM_ARITH_TWO_FLOAT && buf.p >= 6 && buf.p <= 8 && tree.nodes_tf.p &&
        stree.nodes_tf.p && sbuf.mult_tf.p) {
        // the source multipoles split once per node, then the pairs
        const int64_t nq = stree.n_nodes * (int64_t)sbuf.nc_pad;
        k_split_coeffs<<<nblk(nq, 256), 256, 0, s>>>(dptr<double2>(sbuf.multipoles), nq, dptr<float4>(sbuf.mult_tf));
        EDFMM_LAUNCH_CHECK("k_split_coeffs");
        int rc = launch_m2l_rot_tf(buf.p, M, off, src, rows, tree.nodes_tf.p, tree.half.p, stree.nodes_tf.p, stree.half.p,
                                   sbuf.mult_tf.p, buf.locals.p, buf.nc_pad, buf.mask, buf.m2l_tf_block,
                                   buf.m2l_packed != 0, s);
        if (rc == EDFMM_OK) two_float = true;
        else if (rc != EDFMM_ERR_UNSUPPORTED) return rc;
    }
    if (!two_float) {
        if (int rc = launch_m2l_rot(sizeof(T) == 8 ? EDFMM_F64 : EDFMM_F32, buf.p, M, off, src, rows, tree.center.p,
                                    tree.half.p, stree.center.p, stree.half.p, sbuf.multipoles.p, buf.locals.p,
                                    buf.nc_pad, buf.mask, s))
            return rc;
        if (sizeof(T) == 8) return EDFMM_OK;  // FP64 has the range for any scale ratio the tree produces
    }
    // FP32 and two-float: pairs whose source scale exceeds 256x the target's, skipped above
    const T4 *tc = dptr<T4>(tree.center), *th = dptr<T4>(tree.half);
    const T4 *cen = dptr<T4>(stree.center), *hal = dptr<T4>(stree.half);
    ExtremeRows &ext = swapped ? buf.extreme_swapped : buf.extreme;
    if (!ext.built) {
        int rc = build_extreme<T4>(tree, stree, off, src, ext, s);
        if (rc) return rc;
    }
    if (ext.n_pairs > 0) {
        k_m2l_generic<T><<<nblk(ext.n_rows, 4), 128, 0, s>>>(
            ext.n_rows, dptr<int32_t>(ext.rows), dptr<int32_t>(ext.off), dptr<int32_t>(ext.src), tc, th, cen, hal,
            dptr<Cplx<T>>(sbuf.multipoles), dptr<Cplx<T>>(buf.locals), buf.p, buf.nc_pad, 1);
        EDFMM_LAUNCH_CHECK("k_m2l_generic");
    }
    return EDFMM_OK;
}

}  // namespace

int set_charges(const DevTree &tree, const void *a, const void *b, cudaStream_t s) {
    if (tree.n_points == 0) return EDFMM_OK;
    if (tree.dtype == EDFMM_F64 && tree.pts_tf.p) {
        k_set_charges_split<<<nblk(tree.n_points, 256), 256, 0, s>>>(
            dptr<double4>(tree.pts), dptr<float4>(tree.pts_tf), dptr<int32_t>(tree.index_map), tree.n_points,
            static_cast<const double *>(a), static_cast<const double *>(b));
        EDFMM_LAUNCH_CHECK("k_set_charges_split");
        return EDFMM_OK;
    }
    if (tree.dtype == EDFMM_F64)
        k_set_charges<double><<<nblk(tree.n_points, 256), 256, 0, s>>>(dptr<double4>(tree.pts), dptr<int32_t>(tree.index_map),
                                                                      tree.n_points, static_cast<const double *>(a),
                                                                      static_cast<const double *>(b));
    else
        k_set_charges<float><<<nblk(tree.n_points, 256), 256, 0, s>>>(dptr<float4>(tree.pts), dptr<int32_t>(tree.index_map),
                                                                     tree.n_points, static_cast<const float *>(a),
                                                                     static_cast<const float *>(b));
    EDFMM_LAUNCH_CHECK("k_set_charges");
    return EDFMM_OK;
}

int run_p2m(const DevTree &tree, FmmBuffers &buf, cudaStream_t s) {
    return tree.dtype == EDFMM_F64 ? p2m_impl<double>(tree, buf, s) : p2m_impl<float>(tree, buf, s);
}
int run_m2m(const DevTree &tree, FmmBuffers &buf, cudaStream_t s) {
    return tree.dtype == EDFMM_F64 ? m2m_impl<double>(tree, buf, s) : m2m_impl<float>(tree, buf, s);
}
int run_m2l(const DevTree &tree, const DevLists &lists, FmmBuffers &buf, bool swapped, cudaStream_t s) {
    return tree.dtype == EDFMM_F64 ? m2l_impl<double>(tree, tree, lists, buf, buf, swapped, s)
                                   : m2l_impl<float>(tree, tree, lists, buf, buf, swapped, s);
}
int run_m2l_two(const DevTree &tgt_tree, const DevTree &src_tree, const DevLists &lists, const FmmBuffers &src_buf,
                FmmBuffers &tgt_buf, cudaStream_t s) {
    return tgt_tree.dtype == EDFMM_F64 ? m2l_impl<double>(tgt_tree, src_tree, lists, src_buf, tgt_buf, false, s)
                                       : m2l_impl<float>(tgt_tree, src_tree, lists, src_buf, tgt_buf, false, s);
}
int prepare_two_float(DevTree &tree, FmmBuffers &buf, cudaStream_t s) {
    if (tree.dtype != EDFMM_F64) return EDFMM_OK;
    const int64_t M = std::max<int64_t>(tree.n_nodes, 1);
    int rc;
    if ((rc = tree.nodes_tf.reserve(sizeof(float4) * 2 * (size_t)M))) return rc;
    if ((rc = buf.mult_tf.reserve(sizeof(float4) * (size_t)buf.nc_pad * (size_t)M))) return rc;
    if (tree.n_nodes > 0) {
        k_split_nodes<<<nblk(tree.n_nodes, 256), 256, 0, s>>>(dptr<double4>(tree.center), dptr<double4>(tree.half),
                                                              tree.n_nodes, dptr<float4>(tree.nodes_tf));
        EDFMM_LAUNCH_CHECK("k_split_nodes");
    }
    return EDFMM_OK;
}

int prepare_extreme_rows(const DevTree &tree, const DevLists &lists, FmmBuffers &buf, cudaStream_t s) {
    if (buf.extreme.built || tree.n_nodes == 0) return EDFMM_OK;
    const int32_t *off = dptr<int32_t>(lists.m2l_off), *src = dptr<int32_t>(lists.m2l_src);
    return tree.dtype == EDFMM_F64 ? build_extreme<double4>(tree, tree, off, src, buf.extreme, s)
                                   : build_extreme<float4>(tree, tree, off, src, buf.extreme, s);
}
int run_l2l(const DevTree &tree, FmmBuffers &buf, cudaStream_t s) {
    return tree.dtype == EDFMM_F64 ? l2l_impl<double>(tree, buf, s) : l2l_impl<float>(tree, buf, s);
}

}  // namespace edfmm
