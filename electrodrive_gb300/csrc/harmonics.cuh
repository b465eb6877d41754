// Complex solid harmonics with the Condon-Shortley phase, stored for m >= 0
// at index (n, m) -> n (n + 1) / 2 + m:
//   R_n^m(v) = |v|^n P_n^m(cos t) e^{i m phi} / (n + m)!     (regular)
//   I_n^m(v) = (n - m)! P_n^m(cos t) e^{i m phi} / |v|^{n+1} (irregular)
//   X_n^{-m} = (-1)^m conj(X_n^m)
// generated by the Cartesian recurrences
//   R_m^m = -(x + i y) / (2m) R_{m-1}^{m-1}
//   R_n^m = ((2n - 1) z R_{n-1}^m - |v|^2 R_{n-2}^m) / ((n + m)(n - m))
//   I_m^m = -(2m - 1) (x + i y) / |v|^2 I_{m-1}^{m-1}
//   I_n^m = ((2n - 1) z I_{n-1}^m - (n - 1 + m)(n - 1 - m) I_{n-2}^m) / |v|^2
// With these, 1/|x - y| = sum conj(R_n^m(y)) I_n^m(x) for |y| < |x|, and the
// translation operators take the coefficient-free forms used by the stages:
//   M2M  M'_n^m = sum_{k,l} conj(R_k^l(c - c')) M_{n-k}^{m-l}
//   M2L  L_n^m  = (-1)^(n+m) sum_{k,l} M_k^l I_{n+k}^{l-m}(c_L - c_M)
//   L2L  L'_j^u = sum_{k,l} L_{j+k}^{u+l} R_k^l(c' - c)
//   L2P  phi    = sum_{n,m} L_n^m R_n^m(x - c)
#pragma once

namespace edfmm {

constexpr int kPMax = 10;  // largest supported expansion order

__host__ __device__ constexpr int tri(int n, int m) { return n * (n + 1) / 2 + m; }
__host__ __device__ constexpr int ncoef(int p) { return (p + 1) * (p + 2) / 2; }

template <typename T> struct Cplx {
    T re, im;
};

// regular harmonics up to order P at (x, y, z), P a compile-time constant
template <typename T, int P>
__device__ __forceinline__ void regular_harmonics(T x, T y, T z, T (&Rr)[ncoef(P)], T (&Ri)[ncoef(P)]) {
    const T r2 = x * x + y * y + z * z;
    Rr[0] = (T)1;
    Ri[0] = (T)0;
#pragma unroll
    for (int m = 1; m <= P; ++m) {
        const T s = (T)(-1.0 / (2.0 * m));
        const T ar = Rr[tri(m - 1, m - 1)], ai = Ri[tri(m - 1, m - 1)];
        Rr[tri(m, m)] = s * (x * ar - y * ai);
        Ri[tri(m, m)] = s * (x * ai + y * ar);
    }
#pragma unroll
    for (int m = 0; m <= P; ++m) {
#pragma unroll
        for (int n = 1; n <= P; ++n) {
            if (n <= m) continue;
            const T c1 = (T)(2 * n - 1) / (T)((n + m) * (n - m));
            if (n - 2 >= m) {
                const T c2 = (T)1 / (T)((n + m) * (n - m));
                Rr[tri(n, m)] = c1 * z * Rr[tri(n - 1, m)] - c2 * r2 * Rr[tri(n - 2, m)];
                Ri[tri(n, m)] = c1 * z * Ri[tri(n - 1, m)] - c2 * r2 * Ri[tri(n - 2, m)];
            } else {
                Rr[tri(n, m)] = c1 * z * Rr[tri(n - 1, m)];
                Ri[tri(n, m)] = c1 * z * Ri[tri(n - 1, m)];
            }
        }
    }
}

// runtime-order versions writing to (shared) memory
template <typename T>
__device__ inline void regular_harmonics_rt(T x, T y, T z, int p, Cplx<T> *R) {
    const T r2 = x * x + y * y + z * z;
    R[0].re = (T)1;
    R[0].im = (T)0;
    for (int m = 1; m <= p; ++m) {
        const T s = (T)(-1.0 / (2.0 * m));
        Cplx<T> a = R[tri(m - 1, m - 1)];
        R[tri(m, m)].re = s * (x * a.re - y * a.im);
        R[tri(m, m)].im = s * (x * a.im + y * a.re);
    }
    for (int m = 0; m <= p; ++m)
        for (int n = m + 1; n <= p; ++n) {
            const T d = (T)1 / (T)((n + m) * (n - m));
            Cplx<T> a = R[tri(n - 1, m)];
            Cplx<T> b = n - 2 >= m ? R[tri(n - 2, m)] : Cplx<T>{(T)0, (T)0};
            R[tri(n, m)].re = ((T)(2 * n - 1) * z * a.re - r2 * b.re) * d;
            R[tri(n, m)].im = ((T)(2 * n - 1) * z * a.im - r2 * b.im) * d;
        }
}

// X_n^m for any sign of m from m >= 0 storage
template <typename T> __device__ __forceinline__ Cplx<T> harm_at(const Cplx<T> *X, int n, int m) {
    if (m >= 0) return X[tri(n, m)];
    Cplx<T> v = X[tri(n, -m)];
    if ((-m) & 1) return Cplx<T>{-v.re, v.im};
    return Cplx<T>{v.re, -v.im};
}

template <typename T> __device__ __forceinline__ Cplx<T> cmul(Cplx<T> a, Cplx<T> b) {
    return Cplx<T>{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}

}  // namespace edfmm
