// Two-float ("double-FP32") arithmetic: a value is the unevaluated sum
// hi + lo of two floats with |lo| <= ulp(hi) / 2, about 48 significant bits.
// The FP64 operator's dominant stages (M2L, near field) can run on the FP32
// pipe in this form, which on this GPU issues about 60x faster than FP64.
//
// The building blocks are the classical error-free transformations
// (Knuth's two-sum, Dekker's fast two-sum, and the FMA product error
// a*b - fl(a*b)); the sums are the "sloppy" double-float add (relative
// error about 2^-44 of |a| + |b|), which is ample for an operator whose
// truncation error is about 1e-7.  Every step uses the _rn intrinsics so
// the compiler can neither contract nor reorder the error terms.
// Reciprocal, square root and reciprocal square root take one Newton step
// in two-float arithmetic from the FP32 estimate (about 2^-44 relative).
// Exponent range is FP32's: callers keep magnitudes well inside it.
#pragma once

#include <cuda_runtime.h>

namespace edfmm {

// the two-float fma / sqrt below overload the global ones (kept visible for
// the FP32 and FP64 code of this namespace)
using ::fma;
using ::sqrt;

struct tf32x2 {  // "two-float", hi + lo
    float hi, lo;
    tf32x2() = default;
    __host__ __device__ constexpr tf32x2(float h, float l) : hi(h), lo(l) {}
    // exact small integers and constants folded at compile time
    __host__ __device__ constexpr tf32x2(int v) : hi((float)v), lo(0.0f) {}
    __host__ __device__ constexpr tf32x2(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
};

struct tf32x2c {  // complex two-float (16 bytes, the layout of a double2 slot)
    tf32x2 x, y;
};

#ifdef __CUDACC__
__device__ __forceinline__ tf32x2 tf_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return tf32x2(s, e);
}
// requires |a| >= |b| (or a == 0)
__device__ __forceinline__ tf32x2 tf_fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return tf32x2(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ tf32x2 tf_two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return tf32x2(p, __fmaf_rn(a, b, -p));
}

__device__ __forceinline__ tf32x2 tf_from_double(double x) {
    const float h = __double2float_rn(x);
    return tf32x2(h, __double2float_rn(x - (double)h));
}
__device__ __forceinline__ double tf_to_double(tf32x2 a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ tf32x2 operator-(tf32x2 a) { return tf32x2(-a.hi, -a.lo); }
__device__ __forceinline__ tf32x2 operator+(tf32x2 a, tf32x2 b) {
    const tf32x2 s = tf_two_sum(a.hi, b.hi);
    return tf_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ tf32x2 operator-(tf32x2 a, tf32x2 b) { return a + (-b); }
__device__ __forceinline__ tf32x2 operator*(tf32x2 a, tf32x2 b) {
    const tf32x2 p = tf_two_prod(a.hi, b.hi);
    const float e = __fmaf_rn(a.lo, b.hi, __fmaf_rn(a.hi, b.lo, p.lo));
    return tf_fast_two_sum(p.hi, e);
}
__device__ __forceinline__ tf32x2 &operator+=(tf32x2 &a, tf32x2 b) { return a = a + b; }
// a * b + c with one renormalisation
__device__ __forceinline__ tf32x2 fma(tf32x2 a, tf32x2 b, tf32x2 c) {
    const tf32x2 p = tf_two_prod(a.hi, b.hi);
    const float e = __fmaf_rn(a.lo, b.hi, __fmaf_rn(a.hi, b.lo, p.lo));
    const tf32x2 s = tf_two_sum(p.hi, c.hi);
    return tf_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(e, c.lo)));
}
// a * g + c for a compile-time constant g = ghi + glo (glo == 0: one product fewer)
template <bool EXACT>
__device__ __forceinline__ tf32x2 tf_fma_const(float ghi, float glo, tf32x2 a, tf32x2 c) {
    const tf32x2 p = tf_two_prod(a.hi, ghi);
    float e = __fmaf_rn(a.lo, ghi, p.lo);
    if constexpr (!EXACT) e = __fmaf_rn(a.hi, glo, e);
    const tf32x2 s = tf_two_sum(p.hi, c.hi);
    return tf_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(e, c.lo)));
}
__device__ __forceinline__ bool operator>(tf32x2 a, tf32x2 b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }
__device__ __forceinline__ bool operator<(tf32x2 a, tf32x2 b) { return b > a; }

__device__ __forceinline__ tf32x2 tf_recip(tf32x2 a) {
    const float y = __frcp_rn(a.hi);
    const tf32x2 r = tf32x2(1.0f, 0.0f) - a * tf32x2(y, 0.0f);  // 1 - a y, about 2^-24
    return tf_fast_two_sum(y, __fmul_rn(y, r.hi));
}
__device__ __forceinline__ tf32x2 operator/(tf32x2 a, tf32x2 b) { return a * tf_recip(b); }
__device__ __forceinline__ tf32x2 sqrt(tf32x2 a) {
    if (!(a.hi > 0.0f)) return tf32x2(0.0f, 0.0f);
    const float y = __fsqrt_rn(a.hi);
    const tf32x2 r = a - tf_two_prod(y, y);  // a - y^2
    return tf_fast_two_sum(y, __fdiv_rn(r.hi, __fmul_rn(2.0f, y)));
}
// 1 / sqrt(a) for a normal positive a; y0 from the hardware estimate
// (relative error below 2^-22.9), one Newton step y0 + y0 (1 - a y0^2) / 2
__device__ __forceinline__ tf32x2 tf_rsqrt(tf32x2 a, float y0) {
    const tf32x2 h = tf32x2(1.0f, 0.0f) - a * tf_two_prod(y0, y0);
    return tf_fast_two_sum(y0, __fmul_rn(__fmul_rn(0.5f, y0), h.hi));
}
__device__ __forceinline__ tf32x2 tf_shfl_xor(tf32x2 a, int o) {
    return tf32x2(__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o));
}
#endif

}  // namespace edfmm
