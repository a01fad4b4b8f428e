// Double-float arithmetic ("df64"): a value is the unevaluated sum hi + lo of
// two FP32 numbers with |lo| <= ulp(hi)/2, about 48 significant bits.
//
// Why: the TVAL3 loop amplifies rounding differences by ~1e8 over a solve
// (perturbing b by 1e-13 moves the 64^3 result by 1e-5; by 1e-9 it changes
// the line-search decisions), so following an FP64 reference to 1e-3 needs
// ~1e-10 per operation, beyond FP32.  GB300 runs FP32 at 64x its FP64 rate;
// the ~5-20 FP32 operations of a double-float operation are therefore several
// times faster than one native FP64 operation, and the storage (8 bytes) is
// the same.
//
// The operations are the classical error-free transformations: TwoSum
// (Knuth, TAOCP vol. 2), FastTwoSum (Dekker 1971) and the FMA-based TwoProd,
// combined as in the published double-double / double-float algorithms
// (addition with both parts renormalised, multiplication with the cross
// terms folded into the error term, division and square root by one
// correction step on an FP32 first approximation).  No compiler option may
// reassociate them: the library is built without fast-math.
#pragma once

#include <cuda_runtime.h>

namespace tv3 {

struct __align__(8) df64 {
    float hi, lo;
    df64() = default;
    __host__ __device__ constexpr df64(float h, float l) : hi(h), lo(l) {}
    __device__ __forceinline__ df64(float f) : hi(f), lo(0.f) {}
    __device__ __forceinline__ df64(int i) : hi((float)i), lo(0.f) {}
    __device__ __forceinline__ explicit df64(double d) {
        hi = __double2float_rn(d);
        lo = __double2float_rn(d - (double)hi);
    }
    __device__ __forceinline__ explicit operator double() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ df64 two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return df64(s, e);
}
__device__ __forceinline__ df64 fast_two_sum(float a, float b) {  // |a| >= |b|
    float s = __fadd_rn(a, b);
    float e = __fsub_rn(b, __fsub_rn(s, a));
    return df64(s, e);
}
__device__ __forceinline__ df64 two_prod(float a, float b) {
    float p = __fmul_rn(a, b);
    float e = __fmaf_rn(a, b, -p);
    return df64(p, e);
}

__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
    df64 s = two_sum(a.hi, b.hi);
    df64 t = two_sum(a.lo, b.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = fast_two_sum(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }
__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }
__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
    df64 p = two_prod(a.hi, b.hi);
    p.lo = __fmaf_rn(a.hi, b.lo, p.lo);
    p.lo = __fmaf_rn(a.lo, b.hi, p.lo);
    return fast_two_sum(p.hi, p.lo);
}
// df64 times an exact FP32 value (matrix entries)
__device__ __forceinline__ df64 mul_f(df64 a, float b) {
    df64 p = two_prod(a.hi, b);
    p.lo = __fmaf_rn(a.lo, b, p.lo);
    return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ df64 operator/(df64 a, df64 b) {
    float q1 = __fdiv_rn(a.hi, b.hi);
    df64 r = a - mul_f(b, q1);
    float q2 = __fdiv_rn(r.hi, b.hi);
    df64 q = fast_two_sum(q1, q2);
    r = a - b * q;
    float q3 = __fdiv_rn(r.hi, b.hi);
    return q + df64(q3);
}
__device__ __forceinline__ df64& operator+=(df64& a, df64 b) { return a = a + b; }
__device__ __forceinline__ df64& operator-=(df64& a, df64 b) { return a = a - b; }
__device__ __forceinline__ df64& operator*=(df64& a, df64 b) { return a = a * b; }

__device__ __forceinline__ bool operator<(df64 a, df64 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(df64 a, df64 b) { return b < a; }
__device__ __forceinline__ bool operator<=(df64 a, df64 b) { return !(b < a); }
__device__ __forceinline__ bool operator>=(df64 a, df64 b) { return !(a < b); }
__device__ __forceinline__ bool operator==(df64 a, df64 b) { return a.hi == b.hi && a.lo == b.lo; }

// keep the float/double overloads visible next to the df64 ones
using ::fabs;
using ::sqrt;
__device__ __forceinline__ df64 fabs(df64 a) { return (a.hi < 0.f || (a.hi == 0.f && a.lo < 0.f)) ? -a : a; }
__device__ __forceinline__ df64 sqrt(df64 a) {
    if (!(a.hi > 0.f)) return df64(0.f, 0.f);
    float x = __fsqrt_rn(a.hi);
    df64 r = a - two_prod(x, x);
    float c = __fdiv_rn(r.hi, 2.f * x);
    return fast_two_sum(x, c);
}

// a^2 + b^2 + c^2 with the squares' rounding errors and cross terms kept in
// a compensated float (the Dot2 idea, as ProdAcc): all terms are
// non-negative, so the result is accurate to the double-float level.
__device__ __forceinline__ df64 sum_sq3(df64 a, df64 b, df64 c) {
    df64 pa = two_prod(a.hi, a.hi), pb = two_prod(b.hi, b.hi), pc = two_prod(c.hi, c.hi);
    df64 s = two_sum(pa.hi, pb.hi);
    df64 t = two_sum(s.hi, pc.hi);
    float e = __fadd_rn(s.lo, t.lo);
    e = __fadd_rn(e, __fadd_rn(__fadd_rn(pa.lo, pb.lo), pc.lo));
    e = __fmaf_rn(2.f * a.hi, a.lo, e);
    e = __fmaf_rn(2.f * b.hi, b.lo, e);
    e = __fmaf_rn(2.f * c.hi, c.lo, e);
    return fast_two_sum(t.hi, e);
}

// 1/sqrt(s) for s > 0: the correctly rounded FP32 reciprocal square root of
// s.hi, then one Newton step y = y0 + y0 (1 - s y0^2) / 2 with the residual
// formed in double-float (Karp & Markstein, "High-precision division and
// square root", ACM TOMS 1997): the error of y0 (~2^-24) squares to ~2^-48.
__device__ __forceinline__ df64 rsqrt_df(df64 s) {
    const float y0 = __frsqrt_rn(s.hi);
    const df64 y2 = two_prod(y0, y0);
    const df64 r = df64(1.f) - s * y2;  // ~2^-24, exact enough in its high part
    return fast_two_sum(y0, __fmul_rn(__fmul_rn(0.5f, y0), r.hi));
}

}  // namespace tv3
