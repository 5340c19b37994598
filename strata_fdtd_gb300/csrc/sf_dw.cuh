// sf_dw.cuh -- double-word ("float-float") arithmetic on the FP32 pipe.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2,
// about 48 significant bits.  The operations are the error-free
// transformations and double-word algorithms of M. Joldes, J.-M. Muller and
// V. Popescu, "Tight and rigorous error bounds for basic building blocks of
// double-word arithmetic", ACM TOMS 44(2), 2017 (u = 2^-24):
//   sum   AccurateDWPlusDW (their Algorithm 6)   relative error <= 3u^2 + 13u^3
//   mul   DWTimesDW3       (their Algorithm 12)  relative error <= 4u^2
//   mul   DWTimesFP3       (their Algorithm 9)   relative error <= 2u^2
// built from 2Sum (Knuth), Fast2Sum (Dekker) and 2Prod by a fused
// multiply-add.  Every operation is written with explicit round-to-nearest
// intrinsics, so the compiler's contraction setting cannot change it.
//
// The stencil arithmetic (operator+ and operator-) uses a cheaper sum, their
// SloppyDWPlusDW with the final Fast2Sum replaced by a 2Sum: 2Sum of the high
// parts, the low parts added to its error term in two float additions, 2Sum
// of the two (14 operations against 20).  The first and last 2Sums are
// exact, so the result differs from x + y only by the two roundings of the
// low-order additions: |error| <= 3u^2 (|x| + |y|) (1 + u).  That is an
// absolute bound at the operands' scale, not a relative one when x and y
// cancel; the accurate sum (sf_dw::add) stays where a long running sum is
// formed (gradient accumulators, the loss injection).
//
// GB300 runs FP64 at a small fraction of its FP32 rate; a double-word solve
// keeps FP64-class accuracy on the FP32 pipe (the differentiable solve's
// "dw" working precision).
#pragma once
#include <cuda_runtime.h>

struct dwf {
    float hi, lo;
    dwf() = default;
    __host__ __device__ constexpr dwf(float h, float l) : hi(h), lo(l) {}
    // nearest double-word of a double: hi = float(d), lo = float(d - hi)
    __host__ __device__ explicit dwf(double d)
        : hi((float)d), lo((float)(d - (double)(float)d)) {}
    __host__ __device__ explicit dwf(int v) : hi((float)v), lo(0.0f) {}
    __host__ __device__ double to_double() const { return (double)hi + (double)lo; }
};

namespace sf_dw {

// s + e = a + b exactly (Knuth's 2Sum)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bv = __fsub_rn(s, a);
    const float av = __fsub_rn(s, bv);
    e = __fadd_rn(__fsub_rn(a, av), __fsub_rn(b, bv));
}

// s + e = a + b exactly when |a| >= |b| or a == 0 (Dekker's Fast2Sum)
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ dwf add(dwf x, dwf y) {
    float sh, sl, th, tl, vh, vl, zh, zl;
    two_sum(x.hi, y.hi, sh, sl);
    two_sum(x.lo, y.lo, th, tl);
    fast_two_sum(sh, __fadd_rn(sl, th), vh, vl);
    fast_two_sum(vh, __fadd_rn(tl, vl), zh, zl);
    return dwf(zh, zl);
}

// x + y with |error| <= 3u^2 (|x| + |y|) (1 + u) (see the header)
__device__ __forceinline__ dwf add_fast(dwf x, dwf y) {
    float sh, sl, zh, zl;
    two_sum(x.hi, y.hi, sh, sl);
    two_sum(sh, __fadd_rn(sl, __fadd_rn(x.lo, y.lo)), zh, zl);
    return dwf(zh, zl);
}

__device__ __forceinline__ dwf neg(dwf x) { return dwf(-x.hi, -x.lo); }

// x == 1 exactly.  Every double-word this header produces satisfies
// fl(hi + lo) == hi, and for such an x, mul(x, one) and mul(one, x) return x
// (the same hi and lo, up to the sign of a zero lo), so a product with a
// factor known to be one may be skipped without changing any value.
__device__ __forceinline__ bool is_one(dwf x) { return x.hi == 1.0f && x.lo == 0.0f; }

__device__ __forceinline__ dwf mul(dwf x, dwf y) {
    const float ch = __fmul_rn(x.hi, y.hi);
    const float cl1 = __fmaf_rn(x.hi, y.hi, -ch);
    const float tl0 = __fmul_rn(x.lo, y.lo);
    const float tl1 = __fmaf_rn(x.hi, y.lo, tl0);
    const float cl2 = __fmaf_rn(x.lo, y.hi, tl1);
    const float cl3 = __fadd_rn(cl1, cl2);
    float zh, zl;
    fast_two_sum(ch, cl3, zh, zl);
    return dwf(zh, zl);
}

__device__ __forceinline__ dwf mul(dwf x, float y) {
    const float ch = __fmul_rn(x.hi, y);
    const float cl1 = __fmaf_rn(x.hi, y, -ch);
    const float cl3 = __fmaf_rn(x.lo, y, cl1);
    float zh, zl;
    fast_two_sum(ch, cl3, zh, zl);
    return dwf(zh, zl);
}

}  // namespace sf_dw

__device__ __forceinline__ dwf operator+(dwf a, dwf b) { return sf_dw::add_fast(a, b); }
__device__ __forceinline__ dwf operator-(dwf a, dwf b) { return sf_dw::add_fast(a, sf_dw::neg(b)); }
__device__ __forceinline__ dwf operator*(dwf a, dwf b) { return sf_dw::mul(a, b); }
__device__ __forceinline__ dwf& operator+=(dwf& a, dwf b) { return a = a + b; }
__device__ __forceinline__ dwf& operator-=(dwf& a, dwf b) { return a = a - b; }
