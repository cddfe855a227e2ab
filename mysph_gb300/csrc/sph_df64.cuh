// sph_df64.cuh — double-float arithmetic: a value is the unevaluated sum
// hi + lo of two FP32 numbers (|lo| <= ulp(hi)/2), about 48 significant
// bits, computed on the FP32 pipes.
//
// The operations are the error-free transformations of Knuth (two-sum) and
// Dekker (two-product, here with a fused multiply-add), with the
// renormalisation of the double-double literature (Hida, Li and Bailey,
// "Library for double-double and quad-double arithmetic", 2007; Thall,
// "Extended-precision floating-point numbers for GPU computation", 2006).
// Relative error of add/mul about 2^-44 to 2^-46 per operation; the exponent
// range is FP32's.
#pragma once

#include <cuda_runtime.h>

namespace sph {

struct DF {
    float hi, lo;
};

__device__ __forceinline__ DF df(float a) { return DF{a, 0.0f}; }

// FP64 -> double-float (two conversions) and back.
__device__ __forceinline__ DF df_from(double a) {
    const float h = __double2float_rn(a);
    return DF{h, __double2float_rn(a - (double)h)};
}
__device__ __forceinline__ double df_to(const DF& a) { return (double)a.hi + (double)a.lo; }

// s + e = a + b exactly (Knuth); no precondition on |a|, |b|.
__device__ __forceinline__ DF two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return DF{s, e};
}
// s + e = a + b exactly when |a| >= |b| (Dekker).
__device__ __forceinline__ DF quick_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return DF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
// p + e = a b exactly.
__device__ __forceinline__ DF two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return DF{p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ DF df_add(const DF& a, const DF& b) {
    DF s = two_sum(a.hi, b.hi);
    const float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
    return quick_two_sum(s.hi, e);
}
__device__ __forceinline__ DF df_neg(const DF& a) { return DF{-a.hi, -a.lo}; }
__device__ __forceinline__ DF df_sub(const DF& a, const DF& b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ DF df_add_f(const DF& a, float b) {
    DF s = two_sum(a.hi, b);
    return quick_two_sum(s.hi, __fadd_rn(s.lo, a.lo));
}

__device__ __forceinline__ DF df_mul(const DF& a, const DF& b) {
    DF p = two_prod(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.lo, p.lo);
    e = __fmaf_rn(a.lo, b.hi, e);
    return quick_two_sum(p.hi, e);
}
__device__ __forceinline__ DF df_mul_f(const DF& a, float b) {
    DF p = two_prod(a.hi, b);
    return quick_two_sum(p.hi, __fmaf_rn(a.lo, b, p.lo));
}
// a b + c
__device__ __forceinline__ DF df_fma(const DF& a, const DF& b, const DF& c) { return df_add(df_mul(a, b), c); }

// 1 / a: an FP32 estimate refined by one Newton step in double-float,
// y1 = y0 + y0 (1 - a y0).
__device__ __forceinline__ DF df_rcp(const DF& a) {
    const float y0 = __frcp_rn(a.hi);
    const DF r = df_add_f(df_neg(df_mul_f(a, y0)), 1.0f);  // 1 - a y0
    return df_add_f(df_mul_f(r, y0), y0);
}
// 1 / sqrt(a), a > 0: y1 = y0 + y0 (1 - a y0^2) / 2.
__device__ __forceinline__ DF df_rsqrt(const DF& a) {
    const float y0 = rsqrtf(a.hi);
    const DF ay2 = df_mul_f(df_mul_f(a, y0), y0);
    const DF r = df_add_f(df_neg(ay2), 1.0f);              // 1 - a y0^2
    return df_add_f(df_mul_f(r, 0.5f * y0), y0);
}

// A compensated accumulator of products and sums (the Dot2 scheme of
// Ogita, Rump and Oishi, "Accurate sum and dot product", SIAM J. Sci.
// Comput. 26, 2005, extended to double-float inputs): s collects the
// rounded terms, c their exact rounding errors (two-product, two-sum) and
// the low-order cross terms; the pair is normalised once, at the end.
struct DFAcc {
    float s = 0.0f, c = 0.0f;
    // += a b
    __device__ __forceinline__ void add_prod(const DF& a, const DF& b) {
        const float p = __fmul_rn(a.hi, b.hi);
        float e = __fmaf_rn(a.hi, b.hi, -p);
        e = __fmaf_rn(a.hi, b.lo, e);
        e = __fmaf_rn(a.lo, b.hi, e);
        const DF t = two_sum(s, p);
        s = t.hi;
        c = __fadd_rn(c, __fadd_rn(t.lo, e));
    }
    // += a
    __device__ __forceinline__ void add(const DF& a) {
        const DF t = two_sum(s, a.hi);
        s = t.hi;
        c = __fadd_rn(c, __fadd_rn(t.lo, a.lo));
    }
    __device__ __forceinline__ DF value() const { return two_sum(s, c); }
    __device__ __forceinline__ double to_double() const { return (double)s + (double)c; }
};

}  // namespace sph
