// Double-float arithmetic: a value is the unevaluated sum hi + lo of two FP32
// numbers (about 44 significant bits).  Built from error-free transformations
// (Knuth's TwoSum, FMA-based TwoProduct) and one Newton step for 1/sqrt.
// Used for the far-field influence coefficients of the mixed path, where FP32
// alone leaves Cp errors above 1e-5 on clustered trailing edges.
#pragma once
#include <cuda_runtime.h>

struct df32 {
    float hi, lo;
};

__device__ __forceinline__ df32 df_two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return df32{s, e};
}
__device__ __forceinline__ df32 df_fast_two_sum(float a, float b) {  // |a| >= |b|
    float s = __fadd_rn(a, b);
    float e = __fsub_rn(b, __fsub_rn(s, a));
    return df32{s, e};
}
__device__ __forceinline__ df32 df_add(df32 x, df32 y) {
    df32 s = df_two_sum(x.hi, y.hi);
    float e = __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo));
    return df_fast_two_sum(s.hi, e);
}
__device__ __forceinline__ df32 df_sub(df32 x, df32 y) { return df_add(x, df32{-y.hi, -y.lo}); }
__device__ __forceinline__ df32 df_mul(df32 x, df32 y) {
    float p = __fmul_rn(x.hi, y.hi);
    float e = __fmaf_rn(x.hi, y.hi, -p);
    e = __fmaf_rn(x.hi, y.lo, e);
    e = __fmaf_rn(x.lo, y.hi, e);
    return df_fast_two_sum(p, e);
}
// 1/sqrt(x) for x > 0: y0 = rsqrtf, then y1 = y0 + y0*(1 - x*y0^2)/2 with the
// residual formed in double-float (1 - x*y0^2 is exact in its leading part).
__device__ __forceinline__ df32 df_rsqrt(df32 x) {
    float y = rsqrtf(x.hi);
    float p = __fmul_rn(y, y);
    float pe = __fmaf_rn(y, y, -p);
    df32 t = df_mul(x, df32{p, pe});
    float r = __fsub_rn(__fsub_rn(1.0f, t.hi), t.lo);
    return df_fast_two_sum(y, __fmul_rn(__fmul_rn(y, r), 0.5f));
}
__device__ __forceinline__ double df_to_double(df32 x) { return (double)x.hi + (double)x.lo; }
__device__ __forceinline__ df32 df_neg(df32 x) { return df32{-x.hi, -x.lo}; }
// sqrt(x) = x / sqrt(x) for x > 0
__device__ __forceinline__ df32 df_sqrt(df32 x) { return df_mul(x, df_rsqrt(x)); }
// a / b: a float quotient, then the quotient of the double-float remainder
__device__ __forceinline__ df32 df_div(df32 a, df32 b) {
    float q1 = __fdiv_rn(a.hi, b.hi);
    df32 r = df_sub(a, df_mul(df32{q1, 0.f}, b));
    float q2 = __fdiv_rn(r.hi, b.hi);
    return df_fast_two_sum(q1, q2);
}
// a double-precision constant as a double-float (folded at compile time)
#define CPG_DFK(v) df32{(float)(v), (float)((v) - (double)(float)(v))}
