// Pairs of floats (hi + lo, |lo| <= ulp(hi) / 2, about 48 significant bits)
// for the mixed form's FP32-pipe arithmetic where FP32 alone is too coarse:
// error-free transformations (Knuth's two-sum, Dekker's fast two-sum, the FMA
// two-product) as in Hida, Li and Bailey's double-double library, on floats.
// Every product that must stay exact is written with __fmul_rn / fmaf so that
// no contraction changes it.
#pragma once
#include <cuda_runtime.h>

namespace wc {

struct df {
    float hi, lo;
};

__device__ __forceinline__ df df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ df df_fast_two_sum(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ df df_from_double(double x) {
    const float h = __double2float_rn(x);
    return {h, __double2float_rn(x - (double)h)};
}
__device__ __forceinline__ double df_to_double(df a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ df df_add(df a, df b) {
    df s = df_two_sum(a.hi, b.hi);
    s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
    return df_fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ df df_mul(df a, df b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return df_fast_two_sum(p, e);
}
__device__ __forceinline__ df df_div(df a, df b) {
    const float q1 = __fdiv_rn(a.hi, b.hi);
    const df r = df_sub(a, df_mul({q1, 0.f}, b));
    return df_fast_two_sum(q1, __fdiv_rn(r.hi, b.hi));
}
__device__ __forceinline__ df df_sqrt(df a) {  // a > 0
    const float s = __fsqrt_rn(a.hi);
    const df r = df_sub(a, df_mul({s, 0.f}, {s, 0.f}));
    return df_fast_two_sum(s, __fdiv_rn(r.hi, __fmul_rn(2.f, s)));
}

}  // namespace wc
