// Pairs of floats (hi + lo, |lo| <= ulp(hi) / 2, about 48 significant bits)
// for the mixed form's FP32-pipe arithmetic where FP32 alone is too coarse:
// error-free transformations (Knuth's two-sum, Dekker's fast two-sum, the FMA
// two-product) as in Hida, Li and Bailey's double-double library, on floats.
// Every product that must stay exact is written with __fmul_rn / fmaf so that
// no contraction changes it.
#pragma once
#include <cuda_runtime.h>

namespace wc {

struct __align__(8) df {
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
// The rare cases of df_split / f32_of take conversions (FP64-pipe
// instructions), in calls that are not inlined, so that the common path
// carries none of them (a short inlined branch may be predicated and issued
// on every pass).
static __device__ __noinline__ df df_split_slow(double x) { return df_from_double(x); }
static __device__ __noinline__ float f32_slow(double x) { return __double2float_rn(x); }
// The same pair from the double's bits, off the FP64 pipe (conversions from
// and to double issue there): hi = the mantissa rounded to 24 bits (nearest,
// ties to even), lo = the 29-bit remainder (exact as an integer, rounded once
// by the int-to-float conversion) times 2^(e-52).  Doubles outside
// [2^-74, 2^128) other than zero take the conversions.
__device__ __forceinline__ df df_split(double x) {
    const long long b = __double_as_longlong(x);
    if ((b & 0x7fffffffffffffffLL) == 0) return {0.f, 0.f};
    const int ef = (int)((b >> 52) & 0x7ff) - 1023 + 127;
    if (ef < 53 || ef > 254) return df_split_slow(x);
    const unsigned low = (unsigned)(b & 0x1fffffffLL);
    const unsigned top = ((unsigned)ef << 23) | (unsigned)((b >> 29) & 0x7fffff);
    const bool up = low > 0x10000000u || (low == 0x10000000u && (top & 1u));
    const unsigned sign = (unsigned)((unsigned long long)b >> 63) << 31;
    const float hi = __uint_as_float(sign | (top + (up ? 1u : 0u)));
    const int r = up ? (int)low - 0x20000000 : (int)low;
    const float lo = __fmul_rn(__int2float_rn(sign ? -r : r), __uint_as_float((unsigned)(ef - 52) << 23));
    return {hi, lo};
}
// (float)x from the bits (round to nearest, ties to even) while the result is
// a normal float; zero keeps its sign; the rest take the conversion
__device__ __forceinline__ float f32_of(double x) {
    const long long b = __double_as_longlong(x);
    const unsigned sign = (unsigned)((unsigned long long)b >> 63) << 31;
    if ((b & 0x7fffffffffffffffLL) == 0) return __uint_as_float(sign);
    const int ef = (int)((b >> 52) & 0x7ff) - 1023 + 127;
    if (ef < 1 || ef > 254) return f32_slow(x);
    const unsigned low = (unsigned)(b & 0x1fffffffLL);
    const unsigned top = ((unsigned)ef << 23) | (unsigned)((b >> 29) & 0x7fffff);
    const bool up = low > 0x10000000u || (low == 0x10000000u && (top & 1u));
    return __uint_as_float(sign | (top + (up ? 1u : 0u)));
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
// a * b + c with one renormalisation
__device__ __forceinline__ df df_fma(df a, df b, df c) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    df s = df_two_sum(p, c.hi);
    s.lo = __fadd_rn(s.lo, __fadd_rn(e, c.lo));
    return df_fast_two_sum(s.hi, s.lo);
}
// times a power of two (exact, barring underflow)
__device__ __forceinline__ df df_scale(df a, float p2) { return {__fmul_rn(a.hi, p2), __fmul_rn(a.lo, p2)}; }
// the sign of a normalised pair is the sign of hi (hi = 0 implies lo = 0)
__device__ __forceinline__ df df_abs(df a) { return a.hi < 0.f ? df_neg(a) : a; }
__device__ __forceinline__ bool df_lt(df a, df b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ df df_shfl(df a, int src) {
    return {__shfl_sync(0xffffffffu, a.hi, src), __shfl_sync(0xffffffffu, a.lo, src)};
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
