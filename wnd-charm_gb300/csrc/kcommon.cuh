// Device helpers shared by the kernels: block reductions, histogram binning
// with the reference's rules, orderable keys for doubles, launch accounting.
#pragma once
#include <cuda_runtime.h>
#include <cfloat>
#include <cstdint>

#include "wc_internal.h"

namespace wc {

#define WC_LAUNCH(ctx) (++*(ctx).launches)

// signatures::normalize's value of one feature (src/wndchrm_src/signatures.cpp:196-215;
// TrainingSet::normalize, src/wndchrm_src/TrainingSet.cpp:2090-2123): 0 for NaN,
// below the range or a range below DBL_EPSILON, 100 above it, else
// 100 * ((v - mn) / (mx - mn)).  The quotient is the correctly rounded one, by
// Markstein's method (P. Markstein, IBM J. Res. Develop. 34(1), 1990): with
// yh = RN(1/d) and yl ~ 1/d - yh (wnd_recip), q0 = RN(a yh + RN(a yl)) is within
// one ulp of a/d, r = a - d q0 is exact, and RN(q0 + r yh) = RN(a/d); four FP64
// operations where a division takes several more.  Far from the normal range
// (a < 2^-900, d > 2^900) the division itself is used.
__host__ __device__ __forceinline__ double2 wnd_recip(double mn, double mx) {
    const double d = mx - mn;
    const double yh = 1.0 / d;
    return make_double2(yh, fma(-yh, d, 1.0) * yh);
}
static __device__ __noinline__ double wnd_div_far(double a, double d) { return a / d; }
__device__ __forceinline__ double wnd_norm(double v, double mn, double mx, double2 r) {
    const double d = mx - mn;
    if (isnan(v) || v < mn || d < DBL_EPSILON) return 0.0;
    if (v > mx) return 100.0;
    const double a = v - mn;
    if (a == 0.0) return 0.0;
    if (a < 0x1p-900 || d > 0x1p+900) return 100 * wnd_div_far(a, d);
    const double q0 = fma(a, r.x, a * r.y);
    const double res = fma(-q0, d, a);
    return 100 * fma(res, r.x, q0);
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_min(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ long long warp_sum_ll(long long v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Deterministic block reductions (fixed tree); result valid in every thread.
// `sh` must hold 32 doubles.  Block size must be a multiple of 32.
__device__ __forceinline__ double block_sum(double v, double *sh) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double r = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
    if (wid == 0) r = warp_sum(r);
    if (threadIdx.x == 0) sh[0] = r;
    __syncthreads();
    r = sh[0];
    __syncthreads();
    return r;
}
__device__ __forceinline__ double block_min(double v, double *sh) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_min(v);
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double r = (threadIdx.x < nw) ? sh[threadIdx.x] : DBL_MAX;
    if (wid == 0) r = warp_min(r);
    if (threadIdx.x == 0) sh[0] = r;
    __syncthreads();
    r = sh[0];
    __syncthreads();
    return r;
}
__device__ __forceinline__ double block_max(double v, double *sh) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_max(v);
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double r = (threadIdx.x < nw) ? sh[threadIdx.x] : -DBL_MAX;
    if (wid == 0) r = warp_max(r);
    if (threadIdx.x == 0) sh[0] = r;
    __syncthreads();
    r = sh[0];
    __syncthreads();
    return r;
}
__device__ __forceinline__ long long block_sum_ll(long long v, long long *sh) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum_ll(v);
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    long long r = (threadIdx.x < nw) ? sh[threadIdx.x] : 0;
    if (wid == 0) r = warp_sum_ll(r);
    if (threadIdx.x == 0) sh[0] = r;
    __syncthreads();
    r = sh[0];
    __syncthreads();
    return r;
}

// Histogram bin exactly as ImageMatrix::histogram (src/cmatrix.cpp:1088-1100):
// bin = (unsigned long)((v - lo) * scale), clamped to nbins-1, with
// scale = nbins / (hi - lo) or 0 when hi == lo.  A NaN lands in the last bin
// (what the x86-64 conversion of NaN to unsigned long gives before the clamp).
// The comparisons and the truncation act on t's bit pattern (integer
// instructions; the FP64 pipe issues only the subtraction and the product):
// a non-negative double orders as its pattern, and for 1 <= t < 2^31 the
// integer part is the significand shifted by 52 - exponent.
__device__ __forceinline__ long long dbits_of_count(int n) {  // the pattern of (double)n, n >= 1
    const int e = 31 - __clz(n);
    return ((long long)(1023 + e) << 52) | (((long long)n << (52 - e)) & 0x000fffffffffffffLL);
}
__device__ __forceinline__ int hist_bin(double v, double lo, double scale, int nbins) {
    const double t = (v - lo) * scale;
    const long long tb = __double_as_longlong(t);
    if ((tb & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL) return nbins - 1;  // NaN
    if (tb < 0) return 0;                                                    // t < 0, or -0
    if (tb >= dbits_of_count(nbins)) return nbins - 1;                       // t >= nbins, +inf
    const int ex = (int)(tb >> 52) - 1023;
    if (ex < 0) return 0;  // 0 <= t < 1
    const long long b = ((tb & 0x000fffffffffffffLL) | 0x0010000000000000LL) >> (52 - ex);
    return b >= nbins ? nbins - 1 : (int)b;
}
__host__ __device__ __forceinline__ double hist_scale(double lo, double hi, int nbins) {
    return (hi - lo > 0) ? (double)nbins / double(hi - lo) : 0.0;
}

// Total order on doubles as unsigned 64-bit keys (negative values flipped).
__device__ __forceinline__ unsigned long long dkey(double d) {
    unsigned long long u = (unsigned long long)__double_as_longlong(d);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double dkey_inv(unsigned long long k) {
    unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)u);
}

}  // namespace wc
