// Device helpers shared by the kernels: block reductions, histogram binning
// with the reference's rules, orderable keys for doubles, launch accounting.
#pragma once
#include <cuda_runtime.h>
#include <cfloat>
#include <cstdint>

#include "wc_internal.h"

namespace wc {

#define WC_LAUNCH(ctx) (++*(ctx).launches)

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
__device__ __forceinline__ int hist_bin(double v, double lo, double scale, int nbins) {
    double t = (v - lo) * scale;
    if (!(t < (double)nbins)) return nbins - 1;  // also NaN
    if (t < 0) return 0;
    unsigned long long b = (unsigned long long)t;
    return b >= (unsigned long long)nbins ? nbins - 1 : (int)b;
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
