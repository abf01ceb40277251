// Single-CTA stable LSD radix sort of 64-bit keys held in global memory.
// Each thread owns a contiguous segment, so the scatter is stable without
// in-tile ranking: position = base[digit] + count of that digit in earlier
// segments + running count in the own segment.  A pass whose digit is the same
// for every key is skipped.  `cnt` must hold 256 * blockDim.x counters.
// The sorted keys end in `A`.  All threads of the CTA must call it.
#pragma once
#include <cuda_runtime.h>

namespace wc {

__device__ inline void cta_radix_sort_u64(unsigned long long *A, unsigned long long *B, long long n,
                                          unsigned int *__restrict__ cnt) {
    __shared__ unsigned int base[256];
    __shared__ int skip;
    unsigned long long *const A0 = A;
    const int T = blockDim.x, t = threadIdx.x;
    const long long seg = (n + T - 1) / T, s0 = t * seg, s1 = min(n, s0 + seg);
    __syncthreads();
    for (int pass = 0; pass < 8; pass++) {
        const int sh = pass * 8;
        unsigned int local[256];
        for (int d = 0; d < 256; d++) local[d] = 0;
        for (long long i = s0; i < s1; i++) local[(A[i] >> sh) & 255]++;
        for (int d = 0; d < 256; d++) cnt[(size_t)d * T + t] = local[d];
        __syncthreads();
        if (t < 256) {
            unsigned int run = 0;
            for (int u = 0; u < T; u++) {
                unsigned int v = cnt[(size_t)t * T + u];
                cnt[(size_t)t * T + u] = run;
                run += v;
            }
            base[t] = run;
        }
        if (t == 0) skip = 0;
        __syncthreads();
        if (t == 0) {
            unsigned int run = 0;
            for (int d = 0; d < 256; d++) {
                unsigned int v = base[d];
                if ((long long)v == n) skip = 1;
                base[d] = run;
                run += v;
            }
        }
        __syncthreads();
        if (!skip) {
            for (int d = 0; d < 256; d++) local[d] = base[d] + cnt[(size_t)d * T + t];
            for (long long i = s0; i < s1; i++) {
                const unsigned long long k = A[i];
                B[local[(k >> sh) & 255]++] = k;
            }
            __syncthreads();
            unsigned long long *x = A;
            A = B;
            B = x;
        }
        __syncthreads();
    }
    if (A != A0) {
        for (long long i = t; i < n; i += T) A0[i] = A[i];
        __syncthreads();
    }
}

}  // namespace wc
