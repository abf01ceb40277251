// Single-CTA stable LSD radix sort of 64-bit keys held in global memory (A,
// with B as scratch; the sorted keys end in A).  Only the bytes in which the
// keys differ are sorted on.  Each pass: per-warp digit histograms in shared
// memory (shared atomics), per-digit offsets by a scan, then every warp
// scatters its own contiguous segment in order, 32 keys at a time, ranking
// equal digits among the 32 with __match_any_sync, so the pass is stable.
// blockDim.x: a multiple of 32, at most 1024.  All threads of the CTA must
// call it with the same arguments.
#pragma once
#include <cuda_runtime.h>

namespace wc {

__device__ inline void cta_sort_u64(unsigned long long *A, unsigned long long *B, long long n) {
    __shared__ unsigned int hist[32][256];  // per warp: digit count, then the warp's running position
    __shared__ unsigned int base[256];
    __shared__ unsigned long long s_vary;
    const int T = blockDim.x, t = threadIdx.x, lane = t & 31, w = t >> 5, nw = T >> 5;
    if (n <= 1) return;
    unsigned long long *const A0 = A;
    if (t == 0) s_vary = 0;
    __syncthreads();
    const unsigned long long k0 = A[0];
    unsigned long long diff = 0;
    for (long long i = t; i < n; i += T) diff |= A[i] ^ k0;
    for (int o = 16; o > 0; o >>= 1) diff |= __shfl_xor_sync(0xffffffffu, diff, o);
    if (lane == 0 && diff) atomicOr(&s_vary, diff);
    __syncthreads();
    const unsigned long long vary = s_vary;
    const long long seg = (n + nw - 1) / nw, s0 = min(n, (long long)w * seg), s1 = min(n, s0 + seg);
    const unsigned lt = (1u << lane) - 1;
    for (int pass = 0; pass < 8; pass++) {
        const int sh = pass * 8;
        if (((vary >> sh) & 255) == 0) continue;  // the same digit everywhere: nothing to do
        for (int d = lane; d < 256; d += 32) hist[w][d] = 0;
        __syncwarp();
        for (long long i = s0 + lane; i < s1; i += 32) atomicAdd(&hist[w][(unsigned)(A[i] >> sh) & 255u], 1u);
        __syncthreads();
        for (int d = t; d < 256; d += T) {  // within a digit: warps in order
            unsigned run = 0;
            for (int u = 0; u < nw; u++) {
                const unsigned v = hist[u][d];
                hist[u][d] = run;
                run += v;
            }
            base[d] = run;
        }
        __syncthreads();
        if (w == 0) {  // digits in order: exclusive scan of the totals, 8 digits per lane
            unsigned loc[8], sum = 0;
            for (int q = 0; q < 8; q++) {
                loc[q] = sum;
                sum += base[lane * 8 + q];
            }
            unsigned incl = sum;
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            const unsigned excl = incl - sum;
            for (int q = 0; q < 8; q++) base[lane * 8 + q] = excl + loc[q];
        }
        __syncthreads();
        for (long long c = s0; c < s1; c += 32) {
            const long long i = c + lane;
            const bool ok = i < s1;
            const unsigned long long k = ok ? A[i] : 0ull;
            const unsigned d = ok ? ((unsigned)(k >> sh) & 255u) : 256u + lane;  // idle lanes: unique non-digits
            const unsigned peers = __match_any_sync(0xffffffffu, d);
            const unsigned rank = __popc(peers & lt);
            unsigned pos = 0;
            if (ok) pos = base[d] + hist[w][d] + rank;
            __syncwarp();
            if (ok) {
                B[pos] = k;
                if (rank == 0) hist[w][d] += __popc(peers);
            }
            __syncwarp();
        }
        __syncthreads();
        unsigned long long *x = A;
        A = B;
        B = x;
    }
    if (A != A0) {
        for (long long i = t; i < n; i += T) A0[i] = A[i];
        __syncthreads();
    }
}

}  // namespace wc
