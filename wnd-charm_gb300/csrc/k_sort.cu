// Multi-CTA LSD radix sort of many independent arrays ("segments") of 64-bit
// keys at once: 8 passes of 8-bit digits, each pass
//   1. per (tile of 4096 keys, segment): digit histogram;
//   2. per segment: exclusive scan over (digit, tile) -> scatter bases; a
//      segment whose keys all share the digit skips the pass;
//   3. per (tile, segment): stable scatter.  Thread t owns 16 consecutive keys
//      of the tile; its rank among equal digits is the count in earlier
//      threads (a u16 prefix table in shared memory) plus the count earlier in
//      its own 16 keys, so the pass is stable and the sort deterministic;
//   4. flip the segment's ping-pong buffer.
// The sorted keys end in `keys`.
#include "kcommon.cuh"
#include "kernels.h"

namespace wc {

#define RS_THREADS 256
#define RS_ITEMS 16
#define RS_TILE (RS_THREADS * RS_ITEMS)

__global__ void __launch_bounds__(RS_THREADS) k_rs_hist(const unsigned long long *__restrict__ keys,
                                                        const unsigned long long *__restrict__ tmp,
                                                        const SortSeg *__restrict__ seg, const int *__restrict__ cur,
                                                        unsigned int *__restrict__ cnt, int max_tiles, int shift) {
    __shared__ unsigned int h[256];
    const SortSeg S = seg[blockIdx.y];
    const long long t0 = (long long)blockIdx.x * RS_TILE;
    h[threadIdx.x] = 0;
    __syncthreads();
    if (t0 < S.n) {
        const unsigned long long *src = (cur[blockIdx.y] ? tmp : keys) + S.off;
        const long long t1 = min(S.n, t0 + RS_TILE);
        for (long long i = t0 + threadIdx.x; i < t1; i += blockDim.x) atomicAdd(&h[(src[i] >> shift) & 255], 1u);
    }
    __syncthreads();
    cnt[((long long)blockIdx.y * 256 + threadIdx.x) * max_tiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(256) k_rs_scan(const SortSeg *__restrict__ seg, unsigned int *__restrict__ cnt,
                                                 int *__restrict__ skip, int max_tiles) {
    __shared__ unsigned int tot[256];
    const SortSeg S = seg[blockIdx.x];
    const int d = threadIdx.x;
    const int ntiles = (int)((S.n + RS_TILE - 1) / RS_TILE);
    unsigned int *c = cnt + ((long long)blockIdx.x * 256 + d) * max_tiles;
    unsigned int run = 0;
    for (int t = 0; t < ntiles; t++) {
        const unsigned int v = c[t];
        c[t] = run;
        run += v;
    }
    tot[d] = run;
    __syncthreads();
    __shared__ unsigned int base[256];
    __shared__ int sk;
    if (d == 0) {
        unsigned int r = 0;
        sk = 0;
        for (int q = 0; q < 256; q++) {
            if ((long long)tot[q] == S.n) sk = 1;
            base[q] = r;
            r += tot[q];
        }
        skip[blockIdx.x] = sk;
    }
    __syncthreads();
    for (int t = 0; t < ntiles; t++) c[t] += base[d];
}

__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(unsigned long long *__restrict__ keys, unsigned long long *__restrict__ tmp,
                                                           const SortSeg *__restrict__ seg, const int *__restrict__ cur,
                                                           const unsigned int *__restrict__ cnt, const int *__restrict__ skip,
                                                           int max_tiles, int shift) {
    extern __shared__ unsigned short pre[];  // [RS_THREADS][256]
    __shared__ unsigned int tbase[256];
    const SortSeg S = seg[blockIdx.y];
    const long long t0 = (long long)blockIdx.x * RS_TILE;
    if (t0 >= S.n || skip[blockIdx.y]) return;
    const int c = cur[blockIdx.y];
    const unsigned long long *src = (c ? tmp : keys) + S.off;
    unsigned long long *dst = (c ? keys : tmp) + S.off;
    const int t = threadIdx.x;
    tbase[t] = cnt[((long long)blockIdx.y * 256 + t) * max_tiles + blockIdx.x];
    unsigned short *row = pre + (long long)t * 256;
    for (int d = 0; d < 256; d++) row[d] = 0;
    unsigned long long k[RS_ITEMS];
    const long long k0 = t0 + (long long)t * RS_ITEMS;
#pragma unroll
    for (int i = 0; i < RS_ITEMS; i++) {
        const long long idx = k0 + i;
        k[i] = idx < S.n ? src[idx] : 0;
        if (idx < S.n) row[(k[i] >> shift) & 255]++;
    }
    __syncthreads();
    {  // exclusive scan over threads, one digit per thread
        unsigned int run = 0;
        for (int u = 0; u < RS_THREADS; u++) {
            const unsigned short v = pre[(long long)u * 256 + t];
            pre[(long long)u * 256 + t] = (unsigned short)run;
            run += v;
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < RS_ITEMS; i++) {
        const long long idx = k0 + i;
        if (idx >= S.n) break;
        const int d = (int)((k[i] >> shift) & 255);
        int same = 0;
#pragma unroll
        for (int j = 0; j < RS_ITEMS; j++)
            if (j < i && (int)((k[j] >> shift) & 255) == d) same++;
        dst[tbase[d] + row[d] + same] = k[i];
    }
}

__global__ void k_rs_flip(int *__restrict__ cur, const int *__restrict__ skip, int nseg) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nseg && !skip[s]) cur[s] ^= 1;
}

__global__ void k_rs_final(unsigned long long *__restrict__ keys, const unsigned long long *__restrict__ tmp,
                           const SortSeg *__restrict__ seg, const int *__restrict__ cur) {
    const SortSeg S = seg[blockIdx.y];
    if (!cur[blockIdx.y]) return;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < S.n; i += (long long)gridDim.x * blockDim.x)
        keys[S.off + i] = tmp[S.off + i];
}

// keys of every sorted plane: orderable 64-bit images of the doubles
__global__ void k_rs_keys(const double *__restrict__ arena, const Plane *__restrict__ planes, const int *__restrict__ ids,
                          const SortSeg *__restrict__ seg, unsigned long long *__restrict__ keys, int *__restrict__ cur) {
    const Plane P = planes[ids[blockIdx.y]];
    const SortSeg S = seg[blockIdx.y];
    if (blockIdx.x == 0 && threadIdx.x == 0) cur[blockIdx.y] = 0;
    const double *src = arena + P.off;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < S.n; i += (long long)gridDim.x * blockDim.x)
        keys[S.off + i] = dkey(src[i]);
}

size_t sort_scratch_bytes(int nseg, long long max_n) {
    const long long tiles = (max_n + RS_TILE - 1) / RS_TILE;
    return (size_t)nseg * 256 * tiles * 4 + (size_t)nseg * 8 + 512;
}

void launch_sort_planes(Ctx &c, const double *arena, const Plane *planes, const int *ids, const SortSeg *seg, int nseg,
                        long long max_n, unsigned long long *keys, unsigned long long *tmp, void *scratch) {
    if (nseg <= 0) return;
    const int max_tiles = (int)((max_n + RS_TILE - 1) / RS_TILE);
    unsigned int *cnt = (unsigned int *)scratch;
    int *cur = (int *)(cnt + (size_t)nseg * 256 * max_tiles);
    int *skip = cur + nseg;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_rs_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, RS_THREADS * 256 * 2);
        attr = true;
    }
    WC_LAUNCH(c);
    k_rs_keys<<<dim3(64, nseg), 256, 0, c.st>>>(arena, planes, ids, seg, keys, cur);
    for (int pass = 0; pass < 8; pass++) {
        const int shift = pass * 8;
        WC_LAUNCH(c);
        k_rs_hist<<<dim3(max_tiles, nseg), RS_THREADS, 0, c.st>>>(keys, tmp, seg, cur, cnt, max_tiles, shift);
        WC_LAUNCH(c);
        k_rs_scan<<<nseg, 256, 0, c.st>>>(seg, cnt, skip, max_tiles);
        WC_LAUNCH(c);
        k_rs_scatter<<<dim3(max_tiles, nseg), RS_THREADS, RS_THREADS * 256 * 2, c.st>>>(keys, tmp, seg, cur, cnt, skip,
                                                                                      max_tiles, shift);
        WC_LAUNCH(c);
        k_rs_flip<<<(nseg + 255) / 256, 256, 0, c.st>>>(cur, skip, nseg);
    }
    WC_LAUNCH(c);
    k_rs_final<<<dim3(64, nseg), 256, 0, c.st>>>(keys, tmp, seg, cur);
}

}  // namespace wc
