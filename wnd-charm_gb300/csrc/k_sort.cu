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

// One tile of RS_TILE keys per CTA: the tile is ranked by digit in shared
// memory (warp w takes keys [512 w, 512 w + 512) in 16 rounds of 32, equal
// digits ranked by lane with __match_any_sync, per-warp digit counters), so
// its keys land there in digit order with the tile's order kept among equal
// digits; then consecutive threads write each digit's run to consecutive
// places (tbase[d] from the scan of every tile's counts): a stable pass with
// coalesced writes.
__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(unsigned long long *__restrict__ keys, unsigned long long *__restrict__ tmp,
                                                           const SortSeg *__restrict__ seg, const int *__restrict__ cur,
                                                           const unsigned int *__restrict__ cnt, const int *__restrict__ skip,
                                                           int max_tiles, int shift) {
    constexpr int NW = RS_THREADS / 32, PER_W = RS_TILE / NW;  // 8 warps, 512 keys each
    __shared__ unsigned long long sk[RS_TILE];
    __shared__ unsigned int wcnt[NW][256];
    __shared__ unsigned int tbase[256], lstart[256], scan[RS_THREADS];
    const SortSeg S = seg[blockIdx.y];
    const long long t0 = (long long)blockIdx.x * RS_TILE;
    if (t0 >= S.n || skip[blockIdx.y]) return;
    const int c = cur[blockIdx.y];
    const unsigned long long *src = (c ? tmp : keys) + S.off + t0;
    unsigned long long *dst = (c ? keys : tmp) + S.off;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int ntile = (int)min((long long)RS_TILE, S.n - t0);
    const unsigned lt = (1u << lane) - 1;
    for (int i = t; i < NW * 256; i += RS_THREADS) (&wcnt[0][0])[i] = 0;
    tbase[t] = cnt[((long long)blockIdx.y * 256 + t) * max_tiles + blockIdx.x];
    __syncthreads();
    unsigned long long k[PER_W / 32];
    unsigned int off[PER_W / 32];
#pragma unroll
    for (int r = 0; r < PER_W / 32; r++) {
        const int idx = w * PER_W + r * 32 + lane;
        const bool ok = idx < ntile;
        k[r] = ok ? src[idx] : 0ull;
        const unsigned d = ok ? ((unsigned)(k[r] >> shift) & 255u) : 256u + lane;  // idle lanes: unique non-digits
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int leader = __ffs(peers) - 1;
        unsigned base = 0;
        if (ok && lane == leader) {
            base = wcnt[w][d];
            wcnt[w][d] = base + __popc(peers);
        }
        base = __shfl_sync(0xffffffffu, base, leader);
        off[r] = base + __popc(peers & lt);
        __syncwarp();
    }
    __syncthreads();
    {  // digit t: its warps' counts into bases, and its total
        unsigned run = 0;
        for (int u = 0; u < NW; u++) {
            const unsigned v = wcnt[u][t];
            wcnt[u][t] = run;
            run += v;
        }
        scan[t] = run;
    }
    __syncthreads();
    {  // exclusive scan of the digit totals (Hillis-Steele over 256 values)
        unsigned v = scan[t];
        for (int o = 1; o < 256; o <<= 1) {
            const unsigned y = t >= o ? scan[t - o] : 0u;
            __syncthreads();
            v += y;
            scan[t] = v;
            __syncthreads();
        }
        lstart[t] = t ? scan[t - 1] : 0u;  // the inclusive scan is complete after the loop's last barrier
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < PER_W / 32; r++) {
        const int idx = w * PER_W + r * 32 + lane;
        if (idx < ntile) {
            const unsigned d = (unsigned)(k[r] >> shift) & 255u;
            sk[lstart[d] + wcnt[w][d] + off[r]] = k[r];
        }
    }
    __syncthreads();
    for (int i = t; i < ntile; i += RS_THREADS) {
        const unsigned long long key = sk[i];
        const unsigned d = (unsigned)(key >> shift) & 255u;
        dst[tbase[d] + (unsigned)i - lstart[d]] = key;
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
    WC_LAUNCH(c);
    k_rs_keys<<<dim3(64, nseg), 256, 0, c.st>>>(arena, planes, ids, seg, keys, cur);
    for (int pass = 0; pass < 8; pass++) {
        const int shift = pass * 8;
        WC_LAUNCH(c);
        k_rs_hist<<<dim3(max_tiles, nseg), RS_THREADS, 0, c.st>>>(keys, tmp, seg, cur, cnt, max_tiles, shift);
        WC_LAUNCH(c);
        k_rs_scan<<<nseg, 256, 0, c.st>>>(seg, cnt, skip, max_tiles);
        WC_LAUNCH(c);
        k_rs_scatter<<<dim3(max_tiles, nseg), RS_THREADS, 0, c.st>>>(keys, tmp, seg, cur, cnt, skip, max_tiles, shift);
        WC_LAUNCH(c);
        k_rs_flip<<<(nseg + 255) / 256, 256, 0, c.st>>>(cur, skip, nseg);
    }
    WC_LAUNCH(c);
    k_rs_final<<<dim3(64, nseg), 256, 0, c.st>>>(keys, tmp, seg, cur);
}

}  // namespace wc
