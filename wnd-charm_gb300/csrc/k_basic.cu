// Per-plane basics: pixel conversion, plane statistics, the Edge and Wavelet
// transforms, a per-plane radix sort (medians, Gini), and the light feature
// families (multiscale histograms, fractal, comb moments, pixel statistics,
// Gini, Radon, Chebyshev coefficients).  FP64 arithmetic throughout.
#include <cfloat>
#include <cmath>
#include <string>

#include "kcommon.cuh"
#include "kwavelet.cuh"
#include "kdf32.cuh"
#include "kernels.h"

namespace wc {

// ---------------------------------------------------------------- convert
template <typename T>
__global__ void k_convert(const T *__restrict__ src, double *__restrict__ dst, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = (double)src[i];
}

void launch_convert(Ctx &c, const void *src, int dtype, double *dst, long long n) {
    int blocks = (int)((n + 255) / 256);
    if (blocks > c.sms * 8) blocks = c.sms * 8;
    if (blocks < 1) blocks = 1;
    WC_LAUNCH(c);
    switch (dtype) {
        case 0: k_convert<unsigned char><<<blocks, 256, 0, c.st>>>((const unsigned char *)src, dst, n); break;
        case 1: k_convert<unsigned short><<<blocks, 256, 0, c.st>>>((const unsigned short *)src, dst, n); break;
        case 2: k_convert<float><<<blocks, 256, 0, c.st>>>((const float *)src, dst, n); break;
        default: k_convert<double><<<blocks, 256, 0, c.st>>>((const double *)src, dst, n); break;
    }
}

// ---------------------------------------------------------------- plane stats
// Moments2 of every plane (src/statistics/Moments.h:61-107): min, max, mean,
// var = M2/(n-1) for n > 2.  Two deterministic passes per plane, one CTA each.
__global__ void __launch_bounds__(1024) k_plane_stats(const double *__restrict__ arena, const Plane *__restrict__ planes,
                                                      PlaneStats *__restrict__ out, int nn, int sel) {
    __shared__ double sh[32];
    // sel 0: every plane; 1: the root plane of each image (index b*nn); 2: the others
    const int pi = sel == 0 ? blockIdx.x : sel == 1 ? blockIdx.x * nn : (blockIdx.x / (nn - 1)) * nn + 1 + blockIdx.x % (nn - 1);
    const Plane P = planes[pi];
    const double *p = arena + P.off;
    const long long n = (long long)P.w * P.h;
    double mn = DBL_MAX, mx = -DBL_MAX, s = 0;
    long long cnt = 0;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        double v = p[i];
        if (isnan(v) || v > FLT_MAX || v < -FLT_MAX) continue;  // Moments2::add skips these
        mn = fmin(mn, v);
        mx = fmax(mx, v);
        s += v;
        cnt++;
    }
    mn = block_min(mn, sh);
    mx = block_max(mx, sh);
    s = block_sum(s, sh);
    __shared__ long long shl[32];
    cnt = block_sum_ll(cnt, shl);
    double mean = cnt ? s / cnt : 0.0;
    double m2 = 0;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        double v = p[i];
        if (isnan(v) || v > FLT_MAX || v < -FLT_MAX) continue;
        double d = v - mean;
        m2 += d * d;
    }
    m2 = block_sum(m2, sh);
    if (threadIdx.x == 0) {
        PlaneStats r;
        r.mn = mn;
        r.mx = mx;
        r.mean = mean;
        r.var = cnt > 2 ? m2 / (cnt - 1) : 0.0;
        r.sum = s;
        r.n = cnt;
        out[pi] = r;
    }
}

void launch_plane_stats(Ctx &c, const double *arena, const Plane *planes, int nplanes, PlaneStats *out, int nn, int sel) {
    const int nb = sel == 0 ? nplanes : sel == 1 ? nplanes / nn : nplanes / nn * (nn - 1);
    if (nb <= 0) return;
    WC_LAUNCH(c);
    k_plane_stats<<<nb, 1024, 0, c.st>>>(arena, planes, out, nn, sel);
}

// ---------------------------------------------------------------- Edge transform
// ImageMatrix::EdgeTransform, src/cmatrix.cpp:1294-1311.
__global__ void k_edge(double *__restrict__ arena, const Plane *__restrict__ planes, const TJob *__restrict__ jobs) {
    const TJob J = jobs[blockIdx.z];
    const Plane S = planes[J.src], D = planes[J.dst];
    int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= S.w || y >= S.h) return;
    const double *in = arena + S.off;
    const int W = S.w, H = S.h;
    double c = in[(long long)y * W + x], mx = 0, my = 0;
    if (y > 0 && y < H - 1) my = fmax(fabs(c - in[(long long)(y - 1) * W + x]), fabs(c - in[(long long)(y + 1) * W + x]));
    if (x > 0 && x < W - 1) mx = fmax(fabs(c - in[(long long)y * W + x - 1]), fabs(c - in[(long long)y * W + x + 1]));
    arena[D.off + (long long)y * W + x] = fmax(mx, my);
}

void launch_edge(Ctx &c, double *arena, const Plane *planes, const TJob *jobs, int njobs, int maxw, int maxh) {
    if (njobs <= 0) return;
    // block shape from the tuner (per size class): 32 x 8, 64 x 4 or 16 x 16
    const std::string key = "edge/" + std::to_string(maxw / 64) + "x" + std::to_string(maxh / 64) + "/" +
                            std::to_string(njobs / 16);
    const int cand = c.tune ? c.tune->pick(key, 3) : 0;
    const dim3 b = cand == 0 ? dim3(32, 8) : (cand == 1 ? dim3(64, 4) : dim3(16, 16));
    const dim3 g((maxw + b.x - 1) / b.x, (maxh + b.y - 1) / b.y, njobs);
    Tuner::Pending tp;
    const bool timing = c.tune && c.tune->exploring(key);
    if (timing) c.tune->begin(key, cand, c.st, tp);
    WC_LAUNCH(c);
    k_edge<<<g, b, 0, c.st>>>(arena, planes, jobs);
    if (timing) c.tune->end(tp, c.st);
}

// ---------------------------------------------------------------- Wavelet transform
// One level of the zero-padded Symlet-5 decomposition; the tap loops are in
// kwavelet.cuh (shared with the allocation-free entry point and the adjoint).

// pass 1: along y for each column x: tmp[(x*oy + o)*2 + {0: approx, 1: detail}]
__global__ void k_wavelet_y(const double *__restrict__ arena, const Plane *__restrict__ planes,
                            const TJob *__restrict__ jobs, double *__restrict__ tmp, const long long *__restrict__ tmp_off) {
    const TJob J = jobs[blockIdx.z];
    const Plane S = planes[J.src];
    const int X = S.w, Y = S.h, oy = sym5_out(Y);
    int x = blockIdx.x * blockDim.x + threadIdx.x, o = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= X || o >= oy) return;
    double a, d;
    sym5_col(arena + S.off, X, Y, x, o, a, d);
    double *t = tmp + tmp_off[blockIdx.z] + sym5_tmp_index(x, oy, o);
    t[0] = a;
    t[1] = d;
}

// pass 2: along x for each row o of both pass-1 outputs, placed in quadrants
__global__ void k_wavelet_x(double *__restrict__ arena, const Plane *__restrict__ planes, const TJob *__restrict__ jobs,
                            const double *__restrict__ tmp, const long long *__restrict__ tmp_off) {
    const TJob J = jobs[blockIdx.z];
    const Plane S = planes[J.src], D = planes[J.dst];
    const int X = S.w, Y = S.h, ox = sym5_out(X), oy = sym5_out(Y);
    int u = blockIdx.x * blockDim.x + threadIdx.x, o = blockIdx.y * blockDim.y + threadIdx.y;
    if (u >= ox || o >= oy) return;
    double a1, d1, a2, d2;
    sym5_row(tmp + tmp_off[blockIdx.z], X, oy, u, o, a1, d1, a2, d2);
    sym5_store(arena + D.off, ox, oy, u, o, a1, d1, a2, d2);
}

void launch_wavelet(Ctx &c, double *arena, const Plane *planes, const TJob *jobs, int njobs, int maxw, int maxh,
                    double *tmp, const long long *tmp_off) {
    if (njobs <= 0) return;
    int ox = (maxw + 9) / 2, oy = (maxh + 9) / 2;
    // block shape of both passes from the tuner (per size class)
    const std::string key = "wavelet/" + std::to_string(maxw / 64) + "x" + std::to_string(maxh / 64) + "/" +
                            std::to_string(njobs / 16);
    const int cand = c.tune ? c.tune->pick(key, 3) : 0;
    const dim3 b = cand == 0 ? dim3(32, 8) : (cand == 1 ? dim3(64, 4) : dim3(16, 16));
    Tuner::Pending tp;
    const bool timing = c.tune && c.tune->exploring(key);
    if (timing) c.tune->begin(key, cand, c.st, tp);
    WC_LAUNCH(c);
    k_wavelet_y<<<dim3((maxw + b.x - 1) / b.x, (oy + b.y - 1) / b.y, njobs), b, 0, c.st>>>(arena, planes, jobs, tmp,
                                                                                          tmp_off);
    WC_LAUNCH(c);
    k_wavelet_x<<<dim3((ox + b.x - 1) / b.x, (oy + b.y - 1) / b.y, njobs), b, 0, c.st>>>(arena, planes, jobs, tmp,
                                                                                         tmp_off);
    if (timing) c.tune->end(tp, c.st);
}

// ---------------------------------------------------------------- pixel statistics + Gini
// PixelIntensityStatistics (src/FeatureAlgorithms.cpp:272-294) and
// GiniCoefficient (src/FeatureAlgorithms.cpp:448-492) from a sorted plane.
// job.plane indexes `sorted_ids` position via job.img (sort slot).
__global__ void k_pixstats(const Plane *__restrict__ planes, const PlaneStats *__restrict__ stats,
                           const FJob *__restrict__ jobs, const int *__restrict__ sort_slot,
                           const unsigned long long *__restrict__ keys, const long long *__restrict__ key_off,
                           double *__restrict__ feat) {
    const FJob J = jobs[blockIdx.x];
    if (threadIdx.x != 0) return;
    const Plane P = planes[J.plane];
    const PlaneStats S = stats[J.plane];
    const long long n = (long long)P.w * P.h, half = n / 2;
    const unsigned long long *k = keys + key_off[sort_slot[blockIdx.x]];
    double med;
    if (n % 2 == 0) med = (dkey_inv(k[half]) + dkey_inv(k[half - 1])) / 2.0;
    else med = dkey_inv(k[half]);
    double *o = feat + J.out;
    o[0] = S.mean;
    o[1] = med;
    o[2] = S.n > 2 ? sqrt(S.var) : 0.0;
    o[3] = S.mn;
    o[4] = S.mx;
}

__global__ void __launch_bounds__(512) k_gini(const Plane *__restrict__ planes, const FJob *__restrict__ jobs, const int *__restrict__ sort_slot,
                       const unsigned long long *__restrict__ keys, const long long *__restrict__ key_off,
                       double *__restrict__ feat) {
    __shared__ double sh[32];
    const FJob J = jobs[blockIdx.x];
    const Plane P = planes[J.plane];
    const long long n = (long long)P.w * P.h;
    const unsigned long long *k = keys + key_off[sort_slot[blockIdx.x]];
    // positives form a suffix of the sorted keys: find its start by binary search
    long long lo = 0, hi = n;
    while (lo < hi) {
        long long mid = (lo + hi) / 2;
        if (dkey_inv(k[mid]) > 0) hi = mid; else lo = mid + 1;
    }
    const long long first = lo, count = n - first;
    double sum = 0, g = 0;
    for (long long i = threadIdx.x; i < count; i += blockDim.x) {
        double v = dkey_inv(k[first + i]);
        sum += v;
        g += (2. * (double)(i + 1) - (double)count - 1.) * v;
    }
    sum = block_sum(sum, sh);
    g = block_sum(g, sh);
    if (threadIdx.x == 0) {
        double mean = count > 0 ? sum / count : 0.0;
        feat[J.out] = (count <= 1 || mean <= 0.0) ? 0.0 : g / (mean * count * (count - 1));
    }
}

void launch_pixstats(Ctx &c, const Plane *planes, const PlaneStats *stats, const FJob *jobs, int njobs,
                     const int *sort_slot, const unsigned long long *keys, const long long *key_off, double *feat) {
    if (njobs <= 0) return;
    WC_LAUNCH(c);
    k_pixstats<<<njobs, 32, 0, c.st>>>(planes, stats, jobs, sort_slot, keys, key_off, feat);
}
void launch_gini(Ctx &c, const Plane *planes, const FJob *jobs, int njobs, const int *sort_slot,
                 const unsigned long long *keys, const long long *key_off, double *feat) {
    if (njobs <= 0) return;
    WC_LAUNCH(c);
    k_gini<<<njobs, 512, 0, c.st>>>(planes, jobs, sort_slot, keys, key_off, feat);
}

// ---------------------------------------------------------------- multiscale histograms
// ImageMatrix::MultiScaleHistogram, src/cmatrix.cpp:1743-1756.
__global__ void __launch_bounds__(512) k_mshist(const double *__restrict__ arena, const Plane *__restrict__ planes,
                         const PlaneStats *__restrict__ stats, const FJob *__restrict__ jobs, double *__restrict__ feat) {
    __shared__ unsigned int h[24];
    const FJob J = jobs[blockIdx.x];
    const Plane P = planes[J.plane];
    const PlaneStats S = stats[J.plane];
    if (threadIdx.x < 24) h[threadIdx.x] = 0;
    __syncthreads();
    const double *p = arena + P.off;
    const long long n = (long long)P.w * P.h;
    const double s3 = hist_scale(S.mn, S.mx, 3), s5 = hist_scale(S.mn, S.mx, 5), s7 = hist_scale(S.mn, S.mx, 7),
                 s9 = hist_scale(S.mn, S.mx, 9);
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        double v = p[i];
        atomicAdd(&h[hist_bin(v, S.mn, s3, 3)], 1u);
        atomicAdd(&h[3 + hist_bin(v, S.mn, s5, 5)], 1u);
        atomicAdd(&h[8 + hist_bin(v, S.mn, s7, 7)], 1u);
        atomicAdd(&h[15 + hist_bin(v, S.mn, s9, 9)], 1u);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double mx = 0;
        for (int a = 0; a < 24; a++) mx = fmax(mx, (double)h[a]);
        for (int a = 0; a < 24; a++) feat[J.out + a] = (double)h[a] / mx;
    }
}

void launch_mshist(Ctx &c, const double *arena, const Plane *planes, const PlaneStats *stats, const FJob *jobs,
                   int njobs, double *feat) {
    if (njobs <= 0) return;
    WC_LAUNCH(c);
    k_mshist<<<njobs, 512, 0, c.st>>>(arena, planes, stats, jobs, feat);
}

// ---------------------------------------------------------------- fractal
// FractalFeatures::execute, src/FeatureAlgorithms.cpp:232-267: for the k-th
// lag (k = 1 + slot*step, k < K), mean absolute difference along y and x.
__global__ void __launch_bounds__(512) k_fractal(const double *__restrict__ arena, const Plane *__restrict__ planes, const FJob *__restrict__ jobs,
                          double *__restrict__ feat) {
    __shared__ double sh[32];
    const FJob J = jobs[blockIdx.y];
    const Plane P = planes[J.plane];
    const int W = P.w, H = P.h, slot = blockIdx.x;
    const int K = ((W > H) ? H : W) / 5;
    int step = K / 20;
    if (step < 1) step = 1;
    const int k = 1 + slot * step;
    if (k >= K) {
        if (threadIdx.x == 0) feat[J.out + slot] = 0.0;
        return;
    }
    const double *p = arena + P.off;
    double s = 0;
    const long long n1 = (long long)W * (H - k), n2 = (long long)(W - k) * H;
    for (long long i = threadIdx.x; i < n1; i += blockDim.x) {
        long long y = i / W, x = i - y * W;
        s += fabs(p[y * W + x] - p[(y + k) * W + x]);
    }
    for (long long i = threadIdx.x; i < n2; i += blockDim.x) {
        long long y = i / (W - k), x = i - y * (W - k);
        s += fabs(p[y * W + x] - p[y * W + x + k]);
    }
    s = block_sum(s, sh);
    if (threadIdx.x == 0) feat[J.out + slot] = s / (double)(W * (W - k) + H * (H - k));
}

// The mixed form, on the FP32 and integer pipes: a CTA per (plane, group of 4
// lags).  Each pixel is split into a pair of floats from the double's bits
// (df_split), and so is each partner as it is read; every |I(p) - I(q)| is
// formed in pairs (two-sum of the highs, the lows added: ~48 bits of the FP64
// difference) and summed per lag in pairs, then the block's sums are added in
// FP64 in a fixed order (deterministic).  Four lags per CTA keep the
// accumulators few and the CTAs per SM many (the chains are latency-bound).
#define FR_THREADS 512
#define FR_LAGS 4
__global__ void __launch_bounds__(FR_THREADS) k_fractal_df(const double *__restrict__ arena, const Plane *__restrict__ planes,
                                                           const FJob *__restrict__ jobs, double *__restrict__ feat) {
    __shared__ double red[FR_THREADS / 32][FR_LAGS];
    const FJob J = jobs[blockIdx.y];
    const Plane P = planes[J.plane];
    const int W = P.w, H = P.h;
    const int K = ((W > H) ? H : W) / 5;
    int step = K / 20;
    if (step < 1) step = 1;
    const int l0 = blockIdx.x * FR_LAGS;
    int kk[FR_LAGS];
#pragma unroll
    for (int l = 0; l < FR_LAGS; l++) {
        const int k = 1 + (l0 + l) * step;
        kk[l] = k < K ? k : H + W;  // past the last lag: no pair
    }
    const double *p = arena + P.off;
    df acc[FR_LAGS];
#pragma unroll
    for (int l = 0; l < FR_LAGS; l++) acc[l] = {0.f, 0.f};
    const int n = W * H;  // at most 2^28 pixels
    for (int i = threadIdx.x; i < n; i += FR_THREADS) {
        const int y = i / W, x = i - y * W;
        const df a = df_split(p[i]);
#pragma unroll
        for (int l = 0; l < FR_LAGS; l++) {
            const int k = kk[l];
            if (y + k < H) acc[l] = df_add(acc[l], df_abs(df_sub(a, df_split(p[i + (long long)k * W]))));
            if (x + k < W) acc[l] = df_add(acc[l], df_abs(df_sub(a, df_split(p[i + k]))));
        }
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int l = 0; l < FR_LAGS; l++) {
        double v = df_to_double(acc[l]);
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[w][l] = v;
    }
    __syncthreads();
    if (threadIdx.x < FR_LAGS) {
        const int l = threadIdx.x, slot = l0 + l, k = 1 + slot * step;
        double s = 0;
        for (int u = 0; u < FR_THREADS / 32; u++) s += red[u][l];
        if (slot < 20) feat[J.out + slot] = k < K ? s / (double)(W * (W - k) + H * (H - k)) : 0.0;
    }
}

void launch_fractal(Ctx &c, const double *arena, const Plane *planes, const FJob *jobs, int njobs, double *feat) {
    if (njobs <= 0) return;
    WC_LAUNCH(c);
    if (c.prec == WC_PREC_MIXED)
        k_fractal_df<<<dim3(20 / FR_LAGS, njobs), FR_THREADS, 0, c.st>>>(arena, planes, jobs, feat);
    else k_fractal<<<dim3(20, njobs), 512, 0, c.st>>>(arena, planes, jobs, feat);
}

// ---------------------------------------------------------------- comb moments
// CombFirst4Moments2D + matr4moments_to_hist + vd_Comb4Moments,
// src/statistics/CombFirst4Moments.cpp:47-272.  One thread per comb line runs
// Moments4's Welford updates (src/statistics/Moments.h:60-107) over the line's
// pixels in the reference's order, every operation rounded as the CPU rounds
// it (no contraction), so the moments - and the 3-bin histograms of them,
// whose bins mathematically tied lines (the mirrored halves of a Fourier
// plane) decide by their last bits - are the reference's.
__device__ __forceinline__ bool comb_pixel(int dir, long long j, long long ii, long long m, long long n, long long n2,
                                           long long m2, long long &y, long long &x) {
    if (dir == 0) { y = j; x = j + ii; return x >= 0 && x < n; }
    if (dir == 1) { y = j; x = n - 1 - j - ii; return x >= 0 && x < n; }
    if (dir == 2) { x = n2 - 1 - ii; y = j; return x >= 0 && x < n; }
    y = m2 - 1 - ii; x = j; return y >= 0 && y < m;
}

struct CombMom4 {
    double mean = 0, M2 = 0, M3 = 0, M4 = 0;
    unsigned long long n = 0;
    __device__ __forceinline__ void add(double x) {
        if (isnan(x) || x > FLT_MAX || x < -FLT_MAX) return;
        const unsigned long long n1 = n;
        n = n + 1;
        const double dn = (double)n;
        const double delta = __dsub_rn(x, mean);
        const double delta_n = __ddiv_rn(delta, dn);
        const double delta_n2 = __dmul_rn(delta_n, delta_n);
        const double term1 = __dmul_rn(__dmul_rn(delta, delta_n), (double)n1);
        mean = __dadd_rn(mean, delta_n);
        // size_t arithmetic of the reference: n*n - 3n + 3 and n - 2 (wraps at n = 1)
        const double c4 = (double)(n * n - 3 * n + 3);
        const double c3 = (double)(n - 2);
        M4 = __dsub_rn(__dadd_rn(__dadd_rn(M4, __dmul_rn(__dmul_rn(term1, delta_n2), c4)),
                                 __dmul_rn(__dmul_rn(6.0, delta_n2), M2)),
                       __dmul_rn(__dmul_rn(4.0, delta_n), M3));
        M3 = __dsub_rn(__dadd_rn(M3, __dmul_rn(__dmul_rn(term1, delta_n), c3)), __dmul_rn(__dmul_rn(3.0, delta_n), M2));
        M2 = __dadd_rn(M2, term1);
    }
};

__global__ void __launch_bounds__(128) k_comb(const double *__restrict__ arena, const Plane *__restrict__ planes,
                                              const FJob *__restrict__ jobs, double *__restrict__ feat) {
    __shared__ double M[4][4][20];  // dir, moment, sample
    __shared__ int nsamp;
    const FJob J = jobs[blockIdx.x];
    const Plane P = planes[J.plane];
    const long long m = P.h, n = P.w, n2 = n / 2, m2 = m / 2;
    const double *p = arena + P.off;
    if (threadIdx.x == 0) {
        double step = (double)m / 10.0;
        if (step < 1.0) step = 1.0;
        int k = 0;
        for (double mp = 1.0 - m; mp <= m; mp += step) k++;
        nsamp = k < 20 ? k : 20;
    }
    for (int i = threadIdx.x; i < 4 * 4 * 20; i += blockDim.x) (&M[0][0][0])[i] = 0.0;
    __syncthreads();
    for (int line = threadIdx.x; line < 4 * nsamp; line += blockDim.x) {
        const int dir = line / nsamp, si = line % nsamp;
        double step = (double)m / 10.0;
        if (step < 1.0) step = 1.0;
        double mp = 1.0 - m;
        for (int q = 0; q < si; q++) mp += step;  // same accumulation as the reference loop
        const long long ii = llround(mp);
        const long long len = (dir == 3) ? n : m;
        CombMom4 mm;
        for (long long j = 0; j < len; j++) {
            long long y, x;
            if (comb_pixel(dir, j, ii, m, n, n2, m2, y, x)) mm.add(p[y * n + x]);
        }
        const double nn = (double)mm.n;
        M[dir][0][si] = mm.mean;
        M[dir][1][si] = mm.n > 2 ? sqrt(__ddiv_rn(mm.M2, (double)(mm.n - 1))) : 0.0;
        M[dir][2][si] = mm.n > 3 ? __ddiv_rn(__dmul_rn(sqrt(nn), mm.M3), pow(mm.M2, 1.5)) : 0.0;
        M[dir][3][si] = mm.n > 4 ? __ddiv_rn(__dmul_rn(nn, mm.M4), __dmul_rn(mm.M2, mm.M2)) : 0.0;
    }
    __syncthreads();
    if (threadIdx.x < 16) {
        const int dir = threadIdx.x / 4, a = threadIdx.x % 4;
        double lo = 10E200, hi = -10E200;
        for (int b = 0; b < 20; b++) {
            double v = M[dir][a][b];
            if (v > hi) hi = v;
            if (v < lo) lo = v;
        }
        const double sc = hist_scale(lo, hi, 3);
        double bins[3] = {0, 0, 0};
        for (int b = 0; b < 20; b++) bins[hist_bin(M[dir][a][b], lo, sc, 3)] += 1.0;
        // raw position (dir*4 + a)*3 + bin, permuted by vd_Comb4Moments
        const int perm[48] = {45, 46, 47, 36, 37, 38, 42, 43, 44, 39, 40, 41, 33, 34, 35, 24, 25, 26, 30, 31, 32, 27, 28, 29,
                              9, 10, 11, 0, 1, 2, 6, 7, 8, 3, 4, 5, 21, 22, 23, 12, 13, 14, 18, 19, 20, 15, 16, 17};
        for (int b = 0; b < 3; b++) {
            const int raw = (dir * 4 + a) * 3 + b;
            for (int o = 0; o < 48; o++)
                if (perm[o] == raw) feat[J.out + o] = bins[b];
        }
    }
}

void launch_comb(Ctx &c, const double *arena, const Plane *planes, const FJob *jobs, int njobs, double *feat) {
    if (njobs <= 0) return;
    WC_LAUNCH(c);
    k_comb<<<njobs, 128, 0, c.st>>>(arena, planes, jobs, feat);
}

// ---------------------------------------------------------------- Radon
// cos/sin of (theta*M_PI)/180 for theta = 0, 45, 90, 135, from the host libm
// (radon.cpp:51-55), so the sub-pixel bin split matches the CPU arithmetic.
__constant__ double c_radon_cs[8];
void set_radon_table(const double *cs8) { cudaMemcpyToSymbol(c_radon_cs, cs8, 8 * sizeof(double)); }

// ImageMatrix::RadonTransform2D + radon (MATLAB algorithm: 2x2 sub-pixels,
// linear split between two bins) + vd_RadonTextures, src/cmatrix.cpp:1463-1514,
// src/transforms/radon.cpp:14-115.  One CTA per (plane, angle); projections in
// shared memory, then a 3-bin histogram per angle.
__device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }

// R = double: FP64 form.  R = float (mixed form): FP32 projections and splits;
// the bin of a sub-pixel comes from an FP32 estimate of its position, and from
// the exact FP64 position whenever the estimate lies within 4e-3 of a bin
// boundary (the estimate's error is below 1e-3 for images up to 2048 px), so
// every sub-pixel lands in the bin the FP64 form gives it.
// a pixel in the projection's type; to float from the bits (the conversion
// instruction issues on the FP64 pipe)
template <typename R> __device__ __forceinline__ R to_r(double x);
template <> __device__ __forceinline__ float to_r<float>(double x) { return f32_of(x); }
template <> __device__ __forceinline__ double to_r<double>(double x) { return x; }

// One sub-pixel's bin and split in FP64, as the reference computes them (the
// FP64 form's every sub-pixel, the FP32 form's near-boundary ones); a call, so
// that the FP32 form's common path issues none of these FP64 instructions.
template <typename R> struct RadonSplit {
    int rl;
    R pix, pl;
};
template <typename R>
static __device__ __noinline__ RadonSplit<R> radon_exact(int kx, int ky, double cs, double sn, int rFirst, double pd) {
    const double xT = (double)kx * 0.25, yT = (double)ky * 0.25;
    const double ri = __dadd_rn(__dsub_rn(__dmul_rn(xT, cs), (double)rFirst), __dmul_rn(yT, sn));
    RadonSplit<R> r;
    r.rl = (int)ri;
    const double pdq = pd * 0.25;
    r.pix = to_r<R>(pdq);
    r.pl = (R)__dmul_rn(pdq, __dadd_rn(__dsub_rn(1.0, ri), (double)r.rl));
    return r;
}

// x == 0.0 (either sign) from the bits, off the FP64 pipe
__device__ __forceinline__ bool is_zero(double x) { return (__double_as_longlong(x) << 1) == 0; }

template <typename R>
__global__ void __launch_bounds__(1024) k_radon(const double *__restrict__ arena, const Plane *__restrict__ planes, const FJob *__restrict__ jobs,
                        double *__restrict__ feat, int rsize_max) {
    extern __shared__ __align__(16) unsigned char rsm[];
    R *pr = (R *)rsm;
    __shared__ double sh[32];
    const FJob J = jobs[blockIdx.y];
    const Plane P = planes[J.plane];
    const int W = P.w, H = P.h, ang = blockIdx.x;
    const int rLast = (int)ceil(sqrt(pow((double)(W - 1 - (W - 1) / 2), 2) + pow((double)(H - 1 - (H - 1) / 2), 2))) + 1;
    const int rFirst = -rLast, rSize = rLast - rFirst + 1;
    const int xo = (W - 1) / 2, yo = (H - 1) / 2;
    for (int i = threadIdx.x; i < rSize; i += blockDim.x) pr[i] = (R)0;
    __syncthreads();
    const double cs = c_radon_cs[2 * ang], sn = c_radon_cs[2 * ang + 1];
    const double *p = arena + P.off;
    // Sub-pixel lines along which the bin index is constant up to rounding:
    // columns (0 deg), rows (90 deg), diagonals (45 deg), anti-diagonals (135 deg).
    // Each sub-pixel's split is computed exactly as the reference does; a
    // thread adds its run to shared memory only when the bin changes.
    const int NX = 2 * W, NY = 2 * H;
    int nlines, dn, dm;
    if (ang == 0) { nlines = NX; dn = 0; dm = 1; }
    else if (ang == 2) { nlines = NY; dn = 1; dm = 0; }
    else if (ang == 1) { nlines = NX + NY - 1; dn = 1; dm = 1; }
    else { nlines = NX + NY - 1; dn = 1; dm = -1; }
    for (int line = threadIdx.x; line < nlines; line += blockDim.x) {
        int n, m;
        if (ang == 0) { n = line; m = 0; }
        else if (ang == 2) { n = 0; m = line; }
        else if (ang == 1) { if (line < NX) { n = line; m = 0; } else { n = 0; m = line - NX + 1; } }
        else { if (line < NY) { n = 0; m = line; } else { n = line - NY + 1; m = NY - 1; } }
        int cur = -1;
        R lo = 0, hi = 0;
        if (ang == 0 || ang == 2) {
            // columns at 0 deg, rows at 90 deg: the bin position is a rounded,
            // monotone function of the one coordinate that moves along the line
            // (cos 90 deg is 6e-17, not 0), so equal values at both ends mean it
            // is the same for every sub-pixel: split with one fraction
            const int n1 = ang == 0 ? n : NX - 1, m1 = ang == 0 ? NY - 1 : m;
            const double xa = -xo - 0.25 + 0.5 * n, ya = -yo - 0.25 + 0.5 * (NY - 1 - m);
            const double xb = -xo - 0.25 + 0.5 * n1, yb = -yo - 0.25 + 0.5 * (NY - 1 - m1);
            const double ra = __dadd_rn(__dsub_rn(__dmul_rn(xa, cs), (double)rFirst), __dmul_rn(ya, sn));
            const double rb = __dadd_rn(__dsub_rn(__dmul_rn(xb, cs), (double)rFirst), __dmul_rn(yb, sn));
            if (ra == rb) {
                const int rl = (int)ra;
                const R fr = (R)__dadd_rn(__dsub_rn(1.0, ra), (double)rl);
                for (; n >= 0 && n < NX && m >= 0 && m < NY; n += dn, m += dm) {
                    const double pd = p[(long long)(m / 2) * W + n / 2];
                    if (is_zero(pd)) continue;
                    const R pix = to_r<R>(pd) * (R)0.25;
                    const R pl = rmul(pix, fr);  // no contraction into the sum (the FP64 form's rounding)
                    lo += pl;
                    hi += pix - pl;
                }
                if (rl >= 0) {
                    atomicAdd(&pr[rl], lo);
                    atomicAdd(&pr[rl + 1], hi);
                }
                continue;
            }
        }
        const float csf = (float)cs, snf = (float)sn, rff = (float)rFirst;
        for (; n >= 0 && n < NX && m >= 0 && m < NY; n += dn, m += dm) {
            const double pd = p[(long long)(m / 2) * W + n / 2];
            if (is_zero(pd)) continue;
            // sub-pixel centre -xo - 0.25 + 0.5 n (and likewise y): a multiple of 0.25,
            // exact as k / 4 with an integer k in float and in double alike
            const int kx = 2 * n - 4 * xo - 1, ky = 2 * (NY - 1 - m) - 4 * yo - 1;
            int rl;
            R pix, pl;
            bool exact = sizeof(R) == 8;
            if (!exact) {
                const float rif = fmaf((float)ky * 0.25f, snf, fmaf((float)kx * 0.25f, csf, -rff));
                const float fl = floorf(rif), fr = rif - fl;
                if (fr < 4e-3f || fr > 1.f - 4e-3f) exact = true;
                else {
                    rl = (int)fl;
                    pix = to_r<R>(pd) * (R)0.25;
                    pl = rmul(pix, (R)(1.f - fr));
                }
            }
            if (exact) {
                const RadonSplit<R> e = radon_exact<R>(kx, ky, cs, sn, rFirst, pd);
                rl = e.rl;
                pix = e.pix;
                pl = e.pl;
            }
            if (rl != cur) {
                if (cur >= 0) {
                    atomicAdd(&pr[cur], lo);
                    atomicAdd(&pr[cur + 1], hi);
                }
                cur = rl;
                lo = 0;
                hi = 0;
            }
            lo += pl;
            hi += pix - pl;
        }
        if (cur >= 0) {
            atomicAdd(&pr[cur], lo);
            atomicAdd(&pr[cur + 1], hi);
        }
    }
    __syncthreads();
    double lo = 10E200, hi = -10E200;
    for (int i = threadIdx.x; i < rSize; i += blockDim.x) {
        lo = fmin(lo, (double)pr[i]);
        hi = fmax(hi, (double)pr[i]);
    }
    lo = block_min(lo, sh);
    hi = block_max(hi, sh);
    __shared__ unsigned int bins[3];
    if (threadIdx.x < 3) bins[threadIdx.x] = 0;
    __syncthreads();
    const double sc = hist_scale(lo, hi, 3);
    for (int i = threadIdx.x; i < rSize; i += blockDim.x) atomicAdd(&bins[hist_bin((double)pr[i], lo, sc, 3)], 1u);
    __syncthreads();
    if (threadIdx.x < 3) {
        // raw index ang*3 + b, permuted by vd_RadonTextures: out = [0 1 2 9 10 11 3 4 5 6 7 8]
        const int raw = ang * 3 + threadIdx.x;
        const int dst = raw < 3 ? raw : (raw >= 9 ? raw - 6 : raw + 3);
        feat[J.out + dst] = (double)bins[threadIdx.x];
    }
}

void launch_radon(Ctx &c, const double *arena, const Plane *planes, const FJob *jobs, int njobs, int maxw, int maxh,
                  double *feat) {
    if (njobs <= 0) return;
    int rLast = (int)ceil(sqrt(pow((double)(maxw - 1 - (maxw - 1) / 2), 2) + pow((double)(maxh - 1 - (maxh - 1) / 2), 2))) + 1;
    int rsize = 2 * rLast + 1;
    WC_LAUNCH(c);
    if (c.prec == WC_PREC_MIXED) k_radon<float><<<dim3(4, njobs), 1024, rsize * sizeof(float), c.st>>>(arena, planes, jobs, feat, rsize);
    else k_radon<double><<<dim3(4, njobs), 1024, rsize * sizeof(double), c.st>>>(arena, planes, jobs, feat, rsize);
}

// ---------------------------------------------------------------- Chebyshev coefficients
// ImageMatrix::ChebyshevStatistics2D (N = min(20, W, H), 32 bins),
// src/cmatrix.cpp:1274-1281, with Chebyshev2D (src/transforms/chebyshev.cpp:118-165):
// C[j][k] = sum_y B_k(y) * sum_x I(y,x) A_j(x), then a 32-bin histogram of the
// N*N coefficients.  A/B tables (T_j(x)/W scaled, halved) come from the host.
__global__ void __launch_bounds__(512) k_chebcoef(const double *__restrict__ arena, const Plane *__restrict__ planes, const FJob *__restrict__ jobs,
                           const double *__restrict__ tabs, const long long *__restrict__ tab_off,
                           double *__restrict__ mid_ws, const long long *__restrict__ mid_off, double *__restrict__ feat) {
    __shared__ double C[400];
    __shared__ double sh[32];
    const FJob J = jobs[blockIdx.x];
    const Plane P = planes[J.plane];
    const int W = P.w, H = P.h;
    int N = 20;
    if (N > min(W, H)) N = min(W, H);
    const double *TA = tabs + tab_off[2 * blockIdx.x], *TB = tabs + tab_off[2 * blockIdx.x + 1];
    const double *p = arena + P.off;
    double *mid = mid_ws + mid_off[blockIdx.x];  // H x N
    for (int q = threadIdx.x; q < H * N; q += blockDim.x) {
        const int y = q / N, j = q - y * N;
        const double *row = p + (long long)y * W;
        double s = 0;
        for (int x = 0; x < W; x++) s = __dadd_rn(s, __dmul_rn(row[x], TA[(long long)x * N + j]));
        mid[q] = s;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < N * N; q += blockDim.x) {
        const int j = q / N, k = q - j * N;
        double s = 0;
        for (int y = 0; y < H; y++) s = __dadd_rn(s, __dmul_rn(mid[(long long)y * N + j], TB[(long long)y * N + k]));
        C[q] = s;
    }
    __syncthreads();
    double lo = DBL_MAX, hi = -DBL_MAX;
    for (int q = threadIdx.x; q < N * N; q += blockDim.x) {
        lo = fmin(lo, C[q]);
        hi = fmax(hi, C[q]);
    }
    lo = block_min(lo, sh);
    hi = block_max(hi, sh);
    __shared__ unsigned int bins[32];
    if (threadIdx.x < 32) bins[threadIdx.x] = 0;
    __syncthreads();
    const double sc = hist_scale(lo, hi, 32);
    for (int q = threadIdx.x; q < N * N; q += blockDim.x) atomicAdd(&bins[hist_bin(C[q], lo, sc, 32)], 1u);
    __syncthreads();
    if (threadIdx.x < 32) feat[J.out + threadIdx.x] = (double)bins[threadIdx.x];
}

void launch_chebcoef(Ctx &c, const double *arena, const Plane *planes, const FJob *jobs, int njobs, const double *tabs,
                     const long long *tab_off, double *mid_ws, const long long *mid_off, double *feat) {
    if (njobs <= 0) return;
    WC_LAUNCH(c);
    k_chebcoef<<<njobs, 512, 0, c.st>>>(arena, planes, jobs, tabs, tab_off, mid_ws, mid_off, feat);
}

}  // namespace wc
