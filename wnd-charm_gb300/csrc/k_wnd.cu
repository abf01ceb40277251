// WND-5 with the CLI's semantics:
//   TrainingSet::normalize        src/wndchrm_src/TrainingSet.cpp:2090-2123
//   TrainingSet::SetFisherScores  src/wndchrm_src/TrainingSet.cpp:2183-2324 (Fisher part + threshold)
//   signatures::normalize         src/wndchrm_src/signatures.cpp:196-215
//   TrainingSet::classify2        src/wndchrm_src/TrainingSet.cpp:2429-2586
// The distance d(t,s) = sum_f w_f^2 (t_f - x_sf)^2 runs over the features with
// w_f >= DBL_EPSILON only (the reference skips the others), skipping terms with
// |t_f - x_sf| < DBL_EPSILON, in ascending feature order with separate
// multiply and add, as the reference accumulates it.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/wndcharm_gb300.h"
#include "kcommon.cuh"
#include "wc_features.h"

struct wc_engine;
namespace wc {
int engine_device(wc_engine *E, cudaStream_t *st, long long **launches);
int engine_precision(const wc_engine *E);
int engine_sms(const wc_engine *E);
}

namespace wc {

// TrainingSet::normalize + SetFisherScores over X (N x F, row-major), read a
// row at a time: a block takes 32 consecutive features (one per lane, so a
// warp reads 256 contiguous bytes of a row) and one of R contiguous ranges of
// rows (warp w of the block its rows w, w + 8, ...); per-range partial results
// go to global memory and are combined in range order, so every result is
// the same from run to run.

#define FIT_U 8  // rows per warp and iteration

// per-range min / max of each feature, skipping NaN and |v| > FLT_MAX
__global__ void __launch_bounds__(256) k_wnd_fit_minmax(const double *__restrict__ X, int N, int F, int rows_per,
                                                        double *__restrict__ pmin, double *__restrict__ pmax) {
    __shared__ double smn[8][32], smx[8][32];
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const int f = blockIdx.x * 32 + lane, r = blockIdx.y;
    const int s0 = r * rows_per, s1 = min(N, s0 + rows_per);
    double mn = FLT_MAX, mx = -FLT_MAX;
    if (f < F)
        for (int s = s0 + wp; s < s1; s += 8 * FIT_U) {
            // FIT_U rows' loads in flight before any is used
            double v[FIT_U];
#pragma unroll
            for (int u = 0; u < FIT_U; u++) v[u] = s + 8 * u < s1 ? X[(long long)(s + 8 * u) * F + f] : NAN;
#pragma unroll
            for (int u = 0; u < FIT_U; u++) {
                if (isnan(v[u]) || v[u] > FLT_MAX || v[u] < -FLT_MAX) continue;
                mn = fmin(mn, v[u]);
                mx = fmax(mx, v[u]);
            }
        }
    smn[wp][lane] = mn;
    smx[wp][lane] = mx;
    __syncthreads();
    if (wp == 0 && f < F) {
        for (int k = 1; k < 8; k++) {
            mn = fmin(mn, smn[k][lane]);
            mx = fmax(mx, smx[k][lane]);
        }
        pmin[(long long)r * F + f] = mn;
        pmax[(long long)r * F + f] = mx;
    }
}

__global__ void k_wnd_fit_minmax_final(const double *__restrict__ pmin, const double *__restrict__ pmax, int R, int F,
                                       double *__restrict__ mins, double *__restrict__ maxs) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= F) return;
    double mn = FLT_MAX, mx = -FLT_MAX;
    for (int r = 0; r < R; r++) {
        mn = fmin(mn, pmin[(long long)r * F + f]);
        mx = fmax(mx, pmax[(long long)r * F + f]);
    }
    mins[f] = mn;
    maxs[f] = mx;
}

// training rows per label: cnt[0] those with any label (y != 0), cnt[c] class c
__global__ void k_wnd_fit_count(const int *__restrict__ y, int N, int C, long long *__restrict__ cnt) {
    __shared__ unsigned int sc[17];
    if (threadIdx.x <= 16) sc[threadIdx.x] = 0;
    __syncthreads();
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < N; s += gridDim.x * blockDim.x) {
        const int c = y[s];
        if (c) atomicAdd(&sc[0], 1u);
        if (c >= 1 && c <= C) atomicAdd(&sc[c], 1u);
    }
    __syncthreads();
    if (threadIdx.x <= 16 && sc[threadIdx.x]) atomicAdd((unsigned long long *)&cnt[threadIdx.x], sc[threadIdx.x]);
}

// second = 0: per-range sums of the normalised values, slot 0 over every
// labelled row, slot c over class c; second = 1: per-range sums of squared
// deviations from the class means (mean[c * F + f])
__global__ void __launch_bounds__(256) k_wnd_fit_moments(const double *__restrict__ X, const int *__restrict__ y, int N,
                                                         int F, int C, int rows_per, const double *__restrict__ mins,
                                                         const double *__restrict__ maxs,
                                                         const double *__restrict__ mean, int second,
                                                         double *__restrict__ part) {
    __shared__ double acc[8][17][32];
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const int f = blockIdx.x * 32 + lane, r = blockIdx.y;
    const int s0 = r * rows_per, s1 = min(N, s0 + rows_per);
    for (int c = 0; c <= C; c++) acc[wp][c][lane] = 0.0;
    if (f < F) {
        const double mn = mins[f], mx = maxs[f];
        const double2 rc = wnd_recip(mn, mx);
        for (int s = s0 + wp; s < s1; s += 8 * FIT_U) {
            // FIT_U rows' loads in flight, then added in row order
            double xv[FIT_U];
            int cv[FIT_U];
#pragma unroll
            for (int u = 0; u < FIT_U; u++) {
                const bool in = s + 8 * u < s1;
                xv[u] = in ? X[(long long)(s + 8 * u) * F + f] : 0.0;
                cv[u] = in ? y[s + 8 * u] : 0;
            }
#pragma unroll
            for (int u = 0; u < FIT_U; u++) {
                const int c = cv[u];
                const double v = wnd_norm(xv[u], mn, mx, rc);
                if (!second) {
                    if (c) acc[wp][0][lane] += v;
                    if (c >= 1 && c <= C) acc[wp][c][lane] += v;
                } else if (c >= 1 && c <= C) {
                    const double d = v - mean[(long long)c * F + f];
                    acc[wp][c][lane] += d * d;
                }
            }
        }
    }
    __syncthreads();
    if (wp == 0 && f < F)
        for (int c = 0; c <= C; c++) {
            double t = acc[0][c][lane];
            for (int k = 1; k < 8; k++) t += acc[k][c][lane];
            part[((long long)r * (C + 1) + c) * F + f] = t;
        }
}

// combine the ranges: class means (second = 0) into mean[c * F + f]; or
// (second = 1) the Fisher score, between-class variance of the class means
// over the mean within-class variance (0 for classes of <= 2 rows), floor 1e-6
__global__ void k_wnd_fit_combine(const double *__restrict__ part, int R, int F, int C,
                                  const long long *__restrict__ cnt, int second, double *__restrict__ mean,
                                  double *__restrict__ w) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= F) return;
    if (!second) {
        for (int c = 0; c <= C; c++) {
            double t = 0;
            for (int r = 0; r < R; r++) t += part[((long long)r * (C + 1) + c) * F + f];
            mean[(long long)c * F + f] = cnt[c] ? t / cnt[c] : 0.0;
        }
        return;
    }
    const double mean_all = mean[f];
    double dev = 0, var = 0;
    for (int c = 1; c <= C; c++) {
        double m2 = 0;
        for (int r = 0; r < R; r++) m2 += part[((long long)r * (C + 1) + c) * F + f];
        dev += pow(mean[(long long)c * F + f] - mean_all, 2);
        var += cnt[c] > 2 ? m2 / (cnt[c] - 1) : 0.0;
    }
    if (C > 1) {
        dev /= (C - 1);
        var /= C;
    } else {
        dev = 0;
    }
    if (var < 0.000001) var = 0.000001;
    w[f] = dev / var;
}

// the ranges' partial sums added in range order: out[c * F + f]
__global__ void k_wnd_fit_rsum(const double *__restrict__ part, int R, int F, int C, double *__restrict__ out) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= F) return;
    for (int c = 0; c <= C; c++) {
        double t = 0;
        for (int r = 0; r < R; r++) t += part[((long long)r * (C + 1) + c) * F + f];
        out[(long long)c * F + f] = t;
    }
}

// gather the kept features, normalised: Xc is K x rows (column-major per row
// set) so lanes reading consecutive rows coalesce.
__global__ void k_wnd_gather(const double *__restrict__ X, int rows, int F, const int *__restrict__ keep, int K,
                             const double *__restrict__ mins, const double *__restrict__ maxs,
                             const double2 *__restrict__ rec, double *__restrict__ Xc) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= (long long)rows * K) return;
    const int k = (int)(q / rows), s = (int)(q - (long long)k * rows);
    const int f = keep[k];
    const double mn = mins[f], mx = maxs[f];
    Xc[(long long)k * rows + s] = wnd_norm(X[(long long)s * F + f], mn, mx, rec[f]);
}

// rows of X (by index) gathered and normalised into the FP64 kernel's
// column-major layout, Xc[k * n + i]
__global__ void k_wnd_gather_rows(const double *__restrict__ X, const int *__restrict__ rowsel, int n, int F,
                                  const int *__restrict__ keep, int K, const double *__restrict__ mins,
                                  const double *__restrict__ maxs, const double2 *__restrict__ rec,
                                  double *__restrict__ Xc) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= (long long)n * K) return;
    const int k = (int)(q / n), i = (int)(q - (long long)k * n);
    const int f = keep[k];
    const double mn = mins[f], mx = maxs[f];
    Xc[(long long)k * n + i] = wnd_norm(X[(long long)rowsel[i] * F + f], mn, mx, rec[f]);
}

// rows normalised against (mins, maxs), elementwise
__global__ void k_wnd_normalize(const double *__restrict__ X, long long n, int F, const double *__restrict__ mins,
                                const double *__restrict__ maxs, const double2 *__restrict__ rec,
                                double *__restrict__ out) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n * F;
         q += (long long)gridDim.x * blockDim.x) {
        const int f = (int)(q % F);
        out[q] = wnd_norm(X[q], mins[f], maxs[f], rec[f]);
    }
}

// the per-feature reciprocal pairs wnd_norm takes, from the range
__global__ void k_wnd_recip(const double *__restrict__ mins, const double *__restrict__ maxs, int F,
                            double2 *__restrict__ rec) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f < F) rec[f] = wnd_recip(mins[f], maxs[f]);
}

__global__ void k_wnd_scatter_rows(const int *__restrict__ rowsel, int n, int C, const double *__restrict__ sp,
                                   const int *__restrict__ spred, const double *__restrict__ snorm,
                                   double *__restrict__ probs, int *__restrict__ pred, double *__restrict__ norm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int t = rowsel[i];
    for (int c = 0; c < C; c++) probs[(long long)t * C + c] = sp[(long long)i * C + c];
    pred[t] = spred[i];
    norm[t] = snorm[i];
}

#define WT 64
#define WK 16
// distances for a 64-test x 64-train tile, then per-class sums of d^-5 in
// ascending train order for each test row; CTA (tile_t, chunk) covers train
// rows [chunk*per, (chunk+1)*per).
__global__ void __launch_bounds__(256) k_wnd_dist(const double *__restrict__ Tc, int T, const double *__restrict__ Xc, int N,
                                                  const int *__restrict__ y, const double *__restrict__ w2, int K, int C,
                                                  int per, double *__restrict__ psim, long long *__restrict__ pcnt) {
    __shared__ double Ts[WK][WT + 1], Xs[WK][WT + 1];
    __shared__ double D[WT][WT + 1];
    __shared__ double ws[WK];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int t0 = blockIdx.x * WT, chunk = blockIdx.y;
    const int sbeg = chunk * per, send = min(N, sbeg + per);
    double acc[16];  // per class, for test row t0 + threadIdx.x (threads < 64)
    long long cnt[16];
    for (int c = 0; c < 16; c++) { acc[c] = 0; cnt[c] = 0; }
    for (int s0 = sbeg; s0 < send; s0 += WT) {
        double d[4][4];
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) d[a][b] = 0.0;
        for (int k0 = 0; k0 < K; k0 += WK) {
            for (int q = threadIdx.x; q < WK * WT; q += blockDim.x) {
                int kk = q / WT, ii = q - kk * WT;
                int k = k0 + kk;
                Ts[kk][ii] = (k < K && t0 + ii < T) ? Tc[(long long)k * T + t0 + ii] : 0.0;
                Xs[kk][ii] = (k < K && s0 + ii < send) ? Xc[(long long)k * N + s0 + ii] : 0.0;
            }
            if (threadIdx.x < WK) ws[threadIdx.x] = (k0 + threadIdx.x < K) ? w2[k0 + threadIdx.x] : 0.0;
            __syncthreads();
            const int kend = min(WK, K - k0);
            for (int kk = 0; kk < kend; kk++) {
                const double wk = ws[kk];
#pragma unroll
                for (int a = 0; a < 4; a++) {
                    const double tv = Ts[kk][ty + 16 * a];
#pragma unroll
                    for (int b = 0; b < 4; b++) {
                        const double dist = fabs(__dsub_rn(tv, Xs[kk][tx + 16 * b]));
                        if (!(dist < DBL_EPSILON)) d[a][b] = __dadd_rn(d[a][b], __dmul_rn(wk, __dmul_rn(dist, dist)));
                    }
                }
            }
            __syncthreads();
        }
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) D[ty + 16 * a][tx + 16 * b] = d[a][b];
        __syncthreads();
        if (threadIdx.x < WT && t0 + threadIdx.x < T) {
            const int lim = min(WT, send - s0);
            for (int j = 0; j < lim; j++) {
                const double ds = D[threadIdx.x][j];
                if (ds < DBL_EPSILON) continue;
                const int c = y[s0 + j];
                if (c < 1 || c > C) continue;
                acc[c - 1] += pow(ds, -5.0);
                cnt[c - 1] += 1;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x < WT && t0 + threadIdx.x < T) {
        const long long base = ((long long)(t0 + threadIdx.x) * gridDim.y + chunk) * C;
        for (int c = 0; c < C; c++) {
            psim[base + c] = acc[c];
            pcnt[base + c] = cnt[c];
        }
    }
}

// Mixed form of the distance: features as FP32 pairs (hi + lo, 48 significant
// bits), every term w^2 (t - x)^2 formed and summed with error-free
// transformations (two-sum, FMA two-product), so d carries ~1e-14 relative
// error at FP32-pipe speed; d^-5 in FP64.  (The FP64 form above follows the
// reference's rounding and its |t - x| < DBL_EPSILON skip, which drops terms
// below 5e-32 w^2; the mixed form keeps them.)
__global__ void k_wnd_split(const double *__restrict__ src, long long n, float2 *__restrict__ dst) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double v = src[i];
        const float h = (float)v;
        dst[i] = make_float2(h, (float)(v - (double)h));
    }
}

// error-free transformations: explicit roundings (no contraction may fuse them)
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__global__ void __launch_bounds__(256) k_wnd_dist_df(const float2 *__restrict__ Tc, int T, const float2 *__restrict__ Xc,
                                                     int N, const int *__restrict__ y, const float2 *__restrict__ w2,
                                                     int K, int C, int per, double *__restrict__ psim,
                                                     long long *__restrict__ pcnt) {
    __shared__ float2 Ts[WK][WT + 1], Xs[WK][WT + 1];
    __shared__ double D[WT][WT + 1];
    __shared__ float2 ws[WK];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int t0 = blockIdx.x * WT, chunk = blockIdx.y;
    const int sbeg = chunk * per, send = min(N, sbeg + per);
    double acc[16];
    long long cnt[16];
    for (int c = 0; c < 16; c++) { acc[c] = 0; cnt[c] = 0; }
    for (int s0 = sbeg; s0 < send; s0 += WT) {
        float dh[4][4], dl[4][4];
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) dh[a][b] = dl[a][b] = 0.f;
        for (int k0 = 0; k0 < K; k0 += WK) {
            for (int q = threadIdx.x; q < WK * WT; q += blockDim.x) {
                const int kk = q / WT, ii = q - kk * WT, k = k0 + kk;
                Ts[kk][ii] = (k < K && t0 + ii < T) ? Tc[(long long)k * T + t0 + ii] : make_float2(0.f, 0.f);
                Xs[kk][ii] = (k < K && s0 + ii < send) ? Xc[(long long)k * N + s0 + ii] : make_float2(0.f, 0.f);
            }
            if (threadIdx.x < WK) ws[threadIdx.x] = (k0 + threadIdx.x < K) ? w2[k0 + threadIdx.x] : make_float2(0.f, 0.f);
            __syncthreads();
            const int kend = min(WK, K - k0);
            for (int kk = 0; kk < kend; kk++) {
                const float2 wk = ws[kk];
#pragma unroll
                for (int a = 0; a < 4; a++) {
                    const float2 tv = Ts[kk][ty + 16 * a];
#pragma unroll
                    for (int b = 0; b < 4; b++) {
                        const float2 xv = Xs[kk][tx + 16 * b];
                        float s, e;
                        two_sum(tv.x, -xv.x, s, e);  // t - x
                        e = __fadd_rn(e, __fsub_rn(tv.y, xv.y));
                        const float sh = __fadd_rn(s, e);
                        const float sl = __fsub_rn(e, __fsub_rn(sh, s));
                        const float p = __fmul_rn(sh, sh);  // (t - x)^2
                        float pe = __fmaf_rn(sh, sh, -p);
                        pe = __fmaf_rn(2.f * sh, sl, pe);
                        const float q = __fmul_rn(p, wk.x);  // w^2 (t - x)^2
                        float qe = __fmaf_rn(p, wk.x, -q);
                        qe = __fmaf_rn(p, wk.y, __fmaf_rn(pe, wk.x, qe));
                        float u, ue;  // accumulate
                        two_sum(dh[a][b], q, u, ue);
                        ue = __fadd_rn(ue, __fadd_rn(dl[a][b], qe));
                        dh[a][b] = __fadd_rn(u, ue);
                        dl[a][b] = __fsub_rn(ue, __fsub_rn(dh[a][b], u));
                    }
                }
            }
            __syncthreads();
        }
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) D[ty + 16 * a][tx + 16 * b] = (double)dh[a][b] + (double)dl[a][b];
        __syncthreads();
        if (threadIdx.x < WT && t0 + threadIdx.x < T) {
            const int lim = min(WT, send - s0);
            for (int j = 0; j < lim; j++) {
                const double ds = D[threadIdx.x][j];
                if (ds < DBL_EPSILON) continue;
                const int c = y[s0 + j];
                if (c < 1 || c > C) continue;
                const double d2 = ds * ds;
                acc[c - 1] += 1.0 / (d2 * d2 * ds);
                cnt[c - 1] += 1;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x < WT && t0 + threadIdx.x < T) {
        const long long base = ((long long)(t0 + threadIdx.x) * gridDim.y + chunk) * C;
        for (int c = 0; c < C; c++) {
            psim[base + c] = acc[c];
            pcnt[base + c] = cnt[c];
        }
    }
}

// per test row: sum the chunks in order, class means, argmax, probabilities
// (norm: the sum of the class similarities, classify2's normalization_factor)
__global__ void k_wnd_finish(const double *__restrict__ psim, const long long *__restrict__ pcnt, int T, int nchunk, int C,
                             double *__restrict__ probs, int *__restrict__ pred, double *__restrict__ norm) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    double sim[16];
    long long n[16];
    for (int c = 0; c < C; c++) { sim[c] = 0; n[c] = 0; }
    for (int ch = 0; ch < nchunk; ch++)
        for (int c = 0; c < C; c++) {
            sim[c] += psim[((long long)t * nchunk + ch) * C + c];
            n[c] += pcnt[((long long)t * nchunk + ch) * C + c];
        }
    int best = -1;
    double bestv = 0, tot = 0;
    for (int c = 0; c < C; c++) {
        if (n[c] == 0) continue;
        sim[c] /= (double)n[c];
        if (sim[c] > bestv) { bestv = sim[c]; best = c + 1; }
    }
    for (int c = 0; c < C; c++) tot += sim[c];
    for (int c = 0; c < C; c++) probs[(long long)t * C + c] = sim[c] / tot;
    pred[t] = best;
    norm[t] = tot;
}

// the chunks' per-class sums of d^-5 and counts, added in chunk order (the
// first half of k_wnd_finish), for an exchange across ranks
__global__ void k_wnd_sums(const double *__restrict__ psim, const long long *__restrict__ pcnt, int T, int nchunk, int C,
                           double *__restrict__ sums, long long *__restrict__ counts) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    for (int c = 0; c < C; c++) {
        double v = 0;
        long long n = 0;
        for (int ch = 0; ch < nchunk; ch++) {
            v += psim[((long long)t * nchunk + ch) * C + c];
            n += pcnt[((long long)t * nchunk + ch) * C + c];
        }
        sums[(long long)t * C + c] = v;
        counts[(long long)t * C + c] = n;
    }
}

// TrainingSet::ClassifyImage for WND-5 (src/wndchrm_src/TrainingSet.cpp:1603-1800),
// one thread per image over its `tiles` consecutive rows, in tile order:
// marginal probabilities summed as p / tiles (with max_tile, a tile whose
// predicted-class share p[pred] / sum of the other classes' p is the largest so
// far replaces the sums with its own p, the reference's rule), the mean
// normalisation factor, and the class of the largest sum (first one on ties,
// rank 1; a class below 1 from classify2 counts as 0).  The reference's share
// also adds p[0], an element classify2 never sets; it counts as 0 here.
__global__ void k_wnd_tiles(const double *__restrict__ probs, const int *__restrict__ pred,
                            const double *__restrict__ norm, int n_img, int tiles, int C, int max_tile,
                            double *__restrict__ iprobs, int *__restrict__ ipred, double *__restrict__ inorm) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n_img) return;
    double psum[17];
    for (int c = 1; c <= C; c++) psum[c] = 0.0;
    double best_share = 0.0, nf = 0.0;
    int predicted = 0, best_pred = 0;
    for (int k = 0; k < tiles; k++) {
        const long long t = (long long)g * tiles + k;
        const double *p = probs + t * C;  // class c at p[c - 1]
        predicted = pred[t] < 1 ? 0 : pred[t];
        const double pp = predicted ? p[predicted - 1] : 0.0;
        double sum_prob = 0.0;
        if (max_tile) {
            for (int c = 0; c <= C; c++)
                if (c != predicted) sum_prob += c ? p[c - 1] : 0.0;
            if (pp / sum_prob > best_share) {
                best_share = pp / sum_prob;
                best_pred = predicted;
            }
        }
        for (int c = 1; c <= C; c++) {
            if (max_tile && best_share == pp / sum_prob) psum[c] = p[c - 1];
            else psum[c] += p[c - 1] / (double)tiles;
        }
        nf += norm[t];
    }
    if (max_tile) predicted = best_pred;
    nf /= tiles;
    if (C > 1) {
        double mx = 0.0;
        for (int c = 1; c <= C; c++)
            if (psum[c] > mx) {
                mx = psum[c];
                predicted = c;
            }
    }
    for (int c = 1; c <= C; c++) iprobs[(long long)g * C + c - 1] = psum[c];
    ipred[g] = predicted;
    inorm[g] = nf;
}

}  // namespace wc

using namespace wc;

#define CKW(x)                                                                                        \
    do {                                                                                              \
        cudaError_t e_ = (x);                                                                         \
        if (e_ != cudaSuccess) { rc = set_err(WC_ERR_CUDA, "%s: %s", #x, cudaGetErrorString(e_)); goto done; } \
    } while (0)

// SetFisherScores' selection: every weight below the one at sorted
// (descending) rank floor(frac*F + 0.5) set to 0
static void fisher_threshold(double *weights, int F, double frac) {
    const int last = (int)std::floor((frac * (double)F) + 0.5);
    if (last >= F) return;
    std::vector<double> sw(weights, weights + F);
    std::nth_element(sw.begin(), sw.begin() + last, sw.end(), std::greater<double>());
    const double thr = sw[last];
    for (int f = 0; f < F; f++)
        if (weights[f] < thr) weights[f] = 0.0;
}

// normalize + SetFisherScores over device rows: dmin/dmax (device) get the
// per-feature range, weights (host) the thresholded Fisher scores
static int wnd_fit_dev(wc_engine *E, const double *dX, int N, int F, const int *dy, int C, double frac, double *weights,
                       double *dmin, double *dmax) {
    cudaStream_t st;
    long long *launches;
    int rc = engine_device(E, &st, &launches);
    if (rc) return rc;
    const int fb = (F + 31) / 32;
    const int R = std::max(1, std::min((N + 255) / 256, (8 * engine_sms(E) + fb - 1) / fb));
    const int rows_per = (N + R - 1) / R;
    double *dpmin = nullptr, *dpmax = nullptr, *dpart = nullptr, *dmean = nullptr, *dw = nullptr;
    long long *dcnt = nullptr;
    CKW(cudaMalloc(&dpmin, (size_t)R * F * sizeof(double)));
    CKW(cudaMalloc(&dpmax, (size_t)R * F * sizeof(double)));
    CKW(cudaMalloc(&dpart, (size_t)R * (C + 1) * F * sizeof(double)));
    CKW(cudaMalloc(&dmean, (size_t)(C + 1) * F * sizeof(double)));
    CKW(cudaMalloc(&dw, F * sizeof(double)));
    CKW(cudaMalloc(&dcnt, 17 * sizeof(long long)));
    CKW(cudaMemsetAsync(dcnt, 0, 17 * sizeof(long long), st));
    *launches += 7;
    k_wnd_fit_minmax<<<dim3(fb, R), 256, 0, st>>>(dX, N, F, rows_per, dpmin, dpmax);
    k_wnd_fit_minmax_final<<<(F + 255) / 256, 256, 0, st>>>(dpmin, dpmax, R, F, dmin, dmax);
    k_wnd_fit_count<<<std::min(1024, (N + 255) / 256), 256, 0, st>>>(dy, N, C, dcnt);
    k_wnd_fit_moments<<<dim3(fb, R), 256, 0, st>>>(dX, dy, N, F, C, rows_per, dmin, dmax, nullptr, 0, dpart);
    k_wnd_fit_combine<<<(F + 255) / 256, 256, 0, st>>>(dpart, R, F, C, dcnt, 0, dmean, nullptr);
    k_wnd_fit_moments<<<dim3(fb, R), 256, 0, st>>>(dX, dy, N, F, C, rows_per, dmin, dmax, dmean, 1, dpart);
    k_wnd_fit_combine<<<(F + 255) / 256, 256, 0, st>>>(dpart, R, F, C, dcnt, 1, dmean, dw);
    CKW(cudaGetLastError());
    CKW(cudaMemcpyAsync(weights, dw, F * sizeof(double), cudaMemcpyDeviceToHost, st));
    CKW(cudaStreamSynchronize(st));
    fisher_threshold(weights, F, frac);
done:
    cudaFree(dpmin);
    cudaFree(dpmax);
    cudaFree(dpart);
    cudaFree(dmean);
    cudaFree(dw);
    cudaFree(dcnt);
    return rc;
}

extern "C" int wc_wnd_fit(wc_engine *E, const double *train, int N, int F, const int *labels, int C, double frac,
                          double *weights, double *mins, double *maxs) {
    if (!E || !train || !labels || !weights || !mins || !maxs || N < 1 || F < 1 || C < 1 || C > 16)
        return set_err(WC_ERR_ARG, "wc_wnd_fit: bad arguments (C must be 1..16)");
    cudaStream_t st;
    long long *launches;
    int rc = engine_device(E, &st, &launches);
    if (rc) return rc;
    double *dX = nullptr, *dmin = nullptr, *dmax = nullptr;
    int *dy = nullptr;
    const size_t xb = (size_t)N * F * sizeof(double);
    CKW(cudaMalloc(&dX, xb));
    CKW(cudaMalloc(&dmin, F * sizeof(double)));
    CKW(cudaMalloc(&dmax, F * sizeof(double)));
    CKW(cudaMalloc(&dy, N * sizeof(int)));
    CKW(cudaMemcpyAsync(dX, train, xb, cudaMemcpyHostToDevice, st));
    CKW(cudaMemcpyAsync(dy, labels, N * sizeof(int), cudaMemcpyHostToDevice, st));
    if ((rc = wnd_fit_dev(E, dX, N, F, dy, C, frac, weights, dmin, dmax))) goto done;
    CKW(cudaMemcpyAsync(mins, dmin, F * sizeof(double), cudaMemcpyDeviceToHost, st));
    CKW(cudaMemcpyAsync(maxs, dmax, F * sizeof(double), cudaMemcpyDeviceToHost, st));
    CKW(cudaStreamSynchronize(st));
done:
    cudaFree(dX);
    cudaFree(dmin);
    cudaFree(dmax);
    cudaFree(dy);
    return rc;
}

extern "C" int wc_wnd_fit_device(wc_engine *E, const double *train, int N, int F, const int *labels, int C,
                                 double frac, double *weights, double *mins, double *maxs) {
    if (!E || !train || !labels || !weights || !mins || !maxs || N < 1 || F < 1 || C < 1 || C > 16)
        return set_err(WC_ERR_ARG, "wc_wnd_fit_device: bad arguments (C must be 1..16)");
    cudaStream_t st;
    long long *launches;
    int rc = engine_device(E, &st, &launches);
    if (rc) return rc;
    std::vector<double> w(F);
    if ((rc = wnd_fit_dev(E, train, N, F, labels, C, frac, w.data(), mins, maxs))) return rc;
    CKW(cudaMemcpyAsync(weights, w.data(), F * sizeof(double), cudaMemcpyHostToDevice, st));
    CKW(cudaStreamSynchronize(st));
done:
    return rc;
}

namespace wc {
int wnd_tc_classify(cudaStream_t st, long long *launches, int sms, const double *dX, int N, int F, const int *labels,
                    int C, const double *dT, int T, const std::vector<int> &keep, const std::vector<double> &w,
                    const double *dmin, const double *dmax, const double2 *drec, double *dprob, int *dpred,
                    double *dnorm, std::vector<int> &recheck, long long *info);
bool wnd_tc_supported(int K);
}  // namespace wc

namespace {

// what the last classification did (wc_wnd_last_stats)
thread_local long long g_last_stats[6] = {0, 0, 0, 0, 0, 0};

// device buffers freed together
struct WBufs {
    std::vector<void *> ptrs;
    template <typename T>
    int get(T **p, size_t bytes) {
        *p = nullptr;
        void *q = nullptr;
        if (cudaMalloc(&q, bytes ? bytes : 16) != cudaSuccess) {
            cudaGetLastError();
            return set_err(WC_ERR_NOMEM, "cudaMalloc of %zu bytes failed", bytes);
        }
        ptrs.push_back(q);
        *p = (T *)q;
        return WC_OK;
    }
    ~WBufs() {
        for (void *q : ptrs) cudaFree(q);
    }
};

#define CKR(x)                                                                                        \
    do {                                                                                              \
        cudaError_t e_ = (x);                                                                         \
        if (e_ != cudaSuccess) return set_err(WC_ERR_CUDA, "%s: %s", #x, cudaGetErrorString(e_));     \
    } while (0)

// The FP64 kernel (the reference's order and skips) for the test rows `rows`
// of dT; results scattered into dprob/dpred/dnorm.  chunks spread a few rows
// over the whole GPU.
int fp64_rows(cudaStream_t st, long long *launches, const double *dX, const double *dT, int N, int F, const int *dy,
              int C, const std::vector<int> &keep_h, const int *dkeep, const double *dw2, const double *dmin,
              const double *dmax, const double2 *drec, const std::vector<int> &rows, double *dprob, int *dpred, double *dnorm,
              bool all_rows) {
    const int K = (int)keep_h.size();
    const int n = (int)rows.size();
    if (!n) return WC_OK;
    WBufs B;
    double *dXc, *dTc, *dps, *sp, *sn;
    long long *dpc;
    int *drows, *spred;
    const int nchunk = all_rows ? std::max(1, std::min(64, (N + 4095) / 4096)) : std::max(1, std::min(512, N / 256));
    const int per = ((N + nchunk - 1) / nchunk + WT - 1) / WT * WT;
    int rc;
    if ((rc = B.get(&dXc, (size_t)N * std::max(K, 1) * 8)) || (rc = B.get(&dTc, (size_t)n * std::max(K, 1) * 8)) ||
        (rc = B.get(&dps, (size_t)n * nchunk * C * 8)) || (rc = B.get(&dpc, (size_t)n * nchunk * C * 8)) ||
        (rc = B.get(&sp, (size_t)n * C * 8)) || (rc = B.get(&sn, (size_t)n * 8)) || (rc = B.get(&drows, n * 4)) ||
        (rc = B.get(&spred, n * 4)))
        return rc;
    CKR(cudaMemcpyAsync(drows, rows.data(), n * 4, cudaMemcpyHostToDevice, st));
    if (K) {
        ++*launches;
        k_wnd_gather<<<(int)(((long long)N * K + 255) / 256), 256, 0, st>>>(dX, N, F, dkeep, K, dmin, dmax, drec,
                                                                            dXc);
        ++*launches;
        k_wnd_gather_rows<<<(int)(((long long)n * K + 255) / 256), 256, 0, st>>>(dT, drows, n, F, dkeep, K, dmin,
                                                                                     dmax, drec, dTc);
    }
    *launches += 3;
    k_wnd_dist<<<dim3((n + WT - 1) / WT, nchunk), 256, 0, st>>>(dTc, n, dXc, N, dy, dw2, K, C, per, dps, dpc);
    k_wnd_finish<<<(n + 127) / 128, 128, 0, st>>>(dps, dpc, n, nchunk, C, sp, spred, sn);
    k_wnd_scatter_rows<<<(n + 127) / 128, 128, 0, st>>>(drows, n, C, sp, spred, sn, dprob, dpred, dnorm);
    CKR(cudaGetLastError());
    CKR(cudaStreamSynchronize(st));
    return WC_OK;
}

}  // namespace

// classify2 over device-resident rows: dX (N x F), dT (T x F), labels / weights
// on the host, dmin / dmax on the device; probabilities, classes and
// normalisation factors to dprob / dpred / dnorm (device).
static int wnd_classify_dev(wc_engine *E, const double *dX, int N, int F, const int *labels, int C,
                            const double *weights, const double *dmin, const double *dmax, const double *dT, int T,
                            double *dprob, int *dpred, double *dnorm) {
    cudaStream_t st;
    long long *launches;
    int rc = engine_device(E, &st, &launches);
    if (rc) return rc;
    std::vector<int> keep;
    std::vector<double> w, w2;
    for (int f = 0; f < F; f++)
        if (!(weights[f] < DBL_EPSILON)) {
            keep.push_back(f);
            w.push_back(weights[f]);
            w2.push_back(std::pow(weights[f], 2));
        }
    const int K = (int)keep.size();
    const bool mixed = engine_precision(E) == WC_PREC_MIXED;
    WBufs B;
    int *dy, *dkeep;
    double *dw2;
    double2 *drec;
    if ((rc = B.get(&dy, N * 4)) || (rc = B.get(&dkeep, std::max(K, 1) * 4)) || (rc = B.get(&dw2, std::max(K, 1) * 8)) ||
        (rc = B.get(&drec, (size_t)F * 16)))
        return rc;
    ++*launches;
    k_wnd_recip<<<(F + 255) / 256, 256, 0, st>>>(dmin, dmax, F, drec);
    CKR(cudaMemcpyAsync(dy, labels, N * 4, cudaMemcpyHostToDevice, st));
    if (K) {
        CKR(cudaMemcpyAsync(dkeep, keep.data(), K * 4, cudaMemcpyHostToDevice, st));
        CKR(cudaMemcpyAsync(dw2, w2.data(), K * 8, cudaMemcpyHostToDevice, st));
    }
    for (int i = 0; i < 6; i++) g_last_stats[i] = 0;
    g_last_stats[2] = K;
    if (mixed && wnd_tc_supported(K)) {
        // tensor cores, then the FP64 kernel for the rows they cannot certify
        std::vector<int> rows;
        long long info[3] = {0, 0, 0};
        rc = wnd_tc_classify(st, launches, engine_sms(E), dX, N, F, labels, C, dT, T, keep, w, dmin, dmax, drec, dprob, dpred,
                             dnorm, rows, info);
        if (rc == WC_ERR_UNSUPPORTED) goto pairs;
        if (rc) return rc;
        g_last_stats[0] = 1;
        g_last_stats[1] = (long long)rows.size();
        g_last_stats[3] = info[0];
        g_last_stats[4] = info[1];
        g_last_stats[5] = info[2];
        return fp64_rows(st, launches, dX, dT, N, F, dy, C, keep, dkeep, dw2, dmin, dmax, drec, rows, dprob, dpred, dnorm,
                         false);
    }
pairs:
    if (mixed && K) {
        // pairs of floats on the CUDA cores (more features than the tensor-core digits allow)
        const int nchunk = std::max(1, std::min(64, (N + 4095) / 4096));
        const int per = ((N + nchunk - 1) / nchunk + WT - 1) / WT * WT;
        double *dXc, *dTc, *dps;
        long long *dpc;
        float2 *fX, *fT, *fw;
        if ((rc = B.get(&dXc, (size_t)N * K * 8)) || (rc = B.get(&dTc, (size_t)T * K * 8)) ||
            (rc = B.get(&dps, (size_t)T * nchunk * C * 8)) || (rc = B.get(&dpc, (size_t)T * nchunk * C * 8)) ||
            (rc = B.get(&fX, (size_t)N * K * 8)) || (rc = B.get(&fT, (size_t)T * K * 8)) || (rc = B.get(&fw, K * 8)))
            return rc;
        *launches += 7;
        k_wnd_gather<<<(int)(((long long)N * K + 255) / 256), 256, 0, st>>>(dX, N, F, dkeep, K, dmin, dmax, drec,
                                                                            dXc);
        k_wnd_gather<<<(int)(((long long)T * K + 255) / 256), 256, 0, st>>>(dT, T, F, dkeep, K, dmin, dmax, drec,
                                                                            dTc);
        k_wnd_split<<<1024, 256, 0, st>>>(dXc, (long long)N * K, fX);
        k_wnd_split<<<1024, 256, 0, st>>>(dTc, (long long)T * K, fT);
        k_wnd_split<<<1, 256, 0, st>>>(dw2, K, fw);
        k_wnd_dist_df<<<dim3((T + WT - 1) / WT, nchunk), 256, 0, st>>>(fT, T, fX, N, dy, fw, K, C, per, dps, dpc);
        k_wnd_finish<<<(T + 127) / 128, 128, 0, st>>>(dps, dpc, T, nchunk, C, dprob, dpred, dnorm);
        CKR(cudaGetLastError());
        CKR(cudaStreamSynchronize(st));
        return WC_OK;
    }
    {
        std::vector<int> all(T);
        for (int t = 0; t < T; t++) all[t] = t;
        return fp64_rows(st, launches, dX, dT, N, F, dy, C, keep, dkeep, dw2, dmin, dmax, drec, all, dprob, dpred, dnorm,
                         true);
    }
}

// classify2 for T test rows with host buffers; with tiles > 0 the rows are
// n = T / tiles images' tiles and ClassifyImage's per-image results are
// returned instead of the rows'.
static int wnd_classify(wc_engine *E, const double *train, int N, int F, const int *labels, int C,
                        const double *weights, const double *mins, const double *maxs, const double *test, int T,
                        double *probs, int *pred, int tiles, int max_tile, double *iprobs, int *ipred, double *inorm) {
    cudaStream_t st;
    long long *launches;
    int rc = engine_device(E, &st, &launches);
    if (rc) return rc;
    const int n_img = tiles > 0 ? T / tiles : 0;
    WBufs B;
    double *dX, *dT, *dmin, *dmax, *dprob, *dnorm, *diprob = nullptr, *dinorm = nullptr;
    int *dpred, *dipred = nullptr;
    if ((rc = B.get(&dX, (size_t)N * F * 8)) || (rc = B.get(&dT, (size_t)T * F * 8)) || (rc = B.get(&dmin, F * 8)) ||
        (rc = B.get(&dmax, F * 8)) || (rc = B.get(&dprob, (size_t)T * C * 8)) || (rc = B.get(&dpred, (size_t)T * 4)) ||
        (rc = B.get(&dnorm, (size_t)T * 8)))
        return rc;
    if (n_img && ((rc = B.get(&diprob, (size_t)n_img * C * 8)) || (rc = B.get(&dipred, (size_t)n_img * 4)) ||
                  (rc = B.get(&dinorm, (size_t)n_img * 8))))
        return rc;
    CKR(cudaMemcpyAsync(dX, train, (size_t)N * F * 8, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(dT, test, (size_t)T * F * 8, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(dmin, mins, F * 8, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(dmax, maxs, F * 8, cudaMemcpyHostToDevice, st));
    if ((rc = wnd_classify_dev(E, dX, N, F, labels, C, weights, dmin, dmax, dT, T, dprob, dpred, dnorm))) return rc;
    if (n_img) {
        ++*launches;
        k_wnd_tiles<<<(n_img + 127) / 128, 128, 0, st>>>(dprob, dpred, dnorm, n_img, tiles, C, max_tile, diprob, dipred,
                                                         dinorm);
        CKR(cudaGetLastError());
        CKR(cudaMemcpyAsync(iprobs, diprob, (size_t)n_img * C * 8, cudaMemcpyDeviceToHost, st));
        CKR(cudaMemcpyAsync(ipred, dipred, (size_t)n_img * 4, cudaMemcpyDeviceToHost, st));
        if (inorm) CKR(cudaMemcpyAsync(inorm, dinorm, (size_t)n_img * 8, cudaMemcpyDeviceToHost, st));
    } else {
        CKR(cudaMemcpyAsync(probs, dprob, (size_t)T * C * 8, cudaMemcpyDeviceToHost, st));
        CKR(cudaMemcpyAsync(pred, dpred, (size_t)T * 4, cudaMemcpyDeviceToHost, st));
    }
    CKR(cudaStreamSynchronize(st));
    return WC_OK;
}

extern "C" int wc_wnd_classify(wc_engine *E, const double *train, int N, int F, const int *labels, int C,
                               const double *weights, const double *mins, const double *maxs, const double *test, int T,
                               double *probs, int *pred) {
    if (!E || !train || !labels || !weights || !mins || !maxs || !test || !probs || !pred || N < 1 || F < 1 || T < 1 ||
        C < 1 || C > 16)
        return set_err(WC_ERR_ARG, "wc_wnd_classify: bad arguments (C must be 1..16)");
    return wnd_classify(E, train, N, F, labels, C, weights, mins, maxs, test, T, probs, pred, 0, 0, nullptr, nullptr,
                        nullptr);
}

// normalize + SetFisherScores on the training rows, then classify2 of the test
// rows, with host buffers: each array crosses to the GPU once (the test rows'
// copy overlaps the fit's kernels on a second stream)
extern "C" int wc_wnd_fit_classify(wc_engine *E, const double *train, int N, int F, const int *labels, int C,
                                   double frac, const double *test, int T, double *weights, double *mins,
                                   double *maxs, double *probs, int *pred) {
    if (!E || !train || !labels || !test || !weights || !mins || !maxs || !probs || !pred || N < 1 || F < 1 ||
        T < 1 || C < 1 || C > 16)
        return set_err(WC_ERR_ARG, "wc_wnd_fit_classify: bad arguments (C must be 1..16)");
    cudaStream_t st;
    long long *launches;
    int rc = engine_device(E, &st, &launches);
    if (rc) return rc;
    WBufs B;
    double *dX, *dT, *dmin, *dmax, *dprob, *dnorm;
    int *dy, *dpred;
    if ((rc = B.get(&dX, (size_t)N * F * 8)) || (rc = B.get(&dT, (size_t)T * F * 8)) || (rc = B.get(&dmin, F * 8)) ||
        (rc = B.get(&dmax, F * 8)) || (rc = B.get(&dprob, (size_t)T * C * 8)) || (rc = B.get(&dpred, (size_t)T * 4)) ||
        (rc = B.get(&dnorm, (size_t)T * 8)) || (rc = B.get(&dy, (size_t)N * 4)))
        return rc;
    cudaStream_t side = nullptr;
    cudaEvent_t ev = nullptr;
    CKR(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
    if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
        cudaStreamDestroy(side);
        return set_err(WC_ERR_CUDA, "cudaEventCreate failed");
    }
    struct Release {
        cudaStream_t s;
        cudaEvent_t e;
        ~Release() {
            cudaStreamSynchronize(s);
            cudaEventDestroy(e);
            cudaStreamDestroy(s);
        }
    } rel{side, ev};
    CKR(cudaMemcpyAsync(dX, train, (size_t)N * F * 8, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(dy, labels, (size_t)N * 4, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(dT, test, (size_t)T * F * 8, cudaMemcpyHostToDevice, side));
    CKR(cudaEventRecord(ev, side));
    if ((rc = wnd_fit_dev(E, dX, N, F, dy, C, frac, weights, dmin, dmax))) return rc;
    CKR(cudaStreamWaitEvent(st, ev, 0));
    if ((rc = wnd_classify_dev(E, dX, N, F, labels, C, weights, dmin, dmax, dT, T, dprob, dpred, dnorm))) return rc;
    CKR(cudaMemcpyAsync(mins, dmin, F * 8, cudaMemcpyDeviceToHost, st));
    CKR(cudaMemcpyAsync(maxs, dmax, F * 8, cudaMemcpyDeviceToHost, st));
    CKR(cudaMemcpyAsync(probs, dprob, (size_t)T * C * 8, cudaMemcpyDeviceToHost, st));
    CKR(cudaMemcpyAsync(pred, dpred, (size_t)T * 4, cudaMemcpyDeviceToHost, st));
    CKR(cudaStreamSynchronize(st));
    return WC_OK;
}

// classify2's per-class sums over this process's training rows (host
// buffers): sums[t * C + c - 1] = sum of d^-5 over the rows of class c with
// d >= DBL_EPSILON, counts[...] how many; the FP64 kernel's arithmetic.  Summed
// over shards of the training rows they give every shard's classify2.
extern "C" int wc_wnd_class_sums(wc_engine *E, const double *train, int N, int F, const int *labels, int C,
                                 const double *weights, const double *mins, const double *maxs, const double *test,
                                 int T, double *sums, long long *counts) {
    if (!E || !train || !labels || !weights || !mins || !maxs || !test || !sums || !counts || N < 1 || F < 1 ||
        T < 1 || C < 1 || C > 16)
        return set_err(WC_ERR_ARG, "wc_wnd_class_sums: bad arguments (C must be 1..16)");
    cudaStream_t st;
    long long *launches;
    int rc = engine_device(E, &st, &launches);
    if (rc) return rc;
    std::vector<int> keep;
    std::vector<double> w2;
    for (int f = 0; f < F; f++)
        if (!(weights[f] < DBL_EPSILON)) {
            keep.push_back(f);
            w2.push_back(std::pow(weights[f], 2));
        }
    const int K = (int)keep.size();
    const int nchunk = std::max(1, std::min(64, (N + 4095) / 4096));
    const int per = ((N + nchunk - 1) / nchunk + WT - 1) / WT * WT;
    WBufs B;
    double *dX, *dT, *dmin, *dmax, *dw2, *dXc, *dTc, *dps, *dsum;
    double2 *drec;
    long long *dpc, *dcnt;
    int *dy, *dkeep;
    if ((rc = B.get(&dX, (size_t)N * F * 8)) || (rc = B.get(&dT, (size_t)T * F * 8)) || (rc = B.get(&dmin, F * 8)) ||
        (rc = B.get(&dmax, F * 8)) || (rc = B.get(&drec, (size_t)F * 16)) || (rc = B.get(&dy, (size_t)N * 4)) ||
        (rc = B.get(&dkeep, std::max(K, 1) * 4)) || (rc = B.get(&dw2, std::max(K, 1) * 8)) ||
        (rc = B.get(&dXc, (size_t)N * std::max(K, 1) * 8)) || (rc = B.get(&dTc, (size_t)T * std::max(K, 1) * 8)) ||
        (rc = B.get(&dps, (size_t)T * nchunk * C * 8)) || (rc = B.get(&dpc, (size_t)T * nchunk * C * 8)) ||
        (rc = B.get(&dsum, (size_t)T * C * 8)) || (rc = B.get(&dcnt, (size_t)T * C * 8)))
        return rc;
    CKR(cudaMemcpyAsync(dX, train, (size_t)N * F * 8, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(dT, test, (size_t)T * F * 8, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(dmin, mins, F * 8, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(dmax, maxs, F * 8, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(dy, labels, (size_t)N * 4, cudaMemcpyHostToDevice, st));
    if (K) {
        CKR(cudaMemcpyAsync(dkeep, keep.data(), K * 4, cudaMemcpyHostToDevice, st));
        CKR(cudaMemcpyAsync(dw2, w2.data(), K * 8, cudaMemcpyHostToDevice, st));
        *launches += 3;
        k_wnd_recip<<<(F + 255) / 256, 256, 0, st>>>(dmin, dmax, F, drec);
        k_wnd_gather<<<(int)(((long long)N * K + 255) / 256), 256, 0, st>>>(dX, N, F, dkeep, K, dmin, dmax, drec,
                                                                            dXc);
        k_wnd_gather<<<(int)(((long long)T * K + 255) / 256), 256, 0, st>>>(dT, T, F, dkeep, K, dmin, dmax, drec,
                                                                            dTc);
    }
    *launches += 2;
    k_wnd_dist<<<dim3((T + WT - 1) / WT, nchunk), 256, 0, st>>>(dTc, T, dXc, N, dy, dw2, K, C, per, dps, dpc);
    k_wnd_sums<<<(T + 127) / 128, 128, 0, st>>>(dps, dpc, T, nchunk, C, dsum, dcnt);
    CKR(cudaGetLastError());
    CKR(cudaMemcpyAsync(sums, dsum, (size_t)T * C * 8, cudaMemcpyDeviceToHost, st));
    CKR(cudaMemcpyAsync(counts, dcnt, (size_t)T * C * 8, cudaMemcpyDeviceToHost, st));
    CKR(cudaStreamSynchronize(st));
    return WC_OK;
}

// TrainingSet::normalize + SetFisherScores over training rows sharded across
// processes: the statistics of this process's rows, in three stages that an
// exchange (min / max, then sums) separates.  stage 0: out = [mins (F), maxs (F)]
// of the finite values (FLT_MAX / -FLT_MAX where none), counts = rows per label
// (slot 0: every labelled row, slot c: class c); stage 1 (the global mins /
// maxs): out = per-label sums of the normalised values ((C+1) x F); stage 2
// (the global class means, (C+1) x F): out = per-label sums of squared
// deviations from them.
extern "C" int wc_wnd_fit_stats(wc_engine *E, int stage, const double *train, int N, int F, const int *labels, int C,
                                const double *mins, const double *maxs, const double *means, double *out,
                                long long *counts) {
    if (!E || !train || !labels || !out || N < 1 || F < 1 || C < 1 || C > 16 || stage < 0 || stage > 2 ||
        (stage == 0 && !counts) || (stage >= 1 && (!mins || !maxs)) || (stage == 2 && !means))
        return set_err(WC_ERR_ARG, "wc_wnd_fit_stats: bad arguments");
    cudaStream_t st;
    long long *launches;
    int rc = engine_device(E, &st, &launches);
    if (rc) return rc;
    const int fb = (F + 31) / 32;
    const int R = std::max(1, std::min((N + 255) / 256, (8 * engine_sms(E) + fb - 1) / fb));
    const int rows_per = (N + R - 1) / R;
    WBufs B;
    double *dX, *dmin, *dmax, *dmean, *dpa, *dpb, *dout;
    int *dy;
    long long *dcnt;
    if ((rc = B.get(&dX, (size_t)N * F * 8)) || (rc = B.get(&dy, (size_t)N * 4)) || (rc = B.get(&dmin, F * 8)) ||
        (rc = B.get(&dmax, F * 8)) || (rc = B.get(&dmean, (size_t)(C + 1) * F * 8)) ||
        (rc = B.get(&dpa, (size_t)R * (C + 1) * F * 8)) || (rc = B.get(&dpb, (size_t)R * F * 8)) ||
        (rc = B.get(&dout, (size_t)(C + 1) * F * 8)) || (rc = B.get(&dcnt, 17 * 8)))
        return rc;
    CKR(cudaMemcpyAsync(dX, train, (size_t)N * F * 8, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(dy, labels, (size_t)N * 4, cudaMemcpyHostToDevice, st));
    if (stage == 0) {
        CKR(cudaMemsetAsync(dcnt, 0, 17 * 8, st));
        *launches += 3;
        k_wnd_fit_minmax<<<dim3(fb, R), 256, 0, st>>>(dX, N, F, rows_per, dpa, dpb);
        k_wnd_fit_minmax_final<<<(F + 255) / 256, 256, 0, st>>>(dpa, dpb, R, F, dout, dout + F);
        k_wnd_fit_count<<<std::min(1024, (N + 255) / 256), 256, 0, st>>>(dy, N, C, dcnt);
        CKR(cudaGetLastError());
        CKR(cudaMemcpyAsync(out, dout, (size_t)2 * F * 8, cudaMemcpyDeviceToHost, st));
        CKR(cudaMemcpyAsync(counts, dcnt, (size_t)(C + 1) * 8, cudaMemcpyDeviceToHost, st));
    } else {
        CKR(cudaMemcpyAsync(dmin, mins, F * 8, cudaMemcpyHostToDevice, st));
        CKR(cudaMemcpyAsync(dmax, maxs, F * 8, cudaMemcpyHostToDevice, st));
        if (stage == 2) CKR(cudaMemcpyAsync(dmean, means, (size_t)(C + 1) * F * 8, cudaMemcpyHostToDevice, st));
        *launches += 2;
        k_wnd_fit_moments<<<dim3(fb, R), 256, 0, st>>>(dX, dy, N, F, C, rows_per, dmin, dmax,
                                                        stage == 2 ? dmean : nullptr, stage == 2, dpa);
        k_wnd_fit_rsum<<<(F + 255) / 256, 256, 0, st>>>(dpa, R, F, C, dout);
        CKR(cudaGetLastError());
        CKR(cudaMemcpyAsync(out, dout, (size_t)(C + 1) * F * 8, cudaMemcpyDeviceToHost, st));
    }
    CKR(cudaStreamSynchronize(st));
    return WC_OK;
}

// The Fisher weights from the exchanged statistics (wc_wnd_fit_stats summed
// over every process): class means, between-class over mean within-class
// variance as wc_wnd_fit computes them, and SetFisherScores' selection.
extern "C" int wc_wnd_fisher(wc_engine *E, int F, int C, double frac, const double *sums, const long long *counts,
                             const double *sq, double *weights) {
    if (!E || !sums || !counts || !sq || !weights || F < 1 || C < 1 || C > 16)
        return set_err(WC_ERR_ARG, "wc_wnd_fisher: bad arguments");
    cudaStream_t st;
    long long *launches;
    int rc = engine_device(E, &st, &launches);
    if (rc) return rc;
    WBufs B;
    double *dsum, *dsq, *dmean, *dw;
    long long *dcnt;
    if ((rc = B.get(&dsum, (size_t)(C + 1) * F * 8)) || (rc = B.get(&dsq, (size_t)(C + 1) * F * 8)) ||
        (rc = B.get(&dmean, (size_t)(C + 1) * F * 8)) || (rc = B.get(&dw, F * 8)) || (rc = B.get(&dcnt, 17 * 8)))
        return rc;
    CKR(cudaMemcpyAsync(dsum, sums, (size_t)(C + 1) * F * 8, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(dsq, sq, (size_t)(C + 1) * F * 8, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(dcnt, counts, (size_t)(C + 1) * 8, cudaMemcpyHostToDevice, st));
    *launches += 2;
    k_wnd_fit_combine<<<(F + 255) / 256, 256, 0, st>>>(dsum, 1, F, C, dcnt, 0, dmean, nullptr);
    k_wnd_fit_combine<<<(F + 255) / 256, 256, 0, st>>>(dsq, 1, F, C, dcnt, 1, dmean, dw);
    CKR(cudaGetLastError());
    CKR(cudaMemcpyAsync(weights, dw, F * 8, cudaMemcpyDeviceToHost, st));
    CKR(cudaStreamSynchronize(st));
    fisher_threshold(weights, F, frac);
    return WC_OK;
}

// signatures::normalize of n rows (host buffers)
extern "C" int wc_wnd_normalize(wc_engine *E, const double *rows, int n, int F, const double *mins,
                                const double *maxs, double *out) {
    if (!E || !rows || !mins || !maxs || !out || n < 1 || F < 1)
        return set_err(WC_ERR_ARG, "wc_wnd_normalize: bad arguments");
    cudaStream_t st;
    long long *launches;
    int rc = engine_device(E, &st, &launches);
    if (rc) return rc;
    WBufs B;
    double *dX, *dmin, *dmax, *dout;
    double2 *drec;
    const size_t nb = (size_t)n * F * 8;
    if ((rc = B.get(&dX, nb)) || (rc = B.get(&dout, nb)) || (rc = B.get(&dmin, F * 8)) || (rc = B.get(&dmax, F * 8)) ||
        (rc = B.get(&drec, (size_t)F * 16)))
        return rc;
    CKR(cudaMemcpyAsync(dX, rows, nb, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(dmin, mins, F * 8, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(dmax, maxs, F * 8, cudaMemcpyHostToDevice, st));
    *launches += 2;
    k_wnd_recip<<<(F + 255) / 256, 256, 0, st>>>(dmin, dmax, F, drec);
    const long long tot = (long long)n * F;
    k_wnd_normalize<<<(int)std::min<long long>((tot + 255) / 256, 8 * 1024), 256, 0, st>>>(dX, n, F, dmin, dmax, drec,
                                                                                           dout);
    CKR(cudaGetLastError());
    CKR(cudaMemcpyAsync(out, dout, nb, cudaMemcpyDeviceToHost, st));
    CKR(cudaStreamSynchronize(st));
    return WC_OK;
}

extern "C" int wc_wnd_classify_images(wc_engine *E, const double *train, int N, int F, const int *labels, int C,
                                      const double *weights, const double *mins, const double *maxs, const double *test,
                                      int n_images, int tiles, int max_tile, double *probs, int *pred,
                                      double *norm_factors) {
    if (!E || !train || !labels || !weights || !mins || !maxs || !test || !probs || !pred || N < 1 || F < 1 ||
        n_images < 1 || tiles < 1 || (long long)n_images * tiles > (1LL << 30) || C < 1 || C > 16)
        return set_err(WC_ERR_ARG, "wc_wnd_classify_images: bad arguments (C must be 1..16, tiles >= 1)");
    return wnd_classify(E, train, N, F, labels, C, weights, mins, maxs, test, n_images * tiles, nullptr, nullptr, tiles,
                        max_tile ? 1 : 0, probs, pred, norm_factors);
}

extern "C" int wc_wnd_classify_device(wc_engine *E, const double *train, int N, int F, const int *labels, int C,
                                      const double *weights, const double *mins, const double *maxs,
                                      const double *test, int T, double *probs, int *pred) {
    if (!E || !train || !labels || !weights || !mins || !maxs || !test || !probs || !pred || N < 1 || F < 1 || T < 1 ||
        C < 1 || C > 16)
        return set_err(WC_ERR_ARG, "wc_wnd_classify_device: bad arguments (C must be 1..16)");
    cudaStream_t st;
    long long *launches;
    int rc = engine_device(E, &st, &launches);
    if (rc) return rc;
    // the labels and weights drive host-side choices (class order, kept features)
    std::vector<int> y(N);
    std::vector<double> w(F);
    CKR(cudaMemcpyAsync(y.data(), labels, N * sizeof(int), cudaMemcpyDeviceToHost, st));
    CKR(cudaMemcpyAsync(w.data(), weights, F * sizeof(double), cudaMemcpyDeviceToHost, st));
    CKR(cudaStreamSynchronize(st));
    WBufs B;
    double *dnorm;
    if ((rc = B.get(&dnorm, (size_t)T * 8))) return rc;
    return wnd_classify_dev(E, train, N, F, y.data(), C, w.data(), mins, maxs, test, T, probs, pred, dnorm);
}

extern "C" int wc_wnd_last_stats(long long *stats) {
    if (!stats) return set_err(WC_ERR_ARG, "wc_wnd_last_stats: null stats");
    for (int i = 0; i < 6; i++) stats[i] = g_last_stats[i];
    return WC_OK;
}
