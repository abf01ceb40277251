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
}

namespace wc {

// per feature: min/max over the rows (skipping NaN and |v| > FLT_MAX), then the
// normalised column; X is N x F row-major, Xn written in the same layout.
__global__ void k_wnd_minmax(const double *__restrict__ X, int N, int F, double *__restrict__ mins,
                             double *__restrict__ maxs, double *__restrict__ Xn) {
    __shared__ double sh[32];
    const int f = blockIdx.x;
    double mn = FLT_MAX, mx = -FLT_MAX;
    for (int s = threadIdx.x; s < N; s += blockDim.x) {
        double v = X[(long long)s * F + f];
        if (isnan(v) || v > FLT_MAX || v < -FLT_MAX) continue;
        mn = fmin(mn, v);
        mx = fmax(mx, v);
    }
    mn = block_min(mn, sh);
    mx = block_max(mx, sh);
    if (threadIdx.x == 0) {
        mins[f] = mn;
        maxs[f] = mx;
    }
    for (int s = threadIdx.x; s < N; s += blockDim.x) {
        double v = X[(long long)s * F + f];
        if (isnan(v) || v < mn || (mx - mn) < DBL_EPSILON) v = 0;
        else if (v > mx) v = 100;
        else v = 100 * ((v - mn) / (mx - mn));
        Xn[(long long)s * F + f] = v;
    }
}

// Fisher score per feature: between-class variance of class means over the
// mean within-class variance (Moments2 var, 0 for n <= 2), floor 1e-6.
__global__ void k_wnd_fisher(const double *__restrict__ Xn, const int *__restrict__ y, int N, int F, int C,
                             double *__restrict__ w) {
    __shared__ double sh[32];
    __shared__ long long shl[32];
    const int f = blockIdx.x;
    double s_all = 0;
    long long n_all = 0;
    for (int s = threadIdx.x; s < N; s += blockDim.x)
        if (y[s]) { s_all += Xn[(long long)s * F + f]; n_all++; }
    s_all = block_sum(s_all, sh);
    n_all = block_sum_ll(n_all, shl);
    const double mean_all = n_all ? s_all / n_all : 0.0;
    double dev = 0, var = 0;
    for (int c = 1; c <= C; c++) {
        double sc = 0;
        long long nc = 0;
        for (int s = threadIdx.x; s < N; s += blockDim.x)
            if (y[s] == c) { sc += Xn[(long long)s * F + f]; nc++; }
        sc = block_sum(sc, sh);
        nc = block_sum_ll(nc, shl);
        const double mc = nc ? sc / nc : 0.0;
        double m2 = 0;
        for (int s = threadIdx.x; s < N; s += blockDim.x)
            if (y[s] == c) { double d = Xn[(long long)s * F + f] - mc; m2 += d * d; }
        m2 = block_sum(m2, sh);
        dev += pow(mc - mean_all, 2);
        var += nc > 2 ? m2 / (nc - 1) : 0.0;
    }
    if (threadIdx.x == 0) {
        if (C > 1) {
            dev /= (C - 1);
            var /= C;
        } else {
            dev = 0;
        }
        if (var < 0.000001) var = 0.000001;
        w[f] = dev / var;
    }
}

// gather the kept features, normalised: Xc is K x rows (column-major per row
// set) so lanes reading consecutive rows coalesce.
__global__ void k_wnd_gather(const double *__restrict__ X, int rows, int F, const int *__restrict__ keep, int K,
                             const double *__restrict__ mins, const double *__restrict__ maxs, double *__restrict__ Xc) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= (long long)rows * K) return;
    const int k = (int)(q / rows), s = (int)(q - (long long)k * rows);
    const int f = keep[k];
    const double mn = mins[f], mx = maxs[f];
    double v = X[(long long)s * F + f];
    if (isnan(v) || v < mn || (mx - mn) < DBL_EPSILON) v = 0;
    else if (v > mx) v = 100;
    else v = 100 * ((v - mn) / (mx - mn));
    Xc[(long long)k * rows + s] = v;
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

extern "C" int wc_wnd_fit(wc_engine *E, const double *train, int N, int F, const int *labels, int C, double frac,
                          double *weights, double *mins, double *maxs) {
    if (!E || !train || !labels || !weights || !mins || !maxs || N < 1 || F < 1 || C < 1 || C > 16)
        return set_err(WC_ERR_ARG, "wc_wnd_fit: bad arguments (C must be 1..16)");
    cudaStream_t st;
    long long *launches;
    int rc = engine_device(E, &st, &launches);
    if (rc) return rc;
    double *dX = nullptr, *dXn = nullptr, *dmin = nullptr, *dmax = nullptr, *dw = nullptr;
    int *dy = nullptr;
    const size_t xb = (size_t)N * F * sizeof(double);
    CKW(cudaMalloc(&dX, xb));
    CKW(cudaMalloc(&dXn, xb));
    CKW(cudaMalloc(&dmin, F * sizeof(double)));
    CKW(cudaMalloc(&dmax, F * sizeof(double)));
    CKW(cudaMalloc(&dw, F * sizeof(double)));
    CKW(cudaMalloc(&dy, N * sizeof(int)));
    CKW(cudaMemcpyAsync(dX, train, xb, cudaMemcpyHostToDevice, st));
    CKW(cudaMemcpyAsync(dy, labels, N * sizeof(int), cudaMemcpyHostToDevice, st));
    ++*launches;
    k_wnd_minmax<<<F, 256, 0, st>>>(dX, N, F, dmin, dmax, dXn);
    ++*launches;
    k_wnd_fisher<<<F, 256, 0, st>>>(dXn, dy, N, F, C, dw);
    CKW(cudaGetLastError());
    CKW(cudaMemcpyAsync(weights, dw, F * sizeof(double), cudaMemcpyDeviceToHost, st));
    CKW(cudaMemcpyAsync(mins, dmin, F * sizeof(double), cudaMemcpyDeviceToHost, st));
    CKW(cudaMemcpyAsync(maxs, dmax, F * sizeof(double), cudaMemcpyDeviceToHost, st));
    CKW(cudaStreamSynchronize(st));
    {
        // threshold at the weight of sorted (descending) rank floor(frac*F + 0.5)
        int last = (int)std::floor((frac * (double)F) + 0.5);
        if (last < F) {
            std::vector<double> sw(weights, weights + F);
            std::nth_element(sw.begin(), sw.begin() + last, sw.end(), std::greater<double>());
            const double thr = sw[last];
            for (int f = 0; f < F; f++)
                if (weights[f] < thr) weights[f] = 0.0;
        }
    }
done:
    cudaFree(dX);
    cudaFree(dXn);
    cudaFree(dmin);
    cudaFree(dmax);
    cudaFree(dw);
    cudaFree(dy);
    return rc;
}

// classify2 for T test rows; with tiles > 0 the rows are n = T / tiles images'
// tiles and ClassifyImage's per-image results are returned instead of the rows'.
static int wnd_classify(wc_engine *E, const double *train, int N, int F, const int *labels, int C,
                        const double *weights, const double *mins, const double *maxs, const double *test, int T,
                        double *probs, int *pred, int tiles, int max_tile, double *iprobs, int *ipred, double *inorm) {
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
    const int n_img = tiles > 0 ? T / tiles : 0;
    double *dX = nullptr, *dT = nullptr, *dXc = nullptr, *dTc = nullptr, *dmin = nullptr, *dmax = nullptr, *dw2 = nullptr,
           *dps = nullptr, *dprob = nullptr, *dnorm = nullptr, *diprob = nullptr, *dinorm = nullptr;
    int *dipred = nullptr;
    long long *dpc = nullptr;
    int *dkeep = nullptr, *dy = nullptr, *dpred = nullptr;
    CKW(cudaMalloc(&dX, (size_t)N * F * 8));
    CKW(cudaMalloc(&dT, (size_t)T * F * 8));
    CKW(cudaMalloc(&dXc, (size_t)N * std::max(K, 1) * 8));
    CKW(cudaMalloc(&dTc, (size_t)T * std::max(K, 1) * 8));
    CKW(cudaMalloc(&dmin, F * 8));
    CKW(cudaMalloc(&dmax, F * 8));
    CKW(cudaMalloc(&dw2, std::max(K, 1) * 8));
    CKW(cudaMalloc(&dkeep, std::max(K, 1) * 4));
    CKW(cudaMalloc(&dy, N * 4));
    CKW(cudaMalloc(&dps, (size_t)T * nchunk * C * 8));
    CKW(cudaMalloc(&dpc, (size_t)T * nchunk * C * 8));
    CKW(cudaMalloc(&dprob, (size_t)T * C * 8));
    CKW(cudaMalloc(&dpred, (size_t)T * 4));
    CKW(cudaMalloc(&dnorm, (size_t)T * 8));
    if (n_img) {
        CKW(cudaMalloc(&diprob, (size_t)n_img * C * 8));
        CKW(cudaMalloc(&dipred, (size_t)n_img * 4));
        CKW(cudaMalloc(&dinorm, (size_t)n_img * 8));
    }
    CKW(cudaMemcpyAsync(dX, train, (size_t)N * F * 8, cudaMemcpyHostToDevice, st));
    CKW(cudaMemcpyAsync(dT, test, (size_t)T * F * 8, cudaMemcpyHostToDevice, st));
    CKW(cudaMemcpyAsync(dmin, mins, F * 8, cudaMemcpyHostToDevice, st));
    CKW(cudaMemcpyAsync(dmax, maxs, F * 8, cudaMemcpyHostToDevice, st));
    CKW(cudaMemcpyAsync(dy, labels, N * 4, cudaMemcpyHostToDevice, st));
    if (K) {
        CKW(cudaMemcpyAsync(dw2, w2.data(), K * 8, cudaMemcpyHostToDevice, st));
        CKW(cudaMemcpyAsync(dkeep, keep.data(), K * 4, cudaMemcpyHostToDevice, st));
        ++*launches;
        k_wnd_gather<<<(int)(((long long)N * K + 255) / 256), 256, 0, st>>>(dX, N, F, dkeep, K, dmin, dmax, dXc);
        ++*launches;
        k_wnd_gather<<<(int)(((long long)T * K + 255) / 256), 256, 0, st>>>(dT, T, F, dkeep, K, dmin, dmax, dTc);
    }
    if (engine_precision(E) == WC_PREC_MIXED && K) {
        float2 *fX = nullptr, *fT = nullptr, *fw = nullptr;
        CKW(cudaMalloc(&fX, (size_t)N * K * 8));
        CKW(cudaMalloc(&fT, (size_t)T * K * 8));
        CKW(cudaMalloc(&fw, (size_t)K * 8));
        *launches += 4;
        k_wnd_split<<<1024, 256, 0, st>>>(dXc, (long long)N * K, fX);
        k_wnd_split<<<1024, 256, 0, st>>>(dTc, (long long)T * K, fT);
        k_wnd_split<<<1, 256, 0, st>>>(dw2, K, fw);
        k_wnd_dist_df<<<dim3((T + WT - 1) / WT, nchunk), 256, 0, st>>>(fT, T, fX, N, dy, fw, K, C, per, dps, dpc);
        const cudaError_t le = cudaGetLastError();
        cudaStreamSynchronize(st);
        cudaFree(fX);
        cudaFree(fT);
        cudaFree(fw);
        CKW(le);
    } else {
        ++*launches;
        k_wnd_dist<<<dim3((T + WT - 1) / WT, nchunk), 256, 0, st>>>(dTc, T, dXc, N, dy, dw2, K, C, per, dps, dpc);
    }
    ++*launches;
    k_wnd_finish<<<(T + 127) / 128, 128, 0, st>>>(dps, dpc, T, nchunk, C, dprob, dpred, dnorm);
    CKW(cudaGetLastError());
    if (n_img) {
        ++*launches;
        k_wnd_tiles<<<(n_img + 127) / 128, 128, 0, st>>>(dprob, dpred, dnorm, n_img, tiles, C, max_tile, diprob, dipred,
                                                         dinorm);
        CKW(cudaGetLastError());
        CKW(cudaMemcpyAsync(iprobs, diprob, (size_t)n_img * C * 8, cudaMemcpyDeviceToHost, st));
        CKW(cudaMemcpyAsync(ipred, dipred, (size_t)n_img * 4, cudaMemcpyDeviceToHost, st));
        if (inorm) CKW(cudaMemcpyAsync(inorm, dinorm, (size_t)n_img * 8, cudaMemcpyDeviceToHost, st));
    } else {
        CKW(cudaMemcpyAsync(probs, dprob, (size_t)T * C * 8, cudaMemcpyDeviceToHost, st));
        CKW(cudaMemcpyAsync(pred, dpred, (size_t)T * 4, cudaMemcpyDeviceToHost, st));
    }
    CKW(cudaStreamSynchronize(st));
done:
    cudaFree(dX);
    cudaFree(dT);
    cudaFree(dXc);
    cudaFree(dTc);
    cudaFree(dmin);
    cudaFree(dmax);
    cudaFree(dw2);
    cudaFree(dkeep);
    cudaFree(dy);
    cudaFree(dps);
    cudaFree(dpc);
    cudaFree(dprob);
    cudaFree(dpred);
    cudaFree(dnorm);
    cudaFree(diprob);
    cudaFree(dipred);
    cudaFree(dinorm);
    return rc;
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
