// Preprocessing and sampling of opened images (the steps between reading an
// image file and computing its features): crop to a bounding rectangle,
// area downsampling, normalisation, right-angle rotation and tiles.
//
// ImageMatrix::OpenImage (src/cmatrix.cpp:252-294) with submatrix (:414-470),
// Downsample (:579-720) and normalize (:836-888); ImageMatrix::Rotate
// (:727-769) and the tile submatrix of TrainingSet::AddImageFile
// (src/wndchrm_src/TrainingSet.cpp:1455-1481).  FP64 throughout; this file is
// built without multiply-add contraction so each rounded step is the
// reference's.
#include <algorithm>
#include <cfloat>
#include <cmath>

#include "kcommon.cuh"
#include "kernels.h"

namespace wc {

// ---------------------------------------------------------------- crop + convert
// pre[a_off + y*cw + x] = src[(cy + y) * sw + cx + x]
__global__ void k_pre_crop(const PreJob *__restrict__ jobs, double *__restrict__ pre) {
    const PreJob &J = jobs[blockIdx.z];
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= J.cw || y >= J.ch) return;
    const long long si = (long long)(J.cy + y) * J.sw + J.cx + x;
    double v;
    switch (J.dtype) {
        case 0: v = (double)((const unsigned char *)J.src)[si]; break;
        case 1: v = (double)((const unsigned short *)J.src)[si]; break;
        case 2: v = (double)((const float *)J.src)[si]; break;
        default: v = ((const double *)J.src)[si]; break;
    }
    pre[J.a_off + (long long)y * J.cw + x] = v;
}

// ---------------------------------------------------------------- Downsample
// One output of either pass (src/cmatrix.cpp:608-650 along x, :669-712 along
// y): the source line averaged over [x, x + d), d = 1 / ratio, the partial
// pixels at both ends weighted by their covered fraction.  x is the
// reference's accumulated position (x += d from 0), computed on the host.
__device__ __forceinline__ double pre_interval(const double *__restrict__ src, long long stride, int old, double x,
                                               double d) {
    double s = 0, frac;
    unsigned a = (unsigned)floor(x);
    frac = ceil(x) - x;
    if (frac > 0 && a < (unsigned)old) s += src[(long long)a * stride] * frac;
    for (a = (unsigned)ceil(x); a < floor(x + d); a++)
        if (a < (unsigned)old) s += src[(long long)a * stride];
    frac = x + d - floor(x + d);
    if (frac > 0 && a < (unsigned)old) s += src[(long long)a * stride] * frac;
    return s / d;
}

// x pass: t[y*nw + k] for the crop's ch rows and the first nw positions (the
// y pass reads no further)
__global__ void k_pre_down_x(const PreJob *__restrict__ jobs, const double *__restrict__ tab, double *__restrict__ pre) {
    const PreJob &J = jobs[blockIdx.z];
    if (!J.down) return;
    const int k = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (k >= J.nw || y >= J.ch) return;
    pre[J.t_off + (long long)y * J.nw + k] = pre_interval(pre + J.a_off + (long long)y * J.cw, 1, J.cw, tab[J.xs_tab + k], J.dx);
}

// y pass: o[k*nw + x] over the x pass's columns
__global__ void k_pre_down_y(const PreJob *__restrict__ jobs, const double *__restrict__ tab, double *__restrict__ pre) {
    const PreJob &J = jobs[blockIdx.z];
    if (!J.down) return;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= J.nw || k >= J.nh) return;
    pre[J.o_off + (long long)k * J.nw + x] = pre_interval(pre + J.t_off + x, J.nw, J.ch, tab[J.ys_tab + k], J.dy);
}

// ---------------------------------------------------------------- normalize
// Range branch (src/cmatrix.cpp:852-864), elementwise: below n_min -> 0, above
// n_max -> n_range, else (v - n_min) * (n_range / (n_max - n_min)).
__global__ void k_pre_norm_range(const PreJob *__restrict__ jobs, double *__restrict__ pre) {
    const PreJob &J = jobs[blockIdx.y];
    if (!J.mm) return;
    double *p = pre + J.o_off;
    const long long n = (long long)J.ow * J.oh;
    const double nf = J.n_range / (J.n_max - J.n_min);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double v = p[i];
        if (v < J.n_min) v = 0;
        else if (v > J.n_max) v = J.n_range;
        else v = nf * (v - J.n_min);
        p[i] = v;
    }
}

// Mean branch, first half: mean() and std() of the plane as the reference
// computes them, bit for bit: Moments2::add over the pixels in raster order
// (src/statistics/Moments.h:69-85; ImageMatrix::UpdateStats, src/cmatrix.cpp:803-811;
// NaN and |v| > FLT_MAX skipped), a sequential chain run by one thread per
// image.  delta / n is correctly rounded by Markstein's method (P. Markstein,
// IBM J. Res. Develop. 34(1), 1990): with yh = RN(1/n) and yl = RN(1/n - yh),
// q0 = RN(delta*yh + RN(delta*yl)) is within one ulp of delta/n, the residual
// r = delta - n*q0 is exact, and RN(q0 + r*yh) = RN(delta/n); it takes four
// FP64 operations where a division takes more.  Writes d_mean = mean - n_mean
// and std_fact = max(n_std, 0) / std (src/cmatrix.cpp:867).
struct WfState {
    double mean, M2, nprev;
    long long cnt;
};
__device__ __forceinline__ bool wf_skip(double v) { return isnan(v) || v > FLT_MAX || v < -FLT_MAX; }
__device__ __forceinline__ void wf_add(WfState &s, double v, double h, double l) {
    const double nn = s.nprev + 1.0;  // the count after this value, exact
    const double delta = v - s.mean;
    const double q0 = fma(delta, h, delta * l);
    const double r = fma(-q0, nn, delta);
    const double dn = fma(r, h, q0);  // RN(delta / nn)
    const double term1 = delta * dn * s.nprev;
    s.mean = s.mean + dn;
    s.M2 += term1;
    s.nprev = nn;
    s.cnt++;
}

// Values are taken WF_CHUNK at a time, the next chunk loaded ahead; a chunk
// without skipped values reads its reciprocals together.
#define WF_CHUNK 4
__global__ void k_pre_welford(const PreJob *__restrict__ jobs, const double *__restrict__ pre,
                              const double *__restrict__ yh, const double *__restrict__ yl, double *__restrict__ fact) {
    const PreJob &J = jobs[blockIdx.x];
    if (!J.ms || threadIdx.x) return;
    const double *p = pre + J.o_off;
    const long long n = (long long)J.ow * J.oh;
    WfState s{0, 0, 0, 0};
    double cur[WF_CHUNK], nxt[WF_CHUNK];
    long long i = 0;
    if (n >= WF_CHUNK)
        for (int j = 0; j < WF_CHUNK; j++) cur[j] = p[j];
    for (; i + WF_CHUNK <= n; i += WF_CHUNK) {
        const bool more = i + 2 * WF_CHUNK <= n;
        if (more)
            for (int j = 0; j < WF_CHUNK; j++) nxt[j] = p[i + WF_CHUNK + j];
        bool good = true;
        for (int j = 0; j < WF_CHUNK; j++) good &= !wf_skip(cur[j]);
        if (good) {
            double h[WF_CHUNK], l[WF_CHUNK];
            for (int j = 0; j < WF_CHUNK; j++) {
                h[j] = yh[s.cnt + j];
                l[j] = yl[s.cnt + j];
            }
            for (int j = 0; j < WF_CHUNK; j++) wf_add(s, cur[j], h[j], l[j]);
        } else {
            for (int j = 0; j < WF_CHUNK; j++)
                if (!wf_skip(cur[j])) wf_add(s, cur[j], yh[s.cnt], yl[s.cnt]);
        }
        if (more)
            for (int j = 0; j < WF_CHUNK; j++) cur[j] = nxt[j];
    }
    for (; i < n; i++)
        if (!wf_skip(p[i])) wf_add(s, p[i], yh[s.cnt], yl[s.cnt]);
    const double sd = s.cnt > 2 ? sqrt(s.M2 / (double)(s.cnt - 1)) : 0.0;
    fact[2 * blockIdx.x] = s.mean - J.n_mean;
    fact[2 * blockIdx.x + 1] = (J.n_std > 0 ? J.n_std : 0) / sd;
}

// Mean branch, second half (src/cmatrix.cpp:868-878), elementwise:
// v - d_mean, then n_mean + (v - n_mean) * std_fact when n_std > 0, clamped to
// [0, 2^bits - 1].
__global__ void k_pre_norm_mean(const PreJob *__restrict__ jobs, const double *__restrict__ fact,
                                double *__restrict__ pre) {
    const PreJob &J = jobs[blockIdx.y];
    if (!J.ms) return;
    double *p = pre + J.o_off;
    const long long n = (long long)J.ow * J.oh;
    const double d_mean = fact[2 * blockIdx.y], std_fact = fact[2 * blockIdx.y + 1];
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double v = p[i] - d_mean;
        if (J.n_std > 0) v = J.n_mean + (v - J.n_mean) * std_fact;
        if (v < 0) v = 0;
        else if (v > J.max_range) v = J.max_range;
        p[i] = v;
    }
}

// ---------------------------------------------------------------- rotation + tile
// Sample pixel (y, x) is pixel (y1 + y, x1 + x) of the opened plane rotated by
// Rotate's rule: 90 = transpose then reverse each row, 180 = reverse both axes,
// 270 = transpose.
__global__ void k_pre_sample(const PreJob *__restrict__ jobs, const SampleJob *__restrict__ sj, double *__restrict__ pre) {
    const SampleJob &S = sj[blockIdx.z];
    const PreJob &J = jobs[S.img];
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= S.tw || y >= S.th) return;
    const int ri = S.y1 + y, rj = S.x1 + x, W = J.ow, H = J.oh;
    int sy, sx;
    switch (S.rot) {
        case 1: sy = H - 1 - rj; sx = ri; break;
        case 2: sy = H - 1 - ri; sx = W - 1 - rj; break;
        case 3: sy = rj; sx = ri; break;
        default: sy = ri; sx = rj; break;
    }
    pre[S.off + (long long)y * S.tw + x] = pre[J.o_off + (long long)sy * W + sx];
}

void launch_preprocess(Ctx &c, const PreJob *jobs, int n, const PreGeomMax &g, const double *tab, const double *yh,
                       const double *yl, double *fact, double *pre, const SampleJob *sj, int ns) {
    const dim3 b(32, 8);
    WC_LAUNCH(c);
    k_pre_crop<<<dim3((g.cw + 31) / 32, (g.ch + 7) / 8, n), b, 0, c.st>>>(jobs, pre);
    if (g.down) {
        WC_LAUNCH(c);
        k_pre_down_x<<<dim3((g.nw + 31) / 32, (g.ch + 7) / 8, n), b, 0, c.st>>>(jobs, tab, pre);
        WC_LAUNCH(c);
        k_pre_down_y<<<dim3((g.nw + 31) / 32, (g.nh + 7) / 8, n), b, 0, c.st>>>(jobs, tab, pre);
    }
    const long long opx = (long long)std::max(g.ow, 1) * std::max(g.oh, 1);
    const int gx = (int)std::min<long long>((opx + 255) / 256, 64);
    if (g.norm_range) {
        WC_LAUNCH(c);
        k_pre_norm_range<<<dim3(gx, n), 256, 0, c.st>>>(jobs, pre);
    }
    if (g.norm_mean) {
        WC_LAUNCH(c);
        k_pre_welford<<<n, 32, 0, c.st>>>(jobs, pre, yh, yl, fact);
        WC_LAUNCH(c);
        k_pre_norm_mean<<<dim3(gx, n), 256, 0, c.st>>>(jobs, fact, pre);
    }
    WC_LAUNCH(c);
    k_pre_sample<<<dim3((g.tw + 31) / 32, (g.th + 7) / 8, ns), b, 0, c.st>>>(jobs, sj, pre);
}

}  // namespace wc
