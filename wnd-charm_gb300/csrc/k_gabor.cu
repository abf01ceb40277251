// Gabor textures (FP64 form): GaborTextureFilters2D + GaborEnergy + Gabor,
// src/textures/gabor.cpp:103-231.  For f0 = 0.1 (low-pass) and 1..7, the energy
// e = |conv2(I, G_f0)| (full complex convolution with the 38 x 38 normalised
// kernel, cropped at ceil(38/2) = 19); baseline = #(e_lp > 0.4 max e_lp); for
// each high-pass filter, e/max(e) is thresholded at its Otsu level and
// ratio = #(above) / baseline.
//
// The convolutions run as FP64 FFTs: image and kernels zero-padded to a
// 7-smooth size >= (H+37) x (W+37), so the circular product is the linear
// convolution; inverse through the conjugate, |.| / N.
#include <cfloat>
#include <cmath>

#include "kcommon.cuh"
#include "kernels.h"
#include "kfft.cuh"

namespace wc {

// batched 1-D complex DFTs: arrays blockIdx.y, line groups blockIdx.x; element
// k of line l at data + arr*js + l*ls + k*es.  conj_in/conj_out conjugate on
// load/store; scale multiplies on store.
__global__ void k_cfft_lines(double *__restrict__ data, long long js, int nl, int n, long long ls, long long es,
                             const FFTPlan *__restrict__ plan, const double *__restrict__ twd, int lpc) {
    extern __shared__ double smem[];
    const FFTPlan P = *plan;
    const int l0 = blockIdx.x * lpc;
    if (l0 >= nl) return;
    const int lines = min(lpc, nl - l0);
    cplx *base = (cplx *)data + (long long)blockIdx.y * js;
    cplx *b0 = (cplx *)smem, *b1 = b0 + (long long)lpc * n;
    const cplx *tw = (const cplx *)(twd + P.tw_off);
    if (es == 1) {
        for (int i = threadIdx.x; i < lines * n; i += blockDim.x) {
            const int l = i / n, k = i - l * n;
            b0[i] = base[(long long)(l0 + l) * ls + k];
        }
    } else {
        for (int i = threadIdx.x; i < lines * n; i += blockDim.x) {
            const int k = i / lines, l = i - k * lines;
            b0[(long long)l * n + k] = base[(long long)(l0 + l) * ls + (long long)k * es];
        }
    }
    __syncthreads();
    const cplx *r = stockham(b0, b1, lines, P, tw) ? b1 : b0;
    if (es == 1) {
        for (int i = threadIdx.x; i < lines * n; i += blockDim.x) {
            const int l = i / n, k = i - l * n;
            base[(long long)(l0 + l) * ls + k] = r[i];
        }
    } else {
        for (int i = threadIdx.x; i < lines * n; i += blockDim.x) {
            const int k = i / lines, l = i - k * lines;
            base[(long long)(l0 + l) * ls + (long long)k * es] = r[(long long)l * n + k];
        }
    }
}

// forward 2-D DFT of `na` arrays of fh x fw complex values (row-major), in place
void cfft2(Ctx &c, double *data, int na, int fh, int fw, const FFTPlan *plan_w, const FFTPlan *plan_h, const double *tw) {
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_cfft_lines, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr = true;
    }
    const long long js = (long long)fh * fw;
    int lpc = 96 * 1024 / (32 * fw);
    lpc = lpc < 1 ? 1 : (lpc > 8 ? 8 : lpc);
    WC_LAUNCH(c);
    k_cfft_lines<<<dim3((fh + lpc - 1) / lpc, na), 256, (size_t)lpc * fw * 32, c.st>>>(data, js, fh, fw, fw, 1, plan_w, tw, lpc);
    int lpc2 = 96 * 1024 / (32 * fh);
    lpc2 = lpc2 < 1 ? 1 : (lpc2 > 8 ? 8 : lpc2);
    WC_LAUNCH(c);
    k_cfft_lines<<<dim3((fw + lpc2 - 1) / lpc2, na), 256, (size_t)lpc2 * fh * 32, c.st>>>(data, js, fw, fh, 1, fw, plan_h, tw,
                                                                                        lpc2);
}

// zero-padded image (job) into a fh x fw complex array
__global__ void k_gab_pad(const double *__restrict__ arena, const Plane *__restrict__ planes, const FJob *__restrict__ jobs,
                          const GabJob *__restrict__ gj, double *__restrict__ ws) {
    const FJob J = jobs[blockIdx.y];
    const GabJob G = gj[blockIdx.y];
    const Plane P = planes[J.plane];
    cplx *A = (cplx *)(ws + G.a_ws);
    const long long n = (long long)G.fh * G.fw;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int y = (int)(i / G.fw), x = (int)(i - (long long)y * G.fw);
        A[i] = {(y < P.h && x < P.w) ? arena[P.off + (long long)y * P.w + x] : 0.0, 0.0};
    }
}

// the 8 kernels (38 x 38 complex, host-made) zero-padded to fh x fw
__global__ void k_gab_padk(const double *__restrict__ kern, double *__restrict__ G, int fh, int fw) {
    const int f = blockIdx.y;
    cplx *g = (cplx *)G + (long long)f * fh * fw;
    const long long n = (long long)fh * fw;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int y = (int)(i / fw), x = (int)(i - (long long)y * fw);
        cplx v = {0.0, 0.0};
        if (y < 38 && x < 38) v = {kern[((long long)f * 38 * 38 + y * 38 + x) * 2], kern[((long long)f * 38 * 38 + y * 38 + x) * 2 + 1]};
        g[i] = v;
    }
}

// C = conj(A .* G_f)  (the inverse transform is conj(FFT(conj(X))) / N)
__global__ void k_gab_mul(const GabJob *__restrict__ gj, double *__restrict__ ws, int f) {
    const GabJob G = gj[blockIdx.y];
    const cplx *A = (const cplx *)(ws + G.a_ws);
    const cplx *K = (const cplx *)(ws + G.g_ws) + (long long)f * G.fh * G.fw;
    cplx *C = (cplx *)(ws + G.c_ws);
    const long long n = (long long)G.fh * G.fw;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const cplx a = A[i], k = K[i];
        C[i] = {a.x * k.x - a.y * k.y, -(a.x * k.y + a.y * k.x)};
    }
}

// energy map e_f(b, a) = |c(b + 19, a + 19)| / N
__global__ void k_gab_crop(const Plane *__restrict__ planes, const FJob *__restrict__ jobs, const GabJob *__restrict__ gj,
                           double *__restrict__ ws, int f) {
    const FJob J = jobs[blockIdx.y];
    const GabJob G = gj[blockIdx.y];
    const Plane P = planes[J.plane];
    const cplx *C = (const cplx *)(ws + G.c_ws);
    double *e = ws + G.e_ws + (long long)f * P.w * P.h;
    const double invN = 1.0 / ((double)G.fh * G.fw);
    const long long n = (long long)P.w * P.h;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int b = (int)(i / P.w), a = (int)(i - (long long)b * P.w);
        const cplx v = C[(long long)(b + 19) * G.fw + a + 19];
        const double re = v.x * invN, im = v.y * invN;
        e[i] = sqrt(__dadd_rn(__dmul_rn(re, re), __dmul_rn(im, im)));
    }
}

// per (job, filter): max, then the baseline count (f = 0) or the Otsu count
__global__ void __launch_bounds__(1024) k_gab_count(const Plane *__restrict__ planes, const FJob *__restrict__ jobs,
                                                    const GabJob *__restrict__ gj, const double *__restrict__ ws,
                                                    double *__restrict__ counts) {
    __shared__ double sh[32];
    __shared__ long long shl[32];
    __shared__ unsigned int hist[1024];
    const int f = blockIdx.y;
    const FJob J = jobs[blockIdx.x];
    const GabJob G = gj[blockIdx.x];
    const Plane P = planes[J.plane];
    const long long n = (long long)P.w * P.h;
    const double *e = ws + G.e_ws + (long long)f * n;
    double mx = -DBL_MAX, mn = DBL_MAX;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        mx = fmax(mx, e[i]);
        mn = fmin(mn, e[i]);
    }
    mx = block_max(mx, sh);
    mn = block_min(mn, sh);
    long long cnt = 0;
    if (f == 0) {
        const double t = mx * 0.4;
        for (long long i = threadIdx.x; i < n; i += blockDim.x) cnt += (e[i] > t);
    } else {
        // normalised energies e/max: min = min(e)/max, max = 1
        const double lo = mn / mx, hi = mx / mx;
        for (int i = threadIdx.x; i < 1024; i += blockDim.x) hist[i] = 0;
        __syncthreads();
        const double sc = hist_scale(lo, hi, 1024);
        for (long long i = threadIdx.x; i < n; i += blockDim.x) atomicAdd(&hist[hist_bin(e[i] / mx, lo, sc, 1024)], 1u);
        __syncthreads();
        __shared__ double s_thr;
        if (threadIdx.x == 0) {
            const double wh = (double)(unsigned)(P.w * P.h);
            double myL = 0.0;
            for (int i = 1; i < 1024; i++) myL = __dadd_rn(myL, __dmul_rn((double)i, hist[i] / wh));
            double om = hist[0] / wh, my = 0.0, best = 0.0;
            int th = 0;
            for (int i = 0; i < 1023; i++) {
                if (i > 0) {
                    om = __dadd_rn(om, hist[i] / wh);
                    my = __dadd_rn(my, __dmul_rn((double)i, hist[i] / wh));
                }
                double s = 0.0;
                if (om != 0.0 && om != 1.0) {
                    const double d = __dsub_rn(__dmul_rn(myL, om), my);
                    s = __dmul_rn(d, d) / __dmul_rn(om, __dsub_rn(1.0, om));
                }
                if (s > best) { best = s; th = i; }
            }
            s_thr = __dadd_rn(__dmul_rn((double)th / (double)1023, __dsub_rn(hi, lo)), lo);
        }
        __syncthreads();
        const double t = s_thr;
        for (long long i = threadIdx.x; i < n; i += blockDim.x) cnt += (e[i] / mx > t);
    }
    cnt = block_sum_ll(cnt, shl);
    if (threadIdx.x == 0) counts[blockIdx.x * 8 + f] = (double)cnt;
}

__global__ void k_gab_final(const FJob *__restrict__ jobs, const double *__restrict__ counts, double *__restrict__ feat) {
    const FJob J = jobs[blockIdx.x];
    if (threadIdx.x < 7) feat[J.out + threadIdx.x] = counts[blockIdx.x * 8 + 1 + threadIdx.x] / counts[blockIdx.x * 8];
}

void launch_gabor(Ctx &c, const double *arena, const Plane *planes, const FJob *jobs, int njobs, const GabJob *gj_d,
                  const std::vector<GabJob> &gj, const std::vector<GabSize> &sizes, const FFTPlan *plans_d,
                  const double *tabs, long long kern_tab, double *ws, double *counts, double *feat) {
    if (njobs <= 0) return;
    // kernels' spectra, once per padded size
    for (const GabSize &S : sizes) {
        WC_LAUNCH(c);
        k_gab_padk<<<dim3(64, 8), 256, 0, c.st>>>(tabs + kern_tab, ws + S.g_ws, S.fh, S.fw);
        cfft2(c, ws + S.g_ws, 8, S.fh, S.fw, plans_d + S.plan_w, plans_d + S.plan_h, tabs);
    }
    WC_LAUNCH(c);
    k_gab_pad<<<dim3(128, njobs), 256, 0, c.st>>>(arena, planes, jobs, gj_d, ws);
    // the images' spectra (sizes may differ between jobs: one call per job)
    for (int j = 0; j < njobs; j++)
        cfft2(c, ws + gj[j].a_ws, 1, gj[j].fh, gj[j].fw, plans_d + gj[j].plan_w, plans_d + gj[j].plan_h, tabs);
    for (int f = 0; f < 8; f++) {
        WC_LAUNCH(c);
        k_gab_mul<<<dim3(128, njobs), 256, 0, c.st>>>(gj_d, ws, f);
        for (int j = 0; j < njobs; j++)
            cfft2(c, ws + gj[j].c_ws, 1, gj[j].fh, gj[j].fw, plans_d + gj[j].plan_w, plans_d + gj[j].plan_h, tabs);
        WC_LAUNCH(c);
        k_gab_crop<<<dim3(128, njobs), 256, 0, c.st>>>(planes, jobs, gj_d, ws, f);
    }
    WC_LAUNCH(c);
    k_gab_count<<<dim3(njobs, 8), 1024, 0, c.st>>>(planes, jobs, gj_d, ws, counts);
    WC_LAUNCH(c);
    k_gab_final<<<njobs, 32, 0, c.st>>>(jobs, counts, feat);
}

}  // namespace wc
