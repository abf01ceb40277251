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
// k of line l at data + arr*js + l*ls + k*es (units of complex elements), or
// at data + aoff[arr] + l*ls + k*es with a table of array offsets.
// R = double is the FP64 form, R = float the mixed form.
template <typename R>
__global__ void k_cfft_lines(R *__restrict__ data, long long js, int nl, int n, long long ls, long long es,
                             const FFTPlan *__restrict__ plan, const double *__restrict__ twd, int lpc,
                             const long long *__restrict__ aoff) {
    typedef cpx<R> C;
    extern __shared__ __align__(16) unsigned char fsm[];
    const FFTPlan P = *plan;
    const int l0 = blockIdx.x * lpc;
    if (l0 >= nl) return;
    const int lines = min(lpc, nl - l0);
    C *base = (C *)data + (aoff ? aoff[blockIdx.y] : (long long)blockIdx.y * js);
    C *b0 = (C *)fsm, *b1 = b0 + (long long)lpc * n;
    const cplx *tw = (const cplx *)(twd + P.tw_off);
    // the twiddles in the element type, rounded once per block (after the two line buffers)
    C *twr = b1 + (long long)lpc * n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) twr[i] = {(R)tw[i].x, (R)tw[i].y};
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
    const C *r = stockham<R, R>(b0, b1, lines, P, twr) ? b1 : b0;
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

// forward 2-D DFT, in place, of `na` arrays of fh x fw complex values (row-major)
// spaced fh * fw * 16 bytes apart (the workspace is laid out for the FP64 form)
template <typename R>
static void cfft2(Ctx &c, double *data, int na, int fh, int fw, const FFTPlan *plan_w, const FFTPlan *plan_h,
                  const double *tw) {
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_cfft_lines<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr = true;
    }
    const int es = 2 * sizeof(R);
    const long long js = (long long)fh * fw * 16 / es;
    int lpc = 96 * 1024 / (2 * es * fw);
    lpc = lpc < 1 ? 1 : (lpc > 8 ? 8 : lpc);
    WC_LAUNCH(c);
    k_cfft_lines<R><<<dim3((fh + lpc - 1) / lpc, na), 256, ((size_t)lpc * 2 + 1) * fw * es, c.st>>>((R *)data, js, fh, fw, fw, 1,
                                                                                            plan_w, tw, lpc, nullptr);
    int lpc2 = 96 * 1024 / (2 * es * fh);
    lpc2 = lpc2 < 1 ? 1 : (lpc2 > 8 ? 8 : lpc2);
    WC_LAUNCH(c);
    k_cfft_lines<R><<<dim3((fw + lpc2 - 1) / lpc2, na), 256, ((size_t)lpc2 * 2 + 1) * fh * es, c.st>>>((R *)data, js, fw, fh, 1, fw,
                                                                                               plan_h, tw, lpc2, nullptr);
}

// FP64 forward DFTs of na complex arrays of the same shape at complex offsets
// aoff[] from data: the nl lines of length n (element stride es, line stride
// ls) of each, in place (used by the Fourier node's backward pass)
void cfft_lines_fp64(cudaStream_t st, long long *launches, double *data, const long long *aoff, int na, int nl, int n,
                     long long ls, long long es, const FFTPlan *plan, const double *tw) {
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_cfft_lines<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr = true;
    }
    int lpc = 96 * 1024 / (2 * 16 * n);
    lpc = lpc < 1 ? 1 : (lpc > 8 ? 8 : lpc);
    ++*launches;
    k_cfft_lines<double><<<dim3((nl + lpc - 1) / lpc, na), 256, ((size_t)lpc * 2 + 1) * n * 16, st>>>(
        data, 0, nl, n, ls, es, plan, tw, lpc, aoff);
}

// zero-padded image (job) into a fh x fw complex array
template <typename R>
__global__ void k_gab_pad(const double *__restrict__ arena, const Plane *__restrict__ planes, const FJob *__restrict__ jobs,
                          const GabJob *__restrict__ gj, double *__restrict__ ws) {
    const FJob J = jobs[blockIdx.y];
    const GabJob G = gj[blockIdx.y];
    const Plane P = planes[J.plane];
    cpx<R> *A = (cpx<R> *)(ws + G.a_ws);
    const long long n = (long long)G.fh * G.fw;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int y = (int)(i / G.fw), x = (int)(i - (long long)y * G.fw);
        A[i] = {(R)((y < P.h && x < P.w) ? arena[P.off + (long long)y * P.w + x] : 0.0), (R)0};
    }
}

// the 8 kernels (38 x 38 complex, host-made) zero-padded to fh x fw
template <typename R>
__global__ void k_gab_padk(const double *__restrict__ kern, double *__restrict__ Gd, int fh, int fw) {
    const int f = blockIdx.y;
    const long long fstride = (long long)fh * fw * 16 / sizeof(cpx<R>);
    cpx<R> *g = (cpx<R> *)Gd + (long long)f * fstride;
    const long long n = (long long)fh * fw;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int y = (int)(i / fw), x = (int)(i - (long long)y * fw);
        cpx<R> v = {(R)0, (R)0};
        if (y < 38 && x < 38)
            v = {(R)kern[((long long)f * 38 * 38 + y * 38 + x) * 2], (R)kern[((long long)f * 38 * 38 + y * 38 + x) * 2 + 1]};
        g[i] = v;
    }
}

// C_f = conj(A .* G_f) for the 8 filters at once (the inverse transform is
// conj(FFT(conj(X))) / N)
template <typename R>
__global__ void k_gab_mul(const GabJob *__restrict__ gj, double *__restrict__ ws) {
    const GabJob G = gj[blockIdx.y];
    const int f = blockIdx.z;
    const long long fstride = (long long)G.fh * G.fw * 16 / sizeof(cpx<R>);
    const cpx<R> *A = (const cpx<R> *)(ws + G.a_ws);
    const cpx<R> *K = (const cpx<R> *)(ws + G.g_ws) + (long long)f * fstride;
    cpx<R> *Cf = (cpx<R> *)(ws + G.c_ws) + (long long)f * fstride;
    const long long n = (long long)G.fh * G.fw;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const cpx<R> a = A[i], k = K[i];
        Cf[i] = {a.x * k.x - a.y * k.y, -(a.x * k.y + a.y * k.x)};
    }
}

// energy maps e_f(b, a) = |c_f(b + 19, a + 19)| / N, FP64
template <typename R>
__global__ void k_gab_crop(const Plane *__restrict__ planes, const FJob *__restrict__ jobs, const GabJob *__restrict__ gj,
                           double *__restrict__ ws) {
    const FJob J = jobs[blockIdx.y];
    const GabJob G = gj[blockIdx.y];
    const Plane P = planes[J.plane];
    const int f = blockIdx.z;
    const long long fstride = (long long)G.fh * G.fw * 16 / sizeof(cpx<R>);
    const cpx<R> *Cf = (const cpx<R> *)(ws + G.c_ws) + (long long)f * fstride;
    double *e = ws + G.e_ws + (long long)f * P.w * P.h;
    const double invN = 1.0 / ((double)G.fh * G.fw);
    const long long n = (long long)P.w * P.h;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int b = (int)(i / P.w), a = (int)(i - (long long)b * P.w);
        const cpx<R> v = Cf[(long long)(b + 19) * G.fw + a + 19];
        const double re = (double)v.x * invN, im = (double)v.y * invN;
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

template <typename R>
static void gabor_convolve(Ctx &c, const double *arena, const Plane *planes, const FJob *jobs, int njobs,
                           const GabJob *gj_d, const std::vector<GabSize> &sizes, const FFTPlan *plans_d,
                           const double *tabs, long long kern_tab, double *ws) {
    // kernels' spectra, once per padded size
    for (const GabSize &S : sizes) {
        WC_LAUNCH(c);
        k_gab_padk<R><<<dim3(64, 8), 256, 0, c.st>>>(tabs + kern_tab, ws + S.g_ws, S.fh, S.fw);
        cfft2<R>(c, ws + S.g_ws, 8, S.fh, S.fw, plans_d + S.plan_w, plans_d + S.plan_h, tabs);
    }
    WC_LAUNCH(c);
    k_gab_pad<R><<<dim3(128, njobs), 256, 0, c.st>>>(arena, planes, jobs, gj_d, ws);
    // the images' spectra, one batch per padded size (jobs of a size are contiguous)
    for (const GabSize &S : sizes)
        cfft2<R>(c, ws + S.a_ws, S.count, S.fh, S.fw, plans_d + S.plan_w, plans_d + S.plan_h, tabs);
    WC_LAUNCH(c);
    k_gab_mul<R><<<dim3(64, njobs, 8), 256, 0, c.st>>>(gj_d, ws);
    for (const GabSize &S : sizes)
        cfft2<R>(c, ws + S.c_ws, 8 * S.count, S.fh, S.fw, plans_d + S.plan_w, plans_d + S.plan_h, tabs);
    WC_LAUNCH(c);
    k_gab_crop<R><<<dim3(64, njobs, 8), 256, 0, c.st>>>(planes, jobs, gj_d, ws);
}

void launch_gabor(Ctx &c, const double *arena, const Plane *planes, const FJob *jobs, int njobs, const GabJob *gj_d,
                  const std::vector<GabJob> &gj, const std::vector<GabSize> &sizes, const FFTPlan *plans_d,
                  const double *tabs, long long kern_tab, double *ws, double *counts, double *feat) {
    if (njobs <= 0) return;
    (void)gj;
    if (c.prec == WC_PREC_MIXED)
        gabor_convolve<float>(c, arena, planes, jobs, njobs, gj_d, sizes, plans_d, tabs, kern_tab, ws);
    else
        gabor_convolve<double>(c, arena, planes, jobs, njobs, gj_d, sizes, plans_d, tabs, kern_tab, ws);
    WC_LAUNCH(c);
    k_gab_count<<<dim3(njobs, 8), 1024, 0, c.st>>>(planes, jobs, gj_d, ws, counts);
    WC_LAUNCH(c);
    k_gab_final<<<njobs, 32, 0, c.st>>>(jobs, counts, feat);
}

}  // namespace wc
