// Zernike and Chebyshev-Fourier coefficients (FP64 form).
//
// Zernike: mb_zernike2D, src/textures/zernike/zernike.cpp:207-341: order 15,
// rad = min(W,H), unit disc centred on the intensity centroid (1-based
// coordinates), f = I / sum(I), q-recursive radial polynomials with the H1/H2/H3
// coefficients; output |A_nm| for n - m even (72 values).
//
// Chebyshev-Fourier: ChebyshevFourierTransform2D + ChebyshevFourier2D,
// src/cmatrix.cpp:1227-1240, src/transforms/ChebyshevFourier.cpp:42-160: planes
// above 300*300 pixels are area-downsampled first (ImageMatrix::Downsample,
// src/cmatrix.cpp:579-720); then c_{m,a} = sum over pixels in the unit disc of
// I * Ftrm_m e^{-i m phi} * T_a(2r-1) for |m| <= N, a < 2N+1 (N = 11 capped by the
// size), and a 32-bin histogram of |c|.
#include <cfloat>
#include <cmath>

#include "kcommon.cuh"
#include "kdf32.cuh"
#include "kernels.h"

namespace wc {

// ---------------------------------------------------------------- Zernike
__constant__ double c_zH1[16][16], c_zH2[16][16], c_zH3[16][16];
static const double kZPI = 3.14159265358979323846264338328;  // zernike.cpp:38

void set_zernike_tables() {
    double H1[16][16] = {{0}}, H2[16][16] = {{0}}, H3[16][16] = {{0}};
    for (int n = 0; n < 16; n++)
        for (int m = 0; m <= n; m++)
            if (n != m) {
                H3[n][m] = -(double)(4.0 * (m + 2.0) * (m + 1.0)) / (double)((n + m + 2.0) * (n - m));
                H2[n][m] = ((double)(H3[n][m] * (n + m + 4.0) * (n - m - 2.0)) / (double)(4.0 * (m + 3.0))) + (m + 2.0);
                H1[n][m] = ((double)((m + 4.0) * (m + 3.0)) / 2.0) - ((m + 4.0) * H2[n][m]) +
                           ((double)(H3[n][m] * (n + m + 6.0) * (n - m - 4.0)) / 8.0);
            }
    cudaMemcpyToSymbol(c_zH1, H1, sizeof H1);
    cudaMemcpyToSymbol(c_zH2, H2, sizeof H2);
    cudaMemcpyToSymbol(c_zH3, H3, sizeof H3);
}

// first pass: centroid moments per job (sum, sum (x+1) I, sum (y+1) I)
__global__ void k_zern_moments(const double *__restrict__ arena, const Plane *__restrict__ planes,
                               const FJob *__restrict__ jobs, double *__restrict__ mom) {
    __shared__ double sh[32];
    const FJob J = jobs[blockIdx.x];
    const Plane P = planes[J.plane];
    const double *p = arena + P.off;
    double s = 0, sx = 0, sy = 0;
    const long long n = (long long)P.w * P.h;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        const long long y = i / P.w, x = i - y * P.w;
        const double I = p[i];
        s += I;
        sx += (double)(x + 1) * I;
        sy += (double)(y + 1) * I;
    }
    s = block_sum(s, sh);
    sx = block_sum(sx, sh);
    sy = block_sum(sy, sh);
    if (threadIdx.x == 0) {
        mom[3 * blockIdx.x + 0] = s;
        mom[3 * blockIdx.x + 1] = sx / s;
        mom[3 * blockIdx.x + 2] = sy / s;
    }
}

#define ZCHUNK 2048
// second pass: per (chunk of pixels, half, job): per-CTA partial AR/AI.
// HALF 0 covers n = 0..10, HALF 1 covers n = 11..15 (36 (n, m) pairs each).
// (FP64 form, the reference's operations; the mixed form uses k_zern_cmom_df.)
template <int HALF>
__global__ void __launch_bounds__(256) k_zern_accum(const double *__restrict__ arena, const Plane *__restrict__ planes,
                                                    const FJob *__restrict__ jobs, const double *__restrict__ mom,
                                                    double *__restrict__ part, int nchunk) {
    constexpr int NLO = HALF ? 11 : 0, NHI = HALF ? 15 : 10;
    __shared__ double red[8][72];
    const FJob J = jobs[blockIdx.z];
    const Plane P = planes[J.plane];
    const long long npix = (long long)P.w * P.h;
    const long long c0 = (long long)blockIdx.x * ZCHUNK;
    double acc[72];
#pragma unroll
    for (int q = 0; q < 72; q++) acc[q] = 0.0;
    if (c0 < npix) {
        const double sum = mom[3 * blockIdx.z], cx = mom[3 * blockIdx.z + 1], cy = mom[3 * blockIdx.z + 2];
        const double rad = (double)(P.w < P.h ? P.w : P.h);
        const double *p = arena + P.off;
        const long long c1 = min(npix, c0 + ZCHUNK);
        for (long long i = c0 + threadIdx.x; i < c1; i += blockDim.x) {
            const long long yy = i / P.w, xx = i - yy * P.w;
            const double dx = __dsub_rn((double)(xx + 1), cx), dy = __dsub_rn((double)(yy + 1), cy);
            const double x = dx / rad, y = dy / rad;
            const double r2 = __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), r = sqrt(r2);
            if (r < DBL_EPSILON || r > 1.0) continue;
            double R[16], CO[16], SI[16];
            R[0] = 1;
#pragma unroll
            for (int n = 1; n <= 15; n++) R[n] = r * R[n - 1];
            const double a = x / r, b = y / r;
            CO[0] = a;
            SI[0] = b;
#pragma unroll
            for (int m = 1; m <= 15; m++) {
                CO[m] = a * CO[m - 1] - b * SI[m - 1];
                SI[m] = a * SI[m - 1] + b * CO[m - 1];
            }
            const double f = p[i] / sum;
            int q = 0;
#pragma unroll
            for (int n = NLO; n <= NHI; n++) {
                const double ct = (n + 1) * f / kZPI;
                const double Rn = R[n], Rnm2 = n >= 2 ? R[n - 2] : 0.0;
                double Rnm = 0, Rnmp2 = 0, Rnmp4 = 0;
                const int cnt = n / 2 + 1;
#pragma unroll
                for (int t = 0; t < cnt; t++) {
                    const int m = n - 2 * t;
                    if (m == n) {
                        Rnm = Rn;
                        Rnmp4 = Rn;
                    } else if (m == n - 2) {
                        Rnm = n * Rn - (n - 1) * Rnm2;
                        Rnmp2 = Rnm;
                    } else {
                        Rnm = c_zH1[n][m] * Rnmp4 + (c_zH2[n][m] + (c_zH3[n][m] / r2)) * Rnmp2;
                        Rnmp4 = Rnmp2;
                        Rnmp2 = Rnm;
                    }
                    const int slot = q + (cnt - 1 - t);  // m ascending within n
                    acc[2 * slot] += ct * Rnm * CO[m];
                    acc[2 * slot + 1] -= ct * Rnm * SI[m];
                }
                q += cnt;
            }
        }
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int qq = 0; qq < 72; qq++) {
        double v = warp_sum(acc[qq]);
        if (lane == 0) red[wid][qq] = v;
    }
    __syncthreads();
    if (threadIdx.x < 72) {
        double s = 0;
        for (int w = 0; w < 8; w++) s += red[w][threadIdx.x];
        part[(((long long)blockIdx.z * 2 + HALF) * nchunk + blockIdx.x) * 72 + threadIdx.x] = s;
    }
}

__global__ void k_zern_finish(const FJob *__restrict__ jobs, const double *__restrict__ part, int nchunk,
                              double *__restrict__ feat) {
    const FJob J = jobs[blockIdx.x];
    const int t = threadIdx.x;  // 72 outputs
    if (t >= 72) return;
    const int half = t >= 36, slot = t - 36 * half;
    double ar = 0, ai = 0;
    for (int c = 0; c < nchunk; c++) {
        const double *pp = part + (((long long)blockIdx.x * 2 + half) * nchunk + c) * 72;
        ar += pp[2 * slot];
        ai += pp[2 * slot + 1];
    }
    ar *= ar;
    ai *= ai;
    feat[J.out + t] = fabs(sqrt(ar + ai));
}

// Mixed form: the same moments through complex moments.  With the reference's
// angular factor cos((m+1) phi), sin((m+1) phi) (its COST/SINT arrays start at
// the first harmonic, zernike.cpp:287-296) and R_nm(r) = sum_s c_nms r^(n-2s),
//   R_nm e^{-i(m+1) phi} = sum_s c_nms (r^2)^j zbar^(m+1) / r,   j = (n-m)/2 - s,
// zbar = x - i y; so A_nm = (n+1)/pi sum_s c_nms M(j, m+1) with the 72 complex
// moments M(j, m') = sum f (r^2)^j zbar^m' / r, and the exact integer
// coefficients c_nms = (-1)^s (n-s)! / (s! ((n+m)/2-s)! ((n-m)/2-s)!) applied once
// per job in FP64 (k_zern_finish_cmom).  HALF 0: m' = 1..5, HALF 1: m' = 6..16
// (36 moments each, m' ascending, j = 0..(16-m')/2 ascending).
// The moments are summed in pairs of floats (about 48 bits, on the FP32
// pipe instead of the FP64 one).  Whether a pixel lies
// in the unit disc is decided as the FP64 kernel decides it: the pair estimate
// of r^2 decides away from 1 and 0, the FP64 test within 1e-6 of them.  Chunks
// of ZCHUNK_DF pixels per block; the block's sums are reduced in pairs within
// each warp and in FP64 across the warps.
#define ZCHUNK_DF 16384
// the FP64 kernel's disc test, for the pixels near the rim or the centre (a
// call, so that the common path issues none of its FP64 instructions)
static __device__ __noinline__ bool zern_in_disc(long long xx, long long yy, double cx, double cy, double inv_rad) {
    const double xe = __dsub_rn((double)(xx + 1), cx) * inv_rad, ye = __dsub_rn((double)(yy + 1), cy) * inv_rad;
    const double r = sqrt(__dadd_rn(__dmul_rn(xe, xe), __dmul_rn(ye, ye)));
    return !(r < DBL_EPSILON || r > 1.0);
}
template <int HALF>
__global__ void __launch_bounds__(256) k_zern_cmom_df(const double *__restrict__ arena, const Plane *__restrict__ planes,
                                                      const FJob *__restrict__ jobs, const double *__restrict__ mom,
                                                      double *__restrict__ part, int nchunk) {
    constexpr int M0 = HALF ? 6 : 1, M1 = HALF ? 16 : 5, JMAX = (16 - M0) / 2;
    __shared__ double red[8][72];
    const FJob J = jobs[blockIdx.z];
    const Plane P = planes[J.plane];
    const long long npix = (long long)P.w * P.h;
    const long long c0 = (long long)blockIdx.x * ZCHUNK_DF;
    df acc[72];
#pragma unroll
    for (int q = 0; q < 72; q++) acc[q] = {0.f, 0.f};
    if (c0 < npix) {
        const double sum = mom[3 * blockIdx.z], cx = mom[3 * blockIdx.z + 1], cy = mom[3 * blockIdx.z + 2];
        const double inv_rad = 1.0 / (double)(P.w < P.h ? P.w : P.h), inv_sum = 1.0 / sum;
        const df cxd = df_from_double(cx), cyd = df_from_double(cy), ird = df_from_double(inv_rad),
                 isd = df_from_double(inv_sum);
        const double *p = arena + P.off;
        const long long c1 = min(npix, c0 + ZCHUNK_DF);
        for (long long i = c0 + threadIdx.x; i < c1; i += blockDim.x) {
            const long long yy = i / P.w, xx = i - yy * P.w;
            const df x = df_mul(df_sub({(float)(xx + 1), 0.f}, cxd), ird);
            const df y = df_mul(df_sub({(float)(yy + 1), 0.f}, cyd), ird);
            const df r2 = df_add(df_mul(x, x), df_mul(y, y));
            const bool in = (fabsf(r2.hi - 1.f) < 1e-6f || r2.hi < 1e-20f) ? zern_in_disc(xx, yy, cx, cy, inv_rad)
                                                                            : r2.hi < 1.f;
            if (!in) continue;
            const df r = df_sqrt(r2);
            df q[JMAX + 1];
            q[0] = df_div(df_mul(df_split(p[i]), isd), r);
#pragma unroll
            for (int j = 1; j <= JMAX; j++) q[j] = df_mul(q[j - 1], r2);
            df zr = x, zi = df_neg(y);  // zbar^1
#pragma unroll
            for (int mp = 2; mp <= M0; mp++) {
                const df t = df_add(df_mul(zr, x), df_mul(zi, y));
                zi = df_sub(df_mul(zi, x), df_mul(zr, y));
                zr = t;
            }
            int slot = 0;
#pragma unroll
            for (int mp = M0; mp <= M1; mp++) {
                if (mp > M0) {
                    const df t = df_add(df_mul(zr, x), df_mul(zi, y));
                    zi = df_sub(df_mul(zi, x), df_mul(zr, y));
                    zr = t;
                }
#pragma unroll
                for (int j = 0; j <= (16 - mp) / 2; j++) {
                    acc[2 * slot] = df_add(acc[2 * slot], df_mul(q[j], zr));
                    acc[2 * slot + 1] = df_add(acc[2 * slot + 1], df_mul(q[j], zi));
                    slot++;
                }
            }
        }
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int qq = 0; qq < 72; qq++) {
        df v = acc[qq];
        for (int o = 16; o > 0; o >>= 1)
            v = df_add(v, {__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)});
        if (lane == 0) red[wid][qq] = df_to_double(v);
    }
    __syncthreads();
    if (threadIdx.x < 72) {
        double s = 0;
        for (int w = 0; w < 8; w++) s += red[w][threadIdx.x];
        part[(((long long)blockIdx.z * 2 + HALF) * nchunk + blockIdx.x) * 72 + threadIdx.x] = s;
    }
}

__device__ __forceinline__ double dfact(int k) {
    double f = 1;
    for (int i = 2; i <= k; i++) f *= i;
    return f;
}

__global__ void k_zern_finish_cmom(const FJob *__restrict__ jobs, const double *__restrict__ part, int nchunk,
                                   double *__restrict__ feat) {
    __shared__ double M[144];
    const FJob J = jobs[blockIdx.x];
    const int t = threadIdx.x;
    for (int v = t; v < 144; v += blockDim.x) {
        const int half = v >= 72, k = v - 72 * half;
        double s = 0;
        for (int c = 0; c < nchunk; c++) s += part[(((long long)blockIdx.x * 2 + half) * nchunk + c) * 72 + k];
        M[v] = s;
    }
    __syncthreads();
    if (t >= 72) return;
    int n = 0, m = 0, idx = 0;  // output t is the t-th (n, m), n ascending, m ascending, n - m even
    for (n = 0; n <= 15; n++) {
        const int cnt = n / 2 + 1;
        if (t < idx + cnt) {
            m = (n & 1) + 2 * (t - idx);
            break;
        }
        idx += cnt;
    }
    const int mp = m + 1, half = mp >= 6, m0 = half ? 6 : 1;
    int base = 0;
    for (int u = m0; u < mp; u++) base += (16 - u) / 2 + 1;
    double zr = 0, zi = 0;
    for (int s = 0; s <= (n - m) / 2; s++) {
        const double c = ((s & 1) ? -1.0 : 1.0) * dfact(n - s) / (dfact(s) * dfact((n + m) / 2 - s) * dfact((n - m) / 2 - s));
        const int j = (n - m) / 2 - s;
        const int v = 72 * half + 2 * (base + j);
        zr += c * M[v];
        zi += c * M[v + 1];
    }
    const double sc = (n + 1) / kZPI;
    double ar = zr * sc, ai = zi * sc;
    ar *= ar;
    ai *= ai;
    feat[J.out + t] = fabs(sqrt(ar + ai));
}

void launch_zernike(Ctx &c, const double *arena, const Plane *planes, const FJob *jobs, int njobs, long long maxpix,
                    double *mom, double *part, double *feat) {
    if (njobs <= 0) return;
    const int nchunk = (int)((maxpix + ZCHUNK - 1) / ZCHUNK);
    WC_LAUNCH(c);
    k_zern_moments<<<njobs, 512, 0, c.st>>>(arena, planes, jobs, mom);
    if (c.prec == WC_PREC_MIXED) {
        const int nch = (int)((maxpix + ZCHUNK_DF - 1) / ZCHUNK_DF);
        WC_LAUNCH(c);
        k_zern_cmom_df<0><<<dim3(nch, 1, njobs), 256, 0, c.st>>>(arena, planes, jobs, mom, part, nch);
        WC_LAUNCH(c);
        k_zern_cmom_df<1><<<dim3(nch, 1, njobs), 256, 0, c.st>>>(arena, planes, jobs, mom, part, nch);
        WC_LAUNCH(c);
        k_zern_finish_cmom<<<njobs, 160, 0, c.st>>>(jobs, part, nch, feat);
        return;
    }
    WC_LAUNCH(c);
    k_zern_accum<0><<<dim3(nchunk, 1, njobs), 256, 0, c.st>>>(arena, planes, jobs, mom, part, nchunk);
    WC_LAUNCH(c);
    k_zern_accum<1><<<dim3(nchunk, 1, njobs), 256, 0, c.st>>>(arena, planes, jobs, mom, part, nchunk);
    WC_LAUNCH(c);
    k_zern_finish<<<njobs, 96, 0, c.st>>>(jobs, part, nchunk, feat);
}


// ---------------------------------------------------------------- Chebyshev-Fourier
// Downsample pass along x (src/cmatrix.cpp:602-656): for every source row, the
// k-th output averages the source over [xs[k], xs[k] + dx); xs holds the
// reference's accumulated positions (x += dx), computed on the host.
__device__ double ds_interval(const double *__restrict__ src, long long stride, int old, double x, double dx) {
    double s = 0, frac;
    unsigned a = (unsigned)floor(x);
    frac = ceil(x) - x;
    if (frac > 0 && a < (unsigned)old) s += src[(long long)a * stride] * frac;
    for (a = (unsigned)ceil(x); a < floor(x + dx); a++)
        if (a < (unsigned)old) s += src[(long long)a * stride];
    frac = x + dx - floor(x + dx);
    if (frac > 0 && a < (unsigned)old) s += src[(long long)a * stride] * frac;
    return s / dx;
}

__global__ void k_cf_down_x(const double *__restrict__ arena, const Plane *__restrict__ planes, const FJob *__restrict__ jobs,
                            const CFJob *__restrict__ cj, const double *__restrict__ tabs, double *__restrict__ ws) {
    const FJob J = jobs[blockIdx.z];
    const CFJob C = cj[blockIdx.z];
    const Plane P = planes[J.plane];
    const int k = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (y >= P.h) return;
    if (!C.down) {  // copy the plane as the source image
        for (int x = k; x < P.w; x += gridDim.x * blockDim.x)
            ws[C.src_ws + (long long)y * P.w + x] = arena[P.off + (long long)y * P.w + x];
        return;
    }
    if (k >= C.cnt_x) return;
    ws[C.tmp_ws + (long long)y * C.cnt_x + k] =
        ds_interval(arena + P.off + (long long)y * P.w, 1, P.w, tabs[C.xs_tab + k], C.dx);
}

__global__ void k_cf_down_y(const Plane *__restrict__ planes, const FJob *__restrict__ jobs, const CFJob *__restrict__ cj,
                            const double *__restrict__ tabs, double *__restrict__ ws) {
    const FJob J = jobs[blockIdx.z];
    const CFJob C = cj[blockIdx.z];
    if (!C.down) return;
    const Plane P = planes[J.plane];
    const int x = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= C.new_w || k >= C.cnt_y || k >= C.new_h) return;
    ws[C.src_ws + (long long)k * C.new_w + x] =
        ds_interval(ws + C.tmp_ws + x, C.cnt_x, P.h, tabs[C.ys_tab + k], C.dx);
}

#define CF_SUB 128
#define CF_CHUNK 1024
// per (chunk of 1024 pixel indices, job): partial sums of the 2*NN*NN coefficients
__global__ void __launch_bounds__(256) k_cf_accum(const CFJob *__restrict__ cj, const double *__restrict__ ws,
                                                  double *__restrict__ part, int nchunk_max) {
    extern __shared__ double sm[];
    const CFJob C = cj[blockIdx.y];
    const int m = C.new_h, n = C.new_w;  // rows, cols of the source image
    const long long npix = (long long)m * n;
    const long long c0 = (long long)blockIdx.x * CF_CHUNK;
    int N = 11;
    const int Nmax = (min(m, n) - 1) / 2;
    if (N > Nmax) N = Nmax;
    const int NN = 2 * N + 1, NO = NN * NN;
    double *T = sm;                     // CF_SUB x NN
    double *Fc = T + CF_SUB * 23;       // CF_SUB x NN
    double *Fs = Fc + CF_SUB * 23;      // CF_SUB x NN
    double *Iv = Fs + CF_SUB * 23;      // CF_SUB
    __shared__ int valid;
    double acc_r[5], acc_i[5];
    for (int q = 0; q < 5; q++) acc_r[q] = acc_i[q] = 0;
    const double *img = ws + C.src_ws;
    const double tn = 2.0 / ((double)n - 1), tm = 2.0 / ((double)m - 1);
    for (long long s0 = c0; s0 < min(npix, c0 + CF_CHUNK); s0 += CF_SUB) {
        if (threadIdx.x == 0) valid = 0;
        __syncthreads();
        if (threadIdx.x < CF_SUB) {
            const long long ind = s0 + threadIdx.x;  // x-major: ind = x*m + y
            double Ival = 0;
            if (ind < npix && ind < c0 + CF_CHUNK) {
                const long long x = ind / m, y = ind - x * m;
                // exact reference rounding (no contraction): decides r < 1 on the circle
                const double xi = __dadd_rn(-1.0, __dmul_rn((double)x, tn)), yi = __dadd_rn(-1.0, __dmul_rn((double)y, tm));
                const double r = sqrt(__dadd_rn(__dmul_rn(xi, xi), __dmul_rn(yi, yi)));
                if (r < 1) {
                    Ival = img[y * n + x];
                    double xx = __dsub_rn(__dmul_rn(r, 2.0), 1.0);
                    if (xx < -1) xx = -1;
                    if (xx > 1) xx = 1;
                    const double ac = acos(xx);
                    for (int a = 0; a < NN; a++) T[threadIdx.x * 23 + a] = cos(a * ac);
                    T[threadIdx.x * 23 + 0] = 0.5;
                    const double fi = -1 * atan2(yi, xi);
                    for (int im = 1; im <= NN; im++) {
                        const long mf = im - 1 - N;
                        const double Ft = (mf == 0) ? 0.5 : 1.0;
                        Fc[threadIdx.x * 23 + im - 1] = Ft * cos(mf * fi);
                        Fs[threadIdx.x * 23 + im - 1] = Ft * sin(-1 * mf * fi);
                    }
                    atomicAdd(&valid, 1);
                }
            }
            Iv[threadIdx.x] = Ival;
        }
        __syncthreads();
        if (valid) {
            for (int q = 0; q < 5; q++) {
                const int o = threadIdx.x + q * 256;
                if (o >= NO) break;
                const int im = o / NN, a = o - im * NN;
                double sr = acc_r[q], si = acc_i[q];
                for (int pp = 0; pp < CF_SUB; pp++) {
                    const double I = Iv[pp];
                    if (I == 0.0) continue;  // outside the disc, or a zero pixel (adds 0)
                    sr += (Fc[pp * 23 + im] * T[pp * 23 + a]) * I;
                    si += (Fs[pp * 23 + im] * T[pp * 23 + a]) * I;
                }
                acc_r[q] = sr;
                acc_i[q] = si;
            }
        }
        __syncthreads();
    }
    double *out = part + ((long long)blockIdx.y * nchunk_max + blockIdx.x) * (2 * 529);
    for (int q = 0; q < 5; q++) {
        const int o = threadIdx.x + q * 256;
        if (o < NO) {
            out[2 * o] = acc_r[q];
            out[2 * o + 1] = acc_i[q];
        }
    }
}

// Mixed form of the accumulation: the unit-disc test and r stay FP64 (they
// decide which pixels count, exactly as above); the basis is FP32 (T_a(2r-1) by
// the three-term recurrence, e^{-i m phi} by repeated complex multiplication by
// e^{-i phi}), and every thread sums at most CF_CHUNK / 8 products per output in
// FP32 before the FP64 reduction over threads and chunks.
// Threads: 8 pixel streams x 23 rows m; each owns the 2 x NN outputs of its row.
#define CF32_PX 184
__global__ void __launch_bounds__(192) k_cf_accum_f32(const CFJob *__restrict__ cj, const double *__restrict__ ws,
                                                      double *__restrict__ part, int nchunk_max) {
    extern __shared__ __align__(16) float cfsm[];  // Gc, Gs, Tb: [CF32_PX][24] each; red aliases them at the end
    float(*Gc)[24] = (float(*)[24])cfsm;
    float(*Gs)[24] = (float(*)[24])(cfsm + CF32_PX * 24);
    float(*Tb)[24] = (float(*)[24])(cfsm + 2 * CF32_PX * 24);
    double(*red)[47] = (double(*)[47])cfsm;
    const CFJob C = cj[blockIdx.y];
    const int m = C.new_h, n = C.new_w;
    const long long npix = (long long)m * n;
    const long long c0 = (long long)blockIdx.x * CF_CHUNK;
    int N = 11;
    const int Nmax = (min(m, n) - 1) / 2;
    if (N > Nmax) N = Nmax;
    const int NN = 2 * N + 1;
    const double *img = ws + C.src_ws;
    const double tn = 2.0 / ((double)n - 1), tm = 2.0 / ((double)m - 1);
    const int t = threadIdx.x, st = t / 23, row = t - 23 * st;
    float ar[23], ai[23];
#pragma unroll
    for (int a = 0; a < 23; a++) ar[a] = ai[a] = 0.f;
    const long long cend = min(npix, c0 + CF_CHUNK);
    for (long long s0 = c0; s0 < cend; s0 += CF32_PX) {
        if (t < CF32_PX) {
            const long long ind = s0 + t;  // x-major: ind = x*m + y
            float I = 0.f, xx = 0.f, ca = 1.f, sa = 0.f;
            if (ind < cend) {
                const long long x = ind / m, y = ind - x * m;
                const double xi = __dadd_rn(-1.0, __dmul_rn((double)x, tn)), yi = __dadd_rn(-1.0, __dmul_rn((double)y, tm));
                const double r = sqrt(__dadd_rn(__dmul_rn(xi, xi), __dmul_rn(yi, yi)));
                if (r < 1) {
                    I = (float)img[y * n + x];
                    double xd = __dsub_rn(__dmul_rn(r, 2.0), 1.0);
                    xx = (float)fmin(1.0, fmax(-1.0, xd));
                    const float ph = -atan2f((float)yi, (float)xi);  // phi; e^{-i phi} = (cos, -sin)
                    sincosf(ph, &sa, &ca);
                }
            }
            // T_a(xx), T_0 = 0.5 as the reference sets it
            float tp = 1.f, tc = xx;
            Tb[t][0] = 0.5f;
            if (NN > 1) Tb[t][1] = xx;
            for (int a = 2; a < NN; a++) {
                const float tnx = 2.f * xx * tc - tp;
                tp = tc;
                tc = tnx;
                Tb[t][a] = tnx;
            }
            // rows im = mf + N, mf = -N..N: Ft cos(mf phi) I, Ft sin(-mf phi) I
            Gc[t][N] = 0.5f * I;
            Gs[t][N] = 0.f;
            float ck = 1.f, sk = 0.f;
            for (int k = 1; k <= N; k++) {
                const float c2 = ck * ca - sk * sa, s2 = sk * ca + ck * sa;  // cos(k phi), sin(k phi)
                ck = c2;
                sk = s2;
                Gc[t][N + k] = ck * I;
                Gs[t][N + k] = -sk * I;
                Gc[t][N - k] = ck * I;
                Gs[t][N - k] = sk * I;
            }
        }
        __syncthreads();
        if (t < CF32_PX && row < NN) {
            const int npx = (int)min((long long)CF32_PX, cend - s0);
            for (int p = st; p < npx; p += 8) {
                const float gc = Gc[p][row], gs = Gs[p][row];
#pragma unroll
                for (int a = 0; a < 23; a++) {
                    const float tb = Tb[p][a];
                    ar[a] = fmaf(gc, tb, ar[a]);
                    ai[a] = fmaf(gs, tb, ai[a]);
                }
            }
        }
        __syncthreads();
    }
    // reduce the 8 streams in FP64, fixed order (the staging buffers are free now)
    double *out = part + ((long long)blockIdx.y * nchunk_max + blockIdx.x) * (2 * 529);
    for (int s = 0; s < 8; s++) {
        if (st == s && t < CF32_PX)
            for (int a = 0; a < 23; a++) {
                red[row][2 * a] = (s ? red[row][2 * a] : 0.0) + (double)ar[a];
                red[row][2 * a + 1] = (s ? red[row][2 * a + 1] : 0.0) + (double)ai[a];
            }
        __syncthreads();
    }
    for (int o = t; o < NN * NN; o += blockDim.x) {
        const int im = o / NN, a = o - im * NN;
        out[2 * o] = red[im][2 * a];
        out[2 * o + 1] = red[im][2 * a + 1];
    }
}

__global__ void k_cf_finish(const FJob *__restrict__ jobs, const CFJob *__restrict__ cj, const double *__restrict__ part,
                            int nchunk_max, int nch_force, double *__restrict__ feat) {
    __shared__ double co[529];
    __shared__ double sh[32];
    __shared__ unsigned int bins[32];
    const FJob J = jobs[blockIdx.x];
    const CFJob C = cj[blockIdx.x];
    int N = 11;
    const int Nmax = (min(C.new_h, C.new_w) - 1) / 2;
    if (N > Nmax) N = Nmax;
    const int NN = 2 * N + 1, NO = NN * NN;
    const long long npix = (long long)C.new_w * C.new_h;
    const int nch = nch_force > 0 ? nch_force : (int)((npix + CF_CHUNK - 1) / CF_CHUNK);
    double lo = 10E200, hi = -10E200;
    for (int o = threadIdx.x; o < NO; o += blockDim.x) {
        double sr = 0, si = 0;
        for (int c = 0; c < nch; c++) {
            const double *pp = part + ((long long)blockIdx.x * nchunk_max + c) * (2 * 529);
            sr += pp[2 * o];
            si += pp[2 * o + 1];
        }
        const double v = sqrt(sr * sr + si * si);
        co[o] = v;
        lo = fmin(lo, v);
        hi = fmax(hi, v);
    }
    lo = block_min(lo, sh);
    hi = block_max(hi, sh);
    if (threadIdx.x < 32) bins[threadIdx.x] = 0;
    __syncthreads();
    if (hi - lo > 0) {
        const double sc = 32.0 / double(hi - lo);
        for (int o = threadIdx.x; o < NO; o += blockDim.x) atomicAdd(&bins[hist_bin(co[o], lo, sc, 32)], 1u);
    }
    __syncthreads();
    if (threadIdx.x < 32) feat[J.out + threadIdx.x] = (double)bins[threadIdx.x];
}

void launch_chebfourier(Ctx &c, const double *arena, const Plane *planes, const FJob *jobs, int njobs, int maxw,
                        int maxh, int max_cnt_x, int max_src_w, int max_src_h, const CFJob *cj, const double *tabs,
                        double *ws, double *part, int nchunk_max, double *feat, const CFTcPlan *tcp,
                        const CFTcBufs *tcb) {
    if (njobs <= 0) return;
    dim3 b(32, 8);
    WC_LAUNCH(c);
    k_cf_down_x<<<dim3((max(max_cnt_x, maxw) + 31) / 32, (maxh + 7) / 8, njobs), b, 0, c.st>>>(arena, planes, jobs, cj,
                                                                                             tabs, ws);
    WC_LAUNCH(c);
    k_cf_down_y<<<dim3((max_src_w + 31) / 32, (max_src_h + 7) / 8, njobs), b, 0, c.st>>>(planes, jobs, cj, tabs, ws);
    const size_t sm = (size_t)CF_SUB * (3 * 23 + 1) * sizeof(double);
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_cf_accum, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        attr = true;
    }
    // the mixed form: the tensor-core sums where every plane has one size (the
    // host planned their buffers), else FP32 SIMT sums
    const bool tc = c.prec == WC_PREC_MIXED && tcp && tcb &&
                    launch_cf_tc(c, cj, njobs, max_src_h, max_src_w, ws, *tcp, *tcb, part, nchunk_max);
    if (!tc) {
        WC_LAUNCH(c);
        if (c.prec == WC_PREC_MIXED) {
            const int sm32 = 3 * CF32_PX * 24 * sizeof(float);
            static bool attr32 = false;
            if (!attr32) {
                cudaFuncSetAttribute(k_cf_accum_f32, cudaFuncAttributeMaxDynamicSharedMemorySize, sm32);
                attr32 = true;
            }
            k_cf_accum_f32<<<dim3(nchunk_max, njobs), 192, sm32, c.st>>>(cj, ws, part, nchunk_max);
        } else {
            k_cf_accum<<<dim3(nchunk_max, njobs), 256, sm, c.st>>>(cj, ws, part, nchunk_max);
        }
    }
    WC_LAUNCH(c);
    k_cf_finish<<<njobs, 256, 0, c.st>>>(jobs, cj, part, nchunk_max, tc ? 1 : 0, feat);
}

}  // namespace wc
