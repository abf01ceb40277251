// Tamura textures (FP64 form): Tamura3Sigs2D, src/textures/tamura.cpp:10-299.
//   normImg = (p - min) / max
//   coarseness: running sums S(y,x) = I + S(y,x-1) + S(y-1,x) - S(y-1,x-1) with
//     the reference's exact recurrence (an anti-diagonal wavefront, so every
//     entry is rounded exactly as on the CPU), local means over 2^k windows via
//     efficientLocalMean (:106-139), best scale per pixel, mean and a 3-bin
//     histogram normalised by its largest bin;
//   directionality: 3x3 zero-padded correlations with the kernels as the
//     reference's assignments leave them (:45-57), phi = atan(dV/dH)+pi/2+0.001
//     where dH >= 1e-4, 125-bin histogram;
//   contrast: std / (kurtosis / std^4)^(1/4) from Moments4 (no -3).
// Output order: hist0, hist1, hist2, contrast, directionality, coarseness.
#include <algorithm>
#include <cfloat>
#include <cmath>

#include "kcommon.cuh"
#include "kernels.h"

namespace wc {

// S table by anti-diagonals; one CTA per job.  norm written on the fly.
__global__ void __launch_bounds__(1024) k_tam_prefix(const double *__restrict__ arena, const Plane *__restrict__ planes,
                                                     const PlaneStats *__restrict__ stats, const FJob *__restrict__ jobs,
                                                     const TamJob *__restrict__ tj, double *__restrict__ ws) {
    const FJob J = jobs[blockIdx.x];
    const Plane P = planes[J.plane];
    const PlaneStats St = stats[J.plane];
    const TamJob T = tj[blockIdx.x];
    const int W = P.w, H = P.h;
    const double *p = arena + P.off;
    double *nrm = ws + T.norm_ws, *S = ws + T.sum_ws;
    for (long long i = threadIdx.x; i < (long long)W * H; i += blockDim.x) nrm[i] = (p[i] - St.mn) / St.mx;
    __syncthreads();
    for (int d = 0; d < W + H - 1; d++) {
        const int y0 = max(0, d - (W - 1)), y1 = min(d, H - 1);
        for (int y = y0 + threadIdx.x; y <= y1; y += blockDim.x) {
            const int x = d - y;
            const double l = (x < 1) ? 0 : S[(long long)y * W + x - 1];
            const double o = (y < 1) ? 0 : S[(long long)(y - 1) * W + x];
            const double ol = (y < 1 || x < 1) ? 0 : S[(long long)(y - 1) * W + x - 1];
            S[(long long)y * W + x] = __dsub_rn(__dadd_rn(__dadd_rn(nrm[(long long)y * W + x], l), o), ol);
        }
        __syncthreads();
    }
}

// v / cnt for the clipped windows (and the quotients that leave the normal
// range): a call, so that the common path issues none of its FP64 instructions
static __device__ __noinline__ double mean_slow(double v, long long cnt) {
    if ((cnt & (cnt - 1)) == 0) return __dmul_rn(v, __longlong_as_double((long long)(1023 - (__ffsll(cnt) - 1)) << 52));
    return v / (double)cnt;
}

// efficientLocalMean (tamura.cpp:106-139)
__device__ __forceinline__ double local_mean(const double *__restrict__ S, int W, int H, long long x, long long y, long long k) {
    const long long k2 = k / 2;
    long long sy = y - k2, sx = x - k2, ey = y + k2 - 1, ex = x + k2 - 1;
    if (sy < 0) sy = 0;
    if (sx < 0) sx = 0;
    if (ex > W - 1) ex = W - 1;
    if (ey > H - 1) ey = H - 1;
    const double links = (sx - 1 < 0) ? 0 : S[ey * W + sx - 1];
    const double oben = (sy - 1 < 0) ? 0 : S[(ey - 1) * W + sx];
    const double ol = ((sy - 1 < 0) || (sx - 1 < 0)) ? 0 : S[(ey - 1) * W + sx - 1];
    const double unten = S[ey * W + sx];
    const long long cnt = (ey - sy + 1) * (ex - sx + 1);
    const double v = __dadd_rn(__dsub_rn(__dsub_rn(unten, links), oben), ol);
    // an unclipped window holds a power-of-two count: dividing by 2^e and
    // multiplying by the exact 2^-e round identically; while the quotient stays
    // normal that is an exponent decrement on the integer pipe
    if ((cnt & (cnt - 1)) == 0) {
        const int e = __ffsll(cnt) - 1;
        const long long b = __double_as_longlong(v);
        const int E = (int)((b >> 52) & 0x7ff);
        if (E > e && E != 0x7ff) return __longlong_as_double(b - ((long long)e << 52));
        if ((b & 0x7fffffffffffffffLL) == 0) return v;
    }
    return mean_slow(v, cnt);
}

// |a - b| as bits (a nonnegative double orders as its bit pattern)
__device__ __forceinline__ long long absdiff_bits(double a, double b) {
    return __double_as_longlong(__dsub_rn(a, b)) & 0x7fffffffffffffffLL;
}
// a finite double below 2^1022 in magnitude (2x is exact and finite)
__device__ __forceinline__ bool tame(double v) {
    return ((__double_as_longlong(v) >> 52) & 0x7ff) < 0x7fd;
}

// the 3x3 correlations term by term (non-finite or huge neighbourhoods); a
// call, so that the common path issues none of its FP64 instructions
static __device__ __noinline__ double2 tam_dir_slow(const double *__restrict__ nrm, int x, int y, int W, int H) {
    const double fH[3][3] = {{-1, 2, 1}, {-2, 0, 2}, {-1, -2, -1}};
    const double fV[3][3] = {{1, 0, 0}, {0, 0, 0}, {-1, 0, 0}};
    double dH = 0, dV = 0;
    for (int a = -1; a <= 1; a++) {
        const int xx = x + a;
        if (xx < 0 || xx >= W) continue;
        for (int b = -1; b <= 1; b++) {
            const int yy = y + b;
            if (yy < 0 || yy >= H) continue;
            const double v = nrm[(long long)yy * W + xx];
            dH = __dadd_rn(dH, __dmul_rn(fH[b + 1][a + 1], v));
            dV = __dadd_rn(dV, __dmul_rn(fV[b + 1][a + 1], v));
        }
    }
    return make_double2(dH, dV);
}

// Coarseness (tamura.cpp:140-190): for k = 1..7 the window means of side
// 2^k around every pixel position, then per pixel E_h = |mean(x + 2^(k-1)) -
// mean(x - 2^(k-1))| and E_v the same along y, and the first strict maximum
// over k, horizontal before vertical.  Every mean serves four pixels (as the
// right and left, lower and upper window of its neighbours), so it is formed
// once per position (k_tam_mean, the same operations as efficientLocalMean)
// and the pixels compare them (k_tam_best), the running maximum kept per
// pixel between the scales.
__global__ void __launch_bounds__(256) k_tam_mean(const Plane *__restrict__ planes, const FJob *__restrict__ jobs,
                                                  const TamJob *__restrict__ tj, double *__restrict__ ws, int k) {
    const Plane P = planes[jobs[blockIdx.y].plane];
    const TamJob T = tj[blockIdx.y];
    const int W = P.w, H = P.h;
    const long long n = (long long)W * H, len = 1LL << k;
    const double *S = ws + T.sum_ws;
    double *mk = ws + T.mk_ws;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long y = i / W, x = i - y * W;
        mk[i] = local_mean(S, W, H, x, y, len);
    }
}

// E values are |differences| (+0 or more, or NaN): compared as bit patterns,
// NaN never greater, exactly as the double comparison
__global__ void __launch_bounds__(256) k_tam_best(const Plane *__restrict__ planes, const FJob *__restrict__ jobs,
                                                  const TamJob *__restrict__ tj, double *__restrict__ ws, int k) {
    const Plane P = planes[jobs[blockIdx.y].plane];
    const TamJob T = tj[blockIdx.y];
    const int W = P.w, H = P.h;
    const long long n = (long long)W * H;
    const int k2 = 1 << (k - 1);
    const double *mk = ws + T.mk_ws;
    long long *emax = (long long *)(ws + T.emax_ws);
    unsigned char *sb = (unsigned char *)(ws + T.sbest_ws);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int y = (int)(i / W), x = (int)(i - (long long)y * W);
        long long maxE = k == 1 ? 0 : emax[i];
        int maxk = k == 1 ? 0 : sb[i];
        long long eh = 0, ev = 0;
        if (x + k2 < W && x - k2 >= 0) eh = absdiff_bits(mk[i + k2], mk[i - k2]);
        if (y + k2 < H && y - k2 >= 0) ev = absdiff_bits(mk[i + (long long)k2 * W], mk[i - (long long)k2 * W]);
        if (eh > maxE && eh <= 0x7ff0000000000000LL) { maxE = eh; maxk = k; }
        if (ev > maxE && ev <= 0x7ff0000000000000LL) { maxE = ev; maxk = k; }
        emax[i] = maxE;
        sb[i] = (unsigned char)maxk;
    }
}

#define TAM_TILE 1024
// per pixel: the best coarseness scale's statistics, direction angle; per-CTA partials
__global__ void __launch_bounds__(256) k_tam_pixel(const Plane *__restrict__ planes, const FJob *__restrict__ jobs,
                                                   const TamJob *__restrict__ tj, double *__restrict__ ws,
                                                   double *__restrict__ part, int nchunk) {
    __shared__ double sh[32];
    __shared__ long long shl[32];
    const FJob J = jobs[blockIdx.y];
    const Plane P = planes[J.plane];
    const TamJob T = tj[blockIdx.y];
    const int W = P.w, H = P.h;
    const long long n = (long long)W * H;
    const double *nrm = ws + T.norm_ws;
    const unsigned char *sb = (const unsigned char *)(ws + T.sbest_ws);
    double *phi = ws + T.phi_ws;
    long long ksum = 0;
    int kmin = 1 << 30, kmax = -1;
    // pmn from DBL_MAX; pmx from -DBL_MAX, whose pattern is negative as a signed integer
    long long pmnb = __double_as_longlong(DBL_MAX), pmxb = __double_as_longlong(-DBL_MAX);
    double sr = 0;
    const long long i0 = (long long)blockIdx.x * TAM_TILE, i1 = min(n, i0 + TAM_TILE);
    for (long long i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const int y = (int)(i / W), x = (int)(i - (long long)y * W);
        // coarseness: the best scale k_tam_best left for this pixel
        const int maxk = sb[i];
        ksum += maxk;
        kmin = min(kmin, maxk);
        kmax = max(kmax, maxk);
        // directionality: H = [[-1,2,1],[-2,0,2],[-1,-2,-1]], V = [[1,0,0],[0,0,0],[-1,0,0]],
        // accumulated x offset outer, y offset inner, zero outside the image
        // When the neighbourhood is finite and below 2^1022, the zero-coefficient
        // terms add +-0 to sums that are never -0 (they start at +0), the +-1
        // products are exact and x + 2v is one rounding, so the same sums take
        // fused multiply-adds over the nonzero taps, in the same order.
        const double fH[3][3] = {{-1, 2, 1}, {-2, 0, 2}, {-1, -2, -1}};
        double nb[3][3];
        bool fast = true;
        for (int a = -1; a <= 1; a++)
            for (int b = -1; b <= 1; b++) {
                const int xx = x + a, yy = y + b;
                const bool in = xx >= 0 && xx < W && yy >= 0 && yy < H;
                nb[b + 1][a + 1] = in ? nrm[(long long)yy * W + xx] : 0.0;
                fast = fast && tame(nb[b + 1][a + 1]);
            }
        double dH = 0, dV = 0;
        if (fast) {
            // out-of-image taps hold +0 and add nothing (x + 0 = x for x != -0)
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++)
                    if (fH[b][a] != 0) dH = __fma_rn(fH[b][a], nb[b][a], dH);
            dV = __dsub_rn(nb[0][0], nb[2][0]);
        } else {
            const double2 d = tam_dir_slow(nrm, x, y, W, H);
            dH = d.x;
            dV = d.y;
        }
        // dH >= 1e-4 and the running min / max of phi (phi is +0 or positive, or
        // NaN, which fmin / fmax skip) as comparisons of bit patterns
        const long long dHb = __double_as_longlong(dH);
        double ph = 0.0;
        if (dHb >= 0x3f1a36e2eb1c432dLL && dHb <= 0x7ff0000000000000LL) {
            ph = atan(dV / dH) + (M_PI / 2.0 + 0.001);
            sr += __dadd_rn(__dadd_rn(__dmul_rn(dH, dH), __dmul_rn(dV, dV)), __dmul_rn(ph, ph));
        }
        phi[i] = ph;
        const long long phb = __double_as_longlong(ph);
        if ((phb & 0x7fffffffffffffffLL) <= 0x7ff0000000000000LL) {
            pmnb = min(pmnb, phb);
            pmxb = max(pmxb, phb);
        }
    }
    double pmn = __longlong_as_double(pmnb), pmx = __longlong_as_double(pmxb);
    ksum = block_sum_ll(ksum, shl);
    const double dkmin = block_min((double)kmin, sh), dkmax = block_max((double)kmax, sh);
    pmn = block_min(pmn, sh);
    pmx = block_max(pmx, sh);
    sr = block_sum(sr, sh);
    if (threadIdx.x == 0) {
        double *o = part + ((long long)blockIdx.y * nchunk + blockIdx.x) * 6;
        o[0] = (double)ksum;
        o[1] = dkmin;
        o[2] = dkmax;
        o[3] = pmn;
        o[4] = pmx;
        o[5] = sr;
    }
}

// Moments4::add's filter (NaN and |v| > FLT_MAX skipped) on the bit pattern:
// |v| <= FLT_MAX exactly when |v|'s pattern is at most FLT_MAX's (NaN above)
__device__ __forceinline__ bool moments_take(double v) {
    return (__double_as_longlong(v) & 0x7fffffffffffffffLL) <= 0x47efffffe0000000LL;
}

__global__ void __launch_bounds__(1024) k_tam_final(const Plane *__restrict__ planes, const FJob *__restrict__ jobs,
                                                    const TamJob *__restrict__ tj, const double *__restrict__ ws,
                                                    const double *__restrict__ part, int nchunk_max,
                                                    double *__restrict__ feat) {
    __shared__ double sh[32];
    __shared__ unsigned int hs[3], hp[125];
    const FJob J = jobs[blockIdx.x];
    const Plane P = planes[J.plane];
    const TamJob T = tj[blockIdx.x];
    const long long n = (long long)P.w * P.h;
    const int nch = (int)((n + TAM_TILE - 1) / TAM_TILE);
    double ksum = 0, kmin = DBL_MAX, kmax = -DBL_MAX, pmn = DBL_MAX, pmx = -DBL_MAX, sr = 0;
    for (int c = 0; c < nch; c++) {  // every thread reduces the partials in the same order
        const double *o = part + ((long long)blockIdx.x * nchunk_max + c) * 6;
        ksum += o[0];
        kmin = fmin(kmin, o[1]);
        kmax = fmax(kmax, o[2]);
        pmn = fmin(pmn, o[3]);
        pmx = fmax(pmx, o[4]);
        sr += o[5];
    }
    if (threadIdx.x < 3) hs[threadIdx.x] = 0;
    if (threadIdx.x < 125) hp[threadIdx.x] = 0;
    __syncthreads();
    const unsigned char *sb = (const unsigned char *)(ws + T.sbest_ws);
    const double *phi = ws + T.phi_ws, *nrm = ws + T.norm_ws;
    const double ssc = hist_scale(kmin, kmax, 3), psc = hist_scale(pmn, pmx, 125);
    // contrast moments skip NaN and |v| > FLT_MAX, as Moments4::add does
    double s1 = 0;
    long long cnt = 0;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        atomicAdd(&hs[hist_bin((double)sb[i], kmin, ssc, 3)], 1u);
        atomicAdd(&hp[hist_bin(phi[i], pmn, psc, 125)], 1u);
        const double v = nrm[i];
        if (!moments_take(v)) continue;
        s1 += v;
        cnt++;
    }
    s1 = block_sum(s1, sh);
    __shared__ long long shl[32];
    cnt = block_sum_ll(cnt, shl);
    const double mean = cnt ? s1 / (double)cnt : 0.0;
    double m2 = 0, m4 = 0;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        const double v = nrm[i];
        if (!moments_take(v)) continue;
        const double d = v - mean, d2 = d * d;
        m2 += d2;
        m4 += d2 * d2;
    }
    m2 = block_sum(m2, sh);
    m4 = block_sum(m4, sh);
    if (threadIdx.x == 0) {
        // coarseness mean: unsigned 32-bit denominator as in tamura.cpp:246-248
        const unsigned yD = P.h, xD = P.w;
        double coarse = ksum;
        if (yD == 32 || xD == 32) coarse /= (double)((unsigned)((xD + 1 - 32) * (yD + 1 - 32)));
        else coarse /= (double)((unsigned)((yD - 32) * (xD - 32)));
        double hm = 0;
        for (int k = 0; k < 3; k++) hm = fmax(hm, (double)hs[k]);
        double mx = 0;
        long fmx = 0;
        for (int a = 0; a < 125; a++)
            if ((double)hp[a] > mx) { mx = hp[a]; fmx = a; }
        double sum = 0;
        for (int a = 0; a < 125; a++) sum += (double)hp[a] * pow((double)(a + 1 - fmx), 2);
        const double dir = fabs(log(sum / sr + 0.0000001));
        const double nn = (double)cnt;
        const double sd = cnt > 2 ? sqrt(m2 / (nn - 1)) : 0.0;
        const double kurt = cnt > 4 ? (nn * m4) / (m2 * m2) : 0.0;
        const double con = (sd < DBL_EPSILON) ? 0 : sd / pow(kurt / pow(sd, 4), 0.25);
        double *o = feat + J.out;
        o[0] = hs[0] / hm;
        o[1] = hs[1] / hm;
        o[2] = hs[2] / hm;
        o[3] = con;
        o[4] = dir;
        o[5] = coarse;
    }
}

void launch_tamura(Ctx &c, const Plane *planes, const PlaneStats *stats, const double *arena, const FJob *jobs, int njobs,
                   const TamJob *tj, double *ws, double *part, long long maxpix, double *feat) {
    if (njobs <= 0) return;
    const int nchunk = (int)((maxpix + TAM_TILE - 1) / TAM_TILE);
    WC_LAUNCH(c);
    k_tam_prefix<<<njobs, 1024, 0, c.st>>>(arena, planes, stats, jobs, tj, ws);
    const int gx = (int)std::min<long long>((maxpix + 255) / 256, 256);
    for (int k = 1; k <= 7; k++) {
        *c.launches += 2;
        k_tam_mean<<<dim3(gx, njobs), 256, 0, c.st>>>(planes, jobs, tj, ws, k);
        k_tam_best<<<dim3(gx, njobs), 256, 0, c.st>>>(planes, jobs, tj, ws, k);
    }
    WC_LAUNCH(c);
    k_tam_pixel<<<dim3(nchunk, njobs), 256, 0, c.st>>>(planes, jobs, tj, ws, part, nchunk);
    WC_LAUNCH(c);
    k_tam_final<<<njobs, 1024, 0, c.st>>>(planes, jobs, tj, ws, part, nchunk, feat);
}

}  // namespace wc
