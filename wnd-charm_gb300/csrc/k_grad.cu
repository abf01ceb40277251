// Gradients of WND-5 marginal probabilities (no counterpart in the reference):
// the backward pass of classify2 (src/wndchrm_src/TrainingSet.cpp:2429-2586)
// to the test feature vectors and the Fisher weights, and of the smooth
// feature families to the pixels of each test image, through the transform
// chains that feed them.  Everything here is FP64.
//
// Families with a backward (their values move smoothly with the pixels,
// almost everywhere):
//   Zernike Coefficients  |A_nm| of mb_zernike2D (src/textures/zernike/zernike.cpp:207-341),
//                         including the intensity centroid's and the sum's
//                         dependence on every pixel;
//   Pixel Intensity Statistics  mean, median, std, min, max
//                         (src/FeatureAlgorithms.cpp:272-294; ties share the
//                         derivative of the order statistic equally);
//   Fractal Features      mean |I(p) - I(p+k)| (src/FeatureAlgorithms.cpp:232-267);
//   Gini Coefficient      of the sorted positive pixels (src/FeatureAlgorithms.cpp:448-492).
// Families declared piecewise-constant (histograms, counts, thresholds, GLCM
// statistics of a quantised image): zero gradient.  Tamura and Edge
// features have no backward here; a weight on one of them is refused.
//
// Transform adjoints (the derivative of each transform at the image the
// forward pass saw): Fourier |DFT2| (cmatrix.cpp:1107-1200; the mirrored half
// is the same function of the pixels) -> Re DFT2(g conj(X) / |X|); the
// Chebyshev transform (chebyshev.cpp:118-165), a product A^T x^T B, -> B g^T A^T;
// the Symlet-5 wavelet (Wavelet.cpp:136-434), linear, -> the transposed
// decimating convolutions; the Edge transform (cmatrix.cpp:1294-1311), the
// larger absolute neighbour difference, -> +-g to the difference that wins
// (the reference's own max order on ties).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "engine.h"
#include "kcommon.cuh"
#include "ksort.cuh"
#include "kwavelet.cuh"
#include "plan.h"

namespace wc {
namespace gr {

// ---------------------------------------------------------------- WND-5
// One block per test image: the normalised test features, the distances to
// every training row, the class similarities and marginal probabilities, and,
// with a seed s (d loss / d probability), d loss / d distance and from it the
// gradients to the test's raw features and to the weights.
__global__ void __launch_bounds__(256) k_g_wnd(const double *__restrict__ feat, int F, const int *__restrict__ keep, int K,
                                               const double *__restrict__ mins, const double *__restrict__ maxs,
                                               const double *__restrict__ Xn, int N, const int *__restrict__ y, int C,
                                               const double *__restrict__ w, const double *__restrict__ seed,
                                               double *__restrict__ dscr, double *__restrict__ tscr,
                                               double *__restrict__ probs, double *__restrict__ gfeat,
                                               double *__restrict__ gw) {
    __shared__ double sh[32];
    __shared__ long long shl[32];
    __shared__ double Sc[17], T_s, sdot_s;
    __shared__ long long nc[17];
    const int i = blockIdx.x;
    double *t = tscr + (long long)i * 2 * K, *dn = t + K;
    double *d = dscr + (long long)i * N;
    // signatures::normalize of the test row: clipped to [0, 100]; the slope 100
    // / (max - min) inside the range, 0 where the value is clipped or NaN
    for (int f = threadIdx.x; f < K; f += blockDim.x) {
        const int col = keep[f];
        const double mn = mins[col], mx = maxs[col];
        double v = feat[(long long)i * F + col], s = 0.0;
        if (isnan(v) || v < mn || (mx - mn) < DBL_EPSILON) v = 0;
        else if (v > mx) v = 100;
        else {
            v = 100 * ((v - mn) / (mx - mn));
            s = 100.0 / (mx - mn);
        }
        t[f] = v;
        dn[f] = s;
    }
    __syncthreads();
    // distances as classify2 forms them (terms with |t - x| < DBL_EPSILON skipped)
    for (int s = threadIdx.x; s < N; s += blockDim.x) {
        double acc = 0.0;
        for (int f = 0; f < K; f++) {
            const double df = fabs(t[f] - Xn[(long long)s * K + f]);
            if (df < DBL_EPSILON) continue;
            acc += (w[f] * w[f]) * (df * df);
        }
        d[s] = acc;
    }
    __syncthreads();
    // per class: sum of d^-5 over the rows with d >= DBL_EPSILON, and their count
    for (int c = 1; c <= C; c++) {
        double a = 0;
        long long k = 0;
        for (int s = threadIdx.x; s < N; s += blockDim.x)
            if (y[s] == c && !(d[s] < DBL_EPSILON)) {
                a += pow(d[s], -5.0);
                k++;
            }
        a = block_sum(a, sh);
        k = block_sum_ll(k, shl);
        if (threadIdx.x == 0) {
            Sc[c] = k ? a / (double)k : 0.0;
            nc[c] = k;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double T = 0, sd = 0;
        for (int c = 1; c <= C; c++) T += Sc[c];
        for (int c = 1; c <= C; c++) {
            probs[(long long)i * C + c - 1] = Sc[c] / T;
            if (seed) sd += seed[(long long)i * C + c - 1] * Sc[c];
        }
        T_s = T;
        sdot_s = sd;
    }
    __syncthreads();
    if (!seed) return;
    // d loss / d d_s = sum_c seed_c d p_c / d S'_k * d S'_k / d d_s, k the row's class:
    // (seed_k T - sum_c seed_c S'_c) / T^2 * (-5 d^-6 / n_k)
    const double T = T_s, sdot = sdot_s;
    for (int s = threadIdx.x; s < N; s += blockDim.x) {
        const int k = y[s];
        double a = 0.0;
        if (k >= 1 && k <= C && !(d[s] < DBL_EPSILON) && nc[k] > 0)
            a = (seed[(long long)i * C + k - 1] * T - sdot) / (T * T) * (-5.0 * pow(d[s], -6.0) / (double)nc[k]);
        d[s] = a;  // the distances are no longer needed
    }
    __syncthreads();
    // d d_s / d t_f = 2 w_f^2 (t_f - x_sf), d d_s / d w_f = 2 w_f (t_f - x_sf)^2
    for (int f = threadIdx.x; f < K; f += blockDim.x) {
        double gt = 0.0, gwf = 0.0;
        for (int s = 0; s < N; s++) {
            const double a = d[s];
            if (a == 0.0) continue;
            const double diff = t[f] - Xn[(long long)s * K + f];
            if (fabs(diff) < DBL_EPSILON) continue;
            gt += a * 2.0 * (w[f] * w[f]) * diff;
            gwf += a * 2.0 * w[f] * (diff * diff);
        }
        gfeat[(long long)i * F + keep[f]] = gt * dn[f];
        gw[(long long)i * K + f] = gwf;
    }
}

// training rows: the kept features normalised as TrainingSet::normalize does, row-major N x K
__global__ void k_g_train(const double *__restrict__ X, int N, int F, const int *__restrict__ keep, int K,
                          const double *__restrict__ mins, const double *__restrict__ maxs, double *__restrict__ Xn) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= (long long)N * K) return;
    const int s = (int)(q / K), f = (int)(q - (long long)s * K);
    const int col = keep[f];
    const double mn = mins[col], mx = maxs[col];
    double v = X[(long long)s * F + col];
    if (isnan(v) || v < mn || (mx - mn) < DBL_EPSILON) v = 0;
    else if (v > mx) v = 100;
    else v = 100 * ((v - mn) / (mx - mn));
    Xn[q] = v;
}

// ---------------------------------------------------------------- feature VJPs
// A job: one group on one image's node plane: the plane (arena offset, size)
// and the group's slice of d loss / d features.
struct GJob {
    long long poff;  // plane element offset (arena and gradient arena alike)
    int w, h;
    long long goff;  // first element of the group's gradient slice
};

// Fractal: value_b = sum over vertical and horizontal pairs at lag k of
// |I(p) - I(q)| / (W (W - k) + H (H - k)); each pixel gathers the signs of its
// differences with its 4 partners at every lag (sign 0 at a tie).
__global__ void k_g_fractal(const double *__restrict__ arena, double *__restrict__ garena,
                            const GJob *__restrict__ jobs, const double *__restrict__ gf) {
    const GJob J = jobs[blockIdx.y];
    const int W = J.w, H = J.h;
    const double *p = arena + J.poff;
    const double *g = gf + J.goff;
    const int K = (W > H ? H : W) / 5;
    int step = K / 20;
    if (step < 1) step = 1;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < (long long)W * H;
         q += (long long)gridDim.x * blockDim.x) {
        const int y = (int)(q / W), x = (int)(q - (long long)y * W);
        const double v = p[q];
        double acc = 0;
        int bin = 0;
        for (int k = 1; k < K && bin < 20; k += step, bin++) {
            const double gb = g[bin] / (double)(W * (W - k) + H * (H - k));
            if (gb == 0.0) continue;
            double s = 0;
            if (y + k < H) { const double d = v - p[q + (long long)k * W]; s += (d > 0) - (d < 0); }
            if (y - k >= 0) { const double d = v - p[q - (long long)k * W]; s += (d > 0) - (d < 0); }
            if (x + k < W) { const double d = v - p[q + k]; s += (d > 0) - (d < 0); }
            if (x - k >= 0) { const double d = v - p[q - k]; s += (d > 0) - (d < 0); }
            acc += gb * s;
        }
        garena[J.poff + q] += acc;
    }
}

__device__ __forceinline__ unsigned long long okey(double v) {
    const unsigned long long b = __double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double okey_val(unsigned long long k) {
    return __longlong_as_double((k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k);
}
// first index in the sorted keys [0, n) not below / above key
__device__ __forceinline__ long long lower_b(const unsigned long long *a, long long n, unsigned long long k) {
    long long lo = 0, hi = n;
    while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (a[mid] < k) lo = mid + 1; else hi = mid;
    }
    return lo;
}
__device__ __forceinline__ long long upper_b(const unsigned long long *a, long long n, unsigned long long k) {
    long long lo = 0, hi = n;
    while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (a[mid] <= k) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// Pixel statistics (gpix: 5 gradients or none) and Gini (ggini: 1 or none)
// of one plane, one CTA: the plane's keys sorted once give the order
// statistics (median, min, max) and every pixel's rank among the positive
// pixels (tied pixels take their ranks' mean coefficient).
struct SJob {
    long long poff, gpix, ggini;  // gradient slices (element offsets) or -1
    int w, h;
    long long scr;                // scratch offset (2 n keys)
};
__global__ void __launch_bounds__(1024) k_g_sorted(const double *__restrict__ arena, double *__restrict__ garena,
                                                   const SJob *__restrict__ jobs, const double *__restrict__ gf,
                                                   unsigned long long *__restrict__ scr) {
    __shared__ double sh[32];
    const SJob J = jobs[blockIdx.x];
    const long long n = (long long)J.w * J.h;
    const double *p = arena + J.poff;
    double *gp = garena + J.poff;
    unsigned long long *A = scr + J.scr, *B = A + n;
    for (long long q = threadIdx.x; q < n; q += blockDim.x) A[q] = okey(p[q]);
    __syncthreads();
    cta_sort_u64(A, B, n);
    __syncthreads();
    // mean and the centred second moment (two passes, the moments' values)
    double s = 0;
    for (long long q = threadIdx.x; q < n; q += blockDim.x) s += p[q];
    s = block_sum(s, sh);
    const double mean = s / (double)n;
    double m2 = 0;
    for (long long q = threadIdx.x; q < n; q += blockDim.x) m2 += (p[q] - mean) * (p[q] - mean);
    m2 = block_sum(m2, sh);
    const double sd = n > 2 ? sqrt(m2 / (double)(n - 1)) : 0.0;
    // positive pixels: a suffix of the sorted keys
    const long long pos0 = upper_b(A, n, okey(0.0)), cnt = n - pos0;
    double psum = 0;
    for (long long q = pos0 + threadIdx.x; q < n; q += blockDim.x) psum += okey_val(A[q]);
    psum = block_sum(psum, sh);
    double gsum = 0;  // sum over the sorted positives of (2i - c - 1) v_(i), i 1-based
    for (long long q = pos0 + threadIdx.x; q < n; q += blockDim.x)
        gsum += (2.0 * (double)(q - pos0 + 1) - (double)cnt - 1.0) * okey_val(A[q]);
    gsum = block_sum(gsum, sh);
    const double gpix[5] = {J.gpix >= 0 ? gf[J.gpix + 0] : 0.0, J.gpix >= 0 ? gf[J.gpix + 1] : 0.0,
                            J.gpix >= 0 ? gf[J.gpix + 2] : 0.0, J.gpix >= 0 ? gf[J.gpix + 3] : 0.0,
                            J.gpix >= 0 ? gf[J.gpix + 4] : 0.0};
    const double ggini = J.ggini >= 0 ? gf[J.ggini] : 0.0;
    // Gini = g / (sum (c - 1)); d/d v_(i) = (2i - c - 1) / (sum (c - 1)) - Gini / sum
    const bool gini_on = cnt > 1 && psum > 0.0;
    const double gini = gini_on ? gsum / (psum * (double)(cnt - 1)) : 0.0;
    // median: sorted elements half - 1 and half (n even) or half, each a share
    const long long half = n / 2;
    const unsigned long long ka = (n % 2 == 0) ? A[half - 1] : A[half], kb = A[half];
    const long long na = upper_b(A, n, ka) - lower_b(A, n, ka), nb = upper_b(A, n, kb) - lower_b(A, n, kb);
    const long long nmin = upper_b(A, n, A[0]), nmax = n - lower_b(A, n, A[n - 1]);
    for (long long q = threadIdx.x; q < n; q += blockDim.x) {
        const double v = p[q];
        const unsigned long long k = okey(v);
        double g = gpix[0] / (double)n;
        if (sd > 0) g += gpix[2] * (v - mean) / ((double)(n - 1) * sd);
        if (k == A[0]) g += gpix[3] / (double)nmin;
        if (k == A[n - 1]) g += gpix[4] / (double)nmax;
        if (n % 2 == 0) {
            if (k == ka) g += 0.5 * gpix[1] / (double)na;
            if (k == kb) g += 0.5 * gpix[1] / (double)nb;
        } else if (k == kb) {
            g += gpix[1] / (double)nb;
        }
        if (gini_on && v > 0) {
            // mean rank (1-based) of the tied run holding v
            const double r = 0.5 * (double)(lower_b(A, n, k) + upper_b(A, n, k) - 1) - (double)pos0 + 1.0;
            g += ggini * ((2.0 * r - (double)cnt - 1.0) / (psum * (double)(cnt - 1)) - gini / psum);
        }
        gp[q] += g;
    }
}

// Zernike, order 15 (72 values), the reference's q-recursion and angular factor
// e^{-i(m+1) theta}.  A_nm = (n+1)/pi * sum_p f_p V_nm(x_p, y_p) over the disc,
// f = I / S, x = (i + 1 - cx) / rad, y = (j + 1 - cy) / rad.  With h_nm =
// g_nm (n+1)/pi conj(A)/|A|: dL/dI_q = (U(q) [q in disc] - c0 - x_q cgx -
// y_q cgy) / S, U(q) = Re sum h V(q), c0 = Re sum h A^, (cgx, cgy) = Re sum h
// (dV/dx, dV/dy) averaged with f (the centroid's dependence on I_q).
struct ZCoef {
    double H1[16][16], H2[16][16], H3[16][16];
};
__constant__ ZCoef c_z;

// per job: S, cx, cy (1-based coordinates weighted by intensity)
__global__ void __launch_bounds__(256) k_g_zbase(const double *__restrict__ arena, const GJob *__restrict__ jobs,
                                                 double *__restrict__ zb) {
    __shared__ double sh[32];
    const GJob J = jobs[blockIdx.x];
    const double *p = arena + J.poff;
    double s = 0, sx = 0, sy = 0;
    for (long long q = threadIdx.x; q < (long long)J.w * J.h; q += blockDim.x) {
        const int j = (int)(q / J.w), i = (int)(q - (long long)j * J.w);
        s += p[q];
        sx += (i + 1) * p[q];
        sy += (j + 1) * p[q];
    }
    s = block_sum(s, sh);
    sx = block_sum(sx, sh);
    sy = block_sum(sy, sh);
    if (threadIdx.x == 0) {
        zb[blockIdx.x * 16 + 0] = s;
        zb[blockIdx.x * 16 + 1] = sx / s;
        zb[blockIdx.x * 16 + 2] = sy / s;
    }
}

// index of (n, m) in the output order (n ascending, m ascending, n - m even)
__device__ __forceinline__ int zidx(int n, int m) {
    int k = 0;
    for (int a = 0; a < n; a++) k += a / 2 + 1;
    return k + m / 2;
}

// Per-pixel values for one order n, m = n, n-2, ...: R_nm, dR_nm/dr.
__device__ __forceinline__ void zradial(int n, double r, double r2, const double *R, const double *dR, double *Rm,
                                        double *dRm) {
    double Rnmp2 = 0, Rnmp4 = 0, d2 = 0, d4 = 0;
    int k = 0;
    for (int m = n; m >= 0; m -= 2, k++) {
        double Rv, dv;
        if (m == n) {
            Rv = R[n];
            dv = dR[n];
            Rnmp4 = Rv;
            d4 = dv;
        } else if (m == n - 2) {
            Rv = n * R[n] - (n - 1) * R[n - 2];
            dv = n * dR[n] - (n - 1) * dR[n - 2];
            Rnmp2 = Rv;
            d2 = dv;
        } else {
            const double c = c_z.H2[n][m] + c_z.H3[n][m] / r2;
            Rv = c_z.H1[n][m] * Rnmp4 + c * Rnmp2;
            dv = c_z.H1[n][m] * d4 + c * d2 - 2.0 * c_z.H3[n][m] / (r2 * r) * Rnmp2;
            Rnmp4 = Rnmp2;
            d4 = d2;
            Rnmp2 = Rv;
            d2 = dv;
        }
        Rm[k] = Rv;
        dRm[k] = dv;
    }
}

// Partial sums over a chunk of pixels of f V, f dV/dx, f dV/dy (complex) for
// every (n, m): 16 groups of 16 threads, one order n per group.  part:
// [job][chunk][72][6].
__global__ void __launch_bounds__(256) k_g_zmom(const double *__restrict__ arena, const GJob *__restrict__ jobs,
                                                const double *__restrict__ zb, int nchunk, double *__restrict__ part) {
    const GJob J = jobs[blockIdx.y];
    const double *p = arena + J.poff;
    const double S = zb[blockIdx.y * 16], cx = zb[blockIdx.y * 16 + 1], cy = zb[blockIdx.y * 16 + 2];
    const double rad = (double)(J.w < J.h ? J.w : J.h);
    const int n = threadIdx.x >> 4, t16 = threadIdx.x & 15;
    const long long np = (long long)J.w * J.h;
    const long long c0 = np * blockIdx.x / nchunk, c1 = np * (blockIdx.x + 1) / nchunk;
    double acc[8][6];
    for (int k = 0; k < 8; k++)
        for (int e = 0; e < 6; e++) acc[k][e] = 0;
    for (long long q = c0 + t16; q < c1; q += 16) {
        const int j = (int)(q / J.w), i = (int)(q - (long long)j * J.w);
        const double x = (i + 1 - cx) / rad, y = (j + 1 - cy) / rad;
        const double r2 = x * x + y * y, r = sqrt(r2);
        if (r < DBL_EPSILON || r > 1.0) continue;
        const double f = p[q] / S;
        double R[16], dR[16];
        R[0] = 1;
        dR[0] = 0;
        for (int a = 1; a <= n; a++) {
            R[a] = r * R[a - 1];
            dR[a] = a * R[a - 1];
        }
        const double ct = x / r, st = y / r;
        double Rm[8], dRm[8];
        zradial(n, r, r2, R, dR, Rm, dRm);
        // cos / sin of (m + 1) theta for m = n, n-2, ..., by the recurrence from m = 0
        double cm = ct, sm = st;
        double cs[16], ss[16];
        cs[0] = cm;
        ss[0] = sm;
        for (int m = 1; m <= n; m++) {
            const double c2 = ct * cm - st * sm, s2 = ct * sm + st * cm;
            cm = c2;
            sm = s2;
            cs[m] = cm;
            ss[m] = sm;
        }
        int k = 0;
        for (int m = n; m >= 0; m -= 2, k++) {
            const double C = cs[m], Sn = ss[m], Rv = Rm[k], dv = dRm[k], mp = (double)(m + 1);
            // V = R (C - i S)
            const double vr = Rv * C, vi = -Rv * Sn;
            // dV/dx = cos R' E + (sin / r) i (m+1) R E; dV/dy = sin R' E - (cos / r) i (m+1) R E
            const double er = C, ei = -Sn;  // E = e^{-i (m+1) theta}
            const double ax = ct * dv, bx = st / r * mp * Rv;   // dV/dx = (ax + i bx) E
            const double ay = st * dv, by = -ct / r * mp * Rv;  // dV/dy = (ay + i by) E
            acc[k][0] += f * vr;
            acc[k][1] += f * vi;
            acc[k][2] += f * (ax * er - bx * ei);
            acc[k][3] += f * (ax * ei + bx * er);
            acc[k][4] += f * (ay * er - by * ei);
            acc[k][5] += f * (ay * ei + by * er);
        }
    }
    // reduce over the 16 threads of the group (fixed order) and write
    for (int k = 0; k < 8; k++)
        for (int e = 0; e < 6; e++) {
            double v = acc[k][e];
            for (int o = 8; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, 16);
            acc[k][e] = v;
        }
    if (t16 == 0) {
        int k = 0;
        for (int m = n; m >= 0; m -= 2, k++)
            for (int e = 0; e < 6; e++)
                part[(((long long)blockIdx.y * nchunk + blockIdx.x) * 72 + zidx(n, m)) * 6 + e] = acc[k][e];
    }
}

// per job: A^, Gx, Gy summed over the chunks; h_nm and the constants
__global__ void k_g_zcoef(const GJob *__restrict__ jobs, const double *__restrict__ gf, int nchunk,
                          const double *__restrict__ part, double *__restrict__ zb, double *__restrict__ zh) {
    const int jb = blockIdx.x;
    const GJob J = jobs[jb];
    __shared__ double c0s[72], cxs[72], cys[72];
    for (int n = 0; n <= 15; n++)
        for (int m = n & 1; m <= n; m += 2) {
            const int k = zidx(n, m);
            if (k % blockDim.x != threadIdx.x) continue;
            double v[6] = {0, 0, 0, 0, 0, 0};
            for (int c = 0; c < nchunk; c++)
                for (int e = 0; e < 6; e++) v[e] += part[(((long long)jb * nchunk + c) * 72 + k) * 6 + e];
            const double mag = sqrt(v[0] * v[0] + v[1] * v[1]);
            double hr = 0, hi = 0;
            if (mag > 0) {
                const double g = gf[J.goff + k] * (n + 1) / 3.14159265358979323846264338328;
                hr = g * v[0] / mag;   // g (n+1)/pi conj(A^)/|A^|
                hi = -g * v[1] / mag;
            }
            zh[(long long)jb * 144 + 2 * k] = hr;
            zh[(long long)jb * 144 + 2 * k + 1] = hi;
            // Re(h z) = hr zr - hi zi
            c0s[k] = hr * v[0] - hi * v[1];
            cxs[k] = hr * v[2] - hi * v[3];
            cys[k] = hr * v[4] - hi * v[5];
        }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, b = 0, c = 0;
        for (int k = 0; k < 72; k++) {
            a += c0s[k];
            b += cxs[k];
            c += cys[k];
        }
        zb[jb * 16 + 3] = a;
        zb[jb * 16 + 4] = b;
        zb[jb * 16 + 5] = c;
    }
}

__global__ void k_g_zapply(const double *__restrict__ arena, double *__restrict__ garena,
                           const GJob *__restrict__ jobs, const double *__restrict__ zb,
                           const double *__restrict__ zh) {
    const int jb = blockIdx.y;
    const GJob J = jobs[jb];
    const double S = zb[jb * 16], cx = zb[jb * 16 + 1], cy = zb[jb * 16 + 2];
    const double c0 = zb[jb * 16 + 3], cgx = zb[jb * 16 + 4], cgy = zb[jb * 16 + 5];
    const double rad = (double)(J.w < J.h ? J.w : J.h);
    const double *h = zh + (long long)jb * 144;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < (long long)J.w * J.h;
         q += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(q / J.w), i = (int)(q - (long long)j * J.w);
        const double x = (i + 1 - cx) / rad, y = (j + 1 - cy) / rad;
        const double r2 = x * x + y * y, r = sqrt(r2);
        double U = 0;
        if (!(r < DBL_EPSILON || r > 1.0)) {
            double R[16], dR[16];
            R[0] = 1;
            dR[0] = 0;
            for (int a = 1; a <= 15; a++) {
                R[a] = r * R[a - 1];
                dR[a] = a * R[a - 1];
            }
            const double ct = x / r, st = y / r;
            double cs[16], ss[16];
            cs[0] = ct;
            ss[0] = st;
            for (int m = 1; m <= 15; m++) {
                cs[m] = ct * cs[m - 1] - st * ss[m - 1];
                ss[m] = ct * ss[m - 1] + st * cs[m - 1];
            }
            for (int n = 0; n <= 15; n++) {
                double Rm[8], dRm[8];
                zradial(n, r, r2, R, dR, Rm, dRm);
                int k = 0;
                for (int m = n; m >= 0; m -= 2, k++) {
                    const int idx = zidx(n, m);
                    // Re(h V), V = R (C - i S)
                    U += h[2 * idx] * Rm[k] * cs[m] + h[2 * idx + 1] * Rm[k] * ss[m];
                }
            }
        }
        garena[J.poff + q] += (U - c0 - x * cgx - y * cgy) / S;
    }
}

// ---------------------------------------------------------------- transform adjoints
// A transform job: child plane (the transform's output), parent plane (its input)
struct TJobG {
    long long coff, poff;
    int cw, ch, pw, ph;
    long long scr;  // scratch offset (complex work area)
};

// Edge: for each parent pixel, the outputs that read it (itself as the centre
// and its 4 neighbours' outputs), each with the branch the forward's max picks
__device__ __forceinline__ double edge_contrib(const double *in, int W, int H, int y, int x, int ty, int tx) {
    // derivative of out(y, x) with respect to in(ty, tx)
    double mxx = 0, myy = 0;
    int xsel = 0, ysel = 0;  // 1: left/up neighbour, 2: right/down neighbour
    const double c = in[(long long)y * W + x];
    if (y > 0 && y < H - 1) {
        const double a = fabs(c - in[(long long)(y - 1) * W + x]), b = fabs(c - in[(long long)(y + 1) * W + x]);
        // std::max(a, b): b when a < b, else a
        if (a < b) { myy = b; ysel = 2; } else { myy = a; ysel = 1; }
    }
    if (x > 0 && x < W - 1) {
        const double a = fabs(c - in[(long long)y * W + x - 1]), b = fabs(c - in[(long long)y * W + x + 1]);
        if (a < b) { mxx = b; xsel = 2; } else { mxx = a; xsel = 1; }
    }
    // std::max(mxx, myy): myy when mxx < myy, else mxx
    int ny, nx;
    if (mxx < myy) {
        ny = ysel == 1 ? y - 1 : y + 1;
        nx = x;
    } else {
        if (!xsel) return 0.0;  // out = 0 identically (no neighbour on either axis)
        ny = y;
        nx = xsel == 1 ? x - 1 : x + 1;
    }
    const double d = c - in[(long long)ny * W + nx];
    const double s = (d > 0) - (d < 0);
    if (ty == y && tx == x) return s;
    if (ty == ny && tx == nx) return -s;
    return 0.0;
}
__global__ void k_g_edge(const double *__restrict__ arena, double *__restrict__ garena, const TJobG *__restrict__ jobs) {
    const TJobG J = jobs[blockIdx.y];
    const int W = J.pw, H = J.ph;
    const double *in = arena + J.poff;
    const double *g = garena + J.coff;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < (long long)W * H;
         q += (long long)gridDim.x * blockDim.x) {
        const int y = (int)(q / W), x = (int)(q - (long long)y * W);
        double acc = g[q] * edge_contrib(in, W, H, y, x, y, x);
        if (y > 0) acc += g[q - W] * edge_contrib(in, W, H, y - 1, x, y, x);
        if (y < H - 1) acc += g[q + W] * edge_contrib(in, W, H, y + 1, x, y, x);
        if (x > 0) acc += g[q - 1] * edge_contrib(in, W, H, y, x - 1, y, x);
        if (x < W - 1) acc += g[q + 1] * edge_contrib(in, W, H, y, x + 1, y, x);
        garena[J.poff + q] += acc;
    }
}

// Wavelet, row pass adjoint: from the child's four quadrants to the pass-1
// layout t[(x*oy + o)*2 + {0 approx, 1 detail}] (x < parent width)
__global__ void k_g_wav_rows(const double *__restrict__ garena, const TJobG *__restrict__ jobs,
                             double *__restrict__ scr) {
    const TJobG J = jobs[blockIdx.z];
    const int X = J.pw, Y = J.ph, ox = sym5_out(X), oy = sym5_out(Y), W = 2 * ox;
    const double *g = garena + J.coff;
    double *t = scr + J.scr;
    const int k = blockIdx.x * blockDim.x + threadIdx.x, o = blockIdx.y * blockDim.y + threadIdx.y;
    if (k >= X || o >= oy) return;
    // outputs u with 0 <= 2u + 1 - k < 10 read column k with tap j = 2u + 1 - k
    double ga = 0, gd = 0;
    for (int u = max(0, (k - 1 + 1) / 2); u < ox; u++) {
        const int j = 2 * u + 1 - k;
        if (j < 0) continue;
        if (j >= 10) break;
        const double gd2 = g[(long long)o * W + u], ga2 = g[(long long)(oy + o) * W + u];
        const double gd1 = g[(long long)o * W + ox + u], ga1 = g[(long long)(oy + o) * W + ox + u];
        ga += c_sym5_lo[j] * ga1 + c_sym5_hi[j] * gd1;  // a1 = lo * approx, d1 = hi * approx
        gd += c_sym5_lo[j] * ga2 + c_sym5_hi[j] * gd2;  // a2 = lo * detail, d2 = hi * detail
    }
    t[sym5_tmp_index(k, oy, o)] = ga;
    t[sym5_tmp_index(k, oy, o) + 1] = gd;
}
// column pass adjoint: into the parent's gradient
__global__ void k_g_wav_cols(double *__restrict__ garena, const TJobG *__restrict__ jobs, const double *__restrict__ scr) {
    const TJobG J = jobs[blockIdx.z];
    const int X = J.pw, Y = J.ph, oy = sym5_out(Y);
    const double *t = scr + J.scr;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= X || k >= Y) return;
    double acc = 0;
    for (int o = max(0, (k - 1 + 1) / 2); o < oy; o++) {
        const int j = 2 * o + 1 - k;
        if (j < 0) continue;
        if (j >= 10) break;
        const long long q = sym5_tmp_index(x, oy, o);
        acc += c_sym5_lo[j] * t[q] + c_sym5_hi[j] * t[q + 1];
    }
    garena[J.poff + (long long)k * X + x] += acc;
}

// Batched FP64 product C = op(A) op(B) (+ C when acc), small sizes: element
// strides describe transposes.  One job per blockIdx.z.
struct MJob {
    const double *A, *B;
    double *C;
    int M, N, K;
    long long as_m, as_k, bs_k, bs_n, cs_m, cs_n;
    int acc;
};
__global__ void k_g_gemm(const MJob *__restrict__ jobs) {
    const MJob J = jobs[blockIdx.z];
    const int m = blockIdx.y * 16 + threadIdx.y, nn = blockIdx.x * 16 + threadIdx.x;
    if (m >= J.M || nn >= J.N) return;
    double s = 0;
    for (int k = 0; k < J.K; k++) s += J.A[m * J.as_m + k * J.as_k] * J.B[k * J.bs_k + nn * J.bs_n];
    double *c = J.C + m * J.cs_m + nn * J.cs_n;
    *c = J.acc ? *c + s : s;
}

// the parent plane as complex numbers
__global__ void k_g_real2c(const double *__restrict__ arena, const TJobG *__restrict__ jobs, double2 *__restrict__ X) {
    const TJobG J = jobs[blockIdx.y];
    const long long n = (long long)J.pw * J.ph;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        X[J.scr / 2 + q] = make_double2(arena[J.poff + q], 0.0);
}
// H = g conj(X) / |X| (0 where X = 0), g the child's gradient
__global__ void k_g_fgrad(const double *__restrict__ garena, const TJobG *__restrict__ jobs, double2 *__restrict__ X) {
    const TJobG J = jobs[blockIdx.y];
    const long long n = (long long)J.pw * J.ph;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const double2 x = X[J.scr / 2 + q];
        const double g = garena[J.coff + q];
        const double m = sqrt(x.x * x.x + x.y * x.y);
        X[J.scr / 2 + q] = m > 0 ? make_double2(g * x.x / m, -g * x.y / m) : make_double2(0.0, 0.0);
    }
}
__global__ void k_g_addre(const TJobG *__restrict__ jobs, const double2 *__restrict__ X, double *__restrict__ garena) {
    const TJobG J = jobs[blockIdx.y];
    const long long n = (long long)J.pw * J.ph;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        garena[J.poff + q] += X[J.scr / 2 + q].x;
}

}  // namespace gr

int engine_device(wc_engine *E, cudaStream_t *st, long long **launches);
int engine_precision(const wc_engine *E);

}  // namespace wc

using namespace wc;
using namespace wc::gr;

namespace {

#define CKG(x)                                                                                        \
    do {                                                                                              \
        cudaError_t e_ = (x);                                                                         \
        if (e_ != cudaSuccess) return set_err(WC_ERR_CUDA, "%s: %s", #x, cudaGetErrorString(e_));     \
    } while (0)

struct GBufs {
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
    template <typename T>
    int put(T **p, const std::vector<T> &v, cudaStream_t st) {
        int rc = get(p, v.size() * sizeof(T));
        if (rc) return rc;
        if (!v.empty() && cudaMemcpyAsync(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st) != cudaSuccess)
            return set_err(WC_ERR_CUDA, "copy to the device failed");
        return WC_OK;
    }
    ~GBufs() {
        for (void *q : ptrs) cudaFree(q);
    }
};

bool zcoef_ready = false;
int zcoef_init() {
    if (zcoef_ready) return WC_OK;
    ZCoef z;
    std::memset(&z, 0, sizeof z);
    for (int n = 0; n < 16; n++)
        for (int m = 0; m <= n; m++)
            if (n != m) {
                z.H3[n][m] = -(double)(4.0 * (m + 2.0) * (m + 1.0)) / (double)((n + m + 2.0) * (n - m));
                z.H2[n][m] = ((double)(z.H3[n][m] * (n + m + 4.0) * (n - m - 2.0)) / (double)(4.0 * (m + 3.0))) + (m + 2.0);
                z.H1[n][m] = ((double)((m + 4.0) * (m + 3.0)) / 2.0) - ((m + 4.0) * z.H2[n][m]) +
                             ((double)(z.H3[n][m] * (n + m + 6.0) * (n - m - 4.0)) / 8.0);
            }
    CKG(cudaMemcpyToSymbol(c_z, &z, sizeof z));
    zcoef_ready = true;
    return WC_OK;
}

// the Chebyshev transform's factor matrices: A[a][j] = T'[a][j] / 2 with T' the
// reference's weighted basis (getChCoeff1D), len x N
std::vector<double> cheb_factor(int len, int N) {
    std::vector<double> A((size_t)len * N);
    for (int a = 0; a < len; a++) {
        const double x = 2 * (double)(a + 1) / (double)len - 1;
        const double ac = (std::fabs(x) > 1) ? 0 : std::acos(x);
        for (int j = 0; j < N; j++) {
            double t = j == 0 ? 1.0 : std::cos(ac * j);
            t = (j == 0) ? t / (double)len : t * 2 / (double)len;
            A[(size_t)a * N + j] = t / 2;
        }
    }
    return A;
}

}  // namespace

extern "C" int wc_wnd_grad(wc_engine *E, const wc_plan *plan, const double *train, int N, const int *labels, int C,
                           const double *weights, const double *mins, const double *maxs, const wc_image_desc *images,
                           int n, const double *seed, int n_seeds, double *probs, double *grad_pixels,
                           double *grad_weights) {
    if (!E || !plan || !train || !labels || !weights || !mins || !maxs || !images || n < 1 || N < 1 || C < 1 ||
        C > 16 || (seed && n_seeds < 1))
        return set_err(WC_ERR_ARG, "wc_wnd_grad: bad arguments (C must be 1..16, n_seeds >= 1 with a seed)");
    const Plan &P = *plan;
    const int F = P.n_features;
    // the weighted features' families
    std::vector<int> keep;
    std::vector<double> w;
    for (int f = 0; f < F; f++)
        if (!(weights[f] < DBL_EPSILON)) {
            keep.push_back(f);
            w.push_back(weights[f]);
        }
    const int K = (int)keep.size();
    for (size_t g = 0; g < P.groups.size(); g++) {
        const Group &G = P.groups[g];
        bool weighted = false;
        for (int f = G.offset; f < G.offset + kAlgN[G.alg] && !weighted; f++)
            weighted = !(weights[f] < DBL_EPSILON);
        if (!weighted) continue;
        if (G.alg == A_TAMURA || G.alg == A_EDGEF)
            return set_err(WC_ERR_UNSUPPORTED, "wc_wnd_grad: %s has no backward pass (give its features weight 0)",
                           G.name.c_str());
        for (int t : G.chain)
            if (t != X_FOURIER && t != X_CHEBYSHEV && t != X_WAVELET && t != X_EDGE)
                return set_err(WC_ERR_UNSUPPORTED, "wc_wnd_grad: %s: only Fourier, Chebyshev, Wavelet and Edge chains "
                               "have a backward pass", G.name.c_str());
    }
    for (int i = 0; i < n; i++)
        if (images[i].dtype == WC_RGB8 || images[i].dtype == WC_RGB16)
            return set_err(WC_ERR_UNSUPPORTED, "wc_wnd_grad: grayscale images only");
    cudaStream_t st;
    long long *launches;
    int rc = engine_device(E, &st, &launches);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(E->mu);
    if ((rc = zcoef_init())) return rc;
    GBufs B;
    // ---- forward: features of the test images; the planes stay in the arena
    double *dfeat;
    if ((rc = B.get(&dfeat, (size_t)n * F * 8))) return rc;
    CKG(cudaMemsetAsync(dfeat, 0, (size_t)n * F * 8, st));
    std::vector<Plane> planes;
    if ((rc = run_batch(E, P, images, n, dfeat, &planes))) return rc;
    CKG(cudaStreamSynchronize(st));
    {
        int dev_err = 0;
        if ((rc = features_check(st, &dev_err))) return rc;
        E->tune.collect();
        if (dev_err) return set_err(WC_ERR_DEVICE, "a kernel reported error code %d", dev_err);
    }
    const double *arena = (const double *)E->arena.p;
    // the node layout run_batch used: every prefix of every group's chain, parents first
    std::vector<std::vector<int>> chains(1);
    std::vector<int> parent(1, -1), xf(1, -1), group_node(P.groups.size());
    {
        std::map<std::vector<int>, int> node_of;
        node_of[{}] = 0;
        for (size_t g = 0; g < P.groups.size(); g++) {
            std::vector<int> pre;
            int cur = 0;
            for (int t : P.groups[g].chain) {
                pre.push_back(t);
                auto it = node_of.find(pre);
                if (it == node_of.end()) {
                    chains.push_back(pre);
                    parent.push_back(cur);
                    xf.push_back(t);
                    it = node_of.emplace(pre, (int)chains.size() - 1).first;
                }
                cur = it->second;
            }
            group_node[g] = cur;
        }
    }
    const int NN = (int)chains.size();
    if ((long long)planes.size() != (long long)n * NN) return set_err(WC_ERR_CUDA, "wc_wnd_grad: plane layout mismatch");
    // ---- WND-5 per test image, and the inputs of the backward passes
    double *dX, *dXn, *dmin, *dmax, *dw, *dseed, *dprobs, *dgfeat, *dgw, *dscr, *tscr;
    int *dy, *dkeep;
    std::vector<int> ylab(labels, labels + N);
    if ((rc = B.get(&dX, (size_t)N * F * 8)) || (rc = B.get(&dXn, (size_t)N * std::max(K, 1) * 8)) ||
        (rc = B.get(&dmin, F * 8)) || (rc = B.get(&dmax, F * 8)) || (rc = B.put(&dw, w, st)) ||
        (rc = B.put(&dy, ylab, st)) || (rc = B.put(&dkeep, keep, st)) || (rc = B.get(&dprobs, (size_t)n * C * 8)) ||
        (rc = B.get(&dgfeat, (size_t)n * F * 8)) || (rc = B.get(&dgw, (size_t)n * std::max(K, 1) * 8)) ||
        (rc = B.get(&dscr, (size_t)n * N * 8)) || (rc = B.get(&tscr, (size_t)n * 2 * std::max(K, 1) * 8)) ||
        (rc = B.get(&dseed, (size_t)n * C * 8)))
        return rc;
    CKG(cudaMemcpyAsync(dX, train, (size_t)N * F * 8, cudaMemcpyHostToDevice, st));
    CKG(cudaMemcpyAsync(dmin, mins, F * 8, cudaMemcpyHostToDevice, st));
    CKG(cudaMemcpyAsync(dmax, maxs, F * 8, cudaMemcpyHostToDevice, st));
    if (K) {
        ++*launches;
        k_g_train<<<(int)(((long long)N * K + 255) / 256), 256, 0, st>>>(dX, N, F, dkeep, K, dmin, dmax, dXn);
    }
    ++*launches;
    k_g_wnd<<<n, 256, 0, st>>>(dfeat, F, dkeep, K, dmin, dmax, dXn, N, dy, C, dw, nullptr, dscr, tscr, dprobs, dgfeat,
                               dgw);
    CKG(cudaGetLastError());
    if (probs) CKG(cudaMemcpyAsync(probs, dprobs, (size_t)n * C * 8, cudaMemcpyDeviceToHost, st));
    CKG(cudaStreamSynchronize(st));
    if (!seed || n_seeds < 1 || (!grad_pixels && !grad_weights)) return WC_OK;
    // ---- features -> node planes: the gradient arena, one plane per (image, node)
    long long arena_elems = 0;
    for (auto &pl : planes) arena_elems = std::max(arena_elems, pl.off + ((long long)pl.w * pl.h + 31) / 32 * 32);
    double *garena;
    if ((rc = B.get(&garena, (size_t)arena_elems * 8))) return rc;
    std::vector<GJob> fr, zj;
    std::vector<SJob> sj;
    std::map<long long, size_t> sorted_of;  // plane -> its sort job
    long long sscr = 0;
    for (size_t g = 0; g < P.groups.size(); g++) {
        const Group &G = P.groups[g];
        if (G.alg != A_FRACTAL && G.alg != A_ZERNIKE && G.alg != A_PIXSTATS && G.alg != A_GINI) continue;
        for (int i = 0; i < n; i++) {
            const Plane &pl = planes[(size_t)i * NN + group_node[g]];
            const long long goff = (long long)i * F + G.offset;
            if (G.alg == A_FRACTAL) fr.push_back({pl.off, pl.w, pl.h, goff});
            else if (G.alg == A_ZERNIKE) zj.push_back({pl.off, pl.w, pl.h, goff});
            else {
                auto it = sorted_of.find(pl.off);
                if (it == sorted_of.end()) {
                    sj.push_back({pl.off, -1, -1, pl.w, pl.h, sscr});
                    sscr += 2LL * pl.w * pl.h;
                    it = sorted_of.emplace(pl.off, sj.size() - 1).first;
                }
                if (G.alg == A_PIXSTATS) sj[it->second].gpix = goff;
                else sj[it->second].ggini = goff;
            }
        }
    }
    GJob *dfr = nullptr, *dzj = nullptr;
    SJob *dsj = nullptr;
    unsigned long long *sortscr = nullptr;
    double *zb = nullptr, *zpart = nullptr, *zh = nullptr;
    const int nchunk = 16;
    if (!fr.empty() && (rc = B.put(&dfr, fr, st))) return rc;
    if (!sj.empty() && ((rc = B.put(&dsj, sj, st)) || (rc = B.get(&sortscr, (size_t)sscr * 8)))) return rc;
    if (!zj.empty()) {
        if ((rc = B.put(&dzj, zj, st)) || (rc = B.get(&zb, zj.size() * 16 * 8)) ||
            (rc = B.get(&zpart, zj.size() * nchunk * 72 * 6 * 8)) || (rc = B.get(&zh, zj.size() * 144 * 8)))
            return rc;
        // the moments and their coordinate derivatives depend on the planes only
        *launches += 2;
        k_g_zbase<<<(unsigned)zj.size(), 256, 0, st>>>(arena, dzj, zb);
        k_g_zmom<<<dim3(nchunk, (unsigned)zj.size()), 256, 0, st>>>(arena, dzj, zb, nchunk, zpart);
    }
    // transform jobs per node (children before parents: node index descending)
    std::vector<std::vector<TJobG>> tjs(NN);
    std::vector<TJobG *> dtj(NN, nullptr);
    std::vector<long long> tscr_elems(NN, 0);
    long long scr_max = 0;
    for (int k = NN - 1; k >= 1; k--) {
        tjs[k].resize(n);
        for (int i = 0; i < n; i++) {
            const Plane &c = planes[(size_t)i * NN + k], &p = planes[(size_t)i * NN + parent[k]];
            tjs[k][i] = {c.off, p.off, c.w, c.h, p.w, p.h, tscr_elems[k]};
            tscr_elems[k] += xf[k] == X_FOURIER ? 2LL * p.w * p.h : (xf[k] == X_WAVELET ? 2LL * p.w * sym5_out(p.h) : 0);
        }
        if ((rc = B.put(&dtj[k], tjs[k], st))) return rc;
        scr_max = std::max(scr_max, tscr_elems[k]);
    }
    double *tscratch = nullptr;
    if (scr_max && (rc = B.get(&tscratch, (size_t)scr_max * 8)))
        return rc;
    // Chebyshev factor matrices, per (length, N), and the products' temporaries
    std::map<std::pair<int, int>, double *> fac;
    auto factor = [&](int len, int Nn, double **out) -> int {
        auto key = std::make_pair(len, Nn);
        auto it = fac.find(key);
        if (it == fac.end()) {
            double *d;
            int r = B.put(&d, cheb_factor(len, Nn), st);
            if (r) return r;
            it = fac.emplace(key, d).first;
        }
        *out = it->second;
        return WC_OK;
    };
    std::vector<MJob *> dm1(NN, nullptr), dm2(NN, nullptr);
    std::vector<dim3> g1(NN), g2(NN);
    for (int k = NN - 1; k >= 1; k--) {
        if (xf[k] != X_CHEBYSHEV) continue;
        // out = A^T x^T B restricted to rows j < oh: g_x = B g^T A^T, g zero-padded to N rows
        long long tmp_elems = 0;
        for (auto &t : tjs[k]) tmp_elems += (long long)t.ph * t.ch;
        double *tmp;
        if ((rc = B.get(&tmp, (size_t)tmp_elems * 8))) return rc;
        std::vector<MJob> m1, m2;
        long long to = 0;
        int mh = 0, mw = 0, mo = 0;
        for (auto &t : tjs[k]) {
            const int W = t.pw, H = t.ph, Nn = t.cw, oh = t.ch;
            double *dA, *dB;
            if ((rc = factor(W, Nn, &dA)) || (rc = factor(H, Nn, &dB))) return rc;
            // M (H x oh) = B (H x N) g^T (N x oh): g^T[jj][j] = g[j * N + jj]
            m1.push_back({dB, garena + t.coff, tmp + to, H, oh, Nn, Nn, 1, 1, Nn, oh, 1, 0});
            // g_x (H x W) += M (H x oh) A^T (oh x W): A^T[j][a] = A[a * N + j]
            m2.push_back({tmp + to, dA, garena + t.poff, H, W, oh, oh, 1, 1, Nn, W, 1, 1});
            to += (long long)H * oh;
            mh = std::max(mh, H);
            mw = std::max(mw, W);
            mo = std::max(mo, oh);
        }
        if ((rc = B.put(&dm1[k], m1, st)) || (rc = B.put(&dm2[k], m2, st))) return rc;
        g1[k] = dim3((mo + 15) / 16, (mh + 15) / 16, n);
        g2[k] = dim3((mw + 15) / 16, (mh + 15) / 16, n);
    }
    // Fourier nodes: the jobs grouped by shape, each group's complex-array
    // offsets and its two FFT plans (row length, column length)
    struct FGroup {
        int w, h, na;
        long long *aoff;
        FFTPlan *plans;
    };
    std::vector<std::vector<FGroup>> fgroups(NN);
    for (int k = NN - 1; k >= 1; k--) {
        if (xf[k] != X_FOURIER) continue;
        std::map<std::pair<int, int>, std::vector<long long>> by;
        for (int i = 0; i < n; i++) by[std::make_pair(tjs[k][i].pw, tjs[k][i].ph)].push_back(tjs[k][i].scr / 2);
        for (auto &kv : by) {
            const int w = kv.first.first, h = kv.first.second;
            if (w > kMaxFFT || h > kMaxFFT) return set_err(WC_ERR_UNSUPPORTED, "wc_wnd_grad: Fourier side > %d", kMaxFFT);
            std::vector<FFTPlan> pl = {fft_plan(E->tabs, w), fft_plan(E->tabs, h)};
            FGroup g{w, h, (int)kv.second.size(), nullptr, nullptr};
            if ((rc = B.put(&g.aoff, kv.second, st)) || (rc = B.put(&g.plans, pl, st))) return rc;
            fgroups[k].push_back(g);
        }
    }
    if ((rc = E->tabs.sync(st))) return rc;  // twiddles of any new length
    std::vector<long long> img_px(n), img_off(n);
    {
        long long o = 0;
        for (int i = 0; i < n; i++) {
            const Plane &r = planes[(size_t)i * NN];
            img_px[i] = (long long)r.w * r.h;
            img_off[i] = o;
            o += img_px[i] * n_seeds;
        }
    }
    if (grad_weights)
        for (long long f = 0; f < (long long)F * n_seeds; f++) grad_weights[f] = 0.0;
    // ---- one backward pass per seed
    std::vector<double> sd((size_t)n * C), gw((size_t)n * std::max(K, 1));
    for (int sdx = 0; sdx < n_seeds; sdx++) {
        for (int i = 0; i < n; i++)
            for (int c = 0; c < C; c++) sd[(size_t)i * C + c] = seed[((size_t)i * n_seeds + sdx) * C + c];
        CKG(cudaMemcpyAsync(dseed, sd.data(), sd.size() * 8, cudaMemcpyHostToDevice, st));
        CKG(cudaMemsetAsync(dgfeat, 0, (size_t)n * F * 8, st));
        ++*launches;
        k_g_wnd<<<n, 256, 0, st>>>(dfeat, F, dkeep, K, dmin, dmax, dXn, N, dy, C, dw, dseed, dscr, tscr, dprobs,
                                   dgfeat, dgw);
        CKG(cudaGetLastError());
        if (grad_weights) {
            CKG(cudaMemcpyAsync(gw.data(), dgw, gw.size() * 8, cudaMemcpyDeviceToHost, st));
            CKG(cudaStreamSynchronize(st));
            for (int i = 0; i < n; i++)
                for (int k = 0; k < K; k++) grad_weights[(size_t)sdx * F + keep[k]] += gw[(size_t)i * K + k];
        }
        if (!grad_pixels) continue;
        CKG(cudaMemsetAsync(garena, 0, (size_t)arena_elems * 8, st));
        if (dfr) {
            ++*launches;
            k_g_fractal<<<dim3(64, (unsigned)fr.size()), 256, 0, st>>>(arena, garena, dfr, dgfeat);
        }
        if (dsj) {
            ++*launches;
            k_g_sorted<<<(unsigned)sj.size(), 1024, 0, st>>>(arena, garena, dsj, dgfeat, sortscr);
        }
        if (dzj) {
            *launches += 2;
            k_g_zcoef<<<(unsigned)zj.size(), 128, 0, st>>>(dzj, dgfeat, nchunk, zpart, zb, zh);
            k_g_zapply<<<dim3(64, (unsigned)zj.size()), 256, 0, st>>>(arena, garena, dzj, zb, zh);
        }
        CKG(cudaGetLastError());
        for (int k = NN - 1; k >= 1; k--) {
            TJobG *dj = dtj[k];
            int maxw = 0, maxh = 0;
            for (auto &t : tjs[k]) {
                maxw = std::max(maxw, t.pw);
                maxh = std::max(maxh, t.ph);
            }
            if (xf[k] == X_EDGE) {
                ++*launches;
                k_g_edge<<<dim3(64, n), 256, 0, st>>>(arena, garena, dj);
            } else if (xf[k] == X_WAVELET) {
                const dim3 b(32, 8);
                *launches += 2;
                k_g_wav_rows<<<dim3((maxw + 31) / 32, (sym5_out(maxh) + 7) / 8, n), b, 0, st>>>(garena, dj, tscratch);
                k_g_wav_cols<<<dim3((maxw + 31) / 32, (maxh + 7) / 8, n), b, 0, st>>>(garena, dj, tscratch);
            } else if (xf[k] == X_CHEBYSHEV) {
                *launches += 2;
                k_g_gemm<<<g1[k], dim3(16, 16), 0, st>>>(dm1[k]);
                k_g_gemm<<<g2[k], dim3(16, 16), 0, st>>>(dm2[k]);
            } else if (xf[k] == X_FOURIER) {
                // X = DFT2(parent) (rows, then columns), H = g conj(X) / |X|,
                // g_parent += Re DFT2(H): the DFTs are the engine's FP64 FFTs
                // over every image of a shape group at once, in place
                double2 *X = (double2 *)tscratch;
                *launches += 3;
                k_g_real2c<<<dim3(32, n), 256, 0, st>>>(arena, dj, X);
                for (const FGroup &g : fgroups[k]) {
                    cfft_lines_fp64(st, launches, (double *)X, g.aoff, g.na, g.h, g.w, g.w, 1, g.plans, E->tabs.d());
                    cfft_lines_fp64(st, launches, (double *)X, g.aoff, g.na, g.w, g.h, 1, g.w, g.plans + 1, E->tabs.d());
                }
                k_g_fgrad<<<dim3(32, n), 256, 0, st>>>(garena, dj, X);
                for (const FGroup &g : fgroups[k]) {
                    cfft_lines_fp64(st, launches, (double *)X, g.aoff, g.na, g.h, g.w, g.w, 1, g.plans, E->tabs.d());
                    cfft_lines_fp64(st, launches, (double *)X, g.aoff, g.na, g.w, g.h, 1, g.w, g.plans + 1, E->tabs.d());
                }
                k_g_addre<<<dim3(32, n), 256, 0, st>>>(dj, X, garena);
            } else {
                return set_err(WC_ERR_UNSUPPORTED, "wc_wnd_grad: no adjoint for transform %d", xf[k]);
            }
            CKG(cudaGetLastError());
        }
        // the root planes: d loss / d pixel
        for (int i = 0; i < n; i++) {
            const Plane &r = planes[(size_t)i * NN];
            CKG(cudaMemcpyAsync(grad_pixels + img_off[i] + (long long)sdx * img_px[i], garena + r.off,
                                (size_t)img_px[i] * 8, cudaMemcpyDeviceToHost, st));
        }
    }
    CKG(cudaStreamSynchronize(st));
    return WC_OK;
}
