// Haralick textures (FP64 form): haralick2D + Extract_Texture_Features,
// src/textures/haralick/haralick.cpp:12-144, src/textures/haralick/CVIPtexture.cpp:384-1108.
//   * gray = (unsigned char)((p - min) * 255 / (max - min));
//   * tone LUT over the tones present (tone 0 included), Ng tones;
//   * per angle (0, 45, 90, 135) a symmetric co-occurrence matrix at distance 1
//     over pairs whose two pixels are both nonzero, divided by the pair count;
//   * f1..f13 from the matrix; f14 = sqrt(Re lambda_2) of Q in the order of
//     the real Schur form (0 if lambda_2 is complex, or Ng < 3);
//   * (mean, range) over the 4 angles, permuted into the reference's order.
// Counts are integers, so the matrices are bit-identical to the CPU's for the
// same gray image.  The eigen-solver is the same algorithm, loop orders and
// rounding (no contraction) as the oracle's restatement of Eigen 3.1.2.
#include <cfloat>
#include <string>
#include <cmath>

#include "kcommon.cuh"
#include "kdf32.cuh"
#include "kernels.h"

namespace wc {

// one CTA per job: gray image, tone LUT, Ng
__global__ void __launch_bounds__(1024) k_har_quant(const double *__restrict__ arena, const Plane *__restrict__ planes,
                                                    const PlaneStats *__restrict__ stats, const FJob *__restrict__ jobs,
                                                    const HarJob *__restrict__ hj, char *__restrict__ wsb) {
    __shared__ int flag[256];
    const FJob J = jobs[blockIdx.x];
    const Plane P = planes[J.plane];
    const PlaneStats S = stats[J.plane];
    const HarJob H = hj[blockIdx.x];
    unsigned char *g = (unsigned char *)(wsb + H.gray_b);
    int *lut = (int *)(wsb + H.lut_b);
    if (threadIdx.x < 256) flag[threadIdx.x] = 0;
    __syncthreads();
    const double sc = 255.0 / (S.mx - S.mn);
    const double *p = arena + P.off;
    for (long long i = threadIdx.x; i < (long long)P.w * P.h; i += blockDim.x) {
        const double q = (p[i] - S.mn) * sc;
        unsigned char v = 0;
        if (q >= 0 && q < 256) v = (unsigned char)q;  // constant plane (0/0): tone 0
        g[i] = v;
        flag[v] = 1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int ng = 0;
        for (int t = 0; t < 256; t++) lut[t] = flag[t] ? ng++ : -1;
        lut[256] = ng;
    }
}

// one CTA per (job, angle): symmetric GLCM in shared memory (upper triangle),
// written out normalised as a full Ng x Ng matrix.
__global__ void __launch_bounds__(1024) k_har_glcm(const Plane *__restrict__ planes, const FJob *__restrict__ jobs,
                                                   const HarJob *__restrict__ hj, char *__restrict__ wsb) {
    extern __shared__ unsigned int tri[];  // 256*257/2
    __shared__ int lut_s[257];
    __shared__ unsigned long long cnt_s;
    const int ang = blockIdx.y;
    const FJob J = jobs[blockIdx.x];
    const Plane P = planes[J.plane];
    const HarJob H = hj[blockIdx.x];
    const unsigned char *g = (const unsigned char *)(wsb + H.gray_b);
    const int *lut = (const int *)(wsb + H.lut_b);
    for (int t = threadIdx.x; t < 257; t += blockDim.x) lut_s[t] = lut[t];
    for (int t = threadIdx.x; t < 256 * 257 / 2; t += blockDim.x) tri[t] = 0;
    if (threadIdx.x == 0) cnt_s = 0;
    __syncthreads();
    const int Ng = lut_s[256];
    const int dr = ang == 0 ? 0 : 1, dc = ang == 0 ? 1 : (ang == 1 ? -1 : (ang == 2 ? 0 : 1));
    const int rows = P.h, cols = P.w;
    unsigned long long cnt = 0;
    for (long long i = threadIdx.x; i < (long long)rows * cols; i += blockDim.x) {
        const int r = (int)(i / cols), c = (int)(i - (long long)r * cols);
        const unsigned char a = g[i];
        if (a == 0) continue;
        const int r2 = r + dr, c2 = c + dc;
        if (r2 >= rows || c2 < 0 || c2 >= cols) continue;
        const unsigned char b = g[(long long)r2 * cols + c2];
        if (!b) continue;
        int x = lut_s[a], y = lut_s[b];
        if (x > y) { int t = x; x = y; y = t; }
        atomicAdd(&tri[x * 256 - x * (x - 1) / 2 + (y - x)], 1u);
        cnt += 2;
    }
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(&cnt_s, cnt);
    __syncthreads();
    const double count = (double)cnt_s;
    double *Pm = (double *)(wsb + H.glcm_b) + (long long)ang * 256 * 256;
    for (long long q = threadIdx.x; q < (long long)Ng * Ng; q += blockDim.x) {
        const int i = (int)(q / Ng), j = (int)(q - (long long)i * Ng);
        const int x = min(i, j), y = max(i, j);
        double c = (double)tri[x * 256 - x * (x - 1) / 2 + (y - x)];
        if (i == j) c *= 2;
        Pm[q] = (cnt_s == 0) ? 0.0 : c / count;
    }
    // nonzero column range of every row (the matrix is symmetric, so also of every column)
    int *lo = (int *)(wsb + H.mar_b + (long long)ang * HAR_MAR_BYTES + 4096), *hi = lo + 256;
    for (int i = threadIdx.x; i < Ng; i += blockDim.x) {
        int a = Ng, b = -1;
        if (cnt_s != 0)
            for (int j = 0; j < Ng; j++) {
                const int x = min(i, j), y = max(i, j);
                if (tri[x * 256 - x * (x - 1) / 2 + (y - x)]) {
                    a = min(a, j);
                    b = j;
                }
            }
        lo[i] = a;
        hi[i] = b;
    }
}

// f1..f13 for one (job, angle); marginals summed sequentially per entry.
__global__ void __launch_bounds__(256) k_har_stats(const FJob *__restrict__ jobs, const HarJob *__restrict__ hj,
                                                   char *__restrict__ wsb) {
    __shared__ double px[256], py[256], pxpy[512], pxmy[256];
    __shared__ double sh[32];
    const int ang = blockIdx.y;
    const HarJob H = hj[blockIdx.x];
    const int Ng = ((const int *)(wsb + H.lut_b))[256];
    const double *P = (const double *)(wsb + H.glcm_b) + (long long)ang * 256 * 256;
    double *res = (double *)(wsb + H.res_b) + ang * 14;
    const double EPS = 0.000000001, l2 = log10(2.0);
    for (int i = threadIdx.x; i < Ng; i += blockDim.x) {
        double s = 0, t = 0;
        for (int j = 0; j < Ng; j++) {
            s += P[(long long)i * Ng + j];
            t += P[(long long)j * Ng + i];
        }
        px[i] = s;
        py[i] = t;
        double *mar = (double *)(wsb + H.mar_b + (long long)ang * HAR_MAR_BYTES);
        mar[i] = s;
        mar[256 + i] = t;
    }
    for (int k = threadIdx.x; k <= 2 * Ng - 2; k += blockDim.x) {
        double s = 0;
        for (int i = max(0, k - Ng + 1); i <= min(k, Ng - 1); i++) s += P[(long long)i * Ng + (k - i)];
        pxpy[k] = s;
    }
    for (int k = threadIdx.x; k < Ng; k += blockDim.x) {
        double s = 0;
        for (int i = 0; i < Ng; i++) {
            if (i + k < Ng) s += P[(long long)i * Ng + i + k];
            if (k > 0 && i - k >= 0) s += P[(long long)i * Ng + i - k];
        }
        pxmy[k] = s;
    }
    __syncthreads();
    double f1 = 0, tmp3 = 0, mean4 = 0, f5 = 0, e9 = 0, hxy1 = 0, hxy2 = 0;
    for (long long q = threadIdx.x; q < (long long)Ng * Ng; q += blockDim.x) {
        const int i = (int)(q / Ng), j = (int)(q - (long long)i * Ng);
        const double p = P[q];
        const double pp = px[i] * py[j];
        const double lpp = log10(pp + EPS);
        hxy2 -= pp * lpp / l2;
        if (p == 0.0) continue;  // every other term is then a zero: the sums stay as they are
        f1 += p * p;
        tmp3 += i * j * p;
        mean4 += i * p;
        f5 += p / (1 + (i - j) * (i - j));
        e9 += p * log10(p + EPS) / l2;
        hxy1 -= p * lpp / l2;
    }
    f1 = block_sum(f1, sh);
    tmp3 = block_sum(tmp3, sh);
    mean4 = block_sum(mean4, sh);
    f5 = block_sum(f5, sh);
    e9 = block_sum(e9, sh);
    hxy1 = block_sum(hxy1, sh);
    hxy2 = block_sum(hxy2, sh);
    double var4 = 0;
    for (long long q = threadIdx.x; q < (long long)Ng * Ng; q += blockDim.x) {
        const int i = (int)(q / Ng);
        var4 += (i - mean4) * (i - mean4) * P[q];
    }
    var4 = block_sum(var4, sh);
    if (threadIdx.x == 0) {
        double f2 = 0;
        for (int n = 0; n < Ng; n++) f2 += n * n * pxmy[n];
        double meanx = 0, sq = 0;
        for (int i = 0; i < Ng; i++) {
            meanx += px[i] * i;
            sq += px[i] * i * i;
        }
        const double sd = sqrt(sq - meanx * meanx);
        const double f3 = (sd * sd == 0) ? 1 : (tmp3 - meanx * meanx) / (sd * sd);
        double f6 = 0, sent = 0;
        for (int k = 0; k <= 2 * Ng - 2; k++) f6 += k * pxpy[k];
        for (int k = 0; k <= 2 * Ng - 2; k++) sent -= pxpy[k] * log10(pxpy[k] + EPS) / l2;
        double f7 = 0;
        for (int k = 0; k <= 2 * Ng - 2; k++) f7 += (k - sent) * (k - sent) * pxpy[k];
        double s10 = 0, s10sq = 0, e11 = 0;
        for (int k = 0; k < Ng; k++) {
            s10 += k * pxmy[k];
            s10sq += k * k * pxmy[k];
            e11 += pxmy[k] * log10(pxmy[k] + EPS) / l2;
        }
        double hx = 0, hy = 0;
        for (int i = 0; i < Ng; i++) {
            hx -= px[i] * log10(px[i] + EPS) / l2;
            hy -= py[i] * log10(py[i] + EPS) / l2;
        }
        const double hxy = -e9, m = hx > hy ? hx : hy;
        res[0] = f1;
        res[1] = f2;
        res[2] = f3;
        res[3] = var4;
        res[4] = f5;
        res[5] = f6;
        res[6] = f7;
        res[7] = sent;
        res[8] = -e9;
        res[9] = s10sq - s10 * s10;
        res[10] = -e11;
        res[11] = (m == 0) ? 1 : (hxy - hxy1) / m;
        res[12] = sqrt(fabs(1 - exp(-2.0 * (hxy2 - hxy))));
    }
}

// ---------------------------------------------------------------- f14
// Q(i,j) = sum_k P(i,k) P(j,k) / (px_i py_k + 1e-13) (_Q_calc_eigen,
// CVIPtexture.cpp:961-987), then eigenvalue #2 of Q in real-Schur order.
__device__ void hh_make(const double *v, int n, double *ess, double &tau, double &beta) {
    double tail = 0;
    for (int i = 1; i < n; i++) tail = __dadd_rn(tail, __dmul_rn(v[i], v[i]));
    const double c0 = v[0];
    if (n == 1 || tail == 0) {
        tau = 0;
        beta = c0;
        for (int i = 1; i < n; i++) ess[i - 1] = 0;
    } else {
        beta = sqrt(__dadd_rn(__dmul_rn(c0, c0), tail));
        if (c0 >= 0) beta = -beta;
        for (int i = 1; i < n; i++) ess[i - 1] = v[i] / __dsub_rn(c0, beta);
        tau = __dsub_rn(beta, c0) / beta;
    }
}

// Q, one warp per row i: Q(i,j) = sum over k ascending of
// RN(RN(P(i,k) P(j,k)) / RN(RN(px_i py_k) + 1e-13)), as _Q_calc_eigen sums it
// (CVIPtexture.cpp:961-987).  Terms with P(i,k) P(j,k) = 0 add +0 to a sum of
// nonnegative terms, so only k in the nonzeros of row i and j in the nonzeros of
// row k (= column k: the matrix is symmetric) are visited; every Q(i,j) still
// receives its nonzero terms in ascending k, with the same roundings.
// RN(rp / d) (P. Markstein, IBM J. Res. Develop. 34(1), 1990): with yh = RN(1/d)
// and yl ~ 1/d - yh, q0 = RN(rp yh + RN(rp yl)) is within one ulp of rp/d, the
// residual rp - d q0 is exact and RN(q0 + r yh) is the correctly rounded
// quotient.  Here d = px py + 1e-13 lies in [1e-13, 1]; far from the normal
// range (rp < 2^-900) the division itself is used.
static __device__ __noinline__ double q_div_far(double a, double b) { return a / b; }
// rp >= +0 (a product of GLCM entries), so rp < 2^-900 compares as bit patterns
// (integer instructions; a NaN takes the division as well)
__device__ __forceinline__ double q_quot(double rp, double d, double yh, double yl) {
    if (__double_as_longlong(rp) < 0x07b0000000000000LL) return q_div_far(rp, d);
    const double q0 = fma(rp, yh, __dmul_rn(rp, yl));
    const double r = fma(-q0, d, rp);
    return fma(r, yh, q0);
}

#define Q_WARPS 8
__global__ void __launch_bounds__(32 * Q_WARPS) k_har_q(const HarJob *__restrict__ hj, char *__restrict__ wsb) {
    __shared__ double qrow[Q_WARPS][256];
    __shared__ double py[256];
    const int ang = blockIdx.y;
    const HarJob H = hj[blockIdx.x];
    const int n = ((const int *)(wsb + H.lut_b))[256];
    if (n < 3) return;
    const double *P = (const double *)(wsb + H.glcm_b) + (long long)ang * 256 * 256;
    double *A = (double *)(wsb + H.q_b) + (long long)ang * 256 * 256;
    const double *mar = (const double *)(wsb + H.mar_b + (long long)ang * HAR_MAR_BYTES);
    const int *lo = (const int *)(wsb + H.mar_b + (long long)ang * HAR_MAR_BYTES + 4096), *hi = lo + 256;
    for (int k = threadIdx.x; k < n; k += blockDim.x) py[k] = mar[256 + k];
    __syncthreads();
    const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
    double *q = qrow[wq];
    for (int i = blockIdx.z * Q_WARPS + wq; i < n; i += gridDim.z * Q_WARPS) {
        for (int j = lane; j < n; j += 32) q[j] = 0.0;
        __syncwarp();
        const double di = mar[i];
        const double *Pi = P + (long long)i * n;
        const int klo = lo[i], khi = hi[i];
        for (int k0 = klo; k0 <= khi; k0 += 32) {
            const int kk = k0 + lane;
            const double al = kk <= khi ? Pi[kk] : 0.0;
            unsigned m = __ballot_sync(0xffffffffu, al != 0.0);
            while (m) {
                const int b = __ffs(m) - 1;
                m &= m - 1;
                const int k = k0 + b;
                const double a = __shfl_sync(0xffffffffu, al, b);
                const double d = __dadd_rn(__dmul_rn(di, py[k]), 0.0000000000001);
                // rp / d for every j of the row by Markstein's method: one
                // division per (i, k) for yh = RN(1/d), then four FP64
                // operations per term give the correctly rounded quotient
                const double yh = 1.0 / d, yl = __dmul_rn(fma(-yh, d, 1.0), yh);
                const double *Pk = P + (long long)k * n;
                for (int j = lo[k] + lane; j <= hi[k]; j += 32) {
                    const double rp = __dmul_rn(a, Pk[j]);
                    if ((__double_as_longlong(rp) << 1) != 0) q[j] = __dadd_rn(q[j], q_quot(rp, d, yh, yl));
                }
                __syncwarp();
            }
        }
        double *Ai = A + (long long)i * n;
        for (int j = lane; j < n; j += 32) Ai[j] = q[j];
        __syncwarp();
    }
}

// The mixed form's Q, in pairs of floats: the GLCM (no longer read by f1..f13)
// is converted in place on the integer pipe, then each term is
// P(i,k) P(j,k) times the pair reciprocal of px_i py_k + 1e-13, summed in the
// same k order.  Q is written in pairs for k_har_hess_df.
__global__ void __launch_bounds__(256) k_har_p_df(const HarJob *__restrict__ hj, char *__restrict__ wsb) {
    const int ang = blockIdx.y;
    const HarJob H = hj[blockIdx.x];
    const int n = ((const int *)(wsb + H.lut_b))[256];
    if (n < 3) return;
    df *P = (df *)((double *)(wsb + H.glcm_b) + (long long)ang * 256 * 256);
    for (long long q = threadIdx.x; q < (long long)n * n; q += blockDim.x) P[q] = df_split(*(const double *)&P[q]);
}

__global__ void __launch_bounds__(32 * Q_WARPS) k_har_q_df(const HarJob *__restrict__ hj, char *__restrict__ wsb) {
    __shared__ df qrow[Q_WARPS][256];
    __shared__ df py[256];
    const int ang = blockIdx.y;
    const HarJob H = hj[blockIdx.x];
    const int n = ((const int *)(wsb + H.lut_b))[256];
    if (n < 3) return;
    const df *P = (const df *)((const double *)(wsb + H.glcm_b) + (long long)ang * 256 * 256);
    df *A = (df *)((double *)(wsb + H.q_b) + (long long)ang * 256 * 256);
    const double *mar = (const double *)(wsb + H.mar_b + (long long)ang * HAR_MAR_BYTES);
    const int *lo = (const int *)(wsb + H.mar_b + (long long)ang * HAR_MAR_BYTES + 4096), *hi = lo + 256;
    for (int k = threadIdx.x; k < n; k += blockDim.x) py[k] = df_split(mar[256 + k]);
    __syncthreads();
    const df one = {1.f, 0.f}, eps13 = df_from_double(0.0000000000001);
    const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
    df *q = qrow[wq];
    for (int i = blockIdx.z * Q_WARPS + wq; i < n; i += gridDim.z * Q_WARPS) {
        for (int j = lane; j < n; j += 32) q[j] = df{0.f, 0.f};
        __syncwarp();
        const df di = df_split(mar[i]);
        const df *Pi = P + (long long)i * n;
        const int klo = lo[i], khi = hi[i];
        for (int k0 = klo; k0 <= khi; k0 += 32) {
            const int kk = k0 + lane;
            const df al = kk <= khi ? Pi[kk] : df{0.f, 0.f};
            unsigned m = __ballot_sync(0xffffffffu, al.hi != 0.f);
            while (m) {
                const int b = __ffs(m) - 1;
                m &= m - 1;
                const int k = k0 + b;
                const df a = df_shfl(al, b);
                const df rd = df_div(one, df_fma(di, py[k], eps13));
                const df *Pk = P + (long long)k * n;
                for (int j = lo[k] + lane; j <= hi[k]; j += 32) {
                    const df rp = df_mul(a, Pk[j]);
                    if (rp.hi != 0.f) q[j] = df_fma(rp, rd, q[j]);
                }
                __syncwarp();
            }
        }
        df *Ai = A + (long long)i * n;
        for (int j = lane; j < n; j += 32) Ai[j] = q[j];
        __syncwarp();
    }
}

// Hessenberg reduction of Q in place (HessenbergDecomposition::_compute,
// HessenbergDecomposition.h:292-318): column i's reflector from the sequential
// tail sum, then H A on the trailing rows and A H on all rows.  One CTA per
// matrix; products that the reference forms per element (tau * ess_r, tau * t)
// are formed once, with the same value.
__global__ void __launch_bounds__(256) k_har_hess(const HarJob *__restrict__ hj, char *__restrict__ wsb) {
    __shared__ double v[256], vsq[256], ess[256], tess[256];
    __shared__ double s_tau, s_beta, s_den;
    __shared__ int s_triv;
    const int ang = blockIdx.y;
    const HarJob H = hj[blockIdx.x];
    const int n = ((const int *)(wsb + H.lut_b))[256];
    if (n < 3) return;
    double *A = (double *)(wsb + H.q_b) + (long long)ang * 256 * 256;
    for (int i = 0; i < n - 1; i++) {
        const int rem = n - i - 1;
        for (int k = threadIdx.x; k < rem; k += blockDim.x) {
            const double x = A[(long long)(i + 1 + k) * n + i];
            v[k] = x;
            vsq[k] = __dmul_rn(x, x);  // the squares side by side; their sum stays sequential
        }
        __syncthreads();
        if (threadIdx.x == 0) {  // makeHouseholder (Householder.h:65-90)
            double tail = 0;
            for (int k = 1; k < rem; k++) tail = __dadd_rn(tail, vsq[k]);
            const double c0 = v[0];
            if (rem == 1 || tail == 0) {
                s_triv = 1;
                s_tau = 0;
                s_beta = c0;
            } else {
                double beta = sqrt(__dadd_rn(__dmul_rn(c0, c0), tail));
                if (c0 >= 0) beta = -beta;
                s_triv = 0;
                s_beta = beta;
                s_den = __dsub_rn(c0, beta);
                s_tau = __dsub_rn(beta, c0) / beta;
            }
        }
        __syncthreads();
        const double tau = s_tau;
        for (int k = 1 + threadIdx.x; k < rem; k += blockDim.x) {
            const double e = s_triv ? 0.0 : v[k] / s_den;
            ess[k - 1] = e;
            tess[k - 1] = __dmul_rn(tau, e);
            A[(long long)(i + 1 + k) * n + i] = e;
        }
        if (threadIdx.x == 0) A[(long long)(i + 1) * n + i] = s_beta;
        __syncthreads();
        // H A: rows i+1.., columns i+1.. (threads over columns)
        for (int c = i + 1 + threadIdx.x; c < n; c += blockDim.x) {
            double *col = A + (long long)(i + 1) * n + c;
            if (rem == 1) {
                col[0] = __dmul_rn(col[0], __dsub_rn(1.0, tau));
                continue;
            }
            double t = 0;
            for (int r = 1; r < rem; r++) t = __dadd_rn(t, __dmul_rn(ess[r - 1], col[(long long)r * n]));
            t = __dadd_rn(t, col[0]);
            col[0] = __dsub_rn(col[0], __dmul_rn(tau, t));
            for (int r = 1; r < rem; r++) col[(long long)r * n] = __dsub_rn(col[(long long)r * n], __dmul_rn(tess[r - 1], t));
        }
        __syncthreads();
        // A H: all rows, columns i+1.. (threads over rows)
        for (int r = threadIdx.x; r < n; r += blockDim.x) {
            double *row = A + (long long)r * n + i + 1;
            if (rem == 1) {
                row[0] = __dmul_rn(row[0], __dsub_rn(1.0, tau));
                continue;
            }
            double t = 0;
            for (int c = 1; c < rem; c++) t = __dadd_rn(t, __dmul_rn(row[c], ess[c - 1]));
            t = __dadd_rn(t, row[0]);
            const double tt = __dmul_rn(tau, t);
            row[0] = __dsub_rn(row[0], tt);
            for (int c = 1; c < rem; c++) row[c] = __dsub_rn(row[c], __dmul_rn(tt, ess[c - 1]));
        }
        __syncthreads();
    }
    for (long long q = threadIdx.x; q < (long long)n * n; q += blockDim.x) {
        const int r = (int)(q / n), c = (int)(q - (long long)r * n);
        if (c < r - 1) A[q] = 0;
    }
}

// Real-Schur QR iteration of one Hessenberg matrix per warp (RealSchur::compute,
// src/Eigen/src/Eigenvalues/RealSchur.h:204-463), then eigenvalue #2.
// Every update is restricted to the active window [il, iu]: the reflectors act
// on rows/columns independently, so the window's entries get exactly the
// operations they get from the full-width updates, and entries outside the
// window are never read again (columns > iu are deflated, the block above il
// is decoupled).  All lanes take the same decisions from the same (broadcast)
// values; lane-parallel loops run over the columns/rows of a reflector.
// x + 0.0 in round-to-nearest: x, except -0 -> +0 (integer ops, off the FP64 pipe)
__device__ __forceinline__ double plus_zero(double x) {
    const long long b = __double_as_longlong(x);
    return b == (long long)0x8000000000000000ULL ? 0.0 : x;
}

// x == 0 (either sign) and x >= 0 (-0 included, NaN excluded) from the bits:
// integer instructions instead of FP64 comparisons
__device__ __forceinline__ bool zero_bits(double x) { return (__double_as_longlong(x) << 1) == 0; }
__device__ __forceinline__ bool nonneg_bits(double x) {
    const long long b = __double_as_longlong(x);
    return b >= 0 ? b <= 0x7ff0000000000000LL : b == (long long)0x8000000000000000ULL;
}

// makeHouseholder of a 3-vector with the scalar work spread over lanes: lanes
// 1, 2 square v1, v2 at once, and lanes 0, 1, 2 form v1/(c0-beta),
// v2/(c0-beta) and (beta-c0)/beta in one division.  Same operations and
// roundings as the sequential form (0 + v1^2 = v1^2 exactly, as v1^2 >= +0).
// beta - c0 is taken as -(c0 - beta): round-to-nearest is symmetric, and
// c0 - beta is never zero here (beta has c0's opposite sign and |beta| > 0).
__device__ __forceinline__ void hh_make3(const double v0, const double v1, const double v2, int lane, double &e0,
                                         double &e1, double &tau, double &beta) {
    const double vl = lane == 2 ? v2 : v1;
    const double sq = __dmul_rn(vl, vl);
    const double s1 = __shfl_sync(0xffffffffu, sq, 1), s2 = __shfl_sync(0xffffffffu, sq, 2);
    const double tail = __dadd_rn(s1, s2);
    if (zero_bits(tail)) {
        tau = 0;
        beta = v0;
        e0 = e1 = 0;
        return;
    }
    beta = sqrt(__dadd_rn(__dmul_rn(v0, v0), tail));
    if (nonneg_bits(v0)) beta = -beta;
    const double den = __dsub_rn(v0, beta);
    const double nden = __longlong_as_double(__double_as_longlong(den) ^ (long long)0x8000000000000000ULL);
    const double num = lane == 0 ? v1 : (lane == 1 ? v2 : nden);
    const double q = num / (lane < 2 ? den : beta);
    e0 = __shfl_sync(0xffffffffu, q, 0);
    e1 = __shfl_sync(0xffffffffu, q, 1);
    tau = __shfl_sync(0xffffffffu, q, 2);
}

#define QR_BIG 96  // matrices with at least this many tones get a 4-warp group in k_har_qr_queue

// Matrices in descending Ng (counting sort; the order only schedules, every
// matrix is computed alone), so the longest QR runs start first.
__global__ void __launch_bounds__(256) k_har_order(const HarJob *__restrict__ hj, const char *__restrict__ wsb, int nmat,
                                                   int *__restrict__ perm) {
    __shared__ int cnt[258];
    for (int t = threadIdx.x; t < 258; t += blockDim.x) cnt[t] = 0;
    __syncthreads();
    for (int m = threadIdx.x; m < nmat; m += blockDim.x) {
        const int n = ((const int *)(wsb + hj[m >> 2].lut_b))[256];
        atomicAdd(&cnt[256 - n], 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int r = 0;
        for (int k = 0; k < 257; k++) {
            const int c = cnt[k];
            cnt[k] = r;
            r += c;
        }
    }
    __syncthreads();
    for (int m = threadIdx.x; m < nmat; m += blockDim.x) {
        const int n = ((const int *)(wsb + hj[m >> 2].lut_b))[256];
        perm[atomicAdd(&cnt[256 - n], 1)] = m;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        perm[nmat] = cnt[256 - QR_BIG];  // after placement cnt[k] = end of key k: matrices with Ng >= QR_BIG
        perm[nmat + 1] = 0;              // the work queue's tickets (k_har_qr_queue)
        perm[nmat + 2] = 0;
    }
}

#define QR_SYNC()                    \
    do {                             \
        if (NW > 1) __syncthreads(); \
        else __syncwarp();           \
    } while (0)
// One matrix per group of NW warps (tid = thread in the group): every thread
// takes the same decisions from the same values; writes of single entries are
// made by tid 0; the reflector updates spread their columns / rows over the
// group, with a barrier between dependent phases.
template <int NW>
__device__ void har_schur(double *__restrict__ A, const int n, double *__restrict__ rowsum, double *__restrict__ res,
                          const int tid, const int iter_per_tone) {
    const int lane = tid & 31;
    constexpr int GS = 32 * NW;
    if (n < 3) {
        if (tid == 0) res[13] = 0.0;
        return;
    }
#define T_(r, c) A[(long long)(r) * n + (c)]
    // computeNormOfT: row sums (sequential within a row), then rows in order
    for (int j = tid; j < n; j += GS) {
        const int s0 = j - 1 > 0 ? j - 1 : 0;
        double s = 0;
        for (int c = s0; c < n; c++) s = __dadd_rn(s, fabs(T_(j, c)));
        rowsum[j] = s;
    }
    QR_SYNC();
    double norm = 0;
    for (int j = 0; j < n; j++) norm = __dadd_rn(norm, rowsum[j]);
    const double eps = DBL_EPSILON;
    const int maxIter = iter_per_tone * n;  // Eigen: m_maxIterationsPerRow (40) * n
    int iu = n - 1, iter = 0, totalIter = 0;
    double exshift = 0;
    bool failed = false;
    if (norm != 0) {
        while (iu >= 0) {
            // findSmallSubdiagEntry: first il (downwards from iu) with a negligible T(il, il-1)
            int il = 0;
            for (int base = iu; base > 0; base -= 32) {
                const int r = base - lane;
                bool hit = false;
                if (r > 0) {
                    double sm = __dadd_rn(fabs(T_(r - 1, r - 1)), fabs(T_(r, r)));
                    if (sm == 0.0) sm = norm;
                    hit = fabs(T_(r, r - 1)) < __dmul_rn(eps, sm);
                }
                const unsigned b = __ballot_sync(0xffffffffu, hit);
                if (b) {
                    il = base - (__ffs(b) - 1);
                    break;
                }
            }
            if (il == iu) {
                QR_SYNC();
                if (tid == 0) {
                    T_(iu, iu) = __dadd_rn(T_(iu, iu), exshift);
                    if (iu > 0) T_(iu, iu - 1) = 0;
                }
                QR_SYNC();
                iu--;
                iter = 0;
            } else if (il == iu - 1) {
                const double p = __dmul_rn(0.5, __dsub_rn(T_(iu - 1, iu - 1), T_(iu, iu)));
                const double q = __dadd_rn(__dmul_rn(p, p), __dmul_rn(T_(iu, iu - 1), T_(iu - 1, iu)));
                QR_SYNC();
                if (tid == 0) {
                    T_(iu, iu) = __dadd_rn(T_(iu, iu), exshift);
                    T_(iu - 1, iu - 1) = __dadd_rn(T_(iu - 1, iu - 1), exshift);
                }
                QR_SYNC();
                if (q >= 0) {
                    const double z = sqrt(fabs(q));
                    const double gp = (p >= 0) ? __dadd_rn(p, z) : __dsub_rn(p, z), gq = T_(iu, iu - 1);
                    double c, s;
                    if (gq == 0) { c = gp < 0 ? -1 : 1; s = 0; }
                    else if (gp == 0) { c = 0; s = gq < 0 ? 1 : -1; }
                    else if (fabs(gp) > fabs(gq)) {
                        const double t = gq / gp;
                        double u = sqrt(__dadd_rn(1.0, __dmul_rn(t, t)));
                        if (gp < 0) u = -u;
                        c = 1 / u;
                        s = __dmul_rn(-t, c);
                    } else {
                        const double t = gp / gq;
                        double u = sqrt(__dadd_rn(1.0, __dmul_rn(t, t)));
                        if (gq < 0) u = -u;
                        s = -1 / u;
                        c = __dmul_rn(-t, s);
                    }
                    QR_SYNC();  // every thread has read gq before the block changes
                    // the 2x2 block: left (rows iu-1, iu), then right (cols iu-1, iu)
                    if (tid == 0) {
                        for (int col = iu - 1; col <= iu; col++) {
                            const double xi = T_(iu - 1, col), yi = T_(iu, col);
                            T_(iu - 1, col) = __dadd_rn(__dmul_rn(c, xi), __dmul_rn(-s, yi));
                            T_(iu, col) = __dadd_rn(__dmul_rn(s, xi), __dmul_rn(c, yi));
                        }
                        for (int row = iu - 1; row <= iu; row++) {
                            const double xi = T_(row, iu - 1), yi = T_(row, iu);
                            T_(row, iu - 1) = __dadd_rn(__dmul_rn(c, xi), __dmul_rn(-s, yi));
                            T_(row, iu) = __dadd_rn(__dmul_rn(s, xi), __dmul_rn(c, yi));
                        }
                        T_(iu, iu - 1) = 0;
                    }
                }
                if (tid == 0 && iu > 1) T_(iu - 1, iu - 2) = 0;
                QR_SYNC();
                iu -= 2;
                iter = 0;
            } else {
                double sh0 = T_(iu, iu), sh1 = T_(iu - 1, iu - 1), sh2 = __dmul_rn(T_(iu, iu - 1), T_(iu - 1, iu));
                if (iter == 10) {
                    exshift = __dadd_rn(exshift, sh0);
                    QR_SYNC();
                    for (int i = tid; i <= iu; i += GS) T_(i, i) = __dsub_rn(T_(i, i), sh0);
                    QR_SYNC();
                    const double s = __dadd_rn(fabs(T_(iu, iu - 1)), fabs(T_(iu - 1, iu - 2)));
                    sh0 = __dmul_rn(0.75, s);
                    sh1 = __dmul_rn(0.75, s);
                    sh2 = __dmul_rn(__dmul_rn(-0.4375, s), s);
                }
                if (iter == 30) {
                    double s = __dsub_rn(sh1, sh0) / 2.0;
                    s = __dadd_rn(__dmul_rn(s, s), sh2);
                    if (s > 0) {
                        s = sqrt(s);
                        if (sh1 < sh0) s = -s;
                        s = __dadd_rn(s, __dsub_rn(sh1, sh0) / 2.0);
                        s = __dsub_rn(sh0, sh2 / s);
                        exshift = __dadd_rn(exshift, s);
                        QR_SYNC();
                        for (int i = tid; i <= iu; i += GS) T_(i, i) = __dsub_rn(T_(i, i), s);
                        QR_SYNC();
                        sh0 = sh1 = sh2 = 0.964;
                    }
                }
                iter++;
                totalIter++;
                if (totalIter > maxIter) {
                    failed = true;
                    break;
                }
                // initFrancisQRStep: the first im from iu-2 down to il where the bulge may
                // start (il at the latest), with its first reflector column fv.  The
                // candidates are independent, so 32 are evaluated at once, one per lane,
                // each with the sequential search's own operations; the ballot keeps the
                // highest one that qualifies.
                double fv0 = 0, fv1 = 0, fv2 = 0;
                int im = il;
                for (int top = iu - 2; top >= il; top -= 32) {
                    const int cand = top - lane;
                    bool hit = false;
                    double a0 = 0, a1 = 0, a2 = 0;
                    if (cand >= il) {
                        const double Tmm = T_(cand, cand), r = __dsub_rn(sh0, Tmm), s = __dsub_rn(sh1, Tmm);
                        a0 = __dadd_rn(__dsub_rn(__dmul_rn(r, s), sh2) / T_(cand + 1, cand), T_(cand, cand + 1));
                        a1 = __dsub_rn(__dsub_rn(__dsub_rn(T_(cand + 1, cand + 1), Tmm), r), s);
                        a2 = T_(cand + 2, cand + 1);
                        if (cand == il) {
                            hit = true;
                        } else {
                            const double lhs = __dmul_rn(T_(cand, cand - 1), __dadd_rn(fabs(a1), fabs(a2)));
                            const double rhs = __dmul_rn(a0, __dadd_rn(__dadd_rn(fabs(T_(cand - 1, cand - 1)), fabs(Tmm)),
                                                                       fabs(T_(cand + 1, cand + 1))));
                            hit = fabs(lhs) < __dmul_rn(eps, rhs);
                        }
                    }
                    const unsigned b = __ballot_sync(0xffffffffu, hit);
                    if (b) {
                        const int src = __ffs(b) - 1;
                        im = top - src;
                        fv0 = __shfl_sync(0xffffffffu, a0, src);
                        fv1 = __shfl_sync(0xffffffffu, a1, src);
                        fv2 = __shfl_sync(0xffffffffu, a2, src);
                        break;
                    }
                }
                // performFrancisQRStep, restricted to the window
                for (int k = im; k <= iu - 2; ++k) {
                    const bool first = (k == im);
                    double ess[2], tau, beta;
                    if (first) hh_make3(fv0, fv1, fv2, lane, ess[0], ess[1], tau, beta);
                    else hh_make3(T_(k, k - 1), T_(k + 1, k - 1), T_(k + 2, k - 1), lane, ess[0], ess[1], tau, beta);
                    QR_SYNC();
                    if (!zero_bits(beta)) {
                        if (tid == 0) {
                            if (first && k > il) T_(k, k - 1) = -T_(k, k - 1);
                            else if (!first) T_(k, k - 1) = beta;
                        }
                        // tau * ess[0] and tau * ess[1] (alike for every column) in one multiply
                        const double tm = __dmul_rn(tau, lane == 0 ? ess[0] : ess[1]);
                        const double te0 = __shfl_sync(0xffffffffu, tm, 0), te1 = __shfl_sync(0xffffffffu, tm, 1);
                        for (int cc = k + tid; cc <= iu; cc += GS) {  // left: rows k..k+2
                            const double a0 = T_(k, cc), a1 = T_(k + 1, cc), a2 = T_(k + 2, cc);
                            double t = plus_zero(__dmul_rn(ess[0], a1));
                            t = __dadd_rn(t, __dmul_rn(ess[1], a2));
                            t = __dadd_rn(t, a0);
                            T_(k, cc) = __dsub_rn(a0, __dmul_rn(tau, t));
                            T_(k + 1, cc) = __dsub_rn(a1, __dmul_rn(te0, t));
                            T_(k + 2, cc) = __dsub_rn(a2, __dmul_rn(te1, t));
                        }
                        QR_SYNC();
                        const int rend = min(iu, k + 3);
                        for (int rr = il + tid; rr <= rend; rr += GS) {  // right: cols k..k+2
                            const double b0 = T_(rr, k), b1 = T_(rr, k + 1), b2 = T_(rr, k + 2);
                            double t = plus_zero(__dmul_rn(b1, ess[0]));
                            t = __dadd_rn(t, __dmul_rn(b2, ess[1]));
                            t = __dadd_rn(t, b0);
                            const double tt = __dmul_rn(tau, t);
                            T_(rr, k) = __dsub_rn(b0, tt);
                            T_(rr, k + 1) = __dsub_rn(b1, __dmul_rn(tt, ess[0]));
                            T_(rr, k + 2) = __dsub_rn(b2, __dmul_rn(tt, ess[1]));
                        }
                    }
                    QR_SYNC();
                }
                {
                    double vv[2] = {T_(iu - 1, iu - 2), T_(iu, iu - 2)}, ess[1], tau, beta;
                    hh_make(vv, 2, ess, tau, beta);
                    QR_SYNC();
                    if (beta != 0) {
                        if (tid == 0) T_(iu - 1, iu - 2) = beta;
                        const double te0 = __dmul_rn(tau, ess[0]);
                        for (int cc = iu - 1 + tid; cc <= iu; cc += GS) {
                            const double a0 = T_(iu - 1, cc), a1 = T_(iu, cc);
                            double t = __dadd_rn(__dmul_rn(ess[0], a1), 0.0);
                            t = __dadd_rn(t, a0);
                            T_(iu - 1, cc) = __dsub_rn(a0, __dmul_rn(tau, t));
                            T_(iu, cc) = __dsub_rn(a1, __dmul_rn(te0, t));
                        }
                        QR_SYNC();
                        for (int rr = il + tid; rr <= iu; rr += GS) {
                            const double b0 = T_(rr, iu - 1), b1 = T_(rr, iu);
                            double t = __dadd_rn(__dmul_rn(b1, ess[0]), 0.0);
                            t = __dadd_rn(t, b0);
                            const double tt = __dmul_rn(tau, t);
                            T_(rr, iu - 1) = __dsub_rn(b0, tt);
                            T_(rr, iu) = __dsub_rn(b1, __dmul_rn(tt, ess[0]));
                        }
                    }
                    QR_SYNC();
                }
                for (int i = im + 2 + tid; i <= iu; i += GS) {
                    T_(i, i - 2) = 0;
                    if (i > im + 2) T_(i, i - 3) = 0;
                }
                QR_SYNC();
            }
        }
    }
    if (tid == 0) {
        double f = 0;
        if (!failed) {
            // eigenvalue #2 in Schur order (EigenSolver::compute, EigenSolver.h:363-381)
            int i = 0;
            double re2 = 0, im2 = 1;
            while (i < n && i <= 2) {
                if (i == n - 1 || T_(i + 1, i) == 0) {
                    if (i == 2) { re2 = T_(i, i); im2 = 0; }
                    ++i;
                } else {
                    const double p = __dmul_rn(0.5, __dsub_rn(T_(i, i), T_(i + 1, i + 1)));
                    const double z = sqrt(fabs(__dadd_rn(__dmul_rn(p, p), __dmul_rn(T_(i + 1, i), T_(i, i + 1)))));
                    if (i == 2 || i + 1 == 2) { re2 = __dadd_rn(T_(i + 1, i + 1), p); im2 = (i == 2) ? z : -z; }
                    i += 2;
                }
            }
            // the reference's sqrt (NaN for a rounding-negative eigenvalue)
            if (im2 == 0) f = sqrt(re2);
        }
        res[13] = f;  // no convergence: 0, as the oracle
    }
#undef T_
}

// The mixed form's real Schur iteration: the same algorithm, windows and
// decisions as har_schur, with the matrix held and updated in pairs of floats
// (about 48 significant bits, on the FP32 pipe instead of the FP64 one).  The
// deflation threshold is eps = 2^-46 (a few units of the pairs' rounding, as
// Eigen's epsilon is for doubles), relative to the two diagonal entries as
// there, or eps times the matrix's norm: clusters of eigenvalues near 1e-18
// (Q is close to singular) cannot reach the relative threshold within float's
// exponent range, and without the normwise one ran to the iteration limit.
// The choices between candidates compare the leading floats.  The Hessenberg
// matrix arrives in pairs from k_har_hess_df (a double and a pair are both 8
// bytes, in the same place).
// The vector is first scaled by a power of two that brings its largest entry
// into [0.5, 1): exact, leaves ess and tau unchanged and beta scaled back, and
// keeps the squares within float's exponent range (FP64's wider range needs no
// such step; unscaled, bulges of 1e-20 underflowed to 0 / 0).
__device__ __forceinline__ void hh_scale(float m, float &down, float &up) {
    const int eb = (int)((__float_as_uint(m) >> 23) & 0xff);  // m > 0, eb <= 252 for these matrices
    down = __uint_as_float((unsigned)(253 - min(eb, 252)) << 23);
    up = __uint_as_float((unsigned)(min(eb, 252) + 1) << 23);
}
__device__ __forceinline__ void hh_make3_df(const df v0, const df v1, const df v2, int lane, df &e0, df &e1, df &tau,
                                            df &beta) {
    const float m = fmaxf(fabsf(v0.hi), fmaxf(fabsf(v1.hi), fabsf(v2.hi)));
    tau = {0.f, 0.f};
    beta = v0;
    e0 = e1 = {0.f, 0.f};
    if (m == 0.f) return;
    float down, up;
    hh_scale(m, down, up);
    const df w0 = df_scale(v0, down), w1 = df_scale(v1, down), w2 = df_scale(v2, down);
    const df wl = lane == 2 ? w2 : w1;
    const df sq = df_mul(wl, wl);
    const df tail = df_add(df_shfl(sq, 1), df_shfl(sq, 2));
    if (tail.hi == 0.f) return;
    df bb = df_sqrt(df_fma(w0, w0, tail));
    if (w0.hi >= 0.f) bb = df_neg(bb);
    const df den = df_sub(w0, bb);
    const df num = lane == 0 ? w1 : (lane == 1 ? w2 : df_sub(bb, w0));
    const df q = df_div(num, lane < 2 ? den : bb);
    e0 = df_shfl(q, 0);
    e1 = df_shfl(q, 1);
    tau = df_shfl(q, 2);
    beta = df_scale(bb, up);
}

template <int NW>
__device__ void har_schur_df(df *__restrict__ A, const int n, float *__restrict__ rowsum, double *__restrict__ res,
                             const int tid, const int iter_per_tone) {
    const int lane = tid & 31;
    constexpr int GS = 32 * NW;
    if (n < 3) {
        if (tid == 0) res[13] = 0.0;
        return;
    }
#define T_(r, c) A[(long long)(r) * n + (c)]
    for (int j = tid; j < n; j += GS) {
        float s = 0.f;
        for (int c = (j > 0 ? j - 1 : 0); c < n; c++) s = __fadd_rn(s, fabsf(T_(j, c).hi));
        rowsum[j] = s;
    }
    QR_SYNC();
    float norm = 0.f;
    for (int j = 0; j < n; j++) norm = __fadd_rn(norm, rowsum[j]);
    const float eps = 0x1p-46f, nthr = __fmul_rn(eps, norm);
    const int maxIter = iter_per_tone * n;  // Eigen: m_maxIterationsPerRow (40) * n
    int iu = n - 1, iter = 0, totalIter = 0;
    df exshift = {0.f, 0.f};
    bool failed = false;
    const df zero = {0.f, 0.f};
    if (norm != 0.f) {
        while (iu >= 0) {
            int il = 0;
            for (int base = iu; base > 0; base -= 32) {
                const int r = base - lane;
                bool hit = false;
                if (r > 0) {
                    float sm = __fadd_rn(fabsf(T_(r - 1, r - 1).hi), fabsf(T_(r, r).hi));
                    if (sm == 0.f) sm = norm;
                    const float sub = fabsf(T_(r, r - 1).hi);
                    hit = sub < __fmul_rn(eps, sm) || sub < nthr;
                }
                const unsigned b = __ballot_sync(0xffffffffu, hit);
                if (b) {
                    il = base - (__ffs(b) - 1);
                    break;
                }
            }
            if (il == iu) {
                QR_SYNC();
                if (tid == 0) {
                    T_(iu, iu) = df_add(T_(iu, iu), exshift);
                    if (iu > 0) T_(iu, iu - 1) = zero;
                }
                QR_SYNC();
                iu--;
                iter = 0;
            } else if (il == iu - 1) {
                const df p = df_scale(df_sub(T_(iu - 1, iu - 1), T_(iu, iu)), 0.5f);
                const df q = df_fma(p, p, df_mul(T_(iu, iu - 1), T_(iu - 1, iu)));
                QR_SYNC();
                if (tid == 0) {
                    T_(iu, iu) = df_add(T_(iu, iu), exshift);
                    T_(iu - 1, iu - 1) = df_add(T_(iu - 1, iu - 1), exshift);
                }
                QR_SYNC();
                if (q.hi >= 0.f) {
                    const df z = q.hi == 0.f ? zero : df_sqrt(q);
                    const df gp = (p.hi >= 0.f) ? df_add(p, z) : df_sub(p, z), gq = T_(iu, iu - 1);
                    df c, s;
                    const df one = {1.f, 0.f};
                    if (gq.hi == 0.f) { c = {gp.hi < 0.f ? -1.f : 1.f, 0.f}; s = zero; }
                    else if (gp.hi == 0.f) { c = zero; s = {gq.hi < 0.f ? 1.f : -1.f, 0.f}; }
                    else if (df_lt(df_abs(gq), df_abs(gp))) {
                        const df t = df_div(gq, gp);
                        df u = df_sqrt(df_fma(t, t, one));
                        if (gp.hi < 0.f) u = df_neg(u);
                        c = df_div(one, u);
                        s = df_neg(df_mul(t, c));
                    } else {
                        const df t = df_div(gp, gq);
                        df u = df_sqrt(df_fma(t, t, one));
                        if (gq.hi < 0.f) u = df_neg(u);
                        s = df_neg(df_div(one, u));
                        c = df_neg(df_mul(t, s));
                    }
                    QR_SYNC();
                    if (tid == 0) {
                        for (int col = iu - 1; col <= iu; col++) {
                            const df xi = T_(iu - 1, col), yi = T_(iu, col);
                            T_(iu - 1, col) = df_fma(c, xi, df_mul(df_neg(s), yi));
                            T_(iu, col) = df_fma(s, xi, df_mul(c, yi));
                        }
                        for (int row = iu - 1; row <= iu; row++) {
                            const df xi = T_(row, iu - 1), yi = T_(row, iu);
                            T_(row, iu - 1) = df_fma(c, xi, df_mul(df_neg(s), yi));
                            T_(row, iu) = df_fma(s, xi, df_mul(c, yi));
                        }
                        T_(iu, iu - 1) = zero;
                    }
                }
                if (tid == 0 && iu > 1) T_(iu - 1, iu - 2) = zero;
                QR_SYNC();
                iu -= 2;
                iter = 0;
            } else {
                df sh0 = T_(iu, iu), sh1 = T_(iu - 1, iu - 1), sh2 = df_mul(T_(iu, iu - 1), T_(iu - 1, iu));
                if (iter == 10) {
                    exshift = df_add(exshift, sh0);
                    QR_SYNC();
                    for (int i = tid; i <= iu; i += GS) T_(i, i) = df_sub(T_(i, i), sh0);
                    QR_SYNC();
                    const df s = df_add(df_abs(T_(iu, iu - 1)), df_abs(T_(iu - 1, iu - 2)));
                    sh0 = df_mul(s, {0.75f, 0.f});
                    sh1 = sh0;
                    sh2 = df_mul(df_mul(s, {-0.4375f, 0.f}), s);
                }
                if (iter == 30) {
                    df s = df_scale(df_sub(sh1, sh0), 0.5f);
                    s = df_fma(s, s, sh2);
                    if (s.hi > 0.f) {
                        s = df_sqrt(s);
                        if (df_lt(sh1, sh0)) s = df_neg(s);
                        s = df_add(s, df_scale(df_sub(sh1, sh0), 0.5f));
                        s = df_sub(sh0, df_div(sh2, s));
                        exshift = df_add(exshift, s);
                        QR_SYNC();
                        for (int i = tid; i <= iu; i += GS) T_(i, i) = df_sub(T_(i, i), s);
                        QR_SYNC();
                        sh0 = sh1 = sh2 = df{0.964f, 0.f};
                    }
                }
                iter++;
                totalIter++;
                if (totalIter > maxIter) {
                    failed = true;
                    break;
                }
                df fv0 = zero, fv1 = zero, fv2 = zero;
                int im = il;
                for (int top = iu - 2; top >= il; top -= 32) {
                    const int cand = top - lane;
                    bool hit = false;
                    df a0 = zero, a1 = zero, a2 = zero;
                    if (cand >= il) {
                        const df Tmm = T_(cand, cand), r = df_sub(sh0, Tmm), s = df_sub(sh1, Tmm);
                        a0 = df_add(df_div(df_sub(df_mul(r, s), sh2), T_(cand + 1, cand)), T_(cand, cand + 1));
                        a1 = df_sub(df_sub(df_sub(T_(cand + 1, cand + 1), Tmm), r), s);
                        a2 = T_(cand + 2, cand + 1);
                        if (cand == il) {
                            hit = true;
                        } else {
                            const float lhs = __fmul_rn(T_(cand, cand - 1).hi, __fadd_rn(fabsf(a1.hi), fabsf(a2.hi)));
                            const float rhs = __fmul_rn(a0.hi, __fadd_rn(__fadd_rn(fabsf(T_(cand - 1, cand - 1).hi), fabsf(Tmm.hi)),
                                                                         fabsf(T_(cand + 1, cand + 1).hi)));
                            hit = fabsf(lhs) < __fmul_rn(eps, rhs);
                        }
                    }
                    const unsigned b = __ballot_sync(0xffffffffu, hit);
                    if (b) {
                        const int src = __ffs(b) - 1;
                        im = top - src;
                        fv0 = df_shfl(a0, src);
                        fv1 = df_shfl(a1, src);
                        fv2 = df_shfl(a2, src);
                        break;
                    }
                }
                for (int k = im; k <= iu - 2; ++k) {
                    const bool first = (k == im);
                    df e0, e1, tau, beta;
                    if (first) hh_make3_df(fv0, fv1, fv2, lane, e0, e1, tau, beta);
                    else hh_make3_df(T_(k, k - 1), T_(k + 1, k - 1), T_(k + 2, k - 1), lane, e0, e1, tau, beta);
                    QR_SYNC();
                    if (beta.hi != 0.f) {
                        if (tid == 0) {
                            if (first && k > il) T_(k, k - 1) = df_neg(T_(k, k - 1));
                            else if (!first) T_(k, k - 1) = beta;
                        }
                        const df ntau = df_neg(tau), nte0 = df_neg(df_mul(tau, e0)), nte1 = df_neg(df_mul(tau, e1));
                        for (int cc = k + tid; cc <= iu; cc += GS) {  // left: rows k..k+2
                            const df a0 = T_(k, cc), a1 = T_(k + 1, cc), a2 = T_(k + 2, cc);
                            const df t = df_add(df_fma(e1, a2, df_mul(e0, a1)), a0);
                            T_(k, cc) = df_fma(ntau, t, a0);
                            T_(k + 1, cc) = df_fma(nte0, t, a1);
                            T_(k + 2, cc) = df_fma(nte1, t, a2);
                        }
                        QR_SYNC();
                        const int rend = min(iu, k + 3);
                        for (int rr = il + tid; rr <= rend; rr += GS) {  // right: cols k..k+2
                            const df b0 = T_(rr, k), b1 = T_(rr, k + 1), b2 = T_(rr, k + 2);
                            const df ntt = df_neg(df_mul(tau, df_add(df_fma(b2, e1, df_mul(b1, e0)), b0)));
                            T_(rr, k) = df_add(b0, ntt);
                            T_(rr, k + 1) = df_fma(ntt, e0, b1);
                            T_(rr, k + 2) = df_fma(ntt, e1, b2);
                        }
                    }
                    QR_SYNC();
                }
                {
                    const df v0 = T_(iu - 1, iu - 2), v1 = T_(iu, iu - 2);
                    df e0 = zero, tau = zero, beta = v0;
                    const float m = fmaxf(fabsf(v0.hi), fabsf(v1.hi));
                    if (m != 0.f) {
                        float down, up;
                        hh_scale(m, down, up);
                        const df w0 = df_scale(v0, down), w1 = df_scale(v1, down);
                        const df tail = df_mul(w1, w1);
                        if (tail.hi != 0.f) {
                            df bb = df_sqrt(df_fma(w0, w0, tail));
                            if (w0.hi >= 0.f) bb = df_neg(bb);
                            e0 = df_div(w1, df_sub(w0, bb));
                            tau = df_div(df_sub(bb, w0), bb);
                            beta = df_scale(bb, up);
                        }
                    }
                    QR_SYNC();
                    if (beta.hi != 0.f) {
                        if (tid == 0) T_(iu - 1, iu - 2) = beta;
                        const df ntau = df_neg(tau), nte0 = df_neg(df_mul(tau, e0));
                        for (int cc = iu - 1 + tid; cc <= iu; cc += GS) {
                            const df a0 = T_(iu - 1, cc), a1 = T_(iu, cc);
                            const df t = df_fma(e0, a1, a0);
                            T_(iu - 1, cc) = df_fma(ntau, t, a0);
                            T_(iu, cc) = df_fma(nte0, t, a1);
                        }
                        QR_SYNC();
                        for (int rr = il + tid; rr <= iu; rr += GS) {
                            const df b0 = T_(rr, iu - 1), b1 = T_(rr, iu);
                            const df ntt = df_neg(df_mul(tau, df_fma(b1, e0, b0)));
                            T_(rr, iu - 1) = df_add(b0, ntt);
                            T_(rr, iu) = df_fma(ntt, e0, b1);
                        }
                    }
                    QR_SYNC();
                }
                for (int i = im + 2 + tid; i <= iu; i += GS) {
                    T_(i, i - 2) = zero;
                    if (i > im + 2) T_(i, i - 3) = zero;
                }
                QR_SYNC();
            }
        }
    }
    if (tid == 0) {
        double f = 0;
        if (!failed) {
            // eigenvalue #2 in Schur order (EigenSolver::compute, EigenSolver.h:363-381), in FP64 from the pairs
            int i = 0;
            double re2 = 0, im2 = 1;
            while (i < n && i <= 2) {
                if (i == n - 1 || T_(i + 1, i).hi == 0.f) {
                    if (i == 2) { re2 = df_to_double(T_(i, i)); im2 = 0; }
                    ++i;
                } else {
                    const double tii = df_to_double(T_(i, i)), tjj = df_to_double(T_(i + 1, i + 1));
                    const double p = 0.5 * (tii - tjj);
                    const double z = sqrt(fabs(p * p + df_to_double(T_(i + 1, i)) * df_to_double(T_(i, i + 1))));
                    if (i == 2 || i + 1 == 2) { re2 = tjj + p; im2 = (i == 2) ? z : -z; }
                    i += 2;
                }
            }
            if (im2 == 0) f = sqrt(fmax(re2, 0.0));
        }
        res[13] = f;  // no convergence: 0, as the oracle
    }
#undef T_
}

// The mixed form's Hessenberg reduction: the reflectors and updates of
// k_har_hess in pairs of floats (FP32 pipe) on Q from k_har_q_df; a column
// whose largest entry is far from 1 is scaled by a power of two before its
// squares are summed (exact; keeps them within float's exponent range).  The
// matrix stays in pairs for har_schur_df.
__device__ __forceinline__ df block_sum_df(df v, df *sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v = df_add(v, {__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)});
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    df r = (threadIdx.x < nw) ? sh[threadIdx.x] : df{0.f, 0.f};
    if (wid == 0)
        for (int o = 16; o > 0; o >>= 1) r = df_add(r, {__shfl_down_sync(0xffffffffu, r.hi, o), __shfl_down_sync(0xffffffffu, r.lo, o)});
    if (threadIdx.x == 0) sh[0] = r;
    __syncthreads();
    r = sh[0];
    __syncthreads();
    return r;
}

// max of the floats m and sum of the pairs q over the block (fixed tree); m is
// replaced by the block's max, the sum returned; valid in every thread
__device__ __forceinline__ df block_max_sum(float &m, df q, float *shm, df *shq) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
        q = df_add(q, {__shfl_down_sync(0xffffffffu, q.hi, o), __shfl_down_sync(0xffffffffu, q.lo, o)});
    }
    __syncthreads();
    if (lane == 0) {
        shm[wid] = m;
        shq[wid] = q;
    }
    __syncthreads();
    float rm = (threadIdx.x < nw) ? shm[threadIdx.x] : 0.f;
    df rq = (threadIdx.x < nw) ? shq[threadIdx.x] : df{0.f, 0.f};
    if (wid == 0)
        for (int o = 16; o > 0; o >>= 1) {
            rm = fmaxf(rm, __shfl_down_sync(0xffffffffu, rm, o));
            rq = df_add(rq, {__shfl_down_sync(0xffffffffu, rq.hi, o), __shfl_down_sync(0xffffffffu, rq.lo, o)});
        }
    if (threadIdx.x == 0) {
        shm[0] = rm;
        shq[0] = rq;
    }
    __syncthreads();
    m = shm[0];
    rq = shq[0];
    __syncthreads();
    return rq;
}

__global__ void __launch_bounds__(256) k_har_hess_df(const HarJob *__restrict__ hj, char *__restrict__ wsb) {
    __shared__ df v[256], ess[256], tess[256], red[32];
    __shared__ float redf[32];
    __shared__ df s_tau, s_beta, s_den;
    __shared__ int s_triv;
    const int ang = blockIdx.y;
    const HarJob H = hj[blockIdx.x];
    const int n = ((const int *)(wsb + H.lut_b))[256];
    if (n < 3) return;
    df *A = (df *)((double *)(wsb + H.q_b) + (long long)ang * 256 * 256);
    const df zero = {0.f, 0.f};
    for (int i = 0; i < n - 1; i++) {
        const int rem = n - i - 1;
        // the largest entry and the unscaled tail sum in one reduction; the
        // scaled sum is formed only when the largest entry leaves [2^-40, 2^40]
        // (inside it the sum of squares and its low parts stay well within
        // float's normal range, as accurate as the scaled sum)
        float m = 0.f;
        df q = zero;
        for (int k = threadIdx.x; k < rem; k += blockDim.x) {
            const df x = A[(long long)(i + 1 + k) * n + i];
            v[k] = x;
            m = fmaxf(m, fabsf(x.hi));
            if (k > 0) q = df_fma(x, x, q);
        }
        df tail = block_max_sum(m, q, redf, red);
        float down = 1.f, up = 1.f;
        if (m != 0.f) hh_scale(m, down, up);
        if (m != 0.f && (m < 0x1p-40f || m > 0x1p40f)) {
            q = zero;
            for (int k = 1 + threadIdx.x; k < rem; k += blockDim.x) {
                const df w = df_scale(v[k], down);
                q = df_fma(w, w, q);
            }
            tail = block_sum_df(q, red);
        } else {
            tail = df_scale(tail, __fmul_rn(down, down));
        }
        if (threadIdx.x == 0) {  // makeHouseholder (Householder.h:65-90) on the scaled vector
            const df c0 = df_scale(v[0], down);
            if (rem == 1 || tail.hi == 0.f) {
                s_triv = 1;
                s_beta = v[0];
            } else {
                df bb = df_sqrt(df_fma(c0, c0, tail));
                if (c0.hi >= 0.f) bb = df_neg(bb);
                s_triv = 0;
                s_beta = df_scale(bb, up);
                s_den = df_sub(c0, bb);
                s_tau = df_div(df_sub(bb, c0), bb);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) A[(long long)(i + 1) * n + i] = s_beta;
        if (s_triv) {  // tau = 0: both updates are the identity
            __syncthreads();
            continue;
        }
        const df tau = s_tau, ntau = df_neg(tau);
        for (int k = 1 + threadIdx.x; k < rem; k += blockDim.x) {
            const df e = df_div(df_scale(v[k], down), s_den);
            ess[k - 1] = e;
            tess[k - 1] = df_neg(df_mul(tau, e));
        }
        __syncthreads();
        // H A: rows i+1.., columns i+1.. (threads over columns)
        for (int c = i + 1 + threadIdx.x; c < n; c += blockDim.x) {
            df *col = A + (long long)(i + 1) * n + c;
            df t = zero;
            for (int r = 1; r < rem; r++) t = df_fma(ess[r - 1], col[(long long)r * n], t);
            t = df_add(t, col[0]);
            col[0] = df_fma(ntau, t, col[0]);
            for (int r = 1; r < rem; r++) col[(long long)r * n] = df_fma(tess[r - 1], t, col[(long long)r * n]);
        }
        __syncthreads();
        // A H: all rows, columns i+1.. (threads over rows)
        for (int r = threadIdx.x; r < n; r += blockDim.x) {
            df *row = A + (long long)r * n + i + 1;
            df t = zero;
            for (int c = 1; c < rem; c++) t = df_fma(row[c], ess[c - 1], t);
            t = df_add(t, row[0]);
            const df ntt = df_neg(df_mul(tau, t));
            row[0] = df_add(row[0], ntt);
            for (int c = 1; c < rem; c++) row[c] = df_fma(ntt, ess[c - 1], row[c]);
        }
        __syncthreads();
    }
    for (long long q = threadIdx.x; q < (long long)n * n; q += blockDim.x) {
        const int r = (int)(q / n), c = (int)(q - (long long)r * n);
        if (c < r - 1) A[q] = zero;
    }
}

// The real-Schur QR of every matrix as a persistent work queue: a grid of a few CTAs
// per SM, each of 4 warps.  While large matrices remain (those with at least
// QR_BIG tones, first in the descending order, when `groups` is set) a CTA
// takes the next one as a 4-warp group through ticket 0; then every warp
// takes single matrices, largest first, through ticket 1, until the list is
// exhausted.  A CTA that finishes a short matrix takes the next, so uneven
// tone counts (uneven tiles, uneven planes) balance themselves; no thread
// ever waits on another CTA.
template <bool MIXED>
__global__ void __launch_bounds__(128) k_har_qr_queue(const HarJob *__restrict__ hj, char *__restrict__ wsb,
                                                      int *__restrict__ perm, int nmat, int groups,
                                                      int iter_per_tone) {
    __shared__ double rowsum[4][256];
    __shared__ int s_take;
    int *tick = perm + nmat + 1;
    const int nbig = groups ? perm[nmat] : 0;
    const int wq = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // phase 1: 4-warp groups on the large matrices
    for (;;) {
        if (threadIdx.x == 0) s_take = atomicAdd(&tick[0], 1);
        __syncthreads();
        const int b = s_take;
        __syncthreads();
        if (b >= nbig) break;
        const int m = perm[b];
        const HarJob H = hj[m >> 2];
        const int ang = m & 3;
        const int n = ((const int *)(wsb + H.lut_b))[256];
        double *res = (double *)(wsb + H.res_b) + ang * 14;
        double *A = (double *)(wsb + H.q_b) + (long long)ang * 256 * 256;
        if (MIXED) har_schur_df<4>((df *)A, n, (float *)rowsum[0], res, threadIdx.x, iter_per_tone);
        else har_schur<4>(A, n, rowsum[0], res, threadIdx.x, iter_per_tone);
        __syncthreads();
    }
    // phase 2: one warp per matrix
    for (;;) {
        int s = 0;
        if (lane == 0) s = atomicAdd(&tick[1], 1);
        s = __shfl_sync(0xffffffffu, s, 0);
        const int idx = nbig + s;
        if (idx >= nmat) break;
        const int m = perm[idx];
        const HarJob H = hj[m >> 2];
        const int ang = m & 3;
        const int n = ((const int *)(wsb + H.lut_b))[256];
        double *res = (double *)(wsb + H.res_b) + ang * 14;
        double *A = (double *)(wsb + H.q_b) + (long long)ang * 256 * 256;
        if (MIXED) har_schur_df<1>((df *)A, n, (float *)rowsum[wq], res, lane, iter_per_tone);
        else har_schur<1>(A, n, rowsum[wq], res, lane, iter_per_tone);
    }
}

// mean and range over the angles, permuted into the output order
__global__ void k_har_final(const FJob *__restrict__ jobs, const HarJob *__restrict__ hj, const char *__restrict__ wsb,
                            double *__restrict__ feat) {
    const FJob J = jobs[blockIdx.x];
    const HarJob H = hj[blockIdx.x];
    const double *res = (const double *)(wsb + H.res_b);
    if (threadIdx.x != 0) return;
    double mn[14], mx[14], sm[14], tmp[28];
    for (int a = 0; a < 14; a++) { mn[a] = 10E200; mx[a] = -10E200; sm[a] = 0; }
    for (int ang = 0; ang < 4; ang++)
        for (int a = 0; a < 14; a++) {
            const double v = res[ang * 14 + a];
            sm[a] += v;
            if (v < mn[a]) mn[a] = v;
            if (v > mx[a]) mx[a] = v;
        }
    for (int a = 0; a < 14; a++) { tmp[a] = sm[a] / 4; tmp[a + 14] = mx[a] - mn[a]; }
    const int perm[28] = {0, 14, 1, 15, 2, 16, 9, 23, 10, 24, 8, 22, 11, 25, 4, 18, 13, 27, 12, 26, 5, 19, 7, 21, 6, 20, 3, 17};
    for (int k = 0; k < 28; k++) feat[J.out + k] = tmp[perm[k]];
}

void launch_haralick(Ctx &c, const double *arena, const Plane *planes, const PlaneStats *stats, const FJob *jobs,
                     int njobs, const HarJob *hj, char *wsb, int *perm, double *feat) {
    if (njobs <= 0) return;
    const int sm = 256 * 257 / 2 * sizeof(unsigned int);
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_har_glcm, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
        attr = true;
    }
    {
    ProfScope p1(c, "Haralick: quantise, GLCM, f1-f13");
    WC_LAUNCH(c);
    k_har_quant<<<njobs, 1024, 0, c.st>>>(arena, planes, stats, jobs, hj, wsb);
    WC_LAUNCH(c);
    k_har_glcm<<<dim3(njobs, 4), 1024, sm, c.st>>>(planes, jobs, hj, wsb);
    WC_LAUNCH(c);
    k_har_stats<<<dim3(njobs, 4), 256, 0, c.st>>>(jobs, hj, wsb);
    }
    // the mixed form's f14 chain in pairs of floats, or (f14_exact) the FP64
    // chain, whose f14 is bit-identical to the FP64 form's
    const bool df14 = c.prec == WC_PREC_MIXED && !c.opt->f14_exact;
    const int ipt = c.opt->qr_iter_per_tone;
    {
    ProfScope p2(c, "Haralick: Q");
    WC_LAUNCH(c);
    if (df14) {
        k_har_p_df<<<dim3(njobs, 4), 256, 0, c.st>>>(hj, wsb);
        WC_LAUNCH(c);
        k_har_q_df<<<dim3(njobs, 4, 4), 32 * Q_WARPS, 0, c.st>>>(hj, wsb);
    } else {
        k_har_q<<<dim3(njobs, 4, 4), 32 * Q_WARPS, 0, c.st>>>(hj, wsb);
    }
    }
    {
    ProfScope p3(c, "Haralick: Hessenberg");
    WC_LAUNCH(c);
    if (df14) k_har_hess_df<<<dim3(njobs, 4), 256, 0, c.st>>>(hj, wsb);
    else k_har_hess<<<dim3(njobs, 4), 256, 0, c.st>>>(hj, wsb);
    }
    {
    ProfScope p4(c, "Haralick: real Schur (f14)");
    WC_LAUNCH(c);
    k_har_order<<<1, 256, 0, c.st>>>(hj, wsb, 4 * njobs, perm);
    // The work-queue kernel with the shape the tuner picks for this chain and
    // batch size: 4-warp groups for the large matrices or not, 5 or 3 CTAs
    // per SM (candidate 0: groups, 5 per SM, also used with tuning off).
    const int nmat = 4 * njobs;
    int lg = 0;
    while ((1 << lg) < nmat) lg++;
    const std::string key = std::string(df14 ? "har_qr/pairs/" : "har_qr/fp64/") + std::to_string(lg);
    const int cand = c.tune ? c.tune->pick(key, 3) : 0;
    const int groups = cand != 1, per_sm = cand == 2 ? 3 : 5;
    const int grid = std::max(1, std::min(c.sms * per_sm, (nmat + 3) / 4));
    Tuner::Pending tp;
    const bool timing = c.tune && c.tune->exploring(key);
    if (timing) c.tune->begin(key, cand, c.st, tp);
    WC_LAUNCH(c);
    if (df14) k_har_qr_queue<true><<<grid, 128, 0, c.st>>>(hj, wsb, perm, nmat, groups, ipt);
    else k_har_qr_queue<false><<<grid, 128, 0, c.st>>>(hj, wsb, perm, nmat, groups, ipt);
    if (timing) c.tune->end(tp, c.st);
    }
    WC_LAUNCH(c);
    k_har_final<<<njobs, 32, 0, c.st>>>(jobs, hj, wsb, feat);
}

}  // namespace wc
