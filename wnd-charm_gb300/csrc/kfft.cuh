// Stockham mixed-radix DFT of several lines held in shared memory (any
// length; radix-p stages with host-computed FP64 twiddles
// tw[k] = exp(-2 pi i k / n)).  Shared by the Fourier transform node and the
// Gabor FFT convolution; templated on the element type (FP64 form, and FP32
// for the mixed form's Gabor filtering) and on the twiddles' type (FP64, or
// the FP64 twiddles rounded to FP32 once, in shared memory).  Radices 2, 4
// and 8 are butterflies (radix 8 as two radix-4 butterflies and the factors
// 1, (1-i)/sqrt2, -i, -(1+i)/sqrt2); an odd prime is a direct DFT over the
// twiddle table.  The operations and their order are the oracle's DFT's
// (oracle/fft_cpu.h), so the FP64 Fourier planes agree with it bit for bit.
#pragma once
#include "kernels.h"

namespace wc {

template <typename R>
struct cpx {
    R x, y;
};
typedef cpx<double> cplx;
template <typename R>
__device__ __forceinline__ cpx<R> cmul(cpx<R> a, cpx<R> b) {
    return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename R>
__device__ __forceinline__ cpx<R> cadd(cpx<R> a, cpx<R> b) {
    return {a.x + b.x, a.y + b.y};
}
template <typename R>
__device__ __forceinline__ cpx<R> csub(cpx<R> a, cpx<R> b) {
    return {a.x - b.x, a.y - b.y};
}
// X0 = a0 + a2, X1 = a1 - i a3, X2 = a0 - a2, X3 = a1 + i a3 with a0 = v0 + v2,
// a1 = v0 - v2, a2 = v1 + v3, a3 = v1 - v3 (W = -i)
template <typename R>
__device__ __forceinline__ void bfly4(cpx<R> v0, cpx<R> v1, cpx<R> v2, cpx<R> v3, cpx<R> *X) {
    const cpx<R> a0 = cadd(v0, v2), a1 = csub(v0, v2), a2 = cadd(v1, v3), a3 = csub(v1, v3);
    X[0] = cadd(a0, a2);
    X[1] = {a1.x + a3.y, a1.y - a3.x};
    X[2] = csub(a0, a2);
    X[3] = {a1.x - a3.y, a1.y + a3.x};
}
// E = DFT4 of the even inputs, O = DFT4 of the odd ones; X_q = E_q + W8^q O_q,
// X_{q+4} = E_q - W8^q O_q, W8 = (1 - i) / sqrt2
template <typename R>
__device__ __forceinline__ void bfly8(const cpx<R> *v, cpx<R> *X) {
    const R c = (R)0.70710678118654752440;
    cpx<R> E[4], O[4];
    bfly4(v[0], v[2], v[4], v[6], E);
    bfly4(v[1], v[3], v[5], v[7], O);
    const cpx<R> t1 = {c * (O[1].x + O[1].y), c * (O[1].y - O[1].x)};
    const cpx<R> t2 = {O[2].y, -O[2].x};
    const cpx<R> t3 = {c * (O[3].y - O[3].x), -(c * (O[3].x + O[3].y))};
    X[0] = cadd(E[0], O[0]);
    X[4] = csub(E[0], O[0]);
    X[1] = cadd(E[1], t1);
    X[5] = csub(E[1], t1);
    X[2] = cadd(E[2], t2);
    X[6] = csub(E[2], t2);
    X[3] = cadd(E[3], t3);
    X[7] = csub(E[3], t3);
}
template <typename R, typename T>
__device__ __forceinline__ cpx<R> twid(const cpx<T> *tw, long long i) {
    const cpx<T> t = tw[i];
    return {(R)t.x, (R)t.y};
}

// One Stockham pass over `lines` lines of length n held in src (line-major),
// writing dst.  Ns = product of the radices already applied.
template <typename R, typename T>
static __device__ void stockham_stage(const cpx<R> *src, cpx<R> *dst, int lines, int n, int p, int Ns, const cpx<T> *tw) {
    typedef cpx<R> C;
    const int m = n / p;
    const int total = lines * m;
    const int twstep_k = n / (Ns * p);  // twiddle W_{Ns p}^{r k} = tw[r k twstep_k]
    const int twstep_q = m;             // W_p^{r q} = tw[r q (n/p)]
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int l = idx / m, j = idx - l * m;
        const int k = j % Ns;
        const C *s = src + (long long)l * n;
        C *d = dst + (long long)l * n;
        const int obase = (j / Ns) * Ns * p + k;
        if (p <= 8) {
            C v[8];
#pragma unroll
            for (int r = 0; r < 8; r++) {
                if (r < p) {
                    C a = s[j + r * m];
                    if (r > 0 && k > 0) a = cmul(a, twid<R, T>(tw, (long long)r * k * twstep_k % n));
                    v[r] = a;
                }
            }
            if (p == 2) {
                d[obase] = cadd(v[0], v[1]);
                d[obase + Ns] = csub(v[0], v[1]);
            } else if (p == 4) {
                C X[4];
                bfly4(v[0], v[1], v[2], v[3], X);
#pragma unroll
                for (int q = 0; q < 4; q++) d[obase + q * Ns] = X[q];
            } else if (p == 8) {
                C X[8];
                bfly8(v, X);
#pragma unroll
                for (int q = 0; q < 8; q++) d[obase + q * Ns] = X[q];
            } else {
                for (int q = 0; q < p; q++) {
                    C acc = v[0];
                    for (int r = 1; r < p; r++) acc = cadd(acc, cmul(v[r], twid<R, T>(tw, (long long)((r * q) % p) * twstep_q)));
                    d[obase + q * Ns] = acc;
                }
            }
        } else {
            for (int q = 0; q < p; q++) {
                C acc = s[j];
                for (int r = 1; r < p; r++) {
                    C a = s[j + r * m];
                    if (k > 0) a = cmul(a, twid<R, T>(tw, (long long)r * k * twstep_k % n));
                    acc = cadd(acc, cmul(a, twid<R, T>(tw, (long long)((r * q) % p) * twstep_q)));
                }
                d[obase + q * Ns] = acc;
            }
        }
    }
}

// returns which buffer (0 or 1) holds the result
template <typename R, typename T>
static __device__ int stockham(cpx<R> *b0, cpx<R> *b1, int lines, const FFTPlan &P, const cpx<T> *tw) {
    cpx<R> *src = b0, *dst = b1;
    int Ns = 1, cur = 0;
    for (int s = 0; s < P.nstages; s++) {
        stockham_stage(src, dst, lines, P.n, P.radix[s], Ns, tw);
        __syncthreads();
        Ns *= P.radix[s];
        cpx<R> *t = src;
        src = dst;
        dst = t;
        cur ^= 1;
    }
    return cur;
}

}  // namespace wc
