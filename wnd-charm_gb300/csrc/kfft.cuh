// Stockham mixed-radix DFT of several lines held in shared memory (any
// length; radix-p stages with host-computed FP64 twiddles
// tw[k] = exp(-2 pi i k / n)).  Shared by the Fourier transform node and the
// Gabor FFT convolution; templated on the element type (FP64 form, and FP32
// for the mixed form's Gabor filtering) and on the twiddles' type (FP64, or
// the FP64 twiddles rounded to FP32 once, in shared memory).
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
            for (int q = 0; q < p; q++) {
                C acc = v[0];
                for (int r = 1; r < p; r++) acc = cadd(acc, cmul(v[r], twid<R, T>(tw, (long long)((r * q) % p) * twstep_q)));
                d[obase + q * Ns] = acc;
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
