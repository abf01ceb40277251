// TEST INFRASTRUCTURE ONLY (oracle). Not part of the shipped GPU path.
//
// Double-precision complex DFT for any length n, written for this project.
// Used in two places, both CPU-side checkers:
//   * oracle/ref_shim/fftw_shim.cpp: stands in for the 5 FFTW3 symbols that the
//     reference calls in ImageMatrix::fft2 (src/cmatrix.cpp:1128-1160), so the
//     unmodified reference sources link without libfftw3;
//   * oracle/wc_oracle.cpp: the oracle restatement of ImageMatrix::fft2.
//
// The reference leaves the DFT to FFTW (FFTW_MEASURE: the plan, and so the
// rounding, is chosen at run time), so no particular rounding of the DFT is
// the reference's.  This one is a Stockham autosort FFT with the radix order
// 8, 4, 2, then odd primes, twiddles w[k] = (cos(2 pi k / n), -sin(2 pi k / n))
// from the host libm, and every complex product and sum formed as
// (a.x b.x - a.y b.y, a.x b.y + a.y b.x) with separate roundings (this file is
// compiled with -ffp-contract=off).  Radices 2, 4 and 8 use butterflies (the
// radix-8 one as two radix-4 butterflies and the factors 1, (1-i)/sqrt2, -i,
// -(1+i)/sqrt2, sqrt2/2 = 0.70710678118654752440 rounded once); an odd prime
// p is a direct p-point DFT over the table's twiddles.  The GPU's Fourier node
// performs the same operations in the same order, so the two agree bit for
// bit and the integer features of Fourier-derived planes (GLCMs, histograms)
// can be compared exactly; against FFTW both agree to ~1e-12.
#pragma once
#include <cmath>
#include <complex>
#include <vector>

namespace wcfft {

typedef std::complex<double> cd;

struct cx {
    double x, y;
};
static inline cx cx_mul(cx a, cx b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
static inline cx cx_add(cx a, cx b) { return {a.x + b.x, a.y + b.y}; }
static inline cx cx_sub(cx a, cx b) { return {a.x - b.x, a.y - b.y}; }
static const double kSqrtHalf = 0.70710678118654752440;

// radix-4 butterfly, W = -i: X0 = a0 + a2, X1 = a1 - i a3, X2 = a0 - a2, X3 = a1 + i a3
// with a0 = v0 + v2, a1 = v0 - v2, a2 = v1 + v3, a3 = v1 - v3
static inline void bfly4(cx v0, cx v1, cx v2, cx v3, cx *X) {
    const cx a0 = cx_add(v0, v2), a1 = cx_sub(v0, v2), a2 = cx_add(v1, v3), a3 = cx_sub(v1, v3);
    X[0] = cx_add(a0, a2);
    X[1] = {a1.x + a3.y, a1.y - a3.x};
    X[2] = cx_sub(a0, a2);
    X[3] = {a1.x - a3.y, a1.y + a3.x};
}
// radix-8 butterfly: E = DFT4 of the even inputs, O = DFT4 of the odd ones,
// X_q = E_q + W8^q O_q and X_{q+4} = E_q - W8^q O_q, W8 = (1 - i) / sqrt2
static inline void bfly8(const cx *v, cx *X) {
    cx E[4], O[4];
    bfly4(v[0], v[2], v[4], v[6], E);
    bfly4(v[1], v[3], v[5], v[7], O);
    const cx t1 = {kSqrtHalf * (O[1].x + O[1].y), kSqrtHalf * (O[1].y - O[1].x)};
    const cx t2 = {O[2].y, -O[2].x};
    const cx t3 = {kSqrtHalf * (O[3].y - O[3].x), -(kSqrtHalf * (O[3].x + O[3].y))};
    X[0] = cx_add(E[0], O[0]);
    X[4] = cx_sub(E[0], O[0]);
    X[1] = cx_add(E[1], t1);
    X[5] = cx_sub(E[1], t1);
    X[2] = cx_add(E[2], t2);
    X[6] = cx_sub(E[2], t2);
    X[3] = cx_add(E[3], t3);
    X[7] = cx_sub(E[3], t3);
}

struct Plan1D {
    int n = 0;
    std::vector<int> radices;  // product == n
    std::vector<cx> tw;        // tw[k] = exp(-2 pi i k / n)
    explicit Plan1D(int n_) : n(n_) {
        int m = n;
        while (m % 8 == 0) { radices.push_back(8); m /= 8; }
        while (m % 4 == 0) { radices.push_back(4); m /= 4; }
        while (m % 2 == 0) { radices.push_back(2); m /= 2; }
        for (int p = 3; (long)p * p <= m; p += 2)
            while (m % p == 0) { radices.push_back(p); m /= p; }
        if (m > 1) radices.push_back(m);
        tw.resize(n > 0 ? n : 1);
        const double two_pi = 6.283185307179586476925286766559;
        for (int k = 0; k < n; k++) {
            double a = two_pi * (double)k / (double)n;
            tw[k] = {std::cos(a), -std::sin(a)};
        }
    }

    // one Stockham pass of radix p; Ns = product of the radices already applied
    void stage(const cx *src, cx *dst, int p, int Ns) const {
        const int m = n / p;
        const int twstep_k = n / (Ns * p), twstep_q = m;
        std::vector<cx> v(p);
        for (int j = 0; j < m; j++) {
            const int k = j % Ns;
            const int obase = (j / Ns) * Ns * p + k;
            for (int r = 0; r < p; r++) {
                cx a = src[j + r * m];
                if (r > 0 && k > 0) a = cx_mul(a, tw[(long long)r * k * twstep_k % n]);
                v[r] = a;
            }
            if (p == 2) {
                dst[obase] = cx_add(v[0], v[1]);
                dst[obase + Ns] = cx_sub(v[0], v[1]);
            } else if (p == 4 || p == 8) {
                cx X[8];
                if (p == 4) bfly4(v[0], v[1], v[2], v[3], X);
                else bfly8(v.data(), X);
                for (int q = 0; q < p; q++) dst[obase + q * Ns] = X[q];
            } else {
                for (int q = 0; q < p; q++) {
                    cx acc = v[0];
                    for (int r = 1; r < p; r++) acc = cx_add(acc, cx_mul(v[r], tw[(long long)((r * q) % p) * twstep_q]));
                    dst[obase + q * Ns] = acc;
                }
            }
        }
    }

    void forward(const cd *in, long stride, cd *out) const {
        if (n <= 0) return;
        std::vector<cx> b0(n), b1(n);
        for (int i = 0; i < n; i++) b0[i] = {in[(long)i * stride].real(), in[(long)i * stride].imag()};
        cx *src = b0.data(), *dst = b1.data();
        int Ns = 1;
        for (int p : radices) {
            stage(src, dst, p, Ns);
            Ns *= p;
            cx *t = src;
            src = dst;
            dst = t;
        }
        for (int i = 0; i < n; i++) out[i] = cd(src[i].x, src[i].y);
    }
};

// Full 2-D forward DFT of a real n0 x n1 array (row-major, index [i*n1 + j]):
// X[u][v] = sum_{i,j} a[i][j] exp(-2 pi i (u i / n0 + v j / n1)).
// Rows (length n1) first, then columns (length n0).
inline void dft2_real(const double *a, int n0, int n1, std::vector<cd> &X) {
    X.assign((size_t)n0 * n1, cd(0, 0));
    Plan1D p1(n1), p0(n0);
    std::vector<cd> row(n1), rout(n1), col(n0), cout_(n0);
    for (int i = 0; i < n0; i++) {
        for (int j = 0; j < n1; j++) row[j] = cd(a[(size_t)i * n1 + j], 0.0);
        p1.forward(row.data(), 1, rout.data());
        for (int j = 0; j < n1; j++) X[(size_t)i * n1 + j] = rout[j];
    }
    for (int j = 0; j < n1; j++) {
        for (int i = 0; i < n0; i++) col[i] = X[(size_t)i * n1 + j];
        p0.forward(col.data(), 1, cout_.data());
        for (int i = 0; i < n0; i++) X[(size_t)i * n1 + j] = cout_[i];
    }
}

}  // namespace wcfft
