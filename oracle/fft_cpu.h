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
// 8, 4, 2, then odd primes (a prime p costs O(p) per output), twiddles
// w[k] = (cos(2 pi k / n), -sin(2 pi k / n)) from the host libm, and every
// complex product and sum formed as (a.x b.x - a.y b.y, a.x b.y + a.y b.x) with
// separate roundings (this file is compiled with -ffp-contract=off).  The GPU's
// Fourier node performs the same operations in the same order, so the two
// agree bit for bit and the integer features of Fourier-derived planes (GLCMs,
// histograms) can be compared exactly; against FFTW both agree to ~1e-12.
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
            for (int q = 0; q < p; q++) {
                cx acc = v[0];
                for (int r = 1; r < p; r++) acc = cx_add(acc, cx_mul(v[r], tw[(long long)((r * q) % p) * twstep_q]));
                dst[obase + q * Ns] = acc;
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
