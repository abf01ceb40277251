// TEST INFRASTRUCTURE ONLY (oracle). Not part of the shipped GPU path.
//
// Double-precision complex DFT for any length n, written for this project.
// Used in two places, both CPU-side checkers:
//   * oracle/ref_shim/fftw_shim.cpp: stands in for the 5 FFTW3 symbols that the
//     reference calls in ImageMatrix::fft2 (src/cmatrix.cpp:1128-1160), so the
//     unmodified reference sources link without libfftw3;
//   * oracle/wc_oracle.cpp: the oracle restatement of ImageMatrix::fft2.
//
// Algorithm: recursive mixed-radix decimation in time (Cooley-Tukey).  n is
// factored into 4s, 2s, then odd primes; each stage combines p interleaved
// sub-transforms with a direct p-point butterfly, so a prime length p costs
// O(p^2) (a plain DFT).  Twiddles come from one exact table
// w[k] = exp(-2*pi*i*k/n), indexed modulo n, so the result is accurate to a
// few ulps times log(n) for every n.
#pragma once
#include <cmath>
#include <complex>
#include <vector>

namespace wcfft {

typedef std::complex<double> cd;

struct Plan1D {
    int n = 0;
    std::vector<int> radices;   // product == n
    std::vector<cd> tw;         // tw[k] = exp(-2 pi i k / n)
    explicit Plan1D(int n_) : n(n_) {
        int m = n;
        while (m % 4 == 0) { radices.push_back(4); m /= 4; }
        while (m % 2 == 0) { radices.push_back(2); m /= 2; }
        for (int p = 3; (long)p * p <= m; p += 2)
            while (m % p == 0) { radices.push_back(p); m /= p; }
        if (m > 1) radices.push_back(m);
        tw.resize(n > 0 ? n : 1);
        const double two_pi = 6.283185307179586476925286766559;
        for (int k = 0; k < n; k++) {
            double a = two_pi * (double)k / (double)n;
            tw[k] = cd(std::cos(a), -std::sin(a));
        }
    }

    // out[k] = sum_j in[j*stride] * w^(j*k), recursion over radices[level..]
    void rec(const cd *in, long stride, cd *out, int len, int level, long tw_step,
             std::vector<cd> &scratch) const {
        if (len == 1) { out[0] = in[0]; return; }
        const int p = radices[level];
        const int m = len / p;
        for (int r = 0; r < p; r++)
            rec(in + r * stride, stride * p, out + (long)r * m, m, level + 1, tw_step * p, scratch);
        // combine: X[k + q*m] = sum_r w_len^{r (k + q m)} * Y_r[k]
        if ((int)scratch.size() < p) scratch.resize(p);
        std::vector<cd> y(p);
        for (int k = 0; k < m; k++) {
            for (int r = 0; r < p; r++) {
                long e = ((long)r * k * tw_step) % n;
                y[r] = out[(long)r * m + k] * tw[e];
            }
            for (int q = 0; q < p; q++) {
                cd s(0.0, 0.0);
                for (int r = 0; r < p; r++) {
                    long e = ((long)r * q * m % len) * tw_step % n;
                    s += y[r] * tw[e];
                }
                scratch[q] = s;
            }
            for (int q = 0; q < p; q++) out[k + (long)q * m] = scratch[q];
        }
    }

    void forward(const cd *in, long stride, cd *out) const {
        std::vector<cd> scratch;
        if (n <= 0) return;
        rec(in, stride, out, n, 0, 1, scratch);
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
