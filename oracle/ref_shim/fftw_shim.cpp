// TEST INFRASTRUCTURE ONLY: lets the unmodified reference sources link without
// libfftw3.  Implements exactly the five FFTW3 entry points the reference
// calls from ImageMatrix::fft2 (src/cmatrix.cpp:1128-1160), on top of the
// project's own DFT in oracle/fft_cpu.h.  The declarations come from the
// FFTW3 header the reference vendors (src/transforms/fft/bcb_fftw3/fftw3.h).
#include <cstdlib>
#include <cstring>
#include <vector>
#include "transforms/fft/bcb_fftw3/fftw3.h"
#include "../fft_cpu.h"

struct fftw_plan_s {
    int n0, n1;
    double *in;
    fftw_complex *out;
};

extern "C" {

void *fftw_malloc(size_t n) { return std::malloc(n ? n : 1); }
void fftw_free(void *p) { std::free(p); }

fftw_plan fftw_plan_dft_r2c_2d(int nx, int ny, double *in, fftw_complex *out, unsigned) {
    fftw_plan p = new fftw_plan_s;
    p->n0 = nx; p->n1 = ny; p->in = in; p->out = out;
    return p;
}

// r2c layout: out[i*(n1/2+1) + j] = X[i][j] for 0 <= j <= n1/2.
void fftw_execute(const fftw_plan p) {
    std::vector<wcfft::cd> X;
    wcfft::dft2_real(p->in, p->n0, p->n1, X);
    const int h = p->n1 / 2 + 1;
    for (int i = 0; i < p->n0; i++)
        for (int j = 0; j < h; j++) {
            p->out[(size_t)i * h + j][0] = X[(size_t)i * p->n1 + j].real();
            p->out[(size_t)i * h + j][1] = X[(size_t)i * p->n1 + j].imag();
        }
}

void fftw_destroy_plan(fftw_plan p) { delete p; }

}  // extern "C"
