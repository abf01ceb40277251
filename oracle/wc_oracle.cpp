// TEST INFRASTRUCTURE ONLY: CPU oracle (restatement) of the WND-CHARM hot path.
// See wc_oracle.h for who may use it.  Reference citations are paths inside
// the wnd-charm source tree (src/...).  Arithmetic follows the reference's
// order of operations where it decides a bin, a threshold or a label; where it
// only changes the last bits of a mean (stats accumulated in a different pixel
// order) the restatement uses raster order.
#include "wc_oracle.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <chrono>
#include <thread>
#include <vector>
#include <atomic>
#include <functional>
#include <mutex>

#include "fft_cpu.h"

namespace wco {

static const double kINF = 10E200;     // src/cmatrix.h:45
static const double kPI_Z = 3.14159265358979323846264338328;  // src/textures/zernike/zernike.cpp:38

// ---------------------------------------------------------------- moments
// Moments2 / Moments4: src/statistics/Moments.h:10-107 (Welford updates,
// values that are NaN or beyond +-FLT_MAX are skipped).
struct Moments2 {
    double mn, mx, mean, M2;
    size_t n;
    Moments2() { reset(); }
    void reset() { mean = M2 = 0.0; mn = DBL_MAX; mx = -DBL_MAX; n = 0; }
    double add(double x) {
        if (std::isnan(x) || x > FLT_MAX || x < -FLT_MAX) return x;
        size_t n1 = n;
        n = n + 1;
        double delta = x - mean;
        double delta_n = delta / n;
        double term1 = delta * delta_n * n1;
        mean = mean + delta_n;
        M2 += term1;
        if (x > mx) mx = x;
        if (x < mn) mn = x;
        return x;
    }
    double std_() const { return n > 2 ? std::sqrt(M2 / (n - 1)) : 0.0; }
    double var() const { return n > 2 ? (M2 / (n - 1)) : 0.0; }
};

struct Moments4 {
    double mn, mx, mean, M2, M3, M4;
    size_t n;
    Moments4() { reset(); }
    void reset() { mean = M2 = M3 = M4 = 0.0; mn = FLT_MAX; mx = -FLT_MAX; n = 0; }
    void add(double x) {
        if (std::isnan(x) || x > FLT_MAX || x < -FLT_MAX) return;
        size_t n1 = n;
        n = n + 1;
        double delta = x - mean;
        double delta_n = delta / n;
        double delta_n2 = delta_n * delta_n;
        double term1 = delta * delta_n * n1;
        mean = mean + delta_n;
        M4 = M4 + term1 * delta_n2 * (n * n - 3 * n + 3) + 6 * delta_n2 * M2 - 4 * delta_n * M3;
        M3 = M3 + term1 * delta_n * (n - 2) - 3 * delta_n * M2;
        M2 = M2 + term1;
        if (x > mx) mx = x;
        if (x < mn) mn = x;
    }
    double std_() const { return n > 2 ? std::sqrt(M2 / (n - 1)) : 0.0; }
    double skew() const { return n > 3 ? (std::sqrt((double)n) * M3) / std::pow(M2, 1.5) : 0.0; }
    double kurt() const { return n > 4 ? (n * M4) / (M2 * M2) : 0.0; }
    void vec(double *z) const { z[0] = mean; z[1] = std_(); z[2] = skew(); z[3] = kurt(); }
};

// ---------------------------------------------------------------- image
// The pixel plane of ImageMatrix (src/cmatrix.h:164-339): row-major doubles.
struct Img {
    int w = 0, h = 0;
    std::vector<double> p;
    std::vector<unsigned char> hsv;  // colour plane (h, s, v per pixel) of an RGB image, else empty
    Img() {}
    Img(int w_, int h_) : w(w_), h(h_), p((size_t)w_ * h_, 0.0) {}
    double &at(int y, int x) { return p[(size_t)y * w + x]; }
    double at(int y, int x) const { return p[(size_t)y * w + x]; }
    size_t n() const { return p.size(); }
};

static Moments2 stats_of(const Img &im) {
    Moments2 s;
    for (double v : im.p) s.add(v);
    return s;
}

// bin = (unsigned long)((v - lo) * scale), clamped to nbins - 1
// (src/cmatrix.cpp:1097-1099).  A NaN goes to the last bin, as the x86-64
// build of the reference converts it (so the oracle gives the same answer on
// aarch64 hosts, where the raw conversion would give 0).
static inline unsigned long bin_of(double v, double lo, double scale, unsigned long nbins) {
    double t = (v - lo) * scale;
    if (!(t < (double)nbins)) return nbins - 1;
    if (t < 0) return 0;
    unsigned long b = (unsigned long)t;
    return b >= nbins ? nbins - 1 : b;
}

// ImageMatrix::histogram, src/cmatrix.cpp:1069-1103 (bins over [lo, hi]).
static void histogram(const double *v, size_t n, int nbins, double lo, double hi, double *bins) {
    double scale = (hi - lo > 0) ? (double)nbins / double(hi - lo) : 0;
    for (int b = 0; b < nbins; b++) bins[b] = 0;
    for (size_t a = 0; a < n; a++) bins[bin_of(v[a], lo, scale, nbins)] += 1.0;
}

// ImageMatrix::get_median, src/cmatrix.cpp:780-800.
static double median_of(const std::vector<double> &src) {
    std::vector<double> v(src);
    size_t num = v.size(), half = num / 2;
    if (num == 0) return 0;
    double med;
    if (num % 2 == 0) {
        std::nth_element(v.begin(), v.begin() + half, v.end());
        med = v[half];
        std::nth_element(v.begin(), v.begin() + half - 1, v.end());
        med += v[half - 1];
        med /= 2.0;
    } else {
        std::nth_element(v.begin(), v.begin() + half, v.end());
        med = v[half];
    }
    return med;
}

// ImageMatrix::Otsu(dynamic_range=true), src/cmatrix.cpp:1520-1570.
static double otsu(const Img &im, double mn, double mx) {
    const int L = 1024;
    std::vector<double> hist(L), omega(L), myu(L);
    histogram(im.p.data(), im.n(), L, mn, mx, hist.data());
    double wh = (double)im.w * im.h;
    omega[0] = hist[0] / wh;
    myu[0] = 0.0;
    for (int i = 1; i < L; i++) {
        omega[i] = omega[i - 1] + (hist[i] / wh);
        myu[i] = myu[i - 1] + i * (hist[i] / wh);
    }
    int thr = 0;
    double max_sigma = 0.0;
    for (int i = 0; i < L - 1; i++) {
        double s;
        if (omega[i] != 0.0 && omega[i] != 1.0)
            s = std::pow(myu[L - 1] * omega[i] - myu[i], 2) / (omega[i] * (1.0 - omega[i]));
        else
            s = 0.0;
        if (s > max_sigma) { max_sigma = s; thr = i; }
    }
    return (((double)thr / (double)(L - 1)) * (mx - mn)) + mn;
}

// ---------------------------------------------------------------- transforms
// ImageMatrix::fft2, src/cmatrix.cpp:1107-1160: |2-D DFT| of the image, the
// rows y >= H/2+1 copied from their Hermitian mirrors.
static Img fourier(const Img &in) {
    const int W = in.w, H = in.h;
    std::vector<double> a((size_t)W * H);
    for (int x = 0; x < W; x++)
        for (int y = 0; y < H; y++) a[(size_t)H * x + y] = in.at(y, x);
    std::vector<wcfft::cd> X;
    wcfft::dft2_real(a.data(), W, H, X);
    Img out(W, H);
    const int hh = H / 2 + 1;
    for (int x = 0; x < W; x++)
        for (int y = 0; y < hh; y++) {
            wcfft::cd c = X[(size_t)x * H + y];
            out.at(y, x) = std::sqrt(std::pow(c.real(), 2) + std::pow(c.imag(), 2));
        }
    for (int y = hh; y < H; y++) out.at(y, 0) = out.at(H - y, 0);
    for (int y = hh; y < H; y++)
        for (int x = 1; x < W; x++) out.at(y, x) = out.at(H - y, W - x);
    return out;
}

// TNx, src/transforms/chebyshev.cpp:39-80: T[a*N + j] = cos(j * acos(x_a)),
// T[a*N + 0] = 1.
static std::vector<double> cheb_T(int len, int N) {
    std::vector<double> T((size_t)len * N);
    for (int a = 0; a < len; a++) {
        double x = 2 * (double)(a + 1) / (double)len - 1;  // chebyshev.cpp:128-129
        double ac = (std::fabs(x) > 1) ? 0 : std::acos(x);
        for (int j = 0; j < N; j++) T[(size_t)a * N + j] = std::cos(ac * j);
        T[(size_t)a * N + 0] = 1;
    }
    return T;
}

// getChCoeff1D, src/transforms/chebyshev.cpp:82-102.
static void cheb_1d(const double *f, double *out, const std::vector<double> &T, int N, int width) {
    for (int jj = 0; jj < N; jj++) {
        double s = 0;
        for (int a = 0; a < width; a++) {
            double tj = T[(size_t)a * N + jj];
            tj = (jj == 0) ? tj / (double)width : tj * 2 / (double)width;
            s += f[a] * tj / 2;
        }
        out[jj] = s;
    }
}

// Chebyshev2D + ImageMatrix::ChebyshevTransform,
// src/transforms/chebyshev.cpp:118-165, src/cmatrix.cpp:1203-1222.
static Img chebyshev(const Img &in, int N) {
    const int W = in.w, H = in.h;
    if (N < 2) N = std::min(W, H);
    std::vector<double> TW = cheb_T(W, N);
    std::vector<double> mid((size_t)H * N), tr((size_t)N * H), out((size_t)N * N);
    for (int y = 0; y < H; y++) cheb_1d(&in.p[(size_t)y * W], &mid[(size_t)y * N], TW, N, W);
    for (int j = 0; j < N; j++)
        for (int i = 0; i < H; i++) tr[(size_t)j * H + i] = mid[(size_t)i * N + j];
    std::vector<double> TH = (H != W) ? cheb_T(H, N) : TW;
    for (int j = 0; j < N; j++) cheb_1d(&tr[(size_t)j * H], &out[(size_t)j * N], TH, N, H);
    const int oh = std::min(H, N);
    Img o(N, oh);
    for (int y = 0; y < oh; y++)
        for (int x = 0; x < N; x++) o.at(y, x) = out[(size_t)y * N + x];
    return o;
}

// Symlet-5 analysis filters, src/transforms/wavelet/Symlet5.cpp:15-17.
static const double kSymLo[10] = {0.027333068345077982, 0.029519490925774643, -0.039134249302383094,
    0.1993975339773936, 0.72340769040242059, 0.63397896345821192, 0.016602105764522319,
    -0.17532808990845047, -0.021101834024758855, 0.019538882735286728};
static const double kSymHi[10] = {-0.019538882735286728, -0.021101834024758855, 0.17532808990845047,
    0.016602105764522319, -0.63397896345821192, 0.72340769040242059, -0.1993975339773936,
    -0.039134249302383094, -0.029519490925774643, 0.027333068345077982};

// downsampling_convolution in MODE_ZEROPAD with step 2,
// src/transforms/wavelet/convolution.cpp:86-325: out[o] = sum_j f[j]*x[i-j],
// i = 2o+1, over the taps that land inside the input, j ascending.
static void dwt_zeropad(const double *x, int N, const double *f, double *out, int outlen) {
    const int F = 10;
    for (int o = 0; o < outlen; o++) {
        int i = 2 * o + 1;
        double s = 0;
        for (int j = 0; j < F; j++) {
            int k = i - j;
            if (k >= 0 && k < N) s += x[k] * f[j];
        }
        out[o] = s;
    }
}

// ImageMatrix::Symlet5Transform + Wavelet::transform2D (one level),
// src/cmatrix.cpp:1244-1268, src/transforms/wavelet/Wavelet.cpp:136-434.
static Img wavelet(const Img &in) {
    const int X = in.w, Y = in.h;
    const int ox = (X + 10 - 1) / 2, oy = (Y + 10 - 1) / 2;  // dwt_buffer_length
    // pass 1: along y for every column x
    std::vector<double> g1((size_t)X * oy), g2((size_t)X * oy), col(Y);
    for (int x = 0; x < X; x++) {
        for (int y = 0; y < Y; y++) col[y] = in.at(y, x);
        dwt_zeropad(col.data(), Y, kSymLo, &g1[(size_t)x * oy], oy);
        dwt_zeropad(col.data(), Y, kSymHi, &g2[(size_t)x * oy], oy);
    }
    // pass 2: along x for every output row j
    Img o(2 * ox, 2 * oy);
    std::vector<double> r1(X), r2(X), a1(ox), d1(ox), a2(ox), d2(ox);
    for (int j = 0; j < oy; j++) {
        for (int x = 0; x < X; x++) { r1[x] = g1[(size_t)x * oy + j]; r2[x] = g2[(size_t)x * oy + j]; }
        dwt_zeropad(r1.data(), X, kSymLo, a1.data(), ox);
        dwt_zeropad(r1.data(), X, kSymHi, d1.data(), ox);
        dwt_zeropad(r2.data(), X, kSymLo, a2.data(), ox);
        dwt_zeropad(r2.data(), X, kSymHi, d2.data(), ox);
        for (int x = 0; x < ox; x++) {
            o.at(j, x) = d2[x];             // detail(y), detail(x)
            o.at(oy + j, x) = a2[x];        // detail(y), approx(x)
            o.at(j, ox + x) = d1[x];        // approx(y), detail(x)
            o.at(oy + j, ox + x) = a1[x];   // approx(y), approx(x)
        }
    }
    return o;
}

// ImageMatrix::EdgeTransform, src/cmatrix.cpp:1294-1311.
static Img edge(const Img &in) {
    const int W = in.w, H = in.h;
    Img o(W, H);
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            double mxx = 0, myy = 0;
            if (y > 0 && y < H - 1)
                myy = std::max(std::fabs(in.at(y, x) - in.at(y - 1, x)), std::fabs(in.at(y, x) - in.at(y + 1, x)));
            if (x > 0 && x < W - 1)
                mxx = std::max(std::fabs(in.at(y, x) - in.at(y, x - 1)), std::fabs(in.at(y, x) - in.at(y, x + 1)));
            o.at(y, x) = std::max(mxx, myy);
        }
    return o;
}

// ImageMatrix::Downsample (grayscale part), src/cmatrix.cpp:579-720.
static Img downsample(const Img &in, double xr, double yr) {
    if (xr > 1) xr = 1;
    if (yr > 1) yr = 1;
    double dx = 1 / xr, dy = 1 / yr;
    if (dx == 1 && dy == 1) return in;
    const unsigned ow = in.w, oh = in.h;
    unsigned nw = (unsigned)(xr * in.w), nh = (unsigned)(yr * in.h);
    Img cp(ow, oh);
    for (unsigned ny = 0; ny < oh; ny++) {
        double x = 0;
        unsigned nx = 0;
        while (x < ow) {
            double s = 0, frac;
            unsigned a = (unsigned)(std::floor(x));
            frac = std::ceil(x) - x;
            if (frac > 0 && a < ow) s += in.at(ny, a) * frac;
            for (a = (unsigned)(std::ceil(x)); a < std::floor(x + dx); a++)
                if (a < ow) s += in.at(ny, a);
            frac = x + dx - std::floor(x + dx);
            if (frac > 0 && a < ow) s += in.at(ny, a) * frac;
            cp.at(ny, nx) = s / (dx);
            x += dx;
            nx++;
        }
    }
    Img o(nw, nh);
    for (unsigned nx = 0; nx < nw; nx++) {
        double y = 0;
        unsigned ny = 0;
        while (y < oh) {
            double s = 0, frac;
            unsigned a = (unsigned)(std::floor(y));
            frac = std::ceil(y) - y;
            if (frac > 0 && a < oh) s += cp.at(a, nx) * frac;
            for (a = (unsigned)(std::ceil(y)); a < std::floor(y + dy); a++)
                if (a < oh) s += cp.at(a, nx);
            frac = y + dy - std::floor(y + dy);
            if (frac > 0 && a < oh) s += cp.at(a, nx) * frac;
            if (nx < nw && ny < nh) o.at(ny, nx) = s / dy;
            y += dy;
            ny++;
        }
    }
    return o;
}

// ---------------------------------------------------------------- features
// Chebyshev-Fourier: ChebyshevFourierCoefficients::execute,
// ImageMatrix::ChebyshevFourierTransform2D, ChebyshevFourier2D, ChebPol
// (src/FeatureAlgorithms.cpp:54-69, src/cmatrix.cpp:1227-1240,
//  src/transforms/ChebyshevFourier.cpp:42-160).
static void f_cheb_fourier(const Img &src, double *out) {
    Img ds;
    const Img *imp = &src;
    if ((long)src.w * src.h > 300L * 300) {
        double r = std::min(300.0 / (double)src.w, 300.0 / (double)src.h);
        ds = downsample(src, r, r);
        imp = &ds;
    }
    const Img &im = *imp;
    unsigned long N = 11;
    const unsigned long m = im.h, n = im.w;
    std::vector<double> img, r, f;
    img.reserve(m * n);
    const double tn = 2.0 / ((double)n - 1), tm = 2.0 / ((double)m - 1);
    for (unsigned long x = 0; x < n; x++) {
        double xi = -1.0 + (double)x * tn, x2 = std::pow(xi, 2);
        for (unsigned long y = 0; y < m; y++) {
            double yi = -1.0 + (double)y * tm;
            double rr = std::sqrt(x2 + std::pow(yi, 2));
            if (rr < 1) {
                img.push_back(im.at(y, x));
                r.push_back(rr);
                f.push_back(-1 * std::atan2(yi, xi));
            }
        }
    }
    unsigned long Nmax = (unsigned long)((std::min(m, n) - 1) / 2);
    if (N > Nmax) N = Nmax;
    const unsigned long NN = 2 * N + 1;
    std::vector<double> Tn(NN), sr(NN * NN, 0.0), si(NN * NN, 0.0);
    for (size_t k = 0; k < img.size(); k++) {
        double ri = r[k], fi = f[k], ii = img[k];
        double xx = ri * 2 - 1;
        if (xx < -1) xx = -1;
        if (xx > 1) xx = 1;
        double ac = std::acos(xx);
        for (unsigned long a = 0; a < NN; a++) Tn[a] = std::cos(a * ac);
        Tn[0] = 0.5;
        unsigned long ind = 0;
        for (unsigned long im_ = 1; im_ <= NN; im_++) {
            long mf = (long)im_ - 1 - (long)N;
            double Ft = (mf == 0) ? 0.5 : 1.0;
            double fc = Ft * std::cos(mf * fi), fs = Ft * std::sin(-1 * mf * fi);
            for (unsigned long a = 0; a < NN; a++) {
                sr[ind] += (fc * Tn[a]) * ii;
                si[ind] += (fs * Tn[a]) * ii;
                ind++;
            }
        }
    }
    double mn = kINF, mx = -kINF;
    std::vector<double> c(NN * NN);
    for (size_t a = 0; a < NN * NN; a++) {
        c[a] = std::sqrt(std::pow(sr[a], 2) + std::pow(si[a], 2));
        if (c[a] < mn) mn = c[a];
        if (c[a] > mx) mx = c[a];
    }
    for (int a = 0; a < 32; a++) out[a] = 0;
    if (mx - mn > 0) {
        double sc = 32.0 / double(mx - mn);
        for (size_t a = 0; a < NN * NN; a++) out[bin_of(c[a], mn, sc, 32)] += 1;
    }
}

// Chebyshev Coefficients: ImageMatrix::ChebyshevStatistics2D(N=20, 32 bins),
// src/FeatureAlgorithms.cpp:73-93, src/cmatrix.cpp:1274-1281.
static void f_cheb_coeffs(const Img &im, double *out) {
    int N = 20;
    if (N > std::min(im.w, im.h)) N = std::min(im.w, im.h);
    Img t = chebyshev(im, N);
    Moments2 s = stats_of(t);
    histogram(t.p.data(), t.n(), 32, s.mn, s.mx, out);
}

// Zernike: mb_zernike2D (order 15, rad = min(W,H), centroid-centred),
// src/textures/zernike/zernike.cpp:207-341.
static void f_zernike(const Img &im, double *out) {
    const int L = 15, MAXL = 32;
    const int cols = im.w, rows = im.h;
    const double rad = (double)(im.w < im.h ? im.w : im.h);
    double H1[MAXL][MAXL] = {{0}}, H2[MAXL][MAXL] = {{0}}, H3[MAXL][MAXL] = {{0}};
    for (int n = 0; n < MAXL; n++)
        for (int m = 0; m <= n; m++)
            if (n != m) {
                H3[n][m] = -(double)(4.0 * (m + 2.0) * (m + 1.0)) / (double)((n + m + 2.0) * (n - m));
                H2[n][m] = ((double)(H3[n][m] * (n + m + 4.0) * (n - m - 2.0)) / (double)(4.0 * (m + 3.0))) + (m + 2.0);
                H1[n][m] = ((double)((m + 4.0) * (m + 3.0)) / 2.0) - ((m + 4.0) * H2[n][m]) +
                           ((double)(H3[n][m] * (n + m + 6.0) * (n - m - 4.0)) / 8.0);
            }
    double sum = 0, m10 = 0, m00 = 0, m01 = 0;
    for (int i = 0; i < cols; i++)
        for (int j = 0; j < rows; j++) {
            double I = im.at(j, i);
            sum += I;
            m10 += (i + 1) * I;
            m00 += I;
            m01 += (j + 1) * I;
        }
    double cx = m10 / m00, cy = m01 / m00;
    double AR[MAXL][MAXL], AI[MAXL][MAXL];
    for (int n = 0; n <= L; n++)
        for (int m = 0; m <= n; m++) AR[n][m] = AI[n][m] = 0.0;
    double COST[MAXL], SINT[MAXL], R[MAXL];
    for (int i = 0; i < cols; i++) {
        double x = (i + 1 - cx) / rad;
        for (int j = 0; j < rows; j++) {
            double y = (j + 1 - cy) / rad;
            double r2 = x * x + y * y, r = std::sqrt(r2);
            if (r < DBL_EPSILON || r > 1.0) continue;
            R[0] = 1;
            for (int n = 1; n <= L; n++) R[n] = r * R[n - 1];
            double a = COST[0] = x / r, b = SINT[0] = y / r;
            for (int m = 1; m <= L; m++) {
                COST[m] = a * COST[m - 1] - b * SINT[m - 1];
                SINT[m] = a * SINT[m - 1] + b * COST[m - 1];
            }
            double f = im.at(j, i) / sum;
            double Rnmp2 = 0, Rnm2 = 0, Rnm = 0, Rnmp4 = 0;
            for (int n = 0; n <= L; n++) {
                double ct = (n + 1) * f / kPI_Z;
                double Rn = R[n];
                if (n >= 2) Rnm2 = R[n - 2];
                for (int m = n; m >= 0; m -= 2) {
                    if (m == n) {
                        Rnm = Rn;
                        Rnmp4 = Rn;
                    } else if (m == n - 2) {
                        double Rnnm2 = n * Rn - (n - 1) * Rnm2;
                        Rnm = Rnnm2;
                        Rnmp2 = Rnnm2;
                    } else {
                        Rnm = H1[n][m] * Rnmp4 + (H2[n][m] + (H3[n][m] / r2)) * Rnmp2;
                        Rnmp4 = Rnmp2;
                        Rnmp2 = Rnm;
                    }
                    AR[n][m] += ct * Rnm * COST[m];
                    AI[n][m] -= ct * Rnm * SINT[m];
                }
            }
        }
    }
    int k = 0;
    for (int n = 0; n <= L; n++)
        for (int m = 0; m <= n; m++)
            if ((n - m) % 2 == 0) {
                AR[n][m] *= AR[n][m];
                AI[n][m] *= AI[n][m];
                out[k++] = std::fabs(std::sqrt(AR[n][m] + AI[n][m]));
            }
}

// ---- Haralick (src/textures/haralick/haralick.cpp:12-144 and
//      src/textures/haralick/CVIPtexture.cpp:384-1108)
typedef std::vector<double> Mat;  // Ng x Ng row-major

// Eigen 3.1.2 eigenvalues() of a general real matrix, in the order of the
// quasi-triangular real Schur form: HessenbergDecomposition::_compute
// (src/Eigen/src/Eigenvalues/HessenbergDecomposition.h:292-318, Householder
// reflectors from Householder.h:65-90 and the apply-on-left/right updates),
// RealSchur::compute and helpers (RealSchur.h:204-463) and the eigenvalue read
// out of EigenSolver::compute (EigenSolver.h:351-381).  Only T is formed.
struct EigRes { std::vector<double> re, im; bool ok; };

static void householder_make(const double *v, int n, double *ess, double &tau, double &beta) {
    double tail = 0;
    for (int i = 1; i < n; i++) tail += v[i] * v[i];
    double c0 = v[0];
    if (n == 1 || tail == 0) {
        tau = 0; beta = c0;
        for (int i = 1; i < n; i++) ess[i - 1] = 0;
    } else {
        beta = std::sqrt(c0 * c0 + tail);
        if (c0 >= 0) beta = -beta;
        for (int i = 1; i < n; i++) ess[i - 1] = v[i] / (c0 - beta);
        tau = (beta - c0) / beta;
    }
}

// rows r0..r0+m-1, cols c0..c0+nc-1 of A (ld n):  B = H B with v = [1 ess]
static void hh_left(double *A, int ld, int r0, int m, int c0, int nc, const double *ess, double tau) {
    if (m == 1) {
        for (int c = 0; c < nc; c++) A[(size_t)r0 * ld + c0 + c] *= (1.0 - tau);
        return;
    }
    for (int c = 0; c < nc; c++) {
        double t = 0;
        for (int r = 1; r < m; r++) t += ess[r - 1] * A[(size_t)(r0 + r) * ld + c0 + c];
        t += A[(size_t)r0 * ld + c0 + c];
        A[(size_t)r0 * ld + c0 + c] -= tau * t;
        for (int r = 1; r < m; r++) A[(size_t)(r0 + r) * ld + c0 + c] -= tau * ess[r - 1] * t;
    }
}

// B = B H for rows r0..r0+m-1, cols c0..c0+nc-1
static void hh_right(double *A, int ld, int r0, int m, int c0, int nc, const double *ess, double tau) {
    if (nc == 1) {
        for (int r = 0; r < m; r++) A[(size_t)(r0 + r) * ld + c0] *= (1.0 - tau);
        return;
    }
    for (int r = 0; r < m; r++) {
        double *row = &A[(size_t)(r0 + r) * ld + c0];
        double t = 0;
        for (int c = 1; c < nc; c++) t += row[c] * ess[c - 1];
        t += row[0];
        row[0] -= tau * t;
        for (int c = 1; c < nc; c++) row[c] -= tau * t * ess[c - 1];
    }
}

static EigRes eigen_schur_eigenvalues(Mat A, int n) {
    EigRes res;
    res.ok = true;
    std::vector<double> v(n), ess(n);
    // Hessenberg reduction
    for (int i = 0; i < n - 1; i++) {
        int rem = n - i - 1;
        for (int k = 0; k < rem; k++) v[k] = A[(size_t)(i + 1 + k) * n + i];
        double tau, beta;
        householder_make(v.data(), rem, ess.data(), tau, beta);
        A[(size_t)(i + 1) * n + i] = beta;
        for (int k = 1; k < rem; k++) A[(size_t)(i + 1 + k) * n + i] = ess[k - 1];
        hh_left(A.data(), n, i + 1, rem, i + 1, rem, ess.data(), tau);
        hh_right(A.data(), n, 0, n, i + 1, rem, ess.data(), tau);
    }
    for (int r = 0; r < n; r++)
        for (int c = 0; c < r - 1; c++) A[(size_t)r * n + c] = 0;  // matrixH()
    auto T = [&](int r, int c) -> double & { return A[(size_t)r * n + c]; };
    // real Schur iteration
    int iu = n - 1, iter = 0, totalIter = 0;
    double exshift = 0, norm = 0;
    for (int j = 0; j < n; j++) {
        int s0 = std::max(j - 1, 0);
        double s = 0;
        for (int c = s0; c < n; c++) s += std::fabs(T(j, c));
        norm += s;
    }
    const double eps = DBL_EPSILON;
    const int maxIter = 40 * n;
    if (norm != 0) {
        while (iu >= 0) {
            int il = iu;
            while (il > 0) {
                double s = std::fabs(T(il - 1, il - 1)) + std::fabs(T(il, il));
                if (s == 0.0) s = norm;
                if (std::fabs(T(il, il - 1)) < eps * s) break;
                il--;
            }
            if (il == iu) {
                T(iu, iu) = T(iu, iu) + exshift;
                if (iu > 0) T(iu, iu - 1) = 0;
                iu--;
                iter = 0;
            } else if (il == iu - 1) {
                double p = 0.5 * (T(iu - 1, iu - 1) - T(iu, iu));
                double q = p * p + T(iu, iu - 1) * T(iu - 1, iu);
                T(iu, iu) += exshift;
                T(iu - 1, iu - 1) += exshift;
                if (q >= 0) {
                    double z = std::sqrt(std::fabs(q));
                    double gp = (p >= 0) ? p + z : p - z, gq = T(iu, iu - 1);
                    double c, s;  // JacobiRotation::makeGivens (real), Jacobi.h:206-242
                    if (gq == 0) { c = gp < 0 ? -1 : 1; s = 0; }
                    else if (gp == 0) { c = 0; s = gq < 0 ? 1 : -1; }
                    else if (std::fabs(gp) > std::fabs(gq)) {
                        double t = gq / gp, u = std::sqrt(1 + t * t);
                        if (gp < 0) u = -u;
                        c = 1 / u; s = -t * c;
                    } else {
                        double t = gp / gq, u = std::sqrt(1 + t * t);
                        if (gq < 0) u = -u;
                        s = -1 / u; c = -t * s;
                    }
                    // left with adjoint (c, -s) on rows iu-1, iu; cols iu-1..n-1
                    for (int col = iu - 1; col < n; col++) {
                        double xi = T(iu - 1, col), yi = T(iu, col);
                        T(iu - 1, col) = c * xi + (-s) * yi;
                        T(iu, col) = -(-s) * xi + c * yi;
                    }
                    // right with transpose (c, -s) on cols iu-1, iu; rows 0..iu
                    for (int row = 0; row <= iu; row++) {
                        double xi = T(row, iu - 1), yi = T(row, iu);
                        T(row, iu - 1) = c * xi + (-s) * yi;
                        T(row, iu) = -(-s) * xi + c * yi;
                    }
                    T(iu, iu - 1) = 0;
                }
                if (iu > 1) T(iu - 1, iu - 2) = 0;
                iu -= 2;
                iter = 0;
            } else {
                double sh[3] = {T(iu, iu), T(iu - 1, iu - 1), T(iu, iu - 1) * T(iu - 1, iu)};
                if (iter == 10) {
                    exshift += sh[0];
                    for (int i = 0; i <= iu; i++) T(i, i) -= sh[0];
                    double s = std::fabs(T(iu, iu - 1)) + std::fabs(T(iu - 1, iu - 2));
                    sh[0] = 0.75 * s;
                    sh[1] = 0.75 * s;
                    sh[2] = -0.4375 * s * s;
                }
                if (iter == 30) {
                    double s = (sh[1] - sh[0]) / 2.0;
                    s = s * s + sh[2];
                    if (s > 0) {
                        s = std::sqrt(s);
                        if (sh[1] < sh[0]) s = -s;
                        s = s + (sh[1] - sh[0]) / 2.0;
                        s = sh[0] - sh[2] / s;
                        exshift += s;
                        for (int i = 0; i <= iu; i++) T(i, i) -= s;
                        sh[0] = sh[1] = sh[2] = 0.964;
                    }
                }
                iter++;
                totalIter++;
                if (totalIter > maxIter) break;
                // initFrancisQRStep
                double fv[3] = {0, 0, 0};
                int im;
                for (im = iu - 2; im >= il; --im) {
                    double Tmm = T(im, im), r = sh[0] - Tmm, s = sh[1] - Tmm;
                    fv[0] = (r * s - sh[2]) / T(im + 1, im) + T(im, im + 1);
                    fv[1] = T(im + 1, im + 1) - Tmm - r - s;
                    fv[2] = T(im + 2, im + 1);
                    if (im == il) break;
                    double lhs = T(im, im - 1) * (std::fabs(fv[1]) + std::fabs(fv[2]));
                    double rhs = fv[0] * (std::fabs(T(im - 1, im - 1)) + std::fabs(Tmm) + std::fabs(T(im + 1, im + 1)));
                    if (std::fabs(lhs) < eps * rhs) break;
                }
                // performFrancisQRStep
                for (int k = im; k <= iu - 2; ++k) {
                    bool first = (k == im);
                    double vv[3];
                    if (first) { vv[0] = fv[0]; vv[1] = fv[1]; vv[2] = fv[2]; }
                    else { vv[0] = T(k, k - 1); vv[1] = T(k + 1, k - 1); vv[2] = T(k + 2, k - 1); }
                    double e2[2], tau, beta;
                    householder_make(vv, 3, e2, tau, beta);
                    if (beta != 0) {
                        if (first && k > il) T(k, k - 1) = -T(k, k - 1);
                        else if (!first) T(k, k - 1) = beta;
                        hh_left(A.data(), n, k, 3, k, n - k, e2, tau);
                        hh_right(A.data(), n, 0, std::min(iu, k + 3) + 1, k, 3, e2, tau);
                    }
                }
                {
                    double vv[2] = {T(iu - 1, iu - 2), T(iu, iu - 2)};
                    double e1[1], tau, beta;
                    householder_make(vv, 2, e1, tau, beta);
                    if (beta != 0) {
                        T(iu - 1, iu - 2) = beta;
                        hh_left(A.data(), n, iu - 1, 2, iu - 1, n - iu + 1, e1, tau);
                        hh_right(A.data(), n, 0, iu + 1, iu - 1, 2, e1, tau);
                    }
                }
                for (int i = im + 2; i <= iu; ++i) {
                    T(i, i - 2) = 0;
                    if (i > im + 2) T(i, i - 3) = 0;
                }
            }
        }
    }
    if (totalIter > maxIter) { res.ok = false; return res; }
    res.re.resize(n);
    res.im.resize(n);
    int i = 0;
    while (i < n) {
        if (i == n - 1 || T(i + 1, i) == 0) {
            res.re[i] = T(i, i); res.im[i] = 0; ++i;
        } else {
            double p = 0.5 * (T(i, i) - T(i + 1, i + 1));
            double z = std::sqrt(std::fabs(p * p + T(i + 1, i) * T(i, i + 1)));
            res.re[i] = T(i + 1, i + 1) + p; res.im[i] = z;
            res.re[i + 1] = T(i + 1, i + 1) + p; res.im[i + 1] = -z;
            i += 2;
        }
    }
    return res;
}

static const double kEPS_H = 0.000000001;  // CVIPtexture.cpp:86

struct Tex { double v[14]; };

// Extract_Texture_Features for one angle, CVIPtexture.cpp:384-452 with the
// co-occurrence builders :455-614 and f1..f14 :631-1108.
static Tex texture_one(const std::vector<uint8_t> &g, int rows, int cols, int angle, int *tones_out) {
    int lut[256];
    for (int i = 0; i < 256; i++) lut[i] = -1;
    for (size_t i = 0; i < g.size(); i++) lut[g[i]] = g[i];
    int Ng = 0;
    for (int i = 0; i < 256; i++) if (lut[i] != -1) lut[i] = Ng++;
    if (tones_out) *tones_out = Ng;
    Mat P((size_t)Ng * Ng, 0.0);
    int dr = 0, dc = 0;
    if (angle == 0) { dr = 0; dc = 1; }
    else if (angle == 45) { dr = 1; dc = -1; }
    else if (angle == 90) { dr = 1; dc = 0; }
    else { dr = 1; dc = 1; }
    int count = 0;
    for (int r = 0; r < rows; r++)
        for (int c = 0; c < cols; c++) {
            uint8_t a = g[(size_t)r * cols + c];
            if (a == 0) continue;
            int r2 = r + dr, c2 = c + dc;
            if (r2 < rows && c2 >= 0 && c2 < cols) {
                uint8_t b = g[(size_t)r2 * cols + c2];
                if (!b) continue;
                int x = lut[a], y = lut[b];
                P[(size_t)x * Ng + y]++;
                P[(size_t)y * Ng + x]++;
                count += 2;
            }
        }
    for (size_t i = 0; i < P.size(); i++) P[i] = (count == 0) ? 0 : P[i] / count;
    auto p = [&](int i, int j) { return P[(size_t)i * Ng + j]; };
    const double l2 = std::log10(2.0);
    Tex t;
    // f1 ASM
    { double s = 0; for (int i = 0; i < Ng; i++) for (int j = 0; j < Ng; j++) s += p(i, j) * p(i, j); t.v[0] = s; }
    // f2 contrast
    { double big = 0;
      for (int nn = 0; nn < Ng; nn++) { double s = 0;
        for (int i = 0; i < Ng; i++) for (int j = 0; j < Ng; j++) if ((i - j) == nn || (j - i) == nn) s += p(i, j);
        big += nn * nn * s; }
      t.v[1] = big; }
    // f3 correlation
    { std::vector<double> px(Ng, 0.0);
      for (int i = 0; i < Ng; i++) for (int j = 0; j < Ng; j++) px[i] += p(i, j);
      double meanx = 0, sq = 0;
      for (int i = 0; i < Ng; i++) { meanx += px[i] * i; sq += px[i] * i * i; }
      double sd = std::sqrt(sq - (meanx * meanx));
      double tmp = 0;
      for (int i = 0; i < Ng; i++) for (int j = 0; j < Ng; j++) tmp += i * j * p(i, j);
      t.v[2] = (sd * sd == 0) ? 1 : (tmp - meanx * meanx) / (sd * sd); }
    // f4 variance
    { double mean = 0, var = 0;
      for (int i = 0; i < Ng; i++) for (int j = 0; j < Ng; j++) mean += i * p(i, j);
      for (int i = 0; i < Ng; i++) for (int j = 0; j < Ng; j++) var += (i - mean) * (i - mean) * p(i, j);
      t.v[3] = var; }
    // f5 IDM
    { double s = 0; for (int i = 0; i < Ng; i++) for (int j = 0; j < Ng; j++) s += p(i, j) / (1 + (i - j) * (i - j)); t.v[4] = s; }
    // f6 sum average, f8 sum entropy, f7 sum variance (with S = sum entropy)
    std::vector<double> pxpy(2 * Ng + 1, 0.0);
    for (int i = 0; i < Ng; i++) for (int j = 0; j < Ng; j++) pxpy[i + j] += p(i, j);
    { double s = 0; for (int i = 0; i <= 2 * Ng - 2; i++) s += i * pxpy[i]; t.v[5] = s; }
    double sent = 0;
    { std::vector<double> q(2 * Ng + 1, 0.0);
      for (int i = 0; i < Ng; i++) for (int j = 0; j < Ng; j++) q[i + j + 2] += p(i, j);
      for (int i = 2; i <= 2 * Ng; i++) sent -= q[i] * std::log10(q[i] + kEPS_H) / l2;
      t.v[7] = sent; }
    { double var = 0; for (int i = 0; i <= 2 * Ng - 2; i++) var += (i - sent) * (i - sent) * pxpy[i]; t.v[6] = var; }
    // f9 entropy
    { double e = 0; for (int i = 0; i < Ng; i++) for (int j = 0; j < Ng; j++) e += p(i, j) * std::log10(p(i, j) + kEPS_H) / l2; t.v[8] = -e; }
    // f10 difference variance, f11 difference entropy
    { std::vector<double> d(2 * Ng + 1, 0.0);
      for (int i = 0; i < Ng; i++) for (int j = 0; j < Ng; j++) d[std::abs(i - j)] += p(i, j);
      double s = 0, s2 = 0;
      for (int i = 0; i < Ng; i++) { s += i * d[i]; s2 += i * i * d[i]; }
      t.v[9] = s2 - s * s;
      double e = 0;
      for (int i = 0; i < Ng; i++) e += d[i] * std::log10(d[i] + kEPS_H) / l2;
      t.v[10] = -e; }
    // f12, f13 information measures of correlation
    std::vector<double> px(Ng, 0.0), py(Ng, 0.0);
    for (int i = 0; i < Ng; i++) for (int j = 0; j < Ng; j++) { px[i] += p(i, j); py[j] += p(i, j); }
    { double hx = 0, hy = 0, hxy = 0, hxy1 = 0, hxy2 = 0;
      for (int i = 0; i < Ng; i++) for (int j = 0; j < Ng; j++) {
          hxy1 -= p(i, j) * std::log10(px[i] * py[j] + kEPS_H) / l2;
          hxy2 -= px[i] * py[j] * std::log10(px[i] * py[j] + kEPS_H) / l2;
          hxy -= p(i, j) * std::log10(p(i, j) + kEPS_H) / l2;
      }
      for (int i = 0; i < Ng; i++) {
          hx -= px[i] * std::log10(px[i] + kEPS_H) / l2;
          hy -= py[i] * std::log10(py[i] + kEPS_H) / l2;
      }
      double m = hx > hy ? hx : hy;
      t.v[11] = (m == 0) ? 1 : ((hxy - hxy1) / m);
      t.v[12] = std::sqrt(std::fabs(1 - std::exp(-2.0 * (hxy2 - hxy)))); }
    // f14 maximal correlation coefficient: Q from _Q_calc_eigen (:961-987),
    // sqrt(Re lambda_2) in Schur order, 0 if complex.  Ng < 3 has no
    // eigenvalue #2 (the reference reads past the vector): defined as 0.
    { double f = 0;
      if (Ng >= 3) {
          Mat Q((size_t)Ng * Ng);
          std::vector<double> rp(Ng);
          for (int i = 0; i < Ng; i++) {
              for (int j = 0; j < i; j++) {
                  for (int k = 0; k < Ng; k++) rp[k] = p(i, k) * p(j, k);
                  double s1 = 0, s2 = 0;
                  for (int k = 0; k < Ng; k++) s1 += rp[k] / (px[i] * py[k] + 0.0000000000001);
                  for (int k = 0; k < Ng; k++) s2 += rp[k] / (px[j] * py[k] + 0.0000000000001);
                  Q[(size_t)i * Ng + j] = s1;
                  Q[(size_t)j * Ng + i] = s2;
              }
              double s = 0;
              for (int k = 0; k < Ng; k++) s += p(i, k) * p(i, k) / (px[i] * py[k] + 0.0000000000001);
              Q[(size_t)i * Ng + i] = s;
          }
          EigRes e = eigen_schur_eigenvalues(Q, Ng);
          if (e.ok && e.im[2] == 0) f = std::sqrt(e.re[2]);
      }
      t.v[13] = f; }
    return t;
}

// haralick2D, src/textures/haralick/haralick.cpp:12-144.
static void f_haralick(const Img &im, double *out) {
    Moments2 s = stats_of(im);
    double scale = 255.0 / (s.mx - s.mn);
    std::vector<uint8_t> g(im.n());
    for (size_t i = 0; i < im.n(); i++) {
        double q = (im.p[i] - s.mn) * scale;
        g[i] = std::isfinite(q) ? (uint8_t)q : 0;  // constant image: defined as tone 0
    }
    double mn[14], mx[14], sm[14];
    for (int a = 0; a < 14; a++) { mn[a] = kINF; mx[a] = -kINF; sm[a] = 0; }
    for (int ang = 0; ang <= 135; ang += 45) {
        Tex t = texture_one(g, im.h, im.w, ang, nullptr);
        for (int a = 0; a < 14; a++) {
            sm[a] += t.v[a];
            if (t.v[a] < mn[a]) mn[a] = t.v[a];
            if (t.v[a] > mx[a]) mx[a] = t.v[a];
        }
    }
    double tmp[28];
    for (int a = 0; a < 14; a++) { tmp[a] = sm[a] / 4; tmp[a + 14] = mx[a] - mn[a]; }
    static const int perm[28] = {0, 14, 1, 15, 2, 16, 9, 23, 10, 24, 8, 22, 11, 25,
                                 4, 18, 13, 27, 12, 26, 5, 19, 7, 21, 6, 20, 3, 17};
    for (int k = 0; k < 28; k++) out[k] = tmp[perm[k]];
}

// MultiScaleHistogram, src/cmatrix.cpp:1743-1756.
static void f_mshist(const Img &im, double *out) {
    Moments2 s = stats_of(im);
    histogram(im.p.data(), im.n(), 3, s.mn, s.mx, out);
    histogram(im.p.data(), im.n(), 5, s.mn, s.mx, out + 3);
    histogram(im.p.data(), im.n(), 7, s.mn, s.mx, out + 8);
    histogram(im.p.data(), im.n(), 9, s.mn, s.mx, out + 15);
    double mx = 0;
    for (int a = 0; a < 24; a++) if (out[a] > mx) mx = out[a];
    for (int a = 0; a < 24; a++) out[a] /= mx;
}

// ---- Tamura, src/textures/tamura.cpp:10-299
// ImageMatrix::convolve: zero-padded correlation, src/cmatrix.cpp:892-932.
static Img convolve3(const Img &in, const double f[3][3]) {
    Img o(in.w, in.h);
    for (long x = 0; x < in.w; ++x)
        for (long y = 0; y < in.h; ++y) {
            double t = 0.0;
            for (long i = -1; i <= 1; ++i) {
                long xx = x + i;
                if (xx < 0 || xx >= in.w) continue;
                for (long j = -1; j <= 1; ++j) {
                    long yy = y + j;
                    if (yy < 0 || yy >= in.h) continue;
                    t += f[j + 1][i + 1] * in.at(yy, xx);
                }
            }
            o.at(y, x) = t;
        }
    return o;
}

static double t_contrast(const Img &im) {
    Moments4 m;
    for (int x = 0; x < im.w; x++)
        for (int y = 0; y < im.h; y++) m.add(im.at(y, x));
    double z[4];
    m.vec(z);
    if (z[1] < DBL_EPSILON) return 0;
    return z[1] / std::pow(z[3] / std::pow(z[1], 4), 0.25);
}

static double t_directionality(const Img &im) {
    // the kernels as the reference's assignments leave them (tamura.cpp:45-57)
    static const double H[3][3] = {{-1, 2, 1}, {-2, 0, 2}, {-1, -2, -1}};
    static const double V[3][3] = {{1, 0, 0}, {0, 0, 0}, {-1, 0, 0}};
    Img dH = convolve3(im, H), dV = convolve3(im, V);
    Img phi(im.w, im.h);
    Moments2 ps;
    double sum_r = 0;
    for (int y = 0; y < im.h; ++y)
        for (int x = 0; x < im.w; ++x) {
            double h = dH.at(y, x);
            if (h >= 0.0001) {
                double v = std::atan(dV.at(y, x) / h) + (M_PI / 2.0 + 0.001);
                phi.at(y, x) = ps.add(v);
                sum_r += std::pow(h, 2) + std::pow(dV.at(y, x), 2) + std::pow(v, 2);
            } else {
                phi.at(y, x) = ps.add(0.0);
            }
        }
    double Hd[125];
    histogram(phi.p.data(), phi.n(), 125, ps.mn, ps.mx, Hd);
    double mx = 0.0;
    long fmx = 0;
    for (long a = 0; a < 125; a++) if (Hd[a] > mx) { mx = Hd[a]; fmx = a; }
    double sum = 0;
    for (long a = 0; a < 125; a++) sum += Hd[a] * std::pow((double)(a + 1 - fmx), 2);
    return std::fabs(std::log(sum / sum_r + 0.0000001));
}

static double t_coarseness(const Img &im, double *hist) {
    const unsigned yD = im.h, xD = im.w;
    Img S(xD, yD);
    for (unsigned y = 0; y < yD; ++y)
        for (unsigned x = 0; x < xD; ++x) {
            double l = (x < 1) ? 0 : S.at(y, x - 1);
            double o = (y < 1) ? 0 : S.at(y - 1, x);
            double ol = (y < 1 || x < 1) ? 0 : S.at(y - 1, x - 1);
            S.at(y, x) = im.at(y, x) + l + o - ol;
        }
    // efficientLocalMean, tamura.cpp:106-139
    auto localmean = [&](long x, long y, long k) {
        long k2 = k / 2, dimx = xD, dimy = yD;
        long sy = y - k2, sx = x - k2, ey = y + k2 - 1, ex = x + k2 - 1;
        if (sy < 0) sy = 0;
        if (sx < 0) sx = 0;
        if (ex > dimx - 1) ex = dimx - 1;
        if (ey > dimy - 1) ey = dimy - 1;
        double links = (sx - 1 < 0) ? 0 : S.at(ey, sx - 1);
        double oben = (sy - 1 < 0) ? 0 : S.at(ey - 1, sx);
        double ol = ((sy - 1 < 0) || (sx - 1 < 0)) ? 0 : S.at(ey - 1, sx - 1);
        double unten = S.at(ey, sx);
        long cnt = (ey - sy + 1) * (ex - sx + 1);
        return (unten - links - oben + ol) / cnt;
    };
    std::vector<Img> A(7, Img(xD, yD));
    int len = 1;
    for (int k = 1; k <= 7; ++k) {
        len *= 2;
        for (unsigned y = 0; y < yD; ++y)
            for (unsigned x = 0; x < xD; ++x) A[k - 1].at(y, x) = localmean(x, y, len);
    }
    Img Sb(xD, yD);
    Moments2 ss;
    double sum = 0.0;
    for (unsigned y = 0; y < yD; ++y)
        for (unsigned x = 0; x < xD; ++x) {
            double maxE = 0;
            int maxk = 0, kk2 = 1;
            for (int k = 1; k <= 7; ++k, kk2 *= 2) {
                const Img &a = A[k - 1];
                int px1 = x + kk2, px2 = (int)x - kk2, py1 = y + kk2, py2 = (int)y - kk2;
                double eh = (px1 < (int)xD && px2 >= 0) ? std::fabs(a.at(y, px1) - a.at(y, px2)) : 0;
                double ev = (py1 < (int)yD && py2 >= 0) ? std::fabs(a.at(py1, x) - a.at(py2, x)) : 0;
                if (eh > maxE) { maxE = eh; maxk = k; }
                if (ev > maxE) { maxE = ev; maxk = k; }
            }
            Sb.at(y, x) = ss.add(maxk);
            sum += maxk;
        }
    // unsigned arithmetic as in the reference (tamura.cpp:246-248)
    if (yD == 32 || xD == 32) sum /= (double)((uint32_t)((xD + 1 - 32) * (yD + 1 - 32)));
    else sum /= (double)((uint32_t)((yD - 32) * (xD - 32)));
    histogram(Sb.p.data(), Sb.n(), 3, ss.mn, ss.mx, hist);
    double hm = 0.0;
    for (int k = 0; k < 3; k++) if (hist[k] > hm) hm = hist[k];
    for (int k = 0; k < 3; k++) hist[k] = hist[k] / hm;
    return sum;
}

// Tamura3Sigs2D, tamura.cpp:275-299.
static void f_tamura(const Img &im, double *out) {
    Moments2 s = stats_of(im);
    Img n(im.w, im.h);
    for (size_t i = 0; i < im.n(); i++) n.p[i] = (im.p[i] - s.mn) / s.mx;
    double t[6];
    t[0] = t_coarseness(n, &t[1]);
    t[4] = t_directionality(n);
    t[5] = t_contrast(n);
    out[0] = t[1]; out[1] = t[2]; out[2] = t[3]; out[3] = t[5]; out[4] = t[4]; out[5] = t[0];
}

// Comb moments: CombFirst4Moments2D, matr4moments_to_hist, vd_Comb4Moments,
// src/statistics/CombFirst4Moments.cpp:47-272.
static void f_comb(const Img &im, double *out) {
    const long m = im.h, n = im.w, n2 = n / 2, m2 = m / 2;
    double M[4][20];
    for (int a = 0; a < 4; a++) for (int b = 0; b < 20; b++) M[a][b] = 0;
    double raw[48];
    int vi = 0;
    for (int dir = 0; dir < 4; dir++) {
        int idx = 0;
        double step = (double)m / 10.0;
        if (step < 1.0) step = 1.0;
        for (double mp = 1.0 - m; mp <= m; mp += step) {
            long ii = std::lround(mp);
            Moments4 mm;
            if (dir == 0) {          // x = y + ii
                for (long y = 0; y < m; y++) { long x = y + ii; if (x >= 0 && x < n) mm.add(im.at(y, x)); }
            } else if (dir == 1) {   // x = n - 1 - y - ii
                for (long y = 0; y < m; y++) { long x = n - 1 - y - ii; if (x >= 0 && x < n) mm.add(im.at(y, x)); }
            } else if (dir == 2) {   // column x = n2 - 1 - ii
                long x = n2 - 1 - ii;
                if (x >= 0 && x < n) for (long y = 0; y < m; y++) mm.add(im.at(y, x));
            } else {                 // row y = m2 - 1 - ii
                long y = m2 - 1 - ii;
                if (y >= 0 && y < m) for (long x = 0; x < n; x++) mm.add(im.at(y, x));
            }
            double z[4];
            mm.vec(z);
            for (int a = 0; a < 4; a++) M[a][idx] = z[a];
            idx++;
        }
        for (int a = 0; a < 4; a++) {
            double lo = kINF, hi = -kINF;
            for (int b = 0; b < 20; b++) { if (M[a][b] > hi) hi = M[a][b]; if (M[a][b] < lo) lo = M[a][b]; }
            histogram(M[a], 20, 3, lo, hi, &raw[vi]);
            vi += 3;
        }
    }
    static const int perm[48] = {45, 46, 47, 36, 37, 38, 42, 43, 44, 39, 40, 41, 33, 34, 35, 24,
                                 25, 26, 30, 31, 32, 27, 28, 29, 9, 10, 11, 0, 1, 2, 6, 7,
                                 8, 3, 4, 5, 21, 22, 23, 12, 13, 14, 18, 19, 20, 15, 16, 17};
    for (int k = 0; k < 48; k++) out[k] = raw[perm[k]];
}

// Radon: ImageMatrix::RadonTransform2D + radon + vd_RadonTextures,
// src/cmatrix.cpp:1463-1514, src/transforms/radon.cpp:14-115.
static void f_radon(const Img &im, double *out) {
    const int W = im.w, H = im.h;
    int rLast = (int)std::ceil(std::sqrt(std::pow((double)(W - 1 - (W - 1) / 2), 2) +
                                         std::pow((double)(H - 1 - (H - 1) / 2), 2))) + 1;
    int rFirst = -rLast, rSize = rLast - rFirst + 1;
    const int M = H, N = W, xo = (W - 1) / 2, yo = (H - 1) / 2;
    std::vector<double> P((size_t)rSize * 4, 0.0), yT(2 * M), xT(2 * N), xc(2 * N), ys(2 * M);
    yT[2 * M - 1] = -yo - 0.25;
    for (int k = 2 * M - 2; k >= 0; k--) yT[k] = yT[k + 1] + 0.5;
    xT[0] = -xo - 0.25;
    for (int k = 1; k < 2 * N; k++) xT[k] = xT[k - 1] + 0.5;
    const double th[4] = {0, 45, 90, 135};
    for (int k = 0; k < 4; k++) {
        double ang = (th[k] * M_PI) / 180, c = std::cos(ang), s = std::sin(ang);
        double *pr = &P[(size_t)k * rSize];
        for (int q = 0; q < 2 * N; q++) xc[q] = xT[q] * c - rFirst;
        for (int q = 0; q < 2 * M; q++) ys[q] = yT[q] * s;
        for (int nn = 0; nn < 2 * N; nn++)
            for (int mm = 0; mm < 2 * M; mm++) {
                double pix = im.at(mm / 2, nn / 2);
                if (pix) {
                    pix *= 0.25;
                    double ri = xc[nn] + ys[mm];
                    int rl = (int)ri;
                    double pl = pix * (1 - ri + rl);
                    pr[rl++] += pl;
                    pr[rl] += pix - pl;
                }
            }
    }
    double v[12];
    for (int k = 0; k < 4; k++) {
        double lo = kINF, hi = -kINF;
        const double *pr = &P[(size_t)k * rSize];
        for (int i = 0; i < rSize; i++) { if (pr[i] > hi) hi = pr[i]; if (pr[i] < lo) lo = pr[i]; }
        histogram(pr, rSize, 3, lo, hi, &v[3 * k]);
    }
    static const int perm[12] = {0, 1, 2, 9, 10, 11, 3, 4, 5, 6, 7, 8};
    for (int k = 0; k < 12; k++) out[k] = v[perm[k]];
}

// FractalFeatures::execute, src/FeatureAlgorithms.cpp:232-267.
static void f_fractal(const Img &im, double *out) {
    const int bins = 20, W = im.w, H = im.h;
    for (int i = 0; i < bins; i++) out[i] = 0;
    int K = ((W > H) ? H : W) / 5;
    int step = (int)std::floor((double)(K / bins));
    if (step < 1) step = 1;
    int bin = 0;
    for (int k = 1; k < K; k = k + step) {
        double sum = 0.0;
        for (int x = 0; x < W; x++)
            for (int y = 0; y < H - k; y++) sum += std::fabs(im.at(y, x) - im.at(y + k, x));
        for (int x = 0; x < W - k; x++)
            for (int y = 0; y < H; y++) sum += std::fabs(im.at(y, x) - im.at(y, x + k));
        if (bin < bins) out[bin++] = sum / (W * (W - k) + H * (H - k));
    }
}

// PixelIntensityStatistics::execute, src/FeatureAlgorithms.cpp:272-294.
static void f_pixstats(const Img &im, double *out) {
    Moments2 s = stats_of(im);
    out[0] = s.mean;
    out[1] = median_of(im.p);
    out[2] = s.std_();
    out[3] = s.mn;
    out[4] = s.mx;
}

// GiniCoefficient::execute, src/FeatureAlgorithms.cpp:448-492.
static void f_gini(const Img &im, double *out) {
    std::vector<double> v;
    double mean = 0;
    for (double x : im.p) if (x > 0) { v.push_back(x); mean += x; }
    long count = (long)v.size();
    if (count > 0) mean = mean / count;
    std::sort(v.begin(), v.end());
    double g = 0.0;
    for (long i = 1; i <= count; i++) g += (2. * i - count - 1.) * v[i - 1];
    out[0] = (count <= 1 || mean <= 0.0) ? 0.0 : g / (mean * count * (count - 1));
}

// EdgeFeatures: EdgeStatistics with PrewittMagnitude2D / PrewittDirection2D,
// src/FeatureAlgorithms.cpp:299-341, src/cmatrix.cpp:1317-1458.
static void f_edge_features(const Img &im, double *out) {
    const long w = im.w, h = im.h;
    Img mag(w, h), dir(w, h);
    Moments2 ms, ds;  // accumulated in the reference's x-outer order
    for (long x = 0; x < w; x++)
        for (long y = 0; y < h; y++) {
            double sx = 0, sy = 0;
            for (long j = y - 1; j <= y + 1; j++) if (j >= 0 && j < h && x - 1 >= 0) sx += im.at(j, x - 1) * 1;
            for (long j = y - 1; j <= y + 1; j++) if (j >= 0 && j < h && x + 1 < w) sx += im.at(j, x + 1) * -1;
            for (long i = x - 1; i <= x + 1; i++) if (i >= 0 && i < w && y - 1 >= 0) sy += im.at(y - 1, i) * 1;
            for (long i = x - 1; i <= x + 1; i++) if (i >= 0 && i < w && y + 1 < h) sy += im.at(y + 1, i) * -1;
            mag.at(y, x) = ms.add(std::sqrt(sx * sx + sy * sy));
            double d;
            if (sy == 0 || std::fabs(sy) < 1 / kINF) d = 3.1415926 * (sx < 0 ? 1 : 0);
            else d = std::atan2(sy, sx);
            dir.at(y, x) = ds.add(d);
        }
    double MagHist[8], DirHist[8], Diff[4] = {0, 0, 0, 0}, homog = 0;
    double MagMedian = median_of(mag.p), MagMean = ms.mean, MagVar = ms.var();
    histogram(mag.p.data(), mag.n(), 8, ms.mn, ms.mx, MagHist);
    unsigned long area = 0;
    for (double v : mag.p) if (v > MagMean) area++;
    double DirMedian = median_of(dir.p), DirMean = ds.mean, DirVar = ds.var();
    histogram(dir.p.data(), dir.n(), 8, ds.mn, ds.mx, DirHist);
    for (int b = 0; b < 4; b++) Diff[b] = std::fabs(DirHist[b] - DirHist[b + 4]);
    double sum = 0;
    for (int b = 0; b < 4; b++) {
        if (DirHist[b] + DirHist[b + 4] != 0) Diff[b] = Diff[b] / (DirHist[b] + DirHist[b + 4]);
        sum += (DirHist[b] + DirHist[b + 4]);
    }
    if (sum > 0) homog = (DirHist[0] + DirHist[1]) / sum;
    int k = 0;
    out[k++] = (double)area;
    for (int j = 0; j < 4; j++) out[k++] = Diff[j];
    for (int j = 0; j < 8; j++) out[k++] = DirHist[j];
    out[k++] = homog; out[k++] = DirMean; out[k++] = DirMedian; out[k++] = DirVar;
    for (int j = 0; j < 8; j++) out[k++] = MagHist[j];
    out[k++] = MagMean; out[k++] = MagMedian; out[k++] = MagVar;
}

// ObjectFeatures: FeatureStatistics with OtsuBinaryMaskTransform, bwlabel(8),
// GlobalCentroid, FeatureCentroid, EulerNumber,
// src/FeatureAlgorithms.cpp:346-400, src/cmatrix.cpp:1577-1717,
// src/statistics/FeatureStatistics.cpp:44-254.  No object: the reference
// reads element 0 of an empty array; defined here as all-zero statistics.
static void f_objects(const Img &im, double *out) {
    const long w = im.w, h = im.h;
    Moments2 s = stats_of(im);
    double thr = otsu(im, s.mn, s.mx);
    std::vector<long> lab((size_t)w * h);
    for (size_t i = 0; i < im.n(); i++) lab[i] = (im.p[i] > thr) ? 1 : 0;
    double cxm = 0, cym = 0, mass = 0;
    for (long y = 0; y < h; y++)
        for (long x = 0; x < w; x++)
            if (lab[(size_t)y * w + x] > 0) { cxm = cxm + x + 1; cym = cym + y + 1; mass++; }
    double cx = mass ? cxm / mass : 0, cy = mass ? cym / mass : 0;
    // Euler number (mode 8) on the binary mask; Cd never counts (:246)
    long C1 = 0, C3 = 0;
    for (long y = 1; y < h; y++)
        for (long x = 1; x < w; x++) {
            int q = (lab[(size_t)(y - 1) * w + x - 1] > 0) * 8 + (lab[(size_t)(y - 1) * w + x] > 0) * 4 +
                    (lab[(size_t)y * w + x - 1] > 0) * 2 + (lab[(size_t)y * w + x] > 0);
            if (q == 8 || q == 4 || q == 2 || q == 1) C1++;
            else if (q == 7 || q == 11 || q == 13 || q == 14) C3++;
        }
    long euler = (C1 - C3) / 4;
    // bwlabel with the reference's FIFO flood fill: seeds in raster order
    long group = 1;
    std::vector<long> qx, qy;
    qx.reserve(w * h); qy.reserve(w * h);
    for (long y = 0; y < h; y++)
        for (long x = 0; x < w; x++) {
            if (lab[(size_t)y * w + x] != 1) continue;
            group++;
            lab[(size_t)y * w + x] = group;
            qx.clear(); qy.clear();
            qx.push_back(x); qy.push_back(y);
            for (size_t head = 0; head < qx.size(); head++) {
                long bx = qx[head], by = qy[head];
                const long nb[8][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}, {-1, -1}, {1, -1}, {-1, 1}, {1, 1}};
                for (int k = 0; k < 8; k++) {
                    long xx = bx + nb[k][0], yy = by + nb[k][1];
                    if (xx < 0 || xx >= w || yy < 0 || yy >= h) continue;
                    if (lab[(size_t)yy * w + xx] == 1) {
                        lab[(size_t)yy * w + xx] = group;
                        qx.push_back(xx); qy.push_back(yy);
                    }
                }
            }
        }
    unsigned long count = group - 1;
    std::vector<unsigned long> area(count, 0), xm(count, 0), ym(count, 0);
    for (long y = 0; y < h; y++)
        for (long x = 0; x < w; x++) {
            long L = lab[(size_t)y * w + x];
            if (L >= 2) { area[L - 2]++; xm[L - 2] += x + 1; ym[L - 2] += y + 1; }
        }
    std::vector<double> dist(count);
    double sum_a = 0, sum_d = 0;
    for (unsigned long o = 0; o < count; o++) {
        double ox = (double)xm[o] / (double)area[o], oy = (double)ym[o] / (double)area[o];
        dist[o] = std::sqrt(std::pow(ox - cx, 2) + std::pow(oy - cy, 2));
        sum_a += area[o];
        sum_d += dist[o];
    }
    unsigned int ahist[10] = {0}, dhist[10] = {0};
    unsigned long amin = 0, amax = 0;
    unsigned int amed = 0;
    double amean = 0, avar = 0, dmin = 0, dmax = 0, dmean = 0, dmed = 0, dvar = 0;
    if (count > 0) {
        std::sort(area.begin(), area.end());
        amin = area[0]; amax = area[count - 1];
        amean = sum_a / count;
        amed = (unsigned int)area[count / 2];
        double sc = (amax - amin > 0) ? 10.0 / double(amax - amin) : 0;
        double ss = 0;
        if (amax - amin > 0)
            for (unsigned long o = 0; o < count; o++) {
                ss += std::pow(area[o] - amean, 2);
                ahist[bin_of((double)area[o], (double)amin, sc, 10)] += 1;
            }
        avar = (count > 1) ? ss / (count - 1) : ss;
        std::sort(dist.begin(), dist.end());
        dmin = dist[0]; dmax = dist[count - 1];
        dmean = sum_d / count;
        dmed = dist[count / 2];
        double dsc = (dmax - dmin > 0) ? 10.0 / double(dmax - dmin) : 0;
        double sd = 0;
        for (unsigned long o = 0; o < count; o++) {
            sd += std::pow(dist[o] - dmean, 2);
            dhist[bin_of(dist[o], dmin, dsc, 10)] += 1;
        }
        dvar = (count > 1) ? sd / (count - 1) : sd;
    }
    int k = 0;
    for (int j = 0; j < 10; j++) out[k++] = ahist[j];
    out[k++] = amax; out[k++] = amean; out[k++] = amed; out[k++] = amin; out[k++] = avar;
    out[k++] = cx; out[k++] = cy; out[k++] = count;
    for (int j = 0; j < 10; j++) out[k++] = dhist[j];
    out[k++] = dmax; out[k++] = dmean; out[k++] = dmed; out[k++] = dmin; out[k++] = dvar;
    out[k++] = euler;
}

// InverseObjectFeatures: ImageMatrix::invert then ObjectFeatures,
// src/FeatureAlgorithms.cpp:404-417, src/cmatrix.cpp:569-572.
static void f_inv_objects(const Img &im, double *out) {
    Moments2 s = stats_of(im);
    Img inv(im.w, im.h);
    for (size_t i = 0; i < im.n(); i++) inv.p[i] = s.mx - im.p[i] + s.mn;
    f_objects(inv, out);
}

// ---- Gabor, src/textures/gabor.cpp:19-231
static std::vector<double> gabor_kernel(double f0) {
    const int n = 38;
    const double sig2lam = 0.56, gamma = 0.5, theta = 3.14159265 / 2, fi = 0;
    double lambda = 2 * M_PI / f0, ct = std::cos(theta), st = std::sin(theta), sig = sig2lam * lambda;
    std::vector<double> tx(n + 1), ty(n + 1), G((size_t)n * n * 2);
    tx[0] = -(n / 2);
    for (int x = 1; x <= n; x++) tx[x] = tx[x - 1] + 1;
    ty[0] = -(n / 2);
    for (int y = 1; y <= n; y++) ty[y] = ty[y - 1] + 1;
    double sum = 0;
    for (int y = 0; y < n; y++)
        for (int x = 0; x < n; x++) {
            double xte = tx[x] * ct + ty[y] * st, yte = ty[y] * ct - tx[x] * st;
            double rte = xte * xte + gamma * gamma * yte * yte;
            double ge = std::exp(-1 * rte / (2 * sig * sig));
            double argm = xte * f0 + fi;
            G[(size_t)y * n * 2 + x * 2] = ge * std::cos(argm);
            G[(size_t)y * n * 2 + x * 2 + 1] = ge * std::sin(argm);
            sum += std::sqrt(std::pow(G[(size_t)y * n * 2 + x * 2], 2) + std::pow(G[(size_t)y * n * 2 + x * 2 + 1], 2));
        }
    for (auto &g : G) g = g / sum;
    return G;
}

// GaborEnergy: |full complex convolution| cropped at ceil(n/2).
static std::vector<double> gabor_energy(const Img &im, double f0) {
    const int n = 38, W = im.w, H = im.h, off = 19;
    std::vector<double> G = gabor_kernel(f0), e((size_t)W * H);
    for (int b = 0; b < H; b++)
        for (int a = 0; a < W; a++) {
            double re = 0, imv = 0;
            int yy = b + off, xx = a + off;
            for (int j = 0; j < n; j++) {
                int l = yy - j;
                if (l < 0 || l >= H) continue;
                for (int i = 0; i < n; i++) {
                    int k = xx - i;
                    if (k < 0 || k >= W) continue;
                    double v = im.at(l, k);
                    re += v * G[(size_t)j * n * 2 + i * 2];
                    imv += v * G[(size_t)j * n * 2 + i * 2 + 1];
                }
            }
            e[(size_t)b * W + a] = std::sqrt(std::pow(re, 2) + std::pow(imv, 2));
        }
    return e;
}

// GaborTextureFilters2D, gabor.cpp:201-231.
static void f_gabor(const Img &im, double *out) {
    std::vector<double> e = gabor_energy(im, 0.1);
    double mx = *std::max_element(e.begin(), e.end());
    unsigned long base = 0;
    for (double v : e) if (v > mx * 0.4) base++;
    for (int ii = 0; ii < 7; ii++) {
        std::vector<double> g = gabor_energy(im, (double)(ii + 1));
        double gm = *std::max_element(g.begin(), g.end());
        Img e2(im.w, im.h);
        Moments2 s;
        for (size_t i = 0; i < g.size(); i++) e2.p[i] = s.add(g[i] / gm);
        double thr = otsu(e2, s.mn, s.mx);
        unsigned long after = 0;
        for (double v : e2.p) if (v > thr) after++;
        out[ii] = (double)after / (double)base;
    }
}

// ---------------------------------------------------------------- colour
// RGB2HSV and RGB2GRAY (src/cmatrix.h:95-160).
static void rgb2hsv(unsigned char R, unsigned char G, unsigned char B, unsigned char *hsv) {
    double r = (double)R / 255, g = (double)G / 255, b = (double)B / 255;
    double mx = std::max(r, std::max(g, b)), mn = std::min(r, std::min(g, b));
    double delta = mx - mn;
    unsigned char hh = 0, s = 0, v = (unsigned char)(mx * 240.0);
    if (mx != 0.0) s = (unsigned char)((delta / mx) * 240.0);
    if (s != 0) {
        double h = 0;
        if (r == mx) h = (g - b) / delta;
        else if (g == mx) h = 2 + (b - r) / delta;
        else if (b == mx) h = 4 + (r - g) / delta;
        h *= 60.0;
        if (h >= 360) h -= 360.0;
        if (h < 0.0) h += 360.0;
        hh = (unsigned char)(h * (240.0 / 360.0));
    }
    hsv[0] = hh;
    hsv[1] = s;
    hsv[2] = v;
}
static double rgb2gray(unsigned char r, unsigned char g, unsigned char b) {
    return 0.2989 * r + 0.5870 * g + 0.1140 * b;
}

// ImageMatrix::LoadTIFF for 3 samples per pixel (src/cmatrix.cpp:128-199):
// 16-bit samples scaled to bytes over the image's min..max of all channels.
static Img make_rgb_img(const void *pix, int w, int h, int bits) {
    Img im(w, h);
    im.hsv.resize((size_t)3 * w * h);
    const size_t n = (size_t)w * h;
    double lo = 0, scale = 0;
    if (bits > 8) {
        const unsigned short *p = (const unsigned short *)pix;
        double mn = DBL_MAX, mx = -DBL_MAX;
        for (size_t i = 0; i < 3 * n; i++) {
            mn = std::min(mn, (double)p[i]);
            mx = std::max(mx, (double)p[i]);
        }
        lo = mn;
        scale = 255.0 / (mx - mn);
    }
    for (size_t i = 0; i < n; i++) {
        unsigned char c[3];
        for (int k = 0; k < 3; k++) {
            if (bits > 8) {
                double t = ((double)((const unsigned short *)pix)[3 * i + k] - lo) * scale;
                c[k] = std::isnan(t) ? 0 : (unsigned char)t;  // a flat image: 0 * inf
            } else {
                c[k] = ((const unsigned char *)pix)[3 * i + k];
            }
        }
        im.p[i] = rgb2gray(c[0], c[1], c[2]);
        rgb2hsv(c[0], c[1], c[2], &im.hsv[3 * i]);
    }
    return im;
}

// The fuzzy colour classifier (src/colors/FuzzyCalc.cpp:625-834, constants
// src/colors/FuzzyCalc.h:42-148).  Colours: 1 white, 2 light grey, 3 dark
// grey, 4 black, 5 red, 6 pink, 7 dark brown, 8 light brown, 9 dark orange,
// 10 light orange, 11 yellow, 12 olive, 13 light green, 14 dark green, 15 teal,
// 16 aqua, 17 blue, 18 dark fuchsia, 19 light fuchsia.
namespace fuzzy {
struct Trapezoid { int colour; double start, max1, max2, end; };
static const Trapezoid kHueFunctions[11] = {
    {5, 0, 0, 0, 11},       {9, 0, 17, 17, 27},       {10, 20, 27, 27, 37},  {11, 27, 39, 39, 47},
    {13, 40, 50, 50, 80},   {14, 50, 80, 80, 120},    {16, 80, 120, 120, 160}, {17, 120, 160, 160, 200},
    {18, 160, 200, 200, 220}, {19, 200, 220, 220, 230}, {5, 220, 240, 240, 240}};
// the rule base, one rule per (hue colour, saturation class 1..6, value class
// 1..5) in this order; the output colour 0 marks the two rules whose colour
// name the reference misspells (no colour sums them)
static const int kHueColour[10] = {5, 9, 10, 11, 13, 14, 16, 17, 18, 19};
struct Rule { int hue, sat, val, colour; };
static std::vector<Rule> rules() {
    static const unsigned char grid[300] = {
        4, 4, 3, 2, 1, 4, 3, 3, 19, 6, 4, 7, 18, 6, 6, 4, 7, 8, 19, 6, 4, 7, 7, 5, 5, 4, 4, 5, 5, 5,
        4, 3, 3, 2, 1, 4, 3, 3, 2, 1, 4, 7, 3, 8, 6, 4, 7, 7, 8, 10, 4, 7, 7, 8, 9, 4, 7, 7, 8, 9,
        4, 3, 3, 2, 1, 4, 3, 3, 2, 1, 4, 3, 3, 2, 10, 4, 7, 8, 8, 10, 4, 7, 8, 8, 10, 4, 7, 8, 8, 10,
        4, 3, 3, 2, 1, 4, 3, 3, 2, 1, 4, 3, 12, 12, 11, 4, 12, 12, 12, 11, 4, 12, 12, 12, 11, 4, 12, 12, 12, 11,
        4, 3, 3, 2, 1, 4, 3, 3, 2, 1, 4, 12, 12, 13, 13, 4, 14, 14, 13, 13, 4, 14, 14, 13, 13, 4, 14, 14, 13, 13,
        4, 3, 3, 2, 1, 4, 3, 3, 13, 13, 4, 14, 14, 13, 13, 4, 14, 14, 13, 13, 4, 14, 14, 13, 13, 4, 14, 14, 13, 13,
        4, 3, 3, 2, 1, 4, 3, 3, 15, 16, 4, 15, 17, 17, 16, 4, 15, 17, 16, 16, 4, 15, 17, 16, 16, 4, 15, 15, 16, 16,
        4, 3, 3, 2, 1, 4, 3, 0, 16, 16, 4, 18, 0, 19, 16, 4, 17, 17, 17, 17, 4, 17, 17, 17, 17, 4, 17, 17, 17, 17,
        4, 3, 3, 2, 1, 4, 3, 18, 19, 19, 4, 18, 18, 19, 19, 4, 18, 18, 19, 19, 4, 18, 18, 19, 19, 4, 7, 18, 18, 19,
        4, 3, 3, 2, 1, 4, 3, 2, 19, 19, 4, 18, 18, 19, 19, 4, 18, 18, 19, 19, 4, 7, 18, 19, 19, 4, 7, 18, 18, 19};
    std::vector<Rule> r;
    for (int k = 0; k < 300; k++) r.push_back({kHueColour[k / 30], (k / 5) % 6 + 1, k % 5 + 1, grid[k]});
    return r;
}
// color_value: the first trapezoid of the colour giving a positive membership
static double colour_value(int colour, double x) {
    double res = 0;
    for (const Trapezoid &t : kHueFunctions) {
        if (t.colour != colour) continue;
        if (x < t.start || x > t.end) res = 0;
        else if (x >= t.max1 && x <= t.max2) res = 1;
        else if (x < t.max1) res = (x - t.start) / (t.max1 - t.start);
        else res = 1 - (x - t.max2) / (t.end - t.max2);
        if (res > 0) return res;
    }
    return res;
}
// saturation classes 1..6: grey, almost grey, tend grey, medium grey, tend clear, clear
static double saturation_value(int cls, double x) {
    switch (cls) {
        case 1:
            if (x < 0) return 0;  // MIN_GREY
            if (x < -0.1 || x > 40) return 0;
            if (x < 0) return (x - -0.1) / (0 - -0.1);
            return 1 - ((x - 0) / (40 - 0));
        case 2:
            if (x < 10 || x > 70) return 0;
            if (x < 30) return (x - 10) / (30.0 - 10);
            return 1 - ((x - 30) / (70.0 - 30));
        case 3:
            if (x < 30 || x > 120) return 0;
            if (x < 70) return (x - 30) / (70.0 - 30);
            return 1 - ((x - 70) / (120.0 - 70));
        case 4:
            if (x < 60 || x > 180) return 0;
            if (x < 120) return (x - 60) / (120.0 - 60);
            return 1 - ((x - 120) / (180.0 - 120));
        case 5:
            if (x < 120 || x > 240) return 0;
            if (x < 180) return (x - 120) / (180.0 - 120);
            return 1 - ((x - 180) / (240.0 - 180));
        default:
            if (x < 180 || x > 240.1) return 0;
            if (x <= 240) return (x - 180) / (240.0 - 180);
            return 1 - ((x - 240) / (240.1 - 240));
    }
}
// value classes 1..5: dark, almost dark, tend dark, tend light, light
static double value_value(int cls, double x) {
    switch (cls) {
        case 1:
            if (x < 0) return 0;  // MIN_DARK
            if (x < -0.1 || x > 60) return 0;
            if (x < 0) return (x - -0.1) / (0 - -0.1);
            return 1 - ((x - 0) / (60 - 0));
        case 2:
            if (x < 0 || x > 120) return 0;
            if (x < 60) return (x - 0) / (60.0 - 0);
            return 1 - ((x - 60) / (120.0 - 60));
        case 3:
            if (x < 60 || x > 180) return 0;
            if (x < 120) return (x - 60) / (120.0 - 60);
            return 1 - ((x - 120) / (180.0 - 120));
        case 4:
            if (x < 120 || x > 240) return 0;
            if (x < 180) return (x - 120) / (180.0 - 120);
            return 1 - ((x - 180) / (240.0 - 180));
        default:
            if (x < 200 || x > 240.1) return 0;
            if (x <= 240) return (x - 200) / (240.0 - 200);
            return 1 - ((x - 240) / (240.1 - 240));
    }
}
// CalculateRules2 + FindColor: per colour, the rule products in rule order
static int find_colour(int h, int s, int v) {
    static const std::vector<Rule> R = rules();
    double best = 0;
    int res = 2;
    for (int colour = 1; colour <= 19; colour++) {
        double sum = 0;
        for (const Rule &r : R) {
            if (r.colour != colour) continue;
            double ret = colour_value(r.hue, h);
            if (ret == 0) continue;
            ret = ret * saturation_value(r.sat, s);
            if (ret == 0) continue;
            ret = ret * value_value(r.val, v);
            sum = sum + ret;
        }
        if (sum > best) {
            best = sum;
            res = colour;
        }
    }
    return res;
}
}  // namespace fuzzy

// HueTransform / ColorTransform (src/cmatrix.cpp:1023-1066)
static Img hue_plane(const Img &in) {
    Img o(in.w, in.h);
    for (size_t i = 0; i < o.n(); i++) o.p[i] = in.hsv[3 * i];
    return o;
}
static Img colour_plane(const Img &in) {
    Img o(in.w, in.h);
    const double max_range = std::pow((double)2, 8) - 1;
    for (size_t i = 0; i < o.n(); i++) {
        unsigned long c = fuzzy::find_colour(in.hsv[3 * i], in.hsv[3 * i + 1], in.hsv[3 * i + 2]);
        o.p[i] = int((max_range * c) / 19);
    }
    return o;
}
// ColorHistogram::execute (src/FeatureAlgorithms.cpp:506-531)
static void f_color_hist(const Img &im, double *out) {
    for (int c = 0; c < 20; c++) out[c] = 0;
    for (size_t i = 0; i < im.n(); i++) out[fuzzy::find_colour(im.hsv[3 * i], im.hsv[3 * i + 1], im.hsv[3 * i + 2])]++;
    for (int c = 0; c < 20; c++) out[c] /= (unsigned)(im.w * im.h);
}

// ---------------------------------------------------------------- plans
enum Alg { A_CHEBFOURIER, A_CHEB, A_ZERNIKE, A_HARALICK, A_MSHIST, A_TAMURA, A_COMB, A_RADON,
           A_FRACTAL, A_PIXSTATS, A_EDGEF, A_OBJ, A_INVOBJ, A_GABOR, A_GINI, A_COLORHIST, A_COUNT };
static const char *kAlgName[A_COUNT] = {
    "Chebyshev-Fourier Coefficients", "Chebyshev Coefficients", "Zernike Coefficients",
    "Haralick Textures", "Multiscale Histograms", "Tamura Textures", "Comb Moments",
    "Radon Coefficients", "Fractal Features", "Pixel Intensity Statistics", "Edge Features",
    "Otsu Object Features", "Inverse-Otsu Object Features", "Gabor Textures", "Gini Coefficient", "Color Histogram"};
static const int kAlgN[A_COUNT] = {32, 32, 72, 28, 24, 6, 48, 12, 20, 5, 28, 34, 34, 7, 1, 20};

typedef void (*AlgFn)(const Img &, double *);
static const AlgFn kAlgFn[A_COUNT] = {f_cheb_fourier, f_cheb_coeffs, f_zernike, f_haralick, f_mshist,
    f_tamura, f_comb, f_radon, f_fractal, f_pixstats, f_edge_features, f_objects, f_inv_objects,
    f_gabor, f_gini, f_color_hist};

// chain: transforms in application order, space-separated tokens ("Fourier Wavelet");
// the reference's "Color Transform" is the token "ColorTransform"
struct Group { int alg; std::string chain; };

static std::string display_name(const std::string &token) {
    return token == "ColorTransform" ? "Color Transform" : token;
}

static std::string chain_text(const std::string &chain) {
    // "Fourier Wavelet" (Fourier first) -> "(Wavelet (Fourier ()))"
    std::vector<std::string> t;
    size_t p = 0;
    while (p < chain.size()) {
        size_t q = chain.find(' ', p);
        if (q == std::string::npos) q = chain.size();
        if (q > p) t.push_back(chain.substr(p, q - p));
        p = q + 1;
    }
    std::string s = "()";
    for (auto &x : t) s = "(" + display_name(x) + " " + s + ")";
    return s;
}

// StdFeatureComputationPlans, src/Tasks.cpp:354-503.
static std::vector<Group> make_plan(int kind) {
    std::vector<Group> g;
    auto A = [&](const std::string &c) {
        for (int a : {A_EDGEF, A_OBJ, A_INVOBJ, A_GABOR}) g.push_back({a, c});
    };
    auto B = [&](const std::string &c) {
        for (int a : {A_CHEBFOURIER, A_CHEB, A_ZERNIKE}) g.push_back({a, c});
    };
    auto C = [&](const std::string &c) {
        for (int a : {A_COMB, A_HARALICK, A_MSHIST, A_TAMURA, A_RADON, A_FRACTAL, A_PIXSTATS, A_GINI})
            g.push_back({a, c});
    };
    // StdFeatureComputationPlans::addColorFeatures, src/Tasks.cpp:445-459
    auto colour = [&]() {
        g.push_back({A_COLORHIST, ""});
        B("ColorTransform"); C("ColorTransform");
        B("Hue"); C("Hue");
        B("Hue Fourier"); C("Hue Fourier");
        B("Hue Chebyshev"); C("Hue Chebyshev");
    };
    if (kind == 1 || kind == 3) {
        A(""); B(""); C("");
        if (kind == 3) colour();
        B("Fourier"); C("Fourier");
        B("Wavelet"); C("Wavelet");
        B("Chebyshev"); C("Chebyshev");
        C("Fourier Chebyshev");
        C("Fourier Wavelet");
        B("Wavelet Fourier"); C("Wavelet Fourier");
        C("Chebyshev Fourier");
        C("Wavelet Chebyshev");
        B("Edge"); C("Edge");
        B("Edge Fourier"); C("Edge Fourier");
        B("Edge Wavelet"); C("Edge Wavelet");
    } else {
        const Group s[] = {
            {A_CHEBFOURIER, ""}, {A_CHEBFOURIER, "Fourier"}, {A_CHEB, ""}, {A_CHEB, "Fourier"},
            {A_COMB, ""}, {A_COMB, "Chebyshev"}, {A_COMB, "Fourier Chebyshev"}, {A_COMB, "Fourier"},
            {A_COMB, "Wavelet"}, {A_COMB, "Fourier Wavelet"}, {A_EDGEF, ""}, {A_OBJ, ""}, {A_INVOBJ, ""},
            {A_GABOR, ""}, {A_HARALICK, ""}, {A_HARALICK, "Chebyshev"}, {A_HARALICK, "Fourier Chebyshev"},
            {A_HARALICK, "Fourier"}, {A_HARALICK, "Wavelet"}, {A_HARALICK, "Fourier Wavelet"},
            {A_MSHIST, ""}, {A_MSHIST, "Chebyshev"}, {A_MSHIST, "Fourier Chebyshev"}, {A_MSHIST, "Fourier"},
            {A_MSHIST, "Wavelet"}, {A_MSHIST, "Fourier Wavelet"}, {A_RADON, ""}, {A_RADON, "Chebyshev"},
            {A_RADON, "Fourier Chebyshev"}, {A_RADON, "Fourier"}, {A_TAMURA, ""}, {A_TAMURA, "Chebyshev"},
            {A_TAMURA, "Fourier Chebyshev"}, {A_TAMURA, "Fourier"}, {A_TAMURA, "Wavelet"},
            {A_TAMURA, "Fourier Wavelet"}, {A_ZERNIKE, ""}, {A_ZERNIKE, "Fourier"}};
        for (auto &x : s) g.push_back(x);
        if (kind == 2) colour();
    }
    return g;
}

struct PlanInfo {
    std::vector<Group> groups;
    std::vector<int> offset;
    std::vector<std::string> names;
    int n = 0;
};

// kind 0: short, 1: long, 2: short colour, 3: long colour
static const PlanInfo &plan_info(int kind) {
    static PlanInfo P[4];
    static std::once_flag once[4];
    if (kind < 0 || kind > 3) kind = 0;
    std::call_once(once[kind], [kind]() {
        PlanInfo &pi = P[kind];
        pi.groups = make_plan(kind);
        for (auto &g : pi.groups) {
            pi.offset.push_back(pi.n);
            std::string gname = std::string(kAlgName[g.alg]) + " " + chain_text(g.chain);
            for (int i = 0; i < kAlgN[g.alg]; i++) pi.names.push_back(gname + " [" + std::to_string(i) + "]");
            pi.n += kAlgN[g.alg];
        }
    });
    return P[kind];
}

static Img apply_transform(const std::string &t, const Img &in) {
    if (t == "ColorTransform") return in;  // the reference's EmptyTransform: a copy (colour plane included)
    if (t == "Hue") return hue_plane(in);
    if (t == "Color") return colour_plane(in);
    if (t == "Fourier") return fourier(in);
    if (t == "Chebyshev") return chebyshev(in, 0);
    if (t == "Wavelet") return wavelet(in);
    return edge(in);
}

// FeatureComputationPlanExecutor::run (src/Tasks.cpp:275-295): every
// transform chain computed once and cached by its key.
static void run_groups(const std::vector<Group> &groups, const std::vector<int> &offset, const Img &root,
                       double *out) {
    std::map<std::string, Img> cache;
    std::function<const Img &(const std::string &)> get = [&](const std::string &chain) -> const Img & {
        if (chain.empty()) return root;
        auto it = cache.find(chain);
        if (it != cache.end()) return it->second;
        size_t sp = chain.rfind(' ');
        std::string parent = (sp == std::string::npos) ? "" : chain.substr(0, sp);
        std::string last = (sp == std::string::npos) ? chain : chain.substr(sp + 1);
        Img r = apply_transform(last, get(parent));
        return cache.emplace(chain, std::move(r)).first->second;
    };
    for (size_t k = 0; k < groups.size(); k++) kAlgFn[groups[k].alg](get(groups[k].chain), out + offset[k]);
}

static Img make_img(const double *pix, int w, int h) {
    Img im(w, h);
    std::memcpy(im.p.data(), pix, sizeof(double) * (size_t)w * h);
    return im;
}

// ---------------------------------------------------------------- preprocessing
// ImageMatrix::submatrix (src/cmatrix.cpp:414-470): rows y1..y2, columns
// x1..x2 of `in`; false (nothing copied) when x2 or y2 lies outside.
static bool submatrix(const Img &in, unsigned x1, unsigned y1, unsigned x2, unsigned y2, Img &out) {
    if (x2 >= (unsigned)in.w || y2 >= (unsigned)in.h || x2 < x1 || y2 < y1) return false;
    Img o((int)(x2 - x1 + 1), (int)(y2 - y1 + 1));
    for (int y = 0; y < o.h; y++)
        for (int x = 0; x < o.w; x++) o.at(y, x) = in.at((int)y1 + y, (int)x1 + x);
    out = o;
    return true;
}

// ImageMatrix::normalize (src/cmatrix.cpp:836-888).  mean() and std() are the
// Moments2 of the current pixels in raster order (UpdateStats, :803-811).
static void normalize(Img &im, double n_min, double n_max, long n_range, double n_mean, double n_std, int bits) {
    if (n_min >= 0 && n_max > 0 && n_range > 0) {
        double norm_fact = n_range / (n_max - n_min);
        for (double &v : im.p) {
            double val = v;
            if (val < n_min) val = 0;
            else if (val > n_max) val = n_range;
            else val = norm_fact * (val - n_min);
            v = val;
        }
    }
    if (n_mean > 0) {
        Moments2 st = stats_of(im);
        double d_mean = st.mean - n_mean, std_fact = (n_std > 0 ? n_std : 0) / st.std_();
        double max_range = std::pow((double)2, bits) - 1;
        for (double &v : im.p) {
            double val = v - d_mean;
            if (n_std > 0) val = n_mean + (val - n_mean) * std_fact;
            if (val < 0) val = 0;
            else if (val > max_range) val = max_range;
            v = val;
        }
    }
}

// ImageMatrix::Rotate (src/cmatrix.cpp:727-769): 90 = transpose, then each row
// reversed; 180 = both axes reversed; 270 = the transpose.
static Img rotate(const Img &in, int quarter) {
    if (quarter == 2) {
        Img o(in.w, in.h);
        for (int y = 0; y < in.h; y++)
            for (int x = 0; x < in.w; x++) o.at(y, x) = in.at(in.h - 1 - y, in.w - 1 - x);
        return o;
    }
    Img o(in.h, in.w);
    for (int y = 0; y < o.h; y++)
        for (int x = 0; x < o.w; x++) o.at(y, x) = quarter == 1 ? in.at(in.h - 1 - x, y) : in.at(x, y);
    return o;
}

// ImageMatrix::OpenImage's preprocessing (src/cmatrix.cpp:252-294) and the
// sample cut of TrainingSet::AddImageFile (src/wndchrm_src/TrainingSet.cpp:1455-1481).
// opt: crop x, y, w, h; downsample x, y ratios; normalize min, max, range,
// mean, std; rotations; tiles x, y.  Returns -1 where the reference's
// submatrix refuses the rectangle.
static int preprocess(const Img &src, int bits, const double *opt, int sample, Img &out) {
    const int cx = (int)opt[0], cy = (int)opt[1], cw = (int)opt[2], ch = (int)opt[3];
    const double dsx = opt[4], dsy = opt[5];
    const int rotations = (int)opt[11], tiles_x = (int)opt[12], tiles_y = (int)opt[13];
    if (rotations < 1 || rotations > 4 || tiles_x < 1 || tiles_y < 1 || !(dsx > 0) || !(dsy > 0)) return -1;
    const int tiles = tiles_x * tiles_y;
    if (sample < 0 || sample >= rotations * tiles) return -1;
    Img im = src;
    if (cx >= 0) {
        if (cy < 0 || cw < 1 || ch < 1) return -1;
        Img c;
        if (!submatrix(src, (unsigned)cx, (unsigned)cy, (unsigned)cx + cw - 1, (unsigned)cy + ch - 1, c)) return -1;
        im = c;
    }
    if (!(dsx >= 1 && dsy >= 1)) {
        im = downsample(im, dsx, dsy);
        if (im.w < 1 || im.h < 1) return -1;
    }
    normalize(im, opt[6], opt[7], (long)opt[8], opt[9], opt[10], bits);
    const int rot = sample / tiles, rem = sample % tiles, ix = rem / tiles_y, iy = rem % tiles_y;
    Img r = rot ? rotate(im, rot) : im;
    if (tiles == 1) {
        out = r;
        return 0;
    }
    long tx, ty;
    if (rot == 1 || rot == 3) {
        ty = (long)(r.w / tiles_x);
        tx = (long)(r.h / tiles_y);
    } else {
        tx = (long)(r.w / tiles_x);
        ty = (long)(r.h / tiles_y);
    }
    if (!submatrix(r, (unsigned)(ix * tx), (unsigned)(iy * ty), (unsigned)((ix + 1) * tx - 1),
                   (unsigned)((iy + 1) * ty - 1), out))
        return -1;
    return 0;
}

// parse "Alg (T2 (T1 ()))" into a Group
static bool parse_group(const std::string &s, Group &g) {
    size_t p = s.find(" (");
    if (p == std::string::npos) return false;
    std::string alg = s.substr(0, p);
    g.alg = -1;
    for (int a = 0; a < A_COUNT; a++) if (alg == kAlgName[a]) g.alg = a;
    if (g.alg < 0) return false;
    std::vector<std::string> t;
    std::string rest = s.substr(p + 1);
    while (rest.size() > 2 && rest[0] == '(' && rest[1] != ')') {
        if (rest.compare(0, 17, "(Color Transform ") == 0) {
            t.push_back("ColorTransform");
            rest = rest.substr(17);
            continue;
        }
        size_t q = rest.find(' ');
        t.push_back(rest.substr(1, q - 1));
        rest = rest.substr(q + 1);
    }
    g.chain.clear();
    for (int i = (int)t.size() - 1; i >= 0; i--) g.chain += (g.chain.empty() ? "" : " ") + t[i];
    return true;
}

// ---------------------------------------------------------------- WND-5
// TrainingSet::normalize + SetFisherScores: X (N x F, a copy of the training
// rows) normalised in place; weights thresholded at rank floor(frac*F + 0.5).
static void wnd_fit_rows(std::vector<double> &X, int N, int F, const int *labels, int C, double frac,
                         double *weights, double *mins, double *maxs) {
    // TrainingSet::normalize, src/wndchrm_src/TrainingSet.cpp:2090-2123
    for (int f = 0; f < F; f++) {
        double mn = FLT_MAX, mx = -FLT_MAX;
        for (int s = 0; s < N; s++) {
            double v = X[(size_t)s * F + f];
            if (std::isnan(v) || v > FLT_MAX || v < -FLT_MAX) continue;
            if (v > mx) mx = v;
            if (v < mn) mn = v;
        }
        maxs[f] = mx;
        mins[f] = mn;
        for (int s = 0; s < N; s++) {
            double v = X[(size_t)s * F + f];
            if (std::isnan(v) || v < mn || (mx - mn) < DBL_EPSILON) v = 0;
            else if (v > mx) v = 100;
            else v = 100 * ((v - mn) / (mx - mn));
            X[(size_t)s * F + f] = v;
        }
    }
    // TrainingSet::SetFisherScores (Fisher part), TrainingSet.cpp:2183-2324
    std::vector<Moments2> cs(C + 1);
    for (int f = 0; f < F; f++) {
        Moments2 fs;
        for (int c = 1; c <= C; c++) cs[c].reset();
        for (int s = 0; s < N; s++) {
            int c = labels[s];
            if (c) { double v = X[(size_t)s * F + f]; fs.add(v); cs[c].add(v); }
        }
        double dev = 0, var = 0;
        for (int c = 1; c <= C; c++) { dev += std::pow(cs[c].mean - fs.mean, 2); var += cs[c].var(); }
        if (C > 1) { dev /= (C - 1); var /= C; } else dev = 0;
        if (var < 0.000001) var = 0.000001;
        weights[f] = dev / var;
    }
    int last = (int)std::floor((frac * (double)F) + 0.5);
    if (last < F) {
        std::vector<double> sw(weights, weights + F);
        std::nth_element(sw.begin(), sw.begin() + last, sw.end(), std::greater<double>());
        double thr = sw[last];
        for (int f = 0; f < F; f++) if (weights[f] < thr) weights[f] = 0.0;
    }
}

// signatures::normalize + classify2 for test rows [q0, q1) against the
// normalised training rows X.
static void wnd_classify_rows(const std::vector<double> &X, int N, int F, const int *labels, int C,
                              const double *weights, const double *mins, const double *maxs, const double *test,
                              int q0, int q1, double *probs, int *pred, double *norms) {
    // signatures::normalize + TrainingSet::classify2, signatures.cpp:196-215,
    // TrainingSet.cpp:2429-2536
    std::vector<double> t(F), csim(C + 1), ncnt(C + 1);
    for (int q = q0; q < q1; q++) {
        for (int f = 0; f < F; f++) {
            double v = test[(size_t)q * F + f];
            if (std::isnan(v) || v < mins[f] || (maxs[f] - mins[f]) < DBL_EPSILON) v = 0;
            else if (v > maxs[f]) v = 100;
            else v = 100 * ((v - mins[f]) / (maxs[f] - mins[f]));
            t[f] = v;
        }
        std::fill(csim.begin(), csim.end(), 0.0);
        std::fill(ncnt.begin(), ncnt.end(), 0.0);
        for (int s = 0; s < N; s++) {
            double d = 0.0;
            for (int f = 0; f < F; f++) {
                if (weights[f] < DBL_EPSILON) continue;
                double dist = std::fabs(t[f] - X[(size_t)s * F + f]);
                if (dist < DBL_EPSILON) continue;
                d += std::pow(weights[f], 2) * std::pow(dist, 2);
            }
            if (d < DBL_EPSILON) continue;
            csim[labels[s]] += std::pow(d, -5);
            ncnt[labels[s]] += 1;
        }
        long best = -1;
        double bestv = 0, tot = 0;
        for (int c = 1; c <= C; c++) {
            if (ncnt[c] == 0) continue;
            csim[c] /= ncnt[c];
            if (csim[c] > bestv) { bestv = csim[c]; best = c; }
        }
        for (int c = 1; c <= C; c++) tot += csim[c];
        for (int c = 1; c <= C; c++) probs[(size_t)q * C + c - 1] = csim[c] / tot;
        pred[q] = (int)best;
        if (norms) norms[q] = tot;
    }
}


static void wnd_run(const double *train, int N, int F, const int *labels, int C, double frac,
                    const double *test, int T, double *weights, double *mins, double *maxs,
                    double *probs, int *pred, double *norms = nullptr) {
    std::vector<double> X(train, train + (size_t)N * F);
    wnd_fit_rows(X, N, F, labels, C, frac, weights, mins, maxs);
    wnd_classify_rows(X, N, F, labels, C, weights, mins, maxs, test, 0, T, probs, pred, norms);
}

// TrainingSet::ClassifyImage, WND branch (src/wndchrm_src/TrainingSet.cpp:1603-1800),
// rank 1, no ground truth: per image the `tiles` consecutive rows' marginal
// probabilities accumulated as p / tiles in tile order; with max_tile a tile
// whose share probabilities[pred] / (sum of the other entries 0..C) is the
// largest so far overwrites the sums (entry 0, which classify2 never sets, is
// taken as 0); the class of the largest sum; the mean normalisation factor.
static void classify_images(const double *probs, const int *pred, const double *norms, int n_img, int tiles, int C,
                            int max_tile, double *iprobs, int *ipred, double *inorm) {
    std::vector<double> probabilities(C + 1), probabilities_sum(C + 1);
    for (int g = 0; g < n_img; g++) {
        int predicted_class = 0, most_similar_predicted_class = 0;
        double max_tile_similarity = 0.0, sum_prob = 0.0, normalization_factor_avg = 0;
        for (int c = 1; c <= C; c++) probabilities_sum[c] = 0.0;
        for (int k = 0; k < tiles; k++) {
            const size_t t = (size_t)g * tiles + k;
            probabilities[0] = 0.0;
            for (int c = 1; c <= C; c++) probabilities[c] = probs[t * C + c - 1];
            predicted_class = pred[t];
            if (predicted_class < 1) predicted_class = 0;
            if (max_tile) {
                sum_prob = 0.0;
                for (int c = 0; c <= C; c++)
                    if (c != predicted_class) sum_prob += probabilities[c];
                if (probabilities[predicted_class] / sum_prob > max_tile_similarity) {
                    max_tile_similarity = probabilities[predicted_class] / sum_prob;
                    most_similar_predicted_class = predicted_class;
                }
            }
            for (int c = 1; c <= C; c++) {
                if (max_tile && max_tile_similarity == probabilities[predicted_class] / sum_prob)
                    probabilities_sum[c] = probabilities[c];
                else
                    probabilities_sum[c] += (probabilities[c] / (double)tiles);
            }
            normalization_factor_avg += norms[t];
        }
        if (max_tile) predicted_class = most_similar_predicted_class;
        normalization_factor_avg /= tiles;
        if (C > 1) {
            double max = 0.0;
            for (int c = 1; c <= C; c++)
                if (probabilities_sum[c] > max) {
                    max = probabilities_sum[c];
                    predicted_class = c;
                }
        }
        for (int c = 1; c <= C; c++) iprobs[(size_t)g * C + c - 1] = probabilities_sum[c];
        ipred[g] = predicted_class;
        inorm[g] = normalization_factor_avg;
    }
}

}  // namespace wco

using namespace wco;

extern "C" {

int wco_plan_n_features(int kind) { return plan_info(kind).n; }

int wco_plan_feature_name(int kind, int i, char *buf, int buflen) {
    const PlanInfo &pi = plan_info(kind);
    if (i < 0 || i >= pi.n) return -1;
    std::strncpy(buf, pi.names[i].c_str(), (size_t)buflen - 1);
    buf[buflen - 1] = 0;
    return (int)pi.names[i].size();
}

int wco_extract_std(int kind, const double *pix, int w, int h, int bits, double *out) {
    (void)bits;
    const PlanInfo &pi = plan_info(kind);
    Img root = make_img(pix, w, h);
    run_groups(pi.groups, pi.offset, root, out);
    return pi.n;
}

int wco_extract_std_batch(int kind, const double *pix, const long *offs, const int *ws, const int *hs,
                          int n, int bits, double *out, int nthreads) {
    const PlanInfo &pi = plan_info(kind);
    if (nthreads < 1) nthreads = 1;
    std::atomic<int> next(0);
    auto worker = [&]() {
        for (;;) {
            int i = next.fetch_add(1);
            if (i >= n) break;
            wco_extract_std(kind, pix + offs[i], ws[i], hs[i], bits, out + (size_t)i * pi.n);
        }
    };
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; t++) th.emplace_back(worker);
    for (auto &t : th) t.join();
    return pi.n;
}

// Colour: an RGB image (interleaved 8- or 16-bit samples) through a plan.
int wco_extract_rgb(int kind, const void *rgb, int w, int h, int bits, double *out) {
    const PlanInfo &pi = plan_info(kind);
    Img root = make_rgb_img(rgb, w, h, bits);
    run_groups(pi.groups, pi.offset, root, out);
    return pi.n;
}

int wco_load_rgb(const void *rgb, int w, int h, int bits, double *gray, unsigned char *hsv) {
    Img im = make_rgb_img(rgb, w, h, bits);
    std::memcpy(gray, im.p.data(), sizeof(double) * im.n());
    std::memcpy(hsv, im.hsv.data(), im.hsv.size());
    return 0;
}

int wco_find_colour(int h, int s, int v) { return fuzzy::find_colour(h, s, v); }

int wco_extract_group(const char *group, const double *pix, int w, int h, int bits, double *out) {
    (void)bits;
    Group g;
    if (!parse_group(group, g)) return -1;
    std::vector<Group> gs(1, g);
    std::vector<int> off(1, 0);
    Img root = make_img(pix, w, h);
    run_groups(gs, off, root, out);
    return kAlgN[g.alg];
}

int wco_transform(const char *name, const double *pix, int w, int h, double *out, int *ow, int *oh) {
    std::string t(name);
    if (t != "Fourier" && t != "Chebyshev" && t != "Wavelet" && t != "Edge") return -1;
    Img r = apply_transform(t, make_img(pix, w, h));
    *ow = r.w;
    *oh = r.h;
    std::memcpy(out, r.p.data(), sizeof(double) * r.n());
    return 0;
}

int wco_preprocess(const double *pix, int w, int h, int bits, const double *opt, int sample, double *out,
                   long cap, int *ow, int *oh) {
    Img o;
    if (preprocess(make_img(pix, w, h), bits, opt, sample, o)) return -1;
    if ((long)o.n() > cap) return -2;
    *ow = o.w;
    *oh = o.h;
    std::memcpy(out, o.p.data(), sizeof(double) * o.n());
    return 0;
}

int wco_wnd_images(const double *train, int N, int F, const int *labels, int C, double frac, const double *test,
                   int n_img, int tiles, int max_tile, double *iprobs, int *ipred, double *inorm) {
    const int T = n_img * tiles;
    std::vector<double> w(F), mn(F), mx(F), p((size_t)T * C), nf(T);
    std::vector<int> pr(T);
    wnd_run(train, N, F, labels, C, frac, test, T, w.data(), mn.data(), mx.data(), p.data(), pr.data(), nf.data());
    classify_images(p.data(), pr.data(), nf.data(), n_img, tiles, C, max_tile, iprobs, ipred, inorm);
    return 0;
}

int wco_haralick_tones(const double *pix, int w, int h) {
    Img im = make_img(pix, w, h);
    Moments2 s = stats_of(im);
    double scale = 255.0 / (s.mx - s.mn);
    bool seen[256] = {false};
    for (double v : im.p) {
        double q = (v - s.mn) * scale;
        seen[std::isfinite(q) ? (uint8_t)q : 0] = true;
    }
    int n = 0;
    for (bool b : seen) n += b;
    return n;
}

int wco_wnd(const double *train, int N, int F, const int *labels, int C, double frac, const double *test,
            int T, double *weights, double *mins, double *maxs, double *probs, int *pred) {
    wnd_run(train, N, F, labels, C, frac, test, T, weights, mins, maxs, probs, pred);
    return 0;
}

// WND-5 as wndchrm runs it over many test rows: one fit, then the test rows
// split into nthreads contiguous ranges classified concurrently (the
// reference's one process per test split, without repeating the fit).
// Returns the fit's and the classification's wall seconds in secs[0..1].
int wco_wnd_mt(const double *train, int N, int F, const int *labels, int C, double frac, const double *test, int T,
               double *weights, double *mins, double *maxs, double *probs, int *pred, int nthreads, double *secs) {
    auto t0 = std::chrono::steady_clock::now();
    std::vector<double> X(train, train + (size_t)N * F);
    wnd_fit_rows(X, N, F, labels, C, frac, weights, mins, maxs);
    auto t1 = std::chrono::steady_clock::now();
    if (nthreads < 1) nthreads = 1;
    std::vector<std::thread> th;
    for (int k = 0; k < nthreads; k++) {
        const int q0 = (int)((long long)T * k / nthreads), q1 = (int)((long long)T * (k + 1) / nthreads);
        th.emplace_back([&, q0, q1] {
            wnd_classify_rows(X, N, F, labels, C, weights, mins, maxs, test, q0, q1, probs, pred, nullptr);
        });
    }
    for (auto &t : th) t.join();
    auto t2 = std::chrono::steady_clock::now();
    if (secs) {
        secs[0] = std::chrono::duration<double>(t1 - t0).count();
        secs[1] = std::chrono::duration<double>(t2 - t1).count();
    }
    return 0;
}

}  // extern "C"
