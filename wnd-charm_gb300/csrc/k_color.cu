// Colour images and the colour feature plans: RGB ingest (gray plane + HSV
// colour plane), the fuzzy colour classifier, the "Color", "Hue" and
// "Color Transform" transforms, and the Color Histogram family.
//
// ImageMatrix::LoadTIFF's RGB path (src/cmatrix.cpp:85-203) with RGB2GRAY and
// RGB2HSV (src/cmatrix.h:95-160); FindColor / CalculateRules2 / color_value and
// the saturation / value membership functions (src/colors/FuzzyCalc.cpp:625-834,
// constants src/colors/FuzzyCalc.h:42-148); ImageMatrix::ColorTransform and
// HueTransform (src/cmatrix.cpp:1023-1066); ColorHistogram
// (src/FeatureAlgorithms.cpp:502-534).  FP64 in the reference's order of
// operations; this file is built without multiply-add contraction.
#include <cfloat>
#include <cmath>
#include <vector>

#include "kcommon.cuh"
#include "kernels.h"

namespace wc {

// ---------------------------------------------------------------- fuzzy colours
// The reference's rule base is a complete grid: for each of 10 hue membership
// functions (trapezoids named by colour), 6 saturation classes (grey, almost
// grey, tend grey, medium grey, tend clear, clear) and 5 value classes (dark,
// almost dark, tend dark, tend light, light), one output colour.  Colour codes:
// 1 white, 2 light grey, 3 dark grey, 4 black, 5 red, 6 pink, 7 dark brown,
// 8 light brown, 9 dark orange, 10 light orange, 11 yellow, 12 olive,
// 13 light green, 14 dark green, 15 teal, 16 aqua, 17 blue, 18 dark fuchsia,
// 19 light fuchsia.  Code 0: the two rules whose colour names the reference
// misspells, which no colour's sum includes.
#define FZ_HUES 10
#define FZ_SATS 6
#define FZ_VALS 5
__constant__ unsigned char c_rule_colour[FZ_HUES * FZ_SATS * FZ_VALS] = {
    /* red          */ 4, 4, 3, 2, 1, 4, 3, 3, 19, 6, 4, 7, 18, 6, 6, 4, 7, 8, 19, 6, 4, 7, 7, 5, 5, 4, 4, 5, 5, 5,
    /* dark orange  */ 4, 3, 3, 2, 1, 4, 3, 3, 2, 1, 4, 7, 3, 8, 6, 4, 7, 7, 8, 10, 4, 7, 7, 8, 9, 4, 7, 7, 8, 9,
    /* light orange */ 4, 3, 3, 2, 1, 4, 3, 3, 2, 1, 4, 3, 3, 2, 10, 4, 7, 8, 8, 10, 4, 7, 8, 8, 10, 4, 7, 8, 8, 10,
    /* yellow       */ 4, 3, 3, 2, 1, 4, 3, 3, 2, 1, 4, 3, 12, 12, 11, 4, 12, 12, 12, 11, 4, 12, 12, 12, 11, 4, 12, 12, 12, 11,
    /* light green  */ 4, 3, 3, 2, 1, 4, 3, 3, 2, 1, 4, 12, 12, 13, 13, 4, 14, 14, 13, 13, 4, 14, 14, 13, 13, 4, 14, 14, 13, 13,
    /* dark green   */ 4, 3, 3, 2, 1, 4, 3, 3, 13, 13, 4, 14, 14, 13, 13, 4, 14, 14, 13, 13, 4, 14, 14, 13, 13, 4, 14, 14, 13, 13,
    /* aqua         */ 4, 3, 3, 2, 1, 4, 3, 3, 15, 16, 4, 15, 17, 17, 16, 4, 15, 17, 16, 16, 4, 15, 17, 16, 16, 4, 15, 15, 16, 16,
    /* blue         */ 4, 3, 3, 2, 1, 4, 3, 0, 16, 16, 4, 18, 0, 19, 16, 4, 17, 17, 17, 17, 4, 17, 17, 17, 17, 4, 17, 17, 17, 17,
    /* dark fuchsia */ 4, 3, 3, 2, 1, 4, 3, 18, 19, 19, 4, 18, 18, 19, 19, 4, 18, 18, 19, 19, 4, 18, 18, 19, 19, 4, 7, 18, 18, 19,
    /* light fuchsia*/ 4, 3, 3, 2, 1, 4, 3, 2, 19, 19, 4, 18, 18, 19, 19, 4, 18, 18, 19, 19, 4, 7, 18, 19, 19, 4, 7, 18, 18, 19,
};

// Membership tables for 8-bit h, s, v (host-made, identical to evaluating the
// reference's functions on the same doubles): hue[10][256] in the rule grid's
// hue order (red, dark orange, light orange, yellow, light green, dark green,
// aqua, blue, dark fuchsia, light fuchsia), then sat[6][256], then val[5][256].
std::vector<double> fuzzy_membership_table() {
    // color_value's trapezoids (colour, start, max1, max2, end); red has two
    struct Trap { int colour; double start, max1, max2, end; };
    static const Trap traps[11] = {{5, 0, 0, 0, 11},      {9, 0, 17, 17, 27},     {10, 20, 27, 27, 37},
                                   {11, 27, 39, 39, 47},  {13, 40, 50, 50, 80},   {14, 50, 80, 80, 120},
                                   {16, 80, 120, 120, 160}, {17, 120, 160, 160, 200}, {18, 160, 200, 200, 220},
                                   {19, 200, 220, 220, 230}, {5, 220, 240, 240, 240}};
    static const int hue_colour[FZ_HUES] = {5, 9, 10, 11, 13, 14, 16, 17, 18, 19};
    // color_value: the first trapezoid of the colour that gives a positive value
    auto colour_value = [&](int colour, double x) {
        double res = 0;
        for (const Trap &t : traps) {
            if (t.colour != colour) continue;
            if (x < t.start || x > t.end) res = 0;
            else if (x >= t.max1 && x <= t.max2) res = 1;
            else if (x < t.max1) res = (x - t.start) / (t.max1 - t.start);
            else res = 1 - (x - t.max2) / (t.end - t.max2);
            if (res > 0) return res;
        }
        return res;
    };
    // a triangle (start, max, end): rising below max, falling from max on
    // (at max itself the falling branch, except where `top_inclusive` puts max on
    // the rising branch, as the "clear" and "light" functions do)
    auto tri = [](double x, double start, double max, double end, bool top_inclusive, double minimum) {
        if (x < minimum) return 0.0;
        if (x < start || x > end) return 0.0;
        if (top_inclusive ? x <= max : x < max) return (x - start) / (max - start);
        return 1 - ((x - max) / (end - max));
    };
    const double NO_MIN = -DBL_MAX;
    std::vector<double> t((FZ_HUES + FZ_SATS + FZ_VALS) * 256);
    for (int x = 0; x < 256; x++) {
        const double v = x;
        for (int k = 0; k < FZ_HUES; k++) t[k * 256 + x] = colour_value(hue_colour[k], v);
        double *s = t.data() + FZ_HUES * 256;
        s[0 * 256 + x] = tri(v, -0.1, 0, 40, false, 0);     // grey (MIN_GREY 0)
        s[1 * 256 + x] = tri(v, 10, 30, 70, false, NO_MIN);  // almost grey
        s[2 * 256 + x] = tri(v, 30, 70, 120, false, NO_MIN); // tend grey
        s[3 * 256 + x] = tri(v, 60, 120, 180, false, NO_MIN);
        s[4 * 256 + x] = tri(v, 120, 180, 240, false, NO_MIN);
        s[5 * 256 + x] = tri(v, 180, 240, 240.1, true, NO_MIN);  // clear
        double *w = s + FZ_SATS * 256;
        w[0 * 256 + x] = tri(v, -0.1, 0, 60, false, 0);      // dark (MIN_DARK 0)
        w[1 * 256 + x] = tri(v, 0, 60, 120, false, NO_MIN);   // almost dark
        w[2 * 256 + x] = tri(v, 60, 120, 180, false, NO_MIN);
        w[3 * 256 + x] = tri(v, 120, 180, 240, false, NO_MIN);
        w[4 * 256 + x] = tri(v, 200, 240, 240.1, true, NO_MIN);  // light
    }
    return t;
}

// FindColor: per colour the rules' products hue * sat * value summed in rule
// order (a hue factor of 0, or a hue * sat product of 0, skips the rule), then
// the colour with the largest sum (the first on ties; light grey when every
// sum is 0).  One pass over the grid keeps each colour's summation order.
__device__ int find_colour(int h, int s, int v, const double *__restrict__ tab) {
    double sum[20];
#pragma unroll
    for (int c = 0; c < 20; c++) sum[c] = 0;
    const double *sat = tab + FZ_HUES * 256, *val = sat + FZ_SATS * 256;
#pragma unroll
    for (int hf = 0; hf < FZ_HUES; hf++) {
        const double cv = tab[hf * 256 + h];
        if (cv == 0) continue;
#pragma unroll
        for (int k = 0; k < FZ_SATS; k++) {
            const double r1 = cv * sat[k * 256 + s];
            if (r1 == 0) continue;
#pragma unroll
            for (int j = 0; j < FZ_VALS; j++) {
                const int c = c_rule_colour[(hf * FZ_SATS + k) * FZ_VALS + j];
                const double r2 = r1 * val[j * 256 + v];
#pragma unroll
                for (int q = 1; q < 20; q++)
                    if (q == c) sum[q] = sum[q] + r2;
            }
        }
    }
    int best = 2;
    double mx = 0;
#pragma unroll
    for (int c = 1; c < 20; c++)
        if (sum[c] > mx) {
            mx = sum[c];
            best = c;
        }
    return best;
}

// ---------------------------------------------------------------- RGB ingest
__device__ __forceinline__ unsigned char to_byte(double x) {
    // (unsigned char) of a double in [0, 256); NaN (a flat 16-bit image's 0 * inf)
    // gives 0, as the x86-64 reference build converts it
    return x == x ? (unsigned char)(int)x : (unsigned char)0;
}

// RGB2HSV (src/cmatrix.h:95-124): bytes h, s, v in 0..240
__device__ void rgb_to_hsv(int R, int G, int B, unsigned char *o) {
    const double r = (double)R / 255, g = (double)G / 255, b = (double)B / 255;
    const double mgb = g > b ? g : b, ngb = g < b ? g : b;
    const double max = r > mgb ? r : mgb, min = r < ngb ? r : ngb;
    const double delta = max - min;
    const unsigned char v = (unsigned char)(int)(max * 240.0);
    const unsigned char s = max != 0.0 ? (unsigned char)(int)((delta / max) * 240.0) : (unsigned char)0;
    unsigned char hh = 0;
    if (s != 0) {
        double h = 0;
        if (r == max) h = (g - b) / delta;
        else if (g == max) h = 2 + (b - r) / delta;
        else if (b == max) h = 4 + (r - g) / delta;
        h *= 60.0;
        if (h >= 360) h -= 360.0;
        if (h < 0.0) h += 360.0;
        const double k = 240.0 / 360.0;
        hh = (unsigned char)(int)(h * k);
    }
    o[0] = hh;
    o[1] = s;
    o[2] = v;
}

// One CTA per image: 16-bit samples are first scaled to 8 bits over the
// image's RGB range ((x - min) * (255 / (max - min)), truncated); then the gray
// plane is 0.2989 r + 0.5870 g + 0.1140 b and the colour plane HSV.
__global__ void __launch_bounds__(1024) k_rgb_ingest(const void *__restrict__ src, int bits16, long long n,
                                                     double *__restrict__ gray, unsigned char *__restrict__ hsv) {
    __shared__ double sh[32];
    double lo = 0, scale = 0;
    if (bits16) {
        const unsigned short *p = (const unsigned short *)src;
        double mn = DBL_MAX, mx = -DBL_MAX;
        for (long long i = threadIdx.x; i < 3 * n; i += blockDim.x) {
            const double v = p[i];
            mn = fmin(mn, v);
            mx = fmax(mx, v);
        }
        lo = block_min(mn, sh);
        const double hi = block_max(mx, sh);
        scale = 255.0 / (hi - lo);
    }
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        int c[3];
        if (bits16) {
            const unsigned short *p = (const unsigned short *)src + 3 * i;
            for (int k = 0; k < 3; k++) c[k] = to_byte(((double)p[k] - lo) * scale);
        } else {
            const unsigned char *p = (const unsigned char *)src + 3 * i;
            for (int k = 0; k < 3; k++) c[k] = p[k];
        }
        gray[i] = 0.2989 * c[0] + 0.5870 * c[1] + 0.1140 * c[2];
        rgb_to_hsv(c[0], c[1], c[2], hsv + 3 * i);
    }
}

void launch_rgb_ingest(Ctx &c, const void *src, int dtype, long long n, double *gray, unsigned char *hsv) {
    WC_LAUNCH(c);
    k_rgb_ingest<<<1, 1024, 0, c.st>>>(src, dtype == WC_RGB16, n, gray, hsv);
}

// ---------------------------------------------------------------- transforms
// X_CTCOPY: a copy of the source plane (the reference's plans name a "Color
// Transform" that is not registered, so its lookup yields an EmptyTransform,
// which copies); X_HUE: the hue byte (HueTransform); X_COLOR: the fuzzy colour
// index as an 8-bit level, int(255 * colour / 19) (ColorTransform).
__global__ void k_color_xf(double *__restrict__ arena, const Plane *__restrict__ planes, const TJob *__restrict__ jobs,
                           int xf, int nn, const unsigned char *__restrict__ clr, const long long *__restrict__ clr_off,
                           const double *__restrict__ tab) {
    const TJob J = jobs[blockIdx.z];
    const Plane S = planes[J.src], D = planes[J.dst];
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= S.w || y >= S.h) return;
    const long long i = (long long)y * S.w + x;
    double out;
    if (xf == X_CTCOPY) {
        out = arena[S.off + i];
    } else {
        const unsigned char *p = clr + clr_off[J.dst / nn] + 3 * i;
        if (xf == X_HUE) out = p[0];
        else out = (double)(int)((255.0 * (double)find_colour(p[0], p[1], p[2], tab)) / 19);
    }
    arena[D.off + i] = out;
}

void launch_color_xf(Ctx &c, double *arena, const Plane *planes, const TJob *jobs, int njobs, int maxw, int maxh, int xf,
                     int nn, const unsigned char *clr, const long long *clr_off, const double *tab) {
    if (njobs <= 0) return;
    dim3 b(32, 8), g((maxw + 31) / 32, (maxh + 7) / 8, njobs);
    WC_LAUNCH(c);
    k_color_xf<<<g, b, 0, c.st>>>(arena, planes, jobs, xf, nn, clr, clr_off, tab);
}

// ---------------------------------------------------------------- Color Histogram
// 20 bins (index 0 never filled) of the fuzzy colour of every pixel, each
// divided by width * height.  One CTA per job, integer counts in shared memory.
__global__ void __launch_bounds__(256) k_color_hist(const Plane *__restrict__ planes, const FJob *__restrict__ jobs,
                                                    const unsigned char *__restrict__ clr,
                                                    const long long *__restrict__ clr_off, const double *__restrict__ tab,
                                                    double *__restrict__ feat) {
    __shared__ unsigned int cnt[20];
    const FJob J = jobs[blockIdx.x];
    const Plane P = planes[J.plane];
    if (threadIdx.x < 20) cnt[threadIdx.x] = 0;
    __syncthreads();
    const long long n = (long long)P.w * P.h;
    const unsigned char *p = clr + clr_off[J.img];
    for (long long i = threadIdx.x; i < n; i += blockDim.x)
        atomicAdd(&cnt[find_colour(p[3 * i], p[3 * i + 1], p[3 * i + 2], tab)], 1u);
    __syncthreads();
    if (threadIdx.x < 20) feat[J.out + threadIdx.x] = (double)cnt[threadIdx.x] / (double)(unsigned)(P.w * P.h);
}

void launch_color_hist(Ctx &c, const Plane *planes, const FJob *jobs, int njobs, const unsigned char *clr,
                       const long long *clr_off, const double *tab, double *feat) {
    if (njobs <= 0) return;
    WC_LAUNCH(c);
    k_color_hist<<<njobs, 256, 0, c.st>>>(planes, jobs, clr, clr_off, tab, feat);
}

}  // namespace wc
