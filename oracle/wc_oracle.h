// TEST INFRASTRUCTURE ONLY: the CPU oracle for the WND-CHARM hot path.
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
// load it, and only as a checker / baseline.  The shipped GPU library never
// links or calls it.
//
// It restates, in plain C++ written for this project, the reference
// algorithms of the feature-extraction DAG and of WND-5; every function in
// wc_oracle.cpp cites the reference file:line it follows.  It is pinned
// against the reference's golden fixtures and against the unmodified
// reference library built by oracle/build_ref.sh (tests/test_oracle_*.py).
#pragma once
#ifdef __cplusplus
extern "C" {
#endif

// Standard plans: 0 = short (1059 features), 1 = long (2919 features).
int wco_plan_n_features(int kind);
int wco_plan_feature_name(int kind, int i, char *buf, int buflen);

// Whole plan on one grayscale image (row-major doubles, width w, height h).
int wco_extract_std(int kind, const double *pix, int w, int h, int bits, double *out);

// Whole plan, many images, run on nthreads host threads (one image each).
// pix_offsets[i] indexes pix; out is n x n_features.
int wco_extract_std_batch(int kind, const double *pix, const long *pix_offsets,
                          const int *ws, const int *hs, int n, int bits,
                          double *out, int nthreads);

// Colour: an RGB image (interleaved r, g, b; bits 8 or 16) read as LoadTIFF
// reads a 3-sample TIFF (gray plane + HSV colour plane), then a plan (kinds 0-3;
// 2 = short colour, 3 = long colour).  wco_load_rgb gives the two planes
// (hsv: 3 bytes per pixel); wco_find_colour the fuzzy colour (1..19) of h, s, v.
int wco_extract_rgb(int kind, const void *rgb, int w, int h, int bits, double *out);
int wco_load_rgb(const void *rgb, int w, int h, int bits, double *gray, unsigned char *hsv);
int wco_find_colour(int h, int s, int v);

// One group by reference name, e.g. "Zernike Coefficients (Fourier ())".
int wco_extract_group(const char *group, const double *pix, int w, int h, int bits, double *out);

// One transform ("Fourier", "Chebyshev", "Wavelet", "Edge"); out holds >= 4*w*h.
int wco_transform(const char *name, const double *pix, int w, int h, double *out, int *ow, int *oh);

// Preprocessing and one sample (crop, Downsample, normalize, Rotate, tile) of
// a width x height image.  opt[14]: crop x, y, w, h (x < 0: none); downsample
// x, y ratios (>= 1: none); normalize min, max, range, mean, std; rotations;
// tiles x, y.  Returns 0, -1 where the reference refuses a rectangle, -2 when
// out (cap doubles) is too small.
int wco_preprocess(const double *pix, int w, int h, int bits, const double *opt, int sample, double *out,
                   long cap, int *ow, int *oh);

// WND-5 over images of `tiles` consecutive test rows (TrainingSet::ClassifyImage):
// per image the tile-averaged marginal probabilities (n_img x C), the class and
// the mean normalisation factor.  max_tile: the reference's most-similar-tile rule.
int wco_wnd_images(const double *train, int N, int F, const int *labels, int C, double frac, const double *test,
                   int n_img, int tiles, int max_tile, double *iprobs, int *ipred, double *inorm);

// Haralick per-angle tone count Ng of an image (diagnostic for cost models).
int wco_haralick_tones(const double *pix, int w, int h);

// WND-5, CLI semantics (TrainingSet::normalize, SetFisherScores, classify2).
int wco_wnd(const double *train, int N, int F, const int *labels, int C, double frac,
            const double *test, int T, double *weights, double *mins, double *maxs,
            double *probs, int *pred);

// The same over many test rows: one fit, then nthreads contiguous test ranges
// classified concurrently; secs[0] the fit's, secs[1] the classification's wall seconds.
int wco_wnd_mt(const double *train, int N, int F, const int *labels, int C, double frac, const double *test, int T,
               double *weights, double *mins, double *maxs, double *probs, int *pred, int nthreads, double *secs);

#ifdef __cplusplus
}
#endif
