/* wndcharm_gb300.h: C ABI of the GB300 (sm_103a) WND-CHARM hot path.
 *
 * The drop-in boundary for the reference's feature-plan API and its WND-5
 * classifier.  Plain pointers and sizes only; every call returns an int status
 * (WC_OK or a negative WC_ERR_*) and never aborts.  wc_last_error() gives the
 * message of the last failure on the calling thread.
 *
 * Reference interfaces replaced (paths inside the wnd-charm source tree):
 *   StdFeatureComputationPlans::getFeatureSet / getFeatureSetLong   src/Tasks.h:355-377, src/Tasks.cpp:313-352
 *   FeatureComputationPlan::add(name), n_features, getFeatureNameByIndex
 *                                                                    src/Tasks.h:272-316, src/Tasks.cpp:118-173
 *   FeatureComputationPlanExecutor::run(const ImageMatrix*, std::vector<double>&, size_t)
 *                                                                    src/Tasks.h:318-348, src/Tasks.cpp:275-295
 *   ImageTransform::execute (Fourier, Chebyshev, Wavelet, Edge)      src/ImageTransforms.h:45-51, src/ImageTransforms.cpp:59-112
 *   TrainingSet::normalize, SetFisherScores, classify2               src/wndchrm_src/TrainingSet.h:205-243,
 *                                                                    src/wndchrm_src/TrainingSet.cpp:2090-2123, 2183-2324, 2429-2586
 *   signatures::normalize                                            src/wndchrm_src/signatures.cpp:196-215
 *   ImageMatrix::OpenImage, submatrix, Downsample, normalize, Rotate src/cmatrix.cpp:252-294, 414-470, 579-769, 836-888
 *   TrainingSet::AddImageFile's sample loop (rotations x tiles)      src/wndchrm_src/TrainingSet.cpp:1442-1481
 */
#ifndef WNDCHARM_GB300_H
#define WNDCHARM_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define WC_OK 0
#define WC_ERR_ARG (-1)         /* bad argument (null pointer, size, unknown name) */
#define WC_ERR_CUDA (-2)        /* a CUDA runtime call failed */
#define WC_ERR_NOMEM (-3)       /* device allocation failed */
#define WC_ERR_UNSUPPORTED (-4) /* request outside what this build supports */
#define WC_ERR_DEVICE (-5)      /* a kernel reported a bounded-wait timeout or an internal check */
#define WC_ERR_IO (-6)          /* a file could not be read or is malformed */

/* largest image accepted: sides up to WC_MAX_SIDE pixels and at most
 * WC_MAX_PIXELS pixels; larger images give WC_ERR_ARG before any allocation */
#define WC_MAX_SIDE 32768
#define WC_MAX_PIXELS (1LL << 28)

/* plan kinds: the reference's standard feature sets */
#define WC_PLAN_SHORT 0 /* 1059 features, StdFeatureComputationPlans::getFeatureSet */
#define WC_PLAN_LONG 1  /* 2919 features, StdFeatureComputationPlans::getFeatureSetLong */
#define WC_PLAN_SHORT_COLOR 2 /* 2199 features, getFeatureSetColor (RGB images) */
#define WC_PLAN_LONG_COLOR 3  /* 4059 features, getFeatureSetLongColor (RGB images) */

/* pixel types accepted for input images */
#define WC_U8 0
#define WC_U16 1
#define WC_F32 2
#define WC_F64 3
#define WC_RGB8 4  /* interleaved r, g, b bytes */
#define WC_RGB16 5 /* interleaved r, g, b 16-bit samples (scaled to 8 bits over the image's range, as LoadTIFF does) */

/* arithmetic form of an engine */
#define WC_PREC_FP64 0  /* plain FP64 form: every family in double precision */
#define WC_PREC_MIXED 1 /* batched mixed-precision form: FP32 and pairs of floats on the CUDA cores, FP64 where required */

typedef struct wc_plan wc_plan;     /* a feature computation plan (groups, offsets, names) */
typedef struct wc_engine wc_engine; /* one GPU: device, stream, device memory pools */

/* One input image.  `pixels` is a host pointer unless `on_device` is set, in
 * which case it is a device pointer on the engine's GPU.  Row-major, width
 * `width`, height `height`, elements of type `dtype`; `bits` is the image's
 * intensity depth (8 or 16), kept for the ImageMatrix::bits field.  An RGB image
 * (WC_RGB8 / WC_RGB16) becomes, as ImageMatrix::LoadTIFF reads a 3-sample TIFF,
 * a grayscale plane 0.2989 r + 0.5870 g + 0.1140 b plus an HSV colour plane;
 * the colour plans need RGB images, every other plan reads the grayscale plane. */
typedef struct {
    const void *pixels;
    int dtype;
    int width;
    int height;
    int bits;
    int on_device;
} wc_image_desc;

const char *wc_last_error(void);
const char *wc_version(void);

/* ---- plans (host only, no GPU needed) ---- */
/* Standard plan, shared and immutable; do not free.  Replaces
 * StdFeatureComputationPlans::getFeatureSet{,Long} (src/Tasks.cpp:313-352). */
int wc_plan_get(int kind, const wc_plan **out);
/* Plan from feature-group names such as "Zernike Coefficients (Fourier (Edge ()))",
 * in the given order; replaces FeatureComputationPlan::add(name) (src/Tasks.cpp:156-158). */
int wc_plan_from_names(const char *const *groups, int n, wc_plan **out);
void wc_plan_free(wc_plan *plan);
/* FeatureComputationPlan::n_features (src/Tasks.h:280). */
int wc_plan_n_features(const wc_plan *plan);
/* FeatureComputationPlan::getFeatureNameByIndex (src/Tasks.cpp:160-169): copies the
 * name, e.g. "Haralick Textures (Wavelet (Edge ())) [17]"; returns its length. */
int wc_plan_feature_name(const wc_plan *plan, int index, char *buf, int buflen);
int wc_plan_n_groups(const wc_plan *plan);
/* group name and its column offset in a feature row (FeatureComputationPlan::getFGoffset) */
int wc_plan_group(const wc_plan *plan, int g, char *buf, int buflen, int *offset, int *n_features);

/* ---- engines ---- */
int wc_engine_create(int device, int precision, wc_engine **out);
void wc_engine_destroy(wc_engine *engine);
/* Engine options (no reference counterpart; defaults reproduce the reference):
 *   "f14_exact"        1 (default): the mixed form computes Haralick f14 (Q, the
 *                      Hessenberg reduction, the real-Schur QR) through the FP64
 *                      chain, bit-identical to the FP64 form and the oracle;
 *                      0: in pairs of floats on the FP32 pipe (faster; f14 is
 *                      then only as reproducible as a different build).
 *   "qr_iter_per_tone" real-Schur iterations allowed per tone, 40 (Eigen 3.1.2's
 *                      m_maxIterationsPerRow, RealSchur.h); a matrix that runs
 *                      out gives f14 = 0, as the reference's unconverged solver.
 *   "autotune"         1 (default): launch shapes chosen by the tuner (below);
 *                      0: each stage's first candidate.
 *   "union_find_cap"   iterations allowed per union-find link in the object
 *                      labelling; 0 (default): the plane's pixel count, a bound
 *                      no correct run reaches.  A run that reaches the cap
 *                      returns WC_ERR_DEVICE (the bounded-wait error path).
 *   "cf_tensor_cores"  1 (default): in the mixed form, when every Chebyshev-
 *                      Fourier plane of a batch has one size, its 23 x 23
 *                      coefficient sums run on the tensor cores (three bf16
 *                      digits per value, FP32 sums over 1024-pixel chunks
 *                      added in FP64); 0: FP32 sums on the CUDA cores.
 *   "graph"            0 (default); 1: wc_extract / wc_extract_batch capture the
 *                      launches of a batch shape (plan, image types and sizes,
 *                      output) in a CUDA graph the second time the shape is seen,
 *                      once the tuner has chosen every launch shape it is
 *                      timing, and later calls of that shape upload their
 *                      metadata and pixels and replay the graph (no host
 *                      planning, one launch call).  Results are those of the
 *                      ungraphed path bit for bit.  Up to 16 shapes are kept.
 * Unknown names and out-of-range values give WC_ERR_ARG.  Setting any option
 * drops the engine's graphs. */
int wc_engine_set_option(wc_engine *engine, const char *name, long long value);
/* Graph use since creation: stats[0] captures, stats[1] replays, stats[2]
 * shapes that could not be captured (they run without a graph), stats[3]
 * graphs kept.  stats holds 4 values. */
int wc_engine_graph_stats(wc_engine *engine, long long *stats);
/* The engine's launch-shape tuner (no reference counterpart).  Stages with
 * several candidate launch shapes (the real-Schur work queue's grouping and
 * CTAs per SM, the Wavelet and Edge transforms' block shapes) try each once,
 * per stage and size class, timing it with CUDA events, then keep the
 * fastest ("autotune" option, on by default; 0 keeps the first candidate).
 * The report has one line per key: "key<TAB>chosen<TAB>ms of candidate 0
 * <TAB>..." (chosen -1 while still trying; -1 ms for an untried candidate). */
int wc_engine_tuning_report(wc_engine *engine, char *buf, int buflen);
/* CUDA stream the engine launches on (as a cudaStream_t cast to void*); 0 = legacy default */
int wc_engine_set_stream(wc_engine *engine, void *stream);
/* kernels launched by this engine since creation (counts every launch) */
long long wc_engine_launch_count(const wc_engine *engine);
/* Per-stage timing (no reference counterpart; the reference prints a per-node
 * TIME line at verbosity > 4, src/Tasks.cpp:208-253): while on, every
 * transform and feature-family stage is bracketed by CUDA events on the
 * engine's stream (this serialises nothing but adds events); the report lists
 * "stage<TAB>milliseconds<TAB>calls<TAB>start<TAB>end" lines accumulated since
 * the last switch (start / end: the stage's earliest start and latest end in ms
 * after the batch's first stage; -1 for the host-side stages, "host: ...",
 * which are wall-clock milliseconds of the calling thread).  on = 2 also runs
 * every lane on the engine's stream, one stage after another, so that each
 * stage's time is its own (as in a serialised launch list, caches warm). */
int wc_engine_profile(wc_engine *engine, int on);
int wc_engine_profile_report(wc_engine *engine, char *buf, int buflen);

/* ---- feature extraction ----
 * FeatureComputationPlanExecutor::run for one image: writes plan->n_features
 * doubles to out_row (host memory).  Synchronous. */
int wc_extract(wc_engine *engine, const wc_plan *plan, const void *pixels, int dtype, int width, int height,
               int bits, double *out_row);
/* Batched form: n images of any sizes, out is n x n_features row-major, host
 * memory unless out_on_device is set (then a device pointer on the engine's
 * GPU).  Either way the call returns when the rows are written: it reads the
 * kernels' error word at the end, which waits for the engine's stream. */
int wc_extract_batch(wc_engine *engine, const wc_plan *plan, const wc_image_desc *images, int n, double *out,
                     int out_on_device);
/* One transform ("Fourier", "Chebyshev", "Wavelet", "Edge"), host buffers; out
 * must hold out_capacity doubles; writes the output size.  ImageTransform::execute
 * (src/ImageTransforms.cpp:59-112). */
int wc_transform(wc_engine *engine, const char *name, const double *pixels, int width, int height, double *out,
                 long long out_capacity, int *out_width, int *out_height);

/* ---- WND-5 (CLI semantics), host buffers ----
 * wc_wnd_fit: TrainingSet::normalize + SetFisherScores(frac): per-feature min/max of the
 * training rows, Fisher scores, all weights below the score at sorted rank
 * floor(frac*F+0.5) set to 0.  train: N x F, labels in 1..C. */
int wc_wnd_fit(wc_engine *engine, const double *train, int N, int F, const int *labels, int C, double frac,
               double *weights, double *mins, double *maxs);
/* wc_wnd_classify: signatures::normalize of each test row against (mins, maxs),
 * then TrainingSet::classify2 against the training rows normalised the same way:
 * probs T x C marginal probabilities, pred T predicted classes (1-based, -1 if none). */
int wc_wnd_classify(wc_engine *engine, const double *train, int N, int F, const int *labels, int C,
                    const double *weights, const double *mins, const double *maxs, const double *test, int T,
                    double *probs, int *pred);

/* signatures::normalize (src/wndchrm_src/signatures.cpp:196-215) of n rows of F
 * features against (mins, maxs): 0 for NaN, below the range or a range below
 * DBL_EPSILON, 100 above it, else 100 * ((v - min) / (max - min)) with the
 * correctly rounded quotient; the values every WND-5 call compares. */
int wc_wnd_normalize(wc_engine *engine, const double *rows, int n, int F, const double *mins, const double *maxs,
                     double *out);

/* wc_wnd_fit over training rows sharded across processes, in three stages of
 * this process's statistics with an exchange between them (min / max, then
 * sums; TrainingSet::normalize + SetFisherScores, TrainingSet.cpp:2090-2324):
 *   stage 0: out = [mins (F), maxs (F)] of the finite values (FLT_MAX / -FLT_MAX
 *            where none), counts = rows per label (C+1: slot 0 every labelled
 *            row, slot c class c);
 *   stage 1: with the global mins / maxs, out = per-label sums of the normalised
 *            values ((C+1) x F, label-major);
 *   stage 2: with the global class means ((C+1) x F: sums / counts, 0 where a
 *            count is 0), out = per-label sums of squared deviations.
 * wc_wnd_fisher turns the summed statistics into wc_wnd_fit's weights. */
int wc_wnd_fit_stats(wc_engine *engine, int stage, const double *train, int N, int F, const int *labels, int C,
                     const double *mins, const double *maxs, const double *means, double *out, long long *counts);
int wc_wnd_fisher(wc_engine *engine, int F, int C, double frac, const double *sums, const long long *counts,
                  const double *sq, double *weights);

/* classify2's per-class partial sums over the training rows given (a shard of
 * the training set): sums[t*C + c-1] = sum of d(t,s)^-5 over the rows s of class c
 * with d >= DBL_EPSILON, counts[t*C + c-1] how many (FP64, the reference's
 * arithmetic per term).  Summed over the shards of a training set (one
 * all-reduce), then mean per class and normalised, they are classify2's
 * probabilities for the whole set (TrainingSet.cpp:2429-2586). */
int wc_wnd_class_sums(wc_engine *engine, const double *train, int N, int F, const int *labels, int C,
                      const double *weights, const double *mins, const double *maxs, const double *test, int T,
                      double *sums, long long *counts);

/* wc_wnd_fit followed by wc_wnd_classify of `test` against the same training
 * rows, as the reference's classification run does them in one process
 * (TrainingSet::normalize, SetFisherScores, then classify2 per test sample:
 * src/wndchrm_src/wndchrm.cpp, TrainingSet.cpp:2090-2324, 2429-2586): each
 * host array is copied to the GPU once.  Outputs: weights, mins, maxs (F), probs
 * (T x C), pred (T). */
int wc_wnd_fit_classify(wc_engine *engine, const double *train, int N, int F, const int *labels, int C, double frac,
                        const double *test, int T, double *weights, double *mins, double *maxs, double *probs,
                        int *pred);

/* Device-pointer forms of wc_wnd_fit and wc_wnd_classify (same semantics):
 * every array argument is a device pointer on the engine's GPU, so rows that
 * are already in device memory (e.g. feature rows of wc_extract_batch with
 * out_on_device) are classified without a host round trip.  The calls return
 * when the results are written.  In the mixed form, wc_wnd_classify* computes
 * the distances on the tensor cores (when at most 511 features have a
 * non-zero weight): the weighted rows are cut into four 8-bit digits held
 * exactly in bf16, digit pairs are multiplied by tcgen05.mma into FP32 sums
 * that stay exact, and every test row whose error bound, nearest-row distance
 * or top-two class margin is not certified is recomputed by the FP64 kernel
 * (the reference's order), so classes equal the FP64 form's and
 * probabilities stay within 1e-6 of them.  More weighted features: pairs of
 * floats on the CUDA cores. */
int wc_wnd_fit_device(wc_engine *engine, const double *train, int N, int F, const int *labels, int C, double frac,
                      double *weights, double *mins, double *maxs);
int wc_wnd_classify_device(wc_engine *engine, const double *train, int N, int F, const int *labels, int C,
                           const double *weights, const double *mins, const double *maxs, const double *test, int T,
                           double *probs, int *pred);
/* What the calling thread's last wc_wnd_classify* call did (no reference
 * counterpart): stats[0] 1 if the tensor-core path ran, stats[1] the test rows
 * the FP64 kernel recomputed, stats[2] the features with a non-zero weight,
 * stats[3] the tensor-core kernel's CTAs, stats[4] its time in nanoseconds
 * (CUDA events on the engine's stream), stats[5] the tensor FLOPs it issued
 * (13 digit-pair products over the padded sizes).  stats holds 6 values. */
int wc_wnd_last_stats(long long *stats);

/* ---- differentiation (no counterpart in the reference) ----
 * wc_wnd_grad: the marginal probabilities that classify2 gives the n test
 * images (their `plan` features computed by the engine, compared with the N
 * training feature rows `train` (N x plan features, host) under `weights`,
 * `mins`, `maxs` as wc_wnd_classify does), written to probs (n x C; may be
 * NULL), and, when `seed` is given, one backward pass per seed after a
 * single forward pass: seed holds n x n_seeds x C values of d loss / d
 * probability (image-major); grad_pixels receives, for every image, its
 * n_seeds maps of d loss / d pixel (width x height values each; images one
 * after another; may be NULL) and grad_weights n_seeds x F values of d loss
 * / d weight, each summed over the images (may be NULL).  n_seeds = C with
 * one-hot seeds gives the per-class evidence maps d p_c / d pixel.  All in
 * FP64, host buffers.  The backward runs through Zernike
 * Coefficients, Pixel Intensity Statistics, Fractal Features and Gini
 * Coefficient, on planes made by Fourier, Chebyshev, Wavelet and Edge chains;
 * the binned families (histograms, counts, thresholds, Haralick) are
 * piecewise-constant and contribute zero; a non-zero weight on a Tamura or
 * Edge feature, or on a colour chain, gives WC_ERR_UNSUPPORTED. */
int wc_wnd_grad(wc_engine *engine, const wc_plan *plan, const double *train, int N, const int *labels, int C,
                const double *weights, const double *mins, const double *maxs, const wc_image_desc *images, int n,
                const double *seed, int n_seeds, double *probs, double *grad_pixels, double *grad_weights);

/* wc_wnd_classify_images: TrainingSet::ClassifyImage with WND-5
 * (src/wndchrm_src/TrainingSet.cpp:1603-1800) for n_images images of `tiles`
 * samples each: test holds n_images * tiles rows, an image's tiles consecutive.
 * probs (n_images x C) are the tiles' marginal probabilities averaged in tile
 * order (each added as p / tiles); pred is the class with the largest average
 * (the first on ties; rank 1); norm_factors (may be NULL) the tiles' mean
 * classify2 normalisation factor.  With max_tile set, the reference's
 * "most similar tile" rule: a tile whose predicted-class probability divided
 * by the other classes' sum is the largest so far replaces the sums with its
 * own probabilities, and later tiles keep adding p / tiles.  Replaces the
 * per-image loop of TrainingSet::Test (src/wndchrm_src/TrainingSet.cpp:1956-2000). */
int wc_wnd_classify_images(wc_engine *engine, const double *train, int N, int F, const int *labels, int C,
                           const double *weights, const double *mins, const double *maxs, const double *test,
                           int n_images, int tiles, int max_tile, double *probs, int *pred, double *norm_factors);

/* ---- image files ----
 * TIFF as ImageMatrix::LoadTIFF reads it (src/cmatrix.cpp:85-203): one image
 * directory, one sample per pixel (grayscale) or three interleaved (RGB; hand
 * them to the engine as WC_RGB8 / WC_RGB16), 8 or 16 bits, strips
 * uncompressed, LZW (optionally with the horizontal predictor) or PackBits,
 * either byte order.  wc_tiff_info gives the size and bit depth, wc_tiff_layout
 * also the samples per pixel; wc_tiff_read writes the samples row-major and
 * interleaved (uint8, or uint16 in native byte order) into `pixels` (capacity
 * in bytes).  Other layouts and multi-directory files give WC_ERR_UNSUPPORTED. */
int wc_tiff_info(const char *path, int *width, int *height, int *bits);
int wc_tiff_layout(const char *path, int *width, int *height, int *bits, int *samples);
int wc_tiff_read(const char *path, void *pixels, long long capacity);
/* TIFF files decoded into device memory (no reference counterpart beyond
 * LoadTIFF itself): the host reads each file and its directory and copies its
 * strips to the GPU as stored (LZW strips, a serial bit stream, are decoded on
 * the host); PackBits expansion, byte order and the horizontal predictor run on
 * the GPU.  d_pixels: a 256-byte aligned device buffer of `capacity` bytes
 * (wc_tiff_device_bytes gives the size); image i's samples start at
 * descs[i].pixels (256-byte aligned, native uint8 / uint16, RGB interleaved)
 * and descs[i] is filled for wc_extract_batch / wc_extract_samples
 * (on_device = 1, dtype WC_U8 / WC_U16 / WC_RGB8 / WC_RGB16, bits = the file's).
 * The same files, layouts and errors as wc_tiff_read. */
int wc_tiff_device_bytes(const char *const *paths, int n, long long *bytes);
int wc_tiff_read_device(wc_engine *engine, const char *const *paths, int n, void *d_pixels, long long capacity,
                        wc_image_desc *descs);

/* ---- preprocessing and sampling ----
 * How wndchrm turns one opened image into its samples, on the GPU:
 * ImageMatrix::OpenImage (src/cmatrix.cpp:252-294) crops to a bounding
 * rectangle (submatrix, :414-470), area-downsamples (Downsample, :579-720) and
 * normalises (normalize, :836-888); TrainingSet::AddImageFile
 * (src/wndchrm_src/TrainingSet.cpp:1442-1481) then rotates (Rotate, :727-769)
 * and cuts a tile (submatrix) for each sample.  Samples are numbered as
 * wndchrm enumerates them (src/wndchrm_src/wndchrm.cpp:93-124): rotation
 * outermost, then tile x, then tile y; sample k has rotation k / (tx*ty),
 * tile x (k % (tx*ty)) / ty, tile y k % ty.  As in the reference, a
 * "rotation" of 270 degrees is the transpose (Rotate's case 270), and for
 * rotations 1 and 3 the tile width is the rotated image's height / tiles_y and
 * the tile height its width / tiles_x (TrainingSet.cpp:1465-1471).  A tile
 * that does not fit the rotated image (the reference then keeps the previous
 * sample's pixels) is WC_ERR_ARG.  Arithmetic is FP64 in the reference's
 * order (crop, rotation, tiles and Downsample are bit-identical to it); the
 * mean / standard deviation that normalisation divides by come from the
 * reference's own Welford chain (Moments2, in raster order), so normalised
 * pixels are bit-identical too. */
typedef struct {
    int crop_x, crop_y, crop_w, crop_h; /* bounding rectangle; crop_x < 0: the whole image */
    double downsample_x, downsample_y;  /* Downsample ratios in (0, 1); >= 1: no downsampling */
    double norm_min, norm_max;          /* normalize to [0, norm_range] when norm_min >= 0, norm_max > 0 */
    long long norm_range;               /* ... and norm_range > 0 */
    double norm_mean, norm_std;         /* normalize to norm_mean (and norm_std when > 0) when norm_mean > 0 */
    int rotations;                      /* 1 (as is) or 4 (also 90, 180, 270 degrees) */
    int tiles_x, tiles_y;               /* tiles per rotated image, >= 1 each */
} wc_sampling;

/* No crop, no downsampling, no normalisation, 1 rotation, 1 x 1 tile. */
void wc_sampling_default(wc_sampling *s);
/* Samples per image: rotations * tiles_x * tiles_y (or a negative status). */
int wc_sampling_count(const wc_sampling *s);
/* Size of sample `sample` of a width x height image. */
int wc_sample_size(const wc_sampling *s, int width, int height, int sample, int *out_width, int *out_height);
/* One sample plane of one image: out receives out_width * out_height doubles
 * (row-major; out_capacity in doubles), host memory unless out_on_device. */
int wc_preprocess(wc_engine *engine, const wc_image_desc *image, const wc_sampling *s, int sample, double *out,
                  long long out_capacity, int *out_width, int *out_height, int out_on_device);
/* wc_extract_batch over every sample of every image: out is
 * (n * wc_sampling_count(s)) x n_features, image-major, samples in the order
 * above.  The images go to the GPU once; crop, downsampling, normalisation,
 * rotations and tiles run there, and the samples stay in device memory until
 * their feature rows are written. */
int wc_extract_samples(wc_engine *engine, const wc_plan *plan, const wc_image_desc *images, int n,
                       const wc_sampling *s, double *out, int out_on_device);

/* ---- allocation-free entry point ----
 * wc_wavelet_noalloc: the Wavelet transform (one-level Symlet-5, as wc_transform
 * "Wavelet") for callers that may not allocate device memory: d_in is a device
 * pointer to width x height doubles (row-major), d_out a device pointer to
 * (2*floor((width+9)/2)) x (2*floor((height+9)/2)) doubles; the work is queued on
 * `stream` (a cudaStream_t, 0 = legacy default).  No cudaMalloc/cudaFree is
 * called; the intermediate lives in a static device array of 1,081,344 doubles
 * (8.25 MiB per GPU, held until the process exits), enough for inputs up to
 * 1024 x 1024; larger inputs are rejected with WC_ERR_ARG.  All calls share that
 * array: calls whose work overlaps on the GPU race, so order them (one stream).
 * Every call looks up the array's address on the current device (so a
 * cudaDeviceReset in between is harmless); the first call on a device loads
 * the library's device code there, so make it before any stream capture.
 * A CUDA error left pending by an earlier call gives WC_ERR_CUDA before any
 * launch.  It has no counterpart in the reference. */
int wc_wavelet_noalloc(const double *d_in, int width, int height, double *d_out, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* WNDCHARM_GB300_H */
