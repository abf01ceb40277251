// Host-side launchers of the CUDA kernels (one per family or transform).
#pragma once
#include <vector>

#include "wc_internal.h"

namespace wc {

// k_basic.cu
void launch_convert(Ctx &c, const void *src, int dtype, double *dst, long long n);
// sel 0: all planes; 1: each image's root plane (index b*nn); 2: all but the roots
void launch_plane_stats(Ctx &c, const double *arena, const Plane *planes, int nplanes, PlaneStats *out, int nn, int sel);
void launch_edge(Ctx &c, double *arena, const Plane *planes, const TJob *jobs, int njobs, int maxw, int maxh);
void launch_wavelet(Ctx &c, double *arena, const Plane *planes, const TJob *jobs, int njobs, int maxw, int maxh,
                    double *tmp, const long long *tmp_off);
void launch_pixstats(Ctx &c, const Plane *planes, const PlaneStats *stats, const FJob *jobs, int njobs,
                     const int *sort_slot, const unsigned long long *keys, const long long *key_off, double *feat);
void launch_gini(Ctx &c, const Plane *planes, const FJob *jobs, int njobs, const int *sort_slot,
                 const unsigned long long *keys, const long long *key_off, double *feat);
void launch_mshist(Ctx &c, const double *arena, const Plane *planes, const PlaneStats *stats, const FJob *jobs,
                   int njobs, double *feat);
void launch_fractal(Ctx &c, const double *arena, const Plane *planes, const FJob *jobs, int njobs, double *feat);
void launch_comb(Ctx &c, const double *arena, const Plane *planes, const FJob *jobs, int njobs, double *feat);
void set_radon_table(const double *cs8);
void launch_radon(Ctx &c, const double *arena, const Plane *planes, const FJob *jobs, int njobs, int maxw, int maxh,
                  double *feat);
void launch_chebcoef(Ctx &c, const double *arena, const Plane *planes, const FJob *jobs, int njobs, const double *tabs,
                     const long long *tab_off, double *mid_ws, const long long *mid_off, double *feat);

// k_sort.cu: multi-CTA radix sort of many arrays of 64-bit keys
struct SortSeg {
    long long off, n;  // offset and length of the array in the key buffers
};
size_t sort_scratch_bytes(int nseg, long long max_n);
void launch_sort_planes(Ctx &c, const double *arena, const Plane *planes, const int *ids, const SortSeg *seg, int nseg,
                        long long max_n, unsigned long long *keys, unsigned long long *tmp, void *scratch);

// k_fft.cu: 1-D complex DFTs of any length <= kMaxFFT, batched, in shared memory
const int kMaxFFT = 4096;
struct FFTPlan {  // device description of one length
    int n, nstages;
    int radix[16];
    long long tw_off;  // offset of exp(-2 pi i k / n), k < n, in the twiddle table (interleaved re, im)
};
// k_gabor.cu: FP64 forward DFTs of na same-shape complex arrays at complex
// offsets aoff[] from data (nl lines of length n each, in place)
void cfft_lines_fp64(cudaStream_t st, long long *launches, double *data, const long long *aoff, int na, int nl, int n,
                     long long ls, long long es, const FFTPlan *plan, const double *tw);
void launch_fourier(Ctx &c, double *arena, const Plane *planes, const TJob *jobs, int njobs, int maxw, int maxh,
                    const FFTPlan *plans_d, const int *job_plan_y, const int *job_plan_x, const double *tw,
                    double *cbuf, const long long *cbuf_off);

// k_gemm.cu: the Chebyshev transform (two FP64 products with host-made tables)
void launch_chebyshev(Ctx &c, double *arena, const Plane *planes, const TJob *jobs, int njobs, int maxw, int maxh,
                      const double *tabs, const long long *tab_off, double *mid, const long long *mid_off);

// k_groupb.cu: Zernike and Chebyshev-Fourier coefficients
void set_zernike_tables();
void launch_zernike(Ctx &c, const double *arena, const Plane *planes, const FJob *jobs, int njobs, long long maxpix,
                    double *mom, double *part, double *feat);
struct CFJob {
    long long src_ws;          // offset (doubles) of the m x n source image in the workspace
    long long tmp_ws;          // offset of the x-pass buffer (old_h x cnt_x)
    long long xs_tab, ys_tab;  // position tables (doubles) in the table buffer
    int cnt_x, cnt_y, new_w, new_h;
    int down;  // 1 if downsampled
    int nchunk;
    double dx;
};
// k_cf_tc.cu: the mixed form's Chebyshev-Fourier sums on the tensor cores for
// planes of one size (1058 basis columns padded to 17 tiles of 64)
#define CF_TC_COLS 1088
struct CFTcPlan {
    long long K_pad = 0, M_pad = 0;
    int nchunk = 0;
    size_t digA_bytes = 0, digB_bytes = 0, partial_bytes = 0, uA_bytes = 0;
};
struct CFTcBufs {
    void *digA, *digB;
    double *partial, *uA;
};
CFTcPlan cf_tc_plan(int njobs, int m, int n);
bool launch_cf_tc(Ctx &c, const CFJob *cj, int njobs, int m, int n, const double *ws, const CFTcPlan &p,
                  const CFTcBufs &b, double *part, int nchunk_max);
int cf_tc_err_take(cudaStream_t st, int *v);
// tcp / tcb: the tensor-core form's plan and buffers (mixed form, one size), or null
void launch_chebfourier(Ctx &c, const double *arena, const Plane *planes, const FJob *jobs, int njobs, int maxw,
                        int maxh, int max_cnt_x, int max_src_w, int max_src_h, const CFJob *cj, const double *tabs,
                        double *ws, double *part, int nchunk_max, double *feat, const CFTcPlan *tcp = nullptr,
                        const CFTcBufs *tcb = nullptr);

// k_tamura.cu
struct TamJob {
    long long norm_ws, sum_ws, sbest_ws, phi_ws;  // offsets in doubles into the workspace
    long long mk_ws, emax_ws;                     // window means of one scale; each pixel's best E so far
};
void launch_tamura(Ctx &c, const Plane *planes, const PlaneStats *stats, const double *arena, const FJob *jobs, int njobs,
                   const TamJob *tj, double *ws, double *part, long long maxpix, double *feat);

// k_haralick.cu
struct HarJob {
    // byte offsets into the workspace: gray image, tone LUT (+ Ng), 4 co-occurrence
    // matrices, 4 Q / Hessenberg / Schur matrices, 4 x 14 results, and per angle the
    // marginals px[256], py[256] and the nonzero column range of every row
    long long gray_b, lut_b, glcm_b, q_b, res_b, mar_b;
};
#define HAR_MAR_BYTES 6144  // per angle: px, py (2 x 256 doubles), lo, hi (2 x 256 ints)
void launch_haralick(Ctx &c, const double *arena, const Plane *planes, const PlaneStats *stats, const FJob *jobs,
                     int njobs, const HarJob *hj, char *wsb, int *perm, double *feat);

// k_groupa.cu
struct EFJob {
    long long mag_ws, dir_ws;  // Prewitt magnitude / direction planes (doubles offsets)
};
void launch_edgefeat(Ctx &c, const double *arena, const Plane *planes, const FJob *jobs, int njobs, int maxw, int maxh,
                     const EFJob *ej, double *ws, const Plane *aux_planes, const int *aux_ids, PlaneStats *aux_stats,
                     unsigned long long *keys, unsigned long long *tmp, const long long *koff, const SortSeg *seg,
                     long long maxn, void *scratch, double *feat);
struct OBJob {
    int inverse;  // 1: Inverse-Otsu (source = inverted plane at src_ws)
    int pad_;
    long long src_ws, lab_ws, area_ws, xm_ws, ym_ws, roots_ws, keys_ws, tmp_ws, dist_ws;  // doubles offsets
};
// reads and clears the object kernels' error word (0 = ok; else the code); -1 if the copy fails
int objects_err_take(cudaStream_t st, int *v);
void launch_objects(Ctx &c, const double *arena, const Plane *planes, const PlaneStats *stats, const FJob *jobs, int njobs,
                    long long maxpix, const OBJob *oj, double *ws, const Plane *inv_planes, PlaneStats *inv_stats,
                    double *thr, unsigned long long *acc, double *feat);

// k_color.cu: RGB ingest, the fuzzy colour classifier's membership table
// (host-made), the Color / Hue / Color Transform transforms and the Color
// Histogram family.  clr: HSV bytes (3 per pixel) of each image at
// clr_off[image] bytes.
std::vector<double> fuzzy_membership_table();
void launch_rgb_ingest(Ctx &c, const void *src, int dtype, long long n, double *gray, unsigned char *hsv);
void launch_color_xf(Ctx &c, double *arena, const Plane *planes, const TJob *jobs, int njobs, int maxw, int maxh, int xf,
                     int nn, const unsigned char *clr, const long long *clr_off, const double *tab);
void launch_color_hist(Ctx &c, const Plane *planes, const FJob *jobs, int njobs, const unsigned char *clr,
                       const long long *clr_off, const double *tab, double *feat);

// k_pre.cu: preprocessing (crop, Downsample, normalize) of each image into its
// opened plane, then one rotated / tiled plane per sample.  Offsets are in
// doubles into the preprocessing arena (tables: into the position table).
struct PreJob {
    const void *src;  // device address of the image
    int dtype, sw;    // pixel type, row length
    int cx, cy, cw, ch;
    long long a_off;  // crop plane, cw x ch
    int down, nw, nh;
    double dx, dy;              // Downsample steps 1 / ratio
    long long xs_tab, ys_tab;   // accumulated start positions
    long long t_off;            // x pass, ch x nw
    long long o_off;            // opened plane (a_off when not downsampled)
    int ow, oh;
    int mm, ms;                 // normalize: range branch, mean branch
    double n_min, n_max, n_range, n_mean, n_std, max_range;
};
struct SampleJob {
    int img, rot;
    int x1, y1, tw, th;  // tile in the rotated opened plane
    long long off;       // the sample plane, tw x th
};
struct PreGeomMax {  // launch extents: maxima over the batch
    int cw, ch, nw, nh, ow, oh, tw, th;
    int down, norm_range, norm_mean;
};
// tab: Downsample positions; yh, yl: RN(1/k) and RN(1/k - RN(1/k)) for k = 1, 2, ...
// (index k - 1); fact: 2 doubles per image written by the device
void launch_preprocess(Ctx &c, const PreJob *jobs, int n, const PreGeomMax &g, const double *tab, const double *yh,
                       const double *yl, double *fact, double *pre, const SampleJob *sj, int ns);

// k_gabor.cu
struct GabJob {
    long long a_ws, c_ws, e_ws, g_ws;  // doubles offsets: image spectrum, 8 products, 8 energy maps, kernel spectra
    int fh, fw, plan_h, plan_w;
};
struct GabSize {
    int fh, fw, plan_h, plan_w;
    long long g_ws;        // the 8 kernel spectra of this padded size
    long long a_ws, c_ws;  // first job's image spectrum / 8 products; the size's jobs follow contiguously
    int count;             // jobs of this padded size
};
void launch_gabor(Ctx &c, const double *arena, const Plane *planes, const FJob *jobs, int njobs, const GabJob *gj_d,
                  const std::vector<GabJob> &gj, const std::vector<GabSize> &sizes, const FFTPlan *plans_d,
                  const double *tabs, long long kern_tab, double *ws, double *counts, double *feat);

}  // namespace wc
