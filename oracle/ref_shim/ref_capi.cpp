// TEST INFRASTRUCTURE ONLY: a small C ABI over the UNMODIFIED reference
// library, compiled from the reference sources by oracle/build_ref.sh into
// oracle/_ref/libwndref.so.  It is how the tests and the fixture generator
// (tests/golden/make_golden.py) obtain the reference's own answers.
//
// Pixels are handed over the way ImageMatrix::LoadTIFF stores them
// (src/cmatrix.cpp:134-163): row-major doubles, stats accumulated in raster
// order, then finish().
#include <cstring>
#include <string>
#include <vector>
#include <cfloat>
#include "cmatrix.h"
#include "Tasks.h"
#include "FeatureNames.h"
#include "ImageTransforms.h"
#include "FeatureAlgorithms.h"
#include "wndchrm_src/TrainingSet.h"
#include "wndchrm_src/signatures.h"

// the "verbosity" global comes from src/wndchrm_error.cpp

static void load_pixels(ImageMatrix &im, const double *pix, int w, int h, int bits) {
    im.bits = (unsigned short)bits;
    im.allocate(w, h);
    writeablePixels pp = im.WriteablePixels();
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) pp(y, x) = im.stats.add(pix[(size_t)y * w + x]);
    im.finish();
}

// kind 0: short (1059), 1: long (2919), 2: short colour (2199), 3: long colour (4059)
static const FeatureComputationPlan *std_plan(int kind) {
    if (kind == 1) return StdFeatureComputationPlans::getFeatureSetLong();
    if (kind == 2) return StdFeatureComputationPlans::getFeatureSetColor();
    if (kind == 3) return StdFeatureComputationPlans::getFeatureSetLongColor();
    return StdFeatureComputationPlans::getFeatureSet();
}

extern "C" void wcref_tiff_set(const void *data, int w, int h, int bits, int spp);

// ImageMatrix::OpenImage on an in-memory image (the libtiff stand-in serves it
// to the unmodified LoadTIFF): spp 3 = interleaved RGB, 8 or 16 bits.
static int open_memory_image(ImageMatrix &im, const void *pix, int w, int h, int bits, int spp) {
    wcref_tiff_set(pix, w, h, bits, spp);
    char name[] = "memory.tif";
    const int r = im.OpenImage(name, 0, nullptr, 0, 0);
    wcref_tiff_set(nullptr, 0, 0, 0, 0);
    return r;
}

extern "C" {

int wcref_plan_n_features(int kind) { return (int)std_plan(kind)->n_features; }

// Copies the i-th feature name of a standard plan into buf.
int wcref_plan_feature_name(int kind, int i, char *buf, int buflen) {
    const std::string &s = std_plan(kind)->getFeatureNameByIndex((size_t)i);
    std::strncpy(buf, s.c_str(), (size_t)buflen - 1);
    buf[buflen - 1] = 0;
    return (int)s.size();
}

// Runs a whole standard plan (kind 0 = short 1059, 1 = long 2919) through
// FeatureComputationPlanExecutor::run (src/Tasks.cpp:275-295).
int wcref_extract_std(int kind, const double *pix, int w, int h, int bits, double *out) {
    ImageMatrix im;
    load_pixels(im, pix, w, h, bits);
    const FeatureComputationPlan *plan = std_plan(kind);
    std::vector<double> row(plan->n_features, 0.0);
    FeatureComputationPlanExecutor ex(plan);
    ex.run(&im, row, 0);
    std::memcpy(out, row.data(), row.size() * sizeof(double));
    return (int)row.size();
}

// Runs one feature group given by its reference name, e.g.
// "Haralick Textures (Wavelet (Edge ()))".  Returns the feature count.
int wcref_extract_group(const char *group, const double *pix, int w, int h, int bits, double *out) {
    ImageMatrix im;
    load_pixels(im, pix, w, h, bits);
    FeatureComputationPlan plan("one group");
    plan.add(std::string(group));
    plan.finalize();
    std::vector<double> row(plan.n_features, 0.0);
    FeatureComputationPlanExecutor ex(&plan);
    ex.run(&im, row, 0);
    std::memcpy(out, row.data(), row.size() * sizeof(double));
    return (int)row.size();
}

// Applies one registered ImageTransform ("Fourier", "Chebyshev", "Wavelet",
// "Edge"); out must hold 4*w*h doubles.  Writes the output size.
int wcref_transform(const char *name, const double *pix, int w, int h, int bits,
                    double *out, int *ow, int *oh) {
    ImageMatrix im, res;
    load_pixels(im, pix, w, h, bits);
    const ImageTransform *t = FeatureNames::getTransformByName(std::string(name));
    if (!t) return -1;
    t->execute(im, res);
    *ow = (int)res.width;
    *oh = (int)res.height;
    readOnlyPixels rp = res.ReadablePixels();
    for (int y = 0; y < *oh; y++)
        for (int x = 0; x < *ow; x++) out[(size_t)y * (*ow) + x] = rp(y, x);
    return 0;
}

// WND-5 as the CLI runs it: TrainingSet::normalize (TrainingSet.cpp:2090),
// SetFisherScores(frac) (:2183), then classify2 (:2429) for every test row.
// train: N x F row-major; labels 1..C.  Feature names are the long plan's when
// F == 2919, else "Pixel Intensity Statistics () [i]".
// probs: T x C.  pred: T (1-based).  weights/mins/maxs: F.
int wcref_wnd(const double *train, int N, int F, const int *labels, int C, double frac,
              const double *test, int T, double *weights, double *mins, double *maxs,
              double *probs, int *pred) {
    TrainingSet *ts = new TrainingSet(N, C);
    char lab[32];
    for (int c = 1; c <= C; c++) {
        snprintf(lab, sizeof lab, "c%04d", c);
        ts->AddClass(lab);
    }
    const FeatureComputationPlan *plan = (F == 2919) ? std_plan(1) : nullptr;
    char nm[256];
    for (int s = 0; s < N; s++) {
        signatures *sg = new signatures();
        sg->NamesTrainingSet = ts;
        sg->sample_class = (unsigned short)labels[s];
        for (int f = 0; f < F; f++) {
            if (plan) std::strncpy(nm, plan->getFeatureNameByIndex(f).c_str(), sizeof nm - 1), nm[sizeof nm - 1] = 0;
            else snprintf(nm, sizeof nm, "Pixel Intensity Statistics () [%d]", f);
            sg->Add(nm, train[(size_t)s * F + f]);
        }
        ts->AddSample(sg);
    }
    ts->normalize();
    data_split split;
    ts->SetFisherScores(frac, 0, &split);
    for (int f = 0; f < F; f++) {
        weights[f] = ts->SignatureWeights[f];
        mins[f] = ts->SignatureMins[f];
        maxs[f] = ts->SignatureMaxes[f];
    }
    std::vector<double> p(C + 1);
    for (int t = 0; t < T; t++) {
        signatures *sg = new signatures();
        for (int f = 0; f < F; f++) sg->Add(nullptr, test[(size_t)t * F + f]);
        double nf = 0;
        char nmx[8] = "t";
        long c = ts->classify2(nmx, t, sg, p.data(), &nf);
        pred[t] = (int)c;
        for (int k = 1; k <= C; k++) probs[(size_t)t * C + k - 1] = p[k];
        delete sg;
    }
    delete ts;
    return 0;
}

// TrainingSet::ClassifyImage (src/wndchrm_src/TrainingSet.cpp:1603-1800) with
// WND, rank 1, no split, after the CLI's normalize + SetFisherScores, for
// n_img images of `tiles` consecutive test rows each.  probs: n_img x C (the
// `similarities` output, i.e. probabilities_sum); pred: n_img.
extern int verbosity;
int wcref_wnd_images(const double *train, int N, int F, const int *labels, int C, double frac, const double *test,
                     int n_img, int tiles, int max_tile, double *probs, int *pred) {
    const int old_verbosity = verbosity;
    verbosity = 0;
    TrainingSet *ts = new TrainingSet(N, C);
    char lab[32];
    for (int c = 1; c <= C; c++) {
        snprintf(lab, sizeof lab, "c%04d", c);
        ts->AddClass(lab);
    }
    const FeatureComputationPlan *plan = (F == 2919) ? std_plan(1) : nullptr;
    char nm[256];
    for (int s = 0; s < N; s++) {
        signatures *sg = new signatures();
        sg->NamesTrainingSet = ts;
        sg->sample_class = (unsigned short)labels[s];
        for (int f = 0; f < F; f++) {
            if (plan) std::strncpy(nm, plan->getFeatureNameByIndex(f).c_str(), sizeof nm - 1), nm[sizeof nm - 1] = 0;
            else snprintf(nm, sizeof nm, "Pixel Intensity Statistics () [%d]", f);
            sg->Add(nm, train[(size_t)s * F + f]);
        }
        ts->AddSample(sg);
    }
    ts->normalize();
    data_split split;
    ts->SetFisherScores(frac, 0, &split);
    const int T = n_img * tiles;
    TrainingSet *test_set = new TrainingSet(T, C);
    for (int t = 0; t < T; t++) {
        signatures *sg = new signatures();
        sg->sample_class = 0;
        snprintf(sg->full_path, sizeof sg->full_path, "image%06d", t / tiles);
        for (int f = 0; f < F; f++) sg->Add(nullptr, test[(size_t)t * F + f]);
        test_set->AddSample(sg);
    }
    std::vector<double> sims(C + 1);
    for (int g = 0; g < n_img; g++) {
        const double c = ts->ClassifyImage(test_set, g * tiles, WND, tiles, 0, nullptr, max_tile, 1, nullptr, sims.data());
        pred[g] = (int)c;
        for (int k = 1; k <= C; k++) probs[(size_t)g * C + k - 1] = sims[k];
    }
    delete test_set;
    delete ts;
    verbosity = old_verbosity;
    return 0;
}

// LoadTIFF of an RGB image (spp 3): the grayscale plane (RGB2GRAY of the
// 8-bit colour, 16-bit samples scaled to the image's RGB range first) and the
// HSV colour plane (3 bytes per pixel), src/cmatrix.cpp:85-203.
int wcref_load_rgb(const void *rgb, int w, int h, int bits, double *gray, unsigned char *hsv) {
    ImageMatrix im;
    if (open_memory_image(im, rgb, w, h, bits, 3) != 1) return -1;
    readOnlyPixels rp = im.ReadablePixels();
    readOnlyColors rc = im.ReadableColors();
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            gray[(size_t)y * w + x] = rp(y, x);
            const HSVcolor c = rc(y, x);
            unsigned char *o = hsv + 3 * ((size_t)y * w + x);
            o[0] = c.h;
            o[1] = c.s;
            o[2] = c.v;
        }
    return 0;
}

// The reference's fuzzy colour tables need one fix to be well defined:
// LoadColorsFunctions (src/colors/FuzzyCalc.cpp:582-623) returns when it
// reaches the "rules:" line, before it writes the terminating entry (colour
// -1) that color_value's loop (:625-650) stops at, so every membership lookup
// that misses runs past the end of color_functions[] into whatever the linker
// placed next (AddressSanitizer: global-buffer-overflow at FuzzyCalc.cpp:628).
// After the first FindColor has loaded the tables, the entry after the last
// loaded function is given colour -1, as the loader intends; everything else
// runs unmodified.
extern trapez_function color_functions[50];
static void terminate_colour_functions() {
    static bool done = false;
    if (done) return;
    FindColor(0, 0, 0, nullptr);
    int k = 0;
    while (k < 49 && color_functions[k].name[0]) k++;
    color_functions[k].color = (TColor)-1;
    done = true;
}

// FindColor (src/colors/FuzzyCalc.cpp:802-834) of one h, s, v.
int wcref_find_colour(int h, int s, int v) {
    terminate_colour_functions();
    return (int)FindColor((short)h, (short)s, (short)v, nullptr);
}

// A standard plan (kinds as std_plan) on an RGB (spp 3) or grayscale (spp 1)
// image read through LoadTIFF.
int wcref_extract_image(int kind, const void *pix, int w, int h, int bits, int spp, double *out) {
    terminate_colour_functions();
    ImageMatrix im;
    if (open_memory_image(im, pix, w, h, bits, spp) != 1) return -1;
    const FeatureComputationPlan *plan = std_plan(kind);
    std::vector<double> row(plan->n_features, 0.0);
    FeatureComputationPlanExecutor ex(plan);
    ex.run(&im, row, 0);
    std::memcpy(out, row.data(), row.size() * sizeof(double));
    return (int)row.size();
}

// The reference's own preprocessing and sampling of one image: the steps of
// ImageMatrix::OpenImage (src/cmatrix.cpp:252-294) after LoadTIFF, then the
// Rotate and tile submatrix of TrainingSet::AddImageFile
// (src/wndchrm_src/TrainingSet.cpp:1455-1481), on the unmodified ImageMatrix
// methods.  opt[14]: crop x, y, w, h (x < 0: none); Downsample x, y ratios
// (both >= 1: not called); normalize min, max, range, mean, std (called when
// either branch applies); rotations; tiles x, y.  Writes the sample's pixels
// (and, with feat_kind >= 0, its standard-plan features).  Returns -1 where
// submatrix refuses a rectangle.
int wcref_preprocess(const double *pix, int w, int h, int bits, const double *opt, int sample, double *out,
                     long cap, int *ow, int *oh, int feat_kind, double *feat) {
    const int cx = (int)opt[0], cy = (int)opt[1], cw = (int)opt[2], ch = (int)opt[3];
    const double dsx = opt[4], dsy = opt[5], nmin = opt[6], nmax = opt[7], nmean = opt[9], nstd = opt[10];
    const long nrange = (long)opt[8];
    const int rotations = (int)opt[11], tiles_x = (int)opt[12], tiles_y = (int)opt[13];
    const int tiles = tiles_x * tiles_y;
    ImageMatrix image_matrix;
    image_matrix.bits = (unsigned short)bits;
    if (cx >= 0) {
        ImageMatrix copy_matrix;
        copy_matrix.bits = (unsigned short)bits;
        copy_matrix.allocate(w, h);
        writeablePixels cp = copy_matrix.WriteablePixels();
        for (int y = 0; y < h; y++)
            for (int x = 0; x < w; x++) cp(y, x) = copy_matrix.stats.add(pix[(size_t)y * w + x]);
        if (!image_matrix.submatrix(copy_matrix, (unsigned int)cx, (unsigned int)cy, (unsigned int)cx + cw - 1,
                                    (unsigned int)cy + ch - 1))
            return -1;
    } else {
        image_matrix.allocate(w, h);
        writeablePixels pp = image_matrix.WriteablePixels();
        for (int y = 0; y < h; y++)
            for (int x = 0; x < w; x++) pp(y, x) = image_matrix.stats.add(pix[(size_t)y * w + x]);
    }
    if (!(dsx >= 1 && dsy >= 1)) image_matrix.Downsample(image_matrix, dsx, dsy);
    if (nmean > 0 || (nmin >= 0 && nmax > 0 && nrange > 0)) image_matrix.normalize(nmin, nmax, nrange, nmean, nstd);
    image_matrix.finish();
    const int rot_index = sample / tiles, rem = sample % tiles, tile_index_x = rem / tiles_y, tile_index_y = rem % tiles_y;
    if (rot_index >= rotations) return -1;
    ImageMatrix rot_matrix, tile_matrix;
    ImageMatrix *rot_matrix_p = &image_matrix, *tile_matrix_p;
    if (rot_index > 0) {
        rot_matrix.Rotate(image_matrix, 90.0 * rot_index);
        rot_matrix_p = &rot_matrix;
    }
    if (tiles != 1) {
        long tile_x_size, tile_y_size;
        if (rot_index == 1 || rot_index == 3) {
            tile_y_size = (long)(rot_matrix_p->width / tiles_x);
            tile_x_size = (long)(rot_matrix_p->height / tiles_y);
        } else {
            tile_x_size = (long)(rot_matrix_p->width / tiles_x);
            tile_y_size = (long)(rot_matrix_p->height / tiles_y);
        }
        if (!tile_matrix.submatrix(*rot_matrix_p, tile_index_x * tile_x_size, tile_index_y * tile_y_size,
                                   (tile_index_x + 1) * tile_x_size - 1, (tile_index_y + 1) * tile_y_size - 1))
            return -1;
        tile_matrix_p = &tile_matrix;
    } else {
        tile_matrix_p = rot_matrix_p;
    }
    tile_matrix_p->finish();
    *ow = (int)tile_matrix_p->width;
    *oh = (int)tile_matrix_p->height;
    if ((long)(*ow) * (*oh) > cap) return -2;
    readOnlyPixels rp = tile_matrix_p->ReadablePixels();
    for (int y = 0; y < *oh; y++)
        for (int x = 0; x < *ow; x++) out[(size_t)y * (*ow) + x] = rp(y, x);
    if (feat_kind >= 0 && feat) {
        const FeatureComputationPlan *plan = std_plan(feat_kind);
        std::vector<double> row(plan->n_features, 0.0);
        FeatureComputationPlanExecutor ex(plan);
        ex.run(tile_matrix_p, row, 0);
        std::memcpy(feat, row.data(), row.size() * sizeof(double));
    }
    return 0;
}

}  // extern "C"
