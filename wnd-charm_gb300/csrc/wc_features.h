// Feature-family preparation (host) and launch (device) for one batch.
#pragma once
#include <functional>
#include <map>
#include <string>
#include <vector>

#include "kernels.h"
#include "wc_internal.h"

namespace wc {

struct FeatureSetup {
    // inputs
    const std::vector<Plane> *planes;
    const std::vector<std::vector<FJob>> *fj;  // per algorithm
    // table by key; the generator runs only for a key the engine has not seen
    std::function<long long(const std::string &, const std::function<std::vector<double>()> &)> tabs_add;
    std::function<FFTPlan(int)> fft_plan;
    std::function<size_t(const void *, size_t)> put_copy;  // metadata blob, returns offset
    std::function<size_t(size_t)> ws_take;                 // workspace bytes, returns offset
    std::function<size_t(size_t)> meta_take;               // device-written metadata bytes
    // per-family results of the preparation (offsets into meta / ws)
    std::map<std::string, size_t> off;
    std::map<std::string, long long> val;
    std::vector<GabJob> gab_jobs;
    std::vector<GabSize> gab_sizes;
    int prec = 0;   // the engine's form (WC_PREC_*)
    int cf_tc = 1;  // mixed form: Chebyshev-Fourier sums on the tensor cores where every plane has one size
    CFTcPlan cf_tc_plan;
};

#define WC_LANES 6
struct FeatureRun {
    Ctx *ctx;
    Ctx *lanes;  // WC_LANES contexts on streams forked from ctx->st; families run on them concurrently
    double *arena;
    const Plane *planes;
    const PlaneStats *stats;
    char *meta;
    char *ws;
    const double *tabs;
    double *feat;
    const unsigned char *clr;  // HSV colour planes of RGB images, at clr_off[image] bytes
    const long long *clr_off;
    const double *fuzzy;  // the fuzzy colour classifier's membership table
};

void features_init();
int features_prepare(FeatureSetup &fs);
// phase 0: the families that read only root planes (Gabor, object and edge
// features) on lanes 3 and 4; phase 1: the rest (or everything, with early == false)
int features_launch(FeatureSetup &fs, FeatureRun &fr, int phase, bool early);
// reads and clears the device error word; *dev_err != 0 if a kernel flagged one
int features_check(cudaStream_t st, int *dev_err);
int set_err(int code, const char *fmt, ...);

}  // namespace wc
