// Runs the reference's CPU executor and the GB300 executor on the same
// ImageMatrix (a deterministic 96 x 80 12-bit pattern) for the long plan and
// a custom plan, and signatures::compute_plan's GB300 body; prints what each
// gave.  With a GPU the rows must agree (relative 1e-6, f14 excepted: it is
// implementation-defined); without one the GB300 calls must fail with the
// library's message and nothing else.  Exit status 0 when one of the two holds.
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <vector>

#include "FeatureNames.h"
#include "cmatrix.h"
#include "gb300_executor.h"

static void load(ImageMatrix &im, int w, int h) {
    im.bits = 16;
    im.allocate(w, h);
    writeablePixels pp = im.WriteablePixels();
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            const double v = 800 + 600 * std::sin(0.21 * x) * std::cos(0.17 * y) + 40 * ((x * 7 + y * 13) % 23);
            pp(y, x) = im.stats.add(std::floor(v));
        }
    im.finish();
}

static int compare(const FeatureComputationPlan *plan, const std::vector<double> &a, const std::vector<double> &b) {
    int bad = 0;
    for (size_t i = 0; i < plan->n_features; i++) {
        const std::string &nm = plan->getFeatureNameByIndex(i);
        if (nm.compare(0, 8, "Haralick") == 0 && (nm.find("[16]") != std::string::npos || nm.find("[17]") != std::string::npos))
            continue;
        const double d = std::fabs(a[i] - b[i]);
        if (!(d <= 1e-6 * std::fabs(b[i]) + 1e-9) && !(std::isnan(a[i]) && std::isnan(b[i]))) bad++;
    }
    return bad;
}

int main() {
    ImageMatrix im;
    load(im, 96, 80);
    FeatureComputationPlan custom("custom");
    custom.add("Zernike Coefficients (Fourier ())");
    custom.add("Haralick Textures (Wavelet ())");
    custom.add("Pixel Intensity Statistics (Chebyshev (Fourier ()))");
    custom.feature_vec_type = StdFeatureComputationPlans::fv_unknown;
    const FeatureComputationPlan *plans[2] = {StdFeatureComputationPlans::getFeatureSetLong(), &custom};
    int gpu_ok = 0, no_gpu = 0, other = 0;
    for (int p = 0; p < 2; p++) {
        // the caller sizes the row, as signatures::compute_plan does (Resize)
        std::vector<double> ref(plans[p]->n_features), gpu(plans[p]->n_features);
        FeatureComputationPlanExecutor cpu(plans[p]);
        cpu.run(&im, ref, 0);
        try {
            GB300FeatureComputationPlanExecutor g(plans[p]);
            g.run(&im, gpu, 0);
            const int bad = compare(plans[p], gpu, ref);
            std::printf("plan %s (%zu features): GB300 row against the CPU executor: %d outside 1e-6\n",
                        plans[p]->name.c_str(), plans[p]->n_features, bad);
            (bad ? other : gpu_ok)++;
        } catch (std::runtime_error &e) {
            std::printf("plan %s (%zu features): CPU executor ran; %s\n", plans[p]->name.c_str(),
                        plans[p]->n_features, e.what());
            const std::string m = e.what();
            (m.find("GB300 engine") == 0 ? no_gpu : other)++;
        }
    }
    signatures sig;
    try {
        gb300_compute_plan(sig, im, StdFeatureComputationPlans::getFeatureSet());
        std::printf("compute_plan: %ld features\n", sig.count);
    } catch (std::runtime_error &e) {
        std::printf("compute_plan: %s\n", e.what());
    }
    const bool pass = (gpu_ok == 2 && !other) || (no_gpu == 2 && !other);
    std::printf("%s\n", pass ? "adapter OK" : "adapter FAILED");
    return pass ? 0 : 1;
}
