// See gb300_executor.h.
#include "gb300_executor.h"

#include <cstring>
#include <stdexcept>

#include "FeatureNames.h"
#include "cmatrix.h"
#include "wndchrm_src/TrainingSet.h"

static void fail(const char *what) {
    throw std::runtime_error(std::string("GB300 ") + what + ": " + wc_last_error());
}

GB300FeatureComputationPlanExecutor::GB300FeatureComputationPlanExecutor(const FeatureComputationPlan *plan_in,
                                                                         int device_in, int precision_in)
    : FeatureComputationPlanExecutor(plan_in), device(device_in), precision(precision_in), engine(NULL),
      own_plan(NULL), wplan(NULL) {}

GB300FeatureComputationPlanExecutor::~GB300FeatureComputationPlanExecutor() {
    if (own_plan) wc_plan_free(own_plan);
    if (engine) wc_engine_destroy(engine);
}

// the engine and the plan, made on the first run
void GB300FeatureComputationPlanExecutor::open() {
    if (!engine && wc_engine_create(device, precision, &engine) != WC_OK) {
        engine = NULL;
        fail("engine");
    }
    if (wplan) return;
    switch (plan->feature_vec_type) {
        case StdFeatureComputationPlans::fv_short:
            if (wc_plan_get(WC_PLAN_SHORT, &wplan) != WC_OK) fail("plan");
            return;
        case StdFeatureComputationPlans::fv_long:
            if (wc_plan_get(WC_PLAN_LONG, &wplan) != WC_OK) fail("plan");
            return;
        case StdFeatureComputationPlans::fv_short_color:
        case StdFeatureComputationPlans::fv_long_color:
            throw std::runtime_error("GB300 executor: colour plans take the image's RGB samples "
                                     "(wc_extract_batch with WC_RGB8 / WC_RGB16)");
        default:
            break;
    }
    // a custom plan: its groups in column order, by name (FeatureComputationPlan::add)
    std::vector<std::string> names;
    for (size_t off = 0; off < plan->n_features;) {
        const FeatureGroup *fg = plan->getFeatureGroupByIndex(off);
        if (!fg || fg->labels.empty()) throw std::runtime_error("GB300 executor: plan without a group at a column");
        names.push_back(fg->name);
        off += fg->labels.size();
    }
    std::vector<const char *> cn;
    for (size_t i = 0; i < names.size(); i++) cn.push_back(names[i].c_str());
    if (wc_plan_from_names(cn.data(), (int)cn.size(), &own_plan) != WC_OK) fail("plan");
    wplan = own_plan;
    if ((size_t)wc_plan_n_features(wplan) != plan->n_features)
        throw std::runtime_error("GB300 executor: the plan's feature count differs");
}

void GB300FeatureComputationPlanExecutor::run(const ImageMatrix *source_mat, std::vector<double> &feature_mat_in,
                                              size_t dest_row) {
    open();
    const size_t nf = plan->n_features;
    if (feature_mat_in.size() < (dest_row + 1) * nf) feature_mat_in.resize((dest_row + 1) * nf);
    // the ImageMatrix's plane is row-major doubles (src/cmatrix.h), handed over as is
    if (wc_extract(engine, wplan, source_mat->data_ptr(), WC_F64, (int)source_mat->width, (int)source_mat->height,
                   (int)source_mat->bits, &feature_mat_in[dest_row * nf]) != WC_OK)
        fail("extraction");
}

void gb300_compute_plan(signatures &sig, const ImageMatrix &matrix, const FeatureComputationPlan *plan) {
    GB300FeatureComputationPlanExecutor executor(plan);
    sig.version = CURRENT_FEATURE_VERSION;
    sig.feature_vec_type = plan->feature_vec_type;
    sig.Resize(plan->n_features);
    executor.run(&matrix, sig.data, 0);
    sig.count = plan->n_features;
    if (sig.count > signatures::max_sigs) signatures::max_sigs = sig.count;
    // the feature names go to an attached training set once, as the reference does
    if (sig.NamesTrainingSet)
        for (int i = 0; i < sig.count; i++) {
            char *name = ((TrainingSet *)sig.NamesTrainingSet)->SignatureNames[i];
            if (!*name) strcpy(name, plan->getFeatureNameByIndex(i).c_str());
        }
}
