// The reference-side binding of the GB300 path, as a maintainer adds it to
// wndchrm: written against the reference's own headers (src/Tasks.h,
// src/cmatrix.h, src/wndchrm_src/signatures.h) and the C ABI
// (include/wndcharm_gb300.h), and linked into the reference library.
//
//   * GB300FeatureComputationPlanExecutor: a FeatureComputationPlanExecutor
//     (src/Tasks.h:318-348) whose run() computes the whole plan for one
//     ImageMatrix on the GPU (wc_extract) instead of walking the plan's nodes
//     on the CPU (src/Tasks.cpp:275-295): same plans, same column offsets,
//     the feature row written at feature_mat_in[dest_row * n_features].
//   * gb300_compute_plan: the body signatures::compute_plan
//     (src/wndchrm_src/signatures.cpp:167-189) takes in the patch, with this
//     executor in place of the CPU one.
//
// Errors: the reference's run() has no status; a failing GPU call throws
// std::runtime_error with wc_last_error()'s message (an engine on a machine
// without a GPU fails at creation).  Colour plans need the image's RGB samples,
// which an ImageMatrix no longer holds (it keeps the gray plane and HSV bytes):
// they are refused here and go through wc_extract_batch with WC_RGB8/WC_RGB16.
#pragma once
#include <string>
#include <vector>

#include "Tasks.h"
#include "wndchrm_src/signatures.h"
#include "wndcharm_gb300.h"

class ImageMatrix;

class GB300FeatureComputationPlanExecutor : public FeatureComputationPlanExecutor {
   public:
    explicit GB300FeatureComputationPlanExecutor(const FeatureComputationPlan *plan_in, int device = 0,
                                                 int precision = WC_PREC_FP64);
    virtual ~GB300FeatureComputationPlanExecutor();
    virtual void run(const ImageMatrix *source_mat, std::vector<double> &feature_mat_in, size_t dest_row);
    virtual void run() {}

   private:
    GB300FeatureComputationPlanExecutor(const GB300FeatureComputationPlanExecutor &);
    void operator=(const GB300FeatureComputationPlanExecutor &);
    void open();
    int device, precision;
    wc_engine *engine;
    wc_plan *own_plan;       // a custom plan, rebuilt from the plan's group names
    const wc_plan *wplan;
};

void gb300_compute_plan(signatures &sig, const ImageMatrix &matrix, const FeatureComputationPlan *plan);
