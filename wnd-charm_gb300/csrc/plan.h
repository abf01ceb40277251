// Feature computation plans (host side); see plan.cpp.
#pragma once
#include <string>
#include <vector>

#include "wc_internal.h"

namespace wc {

struct Group {
    int alg;
    std::vector<int> chain;  // transforms in application order (first applied first)
    std::string name;        // "Alg (Tn (... (T1 ())))"
    int offset;              // first column in the feature row
};

struct Plan {
    std::vector<Group> groups;
    std::vector<std::string> names;
    int n_features = 0;
    bool standard = false;
};

const Plan *standard_plan(int kind);
Plan *plan_from_names(const char *const *groups, int n, std::string &err);
bool parse_group(const std::string &s, int &alg, std::vector<int> &chain);

}  // namespace wc

struct wc_plan : public wc::Plan {};
