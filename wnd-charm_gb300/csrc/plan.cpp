// Feature computation plans: groups, column offsets and feature names.
//
// Mirrors the reference's FeatureComputationPlan (src/Tasks.h:272-316,
// src/Tasks.cpp:118-173) and its standard plans (src/Tasks.cpp:313-503):
// a group is "Algorithm (Tn (... (T1 ())))", its features occupy
// n_features consecutive columns in the order groups are added, and feature i
// of a group is named "<group> [i]" (src/FeatureNames.cpp:251-296).
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "plan.h"

namespace wc {

const char *const kAlgName[A_COUNT] = {
    "Chebyshev-Fourier Coefficients", "Chebyshev Coefficients", "Zernike Coefficients",
    "Haralick Textures", "Multiscale Histograms", "Tamura Textures", "Comb Moments",
    "Radon Coefficients", "Fractal Features", "Pixel Intensity Statistics", "Edge Features",
    "Otsu Object Features", "Inverse-Otsu Object Features", "Gabor Textures", "Gini Coefficient", "Color Histogram"};
const int kAlgN[A_COUNT] = {32, 32, 72, 28, 24, 6, 48, 12, 20, 5, 28, 34, 34, 7, 1, 20};
const char *const kXfName[X_COUNT] = {"Fourier", "Chebyshev", "Wavelet", "Edge", "Color", "Hue", "Color Transform"};

static std::string chain_text(const std::vector<int> &chain) {
    std::string s = "()";
    for (int t : chain) s = std::string("(") + kXfName[t] + " " + s + ")";
    return s;
}

static void add_group(Plan &p, int alg, std::vector<int> chain) {
    Group g;
    g.alg = alg;
    g.chain = std::move(chain);
    g.name = std::string(kAlgName[alg]) + " " + chain_text(g.chain);
    g.offset = p.n_features;
    for (int i = 0; i < kAlgN[alg]; i++) p.names.push_back(g.name + " [" + std::to_string(i) + "]");
    p.n_features += kAlgN[alg];
    p.groups.push_back(std::move(g));
}

// "Haralick Textures (Wavelet (Edge ()))" -> alg + chain {Edge, Wavelet}
bool parse_group(const std::string &s, int &alg, std::vector<int> &chain) {
    size_t p = s.find(" (");
    if (p == std::string::npos) return false;
    std::string a = s.substr(0, p);
    alg = -1;
    for (int i = 0; i < A_COUNT; i++)
        if (a == kAlgName[i]) alg = i;
    if (alg < 0) return false;
    std::vector<int> outer;
    std::string rest = s.substr(p + 1);
    while (rest.size() > 2 && rest[0] == '(' && rest[1] != ')') {
        // "(Name (" : the longest transform name followed by " ("
        int x = -1;
        size_t len = 0;
        for (int i = 0; i < X_COUNT; i++) {
            const size_t n = strlen(kXfName[i]);
            if (rest.compare(1, n, kXfName[i]) == 0 && rest.compare(1 + n, 2, " (") == 0 && n > len) {
                x = i;
                len = n;
            }
        }
        if (x < 0) return false;
        outer.push_back(x);
        rest = rest.substr(len + 2);
    }
    if (rest.compare(0, 2, "()") != 0) return false;
    chain.assign(outer.rbegin(), outer.rend());
    return true;
}

static Plan make_standard(int kind) {
    Plan p;
    p.standard = true;
    const std::vector<int> R = {}, F = {X_FOURIER}, W = {X_WAVELET}, C = {X_CHEBYSHEV}, E = {X_EDGE};
    auto cat = [](std::vector<int> a, int b) { a.push_back(b); return a; };
    auto A = [&](const std::vector<int> &c) {
        for (int a : {A_EDGEF, A_OBJ, A_INVOBJ, A_GABOR}) add_group(p, a, c);
    };
    auto B = [&](const std::vector<int> &c) {
        for (int a : {A_CHEBFOURIER, A_CHEB, A_ZERNIKE}) add_group(p, a, c);
    };
    auto Cg = [&](const std::vector<int> &c) {
        for (int a : {A_COMB, A_HARALICK, A_MSHIST, A_TAMURA, A_RADON, A_FRACTAL, A_PIXSTATS, A_GINI})
            add_group(p, a, c);
    };
    // StdFeatureComputationPlans::addColorFeatures, src/Tasks.cpp:445-459
    auto colour = [&]() {
        const std::vector<int> CT = {X_CTCOPY}, H = {X_HUE};
        add_group(p, A_COLORHIST, R);
        B(CT); Cg(CT);
        B(H); Cg(H);
        B(cat(H, X_FOURIER)); Cg(cat(H, X_FOURIER));
        B(cat(H, X_CHEBYSHEV)); Cg(cat(H, X_CHEBYSHEV));
    };
    if (kind == 1 || kind == 3) {  // addLongFeatures(plan, colour), src/Tasks.cpp:354-400
        A(R); B(R); Cg(R);
        if (kind == 3) colour();
        B(F); Cg(F);
        B(W); Cg(W);
        B(C); Cg(C);
        Cg(cat(F, X_CHEBYSHEV));
        Cg(cat(F, X_WAVELET));
        B(cat(W, X_FOURIER)); Cg(cat(W, X_FOURIER));
        Cg(cat(C, X_FOURIER));
        Cg(cat(W, X_CHEBYSHEV));
        B(E); Cg(E);
        B(cat(E, X_FOURIER)); Cg(cat(E, X_FOURIER));
        B(cat(E, X_WAVELET)); Cg(cat(E, X_WAVELET));
    } else {  // StdFeatureComputationPlans::addStdFeatures, src/Tasks.cpp:464-503
        const char *names[] = {
            "Chebyshev-Fourier Coefficients ()", "Chebyshev-Fourier Coefficients (Fourier ())",
            "Chebyshev Coefficients ()", "Chebyshev Coefficients (Fourier ())", "Comb Moments ()",
            "Comb Moments (Chebyshev ())", "Comb Moments (Chebyshev (Fourier ()))", "Comb Moments (Fourier ())",
            "Comb Moments (Wavelet ())", "Comb Moments (Wavelet (Fourier ()))", "Edge Features ()",
            "Otsu Object Features ()", "Inverse-Otsu Object Features ()", "Gabor Textures ()",
            "Haralick Textures ()", "Haralick Textures (Chebyshev ())", "Haralick Textures (Chebyshev (Fourier ()))",
            "Haralick Textures (Fourier ())", "Haralick Textures (Wavelet ())",
            "Haralick Textures (Wavelet (Fourier ()))", "Multiscale Histograms ()",
            "Multiscale Histograms (Chebyshev ())", "Multiscale Histograms (Chebyshev (Fourier ()))",
            "Multiscale Histograms (Fourier ())", "Multiscale Histograms (Wavelet ())",
            "Multiscale Histograms (Wavelet (Fourier ()))", "Radon Coefficients ()",
            "Radon Coefficients (Chebyshev ())", "Radon Coefficients (Chebyshev (Fourier ()))",
            "Radon Coefficients (Fourier ())", "Tamura Textures ()", "Tamura Textures (Chebyshev ())",
            "Tamura Textures (Chebyshev (Fourier ()))", "Tamura Textures (Fourier ())", "Tamura Textures (Wavelet ())",
            "Tamura Textures (Wavelet (Fourier ()))", "Zernike Coefficients ()", "Zernike Coefficients (Fourier ())"};
        for (const char *n : names) {
            int alg;
            std::vector<int> ch;
            parse_group(n, alg, ch);
            add_group(p, alg, ch);
        }
        if (kind == 2) colour();  // getFeatureSetColor, src/Tasks.cpp:323-332
    }
    return p;
}

// kind 0: short (1059), 1: long (2919), 2: short colour (2199), 3: long colour (4059)
const Plan *standard_plan(int kind) {
    static wc_plan P[4];
    static std::once_flag once[4];
    if (kind < 0 || kind > 3) kind = 0;
    std::call_once(once[kind], [kind]() { static_cast<Plan &>(P[kind]) = make_standard(kind); });
    return &P[kind];
}

Plan *plan_from_names(const char *const *groups, int n, std::string &err) {
    Plan *p = new wc_plan;
    for (int i = 0; i < n; i++) {
        int alg;
        std::vector<int> ch;
        if (!groups[i] || !parse_group(groups[i], alg, ch)) {
            err = std::string("unknown feature group: ") + (groups[i] ? groups[i] : "(null)");
            delete static_cast<wc_plan *>(p);
            return nullptr;
        }
        for (auto &g : p->groups)
            if (g.alg == alg && g.chain == ch) {
                err = std::string("duplicate feature group: ") + groups[i];
                delete static_cast<wc_plan *>(p);
                return nullptr;
            }
        add_group(*p, alg, ch);
    }
    return p;
}

}  // namespace wc
