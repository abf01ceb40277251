// Internal definitions shared by the host executor and the CUDA kernels.
#pragma once
#include <map>
#include <string>
#include <vector>
#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/wndcharm_gb300.h"

namespace wc {

// Feature algorithms of the reference (src/FeatureAlgorithms.h): the 15
// grayscale FeatureAlgorithm singletons, in this project's numbering.
enum Alg {
    A_CHEBFOURIER = 0, A_CHEB, A_ZERNIKE, A_HARALICK, A_MSHIST, A_TAMURA, A_COMB, A_RADON,
    A_FRACTAL, A_PIXSTATS, A_EDGEF, A_OBJ, A_INVOBJ, A_GABOR, A_GINI, A_COLORHIST, A_COUNT
};
// Image transforms (src/ImageTransforms.h): Fourier, Chebyshev, Wavelet, Edge,
// and for colour images Color (the fuzzy colour index), Hue, and "Color
// Transform", the name the reference's colour plans use, which its lookup
// resolves to an EmptyTransform (a copy of the source plane).
enum Xf { X_FOURIER = 0, X_CHEBYSHEV, X_WAVELET, X_EDGE, X_COLOR, X_HUE, X_CTCOPY, X_COUNT };

extern const char *const kAlgName[A_COUNT];
extern const int kAlgN[A_COUNT];
extern const char *const kXfName[X_COUNT];

// One image plane in the plane arena (row-major doubles).
struct Plane {
    long long off;  // element offset into the arena
    int w, h;
};

// Per-plane statistics (ImageMatrix::stats, a Moments2): min, max, mean,
// M2/(n-1) when n > 2 (0 otherwise), plus the plain sum.
struct PlaneStats {
    double mn, mx, mean, var, sum;
    long long n;
};

// A feature job: compute one algorithm on one plane, write n values at `out`
// (element offset into the feature matrix).
struct FJob {
    int plane;
    int img;
    long long out;
};

// A transform job: dst = T(src).
struct TJob {
    int src, dst;
};

// Optional per-stage timing with CUDA events on the engine's stream.
struct Prof {
    bool on = false;
    bool serial = false;  // every lane on the engine's stream: each stage timed alone
    struct Mark {
        std::string name;
        cudaEvent_t a, b;
    };
    std::vector<Mark> pending;
    std::vector<std::string> order;
    std::vector<double> ms;
    std::vector<double> t0, t1;  // earliest start, latest end (ms after the batch's first mark)
    std::vector<long long> calls;
    long long begin(const std::string &name, cudaStream_t st) {
        if (!on) return -1;
        Mark m{name, nullptr, nullptr};
        cudaEventCreate(&m.a);
        cudaEventCreate(&m.b);
        cudaEventRecord(m.a, st);
        pending.push_back(m);
        return (long long)pending.size() - 1;
    }
    void end(long long idx, cudaStream_t st) {
        if (!on || idx < 0 || idx >= (long long)pending.size()) return;
        cudaEventRecord(pending[idx].b, st);
    }
    // a host-side stage (wall milliseconds); it has no place on the device timeline (start, end -1)
    void host(const std::string &name, double t) {
        if (!on) return;
        size_t k = 0;
        while (k < order.size() && order[k] != name) k++;
        if (k == order.size()) {
            order.push_back(name);
            ms.push_back(0);
            calls.push_back(0);
            t0.push_back(-1);
            t1.push_back(-1);
        }
        ms[k] += t;
        calls[k] += 1;
    }
    void collect() {  // after the stream has been synchronised
        cudaEvent_t ref = pending.empty() ? nullptr : pending[0].a;
        for (auto &m : pending) {
            float t = 0, s0 = 0, s1 = 0;
            cudaEventElapsedTime(&t, m.a, m.b);
            cudaEventElapsedTime(&s0, ref, m.a);
            cudaEventElapsedTime(&s1, ref, m.b);
            size_t k = 0;
            while (k < order.size() && order[k] != m.name) k++;
            if (k == order.size()) {
                order.push_back(m.name);
                ms.push_back(0);
                calls.push_back(0);
                t0.push_back(s0);
                t1.push_back(s1);
            }
            ms[k] += t;
            calls[k] += 1;
            t0[k] = t0[k] < s0 ? t0[k] : s0;
            t1[k] = t1[k] > s1 ? t1[k] : s1;
        }
        for (auto &m : pending) {
            cudaEventDestroy(m.a);
            cudaEventDestroy(m.b);
        }
        pending.clear();
    }
};

// Engine options (wc_engine_set_option).
struct Opts {
    // mixed form: Haralick f14 (Q, Hessenberg reduction, real Schur) through the
    // FP64 chain, bit-identical to the FP64 form, instead of pairs of floats
    int f14_exact = 1;
    // real-Schur iterations allowed per tone (Eigen's m_maxIterationsPerRow)
    int qr_iter_per_tone = 40;
    // union-find iterations allowed per pixel link in the object labelling;
    // 0: the plane's pixel count (a bound no correct run reaches)
    long long union_find_cap = 0;
    // mixed form: Chebyshev-Fourier sums on the tensor cores (planes of one size)
    int cf_tc = 1;
};

// Online autotuner of launch shapes (the engine's own): a stage with several
// candidate shapes asks pick(key, n) per batch; each candidate is tried once
// (explore: its launch bracketed by CUDA events on its stream), and once all
// have a time the fastest is kept for that key (exploit).  Keys name the stage
// and a size class, so a new batch size or image size is tuned again.
struct Tuner {
    bool on = true;
    struct State {
        std::vector<float> ms;  // per candidate: measured time (< 0: not yet)
        int chosen = -1;
    };
    std::map<std::string, State> st;
    struct Pending {
        std::string key;
        int cand;
        cudaEvent_t a, b;
    };
    std::vector<Pending> pend;
    // candidate for this batch (0 when tuning is off)
    int pick(const std::string &key, int n) {
        if (!on || n <= 1) return 0;
        State &s = st[key];
        if ((int)s.ms.size() != n) s.ms.assign(n, -1.f);
        if (s.chosen >= 0) return s.chosen;
        for (int c = 0; c < n; c++)
            if (s.ms[c] < 0) return c;
        return 0;
    }
    bool exploring_any() const {
        if (!on) return false;
        for (auto &kv : st)
            if (kv.second.chosen < 0) return true;
        return false;
    }
    bool exploring(const std::string &key) const {
        auto it = st.find(key);
        return on && it != st.end() && it->second.chosen < 0;
    }
    void begin(const std::string &key, int cand, cudaStream_t s, Pending &p) {
        p.key = key;
        p.cand = cand;
        p.a = p.b = nullptr;
        if (cudaEventCreate(&p.a) != cudaSuccess || cudaEventCreate(&p.b) != cudaSuccess) {
            cudaGetLastError();
            return;
        }
        cudaEventRecord(p.a, s);
    }
    void end(Pending &p, cudaStream_t s) {
        if (!p.a) return;
        cudaEventRecord(p.b, s);
        pend.push_back(p);
    }
    // after the batch has completed: record the times, choose where all are known
    void collect() {
        for (auto &p : pend) {
            float ms = -1.f;
            if (cudaEventElapsedTime(&ms, p.a, p.b) != cudaSuccess) {
                cudaGetLastError();
                ms = -1.f;
            }
            cudaEventDestroy(p.a);
            cudaEventDestroy(p.b);
            State &s = st[p.key];
            if (ms >= 0 && p.cand < (int)s.ms.size() && s.chosen < 0) s.ms[p.cand] = ms;
            bool all = !s.ms.empty();
            for (float v : s.ms) all &= v >= 0;
            if (all && s.chosen < 0) {
                int b = 0;
                for (int c = 1; c < (int)s.ms.size(); c++)
                    if (s.ms[c] < s.ms[b]) b = c;
                s.chosen = b;
            }
        }
        pend.clear();
    }
};

// Launch context handed to every kernel launcher.
struct Ctx {
    cudaStream_t st;
    long long *launches;  // incremented per kernel launch
    int prec;             // WC_PREC_FP64 or WC_PREC_MIXED
    int sms;              // multiprocessors on the device
    Prof *prof;
    const Opts *opt;      // the engine's options
    Tuner *tune;          // the engine's launch-shape tuner
};
struct ProfScope {  // may nest (e.g. a family's phases inside the family)
    Ctx &c;
    long long idx = -1;
    ProfScope(Ctx &c_, const char *name) : c(c_) { if (c.prof) idx = c.prof->begin(name, c.st); }
    ~ProfScope() { if (c.prof) c.prof->end(idx, c.st); }
};

}  // namespace wc
