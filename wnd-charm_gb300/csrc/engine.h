// The engine object behind the C ABI's wc_engine handle, and the device
// buffers it owns.  Shared by the executor (engine.cu) and the sampling entry
// points (sampling.cu).
#pragma once
#include <cuda_runtime.h>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/wndcharm_gb300.h"
#include "wc_features.h"

namespace wc {

#define CK(x)                                                                                         \
    do {                                                                                              \
        cudaError_t e_ = (x);                                                                         \
        if (e_ != cudaSuccess) return set_err(WC_ERR_CUDA, "%s failed: %s", #x, cudaGetErrorString(e_)); \
    } while (0)

// grow-only device buffer
struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    int ensure(size_t bytes) {
        if (bytes <= cap) return WC_OK;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t want = bytes + bytes / 4 + 4096;
        if (cudaMalloc(&p, want) != cudaSuccess) {
            cudaGetLastError();
            return set_err(WC_ERR_NOMEM, "cudaMalloc of %zu bytes failed", want);
        }
        cap = want;
        return WC_OK;
    }
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

// Host-computed tables kept on the device: Chebyshev bases, FFT twiddles.
struct Tables {
    std::vector<double> host;
    std::map<std::string, long long> idx;
    DevBuf dev;
    bool dirty = true;
    // the generator runs only for a key not seen before (tables persist across batches)
    template <typename Gen>
    long long add_lazy(const std::string &key, Gen gen) {
        auto it = idx.find(key);
        if (it != idx.end()) return it->second;
        return add(key, gen());
    }
    long long add(const std::string &key, const std::vector<double> &v) {
        auto it = idx.find(key);
        if (it != idx.end()) return it->second;
        long long off = (long long)host.size();
        host.insert(host.end(), v.begin(), v.end());
        while (host.size() % 32) host.push_back(0.0);
        idx[key] = off;
        dirty = true;
        return off;
    }
    int sync(cudaStream_t st) {
        if (!dirty) return WC_OK;
        int r = dev.ensure(host.size() * sizeof(double));
        if (r) return r;
        CK(cudaMemcpyAsync(dev.p, host.data(), host.size() * sizeof(double), cudaMemcpyHostToDevice, st));
        CK(cudaStreamSynchronize(st));
        dirty = false;
        return WC_OK;
    }
    const double *d() const { return (const double *)dev.p; }
};

// The FFT description of one length, its twiddles added to the tables (engine.cu).
FFTPlan fft_plan(Tables &tabs, int n);

// Runs a plan over a batch on the engine's stream (engine.cu).
struct Plan;
int run_batch(wc_engine *E, const Plan &plan, const wc_image_desc *imgs, int n, double *dfeat,
              std::vector<Plane> *planes_out = nullptr);
// wc_extract_batch with the engine lock held.
int extract_locked(wc_engine *E, const Plan &plan, const wc_image_desc *imgs, int n, double *out, int out_on_device);

}  // namespace wc

namespace wc {
// One captured batch (option "graph"): the launches of a batch of one shape
// (plan, image sizes and types, output), replayed with cudaGraphLaunch after
// the batch's metadata and pixels are uploaded as the normal path uploads them.
struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    std::vector<char> hmeta;        // the batch's metadata blob (jobs, plane table, offsets)
    std::vector<size_t> in_off;     // each host image's place in the staging buffer
    std::vector<void *> bufs;       // the device buffers the launches address, as captured
    long long launches = 0;         // kernels in the graph
};
}  // namespace wc

struct wc_engine {
    int dev = 0;
    cudaStream_t st = 0;
    int prec = WC_PREC_FP64;
    int sms = 1;
    long long launches = 0;
    wc::DevBuf arena, feat, ws, meta, stage;
    wc::DevBuf pre, pre_meta;  // preprocessing: images, opened and sample planes; jobs and positions
    wc::DevBuf clr;            // HSV colour planes of the batch's RGB images
    wc::DevBuf tiffbuf;        // wc_tiff_read_device: stored strips, decoded bytes, tables
    wc::Tables tabs;
    std::vector<char> hmeta, hpre;
    std::mutex mu;
    wc::Prof prof;
    wc::Opts opts;
    wc::Tuner tune;
    cudaStream_t lanes[WC_LANES] = {};
    cudaEvent_t fork_ev = nullptr, early_ev = nullptr, join_ev[WC_LANES] = {};
    // CUDA graphs of repeated batch shapes (option "graph"; engine.cu)
    int graph = 0;
    cudaStream_t own_st = nullptr;  // captures run here when the caller's stream is the legacy default
    bool capture = false;           // run_batch: begin a capture once the uploads are queued
    std::map<std::string, wc::GraphEntry> graphs;
    std::vector<std::string> graph_fifo;
    std::map<std::string, int> graph_seen;  // batches of a shape run without a graph so far
    long long graph_captures = 0, graph_replays = 0, graph_failures = 0;
    std::vector<size_t> last_in_off;  // run_batch: the staging offsets and metadata size it used
    size_t last_meta_used = 0;
};
