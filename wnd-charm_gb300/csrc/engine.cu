// The engine: host-side executor of a feature plan over a batch of images on
// one GPU, and the C ABI (include/wndcharm_gb300.h).
//
// Replaces FeatureComputationPlanExecutor::run (src/Tasks.cpp:275-295).  The
// reference walks the plan's node tree one image at a time and caches each
// transform result by node key; here every node of every image in the batch
// is a plane in one HBM arena, each transform runs as one launch over all
// (source, destination) plane pairs of its depth, and each feature family runs
// as one launch over all (plane, output column) jobs of the batch.
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/wndcharm_gb300.h"
#include "wc_features.h"
#include "kernels.h"
#include "plan.h"
#include "engine.h"

namespace wc {

static thread_local std::string g_err;
int set_err(int code, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}


// Chebyshev basis of Chebyshev2D for a line of `len` samples and N terms:
// tab[x*N + j] = T_j(x_x) * (j ? 2 : 1) / len / 2, x_x = 2(x+1)/len - 1,
// T_j = cos(j * acos(x)) (TNx and getChCoeff1D, src/transforms/chebyshev.cpp:39-102).
std::vector<double> cheb_table(int len, int N) {
    std::vector<double> t((size_t)len * N);
    for (int a = 0; a < len; a++) {
        double x = 2 * (double)(a + 1) / (double)len - 1;
        double ac = (std::fabs(x) > 1) ? 0 : std::acos(x);
        for (int j = 0; j < N; j++) {
            double T = (j == 0) ? 1.0 : std::cos(ac * j);
            double tj = (j == 0) ? T / (double)len : T * 2 / (double)len;
            t[(size_t)a * N + j] = tj / 2;
        }
    }
    return t;
}

FFTPlan fft_plan(Tables &tabs, int n) {
    FFTPlan P;
    memset(&P, 0, sizeof P);
    P.n = n;
    int m = n;
    std::vector<int> r;
    while (m % 8 == 0) { r.push_back(8); m /= 8; }
    while (m % 4 == 0) { r.push_back(4); m /= 4; }
    while (m % 2 == 0) { r.push_back(2); m /= 2; }
    for (int p = 3; (long)p * p <= m; p += 2)
        while (m % p == 0) { r.push_back(p); m /= p; }
    if (m > 1) r.push_back(m);
    P.nstages = (int)r.size();
    for (size_t i = 0; i < r.size() && i < 16; i++) P.radix[i] = r[i];
    P.tw_off = tabs.add_lazy("tw" + std::to_string(n), [n] {
        std::vector<double> tw(2 * (size_t)n);
        const double two_pi = 6.283185307179586476925286766559;
        for (int k = 0; k < n; k++) {
            double a = two_pi * (double)k / (double)n;
            tw[2 * k] = std::cos(a);
            tw[2 * k + 1] = -std::sin(a);
        }
        return tw;
    });
    return P;
}

}  // namespace wc

using namespace wc;


namespace wc {

// Bump allocator over a byte region; `plan` mode only measures.
struct Bump {
    size_t used = 0;
    size_t take(size_t bytes) {
        size_t off = (used + 255) & ~(size_t)255;
        used = off + bytes;
        return off;
    }
};

struct Node {
    int parent, xf, depth;
    std::vector<int> chain;
};

static size_t pixel_bytes(int dtype) {
    switch (dtype) {
        case WC_U8: return 1;
        case WC_U16: return 2;
        case WC_F32: return 4;
        case WC_RGB8: return 3;
        case WC_RGB16: return 6;
        default: return 8;
    }
}

static int out_shape(int xf, int w, int h, int &ow, int &oh) {
    switch (xf) {
        case X_FOURIER: ow = w; oh = h; return 0;
        case X_EDGE:
        case X_COLOR:
        case X_HUE:
        case X_CTCOPY: ow = w; oh = h; return 0;
        case X_WAVELET: ow = 2 * ((w + 9) / 2); oh = 2 * ((h + 9) / 2); return 0;
        case X_CHEBYSHEV: {
            int N = w < h ? w : h;
            ow = N;
            oh = h < N ? h : N;
            return 0;
        }
    }
    return -1;
}

// Runs `plan` over `n` images; `dfeat` receives n x n_features on the device.
int run_batch(wc_engine *E, const Plan &plan, const wc_image_desc *imgs, int n, double *dfeat,
              std::vector<Plane> *planes_out) {
    const auto h0 = std::chrono::steady_clock::now();
    auto host_ms = [&h0]() { return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - h0).count(); };
    Ctx ctx{E->st, &E->launches, E->prec, E->sms, &E->prof, &E->opts, &E->tune};
    // ---- nodes: every prefix of every group's transform chain
    std::vector<Node> nodes(1);
    nodes[0] = {-1, -1, 0, {}};
    std::map<std::vector<int>, int> node_of;
    node_of[{}] = 0;
    std::vector<int> group_node(plan.groups.size());
    for (size_t g = 0; g < plan.groups.size(); g++) {
        std::vector<int> pre;
        int cur = 0;
        for (int t : plan.groups[g].chain) {
            pre.push_back(t);
            auto it = node_of.find(pre);
            if (it == node_of.end()) {
                Node nd{cur, t, (int)pre.size(), pre};
                nodes.push_back(nd);
                it = node_of.emplace(pre, (int)nodes.size() - 1).first;
            }
            cur = it->second;
        }
        group_node[g] = cur;
    }
    const int NN = (int)nodes.size();
    int maxdepth = 0;
    for (auto &nd : nodes) maxdepth = std::max(maxdepth, nd.depth);

    // ---- colour: only the root plane and its "Color Transform" copies carry
    // the HSV plane that Color, Hue and the Color Histogram read
    std::vector<char> colour_node(NN, 0);
    colour_node[0] = 1;
    bool needs_colour = false;
    for (int k = 1; k < NN; k++) {  // parents precede children
        if (nodes[k].xf == X_CTCOPY) colour_node[k] = colour_node[nodes[k].parent];
        if (nodes[k].xf == X_COLOR || nodes[k].xf == X_HUE) {
            if (!colour_node[nodes[k].parent])
                return set_err(WC_ERR_UNSUPPORTED, "the %s transform reads the colour plane, which only the image "
                               "itself (or a Color Transform copy) has", kXfName[nodes[k].xf]);
            needs_colour = true;
        }
    }
    for (size_t g = 0; g < plan.groups.size(); g++)
        if (plan.groups[g].alg == A_COLORHIST) {
            if (!colour_node[group_node[g]])
                return set_err(WC_ERR_UNSUPPORTED, "Color Histogram reads the colour plane: only of the image itself");
            needs_colour = true;
        }
    bool any_rgb = false;
    for (int b = 0; b < n; b++) {
        const bool rgb = imgs[b].dtype == WC_RGB8 || imgs[b].dtype == WC_RGB16;
        if (needs_colour && !rgb) return set_err(WC_ERR_ARG, "image %d: the plan's colour features need an RGB image", b);
        any_rgb |= rgb;
    }

    // ---- planes
    std::vector<Plane> planes((size_t)n * NN);
    size_t arena_elems = 0;
    for (int b = 0; b < n; b++) {
        if (imgs[b].width < 1 || imgs[b].height < 1 || !imgs[b].pixels)
            return set_err(WC_ERR_ARG, "image %d: bad size or null pixels", b);
        if (imgs[b].width > WC_MAX_SIDE || imgs[b].height > WC_MAX_SIDE ||
            (long long)imgs[b].width * imgs[b].height > WC_MAX_PIXELS)
            return set_err(WC_ERR_ARG, "image %d: %d x %d is larger than this build accepts (sides <= %d, <= %lld pixels)",
                           b, imgs[b].width, imgs[b].height, WC_MAX_SIDE, (long long)WC_MAX_PIXELS);
        if (imgs[b].dtype < WC_U8 || imgs[b].dtype > WC_RGB16)
            return set_err(WC_ERR_ARG, "image %d: unknown pixel type %d", b, imgs[b].dtype);
        for (int k = 0; k < NN; k++) {
            Plane &P = planes[(size_t)b * NN + k];
            if (k == 0) {
                P.w = imgs[b].width;
                P.h = imgs[b].height;
            } else {
                const Plane &Q = planes[(size_t)b * NN + nodes[k].parent];
                out_shape(nodes[k].xf, Q.w, Q.h, P.w, P.h);
            }
            P.off = (long long)arena_elems;
            arena_elems += ((size_t)P.w * P.h + 31) & ~(size_t)31;
        }
    }
    int r = E->arena.ensure(arena_elems * sizeof(double));
    if (r) return r;
    double *arena = (double *)E->arena.p;

    // ---- transform jobs, grouped by (depth, transform)
    struct TGroup { std::vector<TJob> jobs; int maxw = 0, maxh = 0; };
    std::vector<std::vector<TGroup>> tg(maxdepth + 1, std::vector<TGroup>(X_COUNT));
    for (int k = 1; k < NN; k++)
        for (int b = 0; b < n; b++) {
            TGroup &G = tg[nodes[k].depth][nodes[k].xf];
            int src = b * NN + nodes[k].parent, dst = b * NN + k;
            G.jobs.push_back({src, dst});
            G.maxw = std::max(G.maxw, planes[src].w);
            G.maxh = std::max(G.maxh, planes[src].h);
        }

    // ---- feature jobs per algorithm
    std::vector<std::vector<FJob>> fj(A_COUNT);
    for (size_t g = 0; g < plan.groups.size(); g++)
        for (int b = 0; b < n; b++)
            fj[plan.groups[g].alg].push_back({b * NN + group_node[g], b, (long long)b * plan.n_features + plan.groups[g].offset});

    // ---- host metadata + workspace plan
    Bump meta, ws;
    struct Blob { size_t off; const void *src; size_t bytes; };
    std::vector<Blob> blobs;
    std::vector<std::vector<char>> owned;
    auto put = [&](const void *p, size_t bytes) -> size_t {
        size_t off = meta.take(bytes ? bytes : 1);
        blobs.push_back({off, p, bytes});
        return off;
    };
    auto put_vec = [&](auto &v) -> size_t { return put(v.data(), v.size() * sizeof(v[0])); };
    auto put_copy = [&](const void *p, size_t bytes) -> size_t {
        owned.emplace_back((const char *)p, (const char *)p + bytes);
        return put(owned.back().data(), bytes);
    };
    const size_t m_planes = put_vec(planes);
    const size_t m_stats = meta.take(sizeof(PlaneStats) * planes.size());
    // colour planes (HSV bytes) of the RGB images, and the fuzzy classifier's table
    std::vector<long long> clr_off(n, 0);
    size_t clr_bytes = 0;
    long long fuzzy_tab = 0;
    for (int b = 0; b < n; b++)
        if (imgs[b].dtype == WC_RGB8 || imgs[b].dtype == WC_RGB16) {
            clr_off[b] = (long long)clr_bytes;
            clr_bytes += ((size_t)3 * imgs[b].width * imgs[b].height + 255) & ~(size_t)255;
        }
    const size_t m_clr = put_vec(clr_off);
    if (any_rgb) fuzzy_tab = E->tabs.add_lazy("fuzzy colours", [] { return fuzzy_membership_table(); });

    struct TL { size_t jobs, aux1, aux2, aux3; size_t ws; };
    std::vector<std::vector<TL>> tl(maxdepth + 1, std::vector<TL>(X_COUNT));
    for (int d = 1; d <= maxdepth; d++)
        for (int x = 0; x < X_COUNT; x++) {
            TGroup &G = tg[d][x];
            if (G.jobs.empty()) continue;
            TL &L = tl[d][x];
            L.jobs = put_vec(G.jobs);
            std::vector<long long> offs;
            if (x == X_WAVELET) {
                size_t tot = 0;
                for (auto &j : G.jobs) {
                    offs.push_back((long long)tot);
                    tot += (size_t)planes[j.src].w * ((planes[j.src].h + 9) / 2) * 2 + 32;
                }
                L.ws = ws.take(tot * sizeof(double));
                L.aux1 = put_copy(offs.data(), offs.size() * sizeof(long long));
            } else if (x == X_FOURIER) {
                size_t tot = 0;
                std::vector<FFTPlan> fp;
                std::map<int, int> idx;
                std::vector<int> py, px;
                for (auto &j : G.jobs) {
                    const Plane &S = planes[j.src];
                    offs.push_back((long long)tot);
                    tot += (size_t)S.w * (S.h / 2 + 1) * 2 + 32;
                    for (int len : {S.h, S.w}) {
                        if (len > kMaxFFT) return set_err(WC_ERR_UNSUPPORTED, "Fourier: side %d > %d", len, kMaxFFT);
                        if (!idx.count(len)) { idx[len] = (int)fp.size(); fp.push_back(fft_plan(E->tabs, len)); }
                    }
                    py.push_back(idx[S.h]);
                    px.push_back(idx[S.w]);
                }
                L.ws = ws.take(tot * sizeof(double));
                L.aux1 = put_copy(offs.data(), offs.size() * sizeof(long long));
                L.aux2 = put_copy(fp.data(), fp.size() * sizeof(FFTPlan));
                std::vector<int> pyx(py);
                pyx.insert(pyx.end(), px.begin(), px.end());
                L.aux3 = put_copy(pyx.data(), pyx.size() * sizeof(int));
            } else if (x == X_CHEBYSHEV) {
                size_t tot = 0;
                std::vector<long long> toff;
                for (auto &j : G.jobs) {
                    const Plane &S = planes[j.src];
                    int N = std::min(S.w, S.h);
                    offs.push_back((long long)tot);
                    tot += (size_t)S.h * N + 32;
                    toff.push_back(E->tabs.add_lazy("ch" + std::to_string(S.w) + "_" + std::to_string(N),
                                                    [&] { return cheb_table(S.w, N); }));
                    toff.push_back(E->tabs.add_lazy("ch" + std::to_string(S.h) + "_" + std::to_string(N),
                                                    [&] { return cheb_table(S.h, N); }));
                }
                L.ws = ws.take(tot * sizeof(double));
                L.aux1 = put_copy(offs.data(), offs.size() * sizeof(long long));
                L.aux2 = put_copy(toff.data(), toff.size() * sizeof(long long));
            }
        }

    // feature-family preparation (tables, workspace, metadata)
    FeatureSetup fs;
    fs.prec = E->prec;
    fs.cf_tc = E->opts.cf_tc;
    fs.planes = &planes;
    fs.fj = &fj;
    fs.tabs_add = [&](const std::string &k, const std::function<std::vector<double>()> &gen) {
        return E->tabs.add_lazy(k, gen);
    };
    fs.fft_plan = [&](int len) { return fft_plan(E->tabs, len); };
    fs.put_copy = put_copy;
    fs.ws_take = [&](size_t bytes) { return ws.take(bytes); };
    fs.meta_take = [&](size_t bytes) { return meta.take(bytes); };
    r = features_prepare(fs);
    if (r) return r;

    // ---- device buffers and uploads
    size_t in_bytes = 0;
    std::vector<size_t> in_off(n);
    for (int b = 0; b < n; b++) {
        if (imgs[b].on_device) continue;
        size_t es = pixel_bytes(imgs[b].dtype);
        in_off[b] = in_bytes;
        in_bytes += ((size_t)imgs[b].width * imgs[b].height * es + 255) & ~(size_t)255;
    }
    if ((r = E->meta.ensure(meta.used + 256))) return r;
    if ((r = E->ws.ensure(ws.used + 256))) return r;
    if ((r = E->stage.ensure(in_bytes + 256))) return r;
    if ((r = E->clr.ensure(clr_bytes + 256))) return r;
    if ((r = E->tabs.sync(E->st))) return r;
    E->hmeta.resize(meta.used + 256);
    for (auto &bl : blobs)
        if (bl.bytes) memcpy(E->hmeta.data() + bl.off, bl.src, bl.bytes);
    char *dm = (char *)E->meta.p;
    char *dw = (char *)E->ws.p;
    E->prof.host("host: plan the batch", host_ms());
    E->last_in_off = in_off;
    E->last_meta_used = meta.used;
    CK(cudaMemcpyAsync(dm, E->hmeta.data(), meta.used, cudaMemcpyHostToDevice, E->st));
    for (int b = 0; b < n; b++)
        if (!imgs[b].on_device)
            CK(cudaMemcpyAsync((char *)E->stage.p + in_off[b], imgs[b].pixels,
                               (size_t)imgs[b].width * imgs[b].height * pixel_bytes(imgs[b].dtype),
                               cudaMemcpyHostToDevice, E->st));
    // a graph holds the launches from here on (the uploads stay outside: a
    // replay repeats them from the new call's buffers)
    if (E->capture) CK(cudaStreamBeginCapture(E->st, cudaStreamCaptureModeThreadLocal));
    for (int b = 0; b < n; b++) {
        const wc_image_desc &I = imgs[b];
        const void *src = I.on_device ? I.pixels : (const void *)((char *)E->stage.p + in_off[b]);
        ProfScope ps(ctx, "convert");
        if (I.dtype == WC_RGB8 || I.dtype == WC_RGB16)
            launch_rgb_ingest(ctx, src, I.dtype, (long long)I.width * I.height, arena + planes[(size_t)b * NN].off,
                              (unsigned char *)E->clr.p + clr_off[b]);
        else
            launch_convert(ctx, src, I.dtype, arena + planes[(size_t)b * NN].off, (long long)I.width * I.height);
    }
    const Plane *dplanes = (const Plane *)(dm + m_planes);
    PlaneStats *dstats = (PlaneStats *)(dm + m_stats);

    FeatureRun fr;
    fr.ctx = &ctx;
    fr.arena = arena;
    fr.planes = dplanes;
    fr.stats = dstats;
    fr.meta = dm;
    fr.ws = dw;
    fr.tabs = E->tabs.d();
    fr.feat = dfeat;
    fr.clr = (const unsigned char *)E->clr.p;
    fr.clr_off = (const long long *)(dm + m_clr);
    fr.fuzzy = E->tabs.d() + fuzzy_tab;
    Ctx lc[WC_LANES];
    for (int k = 0; k < WC_LANES; k++) {
        lc[k] = ctx;
        lc[k].st = E->prof.serial ? ctx.st : E->lanes[k];
    }
    fr.lanes = lc;
    // Families that read only the root planes (Gabor, object and edge features in
    // the standard plans) need nothing from the transforms: once the root planes'
    // statistics exist they start on lanes 3 and 4, beside the transforms.
    bool early = true;
    for (int a : {A_EDGEF, A_OBJ, A_INVOBJ, A_GABOR})
        for (auto &j : fj[a])
            if (j.plane % NN) early = false;
    int r_early = WC_OK;
    if (early) {
        {
            ProfScope ps(ctx, "plane stats");
            launch_plane_stats(ctx, arena, dplanes, (int)planes.size(), dstats, NN, 1);
        }
        CK(cudaEventRecord(E->early_ev, ctx.st));
        for (int k : {3, 4}) CK(cudaStreamWaitEvent(E->lanes[k], E->early_ev, 0));
        r_early = features_launch(fs, fr, 0, true);
    }

    // ---- transforms, depth by depth
    for (int d = 1; d <= maxdepth; d++)
        for (int x = 0; x < X_COUNT; x++) {
            TGroup &G = tg[d][x];
            if (G.jobs.empty()) continue;
            TL &L = tl[d][x];
            const TJob *dj = (const TJob *)(dm + L.jobs);
            const int nj = (int)G.jobs.size();
            ProfScope ps(ctx, kXfName[x]);
            if (x == X_COLOR || x == X_HUE || x == X_CTCOPY)
                launch_color_xf(ctx, arena, dplanes, dj, nj, G.maxw, G.maxh, x, NN, (const unsigned char *)E->clr.p,
                                (const long long *)(dm + m_clr), E->tabs.d() + fuzzy_tab);
            else if (x == X_EDGE) launch_edge(ctx, arena, dplanes, dj, nj, G.maxw, G.maxh);
            else if (x == X_WAVELET)
                launch_wavelet(ctx, arena, dplanes, dj, nj, G.maxw, G.maxh, (double *)(dw + L.ws),
                               (const long long *)(dm + L.aux1));
            else if (x == X_FOURIER)
                launch_fourier(ctx, arena, dplanes, dj, nj, G.maxw, G.maxh, (const FFTPlan *)(dm + L.aux2),
                               (const int *)(dm + L.aux3), (const int *)(dm + L.aux3) + nj, E->tabs.d(),
                               (double *)(dw + L.ws), (const long long *)(dm + L.aux1));
            else
                launch_chebyshev(ctx, arena, dplanes, dj, nj, G.maxw, G.maxh, E->tabs.d(),
                                 (const long long *)(dm + L.aux2), (double *)(dw + L.ws),
                                 (const long long *)(dm + L.aux1));
        }
    {
        ProfScope ps(ctx, "plane stats");
        launch_plane_stats(ctx, arena, dplanes, (int)planes.size(), dstats, NN, early ? 2 : 0);
    }
    // the other families are independent given the planes: fork them onto the
    // lanes (lane 3 takes plane scans after its early Gabor work; lane 4 has
    // nothing that reads a transform), and join every lane back before the
    // caller's next operation
    CK(cudaEventRecord(E->fork_ev, ctx.st));
    for (int k = 0; k < WC_LANES; k++)
        if (!early || k != 4) CK(cudaStreamWaitEvent(E->lanes[k], E->fork_ev, 0));
    r = features_launch(fs, fr, 1, early);
    for (int k = 0; k < WC_LANES; k++) {
        CK(cudaEventRecord(E->join_ev[k], E->lanes[k]));
        CK(cudaStreamWaitEvent(ctx.st, E->join_ev[k], 0));
    }
    E->prof.host("host: plan and queue the batch", host_ms());
    if (r_early) return r_early;
    if (r) return r;
    CK(cudaGetLastError());
    if (planes_out) *planes_out = planes;
    return WC_OK;
}

}  // namespace wc

namespace wc {
int engine_precision(const wc_engine *E) { return E->prec; }
int engine_sms(const wc_engine *E) { return E->sms; }
int engine_device(wc_engine *E, cudaStream_t *st, long long **launches) {
    CK(cudaSetDevice(E->dev));
    *st = E->st;
    *launches = &E->launches;
    return WC_OK;
}
}  // namespace wc

// ================================================================= CUDA graphs
namespace wc {

// What makes two batches replayable by one graph: the plan's groups, the
// images' types, sizes and bit depths (and device addresses), the output.
static std::string batch_key(const Plan &plan, const wc_image_desc *imgs, int n, const double *out,
                             int out_on_device) {
    std::string k;
    auto add = [&](const void *p, size_t b) { k.append((const char *)p, b); };
    add(&plan.n_features, sizeof plan.n_features);
    for (const Group &g : plan.groups) {
        add(&g.alg, sizeof g.alg);
        add(&g.offset, sizeof g.offset);
        for (int t : g.chain) add(&t, sizeof t);
        k.push_back('|');
    }
    add(&n, sizeof n);
    add(&out_on_device, sizeof out_on_device);
    if (out_on_device) add(&out, sizeof out);
    for (int b = 0; b < n; b++) {
        const wc_image_desc &I = imgs[b];
        const int v[5] = {I.dtype, I.width, I.height, I.bits, I.on_device};
        add(v, sizeof v);
        if (I.on_device) add(&I.pixels, sizeof I.pixels);
    }
    return k;
}

// the device buffers a batch's launches address
static std::vector<void *> graph_bufs(wc_engine *E) {
    return {E->arena.p, E->feat.p, E->ws.p, E->meta.p, E->stage.p, E->clr.p, E->tabs.dev.p};
}

static void graph_drop(wc_engine *E, const std::string &key) {
    auto it = E->graphs.find(key);
    if (it == E->graphs.end()) return;
    if (it->second.exec) cudaGraphExecDestroy(it->second.exec);
    E->graphs.erase(it);
    for (size_t i = 0; i < E->graph_fifo.size(); i++)
        if (E->graph_fifo[i] == key) {
            E->graph_fifo.erase(E->graph_fifo.begin() + i);
            break;
        }
}

void graphs_clear(wc_engine *E) {
    for (auto &kv : E->graphs)
        if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    E->graphs.clear();
    E->graph_fifo.clear();
    E->graph_seen.clear();
}

// a replay: the metadata blob and the pixels uploaded as run_batch uploads
// them, then the captured launches
static int graph_replay(wc_engine *E, const GraphEntry &g, const wc_image_desc *imgs, int n) {
    CK(cudaMemcpyAsync(E->meta.p, g.hmeta.data(), g.hmeta.size(), cudaMemcpyHostToDevice, E->st));
    for (int b = 0; b < n; b++) {
        if (imgs[b].on_device) continue;
        if (!imgs[b].pixels) return set_err(WC_ERR_ARG, "image %d: null pixels", b);
        CK(cudaMemcpyAsync((char *)E->stage.p + g.in_off[b], imgs[b].pixels,
                           (size_t)imgs[b].width * imgs[b].height * pixel_bytes(imgs[b].dtype), cudaMemcpyHostToDevice,
                           E->st));
    }
    CK(cudaGraphLaunch(g.exec, E->st));
    E->launches += g.launches;
    E->graph_replays++;
    return WC_OK;
}

static const int kCaptureFailed = 1;  // not a status of the C ABI (those are <= 0)

// after a run_batch that captured: end the capture; on success keep the graph
// and launch it (the capture only recorded the launches)
static int graph_finish(wc_engine *E, const std::string &key, int r, long long launches) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaGraph_t g = nullptr;
    if (cudaStreamIsCapturing(E->st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone &&
        cudaStreamEndCapture(E->st, &g) != cudaSuccess)
        g = nullptr;
    cudaGetLastError();
    if (r) {
        if (g) cudaGraphDestroy(g);
        return r;
    }
    cudaGraphExec_t ex = nullptr;
    const bool ok = g && cudaGraphInstantiate(&ex, g, 0) == cudaSuccess;
    if (g) cudaGraphDestroy(g);
    if (!ok) {
        cudaGetLastError();
        E->graph_failures++;
        return kCaptureFailed;  // the caller runs the batch without a graph
    }
    while (E->graph_fifo.size() >= 16) graph_drop(E, E->graph_fifo.front());
    GraphEntry &ge = E->graphs[key];
    ge.exec = ex;
    ge.hmeta.assign(E->hmeta.begin(), E->hmeta.begin() + E->last_meta_used);
    ge.in_off = E->last_in_off;
    ge.bufs = graph_bufs(E);
    ge.launches = launches;
    E->graph_fifo.push_back(key);
    E->graph_captures++;
    CK(cudaGraphLaunch(ex, E->st));
    return WC_OK;
}

// run_batch, or with the option "graph" a replay of the graph captured for a
// batch of the same shape: a shape is captured the second time it is seen,
// once the launch-shape tuner has chosen every shape it is timing (the
// captured launches then stay those choices), and replays while the device
// buffers it addresses are unchanged
static int run_batch_graphed(wc_engine *E, const Plan &plan, const wc_image_desc *images, int n, double *dfeat,
                             double *out, int out_on_device) {
    if (!E->graph || E->prof.on) return run_batch(E, plan, images, n, dfeat);
    const std::string key = batch_key(plan, images, n, out, out_on_device);
    auto it = E->graphs.find(key);
    if (it != E->graphs.end()) {
        if (it->second.bufs == graph_bufs(E)) return graph_replay(E, it->second, images, n);
        graph_drop(E, key);
    }
    int &seen = E->graph_seen[key];
    const bool cap = seen >= 1 && !E->tune.exploring_any();
    E->capture = cap;
    const long long l0 = E->launches;
    int r = run_batch(E, plan, images, n, dfeat);
    E->capture = false;
    if (!cap) {
        if (!r) seen++;
        return r;
    }
    r = graph_finish(E, key, r, E->launches - l0);
    if (r != kCaptureFailed) return r;
    seen = -1000000;  // this shape does not capture: it runs without a graph from now on
    CK(cudaMemsetAsync(dfeat, 0, (size_t)n * plan.n_features * sizeof(double), E->st));
    return run_batch(E, plan, images, n, dfeat);
}

}  // namespace wc

// ================================================================= C ABI
namespace wc {
int extract_locked(wc_engine *E, const Plan &plan, const wc_image_desc *images, int n, double *out, int out_on_device) {
    CK(cudaSetDevice(E->dev));
    // the legacy default stream cannot be captured: graphs then run on the
    // engine's own blocking stream (ordered with the legacy stream as it is)
    struct Restore {
        wc_engine *E;
        bool on;
        ~Restore() {
            if (on) E->st = 0;
        }
    } restore{E, false};
    if (E->graph && !E->st) {
        if (!E->own_st) CK(cudaStreamCreate(&E->own_st));
        E->st = E->own_st;
        restore.on = true;
    }
    double *dfeat = out;
    size_t fbytes = (size_t)n * plan.n_features * sizeof(double);
    if (!out_on_device) {
        int r = E->feat.ensure(fbytes);
        if (r) return r;
        dfeat = (double *)E->feat.p;
    }
    CK(cudaMemsetAsync(dfeat, 0, fbytes, E->st));
    int r = run_batch_graphed(E, plan, images, n, dfeat, out, out_on_device);
    if (r) return r;
    if (!out_on_device) {
        CK(cudaMemcpyAsync(out, dfeat, fbytes, cudaMemcpyDeviceToHost, E->st));
        CK(cudaStreamSynchronize(E->st));
    }
    if (E->prof.on) {
        CK(cudaStreamSynchronize(E->st));
        E->prof.collect();
    }
    int dev_err = 0;
    if ((r = features_check(E->st, &dev_err))) return r;
    E->tune.collect();  // the batch is complete: its tuning times are final
    if (dev_err) return set_err(WC_ERR_DEVICE, "a kernel reported error code %d", dev_err);
    return WC_OK;
}
}  // namespace wc

extern "C" {

const char *wc_last_error(void) { return g_err.c_str(); }
const char *wc_version(void) { return "wndcharm-gb300 0.1 (sm_103a)"; }

int wc_plan_get(int kind, const wc_plan **out) {
    if (!out || kind < WC_PLAN_SHORT || kind > WC_PLAN_LONG_COLOR) return set_err(WC_ERR_ARG, "wc_plan_get: bad kind");
    *out = static_cast<const wc_plan *>(standard_plan(kind));
    return WC_OK;
}

int wc_plan_from_names(const char *const *groups, int n, wc_plan **out) {
    if (!out || !groups || n < 1) return set_err(WC_ERR_ARG, "wc_plan_from_names: bad arguments");
    std::string err;
    Plan *p = plan_from_names(groups, n, err);
    if (!p) return set_err(WC_ERR_ARG, "%s", err.c_str());
    *out = static_cast<wc_plan *>(p);
    return WC_OK;
}

void wc_plan_free(wc_plan *plan) {
    if (plan && !plan->standard) delete plan;
}

int wc_plan_n_features(const wc_plan *plan) { return plan ? plan->n_features : set_err(WC_ERR_ARG, "null plan"); }

int wc_plan_feature_name(const wc_plan *plan, int i, char *buf, int buflen) {
    if (!plan || !buf || buflen < 1 || i < 0 || i >= plan->n_features) return set_err(WC_ERR_ARG, "bad feature index");
    const std::string &s = plan->names[i];
    strncpy(buf, s.c_str(), (size_t)buflen - 1);
    buf[buflen - 1] = 0;
    return (int)s.size();
}

int wc_plan_n_groups(const wc_plan *plan) { return plan ? (int)plan->groups.size() : set_err(WC_ERR_ARG, "null plan"); }

int wc_plan_group(const wc_plan *plan, int g, char *buf, int buflen, int *offset, int *nf) {
    if (!plan || g < 0 || g >= (int)plan->groups.size()) return set_err(WC_ERR_ARG, "bad group index");
    const Group &G = plan->groups[g];
    if (buf && buflen > 0) {
        strncpy(buf, G.name.c_str(), (size_t)buflen - 1);
        buf[buflen - 1] = 0;
    }
    if (offset) *offset = G.offset;
    if (nf) *nf = kAlgN[G.alg];
    return WC_OK;
}

int wc_engine_create(int device, int precision, wc_engine **out) {
    if (!out) return set_err(WC_ERR_ARG, "null out");
    if (precision != WC_PREC_FP64 && precision != WC_PREC_MIXED) return set_err(WC_ERR_ARG, "bad precision");
    int ndev = 0;
    CK(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return set_err(WC_ERR_ARG, "no CUDA device %d", device);
    CK(cudaSetDevice(device));
    wc_engine *E = new wc_engine;
    E->dev = device;
    E->prec = precision;
    cudaDeviceGetAttribute(&E->sms, cudaDevAttrMultiProcessorCount, device);
    double cs[8];
    const double th[4] = {0, 45, 90, 135};
    for (int k = 0; k < 4; k++) {
        double a = (th[k] * M_PI) / 180;
        cs[2 * k] = cos(a);
        cs[2 * k + 1] = sin(a);
    }
    set_radon_table(cs);
    features_init();
    // lane 0 carries the longest dependent chain (Haralick f14): it gets the
    // highest priority, so its blocks are dispatched ahead of the other lanes'.
    // Lane 5 (the sorts: integer and shared-memory work, no FP64) gets it too:
    // at the lowest priority its blocks waited for SM room until the FP64
    // lanes were done and ended the batch alone.
    int prio_lo = 0, prio_hi = 0;
    CK(cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi));
    for (int k = 0; k < WC_LANES; k++) {
        CK(cudaStreamCreateWithPriority(&E->lanes[k], cudaStreamNonBlocking, (k == 0 || k == 5) ? prio_hi : prio_lo));
        CK(cudaEventCreateWithFlags(&E->join_ev[k], cudaEventDisableTiming));
    }
    CK(cudaEventCreateWithFlags(&E->fork_ev, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&E->early_ev, cudaEventDisableTiming));

    *out = E;
    return WC_OK;
}

void wc_engine_destroy(wc_engine *E) {
    if (!E) return;
    cudaSetDevice(E->dev);
    cudaStreamSynchronize(E->st);
    for (int k = 0; k < WC_LANES; k++) {
        if (E->lanes[k]) cudaStreamDestroy(E->lanes[k]);
        if (E->join_ev[k]) cudaEventDestroy(E->join_ev[k]);
    }
    if (E->fork_ev) cudaEventDestroy(E->fork_ev);
    if (E->early_ev) cudaEventDestroy(E->early_ev);
    graphs_clear(E);
    if (E->own_st) {
        cudaStreamSynchronize(E->own_st);
        cudaStreamDestroy(E->own_st);
    }
    delete E;
}

int wc_engine_set_option(wc_engine *E, const char *name, long long value) {
    if (!E || !name) return set_err(WC_ERR_ARG, "wc_engine_set_option: null argument");
    std::lock_guard<std::mutex> lk(E->mu);
    const std::string k(name);
    if (k == "f14_exact") {
        if (value != 0 && value != 1) return set_err(WC_ERR_ARG, "f14_exact must be 0 or 1");
        E->opts.f14_exact = (int)value;
    } else if (k == "qr_iter_per_tone") {
        if (value < 1 || value > 1000000) return set_err(WC_ERR_ARG, "qr_iter_per_tone must be in 1..1e6");
        E->opts.qr_iter_per_tone = (int)value;
    } else if (k == "autotune") {
        if (value != 0 && value != 1) return set_err(WC_ERR_ARG, "autotune must be 0 or 1");
        E->tune.on = value != 0;
        if (!value) E->tune.st.clear();
    } else if (k == "union_find_cap") {
        if (value < 0) return set_err(WC_ERR_ARG, "union_find_cap must be >= 0");
        E->opts.union_find_cap = value;
    } else if (k == "cf_tensor_cores") {
        if (value != 0 && value != 1) return set_err(WC_ERR_ARG, "cf_tensor_cores must be 0 or 1");
        E->opts.cf_tc = (int)value;
    } else if (k == "graph") {
        if (value != 0 && value != 1) return set_err(WC_ERR_ARG, "graph must be 0 or 1");
        E->graph = (int)value;
    } else {
        return set_err(WC_ERR_ARG, "unknown engine option '%s'", name);
    }
    cudaSetDevice(E->dev);
    graphs_clear(E);  // captured launches hold the old options' choices
    return WC_OK;
}

int wc_engine_tuning_report(wc_engine *E, char *buf, int buflen) {
    if (!E || !buf || buflen < 1) return set_err(WC_ERR_ARG, "bad arguments");
    std::lock_guard<std::mutex> lk(E->mu);
    std::string s;
    for (auto &kv : E->tune.st) {
        s += kv.first + "\t" + std::to_string(kv.second.chosen);
        for (float v : kv.second.ms) s += "\t" + std::to_string(v);
        s += "\n";
    }
    if ((int)s.size() >= buflen) return set_err(WC_ERR_ARG, "buffer too small (%d bytes needed)", (int)s.size() + 1);
    std::memcpy(buf, s.c_str(), s.size() + 1);
    return (int)s.size();
}

int wc_engine_graph_stats(wc_engine *E, long long *stats) {
    if (!E || !stats) return set_err(WC_ERR_ARG, "bad arguments");
    std::lock_guard<std::mutex> lk(E->mu);
    stats[0] = E->graph_captures;
    stats[1] = E->graph_replays;
    stats[2] = E->graph_failures;
    stats[3] = (long long)E->graphs.size();
    return WC_OK;
}

int wc_engine_set_stream(wc_engine *E, void *stream) {
    if (!E) return set_err(WC_ERR_ARG, "null engine");
    E->st = (cudaStream_t)stream;
    return WC_OK;
}

long long wc_engine_launch_count(const wc_engine *E) { return E ? E->launches : 0; }

int wc_engine_profile(wc_engine *E, int on) {
    if (!E) return set_err(WC_ERR_ARG, "null engine");
    E->prof.on = on != 0;
    E->prof.serial = on == 2;
    E->prof.order.clear();
    E->prof.ms.clear();
    E->prof.calls.clear();
    E->prof.t0.clear();
    E->prof.t1.clear();
    return WC_OK;
}

int wc_engine_profile_report(wc_engine *E, char *buf, int buflen) {
    if (!E || !buf || buflen < 1) return set_err(WC_ERR_ARG, "bad arguments");
    std::string s;
    char line[256];
    for (size_t k = 0; k < E->prof.order.size(); k++) {
        snprintf(line, sizeof line, "%s\t%.6f\t%lld\t%.6f\t%.6f\n", E->prof.order[k].c_str(), E->prof.ms[k],
                 E->prof.calls[k], E->prof.t0[k], E->prof.t1[k]);
        s += line;
    }
    strncpy(buf, s.c_str(), (size_t)buflen - 1);
    buf[buflen - 1] = 0;
    return (int)s.size();
}

int wc_extract_batch(wc_engine *E, const wc_plan *plan, const wc_image_desc *images, int n, double *out,
                     int out_on_device) {
    if (!E || !plan || !images || n < 1 || !out) return set_err(WC_ERR_ARG, "wc_extract_batch: bad arguments");
    std::lock_guard<std::mutex> lk(E->mu);
    return extract_locked(E, *plan, images, n, out, out_on_device);
}

int wc_transform(wc_engine *E, const char *name, const double *pixels, int width, int height, double *out,
                 long long cap, int *ow, int *oh) {
    if (!E || !name || !pixels || !out || !ow || !oh || width < 1 || height < 1)
        return set_err(WC_ERR_ARG, "wc_transform: bad arguments");
    int xf = -1;
    for (int i = 0; i < X_COUNT; i++)
        if (!strcmp(name, kXfName[i])) xf = i;
    if (xf < 0) return set_err(WC_ERR_ARG, "wc_transform: unknown transform '%s'", name);
    std::lock_guard<std::mutex> lk(E->mu);
    CK(cudaSetDevice(E->dev));
    Plan p;
    Group g;
    g.alg = A_MSHIST;
    g.chain = {xf};
    g.offset = 0;
    p.groups.push_back(g);
    p.n_features = kAlgN[A_MSHIST];
    int r = E->feat.ensure(p.n_features * sizeof(double));
    if (r) return r;
    wc_image_desc d{pixels, WC_F64, width, height, 16, 0};
    std::vector<Plane> planes;
    if ((r = run_batch(E, p, &d, 1, (double *)E->feat.p, &planes))) return r;
    const Plane &Q = planes[1];
    if ((long long)Q.w * Q.h > cap) return set_err(WC_ERR_ARG, "wc_transform: output needs %d x %d", Q.w, Q.h);
    CK(cudaMemcpyAsync(out, (double *)E->arena.p + Q.off, sizeof(double) * Q.w * Q.h, cudaMemcpyDeviceToHost, E->st));
    CK(cudaStreamSynchronize(E->st));
    *ow = Q.w;
    *oh = Q.h;
    return WC_OK;
}

int wc_extract(wc_engine *E, const wc_plan *plan, const void *pixels, int dtype, int width, int height, int bits,
               double *out_row) {
    wc_image_desc d{pixels, dtype, width, height, bits, 0};
    return wc_extract_batch(E, plan, &d, 1, out_row, 0);
}

}  // extern "C"
