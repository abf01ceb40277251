// Preprocessing and sampling entry points of the C ABI: the geometry of
// ImageMatrix::OpenImage (src/cmatrix.cpp:252-294) and of the samples of
// TrainingSet::AddImageFile (src/wndchrm_src/TrainingSet.cpp:1442-1481) on the
// host, the pixel work on the GPU (k_pre.cu), then the samples go straight
// from the preprocessing arena into the feature executor.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "engine.h"
#include "kernels.h"
#include "plan.h"

namespace wc {

static int check_sampling(const wc_sampling *s) {
    if (!s) return set_err(WC_ERR_ARG, "null sampling options");
    if (s->rotations < 1 || s->rotations > 4) return set_err(WC_ERR_ARG, "rotations must be 1 to 4, not %d", s->rotations);
    if (s->tiles_x < 1 || s->tiles_y < 1 || (long long)s->tiles_x * s->tiles_y > 65535)
        return set_err(WC_ERR_ARG, "bad tiles %d x %d", s->tiles_x, s->tiles_y);
    if (!(s->downsample_x > 0) || !(s->downsample_y > 0))
        return set_err(WC_ERR_ARG, "downsample ratios must be > 0 (>= 1: none)");
    return WC_OK;
}

// The opened image: crop rectangle, then Downsample's new size
// (new_width = (unsigned)(x_ratio * width), src/cmatrix.cpp:602).
struct Opened {
    int cx, cy, cw, ch, ow, oh;
    bool down;
    double dx, dy;
};

static int opened_geometry(const wc_sampling &s, int w, int h, Opened &o) {
    if (w < 1 || h < 1) return set_err(WC_ERR_ARG, "image of %d x %d pixels", w, h);
    if (w > WC_MAX_SIDE || h > WC_MAX_SIDE || (long long)w * h > WC_MAX_PIXELS)
        return set_err(WC_ERR_ARG, "image of %d x %d pixels is larger than this build accepts", w, h);
    o.cx = o.cy = 0;
    o.cw = w;
    o.ch = h;
    if (s.crop_x >= 0) {
        // submatrix(x, y, x + w - 1, y + h - 1) fails unless the rectangle lies inside
        if (s.crop_y < 0 || s.crop_w < 1 || s.crop_h < 1 || (long long)s.crop_x + s.crop_w > w ||
            (long long)s.crop_y + s.crop_h > h)
            return set_err(WC_ERR_ARG, "bounding rectangle (x %d, y %d, w %d, h %d) is not inside the %d x %d image",
                           s.crop_x, s.crop_y, s.crop_w, s.crop_h, w, h);
        o.cx = s.crop_x;
        o.cy = s.crop_y;
        o.cw = s.crop_w;
        o.ch = s.crop_h;
    }
    const double xr = s.downsample_x > 1 ? 1.0 : s.downsample_x, yr = s.downsample_y > 1 ? 1.0 : s.downsample_y;
    o.dx = 1 / xr;
    o.dy = 1 / yr;
    o.down = !(o.dx == 1 && o.dy == 1);
    o.ow = o.cw;
    o.oh = o.ch;
    if (o.down) {
        o.ow = (int)(unsigned)(xr * o.cw);
        o.oh = (int)(unsigned)(yr * o.ch);
        if (o.ow < 1 || o.oh < 1)
            return set_err(WC_ERR_ARG, "downsampling %d x %d by (%g, %g) leaves no pixels", o.cw, o.ch, xr, yr);
    }
    if (o.ch > 65535 * 8 || o.oh > 65535 * 8) return set_err(WC_ERR_UNSUPPORTED, "image height above %d", 65535 * 8);
    return WC_OK;
}

struct Tile {
    int rot, x1, y1, tw, th;
};

// Sample k of an opened ow x oh plane (enumeration of src/wndchrm_src/wndchrm.cpp:93-124;
// tile sizes of TrainingSet.cpp:1465-1476, including the swap for rotations 1 and 3).
static int sample_geometry(const wc_sampling &s, int ow, int oh, int k, Tile &t) {
    const int tiles = s.tiles_x * s.tiles_y;
    if (k < 0 || k >= s.rotations * tiles) return set_err(WC_ERR_ARG, "sample %d of %d", k, s.rotations * tiles);
    t.rot = k / tiles;
    const int rem = k % tiles, ix = rem / s.tiles_y, iy = rem % s.tiles_y;
    const int rw = (t.rot & 1) ? oh : ow, rh = (t.rot & 1) ? ow : oh;
    if (tiles == 1) {
        t.x1 = t.y1 = 0;
        t.tw = rw;
        t.th = rh;
        return WC_OK;
    }
    long tx, ty;
    if (t.rot == 1 || t.rot == 3) {
        ty = rw / s.tiles_x;
        tx = rh / s.tiles_y;
    } else {
        tx = rw / s.tiles_x;
        ty = rh / s.tiles_y;
    }
    const long x2 = (ix + 1) * tx - 1, y2 = (iy + 1) * ty - 1;
    if (tx < 1 || ty < 1 || x2 >= rw || y2 >= rh)
        return set_err(WC_ERR_ARG,
                       "sample %d: tile (%d, %d) of %ld x %ld pixels does not fit the %d x %d rotated image "
                       "(the reference would reuse the previous sample's pixels)",
                       k, ix, iy, tx, ty, rw, rh);
    t.x1 = (int)(ix * tx);
    t.y1 = (int)(iy * ty);
    t.tw = (int)tx;
    t.th = (int)ty;
    return WC_OK;
}

// Start positions of Downsample's loop over a line of `old` pixels
// (x = 0, x += d while x < old; src/cmatrix.cpp:602-652), the first `keep`.
static void ds_starts(int old, double d, int keep, std::vector<double> &tab) {
    int k = 0;
    for (double x = 0; x < old && k < keep; x += d, k++) tab.push_back(x);
    while (k++ < keep) tab.push_back(0);  // not reached: the loop runs at least `keep` times
    while (tab.size() % 32) tab.push_back(0);
}

static size_t elem_size(int dtype) { return dtype == WC_U8 ? 1 : dtype == WC_U16 ? 2 : dtype == WC_F32 ? 4 : 8; }
static size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

// Queues the preprocessing of n images on the engine's stream and describes
// the resulting sample planes (device FP64): every sample of every image, or
// with only >= 0 sample `only` of each image.
static int prepare_samples(wc_engine *E, const wc_image_desc *imgs, int n, const wc_sampling &s, int only,
                           std::vector<wc_image_desc> &descs) {
    const int per = only >= 0 ? 1 : s.rotations * s.tiles_x * s.tiles_y;
    if ((long long)n * per > 65535 || n > 65535)
        return set_err(WC_ERR_ARG, "%d images x %d samples: at most 65535 samples per call", n, per);
    std::vector<PreJob> jobs(n);
    std::vector<SampleJob> sj;
    std::vector<double> tab;
    std::vector<int> bits(n);
    PreGeomMax g;
    memset(&g, 0, sizeof g);
    size_t stage = 0;
    std::vector<size_t> stage_off(n, 0);
    long long wf_max = 0;  // largest plane that the mean branch normalises
    long long elems = 0;
    auto take = [&](long long cnt) {
        long long o = elems;
        elems += (cnt + 31) & ~31LL;
        return o;
    };
    for (int b = 0; b < n; b++) {
        const wc_image_desc &I = imgs[b];
        if (I.dtype == WC_RGB8 || I.dtype == WC_RGB16)
            return set_err(WC_ERR_UNSUPPORTED, "image %d: colour images are not preprocessed (the reference's Rotate "
                           "and Downsample leave or rebuild the colour plane differently from the gray one)", b);
        if (!I.pixels || I.dtype < WC_U8 || I.dtype > WC_F64)
            return set_err(WC_ERR_ARG, "image %d: null pixels or unknown pixel type %d", b, I.dtype);
        Opened o;
        int r = opened_geometry(s, I.width, I.height, o);
        if (r) return r;
        if (!I.on_device) {
            stage_off[b] = stage;
            stage += round256((size_t)I.width * I.height * elem_size(I.dtype));
        }
        PreJob &J = jobs[b];
        memset(&J, 0, sizeof J);
        J.dtype = I.dtype;
        J.sw = I.width;
        J.cx = o.cx;
        J.cy = o.cy;
        J.cw = o.cw;
        J.ch = o.ch;
        J.a_off = take((long long)o.cw * o.ch);
        J.ow = o.ow;
        J.oh = o.oh;
        if (o.down) {
            J.down = 1;
            J.dx = o.dx;
            J.dy = o.dy;
            J.nw = o.ow;
            J.nh = o.oh;
            J.xs_tab = (long long)tab.size();
            ds_starts(o.cw, o.dx, o.ow, tab);
            J.ys_tab = (long long)tab.size();
            ds_starts(o.ch, o.dy, o.oh, tab);
            J.t_off = take((long long)o.ch * o.ow);
            J.o_off = take((long long)o.ow * o.oh);
            g.down = 1;
        } else {
            J.o_off = J.a_off;
        }
        J.mm = s.norm_min >= 0 && s.norm_max > 0 && s.norm_range > 0;
        J.ms = s.norm_mean > 0;
        J.n_min = s.norm_min;
        J.n_max = s.norm_max;
        J.n_range = (double)s.norm_range;
        J.n_mean = s.norm_mean;
        J.n_std = s.norm_std;
        J.max_range = std::ldexp(1.0, I.bits) - 1;  // pow(2, bits) - 1
        if (J.mm) g.norm_range = 1;
        if (J.ms) {
            g.norm_mean = 1;
            wf_max = std::max(wf_max, (long long)o.ow * o.oh);
        }
        bits[b] = I.bits;
        g.cw = std::max(g.cw, o.cw);
        g.ch = std::max(g.ch, o.ch);
        g.nw = std::max(g.nw, J.nw);
        g.nh = std::max(g.nh, J.nh);
        g.ow = std::max(g.ow, o.ow);
        g.oh = std::max(g.oh, o.oh);
        for (int k = only >= 0 ? only : 0; k < (only >= 0 ? only + 1 : per); k++) {
            Tile t;
            if ((r = sample_geometry(s, o.ow, o.oh, k, t))) return r;
            sj.push_back({b, t.rot, t.x1, t.y1, t.tw, t.th, take((long long)t.tw * t.th)});
            g.tw = std::max(g.tw, t.tw);
            g.th = std::max(g.th, t.th);
        }
    }
    if (tab.empty()) tab.push_back(0);
    // reciprocals for the Welford chain: RN(1/k), RN(1/k - RN(1/k)), k = 1 .. cap,
    // kept by the engine for the largest power-of-two size seen
    long long wf_tab = 0, cap = 1024;
    while (cap < wf_max) cap *= 2;
    if (wf_max) {
        wf_tab = E->tabs.add_lazy("welford" + std::to_string(cap), [cap] {
            std::vector<double> t(2 * (size_t)cap);
            for (long long k = 0; k < cap; k++) {
                const double nn = (double)(k + 1);
                t[k] = 1.0 / nn;
                t[cap + k] = std::fma(-t[k], nn, 1.0) / nn;  // 1 - RN(1/k) * k is exact
            }
            return t;
        });
    }
    const size_t stage_r = round256(stage);
    int r = E->pre.ensure(stage_r + (size_t)elems * sizeof(double));
    if (r) return r;
    char *base = (char *)E->pre.p;
    double *planes = (double *)(base + stage_r);
    for (int b = 0; b < n; b++) jobs[b].src = imgs[b].on_device ? imgs[b].pixels : base + stage_off[b];
    const size_t m_jobs = 0, m_sj = round256(jobs.size() * sizeof(PreJob)),
                 m_tab = m_sj + round256(sj.size() * sizeof(SampleJob)),
                 m_fact = m_tab + round256(tab.size() * sizeof(double)), m_up = m_fact,
                 m_end = m_fact + round256(2 * (size_t)n * sizeof(double));
    if ((r = E->pre_meta.ensure(m_end))) return r;
    if ((r = E->tabs.sync(E->st))) return r;
    E->hpre.assign(m_up, 0);
    memcpy(E->hpre.data() + m_jobs, jobs.data(), jobs.size() * sizeof(PreJob));
    memcpy(E->hpre.data() + m_sj, sj.data(), sj.size() * sizeof(SampleJob));
    memcpy(E->hpre.data() + m_tab, tab.data(), tab.size() * sizeof(double));
    char *dm = (char *)E->pre_meta.p;
    CK(cudaMemcpyAsync(dm, E->hpre.data(), m_up, cudaMemcpyHostToDevice, E->st));
    for (int b = 0; b < n; b++)
        if (!imgs[b].on_device)
            CK(cudaMemcpyAsync(base + stage_off[b], imgs[b].pixels,
                               (size_t)imgs[b].width * imgs[b].height * elem_size(imgs[b].dtype),
                               cudaMemcpyHostToDevice, E->st));
    Ctx ctx{E->st, &E->launches, E->prec, E->sms, &E->prof, &E->opts, &E->tune};
    {
        ProfScope ps(ctx, "preprocess");
        const double *yh = E->tabs.d() + wf_tab;
        launch_preprocess(ctx, (const PreJob *)(dm + m_jobs), n, g, (const double *)(dm + m_tab), yh, yh + cap,
                          (double *)(dm + m_fact), planes, (const SampleJob *)(dm + m_sj), (int)sj.size());
    }
    CK(cudaGetLastError());
    descs.clear();
    for (auto &q : sj) descs.push_back({planes + q.off, WC_F64, q.tw, q.th, bits[q.img], 1});
    return WC_OK;
}

}  // namespace wc

using namespace wc;

extern "C" {

void wc_sampling_default(wc_sampling *s) {
    if (!s) return;
    memset(s, 0, sizeof *s);
    s->crop_x = s->crop_y = s->crop_w = s->crop_h = -1;
    s->downsample_x = s->downsample_y = 1.0;
    s->norm_min = s->norm_max = -1;
    s->norm_range = -1;
    s->norm_mean = s->norm_std = -1;
    s->rotations = 1;
    s->tiles_x = s->tiles_y = 1;
}

int wc_sampling_count(const wc_sampling *s) {
    int r = check_sampling(s);
    if (r) return r;
    return s->rotations * s->tiles_x * s->tiles_y;
}

int wc_sample_size(const wc_sampling *s, int width, int height, int sample, int *out_w, int *out_h) {
    if (!out_w || !out_h) return set_err(WC_ERR_ARG, "wc_sample_size: null output");
    int r = check_sampling(s);
    if (r) return r;
    Opened o;
    if ((r = opened_geometry(*s, width, height, o))) return r;
    Tile t;
    if ((r = sample_geometry(*s, o.ow, o.oh, sample, t))) return r;
    *out_w = t.tw;
    *out_h = t.th;
    return WC_OK;
}

int wc_preprocess(wc_engine *E, const wc_image_desc *image, const wc_sampling *s, int sample, double *out,
                  long long cap, int *out_w, int *out_h, int out_on_device) {
    if (!E || !image || !out || !out_w || !out_h) return set_err(WC_ERR_ARG, "wc_preprocess: bad arguments");
    int r = check_sampling(s);
    if (r) return r;
    std::lock_guard<std::mutex> lk(E->mu);
    CK(cudaSetDevice(E->dev));
    std::vector<wc_image_desc> d;
    if ((r = prepare_samples(E, image, 1, *s, sample, d))) return r;
    const long long npx = (long long)d[0].width * d[0].height;
    if (npx > cap) return set_err(WC_ERR_ARG, "wc_preprocess: the sample has %d x %d pixels", d[0].width, d[0].height);
    CK(cudaMemcpyAsync(out, d[0].pixels, (size_t)npx * sizeof(double),
                       out_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, E->st));
    CK(cudaStreamSynchronize(E->st));
    if (E->prof.on) E->prof.collect();
    *out_w = d[0].width;
    *out_h = d[0].height;
    return WC_OK;
}

int wc_extract_samples(wc_engine *E, const wc_plan *plan, const wc_image_desc *images, int n, const wc_sampling *s,
                       double *out, int out_on_device) {
    if (!E || !plan || !images || n < 1 || !out) return set_err(WC_ERR_ARG, "wc_extract_samples: bad arguments");
    int r = check_sampling(s);
    if (r) return r;
    std::lock_guard<std::mutex> lk(E->mu);
    CK(cudaSetDevice(E->dev));
    std::vector<wc_image_desc> d;
    if ((r = prepare_samples(E, images, n, *s, -1, d))) return r;
    return extract_locked(E, *plan, d.data(), (int)d.size(), out, out_on_device);
}

}  // extern "C"
