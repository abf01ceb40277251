// Per-family preparation and launch for one batch: builds each family's job
// list, tables and workspace on the host, then launches the family kernels.
#include <algorithm>
#include <cstring>
#include <map>
#include <vector>

#include "../../include/wndcharm_gb300.h"
#include "wc_features.h"
#include "kcommon.cuh"

namespace wc {

__device__ int g_dev_err = 0;

std::vector<double> cheb_table(int len, int N);

void features_init() { set_zernike_tables(); }

// positions of the reference's Downsample loop (x starts at 0, x += dx while
// x < old): src/cmatrix.cpp:602-606
static std::vector<double> ds_positions(int old, double dx) {
    std::vector<double> v;
    for (double x = 0; x < old; x += dx) v.push_back(x);
    return v;
}

int features_check(cudaStream_t st, int *dev_err) {
    int v = 0;
    if (cudaMemcpyFromSymbolAsync(&v, g_dev_err, sizeof(int), 0, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return set_err(WC_ERR_CUDA, "reading the device error word failed: %s", cudaGetErrorString(cudaGetLastError()));
    if (v) {
        int z = 0;
        cudaMemcpyToSymbolAsync(g_dev_err, &z, sizeof(int), 0, cudaMemcpyHostToDevice, st);
        cudaStreamSynchronize(st);
    }
    *dev_err = v;
    return WC_OK;
}

static int maxw_of(const std::vector<Plane> &P, const std::vector<FJob> &J) {
    int m = 0;
    for (auto &j : J) m = std::max(m, P[j.plane].w);
    return m;
}
static int maxh_of(const std::vector<Plane> &P, const std::vector<FJob> &J) {
    int m = 0;
    for (auto &j : J) m = std::max(m, P[j.plane].h);
    return m;
}

int features_prepare(FeatureSetup &fs) {
    const auto &P = *fs.planes;
    const auto &fj = *fs.fj;
    for (int a = 0; a < A_COUNT; a++)
        if (!fj[a].empty()) fs.off["jobs" + std::to_string(a)] = fs.put_copy(fj[a].data(), fj[a].size() * sizeof(FJob));

    // planes that need a sorted copy: PixStats, Gini
    std::map<int, int> slot_of;
    std::vector<int> sort_planes;
    for (int a : {A_PIXSTATS, A_GINI})
        for (auto &j : fj[a])
            if (!slot_of.count(j.plane)) {
                slot_of[j.plane] = (int)sort_planes.size();
                sort_planes.push_back(j.plane);
            }
    if (!sort_planes.empty()) {
        std::vector<long long> koff;
        size_t tot = 0;
        for (int p : sort_planes) {
            koff.push_back((long long)tot);
            tot += ((size_t)P[p].w * P[p].h + 31) & ~(size_t)31;
        }
        fs.off["sort_ids"] = fs.put_copy(sort_planes.data(), sort_planes.size() * sizeof(int));
        fs.off["sort_koff"] = fs.put_copy(koff.data(), koff.size() * sizeof(long long));
        fs.off["sort_keys"] = fs.ws_take(tot * 8);
        fs.off["sort_tmp"] = fs.ws_take(tot * 8);
        fs.off["sort_cnt"] = fs.ws_take(sort_planes.size() * 256 * 512 * sizeof(unsigned int));
        fs.val["sort_n"] = (long long)sort_planes.size();
        for (int a : {A_PIXSTATS, A_GINI}) {
            std::vector<int> slots;
            for (auto &j : fj[a]) slots.push_back(slot_of[j.plane]);
            if (!slots.empty()) fs.off["slots" + std::to_string(a)] = fs.put_copy(slots.data(), slots.size() * sizeof(int));
        }
    }

    // Chebyshev coefficients: N = min(20, W, H) tables and H x N workspace
    if (!fj[A_CHEB].empty()) {
        std::vector<long long> toff, moff;
        size_t tot = 0;
        for (auto &j : fj[A_CHEB]) {
            const Plane &Q = P[j.plane];
            int N = std::min(20, std::min(Q.w, Q.h));
            toff.push_back(fs.tabs_add("ch" + std::to_string(Q.w) + "_" + std::to_string(N), cheb_table(Q.w, N)));
            toff.push_back(fs.tabs_add("ch" + std::to_string(Q.h) + "_" + std::to_string(N), cheb_table(Q.h, N)));
            moff.push_back((long long)tot);
            tot += (size_t)Q.h * N + 32;
        }
        fs.off["cc_tab"] = fs.put_copy(toff.data(), toff.size() * sizeof(long long));
        fs.off["cc_moff"] = fs.put_copy(moff.data(), moff.size() * sizeof(long long));
        fs.off["cc_mid"] = fs.ws_take(tot * sizeof(double));
    }
    // Zernike: per-job centroid moments and per-chunk partials
    if (!fj[A_ZERNIKE].empty()) {
        long long maxpix = 0;
        for (auto &j : fj[A_ZERNIKE]) maxpix = std::max(maxpix, (long long)P[j.plane].w * P[j.plane].h);
        const long long nchunk = (maxpix + 2047) / 2048;
        fs.val["zk_maxpix"] = maxpix;
        fs.off["zk_mom"] = fs.ws_take(fj[A_ZERNIKE].size() * 3 * sizeof(double));
        fs.off["zk_part"] = fs.ws_take(fj[A_ZERNIKE].size() * 2 * nchunk * 72 * sizeof(double));
    }

    // Chebyshev-Fourier: source image (downsampled above 300*300), chunk partials
    if (!fj[A_CHEBFOURIER].empty()) {
        std::vector<CFJob> cj;
        int max_cnt_x = 0, max_w = 0, max_h = 0, nchunk_max = 1;
        for (auto &j : fj[A_CHEBFOURIER]) {
            const Plane &Q = P[j.plane];
            CFJob c;
            memset(&c, 0, sizeof c);
            if ((long)Q.w * Q.h > 300L * 300) {
                double r = std::min(300.0 / (double)Q.w, 300.0 / (double)Q.h);
                double xr = r > 1 ? 1 : r, yr = r > 1 ? 1 : r;
                c.dx = 1 / xr;
                c.down = 1;
                c.new_w = (unsigned)(xr * Q.w);
                c.new_h = (unsigned)(yr * Q.h);
                std::vector<double> xs = ds_positions(Q.w, c.dx), ys = ds_positions(Q.h, 1 / yr);
                c.cnt_x = (int)xs.size();
                c.cnt_y = (int)ys.size();
                char key[96];
                snprintf(key, sizeof key, "ds%d_%.17g", Q.w, c.dx);
                c.xs_tab = fs.tabs_add(key, xs);
                snprintf(key, sizeof key, "ds%d_%.17g", Q.h, 1 / yr);
                c.ys_tab = fs.tabs_add(key, ys);
                c.tmp_ws = (long long)(fs.ws_take((size_t)Q.h * c.cnt_x * sizeof(double)) / sizeof(double));
            } else {
                c.new_w = Q.w;
                c.new_h = Q.h;
                c.dx = 1;
            }
            c.src_ws = (long long)(fs.ws_take((size_t)c.new_w * c.new_h * sizeof(double)) / sizeof(double));
            c.nchunk = (int)(((long long)c.new_w * c.new_h + 1023) / 1024);
            nchunk_max = std::max(nchunk_max, c.nchunk);
            max_cnt_x = std::max(max_cnt_x, c.cnt_x);
            max_w = std::max(max_w, c.new_w);
            max_h = std::max(max_h, c.new_h);
            cj.push_back(c);
        }
        fs.off["cf_jobs"] = fs.put_copy(cj.data(), cj.size() * sizeof(CFJob));
        fs.off["cf_part"] = fs.ws_take(cj.size() * (size_t)nchunk_max * 2 * 529 * sizeof(double));
        fs.val["cf_nchunk"] = nchunk_max;
        fs.val["cf_cntx"] = max_cnt_x;
        fs.val["cf_w"] = max_w;
        fs.val["cf_h"] = max_h;
    }
    // Tamura: normalised plane, running sums, best scale, phi; partials
    if (!fj[A_TAMURA].empty()) {
        std::vector<TamJob> tj;
        long long maxpix = 0;
        for (auto &j : fj[A_TAMURA]) {
            const size_t n = (size_t)P[j.plane].w * P[j.plane].h;
            maxpix = std::max(maxpix, (long long)n);
            TamJob t;
            t.norm_ws = (long long)(fs.ws_take(n * 8) / 8);
            t.sum_ws = (long long)(fs.ws_take(n * 8) / 8);
            t.sbest_ws = (long long)(fs.ws_take(n) / 8);
            t.phi_ws = (long long)(fs.ws_take(n * 8) / 8);
            tj.push_back(t);
        }
        fs.off["tam_jobs"] = fs.put_copy(tj.data(), tj.size() * sizeof(TamJob));
        fs.off["tam_part"] = fs.ws_take(tj.size() * (size_t)((maxpix + 1023) / 1024) * 6 * 8);
        fs.val["tam_maxpix"] = maxpix;
    }

    // Haralick: gray image, LUT, 4 matrices, 4 Q matrices, 4 x 14 results per job
    if (!fj[A_HARALICK].empty()) {
        std::vector<HarJob> hj;
        for (auto &j : fj[A_HARALICK]) {
            const size_t n = (size_t)P[j.plane].w * P[j.plane].h;
            HarJob h;
            h.gray_b = (long long)fs.ws_take(n);
            h.lut_b = (long long)fs.ws_take(257 * 4);
            h.glcm_b = (long long)fs.ws_take(4 * 256 * 256 * 8);
            h.q_b = (long long)fs.ws_take(4 * 256 * 256 * 8);
            h.res_b = (long long)fs.ws_take(4 * 14 * 8);
            hj.push_back(h);
        }
        fs.off["har_jobs"] = fs.put_copy(hj.data(), hj.size() * sizeof(HarJob));
    }
    return WC_OK;
}

int features_launch(FeatureSetup &fs, FeatureRun &fr) {
    const auto &P = *fs.planes;
    const auto &fj = *fs.fj;
    Ctx &c = *fr.ctx;
    auto jobs = [&](int a) { return (const FJob *)(fr.meta + fs.off["jobs" + std::to_string(a)]); };
    auto nj = [&](int a) { return (int)fj[a].size(); };

    if (fs.val.count("sort_n")) {
        launch_plane_sort(c, fr.arena, fr.planes, (const int *)(fr.meta + fs.off["sort_ids"]), (int)fs.val["sort_n"],
                          (unsigned long long *)(fr.ws + fs.off["sort_keys"]),
                          (unsigned long long *)(fr.ws + fs.off["sort_tmp"]),
                          (const long long *)(fr.meta + fs.off["sort_koff"]),
                          (unsigned int *)(fr.ws + fs.off["sort_cnt"]));
        const unsigned long long *keys = (const unsigned long long *)(fr.ws + fs.off["sort_keys"]);
        const long long *koff = (const long long *)(fr.meta + fs.off["sort_koff"]);
        if (nj(A_PIXSTATS))
            launch_pixstats(c, fr.planes, fr.stats, jobs(A_PIXSTATS), nj(A_PIXSTATS),
                            (const int *)(fr.meta + fs.off["slots" + std::to_string(A_PIXSTATS)]), keys, koff, fr.feat);
        if (nj(A_GINI))
            launch_gini(c, fr.planes, jobs(A_GINI), nj(A_GINI),
                        (const int *)(fr.meta + fs.off["slots" + std::to_string(A_GINI)]), keys, koff, fr.feat);
    }
    if (nj(A_MSHIST)) launch_mshist(c, fr.arena, fr.planes, fr.stats, jobs(A_MSHIST), nj(A_MSHIST), fr.feat);
    if (nj(A_FRACTAL)) launch_fractal(c, fr.arena, fr.planes, jobs(A_FRACTAL), nj(A_FRACTAL), fr.feat);
    if (nj(A_COMB)) launch_comb(c, fr.arena, fr.planes, jobs(A_COMB), nj(A_COMB), fr.feat);
    if (nj(A_RADON))
        launch_radon(c, fr.arena, fr.planes, jobs(A_RADON), nj(A_RADON), maxw_of(P, fj[A_RADON]), maxh_of(P, fj[A_RADON]),
                     fr.feat);
    if (nj(A_CHEB))
        launch_chebcoef(c, fr.arena, fr.planes, jobs(A_CHEB), nj(A_CHEB), fr.tabs,
                        (const long long *)(fr.meta + fs.off["cc_tab"]), (double *)(fr.ws + fs.off["cc_mid"]),
                        (const long long *)(fr.meta + fs.off["cc_moff"]), fr.feat);
    if (nj(A_ZERNIKE))
        launch_zernike(c, fr.arena, fr.planes, jobs(A_ZERNIKE), nj(A_ZERNIKE), fs.val["zk_maxpix"],
                       (double *)(fr.ws + fs.off["zk_mom"]), (double *)(fr.ws + fs.off["zk_part"]), fr.feat);
    if (nj(A_CHEBFOURIER))
        launch_chebfourier(c, fr.arena, fr.planes, jobs(A_CHEBFOURIER), nj(A_CHEBFOURIER),
                           maxw_of(P, fj[A_CHEBFOURIER]), maxh_of(P, fj[A_CHEBFOURIER]), (int)fs.val["cf_cntx"],
                           (int)fs.val["cf_w"], (int)fs.val["cf_h"], (const CFJob *)(fr.meta + fs.off["cf_jobs"]), fr.tabs,
                           (double *)fr.ws, (double *)(fr.ws + fs.off["cf_part"]), (int)fs.val["cf_nchunk"], fr.feat);
    if (nj(A_TAMURA))
        launch_tamura(c, fr.planes, fr.stats, fr.arena, jobs(A_TAMURA), nj(A_TAMURA),
                      (const TamJob *)(fr.meta + fs.off["tam_jobs"]), (double *)fr.ws,
                      (double *)(fr.ws + fs.off["tam_part"]), fs.val["tam_maxpix"], fr.feat);
    if (nj(A_HARALICK))
        launch_haralick(c, fr.arena, fr.planes, fr.stats, jobs(A_HARALICK), nj(A_HARALICK),
                        (const HarJob *)(fr.meta + fs.off["har_jobs"]), fr.ws, fr.feat);
    return WC_OK;
}

}  // namespace wc
