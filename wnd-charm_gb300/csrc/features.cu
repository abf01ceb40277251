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

// Gabor kernel (function Gabor, src/textures/gabor.cpp:103-162): n = 38,
// sig2lam = 0.56, gamma = 0.5, theta = 3.14159265/2, fi = 0, normalised by the
// sum of magnitudes; interleaved (re, im), row-major 38 x 38.
static std::vector<double> gabor_kernel(double f0) {
    const int n = 38;
    const double sig2lam = 0.56, gamma = 0.5, theta = 3.14159265 / 2, fi = 0;
    const double lambda = 2 * M_PI / f0, ct = cos(theta), st = sin(theta), sig = sig2lam * lambda;
    std::vector<double> tx(n + 1), ty(n + 1), G((size_t)n * n * 2);
    tx[0] = -(n / 2);
    for (int x = 1; x <= n; x++) tx[x] = tx[x - 1] + 1;
    ty[0] = -(n / 2);
    for (int y = 1; y <= n; y++) ty[y] = ty[y - 1] + 1;
    double sum = 0;
    for (int y = 0; y < n; y++)
        for (int x = 0; x < n; x++) {
            const double xte = tx[x] * ct + ty[y] * st, yte = ty[y] * ct - tx[x] * st;
            const double rte = xte * xte + gamma * gamma * yte * yte;
            const double ge = exp(-1 * rte / (2 * sig * sig));
            const double argm = xte * f0 + fi;
            G[(size_t)y * n * 2 + x * 2] = ge * cos(argm);
            G[(size_t)y * n * 2 + x * 2 + 1] = ge * sin(argm);
            sum += sqrt(pow(G[(size_t)y * n * 2 + x * 2], 2) + pow(G[(size_t)y * n * 2 + x * 2 + 1], 2));
        }
    for (auto &g : G) g = g / sum;
    return G;
}

static int smooth_size(int n) {  // smallest m >= n with prime factors in {2, 3, 5, 7}
    for (int m = n;; m++) {
        int r = m;
        for (int p : {2, 3, 5, 7})
            while (r % p == 0) r /= p;
        if (r == 1) return m;
    }
}

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
    // the Chebyshev-Fourier tensor-core kernel's word (a bounded wait ran out)
    int vc = 0;
    if (cf_tc_err_take(st, &vc))
        return set_err(WC_ERR_CUDA, "reading the tensor-core error word failed: %s",
                       cudaGetErrorString(cudaGetLastError()));
    if (vc && !v) v = vc;
    // the object kernels' word: a batch whose word cannot be read is failed,
    // never reported as good (a union-find cap hit would otherwise be lost)
    int vo = 0;
    if (objects_err_take(st, &vo))
        return set_err(WC_ERR_CUDA, "reading the object kernels' error word failed: %s",
                       cudaGetErrorString(cudaGetLastError()));
    *dev_err = v ? v : vo;
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
        std::vector<SortSeg> seg;
        long long maxn = 0;
        for (size_t k = 0; k < sort_planes.size(); k++) {
            const long long n = (long long)P[sort_planes[k]].w * P[sort_planes[k]].h;
            seg.push_back({koff[k], n});
            maxn = std::max(maxn, n);
        }
        fs.off["sort_ids"] = fs.put_copy(sort_planes.data(), sort_planes.size() * sizeof(int));
        fs.off["sort_koff"] = fs.put_copy(koff.data(), koff.size() * sizeof(long long));
        fs.off["sort_seg"] = fs.put_copy(seg.data(), seg.size() * sizeof(SortSeg));
        fs.off["sort_keys"] = fs.ws_take(tot * 8);
        fs.off["sort_tmp"] = fs.ws_take(tot * 8);
        fs.off["sort_cnt"] = fs.ws_take(sort_scratch_bytes((int)sort_planes.size(), maxn));
        fs.val["sort_n"] = (long long)sort_planes.size();
        fs.val["sort_maxn"] = maxn;
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
            toff.push_back(fs.tabs_add("ch" + std::to_string(Q.w) + "_" + std::to_string(N), [&] { return cheb_table(Q.w, N); }));
            toff.push_back(fs.tabs_add("ch" + std::to_string(Q.h) + "_" + std::to_string(N), [&] { return cheb_table(Q.h, N); }));
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
                c.xs_tab = fs.tabs_add(key, [&] { return xs; });
                snprintf(key, sizeof key, "ds%d_%.17g", Q.h, 1 / yr);
                c.ys_tab = fs.tabs_add(key, [&] { return ys; });
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
        // the mixed form's tensor-core sums: every plane of one size, 23 x 23 coefficients
        bool one_size = fs.prec == WC_PREC_MIXED && fs.cf_tc;
        for (auto &c : cj) one_size = one_size && c.new_w == cj[0].new_w && c.new_h == cj[0].new_h;
        if (one_size && std::min(cj[0].new_w, cj[0].new_h) >= 23) {
            const CFTcPlan tp = cf_tc_plan((int)cj.size(), cj[0].new_h, cj[0].new_w);
            fs.cf_tc_plan = tp;
            fs.val["cf_tc"] = 1;
            fs.off["cf_tc_a"] = fs.ws_take(tp.digA_bytes);
            fs.off["cf_tc_b"] = fs.ws_take(tp.digB_bytes);
            fs.off["cf_tc_p"] = fs.ws_take(tp.partial_bytes);
            fs.off["cf_tc_u"] = fs.ws_take(tp.uA_bytes);
        }
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
            t.mk_ws = (long long)(fs.ws_take(n * 8) / 8);
            t.emax_ws = (long long)(fs.ws_take(n * 8) / 8);
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
            h.mar_b = (long long)fs.ws_take(4 * HAR_MAR_BYTES);
            hj.push_back(h);
        }
        fs.off["har_jobs"] = fs.put_copy(hj.data(), hj.size() * sizeof(HarJob));
        // + the count of large matrices and the work queue's two tickets
        fs.off["har_perm"] = fs.ws_take((4 * hj.size() + 3) * sizeof(int));
    }
    // Edge features: magnitude / direction planes in the workspace, sorted copies
    if (!fj[A_EDGEF].empty()) {
        std::vector<EFJob> ej;
        std::vector<Plane> aux;
        std::vector<int> ids;
        std::vector<long long> koff;
        size_t ktot = 0;
        for (auto &j : fj[A_EDGEF]) {
            const Plane &Q = P[j.plane];
            const size_t n = (size_t)Q.w * Q.h;
            EFJob e;
            e.mag_ws = (long long)(fs.ws_take(n * 8) / 8);
            e.dir_ws = (long long)(fs.ws_take(n * 8) / 8);
            ej.push_back(e);
            for (long long o : {e.mag_ws, e.dir_ws}) {
                ids.push_back((int)aux.size());
                aux.push_back({o, Q.w, Q.h});
                koff.push_back((long long)ktot);
                ktot += (n + 31) & ~(size_t)31;
            }
        }
        fs.off["ef_jobs"] = fs.put_copy(ej.data(), ej.size() * sizeof(EFJob));
        fs.off["ef_aux"] = fs.put_copy(aux.data(), aux.size() * sizeof(Plane));
        fs.off["ef_ids"] = fs.put_copy(ids.data(), ids.size() * sizeof(int));
        std::vector<SortSeg> seg;
        long long maxn = 0;
        for (size_t k = 0; k < aux.size(); k++) {
            seg.push_back({koff[k], (long long)aux[k].w * aux[k].h});
            maxn = std::max(maxn, (long long)aux[k].w * aux[k].h);
        }
        fs.off["ef_koff"] = fs.put_copy(koff.data(), koff.size() * sizeof(long long));
        fs.off["ef_seg"] = fs.put_copy(seg.data(), seg.size() * sizeof(SortSeg));
        fs.off["ef_stats"] = fs.meta_take(aux.size() * sizeof(PlaneStats));
        fs.off["ef_keys"] = fs.ws_take(ktot * 8);
        fs.off["ef_tmp"] = fs.ws_take(ktot * 8);
        fs.off["ef_cnt"] = fs.ws_take(sort_scratch_bytes((int)aux.size(), maxn));
        fs.val["ef_maxn"] = maxn;
    }

    // Otsu / Inverse-Otsu object features (one job list for both)
    if (!fj[A_OBJ].empty() || !fj[A_INVOBJ].empty()) {
        std::vector<FJob> all;
        std::vector<OBJob> oj;
        std::vector<Plane> inv;
        long long maxpix = 0;
        for (int a : {A_OBJ, A_INVOBJ})
            for (auto &j : fj[a]) all.push_back(j);
        size_t zero_begin = fs.ws_take(0);
        // zeroed block first: area (u32), xm, ym (u64) per job, accumulators
        std::vector<size_t> zoff;
        for (auto &j : all) {
            const size_t n = (size_t)P[j.plane].w * P[j.plane].h;
            zoff.push_back(fs.ws_take(n * 4));
            zoff.push_back(fs.ws_take(n * 8));
            zoff.push_back(fs.ws_take(n * 8));
        }
        const size_t acc_off = fs.ws_take(all.size() * 8 * 8);
        const size_t zero_end = fs.ws_take(0);
        fs.val["ob_zero_begin"] = (long long)zero_begin;
        fs.val["ob_zero_bytes"] = (long long)(zero_end - zero_begin);
        fs.off["ob_acc"] = acc_off;
        for (size_t k = 0; k < all.size(); k++) {
            const Plane &Q = P[all[k].plane];
            const size_t n = (size_t)Q.w * Q.h;
            maxpix = std::max(maxpix, (long long)n);
            OBJob o;
            memset(&o, 0, sizeof o);
            o.inverse = k >= fj[A_OBJ].size();
            o.src_ws = (long long)(fs.ws_take(o.inverse ? n * 8 : 8) / 8);
            o.lab_ws = (long long)(fs.ws_take(n * 4) / 8);
            o.area_ws = (long long)(zoff[3 * k] / 8);
            o.xm_ws = (long long)(zoff[3 * k + 1] / 8);
            o.ym_ws = (long long)(zoff[3 * k + 2] / 8);
            o.roots_ws = (long long)(fs.ws_take(n * 4) / 8);
            o.keys_ws = (long long)(fs.ws_take(2 * n * 8) / 8);
            o.tmp_ws = (long long)(fs.ws_take(n * 8) / 8);
            o.dist_ws = (long long)(fs.ws_take(n * 8) / 8);
            oj.push_back(o);
            inv.push_back({o.src_ws, Q.w, Q.h});
        }
        fs.off["ob_fjobs"] = fs.put_copy(all.data(), all.size() * sizeof(FJob));
        fs.off["ob_jobs"] = fs.put_copy(oj.data(), oj.size() * sizeof(OBJob));
        fs.off["ob_inv"] = fs.put_copy(inv.data(), inv.size() * sizeof(Plane));
        fs.off["ob_invstats"] = fs.meta_take(inv.size() * sizeof(PlaneStats));
        fs.off["ob_thr"] = fs.ws_take(all.size() * 8);
        fs.val["ob_n"] = (long long)all.size();
        fs.val["ob_maxpix"] = maxpix;
    }

    // Gabor: padded spectra, 8 energy maps per job, kernel spectra per size
    if (!fj[A_GABOR].empty()) {
        std::vector<GabJob> gj;
        std::vector<GabSize> sizes;
        std::vector<FFTPlan> plans;
        std::map<int, int> pidx;
        auto plan_of = [&](int n) {
            if (!pidx.count(n)) { pidx[n] = (int)plans.size(); plans.push_back(fs.fft_plan(n)); }
            return pidx[n];
        };
        fs.val["gab_kern"] = fs.tabs_add("gabor38", [] {
            std::vector<double> kt;
            for (double f0 : {0.1, 1.0, 2.0, 3.0, 4.0, 5.0, 6.0, 7.0}) {
                std::vector<double> g = gabor_kernel(f0);
                kt.insert(kt.end(), g.begin(), g.end());
            }
            return kt;
        });
        for (auto &j : fj[A_GABOR]) {
            const Plane &Q = P[j.plane];
            GabJob g;
            g.fh = smooth_size(Q.h + 37);
            g.fw = smooth_size(Q.w + 37);
            if (g.fh > kMaxFFT || g.fw > kMaxFFT) return set_err(WC_ERR_UNSUPPORTED, "Gabor: image too large");
            g.plan_h = plan_of(g.fh);
            g.plan_w = plan_of(g.fw);
            int si = -1;
            for (size_t k = 0; k < sizes.size(); k++)
                if (sizes[k].fh == g.fh && sizes[k].fw == g.fw) si = (int)k;
            if (si < 0) {
                GabSize S{g.fh, g.fw, g.plan_h, g.plan_w, (long long)(fs.ws_take((size_t)8 * g.fh * g.fw * 16) / 8), 0, 0, 0};
                sizes.push_back(S);
                si = (int)sizes.size() - 1;
            }
            g.g_ws = sizes[si].g_ws;
            sizes[si].count++;
            gj.push_back(g);
        }
        // per padded size, the jobs' spectra and 8 products in contiguous blocks
        for (auto &S : sizes) {
            const long long arr = (long long)S.fh * S.fw * 2;  // doubles per complex array
            S.a_ws = (long long)(fs.ws_take((size_t)S.count * arr * 8) / 8);
            S.c_ws = (long long)(fs.ws_take((size_t)S.count * 8 * arr * 8) / 8);
            int k = 0;
            for (auto &g : gj)
                if (g.fh == S.fh && g.fw == S.fw) {
                    g.a_ws = S.a_ws + k * arr;
                    g.c_ws = S.c_ws + (long long)k * 8 * arr;
                    k++;
                }
        }
        for (size_t k = 0; k < gj.size(); k++) {
            const Plane &Q = P[fj[A_GABOR][k].plane];
            gj[k].e_ws = (long long)(fs.ws_take((size_t)8 * Q.w * Q.h * 8) / 8);
        }
        fs.off["gab_jobs"] = fs.put_copy(gj.data(), gj.size() * sizeof(GabJob));
        fs.off["gab_plans"] = fs.put_copy(plans.data(), plans.size() * sizeof(FFTPlan));
        fs.off["gab_counts"] = fs.ws_take(gj.size() * 8 * 8);
        fs.gab_jobs = gj;
        fs.gab_sizes = sizes;
    }
    return WC_OK;
}

int features_launch(FeatureSetup &fs, FeatureRun &fr, int phase, bool early) {
    const auto &P = *fs.planes;
    const auto &fj = *fs.fj;
    // lanes: 0 Haralick; 1 Zernike, Chebyshev-Fourier; 2 Tamura;
    // 3 Gabor, then Radon, fractal, multiscale histograms, comb moments;
    // 4 objects, edge features; 5 sorts (PixStats, Gini), colour histogram,
    // Chebyshev coefficients (lanes 0 and 5 at the higher stream priority)
    Ctx &c = fr.lanes[5];
    auto jobs = [&](int a) { return (const FJob *)(fr.meta + fs.off["jobs" + std::to_string(a)]); };
    auto nj = [&](int a) { return (int)fj[a].size(); };
    // the families that read only the root planes (lanes 3, 4)
    if (early ? phase == 0 : phase == 1) {
        {
            Ctx &c = fr.lanes[4];
            ProfScope ps(c, "Edge Features");
            if (nj(A_EDGEF))
            launch_edgefeat(c, fr.arena, fr.planes, jobs(A_EDGEF), nj(A_EDGEF), maxw_of(P, fj[A_EDGEF]),
                            maxh_of(P, fj[A_EDGEF]), (const EFJob *)(fr.meta + fs.off["ef_jobs"]), (double *)fr.ws,
                            (const Plane *)(fr.meta + fs.off["ef_aux"]), (const int *)(fr.meta + fs.off["ef_ids"]),
                            (PlaneStats *)(fr.meta + fs.off["ef_stats"]), (unsigned long long *)(fr.ws + fs.off["ef_keys"]),
                            (unsigned long long *)(fr.ws + fs.off["ef_tmp"]), (const long long *)(fr.meta + fs.off["ef_koff"]),
                            (const SortSeg *)(fr.meta + fs.off["ef_seg"]), fs.val["ef_maxn"], fr.ws + fs.off["ef_cnt"], fr.feat);
        }
        if (fs.val.count("ob_n")) {
            Ctx &c = fr.lanes[4];
            ProfScope ps(c, "Object Features (Otsu + Inverse)");
            if (cudaMemsetAsync(fr.ws + fs.val["ob_zero_begin"], 0, (size_t)fs.val["ob_zero_bytes"], c.st) != cudaSuccess)
                return set_err(WC_ERR_CUDA, "memset failed");
            launch_objects(c, fr.arena, fr.planes, fr.stats, (const FJob *)(fr.meta + fs.off["ob_fjobs"]), (int)fs.val["ob_n"],
                           fs.val["ob_maxpix"], (const OBJob *)(fr.meta + fs.off["ob_jobs"]), (double *)fr.ws,
                           (const Plane *)(fr.meta + fs.off["ob_inv"]), (PlaneStats *)(fr.meta + fs.off["ob_invstats"]),
                           (double *)(fr.ws + fs.off["ob_thr"]), (unsigned long long *)(fr.ws + fs.off["ob_acc"]), fr.feat);
        }
        {
            Ctx &c = fr.lanes[3];
            ProfScope ps(c, "Gabor Textures");
            if (nj(A_GABOR))
            launch_gabor(c, fr.arena, fr.planes, jobs(A_GABOR), nj(A_GABOR), (const GabJob *)(fr.meta + fs.off["gab_jobs"]),
                         fs.gab_jobs, fs.gab_sizes, (const FFTPlan *)(fr.meta + fs.off["gab_plans"]), fr.tabs,
                         fs.val["gab_kern"], (double *)fr.ws, (double *)(fr.ws + fs.off["gab_counts"]), fr.feat);
        }
    }
    if (phase == 0) return WC_OK;
    // the longest dependent chain (Haralick f14) is issued first
    {
        Ctx &c = fr.lanes[0];
        ProfScope ps(c, "Haralick Textures");
        if (nj(A_HARALICK))
        launch_haralick(c, fr.arena, fr.planes, fr.stats, jobs(A_HARALICK), nj(A_HARALICK),
                        (const HarJob *)(fr.meta + fs.off["har_jobs"]), fr.ws, (int *)(fr.ws + fs.off["har_perm"]),
                        fr.feat);
    }

    // the plane scans on lane 3, after Gabor: beside the sorts rather than
    // behind them (the sorts' integer work waits longest for SM room while the
    // FP64 lanes run, and the scans would otherwise end the batch alone)
    {
        Ctx &c = fr.lanes[3];
        ProfScope ps(c, "Radon Coefficients");
        if (nj(A_RADON))
        launch_radon(c, fr.arena, fr.planes, jobs(A_RADON), nj(A_RADON), maxw_of(P, fj[A_RADON]), maxh_of(P, fj[A_RADON]),
                     fr.feat);
    }
    {
        Ctx &c = fr.lanes[3];
        ProfScope ps(c, "Fractal Features");
        if (nj(A_FRACTAL)) launch_fractal(c, fr.arena, fr.planes, jobs(A_FRACTAL), nj(A_FRACTAL), fr.feat);
    }
    {
        Ctx &c = fr.lanes[3];
        ProfScope ps(c, "Multiscale Histograms");
        if (nj(A_MSHIST)) launch_mshist(c, fr.arena, fr.planes, fr.stats, jobs(A_MSHIST), nj(A_MSHIST), fr.feat);
    }
    {
        Ctx &c = fr.lanes[3];
        ProfScope ps(c, "Comb Moments");
        if (nj(A_COMB)) launch_comb(c, fr.arena, fr.planes, jobs(A_COMB), nj(A_COMB), fr.feat);
    }
    if (fs.val.count("sort_n")) {
        ProfScope ps(c, "PixStats+Gini (sort)");
        launch_sort_planes(c, fr.arena, fr.planes, (const int *)(fr.meta + fs.off["sort_ids"]),
                           (const SortSeg *)(fr.meta + fs.off["sort_seg"]), (int)fs.val["sort_n"], fs.val["sort_maxn"],
                           (unsigned long long *)(fr.ws + fs.off["sort_keys"]),
                           (unsigned long long *)(fr.ws + fs.off["sort_tmp"]), fr.ws + fs.off["sort_cnt"]);
        const unsigned long long *keys = (const unsigned long long *)(fr.ws + fs.off["sort_keys"]);
        const long long *koff = (const long long *)(fr.meta + fs.off["sort_koff"]);
        if (nj(A_PIXSTATS))
            launch_pixstats(c, fr.planes, fr.stats, jobs(A_PIXSTATS), nj(A_PIXSTATS),
                            (const int *)(fr.meta + fs.off["slots" + std::to_string(A_PIXSTATS)]), keys, koff, fr.feat);
        if (nj(A_GINI))
            launch_gini(c, fr.planes, jobs(A_GINI), nj(A_GINI),
                        (const int *)(fr.meta + fs.off["slots" + std::to_string(A_GINI)]), keys, koff, fr.feat);
    }
    {
        ProfScope ps(c, "Color Histogram");
        if (nj(A_COLORHIST)) launch_color_hist(c, fr.planes, jobs(A_COLORHIST), nj(A_COLORHIST), fr.clr, fr.clr_off,
                                               fr.fuzzy, fr.feat);
    }
    {
        Ctx &c = fr.lanes[5];
        ProfScope ps(c, "Chebyshev Coefficients");
        if (nj(A_CHEB))
        launch_chebcoef(c, fr.arena, fr.planes, jobs(A_CHEB), nj(A_CHEB), fr.tabs,
                        (const long long *)(fr.meta + fs.off["cc_tab"]), (double *)(fr.ws + fs.off["cc_mid"]),
                        (const long long *)(fr.meta + fs.off["cc_moff"]), fr.feat);
    }
    {
        Ctx &c = fr.lanes[1];
        ProfScope ps(c, "Zernike Coefficients");
        if (nj(A_ZERNIKE))
        launch_zernike(c, fr.arena, fr.planes, jobs(A_ZERNIKE), nj(A_ZERNIKE), fs.val["zk_maxpix"],
                       (double *)(fr.ws + fs.off["zk_mom"]), (double *)(fr.ws + fs.off["zk_part"]), fr.feat);
    }
    {
        Ctx &c = fr.lanes[1];
        ProfScope ps(c, "Chebyshev-Fourier Coefficients");
        CFTcBufs tb{};
        const bool tc = fs.val.count("cf_tc") && fs.val["cf_tc"];
        if (tc)
            tb = CFTcBufs{fr.ws + fs.off["cf_tc_a"], fr.ws + fs.off["cf_tc_b"], (double *)(fr.ws + fs.off["cf_tc_p"]),
                          (double *)(fr.ws + fs.off["cf_tc_u"])};
        if (nj(A_CHEBFOURIER))
        launch_chebfourier(c, fr.arena, fr.planes, jobs(A_CHEBFOURIER), nj(A_CHEBFOURIER),
                           maxw_of(P, fj[A_CHEBFOURIER]), maxh_of(P, fj[A_CHEBFOURIER]), (int)fs.val["cf_cntx"],
                           (int)fs.val["cf_w"], (int)fs.val["cf_h"], (const CFJob *)(fr.meta + fs.off["cf_jobs"]), fr.tabs,
                           (double *)fr.ws, (double *)(fr.ws + fs.off["cf_part"]), (int)fs.val["cf_nchunk"], fr.feat,
                           tc ? &fs.cf_tc_plan : nullptr, tc ? &tb : nullptr);
    }
    {
        Ctx &c = fr.lanes[2];
        ProfScope ps(c, "Tamura Textures");
        if (nj(A_TAMURA))
        launch_tamura(c, fr.planes, fr.stats, fr.arena, jobs(A_TAMURA), nj(A_TAMURA),
                      (const TamJob *)(fr.meta + fs.off["tam_jobs"]), (double *)fr.ws,
                      (double *)(fr.ws + fs.off["tam_part"]), fs.val["tam_maxpix"], fr.feat);
    }
    return WC_OK;
}

}  // namespace wc
