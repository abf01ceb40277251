// Raw-image families (FP64 form): Edge features, Otsu / Inverse-Otsu object
// features.
//
// Edge features: EdgeStatistics with PrewittMagnitude2D / PrewittDirection2D,
// src/FeatureAlgorithms.cpp:299-341, src/cmatrix.cpp:1317-1458.
// Object features: FeatureStatistics with OtsuBinaryMaskTransform, bwlabel(8),
// GlobalCentroid, FeatureCentroid, EulerNumber, src/FeatureAlgorithms.cpp:346-417,
// src/cmatrix.cpp:1520-1717, src/statistics/FeatureStatistics.cpp:44-254.
//   * labelling: union-find whose links always go from the larger to the
//     smaller root, so every object's root is its first pixel in raster order,
//     which is the order of the reference's flood fill labels;
//   * per-object sums run in that label order, statistics over the sorted
//     areas / distances in ascending order, as on the CPU;
//   * an image with no object gives all-zero statistics (the reference reads
//     element 0 of an empty array there).
#include <cfloat>
#include <cmath>

#include "kcommon.cuh"
#include "kernels.h"
#include "ksort.cuh"

namespace wc {

// The error word of this file's kernels (a device symbol is private to its
// translation unit without relocatable device code, so it is not the one in
// features.cu): the union-find loops set it when their iteration cap runs
// out; objects_err_take reads and clears it for features_check.
__device__ int g_dev_err_ob = 0;

int objects_err_take(cudaStream_t st, int *v) {
    *v = 0;
    if (cudaMemcpyFromSymbolAsync(v, g_dev_err_ob, sizeof(int), 0, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return -1;
    if (*v) {
        const int z = 0;
        cudaMemcpyToSymbolAsync(g_dev_err_ob, &z, sizeof(int), 0, cudaMemcpyHostToDevice, st);
        cudaStreamSynchronize(st);
    }
    return 0;
}

// ---------------------------------------------------------------- Edge features
__global__ void k_ef_prewitt(const double *__restrict__ arena, const Plane *__restrict__ planes, const FJob *__restrict__ jobs,
                             const EFJob *__restrict__ ej, double *__restrict__ ws) {
    const FJob J = jobs[blockIdx.z];
    const Plane P = planes[J.plane];
    const EFJob E = ej[blockIdx.z];
    const long long w = P.w, h = P.h;
    const long long x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const double *p = arena + P.off;
    double sx = 0, sy = 0;
    for (long long j = y - 1; j <= y + 1; j++)
        if (j >= 0 && j < h && x - 1 >= 0) sx = __dadd_rn(sx, p[j * w + x - 1]);
    for (long long j = y - 1; j <= y + 1; j++)
        if (j >= 0 && j < h && x + 1 < w) sx = __dsub_rn(sx, p[j * w + x + 1]);
    for (long long i = x - 1; i <= x + 1; i++)
        if (i >= 0 && i < w && y - 1 >= 0) sy = __dadd_rn(sy, p[(y - 1) * w + i]);
    for (long long i = x - 1; i <= x + 1; i++)
        if (i >= 0 && i < w && y + 1 < h) sy = __dsub_rn(sy, p[(y + 1) * w + i]);
    ws[E.mag_ws + y * w + x] = sqrt(__dadd_rn(__dmul_rn(sx, sx), __dmul_rn(sy, sy)));
    double d;
    if (sy == 0 || fabs(sy) < 1 / 10E200) d = 3.1415926 * (sx < 0 ? 1 : 0);
    else d = atan2(sy, sx);
    ws[E.dir_ws + y * w + x] = d;
}

__global__ void __launch_bounds__(512) k_ef_final(const Plane *__restrict__ planes, const FJob *__restrict__ jobs,
                                                  const EFJob *__restrict__ ej, const double *__restrict__ ws,
                                                  const PlaneStats *__restrict__ ast, const unsigned long long *__restrict__ keys,
                                                  const long long *__restrict__ koff, double *__restrict__ feat) {
    __shared__ unsigned int mh[8], dh[8];
    __shared__ long long shl[32];
    const FJob J = jobs[blockIdx.x];
    const Plane P = planes[J.plane];
    const EFJob E = ej[blockIdx.x];
    const PlaneStats M = ast[2 * blockIdx.x], Dd = ast[2 * blockIdx.x + 1];
    const long long n = (long long)P.w * P.h;
    if (threadIdx.x < 8) { mh[threadIdx.x] = 0; dh[threadIdx.x] = 0; }
    __syncthreads();
    const double msc = hist_scale(M.mn, M.mx, 8), dsc = hist_scale(Dd.mn, Dd.mx, 8);
    long long area = 0;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        const double m = ws[E.mag_ws + i], d = ws[E.dir_ws + i];
        atomicAdd(&mh[hist_bin(m, M.mn, msc, 8)], 1u);
        atomicAdd(&dh[hist_bin(d, Dd.mn, dsc, 8)], 1u);
        if (m > M.mean) area++;
    }
    area = block_sum_ll(area, shl);
    if (threadIdx.x == 0) {
        auto median = [&](const unsigned long long *k) {
            const long long half = n / 2;
            if (n % 2 == 0) return (dkey_inv(k[half]) + dkey_inv(k[half - 1])) / 2.0;
            return dkey_inv(k[half]);
        };
        const double mmed = median(keys + koff[2 * blockIdx.x]), dmed = median(keys + koff[2 * blockIdx.x + 1]);
        double H[8], MH[8], diff[4], sum = 0, homog = 0;
        for (int b = 0; b < 8; b++) { H[b] = dh[b]; MH[b] = mh[b]; }
        for (int b = 0; b < 4; b++) diff[b] = fabs(H[b] - H[b + 4]);
        for (int b = 0; b < 4; b++) {
            if (H[b] + H[b + 4] != 0) diff[b] = diff[b] / (H[b] + H[b + 4]);
            sum += (H[b] + H[b + 4]);
        }
        if (sum > 0) homog = (H[0] + H[1]) / sum;
        double *o = feat + J.out;
        int k = 0;
        o[k++] = (double)area;
        for (int b = 0; b < 4; b++) o[k++] = diff[b];
        for (int b = 0; b < 8; b++) o[k++] = H[b];
        o[k++] = homog;
        o[k++] = Dd.mean;
        o[k++] = dmed;
        o[k++] = Dd.var;
        for (int b = 0; b < 8; b++) o[k++] = MH[b];
        o[k++] = M.mean;
        o[k++] = mmed;
        o[k++] = M.var;
    }
}

void launch_edgefeat(Ctx &c, const double *arena, const Plane *planes, const FJob *jobs, int njobs, int maxw, int maxh,
                     const EFJob *ej, double *ws, const Plane *aux_planes, const int *aux_ids, PlaneStats *aux_stats,
                     unsigned long long *keys, unsigned long long *tmp, const long long *koff, const SortSeg *seg,
                     long long maxn, void *scratch, double *feat) {
    if (njobs <= 0) return;
    WC_LAUNCH(c);
    k_ef_prewitt<<<dim3((maxw + 31) / 32, (maxh + 7) / 8, njobs), dim3(32, 8), 0, c.st>>>(arena, planes, jobs, ej, ws);
    launch_plane_stats(c, ws, aux_planes, 2 * njobs, aux_stats, 1, 0);
    launch_sort_planes(c, ws, aux_planes, aux_ids, seg, 2 * njobs, maxn, keys, tmp, scratch);
    WC_LAUNCH(c);
    k_ef_final<<<njobs, 512, 0, c.st>>>(planes, jobs, ej, ws, aux_stats, keys, koff, feat);
}

// ---------------------------------------------------------------- object features
// inverted image for Inverse-Otsu: (max - p) + min (ImageMatrix::invert)
__global__ void k_ob_invert(const double *__restrict__ arena, const Plane *__restrict__ planes,
                            const PlaneStats *__restrict__ stats, const FJob *__restrict__ jobs, const OBJob *__restrict__ oj,
                            double *__restrict__ ws) {
    const FJob J = jobs[blockIdx.y];
    const OBJob O = oj[blockIdx.y];
    if (!O.inverse) return;
    const Plane P = planes[J.plane];
    const PlaneStats S = stats[J.plane];
    const long long n = (long long)P.w * P.h;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        ws[O.src_ws + i] = __dadd_rn(__dsub_rn(S.mx, arena[P.off + i]), S.mn);
}

// Otsu threshold (ImageMatrix::Otsu, src/cmatrix.cpp:1520-1570) of the source
__global__ void __launch_bounds__(1024) k_ob_otsu(const double *__restrict__ arena, const Plane *__restrict__ planes,
                                                  const PlaneStats *__restrict__ stats, const PlaneStats *__restrict__ inv_stats,
                                                  const FJob *__restrict__ jobs, const OBJob *__restrict__ oj,
                                                  const double *__restrict__ ws, double *__restrict__ thr) {
    __shared__ unsigned int hist[1024];
    const FJob J = jobs[blockIdx.x];
    const OBJob O = oj[blockIdx.x];
    const Plane P = planes[J.plane];
    const PlaneStats S = O.inverse ? inv_stats[blockIdx.x] : stats[J.plane];
    const double *src = O.inverse ? ws + O.src_ws : arena + P.off;
    const long long n = (long long)P.w * P.h;
    for (int i = threadIdx.x; i < 1024; i += blockDim.x) hist[i] = 0;
    __syncthreads();
    const double sc = hist_scale(S.mn, S.mx, 1024);
    for (long long i = threadIdx.x; i < n; i += blockDim.x) atomicAdd(&hist[hist_bin(src[i], S.mn, sc, 1024)], 1u);
    __syncthreads();
    if (threadIdx.x == 0) {
        const double wh = (double)(unsigned)(P.w * P.h);
        double om = hist[0] / wh;
        // myu[L-1] first (sequential, as the reference accumulates the arrays)
        double om_i = om, my_i = 0.0, myL = 0.0;
        for (int i = 1; i < 1024; i++) myL = myL + i * (hist[i] / wh);
        int th = 0;
        double max_sigma = 0.0;
        for (int i = 0; i < 1023; i++) {
            if (i > 0) {
                om_i = om_i + (hist[i] / wh);
                my_i = my_i + i * (hist[i] / wh);
            }
            double s;
            if (om_i != 0.0 && om_i != 1.0) s = pow(myL * om_i - my_i, 2) / (om_i * (1.0 - om_i));
            else s = 0.0;
            if (s > max_sigma) { max_sigma = s; th = i; }
        }
        (void)om;
        thr[blockIdx.x] = (((double)th / (double)(1023)) * (S.mx - S.mn)) + S.mn;
    }
}

__device__ __forceinline__ int uf_find(volatile int *L, int x, long long cap) {
    for (long long it = 0; it < cap; it++) {
        const int p = L[x];
        if (p == x) return x;
        x = p;
    }
    atomicExch(&g_dev_err_ob, 22);
    return x;
}

__device__ void uf_unite(int *L, int a, int b, long long cap) {
    for (long long it = 0; it < cap; it++) {
        a = uf_find(L, a, cap);
        b = uf_find(L, b, cap);
        if (a == b) return;
        if (a < b) { const int t = a; a = b; b = t; }
        const int old = atomicMin(&L[a], b);
        if (old == a) return;
        a = old;
    }
    atomicExch(&g_dev_err_ob, 23);
}

// stage 0: init labels; 1: unions with the 4 earlier 8-neighbours; 2: flatten
__global__ void k_ob_label(const double *__restrict__ arena, const Plane *__restrict__ planes, const FJob *__restrict__ jobs,
                           const OBJob *__restrict__ oj, const double *__restrict__ thr, double *__restrict__ ws, int stage,
                           long long uf_cap) {
    const FJob J = jobs[blockIdx.y];
    const OBJob O = oj[blockIdx.y];
    const Plane P = planes[J.plane];
    const int W = P.w, H = P.h;
    const long long n = (long long)W * H;
    int *L = (int *)(ws + O.lab_ws);
    const double *src = O.inverse ? ws + O.src_ws : arena + P.off;
    const double t = thr[blockIdx.y];
    const long long cap = uf_cap > 0 ? uf_cap : n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        if (stage == 0) {
            L[i] = (src[i] > t) ? (int)i : -1;
        } else if (stage == 1) {
            if (L[i] < 0) continue;
            const int y = (int)(i / W), x = (int)(i - (long long)y * W);
            if (x > 0 && L[i - 1] >= 0) uf_unite(L, (int)i, (int)(i - 1), cap);
            if (y > 0) {
                if (x > 0 && L[i - W - 1] >= 0) uf_unite(L, (int)i, (int)(i - W - 1), cap);
                if (L[i - W] >= 0) uf_unite(L, (int)i, (int)(i - W), cap);
                if (x < W - 1 && L[i - W + 1] >= 0) uf_unite(L, (int)i, (int)(i - W + 1), cap);
            }
        } else {
            if (L[i] >= 0) L[i] = uf_find(L, (int)i, cap);
        }
    }
}

// per pixel: object area / coordinate sums at the root, global centroid sums,
// Euler-number pattern counts (all integers, so atomics are exact)
__global__ void k_ob_accum(const Plane *__restrict__ planes, const FJob *__restrict__ jobs, const OBJob *__restrict__ oj,
                           double *__restrict__ ws, unsigned long long *__restrict__ acc) {
    const FJob J = jobs[blockIdx.y];
    const OBJob O = oj[blockIdx.y];
    const Plane P = planes[J.plane];
    const int W = P.w, H = P.h;
    const long long n = (long long)W * H;
    const int *L = (const int *)(ws + O.lab_ws);
    unsigned int *area = (unsigned int *)(ws + O.area_ws);
    unsigned long long *xm = (unsigned long long *)(ws + O.xm_ws), *ym = (unsigned long long *)(ws + O.ym_ws);
    unsigned long long mass = 0, gx = 0, gy = 0, c1 = 0, c3 = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int y = (int)(i / W), x = (int)(i - (long long)y * W);
        const int r = L[i];
        if (r >= 0) {
            atomicAdd(&area[r], 1u);
            atomicAdd(&xm[r], (unsigned long long)(x + 1));
            atomicAdd(&ym[r], (unsigned long long)(y + 1));
            mass++;
            gx += x + 1;
            gy += y + 1;
        }
        if (x >= 1 && y >= 1) {
            const int q = (L[i - W - 1] >= 0) * 8 + (L[i - W] >= 0) * 4 + (L[i - 1] >= 0) * 2 + (r >= 0);
            if (q == 8 || q == 4 || q == 2 || q == 1) c1++;
            else if (q == 7 || q == 11 || q == 13 || q == 14) c3++;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        mass += __shfl_down_sync(0xffffffffu, mass, o);
        gx += __shfl_down_sync(0xffffffffu, gx, o);
        gy += __shfl_down_sync(0xffffffffu, gy, o);
        c1 += __shfl_down_sync(0xffffffffu, c1, o);
        c3 += __shfl_down_sync(0xffffffffu, c3, o);
    }
    if ((threadIdx.x & 31) == 0) {
        unsigned long long *a = acc + blockIdx.y * 8;
        atomicAdd(&a[0], mass);
        atomicAdd(&a[1], gx);
        atomicAdd(&a[2], gy);
        atomicAdd(&a[3], c1);
        atomicAdd(&a[4], c3);
    }
}

// per job: object list in label order, sorted areas and distances, statistics
__global__ void __launch_bounds__(512) k_ob_final(const Plane *__restrict__ planes, const FJob *__restrict__ jobs,
                                                  const OBJob *__restrict__ oj, double *__restrict__ ws,
                                                  const unsigned long long *__restrict__ acc, double *__restrict__ feat) {
    __shared__ int wsum[32];
    __shared__ long long s_count;
    __shared__ double s_gx, s_gy;
    const FJob J = jobs[blockIdx.x];
    const OBJob O = oj[blockIdx.x];
    const Plane P = planes[J.plane];
    const long long n = (long long)P.w * P.h;
    const int *L = (const int *)(ws + O.lab_ws);
    int *roots = (int *)(ws + O.roots_ws);
    const unsigned int *area = (const unsigned int *)(ws + O.area_ws);
    const unsigned long long *xm = (const unsigned long long *)(ws + O.xm_ws), *ym = (const unsigned long long *)(ws + O.ym_ws);
    const unsigned long long *a = acc + blockIdx.x * 8;
    if (threadIdx.x == 0) {
        s_count = 0;
        const double mass = (double)a[0];
        s_gx = mass ? (double)a[1] / mass : 0;
        s_gy = mass ? (double)a[2] / mass : 0;
    }
    __syncthreads();
    // compaction of the roots (L[i] == i) in raster order: every warp counts the
    // roots of its own contiguous segment, a scan over the warps gives each its
    // first slot, then every warp writes its roots in order
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const unsigned lt = (1u << lane) - 1;
    const long long seg = (n + nw - 1) / nw, s0 = min(n, (long long)wid * seg), s1 = min(n, s0 + seg);
    int mine = 0;
    for (long long b = s0; b < s1; b += 32) {
        const long long i = b + lane;
        mine += __popc(__ballot_sync(0xffffffffu, i < s1 && L[i] == (int)i));
    }
    if (lane == 0) wsum[wid] = mine;
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int w = 0; w < nw; w++) {
            const int v = wsum[w];
            wsum[w] = run;
            run += v;
        }
        s_count = run;
    }
    __syncthreads();
    long long slot = wsum[wid];
    for (long long b = s0; b < s1; b += 32) {
        const long long i = b + lane;
        const bool f = i < s1 && L[i] == (int)i;
        const unsigned bal = __ballot_sync(0xffffffffu, f);
        if (f) roots[slot + __popc(bal & lt)] = (int)i;
        slot += __popc(bal);
    }
    __syncthreads();
    const long long count = s_count;
    const double gx = s_gx, gy = s_gy;
    unsigned long long *ka = (unsigned long long *)(ws + O.keys_ws), *kd = ka + count;
    unsigned long long *tmp = (unsigned long long *)(ws + O.tmp_ws);
    double *dist = ws + O.dist_ws;
    for (long long k = threadIdx.x; k < count; k += blockDim.x) {
        const int r = roots[k];
        const double ar = (double)area[r];
        const double cx = (double)xm[r] / ar, cy = (double)ym[r] / ar;
        const double dx = __dsub_rn(cx, gx), dy = __dsub_rn(cy, gy);
        const double d = sqrt(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
        dist[k] = d;
        ka[k] = (unsigned long long)area[r];
        kd[k] = dkey(d);
    }
    __syncthreads();
    cta_sort_u64(ka, tmp, count);
    cta_sort_u64(kd, tmp, count);
    if (threadIdx.x == 0) {
        double ahist[10] = {0}, dhist[10] = {0};
        double amin = 0, amax = 0, amean = 0, amed = 0, avar = 0, dmin = 0, dmax = 0, dmean = 0, dmed = 0, dvar = 0;
        if (count > 0) {
            double sa = 0, sd = 0;
            for (long long k = 0; k < count; k++) {  // label order, as the reference sums
                sa += (double)area[roots[k]];
                sd += dist[k];
            }
            amin = (double)ka[0];
            amax = (double)ka[count - 1];
            amean = sa / count;
            amed = (double)(unsigned int)ka[count / 2];
            const double sc = (amax - amin > 0) ? 10.0 / double(amax - amin) : 0;
            double ss = 0;
            if (amax - amin > 0)
                for (long long k = 0; k < count; k++) {
                    const double v = (double)ka[k], e = v - amean;
                    ss = __dadd_rn(ss, __dmul_rn(e, e));  // pow(e, 2): the correctly rounded square
                    ahist[hist_bin(v, amin, sc, 10)] += 1;
                }
            avar = (count > 1) ? ss / (count - 1) : ss;
            dmin = dkey_inv(kd[0]);
            dmax = dkey_inv(kd[count - 1]);
            dmean = sd / count;
            dmed = dkey_inv(kd[count / 2]);
            const double dsc = (dmax - dmin > 0) ? 10.0 / double(dmax - dmin) : 0;
            double sdv = 0;
            for (long long k = 0; k < count; k++) {
                const double v = dkey_inv(kd[k]), e = v - dmean;
                sdv = __dadd_rn(sdv, __dmul_rn(e, e));
                dhist[hist_bin(v, dmin, dsc, 10)] += 1;
            }
            dvar = (count > 1) ? sdv / (count - 1) : sdv;
        }
        const long long euler = ((long long)a[3] - (long long)a[4]) / 4;
        double *o = feat + J.out;
        int k = 0;
        for (int j = 0; j < 10; j++) o[k++] = ahist[j];
        o[k++] = amax; o[k++] = amean; o[k++] = amed; o[k++] = amin; o[k++] = avar;
        o[k++] = gx; o[k++] = gy; o[k++] = (double)count;
        for (int j = 0; j < 10; j++) o[k++] = dhist[j];
        o[k++] = dmax; o[k++] = dmean; o[k++] = dmed; o[k++] = dmin; o[k++] = dvar;
        o[k++] = (double)euler;
    }
}

void launch_objects(Ctx &c, const double *arena, const Plane *planes, const PlaneStats *stats, const FJob *jobs, int njobs,
                    long long maxpix, const OBJob *oj, double *ws, const Plane *inv_planes, PlaneStats *inv_stats,
                    double *thr, unsigned long long *acc, double *feat) {
    if (njobs <= 0) return;
    int blocks = (int)((maxpix + 255) / 256);
    if (blocks > 256) blocks = 256;
    WC_LAUNCH(c);
    k_ob_invert<<<dim3(blocks, njobs), 256, 0, c.st>>>(arena, planes, stats, jobs, oj, ws);
    launch_plane_stats(c, ws, inv_planes, njobs, inv_stats, 1, 0);
    WC_LAUNCH(c);
    k_ob_otsu<<<njobs, 1024, 0, c.st>>>(arena, planes, stats, inv_stats, jobs, oj, ws, thr);
    for (int stage = 0; stage < 3; stage++) {
        WC_LAUNCH(c);
        k_ob_label<<<dim3(blocks, njobs), 256, 0, c.st>>>(arena, planes, jobs, oj, thr, ws, stage,
                                                          c.opt->union_find_cap);
    }
    WC_LAUNCH(c);
    k_ob_accum<<<dim3(blocks, njobs), 256, 0, c.st>>>(planes, jobs, oj, ws, acc);
    WC_LAUNCH(c);
    k_ob_final<<<njobs, 512, 0, c.st>>>(planes, jobs, oj, ws, acc, feat);
}

}  // namespace wc
