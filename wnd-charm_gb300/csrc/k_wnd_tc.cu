// WND-5 distances on the tensor cores (sm_103a: tcgen05.mma, TMA, TMEM).
//
// classify2 (src/wndchrm_src/TrainingSet.cpp:2429-2586) needs, for every test
// row t and training row s, d(t,s) = sum_k w_k^2 (t_k - x_sk)^2 over the K
// features with a non-zero weight, then per class the mean of d^-5.  With
// a = w o (t - 50) and b = w o (x - 50) (the normalised values lie in
// [0, 100]), d = |a|^2 + |b|^2 - 2 a.b: the cross term is a T x N x K GEMM.
//
// Exactness.  Every a (and b) is cut, with one power-of-two scale u for the
// whole job, into four 8-bit digits: a/u = q0 + q1 2^-8 + q2 2^-16 + q3 2^-24
// with integers |q_i| <= 128, stored as bf16 values q_i 2^-8i (exact).  The
// tensor core multiplies digit pairs exactly and sums them in FP32 into four
// TMEM accumulators:
//   acc0 = sum q0 q0                        (integers below 2^24 for K <= 511: exact)
//   acc1 = sum (q0 q1 + q1 q0) 2^-8         (multiples of 2^-8 below 2^16: exact)
//   acc2 = sum (q0 q2 + q1 q1 + q2 q0) 2^-16 (exact while its terms' absolute sum,
//                                           bounded per row by Cauchy-Schwarz,
//                                           stays below 2^24 units of 2^-16)
//   acc3 = the pairs with i + j = 3, 4      (FP32; relative weight below 2^-24)
// so their sum is the dot product of the digit-truncated vectors a~ . b~ up
// to acc3's rounding and the dropped pairs (i + j >= 5), both bounded per
// test row, and d~ = |a~|^2 + |b~|^2 - 2 a~.b~ is |a~ - b~|^2 with no
// cancellation error beyond them.  Against the true distance,
// |d - d~| <= 2 sqrt(d~) rho + rho^2 + e_t, rho = |a - a~| + |b - b~| (the
// digit residuals, known per row in FP64) and e_t the row's FP32 bound.
// Each pair's bound is checked in the epilogue; a test row with any pair
// whose relative bound exceeds 2^-26 (or a near-duplicate, or a top-2 class
// margin closer than the bound allows) is recomputed by the FP64 kernel in
// the reference's order.  Every other row's d^-5 carries a relative error
// below ~1e-7, so its probabilities stay within 1e-6 and its class is the
// FP64 form's.
//
// Layout.  Training rows are sorted by class and each class padded to a
// multiple of the 64-row tile, so a tile belongs to one class and the
// epilogue keeps one running class sum.  A CTA takes 128 test rows (the TMEM
// lanes) and a contiguous range of training tiles; per tile and 64-wide K
// block TMA brings the 4 test digit planes (4 x 16 KB) and the 4 training
// digit planes (4 x 8 KB) into shared memory (128-byte swizzle), one thread
// issues the 13 digit-pair MMAs (M=128, N=64, K=16) per K step, and four
// warps read the accumulators (double-buffered in TMEM) and form
// d^-5 = (1/d)^5 in pairs of floats, summed per class in pairs of floats.
//
// Every wait on an mbarrier is bounded; a wait that runs out sets the
// kernel's error word, the CTA stops issuing work, waits (bounded) for what
// it has in flight, frees its TMEM and returns; the host reports
// WC_ERR_DEVICE.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/wndcharm_gb300.h"
#include "kcommon.cuh"
#include "ktcgen05.cuh"
#include "wc_features.h"

namespace wc {

namespace tc {

constexpr int M = 128;       // test rows per CTA (TMEM lanes)
constexpr int N = 64;        // training rows per tile
constexpr int KB = 64;       // K elements per block: one 128-byte swizzle row of bf16
constexpr int S = 4;         // digits per value
constexpr int NACC = 4;      // accumulators per tile (x 2 buffers x N = all 512 TMEM columns)
constexpr int STAGES = 2;
constexpr int A_SLICE = M * KB * 2;  // 16 KB
constexpr int B_SLICE = N * KB * 2;  // 8 KB
constexpr int STAGE_BYTES = S * (A_SLICE + B_SLICE);
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 /* alignment */ + 256 /* barriers */;
constexpr int THREADS = 192;  // warp 0 TMA, warp 1 MMA + TMEM, warps 2..5 epilogue
constexpr int MAX_K = 511;    // acc0 / acc1 exact below this many features

// digit pairs (i, j) and their accumulator; first[] marks the first MMA
// into each accumulator (it overwrites instead of accumulating)
__constant__ unsigned char c_pi[13] = {0, 0, 1, 0, 1, 2, 0, 1, 2, 3, 1, 2, 3};
__constant__ unsigned char c_pj[13] = {0, 1, 0, 2, 1, 0, 3, 2, 1, 0, 3, 2, 1};
__constant__ unsigned char c_pa[13] = {0, 1, 1, 2, 2, 2, 3, 3, 3, 3, 3, 3, 3};
__constant__ unsigned char c_pf[13] = {1, 1, 0, 1, 0, 0, 1, 0, 0, 0, 0, 0, 0};

constexpr uint32_t IDESC = tcg::idesc_bf16_f32(M, N);
using tcg::mbar_arrive;
using tcg::mbar_expect_tx;
using tcg::mbar_init;
using tcg::mbar_wait;
using tcg::mma_commit;
using tcg::sdesc;
using tcg::smem_u32;
using tcg::tc_fence_after;
using tcg::tc_fence_before;
using tcg::tma_load_3d;
using tcg::tmem_ld16;
using tcg::tmem_ld_wait;
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t accumulate) {
    tcg::mma_bf16(tmem_d, a, b, IDESC, accumulate);
}

__device__ int g_err_tc = 0;

// error-free transformations (explicit roundings: no contraction)
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}

struct Params {
    int T_pad, ntiles, nkb, nch, tiles_per_chunk, C;
    const float4 *__restrict__ astat;  // per test row: |a~|^2 (hi, lo), rho_a, e_t (d'' units)
    const float4 *__restrict__ bstat;  // per training row: |b~|^2 (hi, lo), rho_b, valid (1) / pad (NaN)
    const int *__restrict__ tile_cls;  // class of every training tile
    double *__restrict__ psim;         // [T_pad][nch][C] sums of d''^-5 (d'' = d scaled)
    int *__restrict__ flag;            // [T_pad] rows for the FP64 re-check
    float cscale;                      // 2^(1-g): acc units -> 2 a.b in d'' units
    float dmin;                        // d'' below this: near-duplicate (re-check)
    float tol;                         // relative bound above which a row is re-checked
};

__global__ void __launch_bounds__(THREADS, 1)
    k_wnd_tc(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, const Params P) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *bars = (uint64_t *)(smem + STAGES * STAGE_BYTES);
    // bars: full[2], empty[2], acc_full[2], acc_empty[2]; then the TMEM base
    uint32_t *tmem_slot = (uint32_t *)(bars + 8);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int mb = blockIdx.x, ch = blockIdx.y;
    const int j0 = ch * P.tiles_per_chunk, j1 = min(P.ntiles, j0 + P.tiles_per_chunk);
    const int njobs = max(0, j1 - j0);
    const uint32_t full0 = smem_u32(&bars[0]), empty0 = smem_u32(&bars[2]);
    const uint32_t afull0 = smem_u32(&bars[4]), aempty0 = smem_u32(&bars[6]);

    if (threadIdx.x == 0) {
        for (int s = 0; s < 2; s++) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
            mbar_init(afull0 + 8 * s, 1);
            mbar_init(aempty0 + 8 * s, 4);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(512)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    bool bad = false;

    if (warp == 0) {
        // ---- TMA producer
        if (lane == 0) {
            int it = 0;
            for (int jj = 0; jj < njobs && !bad; jj++) {
                const int tile = j0 + jj;
                for (int kb = 0; kb < P.nkb; kb++, it++) {
                    const int st = it & 1;
                    const uint32_t ph = (it >> 1) & 1;
                    if (!mbar_wait(empty0 + 8 * st, ph ^ 1)) { bad = true; break; }
                    const uint32_t sA = smem_u32(smem + st * STAGE_BYTES), sB = sA + S * A_SLICE;
                    mbar_expect_tx(full0 + 8 * st, STAGE_BYTES);
                    tma_load_3d(sA, &mapA, kb * KB, mb * M, 0, full0 + 8 * st);
                    tma_load_3d(sB, &mapB, kb * KB, tile * N, 0, full0 + 8 * st);
                }
            }
            // drain: every stage this thread filled completes before the CTA leaves
            if (bad) atomicExch(&g_err_tc, 31);
            for (int k = max(0, it - 2); k < it; k++) mbar_wait(full0 + 8 * (k & 1), (k >> 1) & 1);
        }
    } else if (warp == 1) {
        // ---- MMA issuer
        if (lane == 0) {
            int it = 0;
            for (int jj = 0; jj < njobs && !bad; jj++) {
                const int buf = jj & 1;
                if (!mbar_wait(aempty0 + 8 * buf, ((jj >> 1) & 1) ^ 1)) { bad = true; break; }
                tc_fence_after();
                for (int kb = 0; kb < P.nkb; kb++, it++) {
                    const int st = it & 1;
                    if (!mbar_wait(full0 + 8 * st, (it >> 1) & 1)) { bad = true; break; }
                    tc_fence_after();
                    const uint32_t sA = smem_u32(smem + st * STAGE_BYTES), sB = sA + S * A_SLICE;
#pragma unroll
                    for (int ks = 0; ks < KB / 16; ks++) {
#pragma unroll
                        for (int p = 0; p < 13; p++) {
                            const uint64_t da = sdesc(sA + c_pi[p] * A_SLICE + ks * 32);
                            const uint64_t db = sdesc(sB + c_pj[p] * B_SLICE + ks * 32);
                            const uint32_t td = tmem + (uint32_t)((buf * NACC + c_pa[p]) * N);
                            mma_bf16(td, da, db, (kb == 0 && ks == 0 && c_pf[p]) ? 0u : 1u);
                        }
                    }
                    mma_commit(empty0 + 8 * st);  // the stage is free once these MMAs are done
                }
                if (bad) break;
                mma_commit(afull0 + 8 * buf);  // the tile's accumulators are complete
            }
            if (bad) {
                atomicExch(&g_err_tc, 32);
            }
            // the MMAs issued last (and the commits that track them) end before teardown
            if (it > 0) mbar_wait(empty0 + 8 * ((it - 1) & 1), ((it - 1) >> 1) & 1);
        }
    } else {
        // ---- epilogue: warps 2..5; warp w reads TMEM lanes 32 (w % 4) ..
        const int q = warp & 3;
        const int row = q * 32 + lane;  // row within the test block
        const int t = mb * M + row;
        const float4 as = P.astat[t];
        const float nAh = as.x, nAl = as.y, rhoA = as.z, eacc = as.w;
        int cls = -1;
        float Sh = 0.f, Sl = 0.f;
        int flagged = 0;
        const uint32_t lane_addr = tmem + ((uint32_t)(q * 32) << 16);
        for (int jj = 0; jj < njobs; jj++) {
            const int buf = jj & 1, tile = j0 + jj;
            // the whole warp leaves together if the wait runs out (the TMEM loads
            // below are warp-collective)
            if (!__all_sync(0xffffffffu, mbar_wait(afull0 + 8 * buf, (jj >> 1) & 1))) { bad = true; break; }
            tc_fence_after();
            const int c = P.tile_cls[tile];
            if (c != cls) {
                if (cls >= 1) P.psim[((long long)t * P.nch + ch) * P.C + cls - 1] = (double)Sh + (double)Sl;
                cls = c;
                Sh = Sl = 0.f;
            }
#pragma unroll 1
            for (int c0 = 0; c0 < N; c0 += 16) {
                float a0[16], a1[16], a2[16], a3[16];
                const uint32_t base = lane_addr + (uint32_t)(buf * NACC * N + c0);
                __syncwarp();
                tmem_ld16(base, a0);
                tmem_ld16(base + N, a1);
                tmem_ld16(base + 2 * N, a2);
                tmem_ld16(base + 3 * N, a3);
                tmem_ld_wait();
#pragma unroll
                for (int i = 0; i < 16; i++) {
                    const float4 bs = __ldg(&P.bstat[(long long)tile * N + c0 + i]);
                    if (!(bs.w > 0.f)) continue;  // padding row
                    // a~.b~ (units) = acc0 + acc1 + acc2 + acc3, then 2 a~.b~ in d'' units
                    float ch_, cl_, h1, l1, l2;
                    two_sum(a0[i], a1[i], h1, l1);
                    two_sum(h1, a2[i], ch_, l2);
                    cl_ = __fadd_rn(__fadd_rn(l1, l2), a3[i]);
                    ch_ = __fmul_rn(ch_, P.cscale);
                    cl_ = __fmul_rn(cl_, P.cscale);
                    // d'' = |a~|^2 + |b~|^2 - 2 a~.b~
                    float s, e, d, f, dh, dl;
                    two_sum(nAh, bs.x, s, e);
                    e = __fadd_rn(e, __fadd_rn(nAl, bs.y));
                    two_sum(s, -ch_, d, f);
                    f = __fadd_rn(f, __fsub_rn(e, cl_));
                    fast_two_sum(d, f, dh, dl);
                    if (!(dh > P.dmin)) { flagged = 1; continue; }
                    // 1/d'' in pairs: r + rl
                    const float r = __frcp_rn(dh);
                    float ee = __fmaf_rn(-r, dh, 1.f);
                    ee = __fmaf_rn(-r, dl, ee);
                    const float rl = __fmul_rn(r, ee);
                    // bound on |d - d~| / d~
                    const float rho = __fadd_rn(rhoA, bs.z);
                    const float rel = __fmaf_rn(__fmul_rn(2.f, rho), rsqrtf(dh), __fmul_rn(__fmaf_rn(rho, rho, eacc), r));
                    if (rel > P.tol) flagged = 1;
                    // r^2, r^4, r^5 in pairs
                    const float p = __fmul_rn(r, r);
                    float pe = __fmaf_rn(r, r, -p);
                    pe = __fmaf_rn(__fmul_rn(2.f, r), rl, pe);
                    const float qq = __fmul_rn(p, p);
                    float qe = __fmaf_rn(p, p, -qq);
                    qe = __fmaf_rn(__fmul_rn(2.f, p), pe, qe);
                    const float z = __fmul_rn(qq, r);
                    float ze = __fmaf_rn(qq, r, -z);
                    ze = __fmaf_rn(qq, rl, ze);
                    ze = __fmaf_rn(qe, r, ze);
                    // class sum in pairs
                    float s2, e2;
                    two_sum(Sh, z, s2, e2);
                    e2 = __fadd_rn(e2, __fadd_rn(Sl, ze));
                    fast_two_sum(s2, e2, Sh, Sl);
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(aempty0 + 8 * buf);
        }
        if (bad) atomicExch(&g_err_tc, 33);
        if (cls >= 1) P.psim[((long long)t * P.nch + ch) * P.C + cls - 1] = (double)Sh + (double)Sl;
        if (flagged) atomicOr(&P.flag[t], 1);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
}

// Digits of one row per warp.  v -> normalised (signatures::normalize /
// the training set's own min-max, the rules of k_wnd_gather) -> a = w (v - 50)
// -> x = a / u in [-128, 128] -> digits q_i (round to nearest) stored as bf16
// q_i 2^-8i in dig[i][pos][0..Kp).  Row statistics in d'' units: |x~|^2 2^-g as
// a pair of floats, rho = |x - x~| 2^-g/2, and 1 (a real row); the digits'
// Euclidean norms |q_i| in dnorm[pos] and, over the rows, their maxima in
// dmax (as float bits: non-negative floats order as integers).
__global__ void k_wnd_tc_digits(const double *__restrict__ X, int rows, int F, const int *__restrict__ keep, int K,
                                int Kp, const double *__restrict__ mins, const double *__restrict__ maxs,
                                const double2 *__restrict__ rec, const double *__restrict__ w, const int *__restrict__ pos, long long rows_pad,
                                double inv_u, double scale_g, double scale_g2, __nv_bfloat16 *__restrict__ dig,
                                float4 *__restrict__ stat, float4 *__restrict__ dnorm, int *__restrict__ dmax) {
    const int lane = threadIdx.x & 31;
    const long long rw = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5);
    if (rw >= rows) return;
    const long long p = pos ? pos[rw] : rw;
    if (p < 0) return;  // a training row without a class 1..C: not compared (as classify2 skips it)
    double n2 = 0.0, r2 = 0.0, qn[4] = {0, 0, 0, 0};
    for (int k = lane; k < Kp; k += 32) {
        double q[4] = {0, 0, 0, 0};
        if (k < K) {
            const int fcol = keep[k];
            const double mn = mins[fcol], mx = maxs[fcol];
            const double v = wnd_norm(X[rw * F + fcol], mn, mx, rec[fcol]);
            const double x = (w[k] * (v - 50.0)) * inv_u;  // |x| <= 128 by the choice of u
            double rem = x;
            double xt = 0.0;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const double qi = rint(rem);
                q[i] = qi;
                xt += ldexp(qi, -8 * i);
                rem = (rem - qi) * 256.0;
            }
            const double res = x - xt;
            n2 += xt * xt;
            r2 += res * res;
#pragma unroll
            for (int i = 0; i < 4; i++) qn[i] += q[i] * q[i];
        }
#pragma unroll
        for (int i = 0; i < 4; i++)
            dig[((long long)i * rows_pad + p) * Kp + k] = __float2bfloat16_rn((float)ldexp(q[i], -8 * i));
    }
    n2 = warp_sum(n2);
    r2 = warp_sum(r2);
#pragma unroll
    for (int i = 0; i < 4; i++) qn[i] = warp_sum(qn[i]);  // integers: exact in any order
    if (lane == 0) {
        const double n = n2 * scale_g;
        const float h = (float)n;
        stat[p] = make_float4(h, (float)(n - (double)h), (float)(sqrt(r2) * scale_g2), 1.f);
        const float4 dn = make_float4((float)sqrt(qn[0]) * 1.0001f, (float)sqrt(qn[1]) * 1.0001f,
                                      (float)sqrt(qn[2]) * 1.0001f, (float)sqrt(qn[3]) * 1.0001f);
        dnorm[p] = dn;
        if (dmax) {
            atomicMax(&dmax[0], __float_as_int(dn.x));
            atomicMax(&dmax[1], __float_as_int(dn.y));
            atomicMax(&dmax[2], __float_as_int(dn.z));
            atomicMax(&dmax[3], __float_as_int(dn.w));
        }
    }
}

// Per test row, from its digit norms and the training rows' maxima
// (Cauchy-Schwarz bounds of the digit-pair sums): the row is listed for the
// FP64 re-check when acc2's terms could reach 2^24 units (its sum would no
// longer be exact), and stat.w gets e_t, the bound of acc3's FP32 rounding
// (n sequential roundings of at most 2^-24 of its terms' absolute sum) and
// of the dropped pairs i + j >= 5, in d'' units (times 2^(1-g)).
__global__ void k_wnd_tc_rowbound(const float4 *__restrict__ dnorm, const int *__restrict__ dmax, int T, double nround,
                                  double scale_c, float4 *__restrict__ stat, int *__restrict__ flag) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    const float4 a = dnorm[t];
    const double m0 = __int_as_float(dmax[0]), m1 = __int_as_float(dmax[1]), m2 = __int_as_float(dmax[2]),
                 m3 = __int_as_float(dmax[3]);
    const double s2 = (double)a.x * m2 + (double)a.y * m1 + (double)a.z * m0;  // units of 2^-16
    if (!(s2 < 16777216.0)) flag[t] |= 1;
    const double s34 = ((double)a.x * m3 + (double)a.y * m2 + (double)a.z * m1 + (double)a.w * m0) * 0x1p-24 +
                       ((double)a.y * m3 + (double)a.z * m2 + (double)a.w * m1) * 0x1p-32;
    const double drop = ((double)a.z * m3 + (double)a.w * m2) * 0x1p-40 + (double)a.w * m3 * 0x1p-48;
    const double e = (nround * 0x1p-24 * s34 * 1.01 + drop) * scale_c;
    float4 st = stat[t];
    st.w = (float)(e * 1.01) + 1e-30f;
    stat[t] = st;
}

// per test row: class means of the chunk sums, probabilities, class, norm;
// rows flagged by the tensor-core kernel, or whose top two classes lie closer
// than the bound allows, are listed for the FP64 re-check
__global__ void k_wnd_tc_finish(const double *__restrict__ psim, const int *__restrict__ flag, int T, int nch, int C,
                                const long long *__restrict__ ncls, double scale5, double margin,
                                double *__restrict__ probs, int *__restrict__ pred, double *__restrict__ norm,
                                int *__restrict__ recheck, int *__restrict__ nrecheck) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    double sim[16];
    for (int c = 0; c < C; c++) sim[c] = 0;
    for (int k = 0; k < nch; k++)
        for (int c = 0; c < C; c++) sim[c] += psim[((long long)t * nch + k) * C + c];
    int best = -1;
    double bestv = 0, second = 0, tot = 0;
    for (int c = 0; c < C; c++) {
        if (ncls[c] == 0) continue;
        sim[c] /= (double)ncls[c];
        if (sim[c] > bestv) {
            second = bestv;
            bestv = sim[c];
            best = c + 1;
        } else if (sim[c] > second) {
            second = sim[c];
        }
    }
    for (int c = 0; c < C; c++) tot += sim[c];
    for (int c = 0; c < C; c++) probs[(long long)t * C + c] = sim[c] / tot;
    pred[t] = best;
    norm[t] = tot * scale5;
    const bool close = best > 0 && second > 0 && (bestv - second) <= margin * bestv;
    if (flag[t] || close || !(tot > 0) || !isfinite(tot)) recheck[atomicAdd(nrecheck, 1)] = t;
}

}  // namespace tc

int tc_err_take(cudaStream_t st, int *v) {
    *v = 0;
    if (cudaMemcpyFromSymbolAsync(v, tc::g_err_tc, sizeof(int), 0, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return -1;
    if (*v) {
        const int z = 0;
        cudaMemcpyToSymbolAsync(tc::g_err_tc, &z, sizeof(int), 0, cudaMemcpyHostToDevice, st);
        cudaStreamSynchronize(st);
    }
    return 0;
}

}  // namespace wc

namespace wc {

int set_err(int code, const char *fmt, ...);

namespace {

// 3-D map over the digit planes [4][rows_pad][Kp] (bf16), box 64 x box_rows x 4
int digit_map(CUtensorMap *m, void *base, long long rows_pad, int Kp, int box_rows) {
    return tcg::digit_map_3d(m, base, rows_pad, Kp, box_rows, tc::KB, 4);
}

// device buffers of one classification, freed together
struct TcBufs {
    std::vector<void *> ptrs;
    template <typename T>
    int get(T **p, size_t bytes) {
        *p = nullptr;
        void *q = nullptr;
        if (cudaMalloc(&q, bytes ? bytes : 16) != cudaSuccess) {
            cudaGetLastError();
            return set_err(WC_ERR_NOMEM, "cudaMalloc of %zu bytes failed", bytes);
        }
        ptrs.push_back(q);
        *p = (T *)q;
        return WC_OK;
    }
    ~TcBufs() {
        for (void *q : ptrs) cudaFree(q);
    }
};

}  // namespace

bool wnd_tc_supported(int K) { return K >= 1 && K <= tc::MAX_K; }

// The tensor-core WND-5 pass over device-resident rows: dX (N x F training
// rows), dT (T x F test rows), normalised with dmin/dmax and weighted by the
// kept features' weights w (host; their squares are the reference's w^2).
// Writes probabilities, classes and normalisation factors of every test row to
// dprob/dpred/dnorm (device) and returns, in recheck, the test rows the FP64
// kernel must recompute (their device results are then to be replaced).
int wnd_tc_classify(cudaStream_t st, long long *launches, int sms, const double *dX, int N, int F,
                    const int *labels, int C, const double *dT, int T, const std::vector<int> &keep,
                    const std::vector<double> &w, const double *dmin, const double *dmax, const double2 *drec,
                    double *dprob, int *dpred, double *dnorm, std::vector<int> &recheck, long long *info) {
    using namespace tc;
    const int K = (int)keep.size();
    if (!wnd_tc_supported(K)) return set_err(WC_ERR_UNSUPPORTED, "tensor-core WND: K = %d", K);
    const int Kp = (K + KB - 1) / KB * KB, nkb = Kp / KB;
    double maxw = 0;
    for (double v : w) maxw = std::max(maxw, v);
    int E = 0;
    std::frexp(50.0 * maxw, &E);  // 50 maxw < 2^E
    const double inv_u = std::ldexp(1.0, 7 - E);
    int g = 14;
    while ((1LL << (g - 14)) < Kp) g++;
    if (g & 1) g++;
    const double scale_g = std::ldexp(1.0, -g), scale_g2 = std::ldexp(1.0, -g / 2), scale_c = std::ldexp(1.0, 1 - g);
    // training rows sorted by class, each class padded to whole tiles
    std::vector<long long> ncls(C, 0);
    for (int s = 0; s < N; s++)
        if (labels[s] >= 1 && labels[s] <= C) ncls[labels[s] - 1]++;
    std::vector<long long> off(C + 1, 0);
    for (int c = 0; c < C; c++) off[c + 1] = off[c] + (ncls[c] + tc::N - 1) / tc::N * tc::N;
    const long long N_pad = off[C];
    if (N_pad == 0) return set_err(WC_ERR_UNSUPPORTED, "tensor-core WND: no labelled training rows");
    std::vector<int> pos(N, -1), tile_cls(N_pad / tc::N);
    {
        std::vector<long long> fill(off.begin(), off.end() - 1);
        for (int s = 0; s < N; s++)
            if (labels[s] >= 1 && labels[s] <= C) pos[s] = (int)fill[labels[s] - 1]++;
        for (int c = 0; c < C; c++)
            for (long long t = off[c] / tc::N; t < off[c + 1] / tc::N; t++) tile_cls[t] = c + 1;
    }
    const int ntiles = (int)(N_pad / tc::N);
    const long long T_pad = (T + M - 1) / M * M;
    const int mblocks = (int)(T_pad / M);
    // chunks of training tiles per test block: fill whole waves of one CTA per SM
    int nch = 1;
    {
        double best = -1;
        const int hi = std::max(1, std::min(ntiles / 4, 1024));
        for (int c = 1; c <= hi; c++) {
            const long long ctas = (long long)mblocks * c;
            const long long waves = (ctas + sms - 1) / sms;
            const int per = (ntiles + c - 1) / c;
            const double eff = (double)ctas / (double)(waves * sms) * (double)ntiles / (double)(c * per);
            if (eff > best + 1e-3) { best = eff; nch = c; }
        }
    }
    const int per_chunk = (ntiles + nch - 1) / nch;
    // info: CTAs, the kernel's time (ns, CUDA events on the stream), issued
    // tensor FLOPs (13 digit-pair products of T_pad x N_pad x Kp)
    info[0] = (long long)mblocks * nch;
    info[1] = 0;
    info[2] = 13LL * 2 * T_pad * N_pad * Kp;

    TcBufs B;
    __nv_bfloat16 *digA, *digB;
    float4 *astat, *bstat, *dnA, *dnB;
    int *dmaxd, *dtile, *dpos, *dflag, *dkeep, *drc, *dnrc;
    double *dw, *dpsim;
    long long *dncls;
    int rc;
    if ((rc = B.get(&digA, (size_t)4 * T_pad * Kp * 2)) || (rc = B.get(&digB, (size_t)4 * N_pad * Kp * 2)) ||
        (rc = B.get(&astat, T_pad * sizeof(float4))) || (rc = B.get(&bstat, N_pad * sizeof(float4))) ||
        (rc = B.get(&dnA, T_pad * sizeof(float4))) || (rc = B.get(&dnB, N_pad * sizeof(float4))) ||
        (rc = B.get(&dmaxd, 4 * sizeof(int))) || (rc = B.get(&dtile, ntiles * sizeof(int))) ||
        (rc = B.get(&dpos, N * sizeof(int))) || (rc = B.get(&dflag, T_pad * sizeof(int))) ||
        (rc = B.get(&dkeep, K * sizeof(int))) || (rc = B.get(&drc, T * sizeof(int))) ||
        (rc = B.get(&dnrc, sizeof(int))) || (rc = B.get(&dw, K * sizeof(double))) ||
        (rc = B.get(&dpsim, (size_t)T_pad * nch * C * sizeof(double))) || (rc = B.get(&dncls, C * sizeof(long long))))
        return rc;
#define CKT(x)                                                                                          \
    do {                                                                                                \
        cudaError_t e_ = (x);                                                                           \
        if (e_ != cudaSuccess) return set_err(WC_ERR_CUDA, "%s: %s", #x, cudaGetErrorString(e_));       \
    } while (0)
    CKT(cudaMemsetAsync(digA, 0, (size_t)4 * T_pad * Kp * 2, st));
    CKT(cudaMemsetAsync(digB, 0, (size_t)4 * N_pad * Kp * 2, st));
    CKT(cudaMemsetAsync(astat, 0, T_pad * sizeof(float4), st));
    CKT(cudaMemsetAsync(bstat, 0xFF, N_pad * sizeof(float4), st));  // NaN: padding rows
    CKT(cudaMemsetAsync(dnA, 0, T_pad * sizeof(float4), st));
    CKT(cudaMemsetAsync(dmaxd, 0, 4 * sizeof(int), st));
    CKT(cudaMemsetAsync(dflag, 0, T_pad * sizeof(int), st));
    CKT(cudaMemsetAsync(dnrc, 0, sizeof(int), st));
    CKT(cudaMemsetAsync(dpsim, 0, (size_t)T_pad * nch * C * sizeof(double), st));
    CKT(cudaMemcpyAsync(dtile, tile_cls.data(), ntiles * sizeof(int), cudaMemcpyHostToDevice, st));
    CKT(cudaMemcpyAsync(dpos, pos.data(), N * sizeof(int), cudaMemcpyHostToDevice, st));
    CKT(cudaMemcpyAsync(dkeep, keep.data(), K * sizeof(int), cudaMemcpyHostToDevice, st));
    CKT(cudaMemcpyAsync(dw, w.data(), K * sizeof(double), cudaMemcpyHostToDevice, st));
    CKT(cudaMemcpyAsync(dncls, ncls.data(), C * sizeof(long long), cudaMemcpyHostToDevice, st));
    *launches += 5;
    k_wnd_tc_digits<<<(N + 7) / 8, 256, 0, st>>>(dX, N, F, dkeep, K, Kp, dmin, dmax, drec, dw, dpos, N_pad, inv_u, scale_g,
                                                  scale_g2, digB, bstat, dnB, dmaxd);
    k_wnd_tc_digits<<<(T + 7) / 8, 256, 0, st>>>(dT, T, F, dkeep, K, Kp, dmin, dmax, drec, dw, nullptr, T_pad, inv_u, scale_g,
                                                  scale_g2, digA, astat, dnA, nullptr);
    k_wnd_tc_rowbound<<<(T + 255) / 256, 256, 0, st>>>(dnA, dmaxd, T, 7.0 * Kp, scale_c, astat, dflag);
    CUtensorMap mA, mB;
    if ((rc = digit_map(&mA, digA, T_pad, Kp, M)) || (rc = digit_map(&mB, digB, N_pad, Kp, tc::N))) return rc;
    static bool attr = false;
    if (!attr) {
        CKT(cudaFuncSetAttribute(k_wnd_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
        attr = true;
    }
    Params P;
    P.T_pad = (int)T_pad;
    P.ntiles = ntiles;
    P.nkb = nkb;
    P.nch = nch;
    P.tiles_per_chunk = per_chunk;
    P.C = C;
    P.astat = astat;
    P.bstat = bstat;
    P.tile_cls = dtile;
    P.psim = dpsim;
    P.flag = dflag;
    P.cscale = (float)scale_c;
    // near-duplicates: d'' below 1e-6, or a true distance below DBL_EPSILON
    // (the reference skips those training rows)
    const double eps_dd = DBL_EPSILON / std::ldexp(1.0, 2 * (E - 7) + g);
    P.dmin = (float)std::min<double>(std::max(1e-6, eps_dd), FLT_MAX);
    P.tol = 0x1p-26f;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    CKT(cudaEventCreate(&ev0));
    CKT(cudaEventCreate(&ev1));
    CKT(cudaEventRecord(ev0, st));
    k_wnd_tc<<<dim3(mblocks, nch), THREADS, SMEM_BYTES, st>>>(mA, mB, P);
    const cudaError_t le = cudaGetLastError();
    cudaEventRecord(ev1, st);
    if (le != cudaSuccess) {
        cudaEventDestroy(ev0);
        cudaEventDestroy(ev1);
        return set_err(WC_ERR_CUDA, "k_wnd_tc launch: %s", cudaGetErrorString(le));
    }
    const double scale5 = std::ldexp(1.0, -5 * (2 * (E - 7) + g));
    k_wnd_tc_finish<<<(T + 127) / 128, 128, 0, st>>>(dpsim, dflag, T, nch, C, dncls, scale5, 20.0 * 0x1p-26, dprob,
                                                     dpred, dnorm, drc, dnrc);
    CKT(cudaGetLastError());
    int nr = 0;
    CKT(cudaMemcpyAsync(&nr, dnrc, sizeof(int), cudaMemcpyDeviceToHost, st));
    CKT(cudaStreamSynchronize(st));
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ev0, ev1) == cudaSuccess) info[1] = (long long)(ms * 1e6);
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    int ev = 0;
    if (tc_err_take(st, &ev)) return set_err(WC_ERR_CUDA, "reading the tensor-core kernel's error word failed");
    if (ev) return set_err(WC_ERR_DEVICE, "tensor-core WND kernel: a bounded wait ran out (code %d)", ev);
    recheck.assign(nr, 0);
    if (nr) {
        CKT(cudaMemcpyAsync(recheck.data(), drc, nr * sizeof(int), cudaMemcpyDeviceToHost, st));
        CKT(cudaStreamSynchronize(st));
        std::sort(recheck.begin(), recheck.end());
    }
#undef CKT
    return WC_OK;
}

}  // namespace wc
