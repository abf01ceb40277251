// Chebyshev-Fourier coefficients on the tensor cores (the mixed form;
// ChebyshevFourier2D, src/transforms/ChebyshevFourier.cpp:42-160): for every
// plane of a batch, c(m, a) = sum over the pixels p of the (downsampled,
// <= 300 x 300) image of I_p F_m(phi_p) T_a(r_p), 23 x 23 complex values, then
// the 32-bin histogram of their magnitudes (k_cf_finish).  All planes of one
// size share the basis B[p][(m, a)], so the sums are a GEMM: planes x pixels
// times pixels x 1058 real basis columns.
//
// Digits.  Pixels and basis values are cut into three 8-bit digits held
// exactly in bf16 (a / u = q0 + q1 2^-8 + q2 2^-16, |q_i| <= 128; u a power of
// two per plane, 2^-7 for the basis, whose values lie in [-1, 1]).  The six
// digit pairs with i + j <= 2 are multiplied by tcgen05.mma into three FP32
// accumulators per basis column over chunks of 1024 pixels: the q0 q0 sums are
// integers below 2^24 there, exact; the others carry their weights 2^-8, 2^-16.
// Each chunk's sum goes to FP64, and the chunks are added in a fixed order, so
// the coefficients carry about 2^-24 of the planes' and the basis' scales -
// more than the FP32 SIMT form (k_cf_accum_f32) they replace.
//
// Layout, pipeline and waits are those of the WND-5 kernel (k_wnd_tc.cu): a
// CTA of 192 threads (warp 0 TMA, warp 1 MMA + TMEM, warps 2..5 epilogue)
// takes 128 planes and one chunk of pixels and walks the 17 basis tiles of 64
// columns; every mbarrier wait is bounded and a wait that runs out sets the
// error word, which the host reports as WC_ERR_DEVICE.
#include <cuda_bf16.h>

#include <cfloat>
#include <cmath>

#include "kcommon.cuh"
#include "kernels.h"
#include "ktcgen05.cuh"

namespace wc {
namespace cft {

constexpr int M = 128, N = 64, KB = 64, SA = 4, SB = 3, NACC = 4, STAGES = 2, NPAIR = 9;
constexpr int A_SLICE = M * KB * 2;  // 16 KB
constexpr int B_SLICE = N * KB * 2;  // 8 KB
constexpr int STAGE_BYTES = SA * A_SLICE + SB * B_SLICE;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 256;
constexpr int THREADS = 192;
constexpr int CHUNK_KB = 16;  // 1024 pixels per chunk
constexpr uint32_t IDESC = tcg::idesc_bf16_f32(M, N);

// digit pairs (i of the pixel, j of the basis) with i + j <= 3, their
// accumulator i + j, and whether the pair is the first into it (it then
// overwrites on a chunk's first K step)
__constant__ unsigned char c_pi[NPAIR] = {0, 0, 1, 0, 1, 2, 1, 2, 3};
__constant__ unsigned char c_pj[NPAIR] = {0, 1, 0, 2, 1, 0, 2, 1, 0};
__constant__ unsigned char c_pa[NPAIR] = {0, 1, 1, 2, 2, 2, 3, 3, 3};
__constant__ unsigned char c_pf[NPAIR] = {1, 1, 0, 1, 0, 0, 1, 0, 0};

__device__ int g_err_cf = 0;

struct Params {
    int M_pad, kb_total, nchunk;
    const double *__restrict__ uA;  // [nchunk][M_pad]: each chunk's digit scale times the basis' (2^-7)
    double *__restrict__ partial;   // [nchunk][M_pad][CF_TC_COLS]
};

__global__ void __launch_bounds__(THREADS, 1)
    k_cf_tc(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, const Params P) {
    using namespace tcg;
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *bars = (uint64_t *)(smem + STAGES * STAGE_BYTES);
    uint32_t *tmem_slot = (uint32_t *)(bars + 8);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int mb = blockIdx.x, ch = blockIdx.y;
    const int kb0 = ch * CHUNK_KB, kb1 = min(P.kb_total, kb0 + CHUNK_KB), nkb = max(0, kb1 - kb0);
    const int ntiles = CF_TC_COLS / N;
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
        if (lane == 0 && nkb > 0) {
            int it = 0;
            for (int tile = 0; tile < ntiles && !bad; tile++)
                for (int kb = kb0; kb < kb1; kb++, it++) {
                    const int st = it & 1;
                    if (!mbar_wait(empty0 + 8 * st, ((it >> 1) & 1) ^ 1)) { bad = true; break; }
                    const uint32_t sA = smem_u32(smem + st * STAGE_BYTES), sB = sA + SA * A_SLICE;
                    mbar_expect_tx(full0 + 8 * st, STAGE_BYTES);
                    tma_load_3d(sA, &mapA, kb * KB, mb * M, 0, full0 + 8 * st);
                    tma_load_3d(sB, &mapB, kb * KB, tile * N, 0, full0 + 8 * st);
                }
            if (bad) atomicExch(&g_err_cf, 41);
            for (int k = max(0, it - 2); k < it; k++) mbar_wait(full0 + 8 * (k & 1), (k >> 1) & 1);
        }
    } else if (warp == 1) {
        // ---- MMA issuer
        if (lane == 0 && nkb > 0) {
            int it = 0;
            for (int tile = 0; tile < ntiles && !bad; tile++) {
                const int buf = tile & 1;
                if (!mbar_wait(aempty0 + 8 * buf, ((tile >> 1) & 1) ^ 1)) { bad = true; break; }
                tc_fence_after();
                for (int kb = 0; kb < nkb; kb++, it++) {
                    const int st = it & 1;
                    if (!mbar_wait(full0 + 8 * st, (it >> 1) & 1)) { bad = true; break; }
                    tc_fence_after();
                    const uint32_t sA = smem_u32(smem + st * STAGE_BYTES), sB = sA + SA * A_SLICE;
#pragma unroll
                    for (int ks = 0; ks < KB / 16; ks++) {
#pragma unroll
                        for (int p = 0; p < NPAIR; p++) {
                            const uint64_t da = sdesc(sA + c_pi[p] * A_SLICE + ks * 32);
                            const uint64_t db = sdesc(sB + c_pj[p] * B_SLICE + ks * 32);
                            const uint32_t td = tmem + (uint32_t)((buf * NACC + c_pa[p]) * N);
                            mma_bf16(td, da, db, IDESC, (kb == 0 && ks == 0 && c_pf[p]) ? 0u : 1u);
                        }
                    }
                    mma_commit(empty0 + 8 * st);
                }
                if (bad) break;
                mma_commit(afull0 + 8 * buf);
            }
            if (bad) atomicExch(&g_err_cf, 42);
            if (it > 0) mbar_wait(empty0 + 8 * ((it - 1) & 1), ((it - 1) >> 1) & 1);
        }
    } else if (nkb > 0) {
        // ---- epilogue: warps 2..5; warp w reads TMEM lanes 32 (w % 4) ..
        const int q = warp & 3;
        const int row = mb * M + q * 32 + lane;
        const double scale = P.uA[(long long)ch * P.M_pad + row];
        double *out = P.partial + ((long long)ch * P.M_pad + row) * CF_TC_COLS;
        const uint32_t lane_addr = tmem + ((uint32_t)(q * 32) << 16);
        for (int tile = 0; tile < ntiles; tile++) {
            const int buf = tile & 1;
            if (!__all_sync(0xffffffffu, mbar_wait(afull0 + 8 * buf, (tile >> 1) & 1))) { bad = true; break; }
            tc_fence_after();
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
                for (int i = 0; i < 16; i++)
                    out[tile * N + c0 + i] =
                        ((((double)a0[i] + (double)a1[i]) + (double)a2[i]) + (double)a3[i]) * scale;
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(aempty0 + 8 * buf);
        }
        if (bad) atomicExch(&g_err_cf, 43);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
}

// a (|a| < 128) into nd balanced digits q_i 2^-8i (|q_i| <= 128) at d[0],
// d[step], ..., each exact in bf16: a is rounded once to the fixed point
// X = RN(a 2^(8 nd - 8)), and the digits come from X by integer shifts (the
// integer pipe, not the FP64 one)
__device__ __forceinline__ void cf_digits(double a, __nv_bfloat16 *d, long long step, int nd) {
    long long X = __double2ll_rn(ldexp(a, 8 * nd - 8));
    for (int i = 0; i < nd; i++) {
        const int sh = 8 * (nd - 1 - i);
        const long long q = sh ? (X + (1LL << (sh - 1))) >> sh : X;  // arithmetic shift: floor
        X -= q * (1LL << sh);
        d[i * step] = __float2bfloat16_rn(ldexpf((float)q, -8 * i));
    }
}

// the basis digits of one size: a thread per pixel k = y n + x (row-major; the
// order of the K dimension is the GEMM's own, the same for both operands);
// pixels off the unit disc (the reference's FP64 test, rounded as k_cf_accum
// rounds it) and padding stay 0 (memset)
__global__ void __launch_bounds__(128) k_cf_tc_basis(int m, int n, long long K_pad, __nv_bfloat16 *__restrict__ dig) {
    const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k >= (long long)m * n) return;
    const long long y = k / n, x = k - y * n;
    const double tn = 2.0 / ((double)n - 1), tm = 2.0 / ((double)m - 1);
    const double xi = __dadd_rn(-1.0, __dmul_rn((double)x, tn)), yi = __dadd_rn(-1.0, __dmul_rn((double)y, tm));
    const double r = sqrt(__dadd_rn(__dmul_rn(xi, xi), __dmul_rn(yi, yi)));
    if (!(r < 1)) return;
    double xx = __dsub_rn(__dmul_rn(r, 2.0), 1.0);
    if (xx < -1) xx = -1;
    if (xx > 1) xx = 1;
    const double ac = acos(xx), fi = -1 * atan2(yi, xi);
    double T[23];
    for (int a = 0; a < 23; a++) T[a] = cos(a * ac);
    T[0] = 0.5;
    const long long plane = (long long)CF_TC_COLS * K_pad;
    for (int im = 0; im < 23; im++) {
        const long mf = im - 11;
        const double Ft = (mf == 0) ? 0.5 : 1.0;
        const double fc = Ft * cos(mf * fi), fs = Ft * sin(-1 * mf * fi);
        for (int a = 0; a < 23; a++) {
            const int o = im * 23 + a;
            __nv_bfloat16 *p = dig + (long long)(2 * o) * K_pad + k;
            cf_digits(fc * T[a] * 128.0, p, plane, SB);
            cf_digits(fs * T[a] * 128.0, p + K_pad, plane, SB);
        }
    }
}

// the digit scale of every (plane, chunk of 1024 pixels): the power of two u
// with max |I| / u in [64, 128) over the chunk (1 for zeros); uA[ch][row] =
// u 2^-7 (the basis' scale folded in).  A scale per chunk keeps a plane's
// small values (most of a Chebyshev or Fourier plane) at 32 bits of their
// own chunk's largest.
__global__ void k_cf_tc_scale(const CFJob *__restrict__ cj, const double *__restrict__ ws, long long M_pad,
                              double *__restrict__ uA) {
    __shared__ double sh[32];
    const int row = blockIdx.y, ch = blockIdx.x;
    const CFJob C = cj[row];
    const int m = C.new_h, n = C.new_w;
    const double *img = ws + C.src_ws;
    const long long k0 = (long long)ch * CHUNK_KB * KB, k1 = min((long long)m * n, k0 + CHUNK_KB * KB);
    double mx = 0, bad = 0;
    for (long long k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
        const double v = img[k];
        if (isfinite(v)) mx = fmax(mx, fabs(v));
        else bad = 1;
    }
    mx = block_max(mx, sh);
    bad = block_max(bad, sh);
    if (threadIdx.x == 0) {
        int e = 0;
        if (mx > 0) frexp(mx, &e);  // mx = f 2^e, f in [0.5, 1)
        // a non-finite pixel makes every coefficient of the plane NaN, as the
        // FP64 sums would: the chunk's scale is NaN
        uA[(long long)ch * M_pad + row] = bad ? __longlong_as_double(0x7ff8000000000000LL)
                                              : (mx > 0 ? ldexp(1.0, e - 7) * 0x1p-7 : 0x1p-7);
    }
}

// the planes' digits, [4][M_pad][K_pad], pixel k = y n + x of plane row
__global__ void k_cf_tc_pixels(const CFJob *__restrict__ cj, int njobs, const double *__restrict__ ws,
                               const double *__restrict__ uA, long long K_pad, long long M_pad,
                               __nv_bfloat16 *__restrict__ dig) {
    const int row = blockIdx.y;
    if (row >= njobs) return;
    const CFJob C = cj[row];
    const int m = C.new_h, n = C.new_w;
    const double *img = ws + C.src_ws;
    const long long plane = M_pad * K_pad;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < (long long)m * n;
         k += (long long)gridDim.x * blockDim.x) {
        const double u = uA[(k / (CHUNK_KB * KB)) * M_pad + row];
        const double inv = isfinite(u) ? 1.0 / (u * 0x1p7) : 0.0;  // a power of two: exact
        const double v = img[k];
        cf_digits(isfinite(v) ? v * inv : 0.0, dig + (long long)row * K_pad + k, plane, SA);
    }
}

// the chunks added in order, into k_cf_finish's partial layout (chunk 0)
__global__ void k_cf_tc_reduce(const double *__restrict__ partial, int nchunk, long long M_pad, int njobs,
                               int nchunk_max, double *__restrict__ part) {
    const int row = blockIdx.y;
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= njobs || col >= 2 * 529) return;
    double s = 0;
    for (int c = 0; c < nchunk; c++) s += partial[((long long)c * M_pad + row) * CF_TC_COLS + col];
    part[(long long)row * nchunk_max * (2 * 529) + col] = s;
}

}  // namespace cft

int cf_tc_err_take(cudaStream_t st, int *v) {
    *v = 0;
    if (cudaMemcpyFromSymbolAsync(v, cft::g_err_cf, sizeof(int), 0, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return -1;
    if (*v) {
        const int z = 0;
        cudaMemcpyToSymbolAsync(cft::g_err_cf, &z, sizeof(int), 0, cudaMemcpyHostToDevice, st);
        cudaStreamSynchronize(st);
    }
    return 0;
}

CFTcPlan cf_tc_plan(int njobs, int m, int n) {
    CFTcPlan p;
    p.K_pad = ((long long)m * n + cft::KB - 1) / cft::KB * cft::KB;
    p.M_pad = ((long long)njobs + cft::M - 1) / cft::M * cft::M;
    const int kb_total = (int)(p.K_pad / cft::KB);
    p.nchunk = (kb_total + cft::CHUNK_KB - 1) / cft::CHUNK_KB;
    p.digA_bytes = (size_t)cft::SA * p.M_pad * p.K_pad * 2;
    p.digB_bytes = (size_t)cft::SB * CF_TC_COLS * p.K_pad * 2;
    p.partial_bytes = (size_t)p.nchunk * p.M_pad * CF_TC_COLS * 8;
    p.uA_bytes = (size_t)p.nchunk * p.M_pad * 8;
    return p;
}

// The coefficients of njobs planes of one m x n size (m, n >= 23) into part
// (k_cf_finish's layout, chunk 0): basis and plane digits, the tensor-core
// products, the chunk sums.  Returns false (nothing launched) where a tensor
// map cannot be made; the caller then runs the SIMT form.
bool launch_cf_tc(Ctx &c, const CFJob *cj, int njobs, int m, int n, const double *ws, const CFTcPlan &p,
                  const CFTcBufs &b, double *part, int nchunk_max) {
    using namespace cft;
    CUtensorMap mapA, mapB;
    if (tcg::digit_map_3d(&mapA, b.digA, p.M_pad, p.K_pad, M, KB, SA) != WC_OK ||
        tcg::digit_map_3d(&mapB, b.digB, CF_TC_COLS, p.K_pad, N, KB, SB) != WC_OK) {
        cudaGetLastError();
        return false;
    }
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_cf_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
        attr = true;
    }
    cudaMemsetAsync(b.digA, 0, p.digA_bytes, c.st);
    cudaMemsetAsync(b.digB, 0, p.digB_bytes, c.st);
    cudaMemsetAsync(b.uA, 0, p.uA_bytes, c.st);
    *c.launches += 5;
    k_cf_tc_basis<<<(unsigned)(((long long)m * n + 127) / 128), 128, 0, c.st>>>(m, n, p.K_pad, (__nv_bfloat16 *)b.digB);
    k_cf_tc_scale<<<dim3((unsigned)p.nchunk, njobs), 256, 0, c.st>>>(cj, ws, p.M_pad, b.uA);
    k_cf_tc_pixels<<<dim3(64, njobs), 256, 0, c.st>>>(cj, njobs, ws, b.uA, p.K_pad, p.M_pad,
                                                      (__nv_bfloat16 *)b.digA);
    Params P{(int)p.M_pad, (int)(p.K_pad / KB), p.nchunk, b.uA, b.partial};
    k_cf_tc<<<dim3((unsigned)(p.M_pad / M), (unsigned)p.nchunk), THREADS, SMEM_BYTES, c.st>>>(mapA, mapB, P);
    k_cf_tc_reduce<<<dim3((2 * 529 + 255) / 256, njobs), 256, 0, c.st>>>(b.partial, p.nchunk, p.M_pad, njobs,
                                                                         nchunk_max, part);
    return true;
}

}  // namespace wc
