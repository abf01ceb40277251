// Fourier transform node: |2-D DFT| of a real plane, as ImageMatrix::fft2
// (src/cmatrix.cpp:1107-1160) defines it: the magnitude of X[kx][ky] for
// ky <= H/2, rows below copied from their Hermitian mirrors
// out(y, x) = out(H - y, (W - x) mod W), no scaling, no shift.
//
// 1-D transforms are Stockham mixed-radix DFTs in shared memory, several
// lines per CTA; any length up to kMaxFFT (radices 8, 4, 2 as butterflies,
// then odd primes as direct DFTs, O(p) per output).  Twiddles
// exp(-2 pi i k / n) come from an FP64 table computed on the host.
#include <cmath>

#include "kcommon.cuh"
#include "kernels.h"
#include "kfft.cuh"

namespace wc {

// pass along y: each CTA transforms `lpc` columns; keeps ky < H/2+1 in
// cbuf[ky * W + x].
__global__ void k_fourier_y(const double *__restrict__ arena, const Plane *__restrict__ planes, const TJob *__restrict__ jobs,
                            const FFTPlan *__restrict__ plans, const int *__restrict__ job_plan,
                            const double *__restrict__ twd, double *__restrict__ cbuf, const long long *__restrict__ cbuf_off,
                            int lpc) {
    extern __shared__ double smem[];
    const TJob J = jobs[blockIdx.y];
    const Plane S = planes[J.src];
    const int W = S.w, H = S.h, hh = H / 2 + 1;
    const int x0 = blockIdx.x * lpc;
    if (x0 >= W) return;
    const int lines = min(lpc, W - x0);
    const FFTPlan P = plans[job_plan[blockIdx.y]];
    const cplx *tw = (const cplx *)(twd + P.tw_off);
    cplx *b0 = (cplx *)smem, *b1 = b0 + (long long)lpc * H;
    const double *in = arena + S.off;
    for (int i = threadIdx.x; i < lines * H; i += blockDim.x) {
        const int y = i / lines, l = i - y * lines;  // consecutive threads: consecutive x
        b0[(long long)l * H + y] = {in[(long long)y * W + x0 + l], 0.0};
    }
    __syncthreads();
    const cplx *r = stockham(b0, b1, lines, P, tw) ? b1 : b0;
    cplx *out = (cplx *)(cbuf + cbuf_off[blockIdx.y]);
    for (int i = threadIdx.x; i < lines * hh; i += blockDim.x) {
        const int ky = i / lines, l = i - ky * lines;
        out[(long long)ky * W + x0 + l] = r[(long long)l * H + ky];
    }
}

// pass along x for each kept row ky: magnitude into the destination plane
__global__ void k_fourier_x(double *__restrict__ arena, const Plane *__restrict__ planes, const TJob *__restrict__ jobs,
                            const FFTPlan *__restrict__ plans, const int *__restrict__ job_plan,
                            const double *__restrict__ twd, const double *__restrict__ cbuf,
                            const long long *__restrict__ cbuf_off, int lpc) {
    extern __shared__ double smem[];
    const TJob J = jobs[blockIdx.y];
    const Plane S = planes[J.src], D = planes[J.dst];
    const int W = S.w, H = S.h, hh = H / 2 + 1;
    const int y0 = blockIdx.x * lpc;
    if (y0 >= hh) return;
    const int lines = min(lpc, hh - y0);
    const FFTPlan P = plans[job_plan[blockIdx.y]];
    const cplx *tw = (const cplx *)(twd + P.tw_off);
    cplx *b0 = (cplx *)smem, *b1 = b0 + (long long)lpc * W;
    const cplx *in = (const cplx *)(cbuf + cbuf_off[blockIdx.y]);
    for (int i = threadIdx.x; i < lines * W; i += blockDim.x) b0[i] = in[(long long)y0 * W + i];
    __syncthreads();
    const cplx *r = stockham(b0, b1, lines, P, tw) ? b1 : b0;
    double *out = arena + D.off;
    for (int i = threadIdx.x; i < lines * W; i += blockDim.x) {
        const int l = i / W, x = i - l * W;
        const cplx c = r[i];
        out[(long long)(y0 + l) * W + x] = sqrt(__dadd_rn(__dmul_rn(c.x, c.x), __dmul_rn(c.y, c.y)));
    }
}

// rows y >= H/2+1: out(y, x) = out(H - y, (W - x) mod W)
__global__ void k_fourier_mirror(double *__restrict__ arena, const Plane *__restrict__ planes, const TJob *__restrict__ jobs) {
    const TJob J = jobs[blockIdx.z];
    const Plane D = planes[J.dst];
    const int W = D.w, H = D.h, hh = H / 2 + 1;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = hh + blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    double *o = arena + D.off;
    o[(long long)y * W + x] = o[(long long)(H - y) * W + (x == 0 ? 0 : W - x)];
}

void launch_fourier(Ctx &c, double *arena, const Plane *planes, const TJob *jobs, int njobs, int maxw, int maxh,
                    const FFTPlan *plans_d, const int *job_plan_y, const int *job_plan_x, const double *tw,
                    double *cbuf, const long long *cbuf_off) {
    if (njobs <= 0) return;
    const int smem_budget = 96 * 1024;
    int lpc_y = smem_budget / (32 * maxh);
    if (lpc_y < 1) lpc_y = 1;
    if (lpc_y > 16) lpc_y = 16;
    int lpc_x = smem_budget / (32 * maxw);
    if (lpc_x < 1) lpc_x = 1;
    if (lpc_x > 16) lpc_x = 16;
    size_t sm_y = (size_t)lpc_y * maxh * 32, sm_x = (size_t)lpc_x * maxw * 32;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_fourier_y, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(k_fourier_x, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr = true;
    }
    WC_LAUNCH(c);
    k_fourier_y<<<dim3((maxw + lpc_y - 1) / lpc_y, njobs), 256, sm_y, c.st>>>(arena, planes, jobs, plans_d, job_plan_y,
                                                                             tw, cbuf, cbuf_off, lpc_y);
    const int hh = maxh / 2 + 1;
    WC_LAUNCH(c);
    k_fourier_x<<<dim3((hh + lpc_x - 1) / lpc_x, njobs), 256, sm_x, c.st>>>(arena, planes, jobs, plans_d, job_plan_x, tw,
                                                                           cbuf, cbuf_off, lpc_x);
    WC_LAUNCH(c);
    k_fourier_mirror<<<dim3((maxw + 31) / 32, (maxh - hh + 7) / 8 + 1, njobs), dim3(32, 8), 0, c.st>>>(arena, planes, jobs);
}

}  // namespace wc
