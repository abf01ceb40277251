// Chebyshev transform node: ImageMatrix::ChebyshevTransform(N = min(W,H))
// with Chebyshev2D (src/cmatrix.cpp:1203-1222, src/transforms/chebyshev.cpp:118-165):
//   Mid[y][j] = sum_x I[y][x] * TA[x][j]      (H x N, TA = T_j(x_x) * w_j / 2)
//   Out[j][k] = sum_y Mid[y][j] * TB[y][k]    (N x N), output pixel (y=j, x=k).
// Both products are FP64 register-tiled GEMMs whose threads accumulate every
// output over k in ascending order with separate multiply and add, which is
// the reference's order of operations (getChCoeff1D, chebyshev.cpp:82-102), so
// on identical input the result is bit-identical to the CPU.
#include "kcommon.cuh"
#include "kernels.h"

namespace wc {

#define GT_M 64
#define GT_N 64
#define GT_K 16

// C[i][j] = sum_k A(i,k) B(k,j); A(i,k) = A[i*sai + k*sak], B(k,j) = B[k*ldb + j],
// C[i*ldc + j].  One CTA per 64x64 tile, 256 threads, up to 4x4 outputs each
// (rows ty + 16 r, columns tx + 16 s).  The K tiles are double-buffered: the
// next tile's global loads are issued into registers before the current
// tile's products, and stored to the other shared buffer after them, so the
// FP64 pipe does not wait on global memory (every output still sums its terms
// in ascending k).  RS x SS is the part of the 4x4 register tile that holds
// valid outputs: a tile on the matrix's edge (planes of 257 or 520 columns
// leave 1 or 8 in the last tile column) issues only the products it needs, as
// the FP64 pipe is charged per warp instruction whatever the lanes.
typedef double GTile[2][GT_K][GT_M + 1];
template <int RS, int SS>
__device__ void gemm_tile(const double *__restrict__ A, long long sai, long long sak, const double *__restrict__ B,
                          long long ldb, double *__restrict__ C, long long ldc, int M, int N, int K, int ti, int tj,
                          GTile &As, GTile &Bs) {
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int i0 = ti * GT_M, j0 = tj * GT_N;
    constexpr int PER = GT_K * GT_M / 256;  // elements of each tile per thread (4)
    double acc[RS][SS];
#pragma unroll
    for (int a = 0; a < RS; a++)
#pragma unroll
        for (int b = 0; b < SS; b++) acc[a][b] = 0.0;
    double ra[PER], rb[PER];
    auto load = [&](int k0) {
#pragma unroll
        for (int u = 0; u < PER; u++) {
            const int q = threadIdx.x + 256 * u;
            const int kk = q / GT_M, ii = q - kk * GT_M;
            const int i = i0 + ii, j = j0 + ii, k = k0 + kk;
            ra[u] = (i < M && k < K) ? A[(long long)i * sai + (long long)k * sak] : 0.0;
            rb[u] = (j < N && k < K) ? B[(long long)k * ldb + j] : 0.0;
        }
    };
    auto store = [&](int buf) {
#pragma unroll
        for (int u = 0; u < PER; u++) {
            const int q = threadIdx.x + 256 * u;
            const int kk = q / GT_M, ii = q - kk * GT_M;
            As[buf][kk][ii] = ra[u];
            Bs[buf][kk][ii] = rb[u];
        }
    };
    load(0);
    store(0);
    __syncthreads();
    int cur = 0;
    for (int k0 = 0; k0 < K; k0 += GT_K) {
        const bool more = k0 + GT_K < K;
        if (more) load(k0 + GT_K);
        const int kend = min(GT_K, K - k0);
        for (int kk = 0; kk < kend; kk++) {
            double a[RS], b[SS];
#pragma unroll
            for (int r = 0; r < RS; r++) a[r] = As[cur][kk][ty + 16 * r];
#pragma unroll
            for (int s2 = 0; s2 < SS; s2++) b[s2] = Bs[cur][kk][tx + 16 * s2];
#pragma unroll
            for (int r = 0; r < RS; r++)
#pragma unroll
                for (int s2 = 0; s2 < SS; s2++) acc[r][s2] = __dadd_rn(acc[r][s2], __dmul_rn(a[r], b[s2]));
        }
        if (more) store(cur ^ 1);
        __syncthreads();
        cur ^= 1;
    }
#pragma unroll
    for (int r = 0; r < RS; r++)
#pragma unroll
        for (int s2 = 0; s2 < SS; s2++) {
            int i = i0 + ty + 16 * r, j = j0 + tx + 16 * s2;
            if (i < M && j < N) C[(long long)i * ldc + j] = acc[r][s2];
        }
}

// the register-tile shape for the tile's valid rows and columns (uniform per CTA)
template <int RS>
__device__ void gemm_tile_ss(int ss, const double *A, long long sai, long long sak, const double *B, long long ldb,
                             double *C, long long ldc, int M, int N, int K, int ti, int tj, GTile &As, GTile &Bs) {
    switch (ss) {
        case 1: gemm_tile<RS, 1>(A, sai, sak, B, ldb, C, ldc, M, N, K, ti, tj, As, Bs); break;
        case 2: gemm_tile<RS, 2>(A, sai, sak, B, ldb, C, ldc, M, N, K, ti, tj, As, Bs); break;
        case 3: gemm_tile<RS, 3>(A, sai, sak, B, ldb, C, ldc, M, N, K, ti, tj, As, Bs); break;
        default: gemm_tile<RS, 4>(A, sai, sak, B, ldb, C, ldc, M, N, K, ti, tj, As, Bs); break;
    }
}
__device__ void gemm_tile_any(const double *A, long long sai, long long sak, const double *B, long long ldb, double *C,
                              long long ldc, int M, int N, int K, int ti, int tj, GTile &As, GTile &Bs) {
    const int rs = min(4, (M - ti * GT_M + 15) / 16), ss = min(4, (N - tj * GT_N + 15) / 16);
    switch (rs) {
        case 1: gemm_tile_ss<1>(ss, A, sai, sak, B, ldb, C, ldc, M, N, K, ti, tj, As, Bs); break;
        case 2: gemm_tile_ss<2>(ss, A, sai, sak, B, ldb, C, ldc, M, N, K, ti, tj, As, Bs); break;
        case 3: gemm_tile_ss<3>(ss, A, sai, sak, B, ldb, C, ldc, M, N, K, ti, tj, As, Bs); break;
        default: gemm_tile_ss<4>(ss, A, sai, sak, B, ldb, C, ldc, M, N, K, ti, tj, As, Bs); break;
    }
}

// stage 0: Mid = I * TA ; stage 1: Out = Mid^T * TB
__global__ void __launch_bounds__(256) k_cheb_gemm(double *__restrict__ arena, const Plane *__restrict__ planes,
                                                   const TJob *__restrict__ jobs, const double *__restrict__ tabs,
                                                   const long long *__restrict__ tab_off, double *__restrict__ mid,
                                                   const long long *__restrict__ mid_off, int stage) {
    __shared__ GTile As, Bs;
    const TJob J = jobs[blockIdx.z];
    const Plane S = planes[J.src];
    const int W = S.w, H = S.h, N = min(W, H);
    double *Mid = mid + mid_off[blockIdx.z];
    const double *TA = tabs + tab_off[2 * blockIdx.z], *TB = tabs + tab_off[2 * blockIdx.z + 1];
    if (stage == 0) {
        if (blockIdx.x * GT_N >= N || blockIdx.y * GT_M >= H) return;
        gemm_tile_any(arena + S.off, W, 1, TA, N, Mid, N, H, N, W, blockIdx.y, blockIdx.x, As, Bs);
    } else {
        const Plane D = planes[J.dst];
        if (blockIdx.x * GT_N >= N || blockIdx.y * GT_M >= N) return;
        gemm_tile_any(Mid, 1, N, TB, N, arena + D.off, N, N, N, H, blockIdx.y, blockIdx.x, As, Bs);
    }
}

void launch_chebyshev(Ctx &c, double *arena, const Plane *planes, const TJob *jobs, int njobs, int maxw, int maxh,
                      const double *tabs, const long long *tab_off, double *mid, const long long *mid_off) {
    if (njobs <= 0) return;
    const int N = maxw < maxh ? maxw : maxh;
    WC_LAUNCH(c);
    k_cheb_gemm<<<dim3((N + GT_N - 1) / GT_N, (maxh + GT_M - 1) / GT_M, njobs), 256, 0, c.st>>>(arena, planes, jobs, tabs,
                                                                                            tab_off, mid, mid_off, 0);
    WC_LAUNCH(c);
    k_cheb_gemm<<<dim3((N + GT_N - 1) / GT_N, (N + GT_M - 1) / GT_M, njobs), 256, 0, c.st>>>(arena, planes, jobs, tabs,
                                                                                         tab_off, mid, mid_off, 1);
}

}  // namespace wc
