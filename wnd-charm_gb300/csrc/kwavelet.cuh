// One level of the zero-padded Symlet-5 decomposition
// (Wavelet::transform2D, src/transforms/wavelet/Wavelet.cpp:136-434, with
// downsampling_convolution MODE_ZEROPAD, convolution.cpp:86-325):
// out[o] = sum_j f[j] * x[2o+1-j] over the taps inside the input, j ascending,
// each product and sum rounded separately (the CPU order, bit for bit).
//
// The per-output tap loops of both passes live here, with the one copy of the
// filter taps (Symlet5.cpp:15-23), so that every kernel that computes this
// transform (the batched engine's, the allocation-free entry point's) and its
// adjoint (the backward pass) shares them.  Each translation unit that includes
// this header gets its own __constant__ copy of the taps.
#pragma once

__constant__ double c_sym5_lo[10] = {0.027333068345077982, 0.029519490925774643, -0.039134249302383094,
                                     0.1993975339773936,   0.72340769040242059,  0.63397896345821192,
                                     0.016602105764522319, -0.17532808990845047, -0.021101834024758855,
                                     0.019538882735286728};
__constant__ double c_sym5_hi[10] = {-0.019538882735286728, -0.021101834024758855, 0.17532808990845047,
                                     0.016602105764522319,  -0.63397896345821192,  0.72340769040242059,
                                     -0.1993975339773936,   -0.039134249302383094, -0.029519490925774643,
                                     0.027333068345077982};

// output size along one axis of length n
__host__ __device__ __forceinline__ int sym5_out(int n) { return (n + 9) / 2; }

// pass 1 (along y) for column x, output row o: approximation a, detail d.
// `in` is X wide, Y tall, row-major.
__device__ __forceinline__ void sym5_col(const double *__restrict__ in, int X, int Y, int x, int o, double &a,
                                         double &d) {
    const int i = 2 * o + 1;
    a = 0;
    d = 0;
#pragma unroll
    for (int j = 0; j < 10; j++) {
        const int k = i - j;
        if (k >= 0 && k < Y) {
            const double v = in[(long long)k * X + x];
            a = __dadd_rn(a, __dmul_rn(v, c_sym5_lo[j]));
            d = __dadd_rn(d, __dmul_rn(v, c_sym5_hi[j]));
        }
    }
}

// pass-1 layout: t[(x*oy + o)*2 + {0: approximation, 1: detail}]
__device__ __forceinline__ long long sym5_tmp_index(int x, int oy, int o) { return ((long long)x * oy + o) * 2; }

// pass 2 (along x) for output column u of row o of both pass-1 outputs:
// a1/d1 from the approximations, a2/d2 from the details.
__device__ __forceinline__ void sym5_row(const double *__restrict__ t, int X, int oy, int u, int o, double &a1,
                                         double &d1, double &a2, double &d2) {
    const int i = 2 * u + 1;
    a1 = d1 = a2 = d2 = 0;
#pragma unroll
    for (int j = 0; j < 10; j++) {
        const int k = i - j;
        if (k >= 0 && k < X) {
            const long long q = sym5_tmp_index(k, oy, o);
            const double va = t[q], vd = t[q + 1];
            a1 = __dadd_rn(a1, __dmul_rn(va, c_sym5_lo[j]));
            d1 = __dadd_rn(d1, __dmul_rn(va, c_sym5_hi[j]));
            a2 = __dadd_rn(a2, __dmul_rn(vd, c_sym5_lo[j]));
            d2 = __dadd_rn(d2, __dmul_rn(vd, c_sym5_hi[j]));
        }
    }
}

// quadrant placement of the four pass-2 outputs in the (2*ox) x (2*oy) plane
// (Wavelet.cpp:359-428): (y<oy, x<ox) d2, (y>=oy, x<ox) a2, (y<oy, x>=ox) d1,
// (y>=oy, x>=ox) a1.
__device__ __forceinline__ void sym5_store(double *__restrict__ out, int ox, int oy, int u, int o, double a1,
                                           double d1, double a2, double d2) {
    const int W = 2 * ox;
    out[(long long)o * W + u] = d2;
    out[(long long)(oy + o) * W + u] = a2;
    out[(long long)o * W + ox + u] = d1;
    out[(long long)(oy + o) * W + ox + u] = a1;
}
