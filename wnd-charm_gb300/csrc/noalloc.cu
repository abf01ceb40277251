// wc_wavelet_noalloc: the Symlet-5 Wavelet transform for callers that cannot
// allocate device memory.
//
// Some callers may not call cudaMalloc at all: a host application that gives
// the library a fixed device-memory budget and forbids it to grow, a plugin
// host that owns every device allocation itself, or a latency-critical loop
// that must not meet the implicit synchronisation a cudaMalloc/cudaFree can
// bring.  They pass device pointers for the input and the output; the one
// intermediate this transform needs (the column pass, width x
// floor((height+9)/2) x 2 doubles) lives in a file-scope static device array of
// fixed size instead of an allocation.
//
// The first call on each device looks up that array's device address (with
// the device current) and keeps it; make that first call before any stream
// capture begins.
//
// The array is loaded with the library on every GPU that uses it and stays
// allocated there until the process exits.  Every call shares it, so calls
// whose kernels overlap on the GPU (different streams, or several host threads)
// race on it: callers must order them, e.g. by using one stream.  The pass
// overwrites every entry it later reads, so nothing needs clearing between
// calls and stale contents from the previous call are never read.
//
// The arithmetic is that of the Wavelet node of the batched engine (one level
// of Wavelet::transform2D with zero padding, src/transforms/wavelet/Wavelet.cpp:136-434).
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/wndcharm_gb300.h"

namespace wc {
int set_err(int code, const char *fmt, ...);
}

namespace {

// capacity of the static scratch, in doubles: enough for 1024 x 1024 inputs
// (1024 * floor((1024 + 9) / 2) * 2 = 1,056,768); 8.25 MiB per GPU.
constexpr long long kScratchDoubles = 1081344;
static __device__ __align__(256) double g_wavelet_scratch[kScratchDoubles];

__constant__ double c_lo[10] = {0.027333068345077982, 0.029519490925774643, -0.039134249302383094,
                                0.1993975339773936,   0.72340769040242059,  0.63397896345821192,
                                0.016602105764522319, -0.17532808990845047, -0.021101834024758855,
                                0.019538882735286728};
__constant__ double c_hi[10] = {-0.019538882735286728, -0.021101834024758855, 0.17532808990845047,
                                0.016602105764522319,  -0.63397896345821192,  0.72340769040242059,
                                -0.1993975339773936,   -0.039134249302383094, -0.029519490925774643,
                                0.027333068345077982};

// column pass: for every column x, approx/detail along y into the scratch
__global__ void k_wav_y(const double *__restrict__ in, int X, int Y, double *__restrict__ tmp) {
    const int oy = (Y + 9) / 2;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, o = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= X || o >= oy) return;
    const int i = 2 * o + 1;
    double a = 0, d = 0;
#pragma unroll
    for (int j = 0; j < 10; j++) {
        const int k = i - j;
        if (k >= 0 && k < Y) {
            const double v = in[(long long)k * X + x];
            a = __dadd_rn(a, __dmul_rn(v, c_lo[j]));
            d = __dadd_rn(d, __dmul_rn(v, c_hi[j]));
        }
    }
    tmp[((long long)x * oy + o) * 2 + 0] = a;
    tmp[((long long)x * oy + o) * 2 + 1] = d;
}

// row pass of both column outputs, placed in the four quadrants
__global__ void k_wav_x(const double *__restrict__ tmp, int X, int Y, double *__restrict__ out) {
    const int ox = (X + 9) / 2, oy = (Y + 9) / 2, W = 2 * ox;
    const int u = blockIdx.x * blockDim.x + threadIdx.x, o = blockIdx.y * blockDim.y + threadIdx.y;
    if (u >= ox || o >= oy) return;
    const int i = 2 * u + 1;
    double a1 = 0, d1 = 0, a2 = 0, d2 = 0;
#pragma unroll
    for (int j = 0; j < 10; j++) {
        const int k = i - j;
        if (k >= 0 && k < X) {
            const double va = tmp[((long long)k * oy + o) * 2 + 0], vd = tmp[((long long)k * oy + o) * 2 + 1];
            a1 = __dadd_rn(a1, __dmul_rn(va, c_lo[j]));
            d1 = __dadd_rn(d1, __dmul_rn(va, c_hi[j]));
            a2 = __dadd_rn(a2, __dmul_rn(vd, c_lo[j]));
            d2 = __dadd_rn(d2, __dmul_rn(vd, c_hi[j]));
        }
    }
    out[(long long)o * W + u] = d2;
    out[(long long)(oy + o) * W + u] = a2;
    out[(long long)o * W + ox + u] = d1;
    out[(long long)(oy + o) * W + ox + u] = a1;
}

// Device address of the static array, looked up once per device with that
// device current (in host code its name is only a host-side stand-in).
std::mutex g_mu;
double *g_ptr[64] = {nullptr};

int scratch_for_current_device(double **out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return wc::set_err(WC_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= 64) return wc::set_err(WC_ERR_UNSUPPORTED, "device %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_wavelet_scratch);
        if (e != cudaSuccess || !p)
            return wc::set_err(WC_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
        g_ptr[dev] = (double *)p;
    }
    *out = g_ptr[dev];
    return WC_OK;
}

}  // namespace

extern "C" int wc_wavelet_noalloc(const double *d_in, int width, int height, double *d_out, void *stream) {
    if (!d_in || !d_out || width < 1 || height < 1) return wc::set_err(WC_ERR_ARG, "wc_wavelet_noalloc: bad arguments");
    const long long need = (long long)width * ((height + 9) / 2) * 2;
    if (need > kScratchDoubles)
        return wc::set_err(WC_ERR_ARG,
                           "wc_wavelet_noalloc: %d x %d needs %lld scratch doubles, the static scratch holds %lld "
                           "(inputs up to 1024 x 1024 fit)",
                           width, height, need, kScratchDoubles);
    double *scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const int ox = (width + 9) / 2, oy = (height + 9) / 2;
    const dim3 b(32, 8);
    k_wav_y<<<dim3((width + 31) / 32, (oy + 7) / 8), b, 0, st>>>(d_in, width, height, scratch);
    k_wav_x<<<dim3((ox + 31) / 32, (oy + 7) / 8), b, 0, st>>>(scratch, width, height, d_out);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return wc::set_err(WC_ERR_CUDA, "wc_wavelet_noalloc launch: %s", cudaGetErrorString(e));
    return WC_OK;
}
