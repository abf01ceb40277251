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
// The array's device address is looked up with the calling thread's current
// device on every call (a cheap query once the library's device code is
// loaded), so a cudaDeviceReset, which can move the array, never leaves a stale
// address behind.  The first call on a device loads the library's device code
// there; make that first call before any stream capture begins.
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

#include <algorithm>
#include <cstdio>

#include "../../include/wndcharm_gb300.h"
#include "kwavelet.cuh"

namespace wc {
int set_err(int code, const char *fmt, ...);
}

namespace {

// capacity of the static scratch, in doubles: enough for 1024 x 1024 inputs
// (1024 * floor((1024 + 9) / 2) * 2 = 1,056,768); 8.25 MiB per GPU.
constexpr long long kScratchDoubles = 1081344;
static __device__ __align__(256) double g_wavelet_scratch[kScratchDoubles];

// column pass: for every column x, approximation/detail along y into the
// scratch; rows o advance by the grid's y extent, so any height fits the grid
__global__ void k_wav_y(const double *__restrict__ in, int X, int Y, double *__restrict__ tmp) {
    const int oy = sym5_out(Y);
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= X) return;
    for (int o = blockIdx.y * blockDim.y + threadIdx.y; o < oy; o += gridDim.y * blockDim.y) {
        double a, d;
        sym5_col(in, X, Y, x, o, a, d);
        double *t = tmp + sym5_tmp_index(x, oy, o);
        t[0] = a;
        t[1] = d;
    }
}

// row pass of both column outputs, placed in the four quadrants
__global__ void k_wav_x(const double *__restrict__ tmp, int X, int Y, double *__restrict__ out) {
    const int ox = sym5_out(X), oy = sym5_out(Y);
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= ox) return;
    for (int o = blockIdx.y * blockDim.y + threadIdx.y; o < oy; o += gridDim.y * blockDim.y) {
        double a1, d1, a2, d2;
        sym5_row(tmp, X, oy, u, o, a1, d1, a2, d2);
        sym5_store(out, ox, oy, u, o, a1, d1, a2, d2);
    }
}

// Device address of the static array on the current device (in host code its
// name is only a host-side stand-in, never a device address).
int scratch_for_current_device(double **out) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_wavelet_scratch);
    if (e != cudaSuccess || !p)
        return wc::set_err(WC_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
    *out = (double *)p;
    return WC_OK;
}

}  // namespace

extern "C" int wc_wavelet_noalloc(const double *d_in, int width, int height, double *d_out, void *stream) {
    if (!d_in || !d_out || width < 1 || height < 1 || width > (1 << 28) || height > (1 << 28))
        return wc::set_err(WC_ERR_ARG, "wc_wavelet_noalloc: bad arguments");
    const long long need = (long long)width * ((height + 9) / 2) * 2;
    if (need > kScratchDoubles)
        return wc::set_err(WC_ERR_ARG,
                           "wc_wavelet_noalloc: %d x %d needs %lld scratch doubles, the static scratch holds %lld "
                           "(inputs up to 1024 x 1024 fit)",
                           width, height, need, kScratchDoubles);
    // an error left pending by an earlier, unrelated call is reported, not
    // taken (cleared) as this call's own
    cudaError_t e = cudaPeekAtLastError();
    if (e != cudaSuccess)
        return wc::set_err(WC_ERR_CUDA, "wc_wavelet_noalloc: a CUDA error from an earlier call is pending: %s",
                           cudaGetErrorString(e));
    double *scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const int ox = sym5_out(width), oy = sym5_out(height);
    const dim3 b(32, 8);
    const int gy = (int)std::min<long long>((oy + 7) / 8, 65535);
    k_wav_y<<<dim3((width + 31) / 32, gy), b, 0, st>>>(d_in, width, height, scratch);
    e = cudaGetLastError();
    if (e == cudaSuccess) {
        k_wav_x<<<dim3((ox + 31) / 32, gy), b, 0, st>>>(scratch, width, height, d_out);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return wc::set_err(WC_ERR_CUDA, "wc_wavelet_noalloc launch: %s", cudaGetErrorString(e));
    return WC_OK;
}
