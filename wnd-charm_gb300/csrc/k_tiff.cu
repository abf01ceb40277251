// TIFF strips decoded on the GPU for ImageMatrix::LoadTIFF's images
// (src/cmatrix.cpp:85-203; the layout rules are those of the host reader,
// tiff.cpp, from the TIFF 6.0 specification).  The host reads each file and
// its directory and copies the strips to the GPU as stored; the GPU expands
// PackBits strips (one thread per strip: a run's length is in its header, so a
// strip is a serial walk, and strips and images run in parallel), swaps byte
// order, undoes the horizontal-differencing predictor and writes native
// uint8 / uint16 samples, interleaved for RGB.  LZW strips are a serial bit
// stream with a growing code table: the host decodes those and they travel as
// stored bytes.  The decoded images stay in device memory for
// wc_extract_batch / wc_extract_samples (on_device descriptors).
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "engine.h"
#include "tiff_internal.h"

namespace wc {

struct TStrip {
    long long src, dst;  // in the staged bytes; in the image's decoded bytes (absolute in raw)
    int nsrc, ndst;      // stored bytes; decoded bytes the strip must give
    int packbits;
};
struct TImg {
    long long raw, out;  // the image's decoded stored bytes; its samples in the output buffer
    int w, h, spp, es, le, pred;
};

// one CTA per strip; produced[s]: decoded bytes, -1 for a run header without its byte
__global__ void k_tiff_strips(const uint8_t *__restrict__ stage, const TStrip *__restrict__ strips,
                              uint8_t *__restrict__ raw, int *__restrict__ produced) {
    const TStrip S = strips[blockIdx.x];
    if (!S.packbits) {
        const int n = min(S.nsrc, S.ndst);
        for (int i = threadIdx.x; i < n; i += blockDim.x) raw[S.dst + i] = stage[S.src + i];
        if (threadIdx.x == 0) produced[blockIdx.x] = n;
        return;
    }
    if (threadIdx.x != 0) return;
    const uint8_t *src = stage + S.src;
    uint8_t *dst = raw + S.dst;
    int i = 0, o = 0;
    bool bad = false;
    while (i < S.nsrc && o < S.ndst) {
        const int c = (int)(int8_t)src[i++];
        if (c >= 0) {  // c + 1 literal bytes
            for (int k = 0; k <= c && i < S.nsrc && o < S.ndst; k++) dst[o++] = src[i++];
        } else if (c != -128) {  // 1 - c copies of the next byte; -128 is a no-op
            if (i >= S.nsrc) {
                bad = true;
                break;
            }
            const uint8_t v = src[i++];
            for (int k = 0; k < 1 - c && o < S.ndst; k++) dst[o++] = v;
        }
    }
    produced[blockIdx.x] = bad ? -1 : o;
}

// image blockIdx.y: stored samples to native ones; without the predictor one
// thread per sample, with it one thread per row (each sample adds the same
// sample of the pixel to its left, modulo 2^bits)
__global__ void k_tiff_samples(const uint8_t *__restrict__ raw, const TImg *__restrict__ imgs,
                               uint8_t *__restrict__ out) {
    const TImg I = imgs[blockIdx.y];
    const long long ns = (long long)I.w * I.spp;
    const uint8_t *s = raw + I.raw;
    if (I.pred != 2) {
        const long long n = ns * I.h;
        for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
             k += (long long)gridDim.x * blockDim.x) {
            if (I.es == 1) out[I.out + k] = s[k];
            else {
                const uint16_t v = I.le ? (uint16_t)(s[2 * k] | (s[2 * k + 1] << 8)) : (uint16_t)((s[2 * k] << 8) | s[2 * k + 1]);
                ((uint16_t *)(out + I.out))[k] = v;
            }
        }
        return;
    }
    for (long long y = blockIdx.x * (long long)blockDim.x + threadIdx.x; y < I.h; y += (long long)gridDim.x * blockDim.x) {
        const uint8_t *r = s + y * ns * I.es;
        if (I.es == 1) {
            uint8_t *d = out + I.out + y * ns;
            for (long long x = 0; x < ns; x++) d[x] = (uint8_t)(r[x] + (x >= I.spp ? d[x - I.spp] : 0));
        } else {
            uint16_t *d = (uint16_t *)(out + I.out) + y * ns;
            for (long long x = 0; x < ns; x++) {
                const uint16_t v = I.le ? (uint16_t)(r[2 * x] | (r[2 * x + 1] << 8)) : (uint16_t)((r[2 * x] << 8) | r[2 * x + 1]);
                d[x] = (uint16_t)(v + (x >= I.spp ? d[x - I.spp] : 0));
            }
        }
    }
}

}  // namespace wc

using namespace wc;

static int tiff_plan(const char *const *paths, int n, std::vector<TiffFile> &files, std::vector<long long> &out_off,
                     long long &out_bytes) {
    files.assign(n, TiffFile());
    out_off.assign(n, 0);
    out_bytes = 0;
    for (int i = 0; i < n; i++) {
        if (!paths[i]) return set_err(WC_ERR_ARG, "wc_tiff_read_device: null path %d", i);
        int rc = parse_tiff(paths[i], files[i]);
        if (rc) return rc;
        out_off[i] = out_bytes;
        out_bytes += ((long long)files[i].row() * files[i].h + 255) & ~255LL;
    }
    return WC_OK;
}

extern "C" int wc_tiff_device_bytes(const char *const *paths, int n, long long *bytes) {
    if (!paths || n < 1 || !bytes) return set_err(WC_ERR_ARG, "wc_tiff_device_bytes: bad arguments");
    std::vector<TiffFile> files;
    std::vector<long long> off;
    return tiff_plan(paths, n, files, off, *bytes);
}

extern "C" int wc_tiff_read_device(wc_engine *E, const char *const *paths, int n, void *d_pixels, long long capacity,
                                   wc_image_desc *descs) {
    if (!E || !paths || n < 1 || n > 65535 || !d_pixels || !descs)
        return set_err(WC_ERR_ARG, "wc_tiff_read_device: bad arguments (1..65535 files)");
    if ((uintptr_t)d_pixels % 256)
        return set_err(WC_ERR_ARG, "wc_tiff_read_device: the output buffer must be 256-byte aligned");
    std::lock_guard<std::mutex> lk(E->mu);
    CK(cudaSetDevice(E->dev));
    std::vector<TiffFile> files;
    std::vector<long long> out_off;
    long long out_bytes = 0;
    int rc = tiff_plan(paths, n, files, out_off, out_bytes);
    if (rc) return rc;
    if (out_bytes > capacity)
        return set_err(WC_ERR_ARG, "wc_tiff_read_device: %lld bytes needed, the buffer holds %lld", out_bytes, capacity);
    // the strips as stored (LZW ones decoded here), their places, the images
    std::vector<uint8_t> stage;
    std::vector<TStrip> strips;
    std::vector<TImg> imgs(n);
    long long raw_bytes = 0;
    for (int i = 0; i < n; i++) {
        const TiffFile &t = files[i];
        const size_t row = t.row();
        imgs[i] = TImg{raw_bytes, out_off[i], (int)t.w, (int)t.h, (int)t.spp, (int)t.es(), t.le ? 1 : 0, (int)t.pred};
        size_t covered = 0;
        for (size_t s = 0; s < t.offs.size() && covered < t.h; s++) {
            const size_t rows = t.strip_rows(s), want = rows * row;
            const uint8_t *src = t.b.data() + t.offs[s];
            TStrip S{(long long)stage.size(), raw_bytes + (long long)(covered * row), 0, (int)want, t.comp == 32773};
            if (t.comp == 5) {
                std::vector<uint8_t> dec;
                if (!tiff_lzw_strip(src, t.counts[s], dec, want))
                    return set_err(WC_ERR_IO, "'%s': corrupt strip %zu", paths[i], s);
                if (dec.size() < want) return set_err(WC_ERR_IO, "'%s': strip %zu too short", paths[i], s);
                stage.insert(stage.end(), dec.begin(), dec.begin() + want);
                S.nsrc = (int)want;
            } else {
                if (t.counts[s] > (1u << 30)) return set_err(WC_ERR_UNSUPPORTED, "'%s': strip %zu over 1 GiB", paths[i], s);
                stage.insert(stage.end(), src, src + t.counts[s]);
                S.nsrc = (int)t.counts[s];
            }
            strips.push_back(S);
            covered += rows;
        }
        if (covered < t.h) return set_err(WC_ERR_IO, "'%s': image data too short", paths[i]);
        raw_bytes += ((long long)row * t.h + 255) & ~255LL;
    }
    const size_t ns = strips.size();
    const size_t o_raw = (stage.size() + 255) & ~(size_t)255, o_str = o_raw + (((size_t)raw_bytes + 255) & ~(size_t)255);
    const size_t o_img = o_str + ((ns * sizeof(TStrip) + 255) & ~(size_t)255);
    const size_t o_prod = o_img + ((n * sizeof(TImg) + 255) & ~(size_t)255), total = o_prod + ns * sizeof(int) + 256;
    if ((rc = E->tiffbuf.ensure(total))) return rc;
    char *d = (char *)E->tiffbuf.p;
    cudaStream_t st = E->st;
    CK(cudaMemcpyAsync(d, stage.data(), stage.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d + o_str, strips.data(), ns * sizeof(TStrip), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d + o_img, imgs.data(), n * sizeof(TImg), cudaMemcpyHostToDevice, st));
    E->launches += 2;
    k_tiff_strips<<<(unsigned)ns, 256, 0, st>>>((const uint8_t *)d, (const TStrip *)(d + o_str), (uint8_t *)(d + o_raw),
                                                 (int *)(d + o_prod));
    k_tiff_samples<<<dim3(64, n), 256, 0, st>>>((const uint8_t *)(d + o_raw), (const TImg *)(d + o_img),
                                                (uint8_t *)d_pixels);
    CK(cudaGetLastError());
    std::vector<int> produced(ns);
    CK(cudaMemcpyAsync(produced.data(), d + o_prod, ns * sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    size_t k = 0;
    for (int i = 0; i < n; i++) {
        const TiffFile &t = files[i];
        size_t covered = 0;
        for (size_t s = 0; s < t.offs.size() && covered < t.h; s++, k++) {
            if (produced[k] < 0) return set_err(WC_ERR_IO, "'%s': corrupt strip %zu", paths[i], s);
            if (produced[k] < strips[k].ndst) return set_err(WC_ERR_IO, "'%s': strip %zu too short", paths[i], s);
            covered += t.strip_rows(s);
        }
        const int rgb = t.spp == 3;
        descs[i] = wc_image_desc{(char *)d_pixels + out_off[i], t.es() == 1 ? (rgb ? WC_RGB8 : WC_U8) : (rgb ? WC_RGB16 : WC_U16),
                                 (int)t.w, (int)t.h, (int)t.bps, 1};
    }
    return WC_OK;
}
