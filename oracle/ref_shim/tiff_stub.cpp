// TEST INFRASTRUCTURE ONLY: definitions for the libtiff stand-in header
// (oracle/ref_shim/include/tiffio.h).  One in-memory image can be registered
// with wcref_tiff_set (row-major samples, interleaved when spp > 1, native
// byte order); TIFFOpen then serves it whatever the path, so the reference's
// unmodified ImageMatrix::LoadTIFF reads it as it would read a file.  With no
// image registered every open fails.
#include <cstdarg>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include "tiffio.h"

struct tiff_stub {
    const unsigned char *data;
    uint32_t w, h;
    uint16_t bits, spp;
};
static tiff_stub g_img = {nullptr, 0, 0, 0, 0};

extern "C" {
void wcref_tiff_set(const void *data, int w, int h, int bits, int spp) {
    g_img.data = (const unsigned char *)data;
    g_img.w = (uint32_t)w;
    g_img.h = (uint32_t)h;
    g_img.bits = (uint16_t)bits;
    g_img.spp = (uint16_t)spp;
}
TIFF *TIFFOpen(const char *, const char *) { return g_img.data ? &g_img : nullptr; }
void TIFFClose(TIFF *) {}
int TIFFGetField(TIFF *t, unsigned int tag, ...) {
    va_list ap;
    va_start(ap, tag);
    int ok = 1;
    switch (tag) {
        case TIFFTAG_IMAGEWIDTH: *va_arg(ap, uint32_t *) = t->w; break;
        case TIFFTAG_IMAGELENGTH: *va_arg(ap, uint32_t *) = t->h; break;
        case TIFFTAG_BITSPERSAMPLE: *va_arg(ap, uint16_t *) = t->bits; break;
        case TIFFTAG_SAMPLESPERPIXEL: *va_arg(ap, uint16_t *) = t->spp; break;
        default: ok = 0;
    }
    va_end(ap);
    return ok;
}
int TIFFSetField(TIFF *, unsigned int, ...) { return 0; }
tsize_t TIFFScanlineSize(TIFF *t) { return (tsize_t)t->w * t->spp * (t->bits / 8); }
int TIFFReadScanline(TIFF *t, void *buf, unsigned int row, unsigned short) {
    if (row >= t->h) return -1;
    const size_t n = (size_t)TIFFScanlineSize(t);
    std::memcpy(buf, t->data + n * row, n);
    return 1;
}
int TIFFWriteScanline(TIFF *, void *, unsigned int, unsigned short) { return -1; }
unsigned short TIFFNumberOfDirectories(TIFF *) { return 1; }
TIFFErrorHandler TIFFSetWarningHandler(TIFFErrorHandler h) { return h; }
void *_TIFFmalloc(tsize_t n) { return std::malloc(n > 0 ? (size_t)n : 1); }
void _TIFFfree(void *p) { std::free(p); }
}
