/* TEST INFRASTRUCTURE ONLY: a stand-in for libtiff's header so the unmodified
 * reference src/cmatrix.cpp compiles here.  Its definitions
 * (oracle/ref_shim/tiff_stub.cpp) serve one in-memory image registered with
 * wcref_tiff_set, so ImageMatrix::LoadTIFF can read RGB and grayscale pixels
 * without files; with none registered every open fails.  Files themselves are
 * decoded in Python (tests/golden/tiffread.py). */
#ifndef WC_TIFF_STUB_H
#define WC_TIFF_STUB_H
#include <stddef.h>
typedef struct tiff_stub TIFF;
typedef long tsize_t;
typedef void (*TIFFErrorHandler)(const char *, const char *, void *);
#define TIFFTAG_IMAGEWIDTH 256
#define TIFFTAG_IMAGELENGTH 257
#define TIFFTAG_BITSPERSAMPLE 258
#define TIFFTAG_COMPRESSION 259
#define TIFFTAG_PHOTOMETRIC 262
#define TIFFTAG_SAMPLESPERPIXEL 277
#define TIFFTAG_PLANARCONFIG 284
#ifdef __cplusplus
extern "C" {
#endif
TIFF *TIFFOpen(const char *, const char *);
void TIFFClose(TIFF *);
int TIFFGetField(TIFF *, unsigned int, ...);
int TIFFSetField(TIFF *, unsigned int, ...);
int TIFFReadScanline(TIFF *, void *, unsigned int, unsigned short s = 0);
int TIFFWriteScanline(TIFF *, void *, unsigned int, unsigned short);
tsize_t TIFFScanlineSize(TIFF *);
unsigned short TIFFNumberOfDirectories(TIFF *);
TIFFErrorHandler TIFFSetWarningHandler(TIFFErrorHandler);
void *_TIFFmalloc(tsize_t);
void _TIFFfree(void *);
#ifdef __cplusplus
}
#endif
#endif
