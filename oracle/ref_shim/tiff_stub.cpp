// TEST INFRASTRUCTURE ONLY: definitions for the libtiff stand-in header
// (oracle/ref_shim/include/tiffio.h).  Opening always fails.
#include <cstdlib>
#include "tiffio.h"
extern "C" {
TIFF *TIFFOpen(const char *, const char *) { return nullptr; }
void TIFFClose(TIFF *) {}
int TIFFGetField(TIFF *, unsigned int, ...) { return 0; }
int TIFFSetField(TIFF *, unsigned int, ...) { return 0; }
int TIFFReadScanline(TIFF *, void *, unsigned int, unsigned short) { return -1; }
int TIFFWriteScanline(TIFF *, void *, unsigned int, unsigned short) { return -1; }
tsize_t TIFFScanlineSize(TIFF *) { return 0; }
unsigned short TIFFNumberOfDirectories(TIFF *) { return 0; }
TIFFErrorHandler TIFFSetWarningHandler(TIFFErrorHandler h) { return h; }
void *_TIFFmalloc(tsize_t n) { return std::malloc(n > 0 ? (size_t)n : 1); }
void _TIFFfree(void *p) { std::free(p); }
}
