// TIFF directory parsing shared by the host reader (tiff.cpp) and the device
// decoder (k_tiff.cu).
#pragma once
#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <vector>

namespace wc {

// One image directory, parsed and checked: the file's bytes, the layout and
// the strips.
struct TiffFile {
    std::vector<uint8_t> b;
    bool le = true;
    uint32_t w = 0, h = 0, bps = 1, comp = 1, spp = 1, rps = 0xffffffffu, pred = 1;
    std::vector<uint32_t> offs, counts;
    size_t es() const { return bps / 8; }
    size_t row() const { return (size_t)w * spp * es(); }
    size_t strip_rows(size_t s) const { return std::min<size_t>(rps, h - std::min<size_t>(h, s * (size_t)rps)); }
};

// reads and checks the file (WC_OK or a WC_ERR_* status with the message set)
int parse_tiff(const char *path, TiffFile &t);
// the stored samples of every row in file order, strips decoded on the host
int host_strips(const char *path, const TiffFile &t, std::vector<uint8_t> &raw);
// one LZW strip decoded on the host (a serial bit stream)
bool tiff_lzw_strip(const uint8_t *src, size_t n, std::vector<uint8_t> &out, size_t want);

}  // namespace wc
