// TIFF reading for the images wndchrm opens (ImageMatrix::LoadTIFF,
// src/cmatrix.cpp:85-203, which goes through libtiff): one image directory,
// one sample per pixel (grayscale) or three interleaved (RGB, which LoadTIFF
// turns into a gray and an HSV plane), 8 or 16 bits, strips stored
// uncompressed, LZW (with or without the horizontal-differencing predictor) or
// PackBits, either byte order.  Pixel values are the stored samples (LoadTIFF
// ignores the photometric interpretation).  Written from the TIFF 6.0
// specification.
#include <cstdint>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/wndcharm_gb300.h"
#include "tiff_internal.h"

namespace wc {
int set_err(int code, const char *fmt, ...);
}

namespace {

struct TiffImage {
    int w = 0, h = 0, bits = 0, spp = 1;
    std::vector<uint8_t> pix;  // row-major, native-order uint8 / uint16, samples interleaved
};

struct Reader {
    const std::vector<uint8_t> &b;
    bool le;
    bool ok = true;
    uint32_t u16(size_t o) {
        if (o + 2 > b.size()) { ok = false; return 0; }
        return le ? (b[o] | (b[o + 1] << 8)) : ((b[o] << 8) | b[o + 1]);
    }
    uint32_t u32(size_t o) {
        if (o + 4 > b.size()) { ok = false; return 0; }
        return le ? (uint32_t)b[o] | ((uint32_t)b[o + 1] << 8) | ((uint32_t)b[o + 2] << 16) | ((uint32_t)b[o + 3] << 24)
                  : ((uint32_t)b[o] << 24) | ((uint32_t)b[o + 1] << 16) | ((uint32_t)b[o + 2] << 8) | (uint32_t)b[o + 3];
    }
};

// TIFF LZW: codes of 9..12 bits, most significant bit first, Clear = 256,
// EndOfInformation = 257, code width grows one code early.
bool lzw_decode(const uint8_t *src, size_t n, std::vector<uint8_t> &out, size_t want) {
    std::vector<uint32_t> start(4096), len(4096);
    std::vector<uint8_t> dict;
    dict.reserve(1 << 16);
    auto reset = [&]() {
        dict.resize(256);
        for (int i = 0; i < 256; i++) { dict[i] = (uint8_t)i; start[i] = i; len[i] = 1; }
    };
    reset();
    int next = 258, width = 9;
    uint64_t buf = 0;
    int bits = 0;
    size_t pos = 0;
    int prev = -1;
    while (out.size() < want) {
        while (bits < width && pos < n) {
            buf = (buf << 8) | src[pos++];
            bits += 8;
        }
        if (bits < width) break;
        const int code = (int)((buf >> (bits - width)) & ((1u << width) - 1));
        bits -= width;
        if (code == 257) break;
        if (code == 256) {
            reset();
            next = 258;
            width = 9;
            prev = -1;
            continue;
        }
        if (prev < 0) {
            if (code > 255) return false;
            out.push_back((uint8_t)code);
            prev = code;
            continue;
        }
        uint32_t s, l;
        if (code < next) {
            s = start[code];
            l = len[code];
            const uint8_t first = dict[s];
            if (next < 4096) {  // new entry: prev + first byte of this one
                start[next] = (uint32_t)dict.size();
                len[next] = len[prev] + 1;
                for (uint32_t k = 0; k < len[prev]; k++) dict.push_back(dict[start[prev] + k]);
                dict.push_back(first);
                next++;
            }
        } else if (code == next && next < 4096) {  // the entry being defined: prev + first byte of prev
            start[next] = (uint32_t)dict.size();
            len[next] = len[prev] + 1;
            for (uint32_t k = 0; k < len[prev]; k++) dict.push_back(dict[start[prev] + k]);
            dict.push_back(dict[start[prev]]);
            s = start[next];
            l = len[next];
            next++;
        } else {
            return false;
        }
        for (uint32_t k = 0; k < l; k++) out.push_back(dict[s + k]);
        prev = code;
        if (next + 1 >= (1 << width) && width < 12) width++;
    }
    return true;
}

bool packbits_decode(const uint8_t *src, size_t n, std::vector<uint8_t> &out, size_t want) {
    size_t i = 0;
    while (i < n && out.size() < want) {
        const int c = (int8_t)src[i++];
        if (c >= 0) {
            for (int k = 0; k <= c && i < n; k++) out.push_back(src[i++]);
        } else if (c != -128) {
            if (i >= n) return false;
            for (int k = 0; k < 1 - c; k++) out.push_back(src[i]);
            i++;
        }
    }
    return true;
}

}  // namespace

namespace wc {

int parse_tiff(const char *path, TiffFile &t) {
    FILE *f = fopen(path, "rb");
    if (!f) return wc::set_err(WC_ERR_IO, "cannot open '%s'", path);
    std::vector<uint8_t> &b = t.b;
    b.clear();
    uint8_t chunk[1 << 16];
    size_t got;
    while ((got = fread(chunk, 1, sizeof chunk, f)) > 0) b.insert(b.end(), chunk, chunk + got);
    fclose(f);
    if (b.size() < 8 || !((b[0] == 'I' && b[1] == 'I') || (b[0] == 'M' && b[1] == 'M')))
        return wc::set_err(WC_ERR_IO, "'%s' is not a TIFF file", path);
    Reader r{b, b[0] == 'I'};
    t.le = r.le;
    if (r.u16(2) != 42) return wc::set_err(WC_ERR_IO, "'%s': not a classic TIFF (BigTIFF is not supported)", path);
    const uint32_t ifd = r.u32(4);
    const uint32_t nent = r.u16(ifd);
    if (!r.ok) return wc::set_err(WC_ERR_IO, "'%s': truncated header", path);
    uint32_t planar = 1;
    bool tiled = false;
    auto values = [&](size_t e, std::vector<uint32_t> &v) {
        const uint32_t type = r.u16(e + 2), cnt = r.u32(e + 4);
        if (cnt > b.size()) {  // a count no file of this size can hold
            r.ok = false;
            v.clear();
            return;
        }
        const size_t sz = type == 3 ? 2 : type == 4 ? 4 : 1;
        const size_t at = sz * cnt <= 4 ? e + 8 : r.u32(e + 8);
        v.resize(cnt);
        for (uint32_t k = 0; k < cnt; k++)
            v[k] = type == 3 ? r.u16(at + 2 * k) : type == 4 ? r.u32(at + 4 * k) : (at + k < b.size() ? b[at + k] : 0);
    };
    for (uint32_t k = 0; k < nent; k++) {
        const size_t e = ifd + 2 + 12 * (size_t)k;
        const uint32_t tag = r.u16(e);
        std::vector<uint32_t> v;
        values(e, v);
        if (v.empty()) continue;
        switch (tag) {
            case 256: t.w = v[0]; break;
            case 257: t.h = v[0]; break;
            case 258: t.bps = v[0]; break;
            case 259: t.comp = v[0]; break;
            case 273: t.offs = v; break;
            case 277: t.spp = v[0]; break;
            case 278: t.rps = v[0]; break;
            case 279: t.counts = v; break;
            case 284: planar = v[0]; break;
            case 317: t.pred = v[0]; break;
            case 322: tiled = true; break;
            default: break;
        }
    }
    const uint32_t next_ifd = r.u32(ifd + 2 + 12 * (size_t)nent);
    if (!r.ok) return wc::set_err(WC_ERR_IO, "'%s': truncated directory", path);
    if (next_ifd != 0) return wc::set_err(WC_ERR_UNSUPPORTED, "'%s': more than one image directory", path);
    if (t.bps != 8 && t.bps != 16)
        return wc::set_err(WC_ERR_UNSUPPORTED, "'%s': %u bits per sample (8 or 16 only)", path, t.bps);
    if ((t.spp != 1 && t.spp != 3) || (t.spp == 3 && planar != 1))
        return wc::set_err(WC_ERR_UNSUPPORTED, "'%s': %u samples per pixel, planar configuration %u (grayscale or "
                           "interleaved RGB only)", path, t.spp, planar);
    if (tiled) return wc::set_err(WC_ERR_UNSUPPORTED, "'%s': tiled TIFF", path);
    if (t.comp != 1 && t.comp != 5 && t.comp != 32773)
        return wc::set_err(WC_ERR_UNSUPPORTED, "'%s': compression %u (none, LZW or PackBits only)", path, t.comp);
    if (t.w == 0 || t.h == 0 || t.offs.empty() || t.offs.size() != t.counts.size())
        return wc::set_err(WC_ERR_IO, "'%s': missing image size or strips", path);
    if ((unsigned long long)t.w * t.h > (1ull << 28) || t.w > 32768 || t.h > 32768)
        return wc::set_err(WC_ERR_UNSUPPORTED, "'%s': %u x %u is larger than this build reads", path, t.w, t.h);
    if (t.rps > t.h) t.rps = t.h;
    if (t.rps == 0) return wc::set_err(WC_ERR_IO, "'%s': zero rows per strip", path);
    for (size_t s = 0; s < t.offs.size(); s++)
        if ((size_t)t.offs[s] + t.counts[s] > b.size())
            return wc::set_err(WC_ERR_IO, "'%s': strip %zu past the end", path, s);
    return WC_OK;
}

// the stored samples of rows [0, h) in file order (strips decoded on the host)
int host_strips(const char *path, const TiffFile &t, std::vector<uint8_t> &raw) {
    const size_t row = t.row(), total = row * t.h;
    raw.clear();
    raw.reserve(total);
    for (size_t s = 0; s < t.offs.size() && raw.size() < total; s++) {
        const size_t rows = t.strip_rows(s);
        const size_t want = raw.size() + rows * row;
        const uint8_t *src = t.b.data() + t.offs[s];
        if (t.comp == 1) {
            raw.insert(raw.end(), src, src + std::min<size_t>(t.counts[s], rows * row));
        } else {
            std::vector<uint8_t> dec;
            const bool good = t.comp == 5 ? lzw_decode(src, t.counts[s], dec, rows * row)
                                          : packbits_decode(src, t.counts[s], dec, rows * row);
            if (!good) return wc::set_err(WC_ERR_IO, "'%s': corrupt strip %zu", path, s);
            raw.insert(raw.end(), dec.begin(), dec.begin() + std::min(dec.size(), rows * row));
        }
        if (raw.size() < want) return wc::set_err(WC_ERR_IO, "'%s': strip %zu too short", path, s);
    }
    if (raw.size() < total) return wc::set_err(WC_ERR_IO, "'%s': image data too short", path);
    return WC_OK;
}

bool tiff_lzw_strip(const uint8_t *src, size_t n, std::vector<uint8_t> &out, size_t want) {
    return lzw_decode(src, n, out, want);
}

}  // namespace wc

namespace {

int read_tiff(const char *path, TiffImage &img) {
    wc::TiffFile t;
    int rc = wc::parse_tiff(path, t);
    if (rc) return rc;
    std::vector<uint8_t> raw;
    if ((rc = wc::host_strips(path, t, raw))) return rc;
    const size_t es = t.es(), row = t.row(), total = row * t.h, spp = t.spp;
    img.w = (int)t.w;
    img.h = (int)t.h;
    img.bits = (int)t.bps;
    img.spp = (int)t.spp;
    img.pix.assign(total, 0);
    const size_t ns = (size_t)t.w * spp;  // samples per row; the predictor differences each sample with its left neighbour
    for (size_t y = 0; y < t.h; y++) {
        const uint8_t *s = raw.data() + y * row;
        if (es == 1) {
            uint8_t *d = img.pix.data() + y * row;
            memcpy(d, s, row);
            if (t.pred == 2)
                for (size_t x = spp; x < ns; x++) d[x] = (uint8_t)(d[x] + d[x - spp]);
        } else {
            uint16_t *d = (uint16_t *)(img.pix.data() + y * row);
            for (size_t x = 0; x < ns; x++)
                d[x] = t.le ? (uint16_t)(s[2 * x] | (s[2 * x + 1] << 8)) : (uint16_t)((s[2 * x] << 8) | s[2 * x + 1]);
            if (t.pred == 2)
                for (size_t x = spp; x < ns; x++) d[x] = (uint16_t)(d[x] + d[x - spp]);
        }
    }
    return WC_OK;
}

}  // namespace

extern "C" {

int wc_tiff_info(const char *path, int *width, int *height, int *bits) {
    if (!path || !width || !height || !bits) return wc::set_err(WC_ERR_ARG, "wc_tiff_info: null argument");
    TiffImage img;
    const int r = read_tiff(path, img);
    if (r) return r;
    *width = img.w;
    *height = img.h;
    *bits = img.bits;
    return WC_OK;
}

int wc_tiff_layout(const char *path, int *width, int *height, int *bits, int *samples) {
    if (!path || !width || !height || !bits || !samples) return wc::set_err(WC_ERR_ARG, "wc_tiff_layout: null argument");
    TiffImage img;
    const int r = read_tiff(path, img);
    if (r) return r;
    *width = img.w;
    *height = img.h;
    *bits = img.bits;
    *samples = img.spp;
    return WC_OK;
}

int wc_tiff_read(const char *path, void *pixels, long long capacity) {
    if (!path || !pixels) return wc::set_err(WC_ERR_ARG, "wc_tiff_read: null argument");
    TiffImage img;
    const int r = read_tiff(path, img);
    if (r) return r;
    if ((long long)img.pix.size() > capacity)
        return wc::set_err(WC_ERR_ARG, "wc_tiff_read: buffer of %lld bytes for an image of %zu", capacity, img.pix.size());
    memcpy(pixels, img.pix.data(), img.pix.size());
    return WC_OK;
}

}  // extern "C"
