// png.cpp -- 8-bit PNG light-field images, as the reference reads and writes them through Qt.
//
// gsl_image_from_qimage (cocolib/cocolib/common/gsl_image.cpp:539-587) converts every channel to value / 255.0;
// gsl_image_to_qimage (:590-620) writes clamp(int(v * 255.0), 0, 255). Here: non-interlaced 8-bit grey, RGB,
// grey+alpha or RGBA PNGs are decoded with zlib (all five scanline filters), returned as planar RGB floats;
// the writer emits 8-bit RGB with filter 0. Without zlib at build time both entry points report LFRV_E_IO.
#include "lfrv.h"
#include "lfrv_internal.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#if defined(LFRV_HAVE_ZLIB)
#include <zlib.h>
#endif

namespace {

uint32_t be32(const uint8_t *p) { return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]; }

void put32(std::vector<uint8_t> &v, uint32_t x) {
    v.push_back((uint8_t)(x >> 24));
    v.push_back((uint8_t)(x >> 16));
    v.push_back((uint8_t)(x >> 8));
    v.push_back((uint8_t)x);
}

int paeth(int a, int b, int c) {
    const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    if (pa <= pb && pa <= pc) return a;
    return (pb <= pc) ? b : c;
}

}  // namespace

extern "C" int lfrv_png_read(const char *path, int *w, int *h, float *rgb, size_t capacity) {
    if (!path || !w || !h) return lfrv::fail(LFRV_E_ARG, "null argument");
#if !defined(LFRV_HAVE_ZLIB)
    (void)rgb;
    (void)capacity;
    return lfrv::fail(LFRV_E_IO, "%s: PNG support needs zlib, absent when this library was built", path);
#else
    FILE *f = std::fopen(path, "rb");
    if (!f) return lfrv::fail(LFRV_E_IO, "cannot open %s", path);
    std::vector<uint8_t> file;
    uint8_t buf[65536];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) file.insert(file.end(), buf, buf + got);
    std::fclose(f);
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    if (file.size() < 33 || std::memcmp(file.data(), sig, 8) != 0) return lfrv::fail(LFRV_E_FORMAT, "%s: not a PNG", path);
    uint32_t W = 0, H = 0;
    int depth = 0, ctype = -1, interlace = 0;
    std::vector<uint8_t> idat;
    size_t pos = 8;
    while (pos + 12 <= file.size()) {
        const uint32_t len = be32(&file[pos]);
        if (pos + 12 + (size_t)len > file.size()) return lfrv::fail(LFRV_E_FORMAT, "%s: truncated chunk", path);
        const uint8_t *type = &file[pos + 4], *data = &file[pos + 8];
        if (!std::memcmp(type, "IHDR", 4) && len >= 13) {
            W = be32(data);
            H = be32(data + 4);
            depth = data[8];
            ctype = data[9];
            interlace = data[12];
        } else if (!std::memcmp(type, "IDAT", 4)) {
            idat.insert(idat.end(), data, data + len);
        } else if (!std::memcmp(type, "IEND", 4)) {
            break;
        }
        pos += 12 + (size_t)len;
    }
    const int chans = ctype == 0 ? 1 : ctype == 2 ? 3 : ctype == 4 ? 2 : ctype == 6 ? 4 : 0;
    if (W == 0 || H == 0 || (uint64_t)W * H > (1ull << 28) || depth != 8 || chans == 0 || interlace != 0)
        return lfrv::fail(LFRV_E_FORMAT, "%s: only non-interlaced 8-bit grey/RGB/RGBA PNGs are supported", path);
    *w = (int)W;
    *h = (int)H;
    if (!rgb) return LFRV_OK;
    const size_t N = (size_t)W * H;
    if (capacity < 3 * N) return lfrv::fail(LFRV_E_ARG, "%s: buffer holds %zu floats, need %zu", path, capacity, 3 * N);
    const size_t stride = (size_t)W * chans;
    std::vector<uint8_t> raw((stride + 1) * H);
    uLongf rawlen = (uLongf)raw.size();
    if (uncompress(raw.data(), &rawlen, idat.data(), (uLong)idat.size()) != Z_OK || rawlen != raw.size())
        return lfrv::fail(LFRV_E_FORMAT, "%s: corrupt image data", path);
    std::vector<uint8_t> prev(stride, 0), cur(stride);
    for (uint32_t y = 0; y < H; ++y) {
        const uint8_t *line = &raw[y * (stride + 1)];
        const int filter = line[0];
        for (size_t i = 0; i < stride; ++i) {
            const int a = i >= (size_t)chans ? cur[i - chans] : 0, b = prev[i], c = i >= (size_t)chans ? prev[i - chans] : 0;
            int pred = 0;
            switch (filter) {
                case 0: pred = 0; break;
                case 1: pred = a; break;
                case 2: pred = b; break;
                case 3: pred = (a + b) / 2; break;
                case 4: pred = paeth(a, b, c); break;
                default: return lfrv::fail(LFRV_E_FORMAT, "%s: bad scanline filter %d", path, filter);
            }
            cur[i] = (uint8_t)(line[1 + i] + pred);
        }
        for (uint32_t x = 0; x < W; ++x) {
            const uint8_t *px = &cur[(size_t)x * chans];
            const int r = px[0], g = chans >= 3 ? px[1] : px[0], bb = chans >= 3 ? px[2] : px[0];
            const size_t o = (size_t)y * W + x;
            rgb[o] = (float)(r / 255.0);
            rgb[N + o] = (float)(g / 255.0);
            rgb[2 * N + o] = (float)(bb / 255.0);
        }
        std::swap(prev, cur);
    }
    return LFRV_OK;
#endif
}

extern "C" int lfrv_png_write(const char *path, int w, int h, const float *rgb) {
    if (!path || !rgb || w <= 0 || h <= 0) return lfrv::fail(LFRV_E_ARG, "bad arguments");
#if !defined(LFRV_HAVE_ZLIB)
    return lfrv::fail(LFRV_E_IO, "%s: PNG support needs zlib, absent when this library was built", path);
#else
    const size_t N = (size_t)w * h, stride = (size_t)w * 3;
    std::vector<uint8_t> raw((stride + 1) * h);
    for (int y = 0; y < h; ++y) {
        raw[y * (stride + 1)] = 0;
        for (int x = 0; x < w; ++x)
            for (int c = 0; c < 3; ++c) {
                const double v = rgb[c * N + (size_t)y * w + x] * 255.0;
                int q = (int)v;  // int( v * 255.0 ) clamped, as gsl_image_to_qimage
                q = q < 0 ? 0 : (q > 255 ? 255 : q);
                raw[y * (stride + 1) + 1 + (size_t)x * 3 + c] = (uint8_t)q;
            }
    }
    uLongf zlen = compressBound((uLong)raw.size());
    std::vector<uint8_t> z(zlen);
    if (compress(z.data(), &zlen, raw.data(), (uLong)raw.size()) != Z_OK) return lfrv::fail(LFRV_E_IO, "deflate failed");
    std::vector<uint8_t> out = {137, 80, 78, 71, 13, 10, 26, 10};
    auto chunk = [&](const char *type, const uint8_t *data, size_t len) {
        put32(out, (uint32_t)len);
        const size_t start = out.size();
        out.insert(out.end(), type, type + 4);
        out.insert(out.end(), data, data + len);
        const uLong crc = crc32(0L, out.data() + start, (uInt)(len + 4));
        put32(out, (uint32_t)crc);
    };
    std::vector<uint8_t> ihdr;
    put32(ihdr, (uint32_t)w);
    put32(ihdr, (uint32_t)h);
    ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0});
    chunk("IHDR", ihdr.data(), ihdr.size());
    chunk("IDAT", z.data(), zlen);
    chunk("IEND", nullptr, 0);
    FILE *f = std::fopen(path, "wb");
    if (!f) return lfrv::fail(LFRV_E_IO, "cannot create %s", path);
    const bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
    std::fclose(f);
    return ok ? LFRV_OK : lfrv::fail(LFRV_E_IO, "write failed: %s", path);
#endif
}
