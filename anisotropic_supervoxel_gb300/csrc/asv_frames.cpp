// asv_frames.cpp -- frame files of any supported format for the Render::run
// frame loop (GPU-AS/Render.cpp:151-157, 229-238: cv::imread(path, 1) of
// every file of the sorted folder).  The format is taken from the file's
// first bytes: PNG (asv_png.cpp), BMP and binary PNM (P5 grey, P6 colour).
// Pixels come out as imread(path, 1) gives them: 8-bit BGR, top row first,
// grey replicated, alpha dropped, 16-bit samples reduced to their high byte.
//
// BMP: the Windows bitmap layout (14-byte file header, then an info header
// of 40 bytes or one of its longer versions): 1/4/8-bit palette images,
// 16-bit (5-5-5, or bit fields), 24-bit and 32-bit (BI_RGB or bit fields),
// rows padded to 4 bytes, bottom-up unless the height is negative.  RLE
// compression is refused as unsupported.
#include "asv_host.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace {

enum { F_OK = 0, F_BAD_ARG = -1, F_IO = -2, F_FORMAT = -3, F_UNSUPPORTED = -4, F_SIZE = -5 };
constexpr uint64_t kMaxPixels = 1ull << 28;

int read_all(const char *path, std::vector<uint8_t> &data)
{
    FILE *f = std::fopen(path, "rb");
    if (!f) return F_IO;
    data.clear();
    uint8_t buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) data.insert(data.end(), buf, buf + n);
    const bool err = std::ferror(f) != 0;
    std::fclose(f);
    return err ? F_IO : F_OK;
}

int read_head(const char *path, std::vector<uint8_t> &data, size_t cap)
{
    FILE *f = std::fopen(path, "rb");
    if (!f) return F_IO;
    data.resize(cap);
    const size_t n = std::fread(data.data(), 1, cap, f);
    std::fclose(f);
    data.resize(n);
    return F_OK;
}

uint32_t le16(const uint8_t *p) { return (uint32_t)p[0] | ((uint32_t)p[1] << 8); }
uint32_t le32(const uint8_t *p) { return le16(p) | (le16(p + 2) << 16); }

enum Kind { K_NONE, K_PNG, K_BMP, K_PNM };

Kind sniff(const std::vector<uint8_t> &d)
{
    static const uint8_t png[8] = { 0x89, 'P', 'N', 'G', 0x0d, 0x0a, 0x1a, 0x0a };
    if (d.size() >= 8 && std::memcmp(d.data(), png, 8) == 0) return K_PNG;
    if (d.size() >= 2 && d[0] == 'B' && d[1] == 'M') return K_BMP;
    if (d.size() >= 2 && d[0] == 'P' && (d[1] == '5' || d[1] == '6')) return K_PNM;
    return K_NONE;
}

// ---- BMP -----------------------------------------------------------------
struct Bmp {
    int W = 0, H = 0;
    bool top_down = false;
    int bpp = 0;
    uint32_t comp = 0, off = 0, hdr = 0;
    uint32_t mask[3] = { 0, 0, 0 };
    int ncolors = 0;
};

int bmp_header(const std::vector<uint8_t> &d, Bmp &b)
{
    if (d.size() < 14 + 40) return F_FORMAT;
    b.off = le32(&d[10]);
    b.hdr = le32(&d[14]);
    if (b.hdr < 40 || 14 + (size_t)b.hdr > d.size()) return F_FORMAT;
    const int32_t w = (int32_t)le32(&d[18]), h = (int32_t)le32(&d[22]);
    if (le16(&d[26]) != 1) return F_FORMAT;                     // planes
    b.bpp = (int)le16(&d[28]);
    b.comp = le32(&d[30]);
    b.ncolors = (int)le32(&d[46]);
    if (w <= 0 || h == 0 || h == INT32_MIN) return F_FORMAT;
    b.W = w;
    b.top_down = h < 0;
    b.H = h < 0 ? -h : h;
    if ((uint64_t)b.W * (uint64_t)b.H > kMaxPixels) return F_UNSUPPORTED;
    if (b.comp == 1 || b.comp == 2 || b.comp > 3) return F_UNSUPPORTED;   // RLE8, RLE4, JPEG/PNG payloads
    if (b.bpp != 1 && b.bpp != 4 && b.bpp != 8 && b.bpp != 16 && b.bpp != 24 && b.bpp != 32) return F_FORMAT;
    if (b.comp == 3) {                                          // BI_BITFIELDS: masks after a 40-byte header
        if (b.bpp != 16 && b.bpp != 32) return F_FORMAT;
        if (14 + 40 + 12 > d.size()) return F_FORMAT;
        for (int k = 0; k < 3; k++) b.mask[k] = le32(&d[14 + 40 + 4 * k]);
    } else if (b.bpp == 16) {                                   // BI_RGB 16-bit: 5-5-5
        b.mask[0] = 0x7c00; b.mask[1] = 0x03e0; b.mask[2] = 0x001f;
    } else if (b.bpp == 32) {
        b.mask[0] = 0x00ff0000; b.mask[1] = 0x0000ff00; b.mask[2] = 0x000000ff;
    }
    if (b.bpp <= 8) {
        if (b.ncolors <= 0 || b.ncolors > (1 << b.bpp)) b.ncolors = 1 << b.bpp;
        if (14 + (size_t)b.hdr + 4 * (size_t)b.ncolors > d.size()) return F_FORMAT;
    }
    return F_OK;
}

// a channel from a bit-field mask as 8 bits: a narrower field shifted up
// (5 bits -> v << 3), a wider one down to its top 8 bits
uint8_t field(uint32_t px, uint32_t mask)
{
    if (!mask) return 0;
    int shift = 0;
    while (!((mask >> shift) & 1u)) shift++;
    int bits = 0;
    while (shift + bits < 32 && ((mask >> (shift + bits)) & 1u)) bits++;
    const uint32_t v = (px & mask) >> shift;
    return (uint8_t)(bits >= 8 ? v >> (bits - 8) : v << (8 - bits));
}

int bmp_decode(const std::vector<uint8_t> &d, int W, int H, uint8_t *bgr)
{
    Bmp b;
    int st = bmp_header(d, b);
    if (st != F_OK) return st;
    if (b.W != W || b.H != H) return F_SIZE;
    const size_t stride = (((size_t)b.W * b.bpp + 31) / 32) * 4;
    if ((size_t)b.off + stride * b.H > d.size()) return F_FORMAT;
    const uint8_t *pal = d.data() + 14 + b.hdr;
    for (int r = 0; r < b.H; r++) {
        const int y = b.top_down ? r : b.H - 1 - r;              // output row (top first)
        const uint8_t *row = d.data() + b.off + stride * r;
        uint8_t *o = bgr + (size_t)y * W * 3;
        for (int x = 0; x < b.W; x++) {
            if (b.bpp <= 8) {
                const int per = 8 / b.bpp;
                const int byte = row[x / per];
                const int idx = (byte >> (8 - b.bpp * (x % per + 1))) & ((1 << b.bpp) - 1);
                if (idx >= b.ncolors) return F_FORMAT;
                o[3 * x] = pal[4 * idx]; o[3 * x + 1] = pal[4 * idx + 1]; o[3 * x + 2] = pal[4 * idx + 2];
            } else if (b.bpp == 24) {
                o[3 * x] = row[3 * x]; o[3 * x + 1] = row[3 * x + 1]; o[3 * x + 2] = row[3 * x + 2];
            } else {
                const uint32_t px = b.bpp == 16 ? le16(row + 2 * x) : le32(row + 4 * x);
                o[3 * x] = field(px, b.mask[2]);
                o[3 * x + 1] = field(px, b.mask[1]);
                o[3 * x + 2] = field(px, b.mask[0]);
            }
        }
    }
    return F_OK;
}

// ---- PNM (P5, P6) --------------------------------------------------------
struct Pnm {
    int W = 0, H = 0, maxval = 0, chans = 0;
    size_t off = 0;
};

int pnm_header(const std::vector<uint8_t> &d, Pnm &p)
{
    p.chans = d[1] == '6' ? 3 : 1;
    size_t i = 2;
    long v[3];
    for (int k = 0; k < 3; k++) {
        for (;;) {                                              // whitespace and # comments
            if (i >= d.size()) return F_FORMAT;
            if (d[i] == '#') { while (i < d.size() && d[i] != '\n') i++; continue; }
            if (d[i] == ' ' || d[i] == '\t' || d[i] == '\n' || d[i] == '\r') { i++; continue; }
            break;
        }
        if (d[i] < '0' || d[i] > '9') return F_FORMAT;
        long x = 0;
        while (i < d.size() && d[i] >= '0' && d[i] <= '9') {
            x = x * 10 + (d[i] - '0');
            if (x > (1L << 30)) return F_FORMAT;
            i++;
        }
        v[k] = x;
    }
    if (i >= d.size()) return F_FORMAT;
    i++;                                                        // one whitespace byte ends the header
    if (v[0] <= 0 || v[1] <= 0 || v[2] <= 0 || v[2] > 65535) return F_FORMAT;
    if ((uint64_t)v[0] * (uint64_t)v[1] > kMaxPixels) return F_UNSUPPORTED;
    if (v[2] != 255 && v[2] != 65535) return F_UNSUPPORTED;    // other depths are not rescaled here
    p.W = (int)v[0]; p.H = (int)v[1]; p.maxval = (int)v[2]; p.off = i;
    return F_OK;
}

int pnm_decode(const std::vector<uint8_t> &d, int W, int H, uint8_t *bgr)
{
    Pnm p;
    int st = pnm_header(d, p);
    if (st != F_OK) return st;
    if (p.W != W || p.H != H) return F_SIZE;
    const int bps = p.maxval > 255 ? 2 : 1;
    if (p.off + (size_t)W * H * p.chans * bps > d.size()) return F_FORMAT;
    const uint8_t *s = d.data() + p.off;
    for (size_t q = 0; q < (size_t)W * H; q++) {
        uint8_t c[3];
        for (int k = 0; k < p.chans; k++) c[k] = s[(q * p.chans + k) * bps];   // 16-bit: the high (first) byte
        if (p.chans == 1) c[1] = c[2] = c[0];
        bgr[3 * q] = c[2]; bgr[3 * q + 1] = c[1]; bgr[3 * q + 2] = c[0];       // RGB -> BGR
    }
    return F_OK;
}

} // namespace

extern "C" int asv_frame_info(const char *path, int *W, int *H)
{
    if (!path || !W || !H) return F_BAD_ARG;
    std::vector<uint8_t> head;
    int st = read_head(path, head, 4096);
    if (st != F_OK) return st;
    switch (sniff(head)) {
    case K_PNG: return asv_png_info(path, W, H);
    case K_BMP: {
        std::vector<uint8_t> d;
        if ((st = read_all(path, d)) != F_OK) return st;
        Bmp b;
        if ((st = bmp_header(d, b)) != F_OK) return st;
        *W = b.W; *H = b.H;
        return F_OK;
    }
    case K_PNM: {
        Pnm p;
        if ((st = pnm_header(head, p)) != F_OK) return st;
        *W = p.W; *H = p.H;
        return F_OK;
    }
    default: return F_UNSUPPORTED;
    }
}

extern "C" int asv_frame_read_bgr(const char *path, uint8_t *bgr, int W, int H)
{
    if (!path || !bgr || W <= 0 || H <= 0 || (uint64_t)W * (uint64_t)H > kMaxPixels) return F_BAD_ARG;
    std::vector<uint8_t> head;
    int st = read_head(path, head, 16);
    if (st != F_OK) return st;
    const Kind k = sniff(head);
    if (k == K_PNG) return asv_png_read_bgr(path, bgr, W, H);
    if (k == K_NONE) return F_UNSUPPORTED;
    std::vector<uint8_t> d;
    if ((st = read_all(path, d)) != F_OK) return st;
    return k == K_BMP ? bmp_decode(d, W, H, bgr) : pnm_decode(d, W, H, bgr);
}

extern "C" int asv_frames_read_bgr(const char *const *paths, int n, int W, int H, uint8_t *bgr)
{
    if (!paths || n < 0 || !bgr || W <= 0 || H <= 0 || (uint64_t)W * (uint64_t)H > kMaxPixels) return F_BAD_ARG;
    for (int i = 0; i < n; i++)
        if (!paths[i]) return F_BAD_ARG;
    std::vector<int> st((size_t)n, F_OK);
    const size_t frame = (size_t)W * H * 3;
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < n; i++) st[i] = asv_frame_read_bgr(paths[i], bgr + frame * i, W, H);
    for (int i = 0; i < n; i++)
        if (st[i] != F_OK) return st[i];
    return F_OK;
}
