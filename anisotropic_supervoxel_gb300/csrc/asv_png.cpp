// asv_png.cpp -- PNG frames in and out of the segmentation path.
//
// Input: Render::run reads a clip as the sorted files of a folder, each with
// cv::imread(path, 1) (GPU-AS/Render.cpp:151-157, 229-238): 8-bit BGR, top
// row first.  asv_png_read_bgr gives those pixels for PNG frames: grey is
// replicated to three channels, alpha is dropped, 16-bit samples keep their
// high byte, palette indices are looked up and 1/2/4-bit grey is scaled to
// 0..255.
// Output: the per-frame PNG files of print_render / output_render_all (their
// imwrite calls are commented out in the reference: GPU-AS/Image.cpp:1930-1932,
// streamGPU-AS/Render.cpp:819-821), pseudo-coloured as asv_write_render_ppm.
//
// Written from the specifications -- PNG (W3C Recommendation, second
// edition), the zlib format (RFC 1950) and DEFLATE (RFC 1951) -- with no codec
// library.  The decoder takes stored, fixed- and dynamic-Huffman blocks, all
// five row filters, every colour type and bit depth, and Adam7 interlacing;
// every read is bounds-checked and a malformed file is an error code, never a
// crash.  The encoder writes 8-bit RGB with a per-row filter choice (least
// sum of absolute filtered bytes) and one fixed-Huffman LZ77 stream.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "asv_host.h"

namespace {

enum { PNG_OK = 0, PNG_BAD_ARG = -1, PNG_IO = -2, PNG_FORMAT = -3, PNG_UNSUPPORTED = -4, PNG_SIZE = -5 };
const uint64_t kMaxPixels = 1ull << 28;           // larger frames are refused

// ---------------------------------------------------------------------------
// checksums: CRC-32 of PNG chunks (PNG Annex D polynomial, evaluated 8 bytes
// at a time with the usual sliced tables) and the zlib stream's Adler-32
// ---------------------------------------------------------------------------
struct CrcTables {
    uint32_t t[8][256];
    CrcTables()
    {
        for (uint32_t n = 0; n < 256; n++) {
            uint32_t c = n;
            for (int k = 0; k < 8; k++) c = (c & 1u) ? 0xedb88320u ^ (c >> 1) : c >> 1;
            t[0][n] = c;
        }
        for (int k = 1; k < 8; k++)
            for (int n = 0; n < 256; n++) t[k][n] = (t[k - 1][n] >> 8) ^ t[0][t[k - 1][n] & 0xffu];
    }
};

const CrcTables &crc_tables()
{
    static const CrcTables tabs;
    return tabs;
}

uint32_t crc32_update(uint32_t crc, const uint8_t *p, size_t n)
{
    const CrcTables &T = crc_tables();
    uint32_t c = ~crc;
    while (n >= 8) {
        const uint32_t a = c ^ ((uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24);
        c = T.t[7][a & 0xffu] ^ T.t[6][(a >> 8) & 0xffu] ^ T.t[5][(a >> 16) & 0xffu] ^ T.t[4][a >> 24] ^
            T.t[3][p[4]] ^ T.t[2][p[5]] ^ T.t[1][p[6]] ^ T.t[0][p[7]];
        p += 8;
        n -= 8;
    }
    while (n--) c = T.t[0][(c ^ *p++) & 0xffu] ^ (c >> 8);
    return ~c;
}

uint32_t adler32(const uint8_t *p, size_t n)
{
    uint32_t a = 1, b = 0;
    while (n) {
        size_t k = n < 5552 ? n : 5552;          // largest run before b can overflow 32 bits
        n -= k;
        while (k--) {
            a += *p++;
            b += a;
        }
        a %= 65521u;
        b %= 65521u;
    }
    return b << 16 | a;
}

uint32_t be32(const uint8_t *p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }

void put_be32(std::vector<uint8_t> &v, uint32_t x)
{
    v.push_back((uint8_t)(x >> 24));
    v.push_back((uint8_t)(x >> 16));
    v.push_back((uint8_t)(x >> 8));
    v.push_back((uint8_t)x);
}

// ---------------------------------------------------------------------------
// DEFLATE constants (RFC 1951 3.2.5-3.2.7)
// ---------------------------------------------------------------------------
const uint16_t kLenBase[29] = { 3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258 };
const uint8_t kLenExtra[29] = { 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0 };
const uint16_t kDistBase[30] = { 1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                 193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577 };
const uint8_t kDistExtra[30] = { 0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13 };
const uint8_t kClenOrder[19] = { 16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15 };

// ---------------------------------------------------------------------------
// inflate
// ---------------------------------------------------------------------------
// LSB-first bit reader; reads past the end yield zero bits and are caught by
// overrun() (the decoder checks it after every symbol)
struct BitIn {
    const uint8_t *p;
    size_t n, pos = 0;
    uint64_t buf = 0;
    int cnt = 0;
    BitIn(const uint8_t *p_, size_t n_) : p(p_), n(n_) {}
    void need(int k)
    {
        if (cnt >= k) return;
        if (pos + 8 <= n) {
            // load 8 bytes and keep the whole ones that fit; the bits of the
            // partly kept byte above cnt are that byte's own and are OR-ed in
            // again, unchanged, by the next refill
            uint64_t v = 0;
            for (int b = 0; b < 8; b++) v |= (uint64_t)p[pos + b] << (8 * b);
            buf |= v << cnt;
            const int take = (63 - cnt) >> 3;
            pos += (size_t)take;
            cnt += 8 * take;
            return;
        }
        while (cnt < k) {
            buf |= (uint64_t)(pos < n ? p[pos] : 0) << cnt;
            pos++;
            cnt += 8;
        }
    }
    uint32_t get(int k)
    {
        if (k == 0) return 0;
        need(k);
        const uint32_t v = (uint32_t)(buf & ((1ull << k) - 1));
        buf >>= k;
        cnt -= k;
        return v;
    }
    uint32_t peek(int k)
    {
        need(k);
        return (uint32_t)(buf & ((1ull << k) - 1));
    }
    void drop(int k)
    {
        buf >>= k;
        cnt -= k;
    }
    void align() { drop(cnt & 7); }
    bool overrun() const { return pos * 8 - (size_t)cnt > n * 8; }
    size_t byte_pos() const { return pos - (size_t)(cnt >> 3); }      // after align()
};

// canonical Huffman code (RFC 1951 3.2.2) from code lengths: a lookup table
// for codes of up to kFast bits, and per-length counts for longer codes
struct Huffman {
    static const int kFast = 10;
    uint16_t fast[1 << kFast];      // (symbol << 4) | length, 0 = longer code
    uint16_t count[16];
    uint16_t symbols[288];

    bool build(const uint8_t *len, int n)
    {
        std::memset(count, 0, sizeof(count));
        std::memset(fast, 0, sizeof(fast));
        for (int s = 0; s < n; s++) count[len[s]]++;
        count[0] = 0;
        int left = 1;
        for (int l = 1; l < 16; l++) {           // over-subscribed lengths are invalid
            left <<= 1;
            left -= count[l];
            if (left < 0) return false;
        }
        uint16_t offs[16];
        offs[1] = 0;
        for (int l = 1; l < 15; l++) offs[l + 1] = (uint16_t)(offs[l] + count[l]);
        for (int s = 0; s < n; s++)
            if (len[s]) symbols[offs[len[s]]++] = (uint16_t)s;
        // codes in canonical order: per length, consecutive values from the
        // first code of that length; the table index is the code bit-reversed
        int code = 0, k = 0;
        for (int l = 1; l <= kFast; l++) {
            for (int i = 0; i < count[l]; i++, k++, code++) {
                int rev = 0;
                for (int b = 0; b < l; b++) rev |= ((code >> b) & 1) << (l - 1 - b);
                for (int f = rev; f < (1 << kFast); f += 1 << l) fast[f] = (uint16_t)(symbols[k] << 4 | l);
            }
            code <<= 1;
        }
        return true;
    }

    // next symbol, -1 for a code that is not assigned
    inline int decode(BitIn &in) const
    {
        const uint16_t e = fast[in.peek(kFast)];
        if (e) {
            in.drop(e & 15);
            return e >> 4;
        }
        return decode_long(in);
    }

    // codes longer than kFast bits (and unassigned ones), one bit at a time
    int decode_long(BitIn &in) const
    {
        int code = 0, first = 0, index = 0;
        for (int l = 1; l < 16; l++) {
            code |= (int)in.get(1);
            const int c = count[l];
            if (code - first < c) return symbols[index + code - first];
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        return -1;
    }
};

// raw DEFLATE stream into out[0..cap); *olen = bytes written.  Returns
// PNG_OK, or PNG_FORMAT for any malformed or over-long stream.
int inflate_raw(BitIn &state, uint8_t *out, size_t cap, size_t *olen)
{
    BitIn in = state;          // a local copy stays in registers across the output stores
    size_t o = 0;
    Huffman lit, dist;
    bool last = false;
    while (!last) {
        last = in.get(1) != 0;
        const uint32_t type = in.get(2);
        if (type == 0) {                                   // stored
            in.align();
            const uint32_t len = in.get(16), nlen = in.get(16);
            if ((len ^ 0xffffu) != nlen) return PNG_FORMAT;
            if (len > cap - o) return PNG_FORMAT;
            for (uint32_t i = 0; i < len; i++) out[o++] = (uint8_t)in.get(8);
            if (in.overrun()) return PNG_FORMAT;
            continue;
        }
        if (type == 3) return PNG_FORMAT;
        if (type == 1) {                                   // fixed codes
            uint8_t l[288];
            for (int s = 0; s < 288; s++) l[s] = s < 144 ? 8 : s < 256 ? 9 : s < 280 ? 7 : 8;
            lit.build(l, 288);
            uint8_t d[30];
            for (int s = 0; s < 30; s++) d[s] = 5;
            dist.build(d, 30);
        } else {                                           // dynamic codes
            const int nlit = (int)in.get(5) + 257, ndist = (int)in.get(5) + 1, nclen = (int)in.get(4) + 4;
            if (nlit > 286 || ndist > 30) return PNG_FORMAT;
            uint8_t cl[19] = { 0 };
            for (int i = 0; i < nclen; i++) cl[kClenOrder[i]] = (uint8_t)in.get(3);
            Huffman clh;
            if (!clh.build(cl, 19)) return PNG_FORMAT;
            uint8_t lens[286 + 30];
            int i = 0;
            while (i < nlit + ndist) {
                const int s = clh.decode(in);
                if (s < 0 || in.overrun()) return PNG_FORMAT;
                if (s < 16) { lens[i++] = (uint8_t)s; continue; }
                int rep, val = 0;
                if (s == 16) {
                    if (i == 0) return PNG_FORMAT;
                    val = lens[i - 1];
                    rep = 3 + (int)in.get(2);
                } else if (s == 17) {
                    rep = 3 + (int)in.get(3);
                } else {
                    rep = 11 + (int)in.get(7);
                }
                if (i + rep > nlit + ndist) return PNG_FORMAT;
                while (rep--) lens[i++] = (uint8_t)val;
            }
            if (lens[256] == 0) return PNG_FORMAT;         // no end-of-block code
            if (!lit.build(lens, nlit) || !dist.build(lens + nlit, ndist)) return PNG_FORMAT;
        }
        // Past the end of the input the reader yields zero bits, so a
        // truncated stream still ends here: at an end-of-block code, at the
        // output bound or at a match; the overrun is checked there rather
        // than after every literal.
        while (true) {
            int s = lit.decode(in);
            if (s < 256) {
                if (s < 0 || o >= cap) return PNG_FORMAT;
                out[o++] = (uint8_t)s;
                continue;
            }
            if (s == 256) break;
            s -= 257;
            if (s >= 29) return PNG_FORMAT;
            const size_t len = kLenBase[s] + in.get(kLenExtra[s]);
            const int ds = dist.decode(in);
            if (ds < 0 || ds >= 30) return PNG_FORMAT;
            const size_t d = kDistBase[ds] + in.get(kDistExtra[ds]);
            if (in.overrun() || d > o || len > cap - o) return PNG_FORMAT;
            if (d == 1) {
                std::memset(out + o, out[o - 1], len);              // a run of one byte
            } else if (d >= len) {
                std::memcpy(out + o, out + o - d, len);              // source and target apart
            } else {
                for (size_t k = 0; k < len; k++) out[o + k] = out[o + k - d];
            }
            o += len;
        }
        if (in.overrun()) return PNG_FORMAT;
    }
    *olen = o;
    state = in;
    return PNG_OK;
}

// zlib stream (RFC 1950) of exactly `want` bytes
int zlib_decode(const uint8_t *src, size_t n, uint8_t *out, size_t want)
{
    if (n < 6) return PNG_FORMAT;
    const uint32_t cmf = src[0], flg = src[1];
    if ((cmf & 15u) != 8 || (cmf >> 4) > 7 || (cmf * 256 + flg) % 31 != 0 || (flg & 32u)) return PNG_FORMAT;
    BitIn in(src + 2, n - 2);
    size_t olen = 0;
    const int st = inflate_raw(in, out, want, &olen);
    if (st != PNG_OK) return st;
    if (olen != want) return PNG_FORMAT;
    in.align();
    const size_t at = 2 + in.byte_pos();
    if (at + 4 > n) return PNG_FORMAT;
    if (be32(src + at) != adler32(out, olen)) return PNG_FORMAT;
    return PNG_OK;
}

// ---------------------------------------------------------------------------
// PNG decoding
// ---------------------------------------------------------------------------
struct PngImage {
    uint32_t W = 0, H = 0;
    int depth = 0, ctype = 0, interlace = 0, channels = 0, npal = 0;
    uint8_t pal[256][3];
    std::vector<uint8_t> idat;
};

int read_file(const char *path, std::vector<uint8_t> &data)
{
    FILE *f = std::fopen(path, "rb");
    if (!f) return PNG_IO;
    data.clear();
    if (std::fseek(f, 0, SEEK_END) == 0) {
        const long size = std::ftell(f);
        if (size > 0 && std::fseek(f, 0, SEEK_SET) == 0) data.reserve((size_t)size);
        else std::rewind(f);
    }
    uint8_t chunk[1 << 16];
    size_t got;
    while ((got = std::fread(chunk, 1, sizeof(chunk), f)) > 0) data.insert(data.end(), chunk, chunk + got);
    const bool bad = std::ferror(f) != 0;
    std::fclose(f);
    return bad ? PNG_IO : PNG_OK;
}

const uint8_t kSignature[8] = { 137, 80, 78, 71, 13, 10, 26, 10 };

int parse_ihdr(const uint8_t *d, PngImage &im)
{
    im.W = be32(d);
    im.H = be32(d + 4);
    im.depth = d[8];
    im.ctype = d[9];
    if (im.W == 0 || im.H == 0 || im.W > 0x7fffffffu || im.H > 0x7fffffffu) return PNG_FORMAT;
    if (d[10] != 0 || d[11] != 0 || d[12] > 1) return PNG_FORMAT;
    im.interlace = d[12];
    const int dp = im.depth;
    switch (im.ctype) {
    case 0: im.channels = 1; if (dp != 1 && dp != 2 && dp != 4 && dp != 8 && dp != 16) return PNG_FORMAT; break;
    case 2: im.channels = 3; if (dp != 8 && dp != 16) return PNG_FORMAT; break;
    case 3: im.channels = 1; if (dp != 1 && dp != 2 && dp != 4 && dp != 8) return PNG_FORMAT; break;
    case 4: im.channels = 2; if (dp != 8 && dp != 16) return PNG_FORMAT; break;
    case 6: im.channels = 4; if (dp != 8 && dp != 16) return PNG_FORMAT; break;
    default: return PNG_FORMAT;
    }
    if ((uint64_t)im.W * im.H > kMaxPixels) return PNG_UNSUPPORTED;
    return PNG_OK;
}

// chunk walk: IHDR first, PLTE, IDAT (concatenated), IEND; ancillary chunks
// are skipped, unknown critical chunks refused; every chunk CRC is checked.
// header_only stops after IHDR.
int parse_png(const std::vector<uint8_t> &f, PngImage &im, bool header_only)
{
    if (f.size() < 8 || std::memcmp(f.data(), kSignature, 8) != 0) return PNG_FORMAT;
    size_t pos = 8;
    bool ihdr = false, iend = false;
    while (!iend) {
        if (f.size() - pos < 12) return PNG_FORMAT;
        const uint32_t len = be32(&f[pos]);
        if (len > 0x7fffffffu || f.size() - pos - 12 < len) return PNG_FORMAT;
        const uint8_t *type = &f[pos + 4], *data = &f[pos + 8];
        if (crc32_update(0, type, 4 + (size_t)len) != be32(data + len)) return PNG_FORMAT;
        const bool is_ihdr = !std::memcmp(type, "IHDR", 4);
        if (!ihdr && !is_ihdr) return PNG_FORMAT;
        if (is_ihdr) {
            if (ihdr || len != 13) return PNG_FORMAT;
            const int st = parse_ihdr(data, im);
            if (st != PNG_OK) return st;
            ihdr = true;
            if (header_only) return PNG_OK;
        } else if (!std::memcmp(type, "PLTE", 4)) {
            if (len % 3 != 0 || len == 0 || len > 768) return PNG_FORMAT;
            im.npal = (int)(len / 3);
            for (int i = 0; i < im.npal; i++)
                for (int c = 0; c < 3; c++) im.pal[i][c] = data[3 * i + c];
        } else if (!std::memcmp(type, "IDAT", 4)) {
            im.idat.insert(im.idat.end(), data, data + len);
        } else if (!std::memcmp(type, "IEND", 4)) {
            iend = true;
        } else if (!(type[0] & 32u)) {
            return PNG_UNSUPPORTED;                        // unknown critical chunk
        }
        pos += 12 + (size_t)len;
    }
    if (im.idat.empty()) return PNG_FORMAT;
    if (im.ctype == 3 && im.npal == 0) return PNG_FORMAT;
    return PNG_OK;
}

struct Pass {
    int x0, y0, dx, dy;
};
const Pass kAdam7[7] = { { 0, 0, 8, 8 }, { 4, 0, 8, 8 }, { 0, 4, 4, 8 }, { 2, 0, 4, 4 },
                         { 0, 2, 2, 4 }, { 1, 0, 2, 2 }, { 0, 1, 1, 2 } };

// Paeth predictor (PNG 9.4), written as selects: noisy rows make its
// branches unpredictable
inline int paeth(int a, int b, int c)
{
    const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    const int bc = pb <= pc ? b : c;
    return (pa <= pb && pa <= pc) ? a : bc;
}

// undoes the filters of h rows of rb bytes (each after its filter byte)
int unfilter(uint8_t *rows, uint32_t h, size_t rb, int bpp)
{
    const uint8_t *prev = nullptr;
    for (uint32_t y = 0; y < h; y++) {
        uint8_t *r = rows + (size_t)y * (rb + 1);
        const int f = r[0];
        uint8_t *c = r + 1;
        switch (f) {
        case 0: break;
        case 1:
            for (size_t i = bpp; i < rb; i++) c[i] = (uint8_t)(c[i] + c[i - bpp]);
            break;
        case 2:
            if (prev)
                for (size_t i = 0; i < rb; i++) c[i] = (uint8_t)(c[i] + prev[i]);
            break;
        case 3:
            for (size_t i = 0; i < rb; i++) {
                const int a = i >= (size_t)bpp ? c[i - bpp] : 0, b = prev ? prev[i] : 0;
                c[i] = (uint8_t)(c[i] + ((a + b) >> 1));
            }
            break;
        case 4:
            for (size_t i = 0; i < rb; i++) {
                const int a = i >= (size_t)bpp ? c[i - bpp] : 0, b = prev ? prev[i] : 0;
                const int cc = (prev && i >= (size_t)bpp) ? prev[i - bpp] : 0;
                c[i] = (uint8_t)(c[i] + paeth(a, b, cc));
            }
            break;
        default: return PNG_FORMAT;
        }
        prev = c;
    }
    return PNG_OK;
}

// sample s of pixel i in an unfiltered row, reduced to 8 bits
inline int sample8(const uint8_t *row, const PngImage &im, uint32_t i, int s)
{
    const int d = im.depth;
    if (d == 8) return row[(size_t)i * im.channels + s];
    if (d == 16) return row[((size_t)i * im.channels + s) * 2];           // high byte
    const size_t bit = (size_t)i * d;                                     // one channel below 8 bits
    return (row[bit >> 3] >> (8 - d - (int)(bit & 7))) & ((1 << d) - 1);
}

inline int pixel_bgr(const uint8_t *row, const PngImage &im, uint32_t i, uint8_t *o)
{
    switch (im.ctype) {
    case 0: case 4: {
        int g = sample8(row, im, i, 0);
        if (im.depth < 8) g = g * 255 / ((1 << im.depth) - 1);
        o[0] = o[1] = o[2] = (uint8_t)g;
        return PNG_OK;
    }
    case 3: {
        const int k = sample8(row, im, i, 0);
        if (k >= im.npal) return PNG_FORMAT;
        o[0] = im.pal[k][2];
        o[1] = im.pal[k][1];
        o[2] = im.pal[k][0];
        return PNG_OK;
    }
    default:                                                             // 2, 6
        o[0] = (uint8_t)sample8(row, im, i, 2);
        o[1] = (uint8_t)sample8(row, im, i, 1);
        o[2] = (uint8_t)sample8(row, im, i, 0);
        return PNG_OK;
    }
}

int decode_png(const std::vector<uint8_t> &file, int W, int H, uint8_t *bgr)
{
    PngImage im;
    int st = parse_png(file, im, false);
    if (st != PNG_OK) return st;
    if ((int)im.W != W || (int)im.H != H) return PNG_SIZE;
    const int bits = im.channels * im.depth, bpp = bits >= 8 ? bits / 8 : 1;
    auto rowbytes = [&](uint32_t w) { return ((size_t)w * bits + 7) / 8; };
    const int npass = im.interlace ? 7 : 1;
    uint32_t pw[7], ph[7];
    size_t off[8];
    off[0] = 0;
    for (int p = 0; p < npass; p++) {
        if (im.interlace) {
            const Pass &a = kAdam7[p];
            pw[p] = im.W > (uint32_t)a.x0 ? (im.W - a.x0 + a.dx - 1) / a.dx : 0;
            ph[p] = im.H > (uint32_t)a.y0 ? (im.H - a.y0 + a.dy - 1) / a.dy : 0;
        } else {
            pw[p] = im.W;
            ph[p] = im.H;
        }
        off[p + 1] = off[p] + ((pw[p] && ph[p]) ? (size_t)ph[p] * (rowbytes(pw[p]) + 1) : 0);
    }
    // DEFLATE expands by at most 258 bytes per 2-bit-minimum match code (about
    // 1032:1): a header claiming more pixels than the stream can hold is refused
    // before the buffer is allocated
    if (off[npass] / 1032 > im.idat.size() + 64) return PNG_FORMAT;
    std::vector<uint8_t> raw(off[npass]);
    st = zlib_decode(im.idat.data(), im.idat.size(), raw.data(), raw.size());
    if (st != PNG_OK) return st;
    for (int p = 0; p < npass; p++) {
        if (!pw[p] || !ph[p]) continue;
        const size_t rb = rowbytes(pw[p]);
        st = unfilter(raw.data() + off[p], ph[p], rb, bpp);
        if (st != PNG_OK) return st;
        const Pass a = im.interlace ? kAdam7[p] : Pass{ 0, 0, 1, 1 };
        for (uint32_t y = 0; y < ph[p]; y++) {
            const uint8_t *row = raw.data() + off[p] + (size_t)y * (rb + 1) + 1;
            const size_t oy = (size_t)(a.y0 + (size_t)y * a.dy);
            if (!im.interlace && im.depth == 8 && (im.ctype == 2 || im.ctype == 6)) {
                const int ch = im.channels;
                uint8_t *o = bgr + 3 * oy * im.W;
                for (uint32_t i = 0; i < pw[p]; i++, o += 3, row += ch) {
                    o[0] = row[2];
                    o[1] = row[1];
                    o[2] = row[0];
                }
                continue;
            }
            for (uint32_t i = 0; i < pw[p]; i++) {
                const size_t ox = (size_t)(a.x0 + (size_t)i * a.dx);
                st = pixel_bgr(row, im, i, bgr + 3 * (oy * im.W + ox));
                if (st != PNG_OK) return st;
            }
        }
    }
    return PNG_OK;
}

// ---------------------------------------------------------------------------
// encoding: filters per row, LZ77 over a 32 KiB window with hash chains,
// fixed Huffman codes (RFC 1951 3.2.6)
// ---------------------------------------------------------------------------
struct BitOut {
    std::vector<uint8_t> &v;
    uint64_t buf = 0;
    int cnt = 0;
    explicit BitOut(std::vector<uint8_t> &v_) : v(v_) {}
    void put(uint32_t bits, int k)
    {
        buf |= (uint64_t)bits << cnt;
        cnt += k;
        while (cnt >= 8) {
            v.push_back((uint8_t)buf);
            buf >>= 8;
            cnt -= 8;
        }
    }
    void flush()
    {
        if (cnt > 0) v.push_back((uint8_t)buf);
        buf = 0;
        cnt = 0;
    }
};

struct FixedCodes {
    uint16_t lit_code[288];
    uint8_t lit_len[288];
    uint8_t dist_code[30];
    uint8_t len_sym[259];             // match length -> length symbol - 257
    FixedCodes()
    {
        auto rev = [](int c, int l) {
            int r = 0;
            for (int b = 0; b < l; b++) r |= ((c >> b) & 1) << (l - 1 - b);
            return r;
        };
        for (int s = 0; s < 288; s++) {
            int c, l;
            if (s < 144) { c = 0x30 + s; l = 8; }
            else if (s < 256) { c = 0x190 + (s - 144); l = 9; }
            else if (s < 280) { c = s - 256; l = 7; }
            else { c = 0xc0 + (s - 280); l = 8; }
            lit_code[s] = (uint16_t)rev(c, l);
            lit_len[s] = (uint8_t)l;
        }
        for (int s = 0; s < 30; s++) dist_code[s] = (uint8_t)rev(s, 5);
        for (int len = 3, s = 0; len <= 258; len++) {
            while (s < 28 && kLenBase[s + 1] <= len) s++;
            len_sym[len] = (uint8_t)s;
        }
    }
};

const FixedCodes &fixed_codes()
{
    static const FixedCodes fc;
    return fc;
}

inline int dist_symbol(int d)
{
    int s = 0;
    while (s < 29 && kDistBase[s + 1] <= d) s++;
    return s;
}

void deflate_fixed(const uint8_t *src, size_t n, std::vector<uint8_t> &out)
{
    const FixedCodes &fc = fixed_codes();
    const int kWin = 32768, kHashBits = 15, kChain = 4, kGood = 64;
    std::vector<int32_t> head(1u << kHashBits, -1), prev(kWin, -1);
    BitOut bo(out);
    bo.put(1, 1);                                        // final block
    bo.put(1, 2);                                        // fixed codes
    auto hash = [&](size_t i) {
        const uint32_t v = (uint32_t)src[i] | (uint32_t)src[i + 1] << 8 | (uint32_t)src[i + 2] << 16;
        return (v * 2654435761u) >> (32 - kHashBits);
    };
    auto insert = [&](size_t i) {
        if (i + 3 > n) return;
        const uint32_t h = hash(i);
        prev[i & (kWin - 1)] = head[h];
        head[h] = (int32_t)i;
    };
    size_t i = 0;
    while (i < n) {
        int best = 0, bdist = 0;
        if (i + 3 <= n) {
            const size_t maxlen = n - i < 258 ? n - i : 258;
            int32_t j = head[hash(i)];
            for (int c = 0; c < kChain && j >= 0 && i - (size_t)j <= (size_t)kWin; c++) {
                // a candidate can only win if it also matches at the current best length
                if (best == 0 || ((size_t)best < maxlen && src[j + best] == src[i + best])) {
                    size_t l = 0;
                    while (l < maxlen && src[j + l] == src[i + l]) l++;
                    if ((int)l > best) {
                        best = (int)l;
                        bdist = (int)(i - (size_t)j);
                        if (l == maxlen || best >= kGood) break;
                    }
                }
                const int32_t nj = prev[j & (kWin - 1)];
                if (nj >= j) break;                      // the slot was reused by a newer position
                j = nj;
            }
        }
        if (best >= 3) {
            const int ls = fc.len_sym[best];
            bo.put(fc.lit_code[257 + ls], fc.lit_len[257 + ls]);
            bo.put((uint32_t)(best - kLenBase[ls]), kLenExtra[ls]);
            const int ds = dist_symbol(bdist);
            bo.put(fc.dist_code[ds], 5);
            bo.put((uint32_t)(bdist - kDistBase[ds]), kDistExtra[ds]);
            for (int k = 0; k < best; k++) insert(i + k);
            i += best;
        } else {
            bo.put(fc.lit_code[src[i]], fc.lit_len[src[i]]);
            insert(i);
            i++;
        }
    }
    bo.put(fc.lit_code[256], fc.lit_len[256]);
    bo.flush();
}

inline long abs_sum(const uint8_t *o, size_t n)
{
    long s = 0;
    for (size_t i = 0; i < n; i++) s += std::abs((int)(int8_t)o[i]);
    return s;
}

// the five filtered versions of row c (row above p) into o0..o4
void filter_candidates(const uint8_t *__restrict__ c, const uint8_t *__restrict__ p, size_t rb,
                       uint8_t *__restrict__ o0, uint8_t *__restrict__ o1, uint8_t *__restrict__ o2,
                       uint8_t *__restrict__ o3, uint8_t *__restrict__ o4)
{
    const size_t head = rb < 3 ? rb : 3;
    for (size_t i = 0; i < head; i++) {                   // no left neighbour
        o0[i] = c[i];
        o1[i] = c[i];
        o2[i] = (uint8_t)(c[i] - p[i]);
        o3[i] = (uint8_t)(c[i] - (p[i] >> 1));
        o4[i] = (uint8_t)(c[i] - p[i]);                    // Paeth of (0, b, 0) is b
    }
    for (size_t i = head; i < rb; i++) {
        o0[i] = c[i];
        o1[i] = (uint8_t)(c[i] - c[i - 3]);
        o2[i] = (uint8_t)(c[i] - p[i]);
        o3[i] = (uint8_t)(c[i] - ((c[i - 3] + p[i]) >> 1));
    }
    for (size_t i = head; i < rb; i++) o4[i] = (uint8_t)(c[i] - paeth(c[i - 3], p[i], p[i - 3]));
}

// filtered scanlines of an 8-bit RGB image: per row the filter whose output
// has the least sum of absolute values (as signed bytes).  Each candidate
// is one branch-free pass over the row; the row above the first is zero.
void filter_rows(const uint8_t *rgb, int W, int H, std::vector<uint8_t> &out)
{
    const size_t rb = (size_t)W * 3;
    out.resize((size_t)H * (rb + 1));
    std::vector<uint8_t> cand(5 * rb), zero(rb, 0);
    for (int y = 0; y < H; y++) {
        const uint8_t *c = rgb + (size_t)y * rb, *p = y ? c - rb : zero.data();
        uint8_t *o = cand.data();
        filter_candidates(c, p, rb, o, o + rb, o + 2 * rb, o + 3 * rb, o + 4 * rb);
        long best_sum = -1;
        int best = 0;
        for (int f = 0; f < 5; f++) {
            const long sum = abs_sum(cand.data() + f * rb, rb);
            if (best_sum < 0 || sum < best_sum) {
                best_sum = sum;
                best = f;
            }
        }
        uint8_t *row = out.data() + (size_t)y * (rb + 1);
        row[0] = (uint8_t)best;
        std::memcpy(row + 1, cand.data() + best * rb, rb);
    }
}

void put_chunk(std::vector<uint8_t> &f, const char *type, const uint8_t *data, size_t len)
{
    put_be32(f, (uint32_t)len);
    const size_t at = f.size();
    f.insert(f.end(), type, type + 4);
    if (len) f.insert(f.end(), data, data + len);
    put_be32(f, crc32_update(0, f.data() + at, 4 + len));
}

int encode_png(const uint8_t *rgb, int W, int H, std::vector<uint8_t> &file)
{
    std::vector<uint8_t> filt;
    filter_rows(rgb, W, H, filt);
    std::vector<uint8_t> z;
    z.push_back(0x78);                                   // deflate, 32 KiB window
    z.push_back(0x01);                                   // check bits: 0x7801 % 31 == 0
    deflate_fixed(filt.data(), filt.size(), z);
    put_be32(z, adler32(filt.data(), filt.size()));
    file.assign(kSignature, kSignature + 8);
    const uint32_t w = (uint32_t)W, h = (uint32_t)H;
    const uint8_t ihdr[13] = { (uint8_t)(w >> 24), (uint8_t)(w >> 16), (uint8_t)(w >> 8), (uint8_t)w,
                               (uint8_t)(h >> 24), (uint8_t)(h >> 16), (uint8_t)(h >> 8), (uint8_t)h,
                               8, 2, 0, 0, 0 };                  // 8-bit RGB, not interlaced
    put_chunk(file, "IHDR", ihdr, 13);
    const size_t kIdat = 1u << 20;
    for (size_t at = 0; at < z.size(); at += kIdat)
        put_chunk(file, "IDAT", z.data() + at, z.size() - at < kIdat ? z.size() - at : kIdat);
    put_chunk(file, "IEND", nullptr, 0);
    return PNG_OK;
}

int write_file(const char *path, const std::vector<uint8_t> &data)
{
    FILE *f = std::fopen(path, "wb");
    if (!f) return PNG_IO;
    const bool ok = std::fwrite(data.data(), 1, data.size(), f) == data.size();
    return (std::fclose(f) == 0 && ok) ? PNG_OK : PNG_IO;
}

bool dims_ok(int W, int H) { return W > 0 && H > 0 && (uint64_t)W * (uint64_t)H <= kMaxPixels; }

}  // namespace

extern "C" int asv_png_info(const char *path, int *W, int *H)
{
    if (!path || !W || !H) return PNG_BAD_ARG;
    FILE *f = std::fopen(path, "rb");
    if (!f) return PNG_IO;
    std::vector<uint8_t> head(33);
    const size_t got = std::fread(head.data(), 1, head.size(), f);
    std::fclose(f);
    head.resize(got);
    PngImage im;
    const int st = parse_png(head, im, true);
    if (st != PNG_OK) return st;
    *W = (int)im.W;
    *H = (int)im.H;
    return PNG_OK;
}

extern "C" int asv_png_read_bgr(const char *path, uint8_t *bgr, int W, int H)
{
    if (!path || !bgr || !dims_ok(W, H)) return PNG_BAD_ARG;
    std::vector<uint8_t> file;
    const int st = read_file(path, file);
    if (st != PNG_OK) return st;
    return decode_png(file, W, H, bgr);
}

extern "C" int asv_png_read_frames_bgr(const char *const *paths, int n, int W, int H, uint8_t *bgr)
{
    if (!paths || n < 0 || !bgr || !dims_ok(W, H)) return PNG_BAD_ARG;
    for (int i = 0; i < n; i++)
        if (!paths[i]) return PNG_BAD_ARG;
    std::vector<int> st((size_t)n, PNG_OK);
    const size_t frame = (size_t)W * H * 3;
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < n; i++) st[i] = asv_png_read_bgr(paths[i], bgr + frame * i, W, H);
    for (int i = 0; i < n; i++)
        if (st[i] != PNG_OK) return st[i];
    return PNG_OK;
}

extern "C" int asv_png_write_rgb(const char *path, const uint8_t *rgb, int W, int H)
{
    if (!path || !rgb || !dims_ok(W, H)) return PNG_BAD_ARG;
    std::vector<uint8_t> file;
    encode_png(rgb, W, H, file);
    return write_file(path, file);
}

extern "C" int asv_render_rgb(const int32_t *labels, int W, int H, int D, int n_labels, uint8_t *rgb)
{
    if (!labels || !rgb || W <= 0 || H <= 0 || D < 0 || n_labels < 0) return PNG_BAD_ARG;
    std::vector<int> col((size_t)n_labels * 3);
    {
        // rand() is one process-wide sequence: renders on several host
        // threads take the palette one at a time
        static std::mutex mu;
        std::lock_guard<std::mutex> lk(mu);
        std::srand(1);    // the default state of rand() when the reference's process starts
        for (auto &c : col) c = std::rand() % 256;
    }
    const size_t fr = (size_t)W * H;
#pragma omp parallel for schedule(static)
    for (int t = 0; t < D; t++)
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) {
                const int l = labels[fr * t + (size_t)y * W + x];
                uint8_t *o = rgb + 3 * (fr * t + (size_t)(H - 1 - y) * W + x);     // un-flip
                if (l < 0 || l >= n_labels) {
                    o[0] = o[1] = o[2] = 0;
                } else {
                    o[0] = (uint8_t)col[3 * (size_t)l];
                    o[1] = (uint8_t)col[3 * (size_t)l + 1];
                    o[2] = (uint8_t)col[3 * (size_t)l + 2];
                }
            }
    return PNG_OK;
}

extern "C" int asv_write_render_png(const char *prefix, const int32_t *labels, int W, int H, int D,
                                    int n_labels, int start_index)
{
    if (!prefix || !labels || !dims_ok(W, H) || D < 0 || n_labels < 0) return PNG_BAD_ARG;
    std::vector<uint8_t> rgb((size_t)W * H * 3 * D);
    int st = asv_render_rgb(labels, W, H, D, n_labels, rgb.data());
    if (st != PNG_OK) return st;
    std::vector<int> sts((size_t)D, PNG_OK);
    const size_t frame = (size_t)W * H * 3;
#pragma omp parallel for schedule(dynamic, 1)
    for (int t = 0; t < D; t++) {
        char name[4096];
        if (start_index < 0) std::snprintf(name, sizeof(name), "%s%05d.png", prefix, t + 1);
        else std::snprintf(name, sizeof(name), "%s%05d_%05d.png", prefix, start_index, t + start_index + 1);
        sts[t] = asv_png_write_rgb(name, rgb.data() + frame * t, W, H);
    }
    for (int t = 0; t < D; t++)
        if (sts[t] != PNG_OK) return sts[t];
    return PNG_OK;
}
