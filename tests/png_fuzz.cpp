// Sanitizer fuzz harness for the PNG decoder (built and run by
// tests/test_png.py::test_sanitized_fuzz with -fsanitize=address,undefined).
// Usage: png_fuzz <corpus folder> <iterations> <seed>
// Each case takes a corpus file (or an image of the codec's own encoder) and
// either damages its bytes (bit flips, byte writes, truncation, insertions,
// deletions, duplicated spans; chunk CRCs re-signed 7 times in 8 so damage
// gets past the chunk layer) or damages its structure (the inflated rows and
// header fields, then deflated and signed again), then decodes it.  Any
// out-of-bounds access or undefined behaviour aborts under the sanitizers;
// the decoder's status counts are printed.
#include "asv_png.cpp"
#include <dirent.h>
#include <string>
#include <random>

static void fix_crcs(std::vector<uint8_t> &f)
{
    size_t pos = 8;
    while (pos + 12 <= f.size()) {
        uint32_t len = be32(&f[pos]);
        if (len > f.size() - pos - 12) break;
        uint32_t c = crc32_update(0, &f[pos + 4], 4 + (size_t)len);
        f[pos + 8 + len] = c >> 24; f[pos + 9 + len] = c >> 16; f[pos + 10 + len] = c >> 8; f[pos + 11 + len] = c;
        pos += 12 + len;
    }
}

// structure-aware damage: inflate the image data, damage the filtered rows
// and/or the header fields, deflate again and re-sign every chunk
static bool semantic(std::vector<uint8_t> &f, std::mt19937_64 &g)
{
    PngImage im;
    if (parse_png(f, im, false) != PNG_OK || im.idat.size() < 6) return false;
    static std::vector<uint8_t> buf(1 << 18);      // corpus images inflate to a few KB
    BitIn in(im.idat.data() + 2, im.idat.size() - 2);
    size_t olen = 0;
    if (inflate_raw(in, buf.data(), buf.size(), &olen) != PNG_OK) return false;
    std::vector<uint8_t> raw(buf.begin(), buf.begin() + olen);
    int k = g() % 4;
    if (k == 0 || k == 3) {                       // damage rows
        int nm = 1 + g() % 4;
        for (int m = 0; m < nm && !raw.empty(); m++) {
            size_t at = g() % raw.size();
            if (g() & 1) raw[at] = (uint8_t)g(); else raw[at] = (uint8_t)(g() % 6);
        }
        if (g() % 4 == 0) raw.resize(g() % (raw.size() + 1));
        if (g() % 4 == 0) raw.insert(raw.end(), g() % 40, (uint8_t)g());
    }
    uint8_t ihdr[13];
    memcpy(ihdr, &f[16], 13);
    if (k >= 1) {                                 // damage header fields
        int field = g() % 6;
        if (field == 0) { uint32_t w = be32(ihdr) + (int)(g() % 5) - 2; ihdr[0] = w >> 24; ihdr[1] = w >> 16; ihdr[2] = w >> 8; ihdr[3] = w; }
        if (field == 1) { uint32_t h = be32(ihdr + 4) + (int)(g() % 5) - 2; ihdr[4] = h >> 24; ihdr[5] = h >> 16; ihdr[6] = h >> 8; ihdr[7] = h; }
        if (field == 2) ihdr[8] = (uint8_t[]){ 1, 2, 4, 8, 16, 3, 0 }[g() % 7];
        if (field == 3) ihdr[9] = (uint8_t[]){ 0, 2, 3, 4, 6, 1, 5 }[g() % 7];
        if (field == 4) ihdr[12] = g() % 3;
        if (field == 5) ihdr[10 + g() % 2] = g() % 2;
    }
    std::vector<uint8_t> z;
    z.push_back(0x78); z.push_back(0x01);
    if (g() % 8 == 0) {
        deflate_fixed(raw.data(), raw.size(), z);
    } else {                                      // stored blocks (RFC 1951 3.2.4)
        size_t at = 0;
        do {
            const size_t n = raw.size() - at < 65535 ? raw.size() - at : 65535;
            z.push_back(at + n == raw.size() ? 1 : 0);
            z.push_back((uint8_t)n); z.push_back((uint8_t)(n >> 8));
            z.push_back((uint8_t)~n); z.push_back((uint8_t)(~n >> 8));
            z.insert(z.end(), raw.begin() + at, raw.begin() + at + n);
            at += n;
        } while (at < raw.size());
    }
    put_be32(z, adler32(raw.data(), raw.size()));
    std::vector<uint8_t> out(kSignature, kSignature + 8);
    put_chunk(out, "IHDR", ihdr, 13);
    if (im.npal) {
        std::vector<uint8_t> pl;
        int np = (g() % 3 == 0) ? 1 + g() % 256 : im.npal;
        for (int i = 0; i < np; i++) for (int c = 0; c < 3; c++) pl.push_back(i < im.npal ? im.pal[i][c] : (uint8_t)g());
        put_chunk(out, "PLTE", pl.data(), pl.size());
    }
    put_chunk(out, "IDAT", z.data(), z.size());
    put_chunk(out, "IEND", nullptr, 0);
    f.swap(out);
    return true;
}

int main(int argc, char **argv)
{
    std::vector<std::vector<uint8_t>> corpus;
    DIR *d = opendir(argv[1]);
    for (dirent *e; (e = readdir(d));) {
        std::string n = e->d_name;
        if (n.size() < 5 || n.substr(n.size() - 4) != ".png") continue;
        std::vector<uint8_t> f;
        read_file((std::string(argv[1]) + "/" + n).c_str(), f);
        corpus.push_back(f);
    }
    closedir(d);
    {   // our own encoder's output: LZ77 matches in fixed-Huffman blocks
        std::mt19937 g(3);
        for (int k = 0; k < 8; k++) {
            int W = 1 + g() % 40, H = 1 + g() % 20;
            std::vector<uint8_t> rgb((size_t)W * H * 3);
            for (auto &v : rgb) v = (g() % 4) * 60;
            std::vector<uint8_t> f;
            encode_png(rgb.data(), W, H, f);
            corpus.push_back(f);
        }
    }
    long iters = atol(argv[2]);
    std::mt19937_64 g(atol(argv[3]));
    std::vector<uint8_t> out;
    long ok = 0, fails[8] = {0};
    for (long it = 0; it < iters; it++) {
        std::vector<uint8_t> f = corpus[g() % corpus.size()];
        if (g() % 2 && semantic(f, g)) goto run;
        {
        int nm = 1 + g() % 6;
        for (int m = 0; m < nm; m++) {
            int op = g() % 7;
            size_t at = f.empty() ? 0 : g() % f.size();
            switch (op) {
            case 0: if (!f.empty()) f[at] ^= 1u << (g() % 8); break;
            case 1: if (!f.empty()) f[at] = (uint8_t)g(); break;
            case 2: if (!f.empty()) f[at] = (g() & 1) ? 0xff : 0; break;
            case 3: f.resize(at); break;
            case 4: f.insert(f.begin() + at, (uint8_t)g()); break;
            case 5: if (!f.empty()) f.erase(f.begin() + at); break;
            case 6: { size_t b = g() % (f.size() + 1), l = g() % 64;   // duplicate a span
                      if (b + l <= f.size()) { std::vector<uint8_t> s(f.begin() + b, f.begin() + b + l);
                                               f.insert(f.begin() + at, s.begin(), s.end()); } } break;
            }
        }
        if (g() % 8) fix_crcs(f);
        }
    run:
        PngImage im;
        int W = 0, H = 0;
        if (parse_png(f, im, true) == PNG_OK) { W = (int)im.W; H = (int)im.H; }
        if (W <= 0 || H <= 0 || (long)W * H > 1 << 16) { W = 1 + g() % 40; H = 1 + g() % 20; }
        out.assign((size_t)W * H * 3, 0);
        int st = decode_png(f, W, H, out.data());
        if (st == PNG_OK) ok++; else fails[-st & 7]++;
    }
    printf("iters %ld ok %ld fails", iters, ok);
    for (int i = 0; i < 8; i++) printf(" %ld", fails[i]);
    printf("\n");
}
