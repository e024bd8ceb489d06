// dr_png.cpp - PNG decoding for textures: the 8-bit RGBA pixels Images::getTexturePNG asks lodepng for
// (Namespaces/Images/Images.cu:38-56: lodepng::decode to RGBA, 8 bits per channel), from the PNG
// specification (ISO/IEC 15948) and the DEFLATE format (RFC 1951) inside a zlib stream (RFC 1950).
//
// Supported: every colour type (grey, RGB, palette, grey + alpha, RGBA) at every bit depth the
// format allows (1, 2, 4, 8, 16), tRNS transparency (palette alphas, grey / RGB colour keys),
// Adam7 interlacing, all five row filters.  Conversion to 8-bit RGBA: 16-bit samples keep their
// high byte; low-bit-depth grey is scaled to 0..255 (value * 255 / (2^depth - 1)); grey expands to
// R = G = B; a colour-key match gets alpha 0, everything else without alpha gets 255.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/dr_api.h"
#include "dr_guard.h"

void dr_internal_set_error(const char *msg);

namespace {

struct PngError {
    std::string msg;
};
[[noreturn]] void bad(const std::string &m) { throw PngError{m}; }

// ---- inflate (RFC 1951) ---------------------------------------------------------------------------
class BitReader {
  public:
    BitReader(const uint8_t *p, size_t n) : p_(p), n_(n) {}
    uint32_t bits(int k) {
        uint32_t v = 0;
        for (int i = 0; i < k; i++) {
            if (pos_ >= n_ * 8) bad("truncated deflate stream");
            v |= (uint32_t)((p_[pos_ >> 3] >> (pos_ & 7)) & 1u) << i;
            pos_++;
        }
        return v;
    }
    void align() { pos_ = (pos_ + 7) & ~(size_t)7; }
    size_t byte_pos() const { return pos_ >> 3; }
    void skip_bytes(size_t k) { pos_ += 8 * k; }
    const uint8_t *data() const { return p_; }
    size_t size() const { return n_; }

  private:
    const uint8_t *p_;
    size_t n_;
    size_t pos_ = 0;
};

// Canonical Huffman code from code lengths; decoding walks the counts per length.
struct Huffman {
    uint16_t count[16] = {0};
    std::vector<uint16_t> symbol;
    void build(const uint8_t *lengths, int n) {
        std::memset(count, 0, sizeof(count));
        for (int i = 0; i < n; i++) count[lengths[i]]++;
        count[0] = 0;
        uint16_t offs[16];
        offs[1] = 0;
        for (int l = 1; l < 15; l++) offs[l + 1] = (uint16_t)(offs[l] + count[l]);
        symbol.assign((size_t)n, 0);
        for (int i = 0; i < n; i++)
            if (lengths[i]) symbol[offs[lengths[i]]++] = (uint16_t)i;
    }
    int decode(BitReader &br) const {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; len++) {
            code |= (int)br.bits(1);
            int c = count[len];
            if (code - c < first) return symbol[(size_t)(index + (code - first))];
            index += c;
            first += c;
            first <<= 1;
            code <<= 1;
        }
        bad("bad Huffman code");
    }
};

const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193, 257, 385, 513, 769, 1025, 1537, 2049, 3073,
                                4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

void inflate_block(BitReader &br, const Huffman &lit, const Huffman &dist, std::vector<uint8_t> &out) {
    for (;;) {
        int s = lit.decode(br);
        if (s < 256) {
            out.push_back((uint8_t)s);
        } else if (s == 256) {
            return;
        } else {
            s -= 257;
            if (s >= 29) bad("bad length symbol");
            size_t len = kLenBase[s] + br.bits(kLenExtra[s]);
            int ds = dist.decode(br);
            if (ds >= 30) bad("bad distance symbol");
            size_t d = kDistBase[ds] + br.bits(kDistExtra[ds]);
            if (d > out.size()) bad("distance beyond the output");
            size_t from = out.size() - d;
            for (size_t k = 0; k < len; k++) out.push_back(out[from + k]);
        }
    }
}

std::vector<uint8_t> inflate(const uint8_t *p, size_t n) {
    BitReader br(p, n);
    std::vector<uint8_t> out;
    int last = 0;
    while (!last) {
        last = (int)br.bits(1);
        int type = (int)br.bits(2);
        if (type == 0) {
            br.align();
            size_t at = br.byte_pos();
            if (at + 4 > n) bad("truncated stored block");
            uint16_t len = (uint16_t)(p[at] | (p[at + 1] << 8)), nlen = (uint16_t)(p[at + 2] | (p[at + 3] << 8));
            if ((uint16_t)~len != nlen) bad("stored block length check failed");
            if (at + 4 + len > n) bad("truncated stored block");
            out.insert(out.end(), p + at + 4, p + at + 4 + len);
            br.skip_bytes(4 + (size_t)len);
        } else if (type == 1) {
            uint8_t l[288], d[30];
            for (int i = 0; i < 144; i++) l[i] = 8;
            for (int i = 144; i < 256; i++) l[i] = 9;
            for (int i = 256; i < 280; i++) l[i] = 7;
            for (int i = 280; i < 288; i++) l[i] = 8;
            for (int i = 0; i < 30; i++) d[i] = 5;
            Huffman lit, dist;
            lit.build(l, 288);
            dist.build(d, 30);
            inflate_block(br, lit, dist, out);
        } else if (type == 2) {
            int hlit = (int)br.bits(5) + 257, hdist = (int)br.bits(5) + 1, hclen = (int)br.bits(4) + 4;
            static const int order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {0};
            for (int i = 0; i < hclen; i++) cl[order[i]] = (uint8_t)br.bits(3);
            Huffman clh;
            clh.build(cl, 19);
            uint8_t lens[320] = {0};
            int k = 0;
            while (k < hlit + hdist) {
                int sym = clh.decode(br);
                if (sym < 16) {
                    lens[k++] = (uint8_t)sym;
                } else {
                    int rep = 0;
                    uint8_t val = 0;
                    if (sym == 16) {
                        if (k == 0) bad("repeat without a previous length");
                        val = lens[k - 1];
                        rep = 3 + (int)br.bits(2);
                    } else if (sym == 17) {
                        rep = 3 + (int)br.bits(3);
                    } else {
                        rep = 11 + (int)br.bits(7);
                    }
                    if (k + rep > hlit + hdist) bad("code lengths overflow");
                    while (rep--) lens[k++] = val;
                }
            }
            Huffman lit, dist;
            lit.build(lens, hlit);
            dist.build(lens + hlit, hdist);
            inflate_block(br, lit, dist, out);
        } else {
            bad("reserved deflate block type");
        }
    }
    return out;
}

// ---- PNG --------------------------------------------------------------------------------------------
uint32_t be32(const uint8_t *p) { return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]; }

int paeth(int a, int b, int c) {
    int p = a + b - c, pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p, pc = p > c ? p - c : c - p;
    if (pa <= pb && pa <= pc) return a;
    if (pb <= pc) return b;
    return c;
}

struct Png {
    uint32_t w = 0, h = 0;
    int depth = 0, ctype = 0, interlace = 0;
    std::vector<uint8_t> palette;   // RGBA per entry
    bool has_key = false;
    uint16_t key[3] = {0, 0, 0};    // grey or RGB colour key (sample values at the image's depth)
    std::vector<uint8_t> rgba;      // output

    int channels() const {
        switch (ctype) {
            case 0: return 1;
            case 2: return 3;
            case 3: return 1;
            case 4: return 2;
            case 6: return 4;
        }
        bad("bad colour type");
    }

    // Undoes the row filters of one (sub)image in place; returns the filtered rows' raw bytes.
    void unfilter(uint8_t *data, uint32_t pw, uint32_t ph, std::vector<uint8_t> &raw) const {
        const size_t bpp_bits = (size_t)channels() * depth;
        const size_t stride = (pw * bpp_bits + 7) / 8;
        const size_t bpp = (bpp_bits + 7) / 8;
        raw.assign(stride * ph, 0);
        std::vector<uint8_t> prev(stride, 0);
        for (uint32_t y = 0; y < ph; y++) {
            const uint8_t f = data[y * (stride + 1)];
            const uint8_t *in = data + y * (stride + 1) + 1;
            uint8_t *cur = raw.data() + y * stride;
            for (size_t i = 0; i < stride; i++) {
                const int a = i >= bpp ? cur[i - bpp] : 0, b = prev[i], c = i >= bpp ? prev[i - bpp] : 0;
                int v = in[i];
                if (f == 1) v += a;
                else if (f == 2) v += b;
                else if (f == 3) v += (a + b) >> 1;
                else if (f == 4) v += paeth(a, b, c);
                else if (f != 0) bad("bad row filter");
                cur[i] = (uint8_t)v;
            }
            std::memcpy(prev.data(), cur, stride);
        }
    }

    // Sample k of pixel x in an unfiltered row.
    uint16_t sample(const uint8_t *row, uint32_t x, int k) const {
        const int ch = channels();
        if (depth == 8) return row[(size_t)x * ch + k];
        if (depth == 16) return (uint16_t)((row[((size_t)x * ch + k) * 2] << 8) | row[((size_t)x * ch + k) * 2 + 1]);
        const size_t bit = ((size_t)x * ch + k) * depth;
        return (uint16_t)((row[bit >> 3] >> (8 - depth - (bit & 7))) & ((1 << depth) - 1));
    }

    void put(uint32_t x, uint32_t y, const uint8_t *row, uint32_t px) {
        uint8_t *o = &rgba[((size_t)y * w + x) * 4];
        auto to8 = [&](uint16_t v) -> uint8_t {
            if (depth == 16) return (uint8_t)(v >> 8);
            if (depth == 8) return (uint8_t)v;
            return (uint8_t)((v * 255) / ((1 << depth) - 1));
        };
        if (ctype == 3) {
            const uint16_t i = sample(row, px, 0);
            if ((size_t)i * 4 + 3 >= palette.size()) bad("palette index out of range");
            std::memcpy(o, &palette[(size_t)i * 4], 4);
            return;
        }
        if (ctype == 0 || ctype == 4) {
            const uint16_t g = sample(row, px, 0);
            o[0] = o[1] = o[2] = to8(g);
            if (ctype == 4) o[3] = to8(sample(row, px, 1));
            else o[3] = (has_key && g == key[0]) ? 0 : 255;
            return;
        }
        const uint16_t r = sample(row, px, 0), g = sample(row, px, 1), b = sample(row, px, 2);
        o[0] = to8(r);
        o[1] = to8(g);
        o[2] = to8(b);
        if (ctype == 6) o[3] = to8(sample(row, px, 3));
        else o[3] = (has_key && r == key[0] && g == key[1] && b == key[2]) ? 0 : 255;
    }

    void decode(const std::vector<uint8_t> &file) {
        static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
        if (file.size() < 8 || std::memcmp(file.data(), sig, 8) != 0) bad("not a PNG file");
        std::vector<uint8_t> idat;
        bool have_header = false, ended = false;
        size_t at = 8;
        while (at + 12 <= file.size() && !ended) {
            const uint32_t len = be32(&file[at]);
            if (at + 12 + (size_t)len > file.size()) bad("truncated chunk");
            const uint8_t *type = &file[at + 4], *d = &file[at + 8];
            if (!std::memcmp(type, "IHDR", 4)) {
                if (len < 13) bad("short IHDR");
                w = be32(d);
                h = be32(d + 4);
                depth = d[8];
                ctype = d[9];
                interlace = d[12];
                if (d[10] != 0 || d[11] != 0) bad("unknown compression or filter method");
                if (interlace > 1) bad("unknown interlace method");
                const bool ok = (ctype == 0 && (depth == 1 || depth == 2 || depth == 4 || depth == 8 || depth == 16)) ||
                                (ctype == 3 && (depth == 1 || depth == 2 || depth == 4 || depth == 8)) ||
                                ((ctype == 2 || ctype == 4 || ctype == 6) && (depth == 8 || depth == 16));
                if (!ok) bad("bad colour type / bit depth");
                if (w == 0 || h == 0 || (uint64_t)w * h > (1ull << 28)) bad("bad image size");
                have_header = true;
            } else if (!std::memcmp(type, "PLTE", 4)) {
                palette.assign((size_t)(len / 3) * 4, 255);
                for (uint32_t i = 0; i < len / 3; i++) std::memcpy(&palette[(size_t)i * 4], d + 3 * i, 3);
            } else if (!std::memcmp(type, "tRNS", 4)) {
                if (ctype == 3) {
                    for (uint32_t i = 0; i < len && (size_t)i * 4 + 3 < palette.size(); i++) palette[(size_t)i * 4 + 3] = d[i];
                } else if (ctype == 0 && len >= 2) {
                    has_key = true;
                    key[0] = (uint16_t)((d[0] << 8) | d[1]);
                } else if (ctype == 2 && len >= 6) {
                    has_key = true;
                    for (int k = 0; k < 3; k++) key[k] = (uint16_t)((d[2 * k] << 8) | d[2 * k + 1]);
                }
            } else if (!std::memcmp(type, "IDAT", 4)) {
                idat.insert(idat.end(), d, d + len);
            } else if (!std::memcmp(type, "IEND", 4)) {
                ended = true;
            }
            at += 12 + (size_t)len;
        }
        if (!have_header) bad("no IHDR chunk");
        if (ctype == 3 && palette.empty()) bad("palette image without PLTE");
        if (idat.size() < 6) bad("no image data");
        if ((idat[0] & 15) != 8 || ((idat[0] << 8) | idat[1]) % 31 != 0) bad("bad zlib header");
        if (idat[1] & 32) bad("zlib preset dictionary");
        std::vector<uint8_t> raw = inflate(idat.data() + 2, idat.size() - 2);
        rgba.assign((size_t)w * h * 4, 0);
        const size_t bpp_bits = (size_t)channels() * depth;
        std::vector<uint8_t> rows;
        if (!interlace) {
            const size_t need = ((w * bpp_bits + 7) / 8 + 1) * h;
            if (raw.size() < need) bad("image data too short");
            unfilter(raw.data(), w, h, rows);
            const size_t stride = (w * bpp_bits + 7) / 8;
            for (uint32_t y = 0; y < h; y++)
                for (uint32_t x = 0; x < w; x++) put(x, y, rows.data() + y * stride, x);
            return;
        }
        // Adam7 passes: start x, start y, step x, step y
        static const uint32_t p7[7][4] = {{0, 0, 8, 8}, {4, 0, 8, 8}, {0, 4, 4, 8}, {2, 0, 4, 4}, {0, 2, 2, 4}, {1, 0, 2, 2}, {0, 1, 1, 2}};
        size_t off = 0;
        for (int p = 0; p < 7; p++) {
            const uint32_t pw = (w > p7[p][0]) ? (w - p7[p][0] + p7[p][2] - 1) / p7[p][2] : 0;
            const uint32_t ph = (h > p7[p][1]) ? (h - p7[p][1] + p7[p][3] - 1) / p7[p][3] : 0;
            if (pw == 0 || ph == 0) continue;
            const size_t stride = (pw * bpp_bits + 7) / 8;
            if (raw.size() < off + (stride + 1) * ph) bad("image data too short");
            unfilter(raw.data() + off, pw, ph, rows);
            for (uint32_t y = 0; y < ph; y++)
                for (uint32_t x = 0; x < pw; x++)
                    put(p7[p][0] + x * p7[p][2], p7[p][1] + y * p7[p][3], rows.data() + y * stride, x);
            off += (stride + 1) * ph;
        }
    }
};

bool read_all(const char *path, std::vector<uint8_t> &out) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    uint8_t buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) out.insert(out.end(), buf, buf + n);
    std::fclose(f);
    return true;
}

dr_status fail(dr_status s, const std::string &m) {
    dr_internal_set_error(m.c_str());
    return s;
}

}  // namespace

extern "C" {

dr_status dr_png_read(const char *path, int32_t *width, int32_t *height, uint8_t *rgba8) try {
    if (!path || !width || !height) return fail(DR_E_ARG, "dr_png_read: NULL argument");
    std::vector<uint8_t> file;
    if (!read_all(path, file)) return fail(DR_E_ARG, std::string("dr_png_read: cannot open ") + path);
    Png png;
    try {
        png.decode(file);
    } catch (const PngError &e) {
        return fail(DR_E_ARG, std::string("dr_png_read: ") + path + ": " + e.msg);
    } catch (const std::bad_alloc &) {
        return fail(DR_E_NOMEM, "dr_png_read: out of host memory");
    }
    *width = (int32_t)png.w;
    *height = (int32_t)png.h;
    if (rgba8) std::memcpy(rgba8, png.rgba.data(), png.rgba.size());
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_png_read");
}

}  // extern "C"
