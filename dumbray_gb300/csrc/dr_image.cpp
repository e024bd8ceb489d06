// dr_image.cpp - frame-buffer images on the host: block-major -> row-major, the reference's 8-bit
// conversion, and PNG / PFM writers (no third-party encoder).
//
// Images::saveBufferPNG (Namespaces/Images/Images.cu:7-40) turns every float channel c of the frame
// buffer into a byte by v = 255 * c; v > 255 -> 255, v < 0 -> 0, else truncation, and writes an
// 8-bit RGBA PNG through lodepng.  Here the same bytes are written into a PNG whose zlib stream uses
// stored (uncompressed) deflate blocks, so any PNG reader decodes the identical pixels.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/dr_api.h"
#include "dr_guard.h"

void dr_internal_set_error(const char *msg);

namespace {

dr_status fail(dr_status s, const std::string &msg) {
    dr_internal_set_error(msg.c_str());
    return s;
}

inline uint8_t channel_byte(float c) {
    const float v = 255.0f * c;
    if (v > 255.0f) return 255;
    if (v < 0.0f) return 0;
    if (!(v == v)) return 0;  // NaN: the reference's float-to-byte cast of NaN is undefined; write 0
    return (uint8_t)v;
}

// CRC-32 (ISO 3309 / PNG, reflected polynomial 0xEDB88320), table built once on first use (a
// function-local static: initialised once even when several threads write images).
struct CrcTable {
    uint32_t t[256];
    CrcTable() {
        for (uint32_t i = 0; i < 256; i++) {
            uint32_t c = i;
            for (int k = 0; k < 8; k++) c = (c & 1u) ? (0xEDB88320u ^ (c >> 1)) : (c >> 1);
            t[i] = c;
        }
    }
};

uint32_t crc32_update(uint32_t crc, const uint8_t *p, size_t n) {
    static const CrcTable table;
    for (size_t i = 0; i < n; i++) crc = table.t[(crc ^ p[i]) & 0xFFu] ^ (crc >> 8);
    return crc;
}

void put_be32(std::vector<uint8_t> &v, uint32_t x) {
    v.push_back((uint8_t)(x >> 24));
    v.push_back((uint8_t)(x >> 16));
    v.push_back((uint8_t)(x >> 8));
    v.push_back((uint8_t)x);
}

void put_chunk(std::vector<uint8_t> &out, const char type[4], const std::vector<uint8_t> &data) {
    put_be32(out, (uint32_t)data.size());
    const size_t at = out.size();
    out.insert(out.end(), type, type + 4);
    out.insert(out.end(), data.begin(), data.end());
    const uint32_t crc = crc32_update(0xFFFFFFFFu, out.data() + at, 4 + data.size()) ^ 0xFFFFFFFFu;
    put_be32(out, crc);
}

// zlib stream (RFC 1950) of stored deflate blocks (RFC 1951 BTYPE 00) with its Adler-32.
std::vector<uint8_t> zlib_stored(const std::vector<uint8_t> &raw) {
    std::vector<uint8_t> z;
    z.reserve(raw.size() + raw.size() / 65535 * 5 + 16);
    z.push_back(0x78);
    z.push_back(0x01);
    size_t pos = 0;
    do {
        const size_t len = std::min<size_t>(65535, raw.size() - pos);
        const bool last = pos + len == raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back((uint8_t)(len & 0xFF));
        z.push_back((uint8_t)(len >> 8));
        z.push_back((uint8_t)(~len & 0xFF));
        z.push_back((uint8_t)((~len >> 8) & 0xFF));
        z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + len);
        pos += len;
    } while (pos < raw.size());
    uint32_t a = 1, b = 0;
    for (uint8_t c : raw) {
        a = (a + c) % 65521u;
        b = (b + a) % 65521u;
    }
    put_be32(z, (b << 16) | a);
    return z;
}

bool write_file(const char *path, const void *data, size_t n) {
    FILE *f = std::fopen(path, "wb");
    if (!f) return false;
    const bool ok = std::fwrite(data, 1, n, f) == n;
    return (std::fclose(f) == 0) && ok;
}

}  // namespace

extern "C" {

dr_status dr_image_from_blocks(const float *fb, int32_t width, int32_t height, float *rgba) try {
    if (!fb || !rgba || width <= 0 || height <= 0) return fail(DR_E_ARG, "dr_image_from_blocks: bad argument");
    const int bw = (width + DR_BLOCK_W - 1) / DR_BLOCK_W;
    for (int y = 0; y < height; y++) {
        const int by = y / DR_BLOCK_H, oy = y % DR_BLOCK_H;
        for (int x = 0; x < width; x++) {
            const size_t src = 4 * ((size_t)(by * bw + x / DR_BLOCK_W) * (DR_BLOCK_W * DR_BLOCK_H) + oy * DR_BLOCK_W + x % DR_BLOCK_W);
            std::memcpy(rgba + 4 * ((size_t)y * width + x), fb + src, 4 * sizeof(float));
        }
    }
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_image_from_blocks");
}

dr_status dr_image_to_rgba8(const float *rgba, int32_t width, int32_t height, uint8_t *out) try {
    if (!rgba || !out || width <= 0 || height <= 0) return fail(DR_E_ARG, "dr_image_to_rgba8: bad argument");
    const size_t n = 4 * (size_t)width * height;
    for (size_t i = 0; i < n; i++) out[i] = channel_byte(rgba[i]);
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_image_to_rgba8");
}

dr_status dr_image_write_png(const float *rgba, int32_t width, int32_t height, const char *path) try {
    if (!rgba || !path || width <= 0 || height <= 0) return fail(DR_E_ARG, "dr_image_write_png: bad argument");
    std::vector<uint8_t> raw((size_t)height * (1 + 4 * (size_t)width));
    for (int y = 0; y < height; y++) {
        uint8_t *row = raw.data() + (size_t)y * (1 + 4 * (size_t)width);
        row[0] = 0;  // filter type None
        dr_image_to_rgba8(rgba + 4 * (size_t)y * width, width, 1, row + 1);
    }
    std::vector<uint8_t> png = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
    std::vector<uint8_t> ihdr;
    put_be32(ihdr, (uint32_t)width);
    put_be32(ihdr, (uint32_t)height);
    ihdr.insert(ihdr.end(), {8, 6, 0, 0, 0});  // 8 bits, RGBA, deflate, adaptive filters, no interlace
    put_chunk(png, "IHDR", ihdr);
    put_chunk(png, "IDAT", zlib_stored(raw));
    put_chunk(png, "IEND", {});
    if (!write_file(path, png.data(), png.size())) return fail(DR_E_ARG, std::string("dr_image_write_png: cannot write ") + path);
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_image_write_png");
}

dr_status dr_image_write_pfm(const float *rgba, int32_t width, int32_t height, const char *path) try {
    if (!rgba || !path || width <= 0 || height <= 0) return fail(DR_E_ARG, "dr_image_write_pfm: bad argument");
    // PFM: "PF", width height, negative scale = little-endian; RGB float rows from the bottom up.
    std::string head = "PF\n" + std::to_string(width) + " " + std::to_string(height) + "\n-1.0\n";
    std::vector<uint8_t> out(head.begin(), head.end());
    const size_t at = out.size();
    out.resize(at + 12 * (size_t)width * height);
    uint8_t *dst = out.data() + at;
    for (int y = 0; y < height; y++) {
        const float *src = rgba + 4 * (size_t)(height - 1 - y) * width;
        for (int x = 0; x < width; x++) std::memcpy(dst + 12 * ((size_t)y * width + x), src + 4 * x, 12);
    }
    // float bytes are written in host order; both the build hosts (x86-64, aarch64) are little-endian
    if (!write_file(path, out.data(), out.size())) return fail(DR_E_ARG, std::string("dr_image_write_pfm: cannot write ") + path);
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_image_write_pfm");
}

}  // extern "C"
