/*
 * image_io.cpp — headless image output: 8-bit RGBA pixels as a PNG file (the window's
 * swapchain of the reference has no headless counterpart; this is where a frame goes instead).
 *
 * The file is a valid PNG (ISO/IEC 15948): signature, IHDR (8-bit RGBA, no interlace), one IDAT
 * holding a zlib stream (RFC 1950) of stored deflate blocks (RFC 1951, BTYPE 00; each row is
 * prefixed with filter type 0), IEND; chunk CRCs are CRC-32 (polynomial 0xEDB88320) and the
 * zlib trailer is Adler-32.
 */
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/grisrt.h"

namespace {

uint32_t crc_table[256];
bool crc_ready = false;

void crc_init() {
    for (uint32_t n = 0; n < 256; n++) {
        uint32_t c = n;
        for (int k = 0; k < 8; k++) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
        crc_table[n] = c;
    }
    crc_ready = true;
}

uint32_t crc_update(uint32_t crc, const uint8_t* p, size_t n) {
    for (size_t i = 0; i < n; i++) crc = crc_table[(crc ^ p[i]) & 0xffu] ^ (crc >> 8);
    return crc;
}

void put_be32(std::vector<uint8_t>& v, uint32_t x) {
    v.push_back((uint8_t)(x >> 24)); v.push_back((uint8_t)(x >> 16));
    v.push_back((uint8_t)(x >> 8)); v.push_back((uint8_t)x);
}

void put_chunk(std::vector<uint8_t>& out, const char type[4], const std::vector<uint8_t>& data) {
    put_be32(out, (uint32_t)data.size());
    size_t start = out.size();
    out.insert(out.end(), type, type + 4);
    out.insert(out.end(), data.begin(), data.end());
    uint32_t crc = crc_update(0xffffffffu, out.data() + start, out.size() - start) ^ 0xffffffffu;
    put_be32(out, crc);
}

int fail(char* err, size_t len, const std::string& msg) {
    if (err && len) {
        size_t n = msg.size() < len - 1 ? msg.size() : len - 1;
        memcpy(err, msg.data(), n);
        err[n] = 0;
    }
    return GRIS_ERR_INVALID_ARGUMENT;
}

}  // namespace

extern "C" int grisWritePNG(const char* path, const uint8_t* rgba, uint32_t width, uint32_t height, char* errBuf,
                            size_t errLen) {
    if (!path || !rgba || width == 0 || height == 0) return fail(errBuf, errLen, "null path or pixels, or empty image");
    if ((uint64_t)width * 4 + 1 > 0x7fffffffull || (uint64_t)height * ((uint64_t)width * 4 + 1) > (1ull << 40))
        return fail(errBuf, errLen, "image too large");
    if (!crc_ready) crc_init();
    /* raw scanlines: filter byte 0, then the row */
    const size_t row = (size_t)width * 4;
    std::vector<uint8_t> raw;
    raw.reserve((row + 1) * height);
    for (uint32_t y = 0; y < height; y++) {
        raw.push_back(0);
        raw.insert(raw.end(), rgba + (size_t)y * row, rgba + (size_t)(y + 1) * row);
    }
    /* zlib stream of stored blocks (at most 65535 bytes each) */
    std::vector<uint8_t> z;
    z.reserve(raw.size() + raw.size() / 65535 * 5 + 16);
    z.push_back(0x78); z.push_back(0x01);   /* CM 8, CINFO 7; FCHECK makes 0x7801 a multiple of 31 */
    size_t pos = 0;
    do {
        size_t n = raw.size() - pos < 65535 ? raw.size() - pos : 65535;
        bool last = pos + n == raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back((uint8_t)n); z.push_back((uint8_t)(n >> 8));
        z.push_back((uint8_t)~n); z.push_back((uint8_t)(~n >> 8));
        z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + n);
        pos += n;
    } while (pos < raw.size());
    uint32_t a = 1, b = 0;
    for (uint8_t c : raw) { a = (a + c) % 65521u; b = (b + a) % 65521u; }
    put_be32(z, (b << 16) | a);

    std::vector<uint8_t> out = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
    std::vector<uint8_t> ihdr;
    put_be32(ihdr, width);
    put_be32(ihdr, height);
    ihdr.push_back(8);   /* bit depth */
    ihdr.push_back(6);   /* colour type RGBA */
    ihdr.push_back(0); ihdr.push_back(0); ihdr.push_back(0);
    put_chunk(out, "IHDR", ihdr);
    put_chunk(out, "IDAT", z);
    put_chunk(out, "IEND", std::vector<uint8_t>());
    FILE* f = fopen(path, "wb");
    if (!f) return fail(errBuf, errLen, std::string("cannot write ") + path);
    size_t w = fwrite(out.data(), 1, out.size(), f);
    int closed = fclose(f);
    if (w != out.size() || closed != 0) return fail(errBuf, errLen, std::string("short write to ") + path);
    return GRIS_OK;
}
