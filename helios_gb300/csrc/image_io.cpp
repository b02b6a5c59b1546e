// image_io.cpp — PNG export of tone-mapped frames (replaces the stb_image_write
// call in Renderer::copy_and_save_tone_mapped_image, renderer.cpp:637-713,
// behind Renderer::save_image_to_disk, renderer.h:97).
//
// The file is a plain PNG (RFC 2083 / ISO 15948): 8-bit RGBA, no interlace,
// filter type 0 on every row, and a zlib stream (RFC 1950) of uncompressed
// deflate blocks (RFC 1951 BTYPE 00) — no compression library is needed and
// every decoder reads it.  CRC-32 (ISO 3309 polynomial, reflected 0xEDB88320)
// per chunk and Adler-32 over the raw scanlines, both computed here.
#include "../../include/hx.h"

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <vector>

void hx_set_error(const char* fmt, ...);

#define HX_CHECK_ARG(cond, ...)        \
    do {                               \
        if (!(cond)) {                 \
            hx_set_error(__VA_ARGS__); \
            return HX_ERR_INVALID_ARG; \
        }                              \
    } while (0)

namespace {

uint32_t crc_table_entry(uint32_t n) {
    uint32_t c = n;
    for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
    return c;
}

struct Crc32 {
    uint32_t table[256];
    Crc32() {
        for (uint32_t n = 0; n < 256; ++n) table[n] = crc_table_entry(n);
    }
    uint32_t update(uint32_t crc, const uint8_t* p, size_t n) const {
        uint32_t c = crc;
        for (size_t i = 0; i < n; ++i) c = table[(c ^ p[i]) & 0xffu] ^ (c >> 8);
        return c;
    }
};

void put_be32(std::vector<uint8_t>& out, uint32_t v) {
    out.push_back((uint8_t)(v >> 24));
    out.push_back((uint8_t)(v >> 16));
    out.push_back((uint8_t)(v >> 8));
    out.push_back((uint8_t)v);
}

// length, type, data, CRC over type + data
void put_chunk(std::vector<uint8_t>& out, const Crc32& crc, const char type[4], const std::vector<uint8_t>& data) {
    put_be32(out, (uint32_t)data.size());
    const size_t type_at = out.size();
    out.insert(out.end(), type, type + 4);
    out.insert(out.end(), data.begin(), data.end());
    const uint32_t c = crc.update(0xffffffffu, out.data() + type_at, 4 + data.size()) ^ 0xffffffffu;
    put_be32(out, c);
}

}  // namespace

extern "C" hx_status hx_encode_png(const uint8_t* rgba8, uint32_t width, uint32_t height, uint8_t* out,
                                   uint64_t capacity, uint64_t* size) {
    HX_CHECK_ARG(rgba8 && size && width > 0 && height > 0, "hx_encode_png: null argument or empty image");
    HX_CHECK_ARG((uint64_t)width * 4 + 1 <= 0x7fffffffu && (uint64_t)width * height <= (1ull << 31),
                 "hx_encode_png: image of %u x %u is too large", width, height);
    static const Crc32 crc;
    // raw scanlines: filter byte 0, then the row's RGBA bytes
    const size_t row = (size_t)width * 4 + 1;
    const size_t raw_n = row * height;
    // zlib stream: CMF/FLG (deflate, 32K window, no dictionary, level 0),
    // stored blocks of at most 65535 bytes, Adler-32 of the raw bytes
    std::vector<uint8_t> z;
    z.reserve(raw_n + raw_n / 65535 * 5 + 16);
    z.push_back(0x78);
    z.push_back(0x01);
    uint32_t a = 1, b = 0;
    size_t left = raw_n, y = 0, x = 0;  // position in the raw stream: row y, byte x of it
    while (left > 0) {
        const uint32_t n = (uint32_t)(left < 65535 ? left : 65535);
        left -= n;
        z.push_back(left == 0 ? 1 : 0);  // BFINAL, BTYPE = 00
        z.push_back((uint8_t)n);
        z.push_back((uint8_t)(n >> 8));
        z.push_back((uint8_t)~n);
        z.push_back((uint8_t)(~n >> 8));
        for (uint32_t i = 0; i < n; ++i) {
            const uint8_t v = x == 0 ? 0 : rgba8[y * (size_t)width * 4 + (x - 1)];
            z.push_back(v);
            a = (a + v) % 65521u;
            b = (b + a) % 65521u;
            if (++x == row) { x = 0; ++y; }
        }
    }
    put_be32(z, (b << 16) | a);

    std::vector<uint8_t> png = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
    std::vector<uint8_t> ihdr;
    put_be32(ihdr, width);
    put_be32(ihdr, height);
    ihdr.push_back(8);  // bit depth
    ihdr.push_back(6);  // colour type: RGBA
    ihdr.push_back(0);  // compression: deflate
    ihdr.push_back(0);  // filter method 0
    ihdr.push_back(0);  // no interlace
    put_chunk(png, crc, "IHDR", ihdr);
    put_chunk(png, crc, "IDAT", z);
    put_chunk(png, crc, "IEND", {});
    *size = png.size();
    if (!out) return HX_OK;  // size query
    HX_CHECK_ARG(capacity >= png.size(), "hx_encode_png: output buffer of %llu bytes, %llu needed",
                 (unsigned long long)capacity, (unsigned long long)png.size());
    std::copy(png.begin(), png.end(), out);
    return HX_OK;
}

extern "C" hx_status hx_save_png(const char* path, const uint8_t* rgba8, uint32_t width, uint32_t height) {
    HX_CHECK_ARG(path && rgba8, "hx_save_png: null argument");
    uint64_t n = 0;
    hx_status st = hx_encode_png(rgba8, width, height, nullptr, 0, &n);
    if (st != HX_OK) return st;
    std::vector<uint8_t> buf(n);
    st = hx_encode_png(rgba8, width, height, buf.data(), n, &n);
    if (st != HX_OK) return st;
    FILE* f = std::fopen(path, "wb");
    if (!f) {
        hx_set_error("hx_save_png: cannot open %s for writing", path);
        return HX_ERR_INVALID_ARG;
    }
    const size_t w = std::fwrite(buf.data(), 1, buf.size(), f);
    const int c = std::fclose(f);
    if (w != buf.size() || c != 0) {
        hx_set_error("hx_save_png: short write to %s", path);
        return HX_ERR_INVALID_ARG;
    }
    return HX_OK;
}

// ---------------------------------------------------------------------------
// Block-compressed textures (BC1-BC5, the S3TC / RGTC block formats of the
// reference's assets, resource_manager.cpp:14-30) decoded to RGBA8 at upload.
// Palettes round to nearest in integers; colour endpoints expand from RGB565
// by bit replication.
// ---------------------------------------------------------------------------
namespace {

uint32_t block_bytes(uint32_t fmt) {
    return (fmt == HX_TEXTURE_BC1_RGB || fmt == HX_TEXTURE_BC1_RGBA || fmt == HX_TEXTURE_BC4) ? 8u : 16u;
}

uint64_t le64(const uint8_t* p) {
    uint64_t v = 0;
    for (int k = 7; k >= 0; --k) v = (v << 8) | p[k];
    return v;
}

// 4x4 colour block: 16 RGBA texels (alpha 255, or 0 for the transparent
// entry of the 3-colour mode when transparent is set).
void decode_colour(const uint8_t* b, bool four_always, bool transparent, uint8_t out[16][4]) {
    const uint32_t c0 = b[0] | (b[1] << 8), c1 = b[2] | (b[3] << 8);
    const uint32_t idx = b[4] | (b[5] << 8) | (b[6] << 16) | ((uint32_t)b[7] << 24);
    uint32_t p[4][4];
    for (int e = 0; e < 2; ++e) {
        const uint32_t c = e ? c1 : c0;
        const uint32_t r5 = c >> 11, g6 = (c >> 5) & 63u, b5 = c & 31u;
        p[e][0] = (r5 << 3) | (r5 >> 2);
        p[e][1] = (g6 << 2) | (g6 >> 4);
        p[e][2] = (b5 << 3) | (b5 >> 2);
        p[e][3] = 255;
    }
    if (four_always || c0 > c1) {
        for (int ch = 0; ch < 3; ++ch) {
            p[2][ch] = (2 * p[0][ch] + p[1][ch] + 1) / 3;
            p[3][ch] = (p[0][ch] + 2 * p[1][ch] + 1) / 3;
        }
        p[2][3] = p[3][3] = 255;
    } else {
        for (int ch = 0; ch < 3; ++ch) {
            p[2][ch] = (p[0][ch] + p[1][ch] + 1) / 2;
            p[3][ch] = 0;
        }
        p[2][3] = 255;
        p[3][3] = transparent ? 0 : 255;
    }
    for (int t = 0; t < 16; ++t) {
        const uint32_t k = (idx >> (2 * t)) & 3u;
        for (int ch = 0; ch < 4; ++ch) out[t][ch] = (uint8_t)p[k][ch];
    }
}

// 4x4 single-channel block (BC4 / BC3 alpha / BC5 halves): 16 values.
void decode_channel(const uint8_t* b, uint8_t out[16]) {
    const uint32_t a0 = b[0], a1 = b[1];
    uint32_t p[8];
    p[0] = a0;
    p[1] = a1;
    if (a0 > a1) {
        for (uint32_t k = 2; k < 8; ++k) p[k] = ((8 - k) * a0 + (k - 1) * a1 + 3) / 7;
    } else {
        for (uint32_t k = 2; k < 6; ++k) p[k] = ((6 - k) * a0 + (k - 1) * a1 + 2) / 5;
        p[6] = 0;
        p[7] = 255;
    }
    const uint64_t idx = le64(b) >> 16;
    for (int t = 0; t < 16; ++t) out[t] = (uint8_t)p[(idx >> (3 * t)) & 7u];
}

}  // namespace

extern "C" hx_status hx_texture_decode(const hx_texture_desc* tex, uint8_t* out) {
    HX_CHECK_ARG(tex && out && tex->rgba8 && tex->width > 0 && tex->height > 0, "hx_texture_decode: null argument or empty texture");
    HX_CHECK_ARG(tex->format <= HX_TEXTURE_BC5, "hx_texture_decode: unknown format %u", tex->format);
    const uint32_t W = tex->width, H = tex->height;
    if (tex->format == HX_TEXTURE_RGBA8) {
        std::copy(tex->rgba8, tex->rgba8 + (size_t)W * H * 4, out);
        return HX_OK;
    }
    const uint32_t bw = (W + 3) / 4, bh = (H + 3) / 4, bb = block_bytes(tex->format);
    for (uint32_t by = 0; by < bh; ++by)
        for (uint32_t bx = 0; bx < bw; ++bx) {
            const uint8_t* b = tex->rgba8 + ((size_t)by * bw + bx) * bb;
            uint8_t px[16][4];
            uint8_t ch[16];
            switch (tex->format) {
                case HX_TEXTURE_BC1_RGB: decode_colour(b, false, false, px); break;
                case HX_TEXTURE_BC1_RGBA: decode_colour(b, false, true, px); break;
                case HX_TEXTURE_BC2:
                    decode_colour(b + 8, true, false, px);
                    for (int t = 0; t < 16; ++t) px[t][3] = (uint8_t)(((le64(b) >> (4 * t)) & 15u) * 17u);
                    break;
                case HX_TEXTURE_BC3:
                    decode_colour(b + 8, true, false, px);
                    decode_channel(b, ch);
                    for (int t = 0; t < 16; ++t) px[t][3] = ch[t];
                    break;
                case HX_TEXTURE_BC4:
                    decode_channel(b, ch);
                    for (int t = 0; t < 16; ++t) { px[t][0] = ch[t]; px[t][1] = px[t][2] = 0; px[t][3] = 255; }
                    break;
                default:  // BC5
                    decode_channel(b, ch);
                    for (int t = 0; t < 16; ++t) { px[t][0] = ch[t]; px[t][2] = 0; px[t][3] = 255; }
                    decode_channel(b + 8, ch);
                    for (int t = 0; t < 16; ++t) px[t][1] = ch[t];
                    break;
            }
            for (uint32_t t = 0; t < 16; ++t) {
                const uint32_t x = bx * 4 + (t & 3), y = by * 4 + (t >> 2);
                if (x < W && y < H) std::copy(px[t], px[t] + 4, out + ((size_t)y * W + x) * 4);
            }
        }
    return HX_OK;
}
