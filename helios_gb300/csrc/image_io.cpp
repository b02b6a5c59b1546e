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
    return (fmt == HX_TEXTURE_BC1_RGB || fmt == HX_TEXTURE_BC1_RGBA || fmt == HX_TEXTURE_BC4) ? 8u : 16u;  // BC2/3/5/7: 16
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

// ---- BC7 (BPTC UNORM; Khronos Data Format Specification, "BC7") -----------
// Eight modes, chosen by the position of the first set bit of the block.  A
// mode fixes the number of subsets (1-3), the partition and rotation fields,
// the endpoint precision (colour / alpha bits, per-endpoint or shared
// p-bits) and the index precision (one or two index sets).  Endpoints widen
// to 8 bits by bit replication, interpolate with the 6-bit weights
// ((64 - w) e0 + w e1 + 32) >> 6; the first index of each subset (its
// anchor) is stored with one bit less.  A block with no mode bit decodes to
// zero.
struct Bc7Mode {
    int subsets, partition_bits, rotation_bits, index_select_bits;
    int colour_bits, alpha_bits, endpoint_pbits, shared_pbits, index_bits, index2_bits;
};
const Bc7Mode kBc7Modes[8] = {
    {3, 4, 0, 0, 4, 0, 1, 0, 3, 0}, {2, 6, 0, 0, 6, 0, 0, 1, 3, 0}, {3, 6, 0, 0, 5, 0, 0, 0, 2, 0},
    {2, 6, 0, 0, 7, 0, 1, 0, 2, 0}, {1, 0, 2, 1, 5, 6, 0, 0, 2, 3}, {1, 0, 2, 0, 7, 8, 0, 0, 2, 2},
    {1, 0, 0, 0, 7, 7, 1, 0, 4, 0}, {2, 6, 0, 0, 5, 5, 1, 0, 2, 0}};
// Two-subset partitions: bit t set = texel t in subset 1 (texel t = x + 4 y).
const uint16_t kBc7Part2[64] = {
    0xCCCC, 0x8888, 0xEEEE, 0xECC8, 0xC880, 0xFEEC, 0xFEC8, 0xEC80, 0xC800, 0xFFEC, 0xFE80, 0xE800, 0xFFE8,
    0xFF00, 0xFFF0, 0xF000, 0xF710, 0x008E, 0x7100, 0x08CE, 0x008C, 0x7310, 0x3100, 0x8CCE, 0x088C, 0x3110,
    0x6666, 0x366C, 0x17E8, 0x0FF0, 0x718E, 0x399C, 0xAAAA, 0xF0F0, 0x5A5A, 0x33CC, 0x3C3C, 0x55AA, 0x9696,
    0xA55A, 0x73CE, 0x13C8, 0x324C, 0x3BDC, 0x6996, 0xC33C, 0x9966, 0x0660, 0x0272, 0x04E4, 0x4E40, 0x2720,
    0xC936, 0x936C, 0x39C6, 0x639C, 0x9336, 0x9CC6, 0x817E, 0xE718, 0xCCF0, 0x0FCC, 0x7744, 0xEE22};
// Three-subset partitions: two bits per texel (texel t at bits 2t).
const uint32_t kBc7Part3[64] = {
    0xAA685050, 0x6A5A5040, 0x5A5A4200, 0x5450A0A8, 0xA5A50000, 0xA0A05050, 0x5555A0A0, 0x5A5A5050,
    0xAA550000, 0xAA555500, 0xAAAA5500, 0x90909090, 0x94949494, 0xA4A4A4A4, 0xA9A59450, 0x2A0A4250,
    0xA5945040, 0x0A425054, 0xA5A5A500, 0x55A0A0A0, 0xA8A85454, 0x6A6A4040, 0xA4A45000, 0x1A1A0500,
    0x0050A4A4, 0xAAA59090, 0x14696914, 0x69691400, 0xA08585A0, 0xAA821414, 0x50A4A450, 0x6A5A0200,
    0xA9A58000, 0x5090A0A8, 0xA8A09050, 0x24242424, 0x00AA5500, 0x24924924, 0x24499224, 0x50A50A50,
    0x500AA550, 0xAAAA4444, 0x66660000, 0xA5A0A5A0, 0x50A050A0, 0x69286928, 0x44AAAA44, 0x66666600,
    0xAA444444, 0x54A854A8, 0x95809580, 0x96969600, 0xA85454A8, 0x80959580, 0xAA141414, 0x96960000,
    0xAAAA1414, 0xA05050A0, 0xA0A5A5A0, 0x96000000, 0x40804080, 0xA9A8A9A8, 0xAAAAAA44, 0x2A4A5254};
// Anchor texel of subset 1 (two subsets), of subsets 1 and 2 (three subsets).
const uint8_t kBc7Anchor2[64] = {15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 2,  8,  2,  2,  8,
                                 8,  15, 2,  8,  2,  2,  8,  8,  2,  2,  15, 15, 6,  8,  2,  8,  15, 15, 2,  8,  2,  2,
                                 2,  15, 15, 6,  6,  2,  6,  8,  15, 15, 2,  2,  15, 15, 15, 15, 15, 2,  2,  15};
const uint8_t kBc7Anchor3a[64] = {3,  3,  15, 15, 8,  3,  15, 15, 8,  8,  6,  6,  6,  5,  3,  3,  3,  3,  8,  15, 3,  3,
                                  6,  10, 5,  8,  8,  6,  8,  5,  15, 15, 8,  15, 3,  5,  6,  10, 8,  15, 15, 3,  15, 5,
                                  15, 15, 15, 15, 3,  15, 5,  5,  5,  8,  5,  10, 5,  10, 8,  13, 15, 12, 3,  3};
const uint8_t kBc7Anchor3b[64] = {15, 8,  8,  3,  15, 15, 3,  8,  15, 15, 15, 15, 15, 15, 15, 8,  15, 8,  15, 3,  15, 8,
                                  15, 8,  3,  15, 6,  10, 15, 15, 10, 8,  15, 3,  15, 10, 10, 8,  9,  10, 6,  15, 8,  15,
                                  3,  6,  6,  8,  15, 3,  15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 3,  15, 15, 8};
const uint8_t kBc7W2[4] = {0, 21, 43, 64};
const uint8_t kBc7W3[8] = {0, 9, 18, 27, 37, 46, 55, 64};
const uint8_t kBc7W4[16] = {0, 4, 9, 13, 17, 21, 26, 30, 34, 38, 43, 47, 51, 55, 60, 64};

struct BitReader {
    const uint8_t* b;
    int pos = 0;
    uint32_t get(int n) {
        uint32_t v = 0;
        for (int k = 0; k < n; ++k, ++pos) v |= (uint32_t)((b[pos >> 3] >> (pos & 7)) & 1u) << k;
        return v;
    }
};

uint32_t bc7_interp(uint32_t e0, uint32_t e1, uint32_t idx, int bits) {
    const uint8_t* w = bits == 2 ? kBc7W2 : (bits == 3 ? kBc7W3 : kBc7W4);
    return ((64u - w[idx]) * e0 + w[idx] * e1 + 32u) >> 6;
}

void decode_bc7(const uint8_t* blk, uint8_t out[16][4]) {
    int mode = 0;
    while (mode < 8 && !(blk[0] & (1u << mode))) ++mode;
    if (mode == 8) {
        for (int t = 0; t < 16; ++t) out[t][0] = out[t][1] = out[t][2] = out[t][3] = 0;
        return;
    }
    const Bc7Mode& M = kBc7Modes[mode];
    BitReader br{blk};
    br.get(mode + 1);
    const uint32_t part = br.get(M.partition_bits);
    const uint32_t rot = br.get(M.rotation_bits);
    const uint32_t isel = br.get(M.index_select_bits);
    const int ne = 2 * M.subsets;
    uint32_t e[6][4];
    for (int ch = 0; ch < 3; ++ch)
        for (int k = 0; k < ne; ++k) e[k][ch] = br.get(M.colour_bits);
    for (int k = 0; k < ne; ++k) e[k][3] = M.alpha_bits ? br.get(M.alpha_bits) : 255u;
    int cbits = M.colour_bits, abits = M.alpha_bits;
    if (M.endpoint_pbits || M.shared_pbits) {
        uint32_t pb[6];
        if (M.endpoint_pbits)
            for (int k = 0; k < ne; ++k) pb[k] = br.get(1);
        else
            for (int s = 0; s < M.subsets; ++s) pb[2 * s] = pb[2 * s + 1] = br.get(1);
        for (int k = 0; k < ne; ++k) {
            for (int ch = 0; ch < 3; ++ch) e[k][ch] = (e[k][ch] << 1) | pb[k];
            if (abits) e[k][3] = (e[k][3] << 1) | pb[k];
        }
        ++cbits;
        if (abits) ++abits;
    }
    for (int k = 0; k < ne; ++k) {
        for (int ch = 0; ch < 3; ++ch) e[k][ch] = (e[k][ch] << (8 - cbits)) | (e[k][ch] >> (2 * cbits - 8));
        if (abits) e[k][3] = (e[k][3] << (8 - abits)) | (e[k][3] >> (2 * abits - 8));
    }
    uint32_t subset[16], anchor[3] = {0, 0, 0};
    for (int t = 0; t < 16; ++t)
        subset[t] = M.subsets == 1 ? 0u : (M.subsets == 2 ? (kBc7Part2[part] >> t) & 1u : (kBc7Part3[part] >> (2 * t)) & 3u);
    if (M.subsets == 2) anchor[1] = kBc7Anchor2[part];
    if (M.subsets == 3) {
        anchor[1] = kBc7Anchor3a[part];
        anchor[2] = kBc7Anchor3b[part];
    }
    auto is_anchor = [&](int t) {
        for (int s = 0; s < M.subsets; ++s)
            if ((uint32_t)t == anchor[s]) return true;
        return false;
    };
    uint32_t idx1[16], idx2[16];
    for (int t = 0; t < 16; ++t) idx1[t] = br.get(M.index_bits - (is_anchor(t) ? 1 : 0));
    if (M.index2_bits)
        for (int t = 0; t < 16; ++t) idx2[t] = br.get(M.index2_bits - (t == 0 ? 1 : 0));
    for (int t = 0; t < 16; ++t) {
        const uint32_t s = subset[t];
        const uint32_t* e0 = e[2 * s];
        const uint32_t* e1 = e[2 * s + 1];
        uint32_t c[4];
        if (M.index2_bits) {
            // modes 4 and 5: colour from one index set, alpha from the other
            // (mode 4 swaps the sets when its selection bit is set)
            const uint32_t ci = isel ? idx2[t] : idx1[t], ai = isel ? idx1[t] : idx2[t];
            const int cb = isel ? M.index2_bits : M.index_bits, ab = isel ? M.index_bits : M.index2_bits;
            for (int ch = 0; ch < 3; ++ch) c[ch] = bc7_interp(e0[ch], e1[ch], ci, cb);
            c[3] = bc7_interp(e0[3], e1[3], ai, ab);
        } else {
            for (int ch = 0; ch < 4; ++ch) c[ch] = bc7_interp(e0[ch], e1[ch], idx1[t], M.index_bits);
        }
        if (rot) std::swap(c[3], c[rot - 1]);  // 1: swap A,R; 2: A,G; 3: A,B
        for (int ch = 0; ch < 4; ++ch) out[t][ch] = (uint8_t)c[ch];
    }
}

// ---- BC6H (BPTC half-float RGB; Khronos Data Format Specification, "BC6H") -
// Fourteen modes, chosen by the low two bits of the block (00, 01) or, when
// those are 10 or 11, by its low five bits (four five-bit codes are
// reserved).  A mode fixes one or two regions (the two-region partitions are
// the first 32 of BC7's), the endpoint precision, and whether endpoints 1-3
// are stored as signed deltas from endpoint 0 ("transformed", with the delta
// widths of the mode).  The mode's header bits scatter the endpoint fields; a
// layout below lists them in stored order as <channel><endpoint><hi>[:<lo>]
// (endpoints w, x = region 0, y, z = region 1), the bits of a field stored
// from <lo> towards <hi>, so "rw10:11" stores bit 11 first.  Endpoints widen
// to 16 bits (unquantisation), interpolate with the BC7 weights and scale to
// the half-float bit pattern (x 31/64 unsigned, x 31/32 signed magnitude).
struct Bc6Mode {
    int regions;
    bool transformed;
    int epb;       // endpoint precision (bits)
    int delta[3];  // stored widths of endpoints 1-3 per channel
    const char* layout;
};
const Bc6Mode kBc6Modes[14] = {
    {2, true, 10, {5, 5, 5},
     "gy4 by4 bz4 rw9:0 gw9:0 bw9:0 rx4:0 gz4 gy3:0 gx4:0 bz0 gz3:0 bx4:0 bz1 by3:0 ry4:0 bz2 rz4:0 bz3"},
    {2, true, 7, {6, 6, 6},
     "gy5 gz4 gz5 rw6:0 bz0 bz1 by4 gw6:0 by5 bz2 gy4 bw6:0 bz3 bz5 bz4 rx5:0 gy3:0 gx5:0 gz3:0 bx5:0 by3:0 ry5:0 "
     "rz5:0"},
    {2, true, 11, {5, 4, 4},
     "rw9:0 gw9:0 bw9:0 rx4:0 rw10 gy3:0 gx3:0 gw10 bz0 gz3:0 bx3:0 bw10 bz1 by3:0 ry4:0 bz2 rz4:0 bz3"},
    {2, true, 11, {4, 5, 4},
     "rw9:0 gw9:0 bw9:0 rx3:0 rw10 gz4 gy3:0 gx4:0 gw10 gz3:0 bx3:0 bw10 bz1 by3:0 ry3:0 bz0 bz2 rz3:0 gy4 bz3"},
    {2, true, 11, {4, 4, 5},
     "rw9:0 gw9:0 bw9:0 rx3:0 rw10 by4 gy3:0 gx3:0 gw10 bz0 gz3:0 bx4:0 bw10 by3:0 ry3:0 bz1 bz2 rz3:0 bz4 bz3"},
    {2, true, 9, {5, 5, 5},
     "rw8:0 by4 gw8:0 gy4 bw8:0 bz4 rx4:0 gz4 gy3:0 gx4:0 bz0 gz3:0 bx4:0 bz1 by3:0 ry4:0 bz2 rz4:0 bz3"},
    {2, true, 8, {6, 5, 5},
     "rw7:0 gz4 by4 gw7:0 bz2 gy4 bw7:0 bz3 bz4 rx5:0 gy3:0 gx4:0 bz0 gz3:0 bx4:0 bz1 by3:0 ry5:0 rz5:0"},
    {2, true, 8, {5, 6, 5},
     "rw7:0 bz0 by4 gw7:0 gy5 gy4 bw7:0 gz5 bz4 rx4:0 gz4 gy3:0 gx5:0 gz3:0 bx4:0 bz1 by3:0 ry4:0 bz2 rz4:0 bz3"},
    {2, true, 8, {5, 5, 6},
     "rw7:0 bz1 by4 gw7:0 by5 gy4 bw7:0 bz5 bz4 rx4:0 gz4 gy3:0 gx4:0 bz0 gz3:0 bx5:0 by3:0 ry4:0 bz2 rz4:0 bz3"},
    {2, false, 6, {6, 6, 6},
     "rw5:0 gz4 bz0 bz1 by4 gw5:0 gy5 by5 bz2 gy4 bw5:0 gz5 bz3 bz5 bz4 rx5:0 gy3:0 gx5:0 gz3:0 bx5:0 by3:0 ry5:0 "
     "rz5:0"},
    {1, false, 10, {10, 10, 10}, "rw9:0 gw9:0 bw9:0 rx9:0 gx9:0 bx9:0"},
    {1, true, 11, {9, 9, 9}, "rw9:0 gw9:0 bw9:0 rx8:0 rw10 gx8:0 gw10 bx8:0 bw10"},
    {1, true, 12, {8, 8, 8}, "rw9:0 gw9:0 bw9:0 rx7:0 rw10:11 gx7:0 gw10:11 bx7:0 bw10:11"},
    {1, true, 16, {4, 4, 4}, "rw9:0 gw9:0 bw9:0 rx3:0 rw10:15 gx3:0 gw10:15 bx3:0 bw10:15"},
};

// Mode index of a block, -1 for the reserved codes.
int bc6_mode(const uint8_t* blk) {
    const uint32_t m2 = blk[0] & 3u;
    if (m2 < 2) return (int)m2;
    switch (blk[0] & 31u) {
        case 2: return 2;
        case 6: return 3;
        case 10: return 4;
        case 14: return 5;
        case 18: return 6;
        case 22: return 7;
        case 26: return 8;
        case 30: return 9;
        case 3: return 10;
        case 7: return 11;
        case 11: return 12;
        case 15: return 13;
        default: return -1;
    }
}

// Reads the endpoint fields of a mode's layout: e[endpoint][channel], raw bits.
void bc6_read_endpoints(const char* layout, BitReader& br, int32_t e[4][3]) {
    for (const char* p = layout; *p;) {
        while (*p == ' ') ++p;
        if (!*p) break;
        const int ch = *p == 'r' ? 0 : (*p == 'g' ? 1 : 2);
        ++p;
        const int ep = *p - 'w';  // w x y z -> 0 1 2 3
        ++p;
        int hi = 0, lo;
        while (*p >= '0' && *p <= '9') hi = 10 * hi + (*p++ - '0');
        lo = hi;
        if (*p == ':') {
            ++p;
            lo = 0;
            while (*p >= '0' && *p <= '9') lo = 10 * lo + (*p++ - '0');
        }
        const int step = hi >= lo ? 1 : -1;
        for (int b = lo;; b += step) {
            e[ep][ch] |= (int32_t)br.get(1) << b;
            if (b == hi) break;
        }
    }
}

int32_t sign_extend(int32_t v, int bits) {
    const int32_t m = 1 << (bits - 1);
    v &= (1 << bits) - 1;
    return (v ^ m) - m;
}

int32_t bc6_unquantize(int32_t c, int epb, bool is_signed) {
    if (!is_signed) {
        if (epb >= 15) return c;
        if (c == 0) return 0;
        if (c == (1 << epb) - 1) return 0xFFFF;
        return ((c << 16) + 0x8000) >> epb;
    }
    if (epb >= 16) return c;
    const bool neg = c < 0;
    int32_t m = neg ? -c : c, u;
    if (m == 0) u = 0;
    else if (m >= (1 << (epb - 1)) - 1) u = 0x7FFF;
    else u = ((m << 15) + 0x4000) >> (epb - 1);
    return neg ? -u : u;
}

// floor(v / 64) for any sign
int32_t floor_div64(int32_t v) { return v >= 0 ? v >> 6 : -((-v + 63) >> 6); }

uint16_t bc6_finish(int32_t c, bool is_signed) {
    if (!is_signed) return (uint16_t)((c * 31) >> 6);
    if (c < 0) {
        const int32_t m = ((-c) * 31) >> 5;
        return (uint16_t)(m ? (0x8000 | m) : 0);
    }
    return (uint16_t)((c * 31) >> 5);
}

// One BC6H block to 16 RGBA half-float texels (alpha 1.0); a reserved mode
// decodes to zero colour.
void decode_bc6h(const uint8_t* blk, bool is_signed, uint16_t out[16][4]) {
    const int mi = bc6_mode(blk);
    if (mi < 0) {
        for (int t = 0; t < 16; ++t) {
            out[t][0] = out[t][1] = out[t][2] = 0;
            out[t][3] = 0x3C00;
        }
        return;
    }
    const Bc6Mode& M = kBc6Modes[mi];
    BitReader br{blk};
    br.get(mi < 2 ? 2 : 5);
    int32_t e[4][3] = {};
    bc6_read_endpoints(M.layout, br, e);
    const uint32_t part = M.regions == 2 ? br.get(5) : 0u;
    const int ne = 2 * M.regions;
    for (int c = 0; c < 3; ++c) {
        if (is_signed) e[0][c] = sign_extend(e[0][c], M.epb);
        for (int k = 1; k < ne; ++k) {
            if (M.transformed) {
                const int32_t d = sign_extend(e[k][c], M.delta[c]);
                e[k][c] = (e[0][c] + d) & ((1 << M.epb) - 1);
                if (is_signed) e[k][c] = sign_extend(e[k][c], M.epb);
            } else if (is_signed) {
                e[k][c] = sign_extend(e[k][c], M.epb);
            }
        }
        for (int k = 0; k < ne; ++k) e[k][c] = bc6_unquantize(e[k][c], M.epb, is_signed);
    }
    const int ib = M.regions == 2 ? 3 : 4;
    const uint32_t anchor1 = M.regions == 2 ? kBc7Anchor2[part] : 0u;
    const uint8_t* w = ib == 3 ? kBc7W3 : kBc7W4;
    for (int t = 0; t < 16; ++t) {
        const bool anchor = t == 0 || (M.regions == 2 && (uint32_t)t == anchor1);
        const uint32_t idx = br.get(ib - (anchor ? 1 : 0));
        const uint32_t s = M.regions == 2 ? (kBc7Part2[part] >> t) & 1u : 0u;
        for (int c = 0; c < 3; ++c) {
            const int32_t v = floor_div64(e[2 * s][c] * (64 - (int32_t)w[idx]) + e[2 * s + 1][c] * (int32_t)w[idx] + 32);
            out[t][c] = bc6_finish(v, is_signed);
        }
        out[t][3] = 0x3C00;
    }
}

}  // namespace

extern "C" hx_status hx_texture_decode_hdr(const hx_texture_desc* tex, uint16_t* out) {
    HX_CHECK_ARG(tex && out && tex->rgba8 && tex->width > 0 && tex->height > 0,
                 "hx_texture_decode_hdr: null argument or empty texture");
    HX_CHECK_ARG(tex->format >= HX_TEXTURE_BC6H_SF16 && tex->format <= HX_TEXTURE_RGBA16F,
                 "hx_texture_decode_hdr: format %u is not a half-float format (8-bit formats: hx_texture_decode)",
                 tex->format);
    const uint32_t W = tex->width, H = tex->height;
    if (tex->format == HX_TEXTURE_RGBA16F) {
        const uint8_t* src = tex->rgba8;
        for (size_t i = 0; i < (size_t)W * H * 4; ++i) out[i] = (uint16_t)(src[2 * i] | (src[2 * i + 1] << 8));
        return HX_OK;
    }
    const bool is_signed = tex->format == HX_TEXTURE_BC6H_SF16;
    const uint32_t bw = (W + 3) / 4, bh = (H + 3) / 4;
    for (uint32_t by = 0; by < bh; ++by)
        for (uint32_t bx = 0; bx < bw; ++bx) {
            uint16_t px[16][4];
            decode_bc6h(tex->rgba8 + ((size_t)by * bw + bx) * 16, is_signed, px);
            for (uint32_t t = 0; t < 16; ++t) {
                const uint32_t x = bx * 4 + (t & 3), y = by * 4 + (t >> 2);
                if (x < W && y < H) std::copy(px[t], px[t] + 4, out + ((size_t)y * W + x) * 4);
            }
        }
    return HX_OK;
}

extern "C" hx_status hx_texture_decode(const hx_texture_desc* tex, uint8_t* out) {
    HX_CHECK_ARG(tex && out && tex->rgba8 && tex->width > 0 && tex->height > 0, "hx_texture_decode: null argument or empty texture");
    HX_CHECK_ARG(tex->format <= HX_TEXTURE_BC7 || tex->format == HX_TEXTURE_RGBA8_SNORM,
                 "hx_texture_decode: format %u is not an 8-bit format (half-float formats: hx_texture_decode_hdr)",
                 tex->format);
    const uint32_t W = tex->width, H = tex->height;
    if (tex->format == HX_TEXTURE_RGBA8 || tex->format == HX_TEXTURE_RGBA8_SNORM) {  // the bytes as they are
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
                case HX_TEXTURE_BC7: decode_bc7(b, px); break;
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
