"""Block-compressed texture decoding, restated in numpy (TEST INFRASTRUCTURE).

The checker for the library's hx_texture_decode.  The formats are the BCn
(S3TC / RGTC) blocks the reference's assets carry (kCompressedFormats,
src/engine/core/resource_manager.cpp:14-30), as published in the Khronos
Data Format Specification (S3TC and RGTC sections):

* colour block (8 bytes): two little-endian RGB565 endpoints c0, c1, then
  sixteen 2-bit indices (texel t at bits 2t).  Endpoints widen to 8 bits by
  bit replication.  Four-colour mode (c0 > c1, and always inside BC2/BC3):
  the two middle entries are 2/3 c0 + 1/3 c1 and 1/3 c0 + 2/3 c1.  Otherwise
  entry 2 is the mean and entry 3 black — transparent for BC1 with alpha.
* channel block (8 bytes, BC4 and the alpha of BC3): endpoints a0, a1, then
  sixteen 3-bit indices (texel t at bits 3t of the 48-bit tail).  a0 > a1:
  six interpolated values in sevenths; otherwise four in fifths, then 0, 255.
* BC2 alpha: sixteen 4-bit values (texel t at bits 4t), widened by * 17.
* BC7 (BPTC): eight modes selected by the first set bit; 1-3 subsets chosen
  by a partition table, endpoints with optional p-bits widened by bit
  replication, anchor indices one bit shorter, interpolation
  ((64 - w) e0 + w e1 + 32) >> 6 with the 2/3/4-bit weight tables, optional
  channel rotation and a second index set (modes 4 and 5).
* BC6H (BPTC half float): fourteen modes chosen by the low two bits (00, 01)
  or low five bits of the block; one or two regions (the two-region
  partitions are BC7's first 32); endpoint fields scattered through the
  header in a per-mode order; endpoints 1-3 optionally stored as signed
  deltas from endpoint 0; endpoints unquantised to 16 bits, interpolated
  with BC7's 3- or 4-bit weights in integers, then scaled to the half-float
  bit pattern (x 31/64, or for the signed format the magnitude x 31/32 with
  the sign bit).  Reserved mode codes decode to zero colour; alpha is 1.0.

The specification leaves the rounding of interpolated entries to the
implementation; this library rounds to nearest in integers and so does
this restatement.
"""
import numpy as np

BC1_RGB, BC1_RGBA, BC2, BC3, BC4, BC5, BC7 = 1, 2, 3, 4, 5, 6, 7
BC6H_SF16, BC6H_UF16 = 8, 9
BLOCK_BYTES = {BC1_RGB: 8, BC1_RGBA: 8, BC2: 16, BC3: 16, BC4: 8, BC5: 16, BC7: 16}

# BC7 (BPTC), Khronos Data Format Specification: per mode (subsets,
# partition bits, rotation bits, index-selection bits, colour bits, alpha
# bits, per-endpoint p-bits, shared p-bits, index bits, second index bits)
BC7_MODES = [(3, 4, 0, 0, 4, 0, 1, 0, 3, 0), (2, 6, 0, 0, 6, 0, 0, 1, 3, 0), (3, 6, 0, 0, 5, 0, 0, 0, 2, 0),
             (2, 6, 0, 0, 7, 0, 1, 0, 2, 0), (1, 0, 2, 1, 5, 6, 0, 0, 2, 3), (1, 0, 2, 0, 7, 8, 0, 0, 2, 2),
             (1, 0, 0, 0, 7, 7, 1, 0, 4, 0), (2, 6, 0, 0, 5, 5, 1, 0, 2, 0)]
# partitions as rows of subset digits, texel t = x + 4 y
BC7_PART2 = [
    "0011001100110011", "0001000100010001", "0111011101110111", "0001001100110111", "0000000100010011",
    "0011011101111111", "0001001101111111", "0000000100110111", "0000000000010011", "0011011111111111",
    "0000000101111111", "0000000000010111", "0001011111111111", "0000000011111111", "0000111111111111",
    "0000000000001111", "0000100011101111", "0111000100000000", "0000000010001110", "0111001100010000",
    "0011000100000000", "0000100011001110", "0000000010001100", "0111001100110001", "0011000100010000",
    "0000100010001100", "0110011001100110", "0011011001101100", "0001011111101000", "0000111111110000",
    "0111000110001110", "0011100110011100", "0101010101010101", "0000111100001111", "0101101001011010",
    "0011001111001100", "0011110000111100", "0101010110101010", "0110100101101001", "0101101010100101",
    "0111001111001110", "0001001111001000", "0011001001001100", "0011101111011100", "0110100110010110",
    "0011110011000011", "0110011010011001", "0000011001100000", "0100111001000000", "0010011100100000",
    "0000001001110010", "0000010011100100", "0110110010010011", "0011011011001001", "0110001110011100",
    "0011100111000110", "0110110011001001", "0110001100111001", "0111111010000001", "0001100011100111",
    "0000111100110011", "0011001111110000", "0010001011101110", "0100010001110111"]
BC7_PART3 = [
    "0011001102212222", "0001001122112221", "0000200122112211", "0222002200110111", "0000000011221122",
    "0011001100220022", "0022002211111111", "0011001122112211", "0000000011112222", "0000111111112222",
    "0000111122222222", "0012001200120012", "0112011201120112", "0122012201220122", "0011011211221222",
    "0011200122002220", "0001001101121122", "0111001120012200", "0000112211221122", "0022002200221111",
    "0111011102220222", "0001000122212221", "0000001101220122", "0000110022102210", "0122012200110000",
    "0012001211222222", "0110122112210110", "0000011012211221", "0022110211020022", "0110011020022222",
    "0011012201220011", "0000200022112221", "0000000211221222", "0222002200120011", "0011001200220222",
    "0120012001200120", "0000111122220000", "0120120120120120", "0120201212010120", "0011220011220011",
    "0011112222000011", "0101010122222222", "0000000021212121", "0022112200221122", "0022001100220011",
    "0220122102201221", "0101222222220101", "0000212121212121", "0101010101012222", "0222011102220111",
    "0002111200021112", "0000211221122112", "0222011101110222", "0002111211120002", "0110011001102222",
    "0000000021122112", "0110011022222222", "0022001100110022", "0022112211220022", "0000000000002112",
    "0002000100020001", "0222122202221222", "0101222222222222", "0111201122012220"]
BC7_ANCHOR2 = [15] * 16 + [15, 2, 8, 2, 2, 8, 8, 15, 2, 8, 2, 2, 8, 8, 2, 2, 15, 15, 6, 8, 2, 8, 15, 15, 2, 8, 2, 2,
                          2, 15, 15, 6, 6, 2, 6, 8, 15, 15, 2, 2, 15, 15, 15, 15, 15, 2, 2, 15]
BC7_ANCHOR3A = [3, 3, 15, 15, 8, 3, 15, 15, 8, 8, 6, 6, 6, 5, 3, 3, 3, 3, 8, 15, 3, 3, 6, 10, 5, 8, 8, 6, 8, 5, 15, 15,
                8, 15, 3, 5, 6, 10, 8, 15, 15, 3, 15, 5, 15, 15, 15, 15, 3, 15, 5, 5, 5, 8, 5, 10, 5, 10, 8, 13, 15, 12,
                3, 3]
BC7_ANCHOR3B = [15, 8, 8, 3, 15, 15, 3, 8, 15, 15, 15, 15, 15, 15, 15, 8, 15, 8, 15, 3, 15, 8, 15, 8, 3, 15, 6, 10, 15,
                15, 10, 8, 15, 3, 15, 10, 10, 8, 9, 10, 6, 15, 8, 15, 3, 6, 6, 8, 15, 3, 15, 15, 15, 15, 15, 15, 15, 15,
                15, 15, 3, 15, 15, 8]
BC7_WEIGHTS = {2: [0, 21, 43, 64], 3: [0, 9, 18, 27, 37, 46, 55, 64],
               4: [0, 4, 9, 13, 17, 21, 26, 30, 34, 38, 43, 47, 51, 55, 60, 64]}


def decode_bc7_block(block):
    """16 RGBA texels of one 16-byte BC7 block (texel t = x + 4 y)."""
    bits = int.from_bytes(bytes(block), "little")
    pos = [0]

    def take(n):
        v = (bits >> pos[0]) & ((1 << n) - 1)
        pos[0] += n
        return v
    mode = next((m for m in range(8) if (bits >> m) & 1), 8)
    if mode == 8:
        return [[0, 0, 0, 0] for _ in range(16)]
    ns, pb, rb, isb, cb, ab, epb, spb, ib, ib2 = BC7_MODES[mode]
    take(mode + 1)
    part, rot, isel = take(pb), take(rb), take(isb)
    ends = [[0, 0, 0, 255] for _ in range(2 * ns)]
    for ch in range(3):
        for e in ends:
            e[ch] = take(cb)
    if ab:
        for e in ends:
            e[3] = take(ab)
    if epb or spb:
        p = [take(1) for _ in range(2 * ns)] if epb else [b for s in range(ns) for b in [take(1)] * 2]
        for e, pbit in zip(ends, p):
            for ch in range(3):
                e[ch] = (e[ch] << 1) | pbit
            if ab:
                e[3] = (e[3] << 1) | pbit
        cb, ab = cb + 1, (ab + 1 if ab else 0)
    for e in ends:
        for ch in range(3):
            e[ch] = (e[ch] << (8 - cb)) | (e[ch] >> (2 * cb - 8))
        if ab:
            e[3] = (e[3] << (8 - ab)) | (e[3] >> (2 * ab - 8))
    if ns == 1:
        subset, anchors = [0] * 16, {0}
    elif ns == 2:
        subset, anchors = [int(c) for c in BC7_PART2[part]], {0, BC7_ANCHOR2[part]}
    else:
        subset, anchors = [int(c) for c in BC7_PART3[part]], {0, BC7_ANCHOR3A[part], BC7_ANCHOR3B[part]}
    idx1 = [take(ib - (1 if t in anchors else 0)) for t in range(16)]
    idx2 = [take(ib2 - (1 if t == 0 else 0)) for t in range(16)] if ib2 else None

    def lerp(a, b, i, n):
        w = BC7_WEIGHTS[n][i]
        return ((64 - w) * a + w * b + 32) >> 6
    out = []
    for t in range(16):
        e0, e1 = ends[2 * subset[t]], ends[2 * subset[t] + 1]
        if ib2:
            ci, ai, cn, an = (idx2[t], idx1[t], ib2, ib) if isel else (idx1[t], idx2[t], ib, ib2)
            c = [lerp(e0[ch], e1[ch], ci, cn) for ch in range(3)] + [lerp(e0[3], e1[3], ai, an)]
        else:
            c = [lerp(e0[ch], e1[ch], idx1[t], ib) for ch in range(4)]
        if rot:
            c[3], c[rot - 1] = c[rot - 1], c[3]
        out.append(c)
    return out


def _bits(field, *spec):
    """Storage-order bit list of one endpoint field: spec items are value-bit
    numbers or (lo, hi) runs stored from lo to hi (hi < lo: stored reversed)."""
    out = []
    for s in spec:
        if isinstance(s, tuple):
            lo, hi = s
            step = 1 if hi >= lo else -1
            out += [(field, b) for b in range(lo, hi + step, step)]
        else:
            out.append((field, s))
    return out


def _layout(*items):
    return [fb for it in items for fb in it]


R = _bits
# per mode code: (mode bits, regions, transformed, endpoint bits, delta bits (r, g, b), header layout after the
# mode bits as (field, value bit) in storage order; fields r/g/b + endpoint w, x (region 0), y, z (region 1))
BC6H_MODES = {
    0b00: (2, 2, True, 10, (5, 5, 5), _layout(
        R("gy", 4), R("by", 4), R("bz", 4), R("rw", (0, 9)), R("gw", (0, 9)), R("bw", (0, 9)), R("rx", (0, 4)),
        R("gz", 4), R("gy", (0, 3)), R("gx", (0, 4)), R("bz", 0), R("gz", (0, 3)), R("bx", (0, 4)), R("bz", 1),
        R("by", (0, 3)), R("ry", (0, 4)), R("bz", 2), R("rz", (0, 4)), R("bz", 3))),
    0b01: (2, 2, True, 7, (6, 6, 6), _layout(
        R("gy", 5), R("gz", 4, 5), R("rw", (0, 6)), R("bz", 0, 1), R("by", 4), R("gw", (0, 6)), R("by", 5),
        R("bz", 2), R("gy", 4), R("bw", (0, 6)), R("bz", 3, 5, 4), R("rx", (0, 5)), R("gy", (0, 3)),
        R("gx", (0, 5)), R("gz", (0, 3)), R("bx", (0, 5)), R("by", (0, 3)), R("ry", (0, 5)), R("rz", (0, 5)))),
    0b00010: (5, 2, True, 11, (5, 4, 4), _layout(
        R("rw", (0, 9)), R("gw", (0, 9)), R("bw", (0, 9)), R("rx", (0, 4)), R("rw", 10), R("gy", (0, 3)),
        R("gx", (0, 3)), R("gw", 10), R("bz", 0), R("gz", (0, 3)), R("bx", (0, 3)), R("bw", 10), R("bz", 1),
        R("by", (0, 3)), R("ry", (0, 4)), R("bz", 2), R("rz", (0, 4)), R("bz", 3))),
    0b00110: (5, 2, True, 11, (4, 5, 4), _layout(
        R("rw", (0, 9)), R("gw", (0, 9)), R("bw", (0, 9)), R("rx", (0, 3)), R("rw", 10), R("gz", 4),
        R("gy", (0, 3)), R("gx", (0, 4)), R("gw", 10), R("gz", (0, 3)), R("bx", (0, 3)), R("bw", 10), R("bz", 1),
        R("by", (0, 3)), R("ry", (0, 3)), R("bz", 0, 2), R("rz", (0, 3)), R("gy", 4), R("bz", 3))),
    0b01010: (5, 2, True, 11, (4, 4, 5), _layout(
        R("rw", (0, 9)), R("gw", (0, 9)), R("bw", (0, 9)), R("rx", (0, 3)), R("rw", 10), R("by", 4),
        R("gy", (0, 3)), R("gx", (0, 3)), R("gw", 10), R("bz", 0), R("gz", (0, 3)), R("bx", (0, 4)), R("bw", 10),
        R("by", (0, 3)), R("ry", (0, 3)), R("bz", 1, 2), R("rz", (0, 3)), R("bz", 4, 3))),
    0b01110: (5, 2, True, 9, (5, 5, 5), _layout(
        R("rw", (0, 8)), R("by", 4), R("gw", (0, 8)), R("gy", 4), R("bw", (0, 8)), R("bz", 4), R("rx", (0, 4)),
        R("gz", 4), R("gy", (0, 3)), R("gx", (0, 4)), R("bz", 0), R("gz", (0, 3)), R("bx", (0, 4)), R("bz", 1),
        R("by", (0, 3)), R("ry", (0, 4)), R("bz", 2), R("rz", (0, 4)), R("bz", 3))),
    0b10010: (5, 2, True, 8, (6, 5, 5), _layout(
        R("rw", (0, 7)), R("gz", 4), R("by", 4), R("gw", (0, 7)), R("bz", 2), R("gy", 4), R("bw", (0, 7)),
        R("bz", 3, 4), R("rx", (0, 5)), R("gy", (0, 3)), R("gx", (0, 4)), R("bz", 0), R("gz", (0, 3)),
        R("bx", (0, 4)), R("bz", 1), R("by", (0, 3)), R("ry", (0, 5)), R("rz", (0, 5)))),
    0b10110: (5, 2, True, 8, (5, 6, 5), _layout(
        R("rw", (0, 7)), R("bz", 0), R("by", 4), R("gw", (0, 7)), R("gy", 5, 4), R("bw", (0, 7)), R("gz", 5),
        R("bz", 4), R("rx", (0, 4)), R("gz", 4), R("gy", (0, 3)), R("gx", (0, 5)), R("gz", (0, 3)),
        R("bx", (0, 4)), R("bz", 1), R("by", (0, 3)), R("ry", (0, 4)), R("bz", 2), R("rz", (0, 4)), R("bz", 3))),
    0b11010: (5, 2, True, 8, (5, 5, 6), _layout(
        R("rw", (0, 7)), R("bz", 1), R("by", 4), R("gw", (0, 7)), R("by", 5), R("gy", 4), R("bw", (0, 7)),
        R("bz", 5, 4), R("rx", (0, 4)), R("gz", 4), R("gy", (0, 3)), R("gx", (0, 4)), R("bz", 0),
        R("gz", (0, 3)), R("bx", (0, 5)), R("by", (0, 3)), R("ry", (0, 4)), R("bz", 2), R("rz", (0, 4)),
        R("bz", 3))),
    0b11110: (5, 2, False, 6, (6, 6, 6), _layout(
        R("rw", (0, 5)), R("gz", 4), R("bz", 0, 1), R("by", 4), R("gw", (0, 5)), R("gy", 5), R("by", 5),
        R("bz", 2), R("gy", 4), R("bw", (0, 5)), R("gz", 5), R("bz", 3, 5, 4), R("rx", (0, 5)), R("gy", (0, 3)),
        R("gx", (0, 5)), R("gz", (0, 3)), R("bx", (0, 5)), R("by", (0, 3)), R("ry", (0, 5)), R("rz", (0, 5)))),
    0b00011: (5, 1, False, 10, (10, 10, 10), _layout(
        R("rw", (0, 9)), R("gw", (0, 9)), R("bw", (0, 9)), R("rx", (0, 9)), R("gx", (0, 9)), R("bx", (0, 9)))),
    0b00111: (5, 1, True, 11, (9, 9, 9), _layout(
        R("rw", (0, 9)), R("gw", (0, 9)), R("bw", (0, 9)), R("rx", (0, 8)), R("rw", 10), R("gx", (0, 8)),
        R("gw", 10), R("bx", (0, 8)), R("bw", 10))),
    0b01011: (5, 1, True, 12, (8, 8, 8), _layout(
        R("rw", (0, 9)), R("gw", (0, 9)), R("bw", (0, 9)), R("rx", (0, 7)), R("rw", (11, 10)), R("gx", (0, 7)),
        R("gw", (11, 10)), R("bx", (0, 7)), R("bw", (11, 10)))),
    0b01111: (5, 1, True, 16, (4, 4, 4), _layout(
        R("rw", (0, 9)), R("gw", (0, 9)), R("bw", (0, 9)), R("rx", (0, 3)), R("rw", (15, 10)), R("gx", (0, 3)),
        R("gw", (15, 10)), R("bx", (0, 3)), R("bw", (15, 10)))),
}
del R


def _sext(v, n):
    v &= (1 << n) - 1
    return v - (1 << n) if v >> (n - 1) else v


def _bc6_unq(c, epb, signed):
    if not signed:
        if epb >= 15:
            return c
        if c == 0:
            return 0
        if c == (1 << epb) - 1:
            return 0xFFFF
        return ((c << 16) + 0x8000) >> epb
    if epb >= 16:
        return c
    m = abs(c)
    if m == 0:
        u = 0
    elif m >= (1 << (epb - 1)) - 1:
        u = 0x7FFF
    else:
        u = ((m << 15) + 0x4000) >> (epb - 1)
    return -u if c < 0 else u


def _bc6_half(c, signed):
    if not signed:
        return (c * 31) >> 6
    m = (abs(c) * 31) >> 5
    return (0x8000 | m) if (c < 0 and m) else m


def decode_bc6h_block(block, signed):
    """16 RGBA half-float bit patterns of one 16-byte BC6H block (texel t = x + 4 y)."""
    bits = int.from_bytes(bytes(block), "little")
    code = bits & 3 if (bits & 3) < 2 else bits & 31
    if code not in BC6H_MODES:
        return [[0, 0, 0, 0x3C00] for _ in range(16)]
    nmode, regions, transformed, epb, delta, layout = BC6H_MODES[code]
    pos = nmode
    ep = {f + e: 0 for f in "rgb" for e in "wxyz"}
    for field, b in layout:
        ep[field] |= ((bits >> pos) & 1) << b
        pos += 1
    part = 0
    if regions == 2:
        part = (bits >> pos) & 31
        pos += 5
    names = "wxyz"[: 2 * regions]
    ends = {}
    for ci, ch in enumerate("rgb"):
        w = ep[ch + "w"]
        if signed:
            w = _sext(w, epb)
        vals = [w]
        for e in names[1:]:
            v = ep[ch + e]
            if transformed:
                v = (w + _sext(v, delta[ci])) & ((1 << epb) - 1)
                if signed:
                    v = _sext(v, epb)
            elif signed:
                v = _sext(v, epb)
            vals.append(v)
        ends[ch] = [_bc6_unq(v, epb, signed) for v in vals]
    nbits = 3 if regions == 2 else 4
    subset = [int(c) for c in BC7_PART2[part]] if regions == 2 else [0] * 16
    anchors = {0, BC7_ANCHOR2[part]} if regions == 2 else {0}
    wts = BC7_WEIGHTS[nbits]
    out = []
    for t in range(16):
        n = nbits - (1 if t in anchors else 0)
        idx = (bits >> pos) & ((1 << n) - 1)
        pos += n
        s, w = subset[t], wts[idx]
        px = [_bc6_half((ends[ch][2 * s] * (64 - w) + ends[ch][2 * s + 1] * w + 32) >> 6, signed) for ch in "rgb"]
        out.append(px + [0x3C00])
    return out


def decode_hdr(data, width, height, fmt):
    """(height, width, 4) uint16 half-float bit patterns of width x height BC6H data (row-major blocks)."""
    bw, bh = (width + 3) // 4, (height + 3) // 4
    blocks = np.frombuffer(bytes(data), np.uint8)[: bw * bh * 16].reshape(bw * bh, 16)
    px = np.array([decode_bc6h_block(b, fmt == BC6H_SF16) for b in blocks], np.int64).reshape(bh, bw, 4, 4, 4)
    img = px.transpose(0, 2, 1, 3, 4).reshape(bh * 4, bw * 4, 4)
    return img[:height, :width].astype(np.uint16)


def _le(blocks, off, n):
    v = np.zeros(blocks.shape[0], np.uint64)
    for k in range(n - 1, -1, -1):
        v = (v << np.uint64(8)) | blocks[:, off + k].astype(np.uint64)
    return v


def _colour(blocks, off, four_always, transparent):
    c0 = _le(blocks, off, 2).astype(np.int64)
    c1 = _le(blocks, off + 2, 2).astype(np.int64)
    idx = _le(blocks, off + 4, 4).astype(np.int64)

    def widen(c):
        r, g, b = c >> 11, (c >> 5) & 63, c & 31
        return np.stack([(r << 3) | (r >> 2), (g << 2) | (g >> 4), (b << 3) | (b >> 2)], -1)

    e0, e1 = widen(c0), widen(c1)
    four = (c0 > c1) | four_always
    pal = np.zeros((blocks.shape[0], 4, 4), np.int64)
    pal[:, 0, :3], pal[:, 1, :3] = e0, e1
    pal[:, 2, :3] = np.where(four[:, None], (2 * e0 + e1 + 1) // 3, (e0 + e1 + 1) // 2)
    pal[:, 3, :3] = np.where(four[:, None], (e0 + 2 * e1 + 1) // 3, 0)
    pal[:, :, 3] = 255
    if transparent:
        pal[:, 3, 3] = np.where(four, 255, 0)
    sel = (idx[:, None] >> (2 * np.arange(16))) & 3
    return np.take_along_axis(pal, sel[:, :, None].repeat(4, 2), 1)


def _channel(blocks, off):
    a0 = blocks[:, off].astype(np.int64)
    a1 = blocks[:, off + 1].astype(np.int64)
    idx = _le(blocks, off + 2, 6).astype(np.int64)
    k = np.arange(8)
    sev = ((8 - k)[None] * a0[:, None] + (k - 1)[None] * a1[:, None] + 3) // 7
    fif = ((6 - k)[None] * a0[:, None] + (k - 1)[None] * a1[:, None] + 2) // 5
    fif[:, 6], fif[:, 7] = 0, 255
    pal = np.where((a0 > a1)[:, None], sev, fif)
    pal[:, 0], pal[:, 1] = a0, a1
    sel = (idx[:, None] >> (3 * np.arange(16))) & 7
    return np.take_along_axis(pal, sel, 1)


def decode(data, width, height, fmt):
    """(height, width, 4) uint8 texels of width x height BCn data (row-major blocks)."""
    bw, bh = (width + 3) // 4, (height + 3) // 4
    blocks = np.frombuffer(bytes(data), np.uint8)[: bw * bh * BLOCK_BYTES[fmt]].reshape(bw * bh, BLOCK_BYTES[fmt])
    n = blocks.shape[0]
    px = np.zeros((n, 16, 4), np.int64)
    if fmt == BC7:
        px = np.array([decode_bc7_block(b) for b in blocks], np.int64).reshape(n, 16, 4)
    elif fmt in (BC1_RGB, BC1_RGBA):
        px = _colour(blocks, 0, False, fmt == BC1_RGBA)
    elif fmt == BC2:
        px = _colour(blocks, 8, True, False)
        a = _le(blocks, 0, 8).astype(np.uint64)
        px[:, :, 3] = ((a[:, None] >> (4 * np.arange(16, dtype=np.uint64))) & np.uint64(15)).astype(np.int64) * 17
    elif fmt == BC3:
        px = _colour(blocks, 8, True, False)
        px[:, :, 3] = _channel(blocks, 0)
    elif fmt == BC4:
        px[:, :, 0] = _channel(blocks, 0)
        px[:, :, 3] = 255
    else:
        px[:, :, 0] = _channel(blocks, 0)
        px[:, :, 1] = _channel(blocks, 8)
        px[:, :, 3] = 255
    img = px.reshape(bh, bw, 4, 4, 4).transpose(0, 2, 1, 3, 4).reshape(bh * 4, bw * 4, 4)
    return img[:height, :width].astype(np.uint8)
