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

The specification leaves the rounding of interpolated entries to the
implementation; this library rounds to nearest in integers and so does
this restatement.
"""
import numpy as np

BC1_RGB, BC1_RGBA, BC2, BC3, BC4, BC5, BC7 = 1, 2, 3, 4, 5, 6, 7
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
