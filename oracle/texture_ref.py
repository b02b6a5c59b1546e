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

The specification leaves the rounding of interpolated entries to the
implementation; this library rounds to nearest in integers and so does
this restatement.
"""
import numpy as np

BC1_RGB, BC1_RGBA, BC2, BC3, BC4, BC5 = 1, 2, 3, 4, 5, 6
BLOCK_BYTES = {BC1_RGB: 8, BC1_RGBA: 8, BC2: 16, BC3: 16, BC4: 8, BC5: 16}


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
    if fmt in (BC1_RGB, BC1_RGBA):
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
