"""CPU tests of the product library's host side: the C-ABI loads and exports
every declared symbol; host-only entry points (policies, camera, procedural
scenes, Hosek-Wilkie coefficients) behave; no device call is made."""
import ctypes as C
import json
import os
import re

import numpy as np
import pytest

import helios_gb300 as hx
from tests.helpers import decode_png

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    src = open(os.path.join(ROOT, "include", "hx.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"HX_API\s+[^;(]*?\b(hx_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    names = _declared_symbols()
    assert len(names) > 30
    lib = hx.lib()
    for n in names:
        assert hasattr(lib, n), n
    # the binding covers every declared entry point
    assert set(names) <= set(hx.exported_symbols()) | {"hx_scene_export_env"}


def test_policies():
    r, s = hx.policy_reference(), hx.policy_spec()
    assert (r.rng, r.rr_start_depth, r.rr_clamp, r.area_count_from_x, r.area_w_one) == (0, 0, 0, 0, 0)
    assert r.radiance_clamp == 1.0 and r.accumulation == hx.ACCUM_RUNNING_MEAN
    assert (s.rng, s.rr_start_depth, s.rr_clamp, s.area_count_from_x, s.area_w_one) == (1, 3, 1, 1, 1)
    assert s.env_sampling == hx.ENV_SAMPLE_IMPORTANCE


def test_camera_frame_desc():
    cam = hx.Camera((0.5, 0.5, 2.5), (0.5, 0.5, 0.0), (0, 1, 0), 40.0, 1.0, 1000.0, 8.0, 0.0)
    f = hx.frame_desc(cam, 256, 256)
    assert list(f.camera_pos)[:3] == [0.5, 0.5, 2.5]
    # focal plane: normal = -forward = +z, through z = 2.5 - 8
    assert np.allclose(list(f.focal_plane), [0, 0, 1, 5.5], atol=1e-5)
    # unproject the image centre: lies on the view axis
    M = np.array(f.view_proj_inverse[:], np.float64).reshape(4, 4).T
    p = M @ np.array([0, 0, 0, 1.0])
    p = p[:3] / p[3]
    d = p - np.array([0.5, 0.5, 2.5])
    assert np.allclose(d / np.linalg.norm(d), [0, 0, -1], atol=1e-5)


def test_procedural_scene_sizes():
    hs = hx.HostScene(hx.SCENE_BOX)
    d = hs.desc.contents
    tris = sum(d.meshes[d.instances[i].mesh_index].num_indices // 3 for i in range(d.num_instances))
    assert tris == 36
    ico = hx.HostScene(hx.SCENE_ICOSPHERES, icosphere_level=6, num_alpha_quads=100000, mask_pool=2, mask_size=32,
                       env_width=64, env_height=32)
    d = ico.desc.contents
    tris = sum(d.meshes[d.instances[i].mesh_index].num_indices // 3 for i in range(d.num_instances))
    assert tris == 12 * 81920 + 2 + 200000
    assert d.num_punctual_lights == 4 and d.environment.kind == hx.ENV_HOSEK_WILKIE


def test_alpha_masks_are_half_cut_out():
    ico = hx.HostScene(hx.SCENE_ICOSPHERES, icosphere_level=1, num_alpha_quads=10, mask_pool=3, mask_size=128,
                       env_width=16, env_height=8)
    d = ico.desc.contents
    for t in range(d.num_textures):
        tx = d.textures[t]
        a = np.ctypeslib.as_array(tx.rgba8, shape=(tx.width * tx.height * 4,))[3::4]
        assert abs((a >= 26).mean() - 0.5) < 0.01


def test_hosek_coefficients_match_reference_golden():
    """The reference's own evaluate + normalisation (compiled from its source
    by oracle/hosek/build_ref.sh) at on- and off-grid sun elevations,
    fractional turbidities and ground albedos 0..1.  The library builds each
    quintic from six samples (Lagrange, in double) where the reference sums
    Bernstein terms, so the FP32 results differ by rounding: within 2e-6 of
    each coefficient's range over the cases (a few ulps of it; a value that
    cancels toward zero can differ by more ulps of itself)."""
    g = json.load(open(os.path.join(ROOT, "tests", "golden", "hosek_coeffs.json")))
    assert len(g["cases"]) > 150
    assert {round(c["turbidity"], 3) for c in g["cases"]} >= {1.0, 2.5, 4.7, 7.25, 10.0}
    assert {round(c["albedo"], 3) for c in g["cases"]} >= {0.0, 0.35, 1.0}
    got = np.array([hx.hosek_wilkie_coefficients(c["sun_direction"], c["turbidity"], 1.15, albedo=c["albedo"])
                    for c in g["cases"]])
    ref = np.array([c["coeffs"] for c in g["cases"]], np.float32).reshape(-1, 10, 3)
    scale = np.abs(ref).max(axis=0)
    assert (np.abs(got - ref) <= 2e-6 * scale).all(), np.abs((got - ref) / scale).max()
    assert np.median(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-30)) < 1e-6


def test_cpp_driver_builds_and_links():
    """The C++ engine surface (include/helios_gb300.hpp) compiles and links
    against the C-ABI; without arguments the driver prints its usage."""
    import subprocess
    from helios_gb300 import build as b
    exe = b.build_driver()
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


def test_png_export_round_trip(tmp_path):
    """hx_save_png / hx_encode_png (the stb_image_write PNG behind
    Renderer::save_image_to_disk): a valid PNG whose pixels are the input's,
    for a 1x1 image, odd sizes and one spanning several 64 KiB deflate blocks."""
    rng = np.random.default_rng(4)
    for h, w in ((1, 1), (3, 7), (181, 97)):
        img = rng.integers(0, 256, size=(h, w, 4), dtype=np.uint8)
        data = hx.encode_png(img)
        assert np.array_equal(decode_png(data), img)
        p = tmp_path / ("img_%d_%d.png" % (h, w))
        hx.save_png(str(p), img)
        assert p.read_bytes() == data
    try:
        hx.save_png(str(tmp_path / "no_such_dir" / "x.png"), np.zeros((2, 2, 4), np.uint8))
        assert False, "writing into a missing directory must fail"
    except hx.HxError as e:
        assert "cannot open" in str(e)


def test_block_compressed_texture_decode_matches_restatement():
    """hx_texture_decode (BC1-BC5, the reference's compressed asset formats)
    equals the numpy restatement of the published block formats on random
    blocks (both BC1 modes, all index values, sizes not multiples of 4), and
    a hand-computed block: red/blue endpoints, every texel on entry 2."""
    from oracle import texture_ref as tr
    rng = np.random.default_rng(11)
    for fmt in (hx.TEXTURE_BC1_RGB, hx.TEXTURE_BC1_RGBA, hx.TEXTURE_BC2, hx.TEXTURE_BC3, hx.TEXTURE_BC4,
                hx.TEXTURE_BC5):
        for w, h in ((4, 4), (13, 7), (64, 36)):
            nb = ((w + 3) // 4) * ((h + 3) // 4)
            data = rng.integers(0, 256, size=nb * tr.BLOCK_BYTES[fmt], dtype=np.uint8)
            assert np.array_equal(hx.texture_decode(data, w, h, fmt), tr.decode(data, w, h, fmt)), (fmt, w, h)
    # c0 = 0xF800 (red), c1 = 0x001F (blue), all indices 2: (2 * 255 + 0 + 1) // 3 = 170, (0 + 255 + 1) // 3 = 85
    blk = np.array([0x00, 0xF8, 0x1F, 0x00, 0xAA, 0xAA, 0xAA, 0xAA], np.uint8)
    out = hx.texture_decode(blk, 4, 4, hx.TEXTURE_BC1_RGB)
    assert (out.reshape(-1, 4) == np.array([170, 0, 85, 255], np.uint8)).all()
    # the same endpoints swapped select the 3-colour mode: entry 2 is the mean, entry 3 transparent black
    blk2 = np.array([0x1F, 0x00, 0x00, 0xF8, 0xAA, 0xAA, 0xFF, 0xFF], np.uint8)
    out2 = hx.texture_decode(blk2, 4, 4, hx.TEXTURE_BC1_RGBA).reshape(-1, 4)
    assert (out2[:8] == np.array([128, 0, 128, 255], np.uint8)).all()
    assert (out2[8:] == 0).all()


def test_bc7_decode_matches_restatement():
    """BC7 (BPTC): hx_texture_decode equals the restatement of the published
    format on random blocks of all eight modes (and the reserved all-zero
    mode byte), and a hand-computed mode-6 block.  The GPU's own texture
    unit checks the same decoder in tests/test_gpu_textures.py."""
    from oracle import texture_ref as tr
    from tests.helpers import random_bc7_blocks
    blocks = random_bc7_blocks(4096, seed=7)
    blocks[5, 0] = 0  # reserved: decodes to zero
    data = blocks.reshape(-1)
    w, h = 4 * 64, 4 * 64
    got = hx.texture_decode(data, w, h, hx.TEXTURE_BC7)
    ref = tr.decode(data, w, h, tr.BC7)
    assert np.array_equal(got, ref)
    assert (got[0:4, 20:24] == 0).all()
    assert np.array_equal(hx.texture_decode(data[:16 * 12], 13, 7, hx.TEXTURE_BC7), tr.decode(data[:16 * 12], 13, 7, tr.BC7))
    # mode 6 (bit 6 of byte 0), RGBA 7+7 bits with per-endpoint p-bits, 4-bit
    # indices: e0 = (0, 127, 254, 1) p 0 -> (0, 254, 252, 2), e1 = (127, 0, 0, 127)
    # p 1 -> (255, 1, 1, 255) after 8-bit widening; every index 15 except the
    # anchor (3 bits, value 7); weights 64 -> e1, 30 (index 7) ->
    # ((64 - 30) e0 + 30 e1 + 32) >> 6
    bits = 1 << 6
    pos = 7
    fields = [(0, 7), (127, 7), (127, 7), (0, 7), (254 >> 1, 7), (0, 7), (1, 7), (127, 7), (0, 1), (1, 1), (7, 3)]
    fields += [(15, 4)] * 15
    for v, nb in fields:
        bits |= v << pos
        pos += nb
    blk = np.frombuffer(bits.to_bytes(16, "little"), np.uint8)
    px = hx.texture_decode(blk, 4, 4, hx.TEXTURE_BC7).reshape(16, 4)
    e0 = np.array([0, 254, 254, 2])
    e1 = np.array([255, 1, 1, 255])
    assert (px[1:] == e1).all(), px[1]
    assert (px[0] == ((64 - 30) * e0 + 30 * e1 + 32) >> 6).all(), px[0]


def _bc6h_block(code, fields, indices):
    """A BC6H block from its mode code, (value, bits) endpoint fields in stored
    order and the per-texel index values (texel 0 one bit shorter)."""
    bits, pos = code, (2 if code < 2 else 5)
    for v, nb in fields:
        bits |= (v & ((1 << nb) - 1)) << pos
        pos += nb
    for t, v in enumerate(indices):
        nb = 3 if t == 0 else 4
        bits |= v << pos
        pos += nb
    assert pos == 128
    return np.frombuffer(bits.to_bytes(16, "little"), np.uint8)


def test_bc6h_decode_matches_restatement():
    """BC6H (BPTC half float, the reference's VK_FORMAT_BC6H_SFLOAT_BLOCK, and
    the unsigned variant): hx_texture_decode_hdr equals the restatement of the
    published format on random blocks of all fourteen modes and the four
    reserved codes (half bit patterns, bit-exact), also for sizes that are
    not multiples of 4.  The GPU's texture unit checks the same decoder in
    tests/test_gpu_textures.py."""
    from oracle import texture_ref as tr
    from tests.helpers import random_bc6h_blocks
    for fmt in (hx.TEXTURE_BC6H_SF16, hx.TEXTURE_BC6H_UF16):
        blocks = random_bc6h_blocks(48 * 48, seed=fmt)
        data = blocks.reshape(-1)
        got = hx.texture_decode_hdr(data, 192, 192, fmt).view(np.uint16)
        ref = tr.decode_hdr(data, 192, 192, fmt)
        assert np.array_equal(got, ref), fmt
        assert (got[..., 3] == 0x3C00).all()
        small = hx.texture_decode_hdr(data[:16 * 8], 13, 6, fmt).view(np.uint16)
        assert np.array_equal(small, tr.decode_hdr(data[:16 * 8], 13, 6, fmt))
        # reserved code 10011 (block 14 of the cycle): zero colour
        assert (got[0:4, 56:60, :3] == 0).all()


def test_bc6h_hand_computed_blocks():
    """Mode 11 (code 00011: one region, 10-bit endpoints, no transform, 4-bit
    indices) worked by hand from the format's arithmetic."""
    # unsigned: e0 = (1023, 512, 0), e1 = (0, 1023, 1023); unquantised
    # 1023 -> 0xFFFF, 512 -> ((512 << 16) + 0x8000) >> 10 = 32800, 0 -> 0;
    # texel 0 index 0 (e0), texel 1 index 15 (e1), texel 2 index 8 (weight 34):
    #   R: (65535 * 30 + 0 * 34 + 32) >> 6 = 30720 -> 30720 * 31 >> 6 = 14880
    #   G: (32800 * 30 + 65535 * 34 + 32) >> 6 = 50190 -> 24310
    #   B: (0 * 30 + 65535 * 34 + 32) >> 6 = 34815 -> 16863
    # and e0 -> (65535 * 31 >> 6, 32800 * 31 >> 6, 0) = (31743, 15887, 0)
    blk = _bc6h_block(0b00011, [(1023, 10), (512, 10), (0, 10), (0, 10), (1023, 10), (1023, 10)],
                      [0, 15, 8] + [0] * 13)
    px = hx.texture_decode_hdr(blk, 4, 4, hx.TEXTURE_BC6H_UF16).view(np.uint16).reshape(16, 4)
    assert px[0].tolist() == [31743, 15887, 0, 0x3C00]
    assert px[1].tolist() == [0, 31743, 31743, 0x3C00]
    assert px[2].tolist() == [14880, 24310, 16863, 0x3C00]
    assert (px[3:] == px[0]).all()
    # signed: e0 = (0x3FF, 0x1FF, 0x200) sign-extends to (-1, 511, -512);
    # unquantised: -1 -> -(((1 << 15) + 0x4000) >> 9) = -96, 511 and -512 clamp
    # to +-0x7FFF; index 0 everywhere: floor((64 e0 + 32) / 64) = e0, then the
    # magnitude * 31 >> 5 with the sign bit: 96 -> 93 (0x805D), 32767 -> 31743
    blk = _bc6h_block(0b00011, [(0x3FF, 10), (0x1FF, 10), (0x200, 10), (0, 10), (0, 10), (0, 10)], [0] * 16)
    px = hx.texture_decode_hdr(blk, 4, 4, hx.TEXTURE_BC6H_SF16).view(np.uint16).reshape(16, 4)
    assert (px == np.array([0x805D, 31743, 0x8000 | 31743, 0x3C00])).all(), px[0]
    assert float(px[0].view(np.float16)[0]) == -93 * 2.0 ** -24  # a subnormal half


def test_half_float_formats_host_checks():
    """RGBA16F passes through hx_texture_decode_hdr unchanged; each decoder
    refuses the other family's formats."""
    rng = np.random.default_rng(3)
    tex = rng.normal(0, 4, (5, 7, 4)).astype(np.float16)
    assert np.array_equal(hx.texture_decode_hdr(tex.view(np.uint8), 7, 5, hx.TEXTURE_RGBA16F).view(np.uint16),
                          tex.view(np.uint16))
    with pytest.raises(hx.HxError) as e:
        hx.texture_decode(np.zeros(16, np.uint8), 4, 4, hx.TEXTURE_BC6H_SF16)
    assert e.value.status == hx.HX_ERR_INVALID_ARG and "hdr" in str(e.value)
    with pytest.raises(hx.HxError) as e:
        hx.texture_decode_hdr(np.zeros(16, np.uint8), 4, 4, hx.TEXTURE_BC7)
    assert e.value.status == hx.HX_ERR_INVALID_ARG
