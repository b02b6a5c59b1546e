"""GPU tests of the texture pipeline beyond alpha masks: sRGB-encoded albedo
textures (decoded before filtering, resource_manager.cpp:48-67) and
tangent-space normal maps (path_trace_rchit.glsl:190-219), against the
oracle's restatement."""
import numpy as np
import pytest

import helios_gb300 as hx
from oracle import binding as ob
from tests.helpers import TexturedQuadScene, bump_normal_map, checker_texture, integrator_desc, rel_rmse

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def quad(gpu_ctx):
    qs = TexturedQuadScene(checker_texture(), albedo_srgb=True, normal_map=bump_normal_map())
    sc = hx.Scene(gpu_ctx, qs)
    yield qs, sc, ob.OracleScene(qs)
    sc.close()


@pytest.mark.parametrize("policy", ["reference", "spec"])
def test_normal_mapped_srgb_samples_match_oracle(gpu_ctx, quad, policy):
    """Per-sample radiance on the normal-mapped, sRGB-textured quad equals the
    oracle's FP32 restatement to float rounding."""
    qs, sc, osc = quad
    W, H = 96, 64
    d = integrator_desc(W, H, bounces=4, policy=policy)
    f = hx.frame_desc(qs.camera(), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=4, policy=d.policy)
    for frame in (0, 3):
        g = it.sample_radiance(f, frame)
        o, _ = osc.sample_radiance(d, f, frame, precision=32)
        close = np.all(np.abs(g - o) <= 1e-4 * (1 + np.abs(o)), axis=1)
        info = (frame, rel_rmse(g, o), int((~close).sum()))
        assert close.mean() > 0.995, info
        assert rel_rmse(g, o) < 1e-3, info
        assert np.abs(g).max() > 0.0
    it.close()


def test_normal_map_and_srgb_views_match_oracle(gpu_ctx, quad):
    qs, sc, osc = quad
    W, H = 96, 64
    f = hx.frame_desc(qs.camera(), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H)
    for which in (hx.OUTPUT_ALBEDO, hx.OUTPUT_NORMALS):
        g = it.render_output(f, which)
        o = osc.output_view(f, W, H, which)
        assert np.max(np.abs(g - o)) <= 2e-6, which
    it.close()


def test_normal_map_and_srgb_change_the_result(gpu_ctx):
    """The normal map moves the shading normals (and the converged image);
    the sRGB flag darkens mid-tone albedo (decode below q / 255)."""
    tex = checker_texture()
    W, H = 64, 48
    out = {}
    for key, kw in (("plain", dict(albedo_srgb=False)), ("srgb", dict(albedo_srgb=True)),
                    ("nmap", dict(albedo_srgb=False, normal_map=bump_normal_map()))):
        qs = TexturedQuadScene(tex, **kw)
        sc = hx.Scene(gpu_ctx, qs)
        f = hx.frame_desc(qs.camera(), W, H)
        it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=3)
        it.render(f, 32)
        out[key] = (it.read_accumulation()[..., :3], it.render_output(f, hx.OUTPUT_ALBEDO)[..., :3],
                    it.render_output(f, hx.OUTPUT_NORMALS)[..., :3])
        it.close()
        sc.close()
    hit = np.any(out["plain"][1] != 0, axis=-1)
    assert np.all(out["srgb"][1][hit] < out["plain"][1][hit])
    assert np.array_equal(out["nmap"][1], out["plain"][1])
    dn = np.abs(out["nmap"][2] - out["plain"][2])[hit].max()
    assert dn > 0.05
    assert rel_rmse(out["nmap"][0], out["plain"][0]) > 0.01


@pytest.mark.parametrize("fmt", [hx.TEXTURE_BC1_RGB, hx.TEXTURE_BC3, hx.TEXTURE_BC5, hx.TEXTURE_BC7])
def test_block_compressed_albedo_renders_like_its_decoded_texels(gpu_ctx, fmt):
    """A BCn albedo texture (decoded at upload) gives the same accumulated
    image and albedo view, bit for bit, as uploading its RGBA8 decode."""
    from oracle import texture_ref as tr
    rng = np.random.default_rng(fmt)
    w, h = 30, 22
    nb = ((w + 3) // 4) * ((h + 3) // 4)
    data = rng.integers(0, 256, size=nb * tr.BLOCK_BYTES[fmt], dtype=np.uint8)
    texels = tr.decode(data, w, h, fmt)
    W, H = 64, 48
    out = []
    for kw in (dict(albedo=data, albedo_format=fmt, albedo_wh=(w, h)), dict(albedo=texels)):
        qs = TexturedQuadScene(albedo_srgb=True, normal_map=bump_normal_map(), **kw)
        sc = hx.Scene(gpu_ctx, qs)
        f = hx.frame_desc(qs.camera(), W, H)
        it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=3)
        it.render(f, 4)
        out.append((it.read_accumulation(), it.render_output(f, hx.OUTPUT_ALBEDO)))
        it.close()
        sc.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert np.any(out[0][1][..., :3] != 0)


def _texture_unit_bc7():
    """tests/hw/bc7_texture_unit.cu built for sm_103a into a temporary library:
    BC7 blocks decoded by the GPU's own texture unit."""
    import ctypes
    import os
    import shutil
    import subprocess
    import tempfile
    src = os.path.join(os.path.dirname(os.path.abspath(__file__)), "hw", "bc7_texture_unit.cu")
    out = os.path.join(tempfile.mkdtemp(), "libbc7tu.so")
    nvcc = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-shared", "-Xcompiler", "-fPIC",
                    "-o", out, src], check=True, capture_output=True)
    lib = ctypes.CDLL(out)
    lib.bc7_texture_unit_decode.restype = ctypes.c_int
    lib.bc7_texture_unit_decode.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    return lib


def test_bc7_decode_matches_the_texture_unit(gpu_ctx):
    """The library's BC7 decoder (hx_texture_decode) against the GPU's
    texture unit on 4,096 random blocks of all eight modes (every partition,
    rotation and index-selection value occurs): identical RGBA8 texels.  The
    format's interpolation is exact integer arithmetic, so any mismatch is a
    decoding error (a table entry, a bit field)."""
    from tests.helpers import random_bc7_blocks
    lib = _texture_unit_bc7()
    blocks = np.ascontiguousarray(random_bc7_blocks(64 * 64, seed=3))
    got = hx.texture_decode(blocks.reshape(-1), 256, 256, hx.TEXTURE_BC7)
    hw = np.zeros((256, 256, 4), np.uint8)
    rc = lib.bc7_texture_unit_decode(blocks.ctypes.data, 64, 64, hw.ctypes.data)
    assert rc == 0, "CUDA error %d" % rc
    bad = np.nonzero((got != hw).any(-1).reshape(64, 4, 64, 4).any(axis=(1, 3)).reshape(-1))[0]
    info = [(int(b), int(b % 8), blocks[b].tobytes().hex()) for b in bad[:8]]
    assert bad.size == 0, (bad.size, info)


def _texture_unit_bc6h():
    """tests/hw/bc6h_texture_unit.cu built for sm_103a into a temporary
    library: BC6H blocks decoded by the GPU's own texture unit."""
    import ctypes
    import os
    import shutil
    import subprocess
    import tempfile
    src = os.path.join(os.path.dirname(os.path.abspath(__file__)), "hw", "bc6h_texture_unit.cu")
    out = os.path.join(tempfile.mkdtemp(), "libbc6tu.so")
    nvcc = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-shared", "-Xcompiler", "-fPIC",
                    "-o", out, src], check=True, capture_output=True)
    lib = ctypes.CDLL(out)
    lib.bc6h_texture_unit_decode.restype = ctypes.c_int
    lib.bc6h_texture_unit_decode.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_void_p]
    return lib


@pytest.mark.parametrize("fmt", [hx.TEXTURE_BC6H_SF16, hx.TEXTURE_BC6H_UF16])
def test_bc6h_decode_matches_the_texture_unit(gpu_ctx, fmt):
    """The library's BC6H decoder (hx_texture_decode_hdr) against the GPU's
    texture unit on 4,096 random blocks cycling through the fourteen modes
    (every partition and index value occurs): identical half-float bit
    patterns, signed and unsigned.  The format's arithmetic is exact
    integers, so any mismatch is a decoding error (a bit field of a mode's
    header, a table entry, a rounding step)."""
    from tests.helpers import random_bc6h_blocks
    lib = _texture_unit_bc6h()
    blocks = np.ascontiguousarray(random_bc6h_blocks(64 * 64, seed=11 + fmt, reserved=False))
    got = hx.texture_decode_hdr(blocks.reshape(-1), 256, 256, fmt).view(np.uint16)
    hw = np.zeros((256, 256, 4), np.uint16)
    rc = lib.bc6h_texture_unit_decode(blocks.ctypes.data, 64, 64, 1 if fmt == hx.TEXTURE_BC6H_SF16 else 0,
                                      hw.ctypes.data)
    assert rc == 0, "CUDA error %d" % rc
    bad = np.nonzero((got[..., :3] != hw[..., :3]).any(-1).reshape(64, 4, 64, 4).any(axis=(1, 3)).reshape(-1))[0]
    info = [(int(b), int(b % 14), blocks[b].tobytes().hex()) for b in bad[:8]]
    assert bad.size == 0, (bad.size, info)


def _hdr_quad(gpu_ctx, **kw):
    qs = TexturedQuadScene(albedo_srgb=False, normal_map=bump_normal_map(), **kw)
    return qs, hx.Scene(gpu_ctx, qs)


@pytest.mark.parametrize("case", ["bc6h_sf16", "rgba16f_alpha_roughness", "rgba8_snorm_alpha_roughness"])
def test_half_float_and_snorm_textures_match_oracle(gpu_ctx, case):
    """Per-sample radiance with a half-float or SNORM albedo texture against
    the oracle's FP32 restatement, which samples the same texel values: a
    BC6H (signed, the reference's format) texture given to the device as
    blocks and to the oracle as the restatement's decode
    (oracle/texture_ref.py); an uncompressed RGBA16F texture; and an RGBA8
    SNORM texture (the reference's format for uncompressed 8-bit images that
    are not sRGB: bytes 128-255 read negative).  In the last two the alpha
    (cut out below 0.1 on an alpha-tested quad) and the green channel (the
    roughness channel) vary."""
    from oracle import texture_ref as tr
    from tests.helpers import bc6h_mode11_blocks
    w, h = 24, 20
    if case == "bc6h_sf16":
        blocks = bc6h_mode11_blocks(((w + 3) // 4) * ((h + 3) // 4), seed=5)
        texels = tr.decode_hdr(blocks.reshape(-1).tobytes(), w, h, tr.BC6H_SF16).view(np.float16)
        dev = dict(albedo=blocks.reshape(-1), albedo_format=hx.TEXTURE_BC6H_SF16, albedo_wh=(w, h))
        extra = {}
    else:
        rng = np.random.default_rng(8)
        texels = rng.uniform(0.0, 1.6, (h, w, 4)).astype(np.float16)
        texels[..., 1] = rng.uniform(0.05, 0.95, (h, w)).astype(np.float16)
        texels[..., 3] = np.where(rng.uniform(0, 1, (h, w)) < 0.3, 0.02, 1.0).astype(np.float16)
        dev = dict(albedo=texels, albedo_format=hx.TEXTURE_RGBA16F, albedo_wh=(w, h))
        extra = dict(non_opaque=True, roughness_channel=1)
    if case == "rgba8_snorm_alpha_roughness":
        rng = np.random.default_rng(12)
        texels = rng.integers(0, 256, (h, w, 4)).astype(np.uint8)
        texels[..., 1] = rng.integers(6, 127, (h, w))
        texels[..., 3] = rng.choice(np.array([127, 200, 5], np.uint8), (h, w), p=[0.7, 0.15, 0.15])
        dev = dict(albedo=texels, albedo_format=hx.TEXTURE_RGBA8_SNORM, albedo_wh=(w, h))
    qs, sc = _hdr_quad(gpu_ctx, **dev, **extra)
    ofmt = hx.TEXTURE_RGBA8_SNORM if case == "rgba8_snorm_alpha_roughness" else hx.TEXTURE_RGBA16F
    oq = TexturedQuadScene(texels, albedo_srgb=False, normal_map=bump_normal_map(), albedo_format=ofmt,
                           albedo_wh=(w, h), **extra)
    osc = ob.OracleScene(oq)
    W, H = 96, 64
    d = integrator_desc(W, H, bounces=4, policy="reference")
    f = hx.frame_desc(qs.camera(), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=4, policy=d.policy)
    for frame in (0, 5):
        g = it.sample_radiance(f, frame)
        o, _ = osc.sample_radiance(d, f, frame, precision=32)
        close = np.all(np.abs(g - o) <= 1e-4 * (1 + np.abs(o)), axis=1)
        info = (frame, rel_rmse(g, o), int((~close).sum()))
        assert close.mean() > 0.995, info
        assert rel_rmse(g, o) < 1e-3, info
        assert np.abs(g).max() > 0.0
    a = it.render_output(f, hx.OUTPUT_ALBEDO)
    assert np.max(np.abs(a - osc.output_view(f, W, H, hx.OUTPUT_ALBEDO))) <= 2e-6
    if case == "rgba8_snorm_alpha_roughness":
        assert a[..., :3].min() < 0.0  # negative SNORM texels reach the albedo view
    if case != "bc6h_sf16":
        r = it.render_output(f, hx.OUTPUT_ROUGHNESS)
        assert np.max(np.abs(r - osc.output_view(f, W, H, hx.OUTPUT_ROUGHNESS))) <= 2e-6
    it.close()
    sc.close()


def test_wide_alpha_with_16bit_payloads_matches_oracle(gpu_ctx):
    """The any-hit alpha test on an RGBA16F texture (the traversal's wide-alpha
    instantiation) under 16-bit ray / hit payloads, against the oracle's
    emulation of the same payload rounding."""
    w, h = 24, 20
    rng = np.random.default_rng(8)
    texels = rng.uniform(0.0, 1.6, (h, w, 4)).astype(np.float16)
    texels[..., 1] = rng.uniform(0.05, 0.95, (h, w)).astype(np.float16)
    texels[..., 3] = np.where(rng.uniform(0, 1, (h, w)) < 0.3, 0.02, 1.0).astype(np.float16)
    extra = dict(non_opaque=True, roughness_channel=1)
    qs, sc = _hdr_quad(gpu_ctx, albedo=texels, albedo_format=hx.TEXTURE_RGBA16F, albedo_wh=(w, h), **extra)
    oq = TexturedQuadScene(texels, albedo_srgb=False, normal_map=bump_normal_map(), albedo_format=hx.TEXTURE_RGBA16F,
                           albedo_wh=(w, h), **extra)
    osc = ob.OracleScene(oq)
    W, H = 96, 64
    d = integrator_desc(W, H, bounces=4, policy="reference")
    d.policy.payload = hx.PAYLOAD_FP16
    f = hx.frame_desc(qs.camera(), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=4, policy=d.policy)
    for frame in (0, 5):
        g = it.sample_radiance(f, frame)
        o, _ = osc.sample_radiance(d, f, frame, precision=32)
        close = np.all(np.abs(g - o) <= 1e-4 * (1 + np.abs(o)), axis=1)
        info = (frame, rel_rmse(g, o), int((~close).sum()))
        assert close.mean() > 0.995, info
        assert rel_rmse(g, o) < 1e-2, info
    it.close()
    sc.close()


def test_bc6h_renders_like_its_rgba16f_texels(gpu_ctx):
    """A BC6H albedo texture (decoded at upload) gives the same accumulated
    image and albedo view, bit for bit, as uploading its RGBA16F decode; a
    half-float texture flagged sRGB is refused (the reference has no sRGB
    BC6H format)."""
    from tests.helpers import bc6h_mode11_blocks
    w, h = 30, 22
    blocks = bc6h_mode11_blocks(((w + 3) // 4) * ((h + 3) // 4), seed=9).reshape(-1)
    texels = hx.texture_decode_hdr(blocks, w, h, hx.TEXTURE_BC6H_SF16)
    W, H = 64, 48
    out = []
    for kw in (dict(albedo=blocks, albedo_format=hx.TEXTURE_BC6H_SF16, albedo_wh=(w, h)),
               dict(albedo=texels, albedo_format=hx.TEXTURE_RGBA16F, albedo_wh=(w, h))):
        qs, sc = _hdr_quad(gpu_ctx, **kw)
        f = hx.frame_desc(qs.camera(), W, H)
        it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=3)
        it.render(f, 4)
        out.append((it.read_accumulation(), it.render_output(f, hx.OUTPUT_ALBEDO)))
        it.close()
        sc.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert np.any(out[0][1][..., :3] > 0)
    qs = TexturedQuadScene(blocks, albedo_srgb=True, albedo_format=hx.TEXTURE_BC6H_SF16, albedo_wh=(w, h))
    with pytest.raises(hx.HxError) as e:
        hx.Scene(gpu_ctx, qs)
    assert e.value.status == hx.HX_ERR_INVALID_ARG and "sRGB" in str(e.value)
