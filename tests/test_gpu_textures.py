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
