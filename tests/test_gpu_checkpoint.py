"""GPU tests of bake checkpoint / resume (hx_integrator_save_checkpoint,
hx_integrator_load_checkpoint).

The reference keeps its progressive state (accumulation image,
num_accumulated_samples, tile_idx; include/gfx/path_integrator.h:46-53) for
the life of the process.  A bake that is checkpointed after k frames, restored
into a fresh integrator and continued must equal the uninterrupted bake bit
for bit: the accumulation image, the Kahan compensation, the per-pixel counts,
the AOV images and the progress counters (integer and bit-exact float
comparison: the same samples are added in the same order).  Damaged or
mismatched checkpoints are rejected with HX_ERR_INVALID_ARG and leave the
integrator's state unchanged.
"""
import numpy as np
import pytest

import helios_gb300 as hx
from tests.helpers import small_icosphere_scene

pytestmark = pytest.mark.gpu

HEADER = 64


@pytest.fixture(scope="module")
def ico(gpu_ctx):
    hs = small_icosphere_scene(level=3, quads=800, pool=4, mask=32, env=(128, 64))
    sc = hx.Scene(gpu_ctx, hs)
    yield hs, sc
    sc.close()


def _integrator(ctx, sc, W, H, kahan, tiled, max_samples):
    pol = hx.policy_spec()
    if kahan:
        pol.accumulation = hx.ACCUM_KAHAN
    return hx.PathIntegrator(ctx, sc, W, H, max_ray_bounces=4, max_samples=max_samples, tiled=tiled, policy=pol)


@pytest.mark.parametrize("kahan,tiled,aov,split", [
    (False, False, False, 5),
    (True, False, True, 3),
    (True, True, False, 6),    # 2 x 1 tiles of 4 samples: the checkpoint falls inside the second tile
    (False, True, True, 4),    # exactly at a tile boundary
])
def test_resume_equals_uninterrupted_bake(gpu_ctx, ico, kahan, tiled, aov, split):
    hs, sc = ico
    W, H = (200, 96) if tiled else (96, 64)
    max_samples = 4 if tiled else 5000
    total = 8 if tiled else 9
    f = hx.frame_desc(hs.camera(), W, H)
    whole = _integrator(gpu_ctx, sc, W, H, kahan, tiled, max_samples)
    first = _integrator(gpu_ctx, sc, W, H, kahan, tiled, max_samples)
    resumed = _integrator(gpu_ctx, sc, W, H, kahan, tiled, max_samples)
    for it in (whole, first, resumed):
        it.set_aov_accumulation(aov)
    resumed.set_aov_accumulation(False)  # the checkpoint switches it to its own setting
    whole.render(f, total)
    for _ in range(split):
        first.render(f, 1)
    ckpt = first.save_checkpoint()
    hdr = np.frombuffer(ckpt[:HEADER], np.uint32)
    assert hdr[0] == 0x4B425848  # "HXBK"
    assert (hdr[2], hdr[3], hdr[9]) == (W, H, int(aov))
    assert len(ckpt) == HEADER + W * H * (36 + (32 if aov else 0))
    resumed.load_checkpoint(ckpt)
    assert resumed.progress() == first.progress()
    resumed.render(f, total - split)
    assert resumed.progress() == whole.progress()
    a, b = whole.read_accumulation(), resumed.read_accumulation()
    assert a.tobytes() == b.tobytes()
    # every byte of the state (comp, counts, AOVs, progress) matches too
    assert whole.save_checkpoint() == resumed.save_checkpoint()
    for it in (whole, first, resumed):
        it.close()


def test_damaged_or_mismatched_checkpoints_are_rejected(gpu_ctx, ico):
    hs, sc = ico
    W, H = 64, 48
    f = hx.frame_desc(hs.camera(), W, H)
    src = _integrator(gpu_ctx, sc, W, H, True, False, 5000)
    src.render(f, 3)
    ckpt = bytearray(src.save_checkpoint())
    dst = _integrator(gpu_ctx, sc, W, H, True, False, 5000)
    dst.render(f, 2)
    before = (dst.progress(), dst.read_accumulation().tobytes())

    def rejected(data, words):
        with pytest.raises(hx.HxError) as e:
            dst.load_checkpoint(bytes(data))
        assert e.value.status == hx.HX_ERR_INVALID_ARG
        msg = str(e.value)
        assert any(w in msg for w in words), msg
        assert (dst.progress(), dst.read_accumulation().tobytes()) == before

    bad = bytearray(ckpt)
    bad[HEADER + 1000] ^= 0x40  # one flipped bit in the accumulation image
    rejected(bad, ["checksum"])
    rejected(ckpt[:-1], ["payload"])
    rejected(ckpt[:10], ["header"])
    bad = bytearray(ckpt)
    bad[0] ^= 1
    rejected(bad, ["magic"])
    other = _integrator(gpu_ctx, sc, W + 8, H, True, False, 5000)
    with pytest.raises(hx.HxError) as e:
        other.load_checkpoint(bytes(ckpt))
    assert e.value.status == hx.HX_ERR_INVALID_ARG and "64x48" in str(e.value)
    mean = _integrator(gpu_ctx, sc, W, H, False, False, 5000)
    with pytest.raises(hx.HxError) as e:
        mean.load_checkpoint(bytes(ckpt))
    assert e.value.status == hx.HX_ERR_INVALID_ARG and "accumulation" in str(e.value)
    # the intact checkpoint still loads, and the small buffer case of save is refused
    dst.load_checkpoint(bytes(ckpt))
    assert dst.progress() == src.progress()
    buf = np.zeros(100, np.uint8)
    assert hx.lib().hx_integrator_save_checkpoint(dst.handle, buf.ctypes.data_as(hx.C.c_void_p), buf.size) == \
        hx.HX_ERR_INVALID_ARG
    for it in (src, dst, other, mean):
        it.close()
