"""GPU error paths: device-side faults reach the caller as status codes, the
GPU context stays usable, and nothing traps or hangs.

* A traversal stack of one entry (hx_scene_set_traversal_stack_limit) makes
  rays drop stack entries: the production render path sets the overflow bit
  of the device status word, and the next synchronising call
  (hx_integrator_tonemap to host memory, hx_integrator_read_accumulation)
  returns HX_ERR_DEVICE.  With the limit restored the next frame is clean.
* A tensor-core pipeline-wait budget of a few cycles
  (hx_denoiser_set_wait_budget) makes the denoiser's mbarrier waits run out:
  every CTA records the error, drains its own TMA copies and MMAs, frees its
  TMEM and exits; hx_denoiser_check returns HX_ERR_TIMEOUT, and with the
  budget restored the same inference is bit-identical to one run before.
"""
import numpy as np
import pytest

import helios_gb300 as hx
from tests.helpers import small_icosphere_scene

pytestmark = pytest.mark.gpu


def test_traversal_stack_overflow_reaches_the_caller(gpu_ctx):
    hs = small_icosphere_scene(level=4, quads=5000, pool=8, mask=128, env=(256, 128))
    sc = hx.Scene(gpu_ctx, hs)
    W, H = 160, 90
    f = hx.frame_desc(hs.camera(), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=8)
    it.render(f, 2)
    it.tonemap()  # clean
    with pytest.raises(hx.HxError):
        sc.set_traversal_stack_limit(0)
    sc.set_traversal_stack_limit(1)
    it.render(f, 1)  # render does not wait; the fault is reported by the next synchronising call
    with pytest.raises(hx.HxError) as e:
        it.tonemap()
    assert e.value.status == hx.HX_ERR_DEVICE and "stack overflow" in str(e.value)
    it.render(f, 1)
    with pytest.raises(hx.HxError) as e:
        it.read_accumulation()
    assert e.value.status == hx.HX_ERR_DEVICE
    # restored: the word was cleared when reported, the next frames are clean
    sc.set_traversal_stack_limit(32)
    it.restart_bake()
    it.render(f, 2)
    it.tonemap()
    clean = it.read_accumulation()
    assert np.isfinite(clean).all()
    it.close()
    sc.close()


def _features(n, h, w, seed=5):
    rng = np.random.default_rng(seed)
    feats = np.zeros((n, h, w, 12), np.float32)
    feats[..., 0:3] = rng.exponential(0.5, (n, h, w, 3))
    feats[..., 4:7] = rng.uniform(0, 1, (n, h, w, 3))
    feats[..., 7] = rng.uniform(0, 1, (n, h, w))
    nrm = rng.normal(size=(n, h, w, 3))
    feats[..., 8:11] = nrm / np.linalg.norm(nrm, axis=-1, keepdims=True)
    return feats


def test_tensor_core_wait_timeout_is_reported_and_recovers(gpu_ctx):
    dn = hx.Denoiser(gpu_ctx)
    dn.init_params(7)
    n, h, w = 1, 64, 96
    feats = _features(n, h, w)
    tg = np.ones((n, h, w, 4), np.float32)
    fb = hx.DeviceBuffer(gpu_ctx, feats.nbytes)
    tb = hx.DeviceBuffer(gpu_ctx, tg.nbytes)
    ob = hx.DeviceBuffer(gpu_ctx, n * h * w * 16)
    fb.upload(feats)
    tb.upload(tg)
    dn.infer(fb, n, h, w, ob)
    dn.check()
    before = ob.download((n, h, w, 4))
    with pytest.raises(hx.HxError):
        dn.set_wait_budget(1 << 40)  # above the default: rejected
    dn.set_wait_budget(8)
    dn.infer(fb, n, h, w, ob)  # forward / backward-data kernels give up their waits
    with pytest.raises(hx.HxError) as e:
        dn.check()
    assert e.value.status == hx.HX_ERR_TIMEOUT
    with pytest.raises(hx.HxError) as e:  # a training pass (backward-weights kernel too) checks by itself
        dn.forward_backward(fb, tb, n, h, w)
    assert e.value.status == hx.HX_ERR_TIMEOUT
    dn.check()  # reported once, then cleared
    dn.set_wait_budget(0)
    dn.infer(fb, n, h, w, ob)
    dn.check()
    assert np.array_equal(ob.download((n, h, w, 4)), before)
    for b in (fb, tb, ob):
        b.close()
    dn.close()


def test_read_bandwidth_probe(gpu_ctx):
    """hx_measure_read_bandwidth: positive GB/s for an L2-sized and an
    HBM-sized working set; malformed sizes are rejected before any launch."""
    l2 = gpu_ctx.read_bandwidth(32 << 20, 50)
    hbm = gpu_ctx.read_bandwidth(1 << 30, 2)
    print("read bandwidth GB/s: 32 MiB", l2, "1 GiB", hbm)
    assert l2 > 0 and hbm > 0
    for nbytes, passes in (((32 << 20) + 8, 1), (1 << 10, 1), (32 << 20, 0)):
        with pytest.raises(hx.HxError) as e:
            gpu_ctx.read_bandwidth(nbytes, passes)
        assert e.value.status == hx.HX_ERR_INVALID_ARG

