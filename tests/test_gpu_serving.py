"""GPU tests of the serving loop (hx_server_*): continuous batching of
requests of different scenes, resolutions and sample counts; each result is
the same alone and in the mix (bit-exact RGBA8, the same as the progressive
integrator's image); admission by the HBM arena budget."""
import numpy as np
import pytest

import helios_gb300 as hx
from tests.helpers import small_icosphere_scene

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scenes(gpu_ctx):
    box = hx.HostScene(hx.SCENE_BOX)
    ico = small_icosphere_scene(level=3, quads=3000, pool=4, mask=64, env=(256, 128))
    s_box, s_ico = hx.Scene(gpu_ctx, box), hx.Scene(gpu_ctx, ico)
    yield (box, s_box), (ico, s_ico)
    s_box.close()
    s_ico.close()


def _wait_all(srv, ids, timeout=120.0, images=None):
    """Waits for the requests; with images (a dict) fetches each result as
    it arrives (finished images hold the pinned result arena until fetched,
    so a client that never fetches stalls admission)."""
    import time
    done = {}
    t0 = time.time()
    while len(done) < len(ids):
        for r in srv.poll(wait_seconds=0.5):
            # every tick's device status word was clean
            assert r.status == hx.HX_OK, (r.request_id, r.status)
            done[r.request_id] = r
            if images is not None:
                images[r.request_id] = srv.fetch(r.request_id)
        assert time.time() - t0 < timeout, "requests did not finish"
    return done


def _reference_image(ctx, scene, hs, w, h, spp, pol, bounces):
    it = hx.PathIntegrator(ctx, scene, w, h, max_ray_bounces=bounces, max_samples=spp, policy=pol)
    it.render(hx.frame_desc(hs.camera(), w, h), spp)
    img = it.tonemap(hx.TONEMAP_ACES, 1.0)
    it.close()
    return img


@pytest.mark.parametrize("ray_offset", [hx.RAY_OFFSET_REFERENCE, hx.RAY_OFFSET_SCALED])
def test_results_identical_alone_and_in_the_mix(gpu_ctx, scenes, ray_offset):
    (box, s_box), (ico, s_ico) = scenes
    pol = hx.policy_reference()
    pol.env_sampling = hx.ENV_SAMPLE_IMPORTANCE
    pol.ray_offset = ray_offset
    srv = hx.Server(gpu_ctx, arena_bytes=1 << 30, max_paths_per_tick=1 << 20, max_ray_bounces=6, policy=pol)
    ib, ii = srv.add_scene(s_box), srv.add_scene(s_ico)
    srv.start()
    reqs = [  # (scene id, host scene, device scene, w, h, spp)
        (ib, box, s_box, 256, 256, 16),
        (ii, ico, s_ico, 320, 180, 4),
        (ib, box, s_box, 640, 360, 2),
        (ii, ico, s_ico, 1280, 720, 2),   # one sample per tick (921,600 px)
        (ib, box, s_box, 1920, 1080, 1),  # larger than a tick: split into pixel chunks
        (ii, ico, s_ico, 96, 54, 64),
    ]
    # alone: one request in the server at a time
    alone = []
    for sid, hs, sc, w, h, spp in reqs:
        rid = srv.submit(sid, hx.frame_desc(hs.camera(), w, h), w, h, spp)
        _wait_all(srv, [rid])
        alone.append(srv.fetch(rid))
    # the mix: all at once
    ids = [srv.submit(sid, hx.frame_desc(hs.camera(), w, h), w, h, spp) for sid, hs, sc, w, h, spp in reqs]
    res = _wait_all(srv, ids)
    mixed = [srv.fetch(i) for i in ids]
    for k, (a, m) in enumerate(zip(alone, mixed)):
        assert np.array_equal(a, m), k
        assert res[ids[k]].paths == reqs[k][3] * reqs[k][4] * reqs[k][5]
    st = srv.stats()
    srv.close()
    assert st.requests_done == 2 * len(reqs)
    # and identical to the progressive integrator's image for the same view
    for k in (0, 1, 4):
        sid, hs, sc, w, h, spp = reqs[k]
        ref = _reference_image(gpu_ctx, sc, hs, w, h, spp, pol, 6)
        assert np.array_equal(ref, alone[k]), k


def test_admission_by_hbm_budget(gpu_ctx, scenes):
    (box, s_box), _ = scenes
    # arena for two 512x512 requests (20 B per pixel each); each request fits
    # one tick, so memory alone bounds how many are admitted at once
    srv = hx.Server(gpu_ctx, arena_bytes=11 << 20, max_paths_per_tick=1 << 21, max_ray_bounces=4)
    sid = srv.add_scene(s_box)
    srv.start()
    with pytest.raises(hx.HxError) as e:
        srv.submit(sid, hx.frame_desc(box.camera(), 1024, 1024), 1024, 1024, 1)
    assert e.value.status == hx.HX_ERR_OOM_BUDGET
    ids = [srv.submit(sid, hx.frame_desc(box.camera(), 512, 512), 512, 512, 8) for _ in range(6)]
    got = {}
    res = _wait_all(srv, ids, images=got)
    # at most two fit at a time: the server never held more than two of them,
    # nor more arena bytes than two need
    st = srv.stats()
    assert st.requests_active_peak == 2, st.requests_active_peak
    per_request = 16 * 512 * 512 + 4 * 512 * 512
    assert 2 * per_request <= st.arena_used_peak <= 11 << 20
    imgs = [got[i] for i in ids]
    for im in imgs[1:]:
        assert np.array_equal(im, imgs[0])
    assert st.arena_used == 0
    srv.close()


def test_cancel_pending_and_admitted_requests(gpu_ctx, scenes):
    """hx_server_cancel: a pending request ends at once, an admitted one as
    soon as none of its samples is on the GPU; both report HX_ERR_CANCELLED,
    release their slot and arena space, and the requests around them finish
    with the same images as alone."""
    import time
    (box, s_box), _ = scenes
    srv = hx.Server(gpu_ctx, arena_bytes=256 << 20, max_paths_per_tick=1 << 16, max_ray_bounces=4)
    sid = srv.add_scene(s_box)
    srv.start()
    f = hx.frame_desc(box.camera(), 256, 256)
    rid = srv.submit(sid, f, 256, 256, 4)
    _wait_all(srv, [rid])
    alone = srv.fetch(rid)
    # long requests (4,096 ticks each): one is admitted, the others wait behind
    # the admitted-work cap, and so do the short ones
    W = 2048
    long_ids = [srv.submit(sid, hx.frame_desc(box.camera(), W, W), W, W, 64) for _ in range(4)]
    short_ids = [srv.submit(sid, f, 256, 256, 4) for _ in range(3)]
    time.sleep(0.05)
    st = srv.stats()
    assert st.requests_active >= 1
    for i in long_ids:
        srv.cancel(i)
    with pytest.raises(hx.HxError) as e:
        srv.cancel(987654321)
    assert e.value.status == hx.HX_ERR_INVALID_ARG
    results, imgs = {}, {}
    t0 = time.time()
    while len(results) < len(long_ids) + len(short_ids):
        for r in srv.poll(wait_seconds=0.5):
            results[r.request_id] = r
            if r.request_id in short_ids:
                assert r.status == hx.HX_OK
                imgs[r.request_id] = srv.fetch(r.request_id)
        assert time.time() - t0 < 120, "requests did not finish"
    for i in long_ids:
        assert results[i].status == hx.HX_ERR_CANCELLED
        assert results[i].paths < W * W * 64
        with pytest.raises(hx.HxError) as e:
            srv.fetch(i)
        assert e.value.status == hx.HX_ERR_CANCELLED
    for i in short_ids:
        assert np.array_equal(imgs[i], alone)
    st = srv.stats()
    assert st.arena_used == 0 and st.requests_active == 0 and st.requests_pending == 0
    srv.close()


def test_denoised_requests_identical_alone_in_the_mix_and_to_the_integrator(gpu_ctx, scenes):
    """Requests with denoise set: the served RGBA8 equals the integrator's
    denoise (with AOV accumulation) of the same view and sample count, alone
    and in a mix with plain requests (the denoiser's kernels are
    deterministic)."""
    from oracle import denoiser_ref as dr
    (box, s_box), (ico, s_ico) = scenes
    pol = hx.policy_reference()
    dn = hx.Denoiser(gpu_ctx)
    dn.set_params(dr.init_params(5))
    srv = hx.Server(gpu_ctx, arena_bytes=1 << 30, max_paths_per_tick=1 << 18, max_ray_bounces=6, policy=pol)
    ii = srv.add_scene(s_ico)
    srv.set_denoiser(dn)
    srv.start()
    w, h, spp = 640, 360, 2  # 230,400 px: one sample per 2^18-path tick
    f = hx.frame_desc(ico.camera(), w, h)
    rid = srv.submit(ii, f, w, h, spp, denoise=True)
    _wait_all(srv, [rid])
    alone = srv.fetch(rid)
    ids = [srv.submit(ii, f, 256, 256, 8), srv.submit(ii, f, w, h, spp, denoise=True), srv.submit(ii, f, 96, 54, 4)]
    imgs = {}
    _wait_all(srv, ids, images=imgs)
    st = srv.stats()
    srv.close()
    assert np.array_equal(alone, imgs[ids[1]])
    assert st.requests_denoised == 2
    it = hx.PathIntegrator(gpu_ctx, s_ico, w, h, max_ray_bounces=6, max_samples=spp, policy=pol)
    it.set_aov_accumulation(True)
    it.render(f, spp)
    ldr, _ = it.denoise(dn, f, op=hx.TONEMAP_ACES, exposure=1.0, hdr=False, ldr=True)
    it.close()
    dn.close()
    assert np.array_equal(ldr, alone)
