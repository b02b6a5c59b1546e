"""GPU tests of the precision form: 16-bit ray/hit payloads (directions as two
snorm16 octahedral coordinates, FP16 barycentrics; FP32 traversal), Kahan
accumulation, and the terrain scene (spheres + fBm heightfield) through the
same parity checks as the other scenes."""
import numpy as np
import pytest

import helios_gb300 as hx
from oracle import binding as ob
from tests.helpers import integrator_desc, rel_rmse, small_icosphere_scene

pytestmark = pytest.mark.gpu


def _policy(base, fp16=True, kahan=False):
    p = hx.policy_spec() if base == "spec" else hx.policy_reference()
    if base != "spec":
        p.env_sampling = hx.ENV_SAMPLE_IMPORTANCE
    p.payload = hx.PAYLOAD_FP16 if fp16 else hx.PAYLOAD_FP32
    p.accumulation = hx.ACCUM_KAHAN if kahan else hx.ACCUM_RUNNING_MEAN
    return p


@pytest.fixture(scope="module")
def terrain(gpu_ctx):
    hs = hx.HostScene(hx.SCENE_TERRAIN, terrain_size=512, num_spheres=40, env_width=256, env_height=128)
    sc = hx.Scene(gpu_ctx, hs)
    yield hs, sc, ob.OracleScene(hs)
    sc.close()


@pytest.mark.parametrize("which", ["box", "ico", "terrain"])
def test_fp16_payload_samples_match_oracle(which, gpu_ctx, terrain):
    """FP16-payload per-sample radiance, device vs the oracle's emulation of
    the same payload rounding: all but rare samples agree to float rounding."""
    if which == "box":
        hs = hx.HostScene(hx.SCENE_BOX)
        sc, osc, pol, W, H, b = hx.Scene(gpu_ctx, hs), None, _policy("spec"), 64, 64, 5
    elif which == "ico":
        hs = small_icosphere_scene(level=3, quads=2000, pool=4, mask=64, env=(256, 128))
        sc, osc, pol, W, H, b = hx.Scene(gpu_ctx, hs), None, _policy("reference"), 96, 54, 8
    else:
        hs, sc, osc = terrain
        pol, W, H, b = _policy("reference"), 96, 54, 8
    osc = osc or ob.OracleScene(hs)
    d = integrator_desc(W, H, bounces=b)
    d.policy = pol
    f = hx.frame_desc(hs.camera(), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=b, policy=pol)
    for frame in (0, 5):
        g = it.sample_radiance(f, frame)
        o, _ = osc.sample_radiance(d, f, frame, precision=32)
        close = np.all(np.abs(g - o) <= 1e-4 * (1 + np.abs(o)), axis=1)
        info = (frame, rel_rmse(g, o), int((~close).sum()))
        assert close.mean() > 0.995, info
        assert rel_rmse(g, o) < 1e-2, info
    it.close()


@pytest.mark.parametrize("which,fp16", [("box", False), ("terrain", False), ("terrain", True)])
def test_scaled_ray_offset_samples_match_oracle(which, fp16, gpu_ctx, terrain):
    """HX_RAY_OFFSET_SCALED origins (geometric normal, position-relative
    offset; shadow rays shortened by the offset): per-sample radiance, device
    vs the oracle's FP32 evaluation of the same policy.  The box has an area
    light (shadow rays end 1e-4 before it, so the shortening matters); the
    terrain's coordinates reach 2048."""
    if which == "box":
        hs = hx.HostScene(hx.SCENE_BOX)
        sc, osc, pol, W, H, b = hx.Scene(gpu_ctx, hs), None, _policy("spec", fp16=fp16), 64, 64, 5
    else:
        hs, sc, osc = terrain
        pol, W, H, b = _policy("reference", fp16=fp16), 96, 54, 8
    pol.ray_offset = hx.RAY_OFFSET_SCALED
    osc = osc or ob.OracleScene(hs)
    d = integrator_desc(W, H, bounces=b)
    d.policy = pol
    f = hx.frame_desc(hs.camera(), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=b, policy=pol)
    for frame in (0, 5):
        g = it.sample_radiance(f, frame)
        o, _ = osc.sample_radiance(d, f, frame, precision=32)
        close = np.all(np.abs(g - o) <= 1e-4 * (1 + np.abs(o)), axis=1)
        info = (frame, rel_rmse(g, o), int((~close).sum()))
        assert close.mean() > 0.995, info
        assert rel_rmse(g, o) < 1e-2, info
    it.close()


def test_scaled_ray_offset_converges_to_fp64(gpu_ctx, terrain):
    """Terrain at world scale (coordinates to 2048), 1024 spp: the device's
    FP32 image against the FP64 oracle's image of the same samples, with the
    reference's ray origins and with HX_RAY_OFFSET_SCALED.  The reference's
    fixed tmin of 1e-4 is below the FP32 rounding of hit positions there, so
    FP32 re-hits surfaces that FP64 leaves (a bias); scaled origins remove it
    and leave the noise of paths that diverge by rounding."""
    hs, sc, osc = terrain
    W, H, spp = 1920, 1080, 1024
    f = hx.frame_desc(hs.camera(), W, H)
    pix = np.random.default_rng(12).choice(W * H, size=1024, replace=False).astype(np.uint32)
    err = {}
    for off in (hx.RAY_OFFSET_REFERENCE, hx.RAY_OFFSET_SCALED):
        pol = _policy("reference", fp16=False)
        pol.ray_offset = off
        d = integrator_desc(W, H, bounces=8, max_samples=1 << 30)
        d.policy = pol
        ref, _ = osc.render(d, f, spp, precision=64, pixels=pix)
        it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=8, max_samples=spp, policy=pol)
        it.render(f, spp)
        img = it.read_accumulation()[:, :, :3].reshape(-1, 3)
        it.close()
        err[off] = rel_rmse(img[pix], ref)
    print("device FP32 vs FP64 oracle (reference origins, scaled origins):", err)
    assert err[hx.RAY_OFFSET_SCALED] < 0.5 * err[hx.RAY_OFFSET_REFERENCE], err
    assert err[hx.RAY_OFFSET_SCALED] < 2e-3, err


def test_fp16_counting_mode_renders_the_same_image(gpu_ctx, terrain):
    """16-bit payloads through the batched traversal in its counting
    instantiation (node visits, triangle tests, SIMD counters) accumulate the
    same image as without counting."""
    hs, sc, _ = terrain
    W, H = 320, 180
    pol = _policy("reference", fp16=True, kahan=True)
    f = hx.frame_desc(hs.camera(), W, H)
    imgs, stats = [], None
    for counting in (False, True):
        it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=8, policy=pol)
        it.set_counting(counting)
        it.render(f, 2)
        if counting:
            stats = it.stats()
        imgs.append(it.read_accumulation())
        it.close()
    assert imgs[0].tobytes() == imgs[1].tobytes()
    assert stats.node_visits > 0 and stats.tri_tests > 0 and stats.warp_node_steps > 0


def test_fp16_primary_hit_agreement(gpu_ctx, terrain):
    """Hit-ID agreement of primary rays whose directions went through the
    16-bit octahedral payload with FP32 rays.  The quantised BVH itself never
    changes a hit (bit-exact tests); what moves a hit here is the direction
    rounding (spacing 2/65534 of the octahedral square) at triangle edges, so
    the agreement falls with the triangles' screen size: 98.5% on this
    512^2 heightfield at 320x180."""
    hs, sc, osc = terrain
    W, H = 320, 180
    d32 = integrator_desc(W, H)
    d32.policy = _policy("reference", fp16=False)
    d16 = integrator_desc(W, H)
    d16.policy = _policy("reference", fp16=True)
    f = hx.frame_desc(hs.camera(), W, H)
    r32 = ob.primary_rays(d32, f, 0)
    h32 = sc.trace(r32, any_hit=True)
    # the same rays with directions through the 16-bit octahedral payload: the
    # oracle's primary hits under that codec, checked against the device
    o16, prim16 = osc.sample_radiance(d16, f, 0, precision=32)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, policy=d16.policy)
    g16 = it.sample_radiance(f, 0)
    it.close()
    assert rel_rmse(g16, o16) < 1e-2
    agree = (prim16["prim"] == h32["prim"]).mean()
    print("16-bit vs FP32 payload primary hit-ID agreement:", agree)
    assert agree > 0.98, agree


def test_fp16_kahan_converged_vs_fp64(gpu_ctx):
    """Box scene, spec policy, 16384 spp: the FP16-payload + Kahan image and
    the FP32 image against the FP64 oracle (FP32 payloads) at the same seeds;
    both are held to the 1e-3 relative-RMSE bar (16-bit payloads measured
    4.4e-4, FP32 payloads 2e-5)."""
    hs = hx.HostScene(hx.SCENE_BOX)
    sc = hx.Scene(gpu_ctx, hs)
    osc = ob.OracleScene(hs)
    W = H = 128
    spp = 16384
    f = hx.frame_desc(hs.camera(), W, H)
    pix = np.random.default_rng(4).choice(W * H, size=128, replace=False).astype(np.uint32)
    d = integrator_desc(W, H, policy="spec", max_samples=spp)
    ref, _ = osc.render(d, f, spp, precision=64, pixels=pix)
    errs = {}
    for name, pol in (("fp32", _policy("spec", fp16=False)), ("fp16+kahan", _policy("spec", fp16=True, kahan=True))):
        it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=5, max_samples=spp, policy=pol)
        it.render(f, spp)
        img = it.read_accumulation()[:, :, :3].reshape(-1, 3)
        errs[name] = rel_rmse(img[pix], ref)
        it.close()
    print("relative RMSE vs FP64 oracle:", errs)
    assert errs["fp32"] <= 1e-3, errs
    assert errs["fp16+kahan"] <= 1e-3, errs
    sc.close()


def test_terrain_bvh_and_primary_hits_bit_exact(gpu_ctx, terrain):
    hs, sc, osc = terrain
    g, o = sc.export_bvh(), osc.export_bvh()
    for k in ("morton", "sorted", "children", "leaf_prims"):
        assert np.array_equal(g[k], o[k]), k
    assert g["nodes"].tobytes() == o["nodes"].tobytes()
    W, H = 320, 180
    d = integrator_desc(W, H, policy="reference")
    f = hx.frame_desc(hs.camera(), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, policy=d.policy)
    gh = it.primary_hits(f, 0)
    oh = osc.trace(ob.primary_rays(d, f, 0), any_hit=True)
    assert np.array_equal(gh["prim"], oh["prim"]) and np.array_equal(gh["t"], oh["t"])
    it.close()
