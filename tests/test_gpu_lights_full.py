"""GPU parity on the light types and camera the benchmark scenes leave out,
and on the benchmark scenes at full size.

* Spot lights (distinct cone edges, and equal edges: the step of Q15),
  directional lights, point and area lights, an equirect environment, an
  alpha-tested quad and a normal-mapped sRGB floor, with a pinhole camera and
  with the reference's default thin lens (aperture 0.1, scene.h:260):
  per-sample radiance against the oracle (path_trace_rchit.glsl:284-451,
  path_trace_rgen.glsl:156-171).
* Primary-ray hit triangle IDs bit-exact on every pixel of the full
  1.18 M-triangle benchmark scene at 1920x1080 (frames 0 and 7, any-hit on),
  and on 65,536 seeded pixels of the full 4096^2 terrain (34.5 M triangles),
  where the device walks the 8-bit quantised BVH8 and the oracle the
  unquantised binary tree.
"""
import numpy as np
import pytest

import helios_gb300 as hx
from oracle import binding as ob
from tests.helpers import LightsScene, integrator_desc, rel_rmse

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lights(gpu_ctx):
    hs = LightsScene()
    sc = hx.Scene(gpu_ctx, hs)
    yield hs, sc, ob.OracleScene(hs)
    sc.close()


@pytest.mark.parametrize("policy", ["reference", "spec"])
@pytest.mark.parametrize("aperture", [0.0, 0.1])
def test_light_types_and_thin_lens_match_oracle(policy, aperture, gpu_ctx, lights):
    hs, sc, osc = lights
    kinds = sorted(int(l.data0[0]) for l in sc.lights())
    assert kinds == [hx.LIGHT_DIRECTIONAL, hx.LIGHT_SPOT, hx.LIGHT_POINT, hx.LIGHT_ENVIRONMENT, hx.LIGHT_AREA]
    W, H = 128, 96
    d = integrator_desc(W, H, bounces=6, policy=policy, bias=0.0005)
    f = hx.frame_desc(hs.camera(aperture=aperture), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=6, shadow_ray_bias=0.0005, policy=d.policy)
    for frame in (0, 3):
        hits = it.primary_hits(f, frame)
        o_hits = osc.trace(ob.primary_rays(d, f, frame), any_hit=True)
        assert np.array_equal(hits["prim"], o_hits["prim"])
        g = it.sample_radiance(f, frame)
        o, _ = osc.sample_radiance(d, f, frame, precision=32)
        close = np.all(np.abs(g - o) <= 1e-4 * (1 + np.abs(o)), axis=1)
        assert close.mean() > 0.999, (frame, int((~close).sum()))
        assert rel_rmse(g, o) < 1e-3
    # the thin lens spreads the primary rays: a defocused image differs from the pinhole one
    if aperture > 0:
        f0 = hx.frame_desc(hs.camera(aperture=0.0), W, H)
        assert not np.array_equal(it.primary_hits(f0, 0)["prim"], it.primary_hits(f, 0)["prim"])
    it.close()


def test_spot_with_equal_cone_edges_is_a_step(gpu_ctx):
    """Spot lights loaded from a file get inner = outer cone
    (resource_manager.cpp:592), where GLSL's smoothstep is undefined; both
    sides define it as a step at the cone edge."""
    hs = LightsScene(spot_equal_edges=True)
    sc = hx.Scene(gpu_ctx, hs)
    osc = ob.OracleScene(hs)
    W, H = 96, 64
    d = integrator_desc(W, H, bounces=4, policy="reference")
    f = hx.frame_desc(hs.camera(), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=4, policy=d.policy)
    g = it.sample_radiance(f, 1)
    o, _ = osc.sample_radiance(d, f, 1, precision=32)
    close = np.all(np.abs(g - o) <= 1e-4 * (1 + np.abs(o)), axis=1)
    assert close.mean() > 0.999
    it.close()
    sc.close()


def test_primary_hit_ids_full_benchmark_scene(gpu_ctx):
    hs = hx.HostScene(hx.SCENE_ICOSPHERES)
    sc = hx.Scene(gpu_ctx, hs)
    assert sc.info().num_triangles == 1183042
    osc = ob.OracleScene(hs)
    W, H = 1920, 1080
    d = integrator_desc(W, H, bounces=8, policy="reference")
    f = hx.frame_desc(hs.camera(), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=8, policy=d.policy)
    for frame in (0, 7):
        g = it.primary_hits(f, frame)
        o = osc.trace(ob.primary_rays(d, f, frame), any_hit=True)
        assert np.array_equal(g["prim"], o["prim"])
        assert np.array_equal(g["t"], o["t"])
        assert 0.5 < (o["prim"] != hx.NO_HIT).mean() < 1.0
    it.close()
    sc.close()
    osc.close()


def test_primary_hit_ids_full_terrain(gpu_ctx):
    """34.5 M triangles: the conservatively quantised BVH8 loses no hit
    against the oracle's unquantised binary tree (65,536 seeded pixels)."""
    hs = hx.HostScene(hx.SCENE_TERRAIN)
    sc = hx.Scene(gpu_ctx, hs)
    n_tri = sc.info().num_triangles
    assert n_tri > 33_000_000
    osc = ob.OracleScene(hs)
    W, H = 1920, 1080
    d = integrator_desc(W, H, bounces=8, policy="reference")
    f = hx.frame_desc(hs.camera(), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=8, policy=d.policy)
    pix = np.sort(np.random.default_rng(17).choice(W * H, 65536, replace=False))
    for frame in (0, 7):
        g = it.primary_hits(f, frame)
        o = osc.trace(ob.primary_rays(d, f, frame)[pix], any_hit=True)
        assert np.array_equal(g["prim"][pix], o["prim"])
        assert np.array_equal(g["t"][pix], o["t"])
        assert (o["prim"] != hx.NO_HIT).mean() > 0.5
    it.close()
    sc.close()
    osc.close()


def _window_frame(frame, W, H, x0, y0, w, h):
    """Frame constants of the w x h window at (x0, y0) of a W x H image: the
    camera's inverse view-projection composed with the map from the window's
    normalised device coordinates to the full image's, so each window pixel
    has the full-resolution pixel footprint (rows counted as the camera's
    launch rows)."""
    import copy
    vpi = np.array(frame.view_proj_inverse[:], np.float64).reshape(4, 4).T  # column-major -> matrix
    m = np.eye(4)
    m[0, 0], m[0, 3] = w / W, (2.0 * x0 + w) / W - 1.0
    m[1, 1], m[1, 3] = h / H, (2.0 * y0 + h) / H - 1.0
    out = copy.copy(frame)
    out.view_proj_inverse[:] = (vpi @ m).T.reshape(-1).astype(np.float32).tolist()
    return out


def test_converged_radiance_full_resolution_window_vs_fp64_oracle(gpu_ctx):
    """The benchmark scene at 1920x1080 pixel footprints (a 128x128 window at
    the image centre), reference policy with the importance-sampled sky,
    16,384 samples per pixel: relative RMSE <= 1e-3 against the FP64 oracle
    at the same seeds on 128 seeded pixels of the window."""
    hs = hx.HostScene(hx.SCENE_ICOSPHERES)
    sc = hx.Scene(gpu_ctx, hs)
    osc = ob.OracleScene(hs)
    W, H, w, h, spp = 1920, 1080, 128, 128, 16384
    f = _window_frame(hx.frame_desc(hs.camera(), W, H), W, H, (W - w) // 2, (H - h) // 2, w, h)
    pol = hx.policy_reference()
    pol.env_sampling = hx.ENV_SAMPLE_IMPORTANCE
    d = integrator_desc(w, h, bounces=8, policy="reference", max_samples=spp)
    d.policy = pol
    it = hx.PathIntegrator(gpu_ctx, sc, w, h, max_ray_bounces=8, max_samples=spp, policy=pol)
    it.render(f, spp)
    img = it.read_accumulation()[:, :, :3].reshape(-1, 3)
    pix = np.random.default_rng(19).choice(w * h, size=128, replace=False).astype(np.uint32)
    o, _ = osc.render(d, f, spp, precision=64, pixels=pix)
    err = rel_rmse(img[pix], o)
    it.close()
    sc.close()
    osc.close()
    assert (np.abs(o).sum(1) > 0).mean() > 0.9
    assert err <= 1e-3, err
