"""GPU tests of the renderer's debug outputs: the output-buffer views of
Renderer::render_debug_visualization (renderer.cpp:491-545,
debug_visualization.frag) against the oracle, and HX_OUTPUT_FINAL against
the accumulation image."""
import numpy as np
import pytest

import helios_gb300 as hx
from oracle import binding as ob
from tests.helpers import small_icosphere_scene

pytestmark = pytest.mark.gpu

VIEWS = [("albedo", hx.OUTPUT_ALBEDO), ("normals", hx.OUTPUT_NORMALS), ("roughness", hx.OUTPUT_ROUGHNESS),
         ("metallic", hx.OUTPUT_METALLIC), ("emissive", hx.OUTPUT_EMISSIVE)]


@pytest.fixture(scope="module", params=["box", "ico"])
def scene(request, gpu_ctx):
    if request.param == "box":
        hs = hx.HostScene(hx.SCENE_BOX)
    else:
        hs = small_icosphere_scene(level=4, quads=5000, pool=8, mask=128, env=(256, 128))
    sc = hx.Scene(gpu_ctx, hs)
    yield request.param, hs, sc, ob.OracleScene(hs)
    sc.close()


@pytest.mark.parametrize("name,which", VIEWS)
def test_output_view_matches_oracle(gpu_ctx, scene, name, which):
    """Every output buffer equals the oracle's restatement of the debug pass:
    the same pixels hit (the rest keep the clear colour) and the same
    fragment values (FP32, same operation order)."""
    kind, hs, sc, osc = scene
    W, H = 160, 96
    f = hx.frame_desc(hs.camera(), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H)
    g = it.render_output(f, which)
    o = osc.output_view(f, W, H, which)
    it.close()
    assert g.shape == (H, W, 4) and np.all(g[..., 3] == 1.0)
    miss_g = np.all(g[..., :3] == 0.0, axis=-1)
    miss_o = np.all(o[..., :3] == 0.0, axis=-1)
    assert np.array_equal(miss_g, miss_o)
    assert np.max(np.abs(g - o)) <= 2e-6, (kind, name)
    if which == hx.OUTPUT_NORMALS:
        hit = ~miss_g
        assert hit.mean() > 0.5
        assert np.all((g[hit, :3] >= -1e-6) & (g[hit, :3] <= 1.0 + 1e-6))


def test_output_final_is_accumulation_in_display_order(gpu_ctx, scene):
    kind, hs, sc, _ = scene
    W, H = 64, 48
    f = hx.frame_desc(hs.camera(), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=4)
    it.render(f, 3)
    final = it.render_output(f, hx.OUTPUT_FINAL)
    acc = it.read_accumulation()
    assert np.array_equal(final, acc[::-1])
    with pytest.raises(hx.HxError) as e:
        it.render_output(f, 6)
    assert e.value.status == hx.HX_ERR_INVALID_ARG
    it.close()


def test_output_albedo_is_unlit_and_orientation_matches_tonemap(gpu_ctx):
    """The box's albedo view shows the red wall on the left of the displayed
    frame, the same side the tone-mapped path-traced frame shows it on."""
    hs = hx.HostScene(hx.SCENE_BOX)
    sc = hx.Scene(gpu_ctx, hs)
    W, H = 96, 96
    f = hx.frame_desc(hs.camera(), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=3)
    alb = it.render_output(f, hx.OUTPUT_ALBEDO)
    it.render(f, 16)
    ldr = it.tonemap().astype(np.float32)
    it.close()
    sc.close()
    red = alb[..., 0] - alb[..., 1]
    left, right = red[:, : W // 4].mean(), red[:, -W // 4:].mean()
    red_ldr = ldr[..., 0] - ldr[..., 1]
    assert (left > right) == (red_ldr[:, : W // 4].mean() > red_ldr[:, -W // 4:].mean())


def _nan_quad_scene():
    """A 2 x 2 quad at z = 0 whose material emits NaN: every camera ray that
    hits it carries a NaN radiance (emission is added at depth 0)."""
    from tests.helpers import TriangleSoupScene
    q = np.array([[[-1, -1, 0], [1, -1, 0], [1, 1, 0]], [[-1, -1, 0], [1, 1, 0], [-1, 1, 0]]], np.float32)
    soup = TriangleSoupScene(q)
    soup._mat[0].emissive[0] = float("nan")
    cam = hx.Camera()
    cam.position[:] = [0.0, 0.0, 4.0]
    cam.target[:] = [0.0, 0.0, 0.0]
    cam.up[:] = [0.0, 1.0, 0.0]
    cam.fov_y_degrees, cam.near_plane, cam.far_plane = 60.0, 1.0, 1000.0
    cam.focal_length, cam.aperture_radius = 8.0, 0.0
    return soup, cam


def test_visualize_nans_marks_nan_samples_red(gpu_ctx):
    """VISUALIZE_NANS (path_trace_rgen.glsl:225-244): a pixel whose sample is
    NaN stores exactly (1, 0, 0); without it the NaN stays in the image.  The
    same pixels as the oracle's restatement, on the first frame and after the
    running mean of later frames; rejected with Kahan accumulation."""
    from tests.helpers import integrator_desc
    soup, cam = _nan_quad_scene()
    sc = hx.Scene(gpu_ctx, soup)
    osc = ob.OracleScene(soup)
    W, H = 48, 40
    f = hx.frame_desc(cam, W, H)
    red_by_frames = {}
    for nframes in (1, 3):
        d = integrator_desc(W, H, bounces=3, policy="reference")
        d.policy.visualize_nans = 1
        it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=3, policy=d.policy)
        it.render(f, nframes)
        g = it.read_accumulation()[..., :3].reshape(-1, 3)
        it.close()
        o, _ = osc.render(d, f, nframes)
        red = np.all(g == np.array([1.0, 0.0, 0.0], np.float32), axis=1)
        assert 0.1 < red.mean() < 0.9
        assert np.array_equal(red, np.all(o == np.array([1.0, 0.0, 0.0]), axis=1))
        assert not np.isnan(g).any()
        # a red frame followed by clean ones is averaged like any other value
        assert np.max(np.abs(g - o)) <= 1e-6
        red_by_frames[nframes] = red
    plain = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=3, policy=hx.policy_reference())
    plain.render(f, 1)
    p = plain.read_accumulation()[..., :3].reshape(-1, 3)
    assert np.array_equal(np.isnan(p[:, 0]), red_by_frames[1])
    plain.close()
    d = integrator_desc(W, H, policy="reference")
    d.policy.visualize_nans, d.policy.accumulation = 1, hx.ACCUM_KAHAN
    with pytest.raises(hx.HxError) as e:
        hx.PathIntegrator(gpu_ctx, sc, W, H, policy=d.policy)
    assert e.value.status == hx.HX_ERR_INVALID_ARG
    sc.close()


def _paths(v):
    """(V, 8) vertices -> {path colour: (S, 16) segments in bounce order}."""
    seg = v.reshape(-1, 16)
    out = {}
    for row in seg:
        out.setdefault(tuple(row[4:7].tolist()), []).append(row)
    return {k: np.array(r) for k, r in out.items()}


@pytest.mark.parametrize("policy", ["reference", "spec"])
def test_gather_debug_rays_matches_oracle(gpu_ctx, scene, policy):
    """Ray-debug capture (gather_debug_rays / RAY_DEBUG_VIEW): the same
    segments as the oracle's paths through the same pixel — origins, hit
    points and per-path colours — after the camera ray."""
    from tests.helpers import integrator_desc
    kind, hs, sc, osc = scene
    W, H = 64, 48
    f = hx.frame_desc(hs.camera(), W, H)
    d = integrator_desc(W, H, bounces=5, policy=policy)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=5, policy=d.policy)
    # a display pixel whose camera rays hit geometry (display row r is launch
    # row H - 1 - r; the capture's pixel row py is launch row H - py)
    alb = it.render_output(f, hx.OUTPUT_ALBEDO)
    hit = np.argwhere(np.any(alb[:-1, :, :3] != 0.0, axis=-1))
    r, x = hit[len(hit) // 2]
    it.render(f, 2)  # the capture is seeded with the accumulated sample count
    total = 0
    for px, py in ((int(x), int(r) + 1), (W // 2, H // 2), (5, 40)):
        g = it.gather_debug_rays(f, px, py, 256)
        o = osc.debug_rays(d, f, px, py, 256, 2)
        assert g.shape == o.shape and g.shape[0] % 2 == 0
        total += g.shape[0]
        if g.shape[0] == 0:
            continue
        assert np.all(g[:, 3] == 1.0) and np.all(g[:, 7] == 1.0)
        assert np.all((g[:, 4:7] >= 0.5) & (g[:, 4:7] < 1.0))
        gp, op = _paths(g), _paths(o)
        assert gp.keys() == op.keys()
        bad = [(k, gp[k].shape[0], op[k].shape[0], float(np.max(np.abs(gp[k] - op[k]))) if gp[k].shape == op[k].shape else -1.0)
               for k in op if gp[k].shape != op[k].shape or np.max(np.abs(gp[k] - op[k])) > 1e-4]
        assert not bad, "%d of %d paths differ, e.g. %s; first device / oracle segments %s / %s" % (
            len(bad), len(op), bad[:4], gp[bad[0][0]][:2].tolist(), op[bad[0][0]][:2].tolist())
    assert total > 0
    # the accumulation is untouched
    before = it.read_accumulation()
    it.gather_debug_rays(f, 3, 3, 64)
    assert np.array_equal(before, it.read_accumulation())
    with pytest.raises(hx.HxError):
        it.gather_debug_rays(f, W, 0, 16)
    it.close()
