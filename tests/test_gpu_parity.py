"""GPU parity tests: the CUDA path (through the C-ABI) against the oracle.

Integer outputs (RNG draws, Morton codes, BVH topology and node order,
hit triangle IDs) must be bit-exact; radiance is compared by relative RMSE
with the tolerance stated in each test.
"""
import json
import os

import numpy as np
import pytest

import helios_gb300 as hx
from oracle import binding as ob
from tests.helpers import TriangleSoupScene, decode_png, integrator_desc, random_rays, rel_rmse, small_icosphere_scene

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def box(gpu_ctx):
    hs = hx.HostScene(hx.SCENE_BOX)
    sc = hx.Scene(gpu_ctx, hs)
    yield hs, sc, ob.OracleScene(hs)
    sc.close()


@pytest.fixture(scope="module")
def ico(gpu_ctx):
    hs = small_icosphere_scene(level=4, quads=5000, pool=8, mask=128, env=(256, 128))
    sc = hx.Scene(gpu_ctx, hs)
    yield hs, sc, ob.OracleScene(hs)
    sc.close()


def test_rng_streams_bit_exact(gpu_ctx):
    kat = json.load(open(os.path.join(GOLDEN, "rng_kat.json")))
    rng = np.random.default_rng(5)
    seeds = np.concatenate([np.array([c["seed"] for c in kat["streams"]], np.uint32).ravel(),
                            rng.integers(0, 2**32, size=2 * 4096, dtype=np.uint64).astype(np.uint32)])
    for kind in (hx.RNG_XOROSHIRO64STAR, hx.RNG_PCG):
        g = gpu_ctx.rng_streams(kind, seeds, 64)
        o = ob.rng_streams(kind, seeds, 64)
        assert np.array_equal(g, o)
    g = gpu_ctx.rng_streams(0, seeds[:16], kat["draws"])
    for i, c in enumerate(kat["streams"]):
        assert g[i].tolist() == c["xoroshiro64star"]


@pytest.mark.parametrize("which", ["box", "ico"])
def test_bvh_bit_exact(which, box, ico):
    hs, sc, osc = box if which == "box" else ico
    g, o = sc.export_bvh(), osc.export_bvh()
    assert np.array_equal(g["morton"], o["morton"])
    assert np.array_equal(g["sorted"], o["sorted"])
    assert np.array_equal(g["children"], o["children"])
    assert g["nodes"].shape == o["nodes"].shape
    assert g["nodes"].tobytes() == o["nodes"].tobytes()
    assert np.array_equal(g["leaf_prims"], o["leaf_prims"])


@pytest.mark.parametrize("which", ["box", "ico"])
@pytest.mark.parametrize("any_hit", [False, True])
def test_trace_hits_bit_exact(which, any_hit, box, ico):
    # caller rays through the production traversal kernel (hx_scene_trace)
    hs, sc, osc = box if which == "box" else ico
    lo, hi = (0.05, 0.95) if which == "box" else (-25, 25)
    rays = random_rays(20000, lo, hi, seed=11)
    g = sc.trace(rays, any_hit=any_hit)
    o = osc.trace(rays, any_hit=any_hit)
    assert np.array_equal(g["prim"], o["prim"])
    hit = o["prim"] != hx.NO_HIT
    assert np.array_equal(g["t"][hit], o["t"][hit])
    assert np.array_equal(g["u"][hit], o["u"][hit]) and np.array_equal(g["v"][hit], o["v"][hit])


@pytest.mark.parametrize("origin", ["inside", "surface"])
def test_dense_cluster_hits_bit_exact(origin, gpu_ctx):
    # 30k small triangles in a unit cube: node visits expose many triangles at
    # once, so the warp's shared triangle queue fills, lanes carry triangles
    # across flushes, and rays starting on a triangle must skip it (tmin)
    rng = np.random.default_rng(21)
    centres = rng.uniform(0.0, 1.0, (30000, 1, 3))
    tris = (centres + rng.normal(0.0, 0.02, (30000, 3, 3))).astype(np.float32)
    soup = TriangleSoupScene(tris)
    sc = hx.Scene(gpu_ctx, soup)
    osc = ob.OracleScene(soup)
    n = 20000
    if origin == "inside":
        rays = random_rays(n, 0.1, 0.9, seed=22)
    else:
        k = rng.integers(0, len(tris), n)
        u, v = rng.random(n), rng.random(n)
        flip = u + v > 1.0
        u[flip], v[flip] = 1.0 - u[flip], 1.0 - v[flip]
        t = tris[k].astype(np.float64)
        o = t[:, 0] * (1 - u - v)[:, None] + t[:, 1] * u[:, None] + t[:, 2] * v[:, None]
        d = rng.normal(size=(n, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        rays = np.zeros((n, 8), np.float32)
        rays[:, 0:3], rays[:, 3], rays[:, 4:7], rays[:, 7] = o, 1e-4, d, 1e4
    g = sc.trace(rays)
    o = osc.trace(rays)
    assert np.array_equal(g["prim"], o["prim"])
    hit = o["prim"] != hx.NO_HIT
    assert hit.mean() > 0.3
    assert np.array_equal(g["t"][hit], o["t"][hit])
    assert np.array_equal(g["u"][hit], o["u"][hit]) and np.array_equal(g["v"][hit], o["v"][hit])
    sc.close()


@pytest.mark.parametrize("which,policy", [("box", "spec"), ("box", "reference"), ("ico", "reference")])
def test_primary_hit_ids_bit_exact(which, policy, gpu_ctx, box, ico):
    hs, sc, osc = box if which == "box" else ico
    W, H = (256, 256) if which == "box" else (320, 180)
    d = integrator_desc(W, H, policy=policy)
    f = hx.frame_desc(hs.camera(), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, policy=d.policy)
    for frame in (0, 7):
        g = it.primary_hits(f, frame)
        o = osc.trace(ob.primary_rays(d, f, frame), any_hit=True)
        assert np.array_equal(g["prim"], o["prim"])
        assert np.array_equal(g["t"], o["t"])
    it.close()


@pytest.mark.parametrize("W,H", [(97, 53), (7, 3), (1, 1)])
def test_primary_hit_ids_bit_exact_ragged_frames(W, H, gpu_ctx, ico):
    """Frames whose sides are not multiples of the 8 x 4-pixel tile the paths
    are traced in (the right and bottom remainders take the row-major part of
    the pixel order): hits still land on their own pixels, bit-exact, and the
    per-sample radiance of the remainders matches the oracle."""
    hs, sc, osc = ico
    d = integrator_desc(W, H, bounces=4, policy="reference")
    f = hx.frame_desc(hs.camera(), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=4, policy=d.policy)
    g = it.primary_hits(f, 2)
    o = osc.trace(ob.primary_rays(d, f, 2), any_hit=True)
    assert np.array_equal(g["prim"], o["prim"]) and np.array_equal(g["t"], o["t"])
    gr = it.sample_radiance(f, 1)
    orad, _ = osc.sample_radiance(d, f, 1, precision=32)
    close = np.all(np.abs(gr - orad) <= 1e-4 * (1 + np.abs(orad)), axis=1)
    assert close.mean() > 0.99 or close.sum() >= close.size - 1, (W, H, rel_rmse(gr, orad))
    it.close()


@pytest.mark.parametrize("which,policy", [("box", "spec"), ("box", "reference"), ("ico", "reference"), ("ico", "spec")])
def test_sample_radiance_matches_oracle(which, policy, gpu_ctx, box, ico):
    """Per-sample radiance of one frame, FP32 device vs FP32 oracle: the same
    paths; differences come only from transcendental rounding (relative RMSE
    tolerance 1e-3 over the frame)."""
    hs, sc, osc = box if which == "box" else ico
    W, H = (64, 64) if which == "box" else (96, 54)
    bounces = 5 if which == "box" else 8
    d = integrator_desc(W, H, bounces=bounces, policy=policy)
    f = hx.frame_desc(hs.camera(), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=bounces, policy=d.policy)
    for frame in (0, 3):
        g = it.sample_radiance(f, frame)
        o, _ = osc.sample_radiance(d, f, frame, precision=32)
        close = np.all(np.abs(g - o) <= 1e-4 * (1 + np.abs(o)), axis=1)
        far = np.nonzero(~close)[0]
        info = (frame, rel_rmse(g, o), far.size, [(int(i), g[i].tolist(), o[i].tolist()) for i in far[:4]])
        # the same paths: all but a few samples agree to float rounding; a
        # rare sample may take another branch (a sky texel rounded to a
        # neighbouring FP16 value moves an importance-sampled direction)
        assert close.mean() > 0.995, info
        assert rel_rmse(g, o) < 1e-2, info
    it.close()


@pytest.mark.parametrize("bounces", [0, 1, 2, 24])
def test_sample_radiance_at_depth_limits_matches_oracle(bounces, gpu_ctx, ico):
    """The depth limit's edges: 0 and 1 (the camera hit is shaded, emission and
    NEE, but no indirect ray leaves it: (depth + 1) < max_ray_bounces fails for
    both, as in the reference), two, and 24 (paths end by Russian roulette
    long before the limit), per-sample against the oracle."""
    hs, sc, osc = ico
    W, H = 96, 54
    d = integrator_desc(W, H, bounces=bounces, policy="spec")
    f = hx.frame_desc(hs.camera(), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=bounces, policy=d.policy)
    for frame in (0, 3):
        g = it.sample_radiance(f, frame)
        o, _ = osc.sample_radiance(d, f, frame, precision=32)
        close = np.all(np.abs(g - o) <= 1e-4 * (1 + np.abs(o)), axis=1)
        assert close.mean() > 0.995, (bounces, frame, rel_rmse(g, o))
        assert rel_rmse(g, o) < 1e-2, (bounces, frame, rel_rmse(g, o))
    it.close()


def test_partitioned_shading_list_samples_match_oracle(gpu_ctx, ico):
    """A wavefront of 2^19 paths (1024 x 512, one frame) is shaded from the
    slot-order partition of each bounce's rays (misses ascending, hits
    descending) instead of the traversal's appends: per-sample radiance on
    4,096 seeded pixels against the FP32 oracle, as for small frames.  A
    lost or doubled list entry would leave a path unshaded or shade it twice
    (the kernel also flags a list that does not cover the bounce)."""
    hs, sc, osc = ico
    W, H = 1024, 512
    d = integrator_desc(W, H, bounces=8, policy="reference")
    f = hx.frame_desc(hs.camera(), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=8, policy=d.policy)
    pix = np.random.default_rng(17).choice(W * H, size=4096, replace=False).astype(np.uint32)
    for frame in (0, 3):
        g = it.sample_radiance(f, frame)[pix]
        o, _ = osc.sample_radiance(d, f, frame, precision=32, pixels=pix)
        close = np.all(np.abs(g - o) <= 1e-4 * (1 + np.abs(o)), axis=1)
        info = (frame, rel_rmse(g, o), int((~close).sum()))
        assert close.mean() > 0.995, info
        assert rel_rmse(g, o) < 1e-2, info
        assert np.abs(g).max() > 0.0
    it.close()


def test_shading_list_modes_give_identical_images(gpu_ctx, ico):
    """512 x 512 frames one per wavefront (2^18 paths: the traversal appends
    the shading list) and two per wavefront (2^19 paths: the partition builds
    it) accumulate bit-identical images — shading order never changes a
    path's arithmetic."""
    hs, sc, _ = ico
    W = H = 512
    f = hx.frame_desc(hs.camera(), W, H)
    one = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=6, max_paths_in_flight=W * H)
    two = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=6, max_paths_in_flight=2 * W * H)
    for _ in range(4):
        one.render(f, 1)
    two.render(f, 4)
    a, b = one.read_accumulation(), two.read_accumulation()
    assert a.tobytes() == b.tobytes()
    assert one.num_accumulated_samples() == two.num_accumulated_samples() == 4
    one.close()
    two.close()


def test_accumulation_and_tonemap_match_oracle(gpu_ctx, box):
    hs, sc, osc = box
    W = H = 64
    d = integrator_desc(W, H, policy="spec")
    f = hx.frame_desc(hs.camera(), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=5, policy=d.policy)
    it.render(f, 32)
    acc = it.read_accumulation()
    o, _ = osc.render(d, f, 32, precision=32)
    assert rel_rmse(acc[:, :, :3].reshape(-1, 3), o) < 1e-3
    ldr = it.tonemap(hx.TONEMAP_ACES, 1.0)
    ref = ob.tonemap(acc, hx.TONEMAP_ACES, 1.0)
    assert np.abs(ldr.astype(int) - ref.astype(int)).max() <= 1
    ldr = it.tonemap(hx.TONEMAP_REINHARD, 2.0)
    ref = ob.tonemap(acc, hx.TONEMAP_REINHARD, 2.0)
    assert np.abs(ldr.astype(int) - ref.astype(int)).max() <= 1
    it.close()


def test_batched_frames_equal_sequential(gpu_ctx, box):
    hs, sc, _ = box
    W = H = 48
    f = hx.frame_desc(hs.camera(), W, H)
    a = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=5)
    b = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=5)
    a.render(f, 12)
    for _ in range(12):
        b.render(f, 1)
    assert np.array_equal(a.read_accumulation(), b.read_accumulation())
    assert a.num_accumulated_samples() == b.num_accumulated_samples() == 12
    a.close()
    b.close()


def test_progressive_and_tiled_schedule(gpu_ctx, box):
    hs, sc, _ = box
    W, H = 200, 150  # 2 x 2 tiles of 128
    f = hx.frame_desc(hs.camera(), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=3, max_samples=4, tiled=True)
    assert it.num_target_samples() == 16
    it.render(f, 5)
    acc, tile, _ = it.progress()
    assert (acc, tile) == (5, 1)
    img = it.read_accumulation()
    assert np.all(img[:128, :128, 3] == 1.0) and np.all(img[:, 128:, 3] == 0.0)
    it.render(f, 100)
    assert it.progress()[:2] == (16, 4)
    before = it.read_accumulation()
    it.render(f, 3)  # bake finished: nothing more is traced
    assert np.array_equal(before, it.read_accumulation())
    it.restart_bake()
    assert it.progress()[:2] == (0, 0)
    it.close()


def test_converged_radiance_vs_fp64_oracle(gpu_ctx, box):
    """Box scene, spec policy, 16384 samples per pixel: relative RMSE of the
    device image against the FP64 oracle at the same seeds <= 1e-3 on a seeded
    subset of 256 pixels."""
    hs, sc, osc = box
    W = H = 256
    spp = 16384
    d = integrator_desc(W, H, policy="spec", max_samples=spp)
    f = hx.frame_desc(hs.camera(), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=5, max_samples=spp, policy=d.policy)
    it.render(f, spp)
    img = it.read_accumulation()[:, :, :3].reshape(-1, 3)
    pix = np.random.default_rng(3).choice(W * H, size=256, replace=False).astype(np.uint32)
    o, _ = osc.render(d, f, spp, precision=64, pixels=pix)
    err = rel_rmse(img[pix], o)
    assert err <= 1e-3, err
    it.close()


@pytest.mark.parametrize("scene", ["ico", "bench"])
def test_converged_radiance_sky_scenes_vs_fp64_oracle(scene, gpu_ctx, ico):
    """Scenes with the Hosek-Wilkie sky (importance-sampled), point lights and
    alpha-tested quads, reference policy, 16384 samples per pixel: relative
    RMSE <= 1e-3 against the FP64 oracle at the same seeds on a seeded pixel
    subset.  "bench" is the full 1.18M-triangle benchmark scene at 96x54."""
    if scene == "ico":
        hs, sc, osc = ico
        close = False
    else:
        hs = hx.HostScene(hx.SCENE_ICOSPHERES)
        sc = hx.Scene(gpu_ctx, hs)
        osc = ob.OracleScene(hs)
        close = True
    W, H, spp = 96, 54, 16384
    pol = hx.policy_reference()
    pol.env_sampling = hx.ENV_SAMPLE_IMPORTANCE
    d = integrator_desc(W, H, bounces=8, policy="reference", max_samples=spp)
    d.policy = pol
    f = hx.frame_desc(hs.camera(), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=8, max_samples=spp, policy=pol)
    it.render(f, spp)
    img = it.read_accumulation()[:, :, :3].reshape(-1, 3)
    pix = np.random.default_rng(9).choice(W * H, size=96, replace=False).astype(np.uint32)
    o, _ = osc.render(d, f, spp, precision=64, pixels=pix)
    err = rel_rmse(img[pix], o)
    it.close()
    if close:
        sc.close()
    assert err <= 1e-3, err


def test_environment_bake_matches_oracle(ico, gpu_ctx):
    hs, sc, osc = ico
    w, h = hs.params.env_width, hs.params.env_height
    g = sc.export_env(w, h)
    o = osc.env(w, h)
    # FP16 texels from FP32 device math vs FP64 host math: within 2 half ulps
    assert np.allclose(g, o, rtol=2e-3, atol=1e-6)


def test_errors_are_reported_not_raised_on_device(gpu_ctx, box):
    hs, sc, _ = box
    with pytest.raises(hx.HxError) as e:
        hx.PathIntegrator(gpu_ctx, sc, 0, 10)
    assert e.value.status == hx.HX_ERR_INVALID_ARG
    small = hx.Context(0, hbm_budget_bytes=1 << 20)
    with pytest.raises(hx.HxError) as e:
        hx.PathIntegrator(small, hx.Scene(small, hs) if False else sc, 512, 512)
    assert e.value.status == hx.HX_ERR_OOM_BUDGET
    small.close()


def test_cpp_driver_renders(tmp_path):
    """The C++ surface renders through the C-ABI on the GPU."""
    import subprocess
    from helios_gb300 import build as b
    exe = b.build_driver()
    out = tmp_path / "box.png"
    r = subprocess.run([exe, "box", "128", "128", "16", str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    img = decode_png(out.read_bytes())
    assert img.shape == (128, 128, 4) and (img[..., 3] == 255).all() and img[..., :3].max() > 0
    assert "16 samples accumulated" in r.stdout


def test_importance_sampled_sky_samples_match_oracle(gpu_ctx, ico):
    """Per-sample radiance with the importance-sampled sky (2-D CDF inversion,
    guide-table-accelerated on the device, plain binary search in the
    oracle): the same texel choices, so FP32 samples agree to rounding."""
    hs, sc, osc = ico
    W, H = 96, 64
    pol = hx.policy_reference()
    pol.env_sampling = hx.ENV_SAMPLE_IMPORTANCE
    d = integrator_desc(W, H, bounces=6, policy="reference")
    d.policy = pol
    f = hx.frame_desc(hs.camera(), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=6, policy=pol)
    for frame in (0, 7):
        g = it.sample_radiance(f, frame)
        o, _ = osc.sample_radiance(d, f, frame, precision=32)
        close = np.all(np.abs(g - o) <= 1e-4 * (1 + np.abs(o)), axis=1)
        assert close.mean() > 0.999, (frame, int((~close).sum()))
        assert rel_rmse(g, o) < 1e-4
    it.close()


@pytest.mark.parametrize("case", ["one_triangle", "no_geometry", "no_lights"])
def test_degenerate_scenes_match_oracle(gpu_ctx, case):
    """Edge scenes: a single triangle (a one-leaf BVH), no geometry at all
    (every ray misses; no BVH nodes), and geometry without any light (no NEE
    draw).  Primary hits bit-exact and per-sample radiance against the
    oracle; the accumulated image stays finite."""
    from tests.helpers import TexturedQuadScene
    q = TexturedQuadScene(np.full((8, 8, 4), 200, np.uint8), albedo_srgb=False)
    if case == "one_triangle":
        q._sub[0].index_count = 3
        q._mesh[0].num_indices = 3
    elif case == "no_geometry":
        q._desc.num_meshes = 0
        q._desc.num_instances = 0
    else:
        q._desc.num_punctual_lights = 0
    sc = hx.Scene(gpu_ctx, q)
    osc = ob.OracleScene(q)
    W = H = 32
    d = integrator_desc(W, H, bounces=4, policy="reference")
    f = hx.frame_desc(q.camera(), W, H)
    it = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=4, policy=d.policy)
    gh = it.primary_hits(f, 0)
    oh = osc.trace(ob.primary_rays(d, f, 0), any_hit=True)
    assert np.array_equal(gh["prim"], oh["prim"]) and np.array_equal(gh["t"], oh["t"])
    if case == "no_geometry":
        assert (gh["prim"] == hx.NO_HIT).all()
    else:
        assert (gh["prim"] != hx.NO_HIT).any()
    for frame in (0, 3):
        g = it.sample_radiance(f, frame)
        o, _ = osc.sample_radiance(d, f, frame, precision=32)
        assert np.all(np.abs(g - o) <= 1e-4 * (1 + np.abs(o))), (frame, rel_rmse(g, o))
    it.render(f, 8)
    acc = it.read_accumulation()
    assert np.isfinite(acc).all()
    if case != "one_triangle":
        assert np.abs(acc[..., :3]).max() == 0.0
    it.close()
    sc.close()

