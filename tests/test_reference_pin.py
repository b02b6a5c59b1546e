"""CPU tests: the oracle's restatement against the reference's own shader code.

oracle/glslref/build.py copies the reference's GLSL functions (random.glsl,
sampling.glsl, brdf.glsl, common.glsl, path_trace_rgen/rchit/rahit/rmiss,
the shadow shaders, tone_map.frag) out of the reference tree, compiles them
as C++ with a GLSL shim, and runs them beside the oracle on the same inputs.
Ray/triangle intersection (driver / RT-core work in the reference) is the
same watertight test on both sides, so the comparisons isolate the shading
code.  GLSL leaves the precision of normalize, division and the built-ins to
the implementation; the oracle (like the device) evaluates normalize and
vector / scalar as a reciprocal times the components, the shim as written,
so floating-point results agree to a few ulps and a path can take another
branch where a comparison lands within those ulps.  Integer outputs (RNG
streams, draws consumed, primary hit triangles, flags) must be identical.

Needs the reference tree (in this container); skipped without it.
"""
import numpy as np
import pytest

import helios_gb300 as hx
from oracle import binding as ob
from oracle import glslref
from tests.helpers import LightsScene, integrator_desc, rel_rmse, small_icosphere_scene

pytestmark = pytest.mark.skipif(glslref.load() is None, reason="reference tree absent: nothing to pin against")


def _unit(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def test_rng_streams_equal_reference_code():
    """rng_init / rng_next / next_float / next_uint (random.glsl:11-50,
    sampling.glsl:6-16): identical bits for 5,000 seeds x 16 draws."""
    rng = np.random.default_rng(11)
    n = 5000
    seeds = np.stack([rng.integers(0, 1 << 16, n), rng.integers(0, 1 << 16, n), rng.integers(0, 1 << 30, n)], 1)
    a, b = glslref.rng_cases(seeds.astype(np.uint32), 16)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("aperture", [0.0, 0.1])
def test_camera_rays_equal_reference_code(aperture):
    """generate_ray (path_trace_rgen.glsl:132-174), pinhole and the
    reference's default thin lens (aperture 0.1, scene.h:260): the same four
    draws consumed (RNG state bit-exact), origin and direction within 2 ulps
    (of the component, and of 1 for the unit direction)."""
    hs = LightsScene()
    W, H = 80, 48
    f = hx.frame_desc(hs.camera(aperture=aperture), W, H)
    d = integrator_desc(W, H, policy="reference")
    pix = np.arange(W * H, dtype=np.uint32)
    for frame in (0, 5):
        a, b = glslref.camera_cases(d, f, frame, pix)
        assert np.array_equal(a[:, 6:8].view(np.uint32), b[:, 6:8].view(np.uint32))
        tol = 2 * np.spacing(np.maximum(np.abs(a[:, :3]), np.abs(b[:, :3])).astype(np.float32))
        assert (np.abs(a[:, :3] - b[:, :3]) <= tol).all()               # origins
        assert np.abs(a[:, 3:6] - b[:, 3:6]).max() <= 2 * 2.0 ** -23    # unit directions


def test_bsdf_equals_reference_code():
    """D_ggx, G1_schlick_ggx, evaluate_uber, pdf_uber, sample_uber,
    sample_cosine_lobe, uniform_sample_triangle (brdf.glsl:6-167) on 10^5
    random surfaces and directions.  G1 and the triangle sample are
    bit-identical; the rest differ only through normalize's rounding
    (Wh = normalize(Wo + Wi)), amplified where GGX is steep."""
    rng = np.random.default_rng(12)
    n = 100000
    N, Wo, Wi = _unit(rng, n), _unit(rng, n), _unit(rng, n)
    Wo = np.where((Wo * N).sum(1, keepdims=True) < 0, -Wo, Wo)
    cases = np.concatenate([N, Wo, Wi, rng.uniform(0, 1, (n, 3)), rng.uniform(0.1, 1, (n, 1)),
                            rng.uniform(0, 1, (n, 1)), rng.uniform(0, 1, (n, 2))], 1)
    states = rng.integers(0, 2 ** 32, (n, 2), dtype=np.uint64).astype(np.uint32)
    a, b = glslref.brdf_cases(cases, states)
    assert np.array_equal(a[:, 1], b[:, 1])          # G1
    assert np.array_equal(a[:, 16:18], b[:, 16:18])  # uniform_sample_triangle
    scal = [0, 2, 3, 4, 5, 9, 10, 11, 12]            # D, evaluate rgb, pdf, sampled pdf and value
    rel = np.abs(a[:, scal] - b[:, scal]) / np.maximum(np.abs(b[:, scal]), 1e-6)
    assert np.quantile(rel, 0.9999) < 2e-4
    dirs = [6, 7, 8, 13, 14, 15]                     # sampled Wi, cosine-lobe direction
    err = np.abs(a[:, dirs] - b[:, dirs])
    assert np.quantile(err, 0.9999) < 2e-6
    # a sampled lobe may flip where NdotL lands within an ulp of 0
    assert ((rel > 1e-3).any(1) | (err > 1e-4).any(1)).mean() < 1e-4


def test_sample_light_equals_reference_code():
    """sample_light (path_trace_rchit.glsl:284-451) for the area, environment,
    directional, point and spot lights of one scene: the same draws consumed,
    the same shadow-ray flags (any-hit only at depth 0), origin and tmax;
    direction, radiance and pdf within a few ulps."""
    hs = LightsScene()
    osc = ob.OracleScene(hs)
    world = glslref.RefWorld(hs, osc, env_size=(64, 32))
    types = world.lights[:, 0].astype(int)
    assert sorted(types.tolist()) == [hx.LIGHT_DIRECTIONAL, hx.LIGHT_SPOT, hx.LIGHT_POINT, hx.LIGHT_ENVIRONMENT,
                                      hx.LIGHT_AREA]
    rng = np.random.default_rng(13)
    n = 25000
    pos = np.concatenate([rng.uniform(-2.5, 2.5, (n, 1)), rng.uniform(0, 1.5, (n, 1)), rng.uniform(-2.5, 2.5, (n, 1))], 1)
    nrm = rng.normal(size=(n, 3))
    nrm[:, 1] = np.abs(nrm[:, 1]) + 0.3
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    li = np.arange(n) % len(types)
    cases = np.concatenate([pos, nrm, rng.integers(0, 3, (n, 1)), li[:, None]], 1)
    states = rng.integers(0, 2 ** 32, (n, 2), dtype=np.uint64).astype(np.uint32)
    d = integrator_desc(64, 64, bounces=6, policy="reference", bias=0.001)
    a, b = world.sample_light_cases(osc, d, cases, states)
    assert np.array_equal(a[:, 13:15].view(np.uint32), b[:, 13:15].view(np.uint32))  # draws consumed
    lit = np.abs(b[:, 3:6]).sum(1) > 0
    assert np.array_equal(a[lit, 8], b[lit, 8]) and np.array_equal(a[lit, 9], b[lit, 9])
    assert np.abs(a[lit, 7] - b[lit, 7]).max() <= 1e-6 * np.abs(b[lit, 7]).max()
    assert np.array_equal(a[lit, 10:13], b[lit, 10:13])
    assert np.abs(a[:, 0:3] - b[:, 0:3]).max() < 5e-7
    for k, t in enumerate(types):
        s = li == k
        rel_li = np.abs(a[s, 3:6] - b[s, 3:6]) / np.maximum(np.abs(b[s, 3:6]), 1e-3)
        rel_pdf = np.abs(a[s, 6] - b[s, 6]) / np.maximum(np.abs(b[s, 6]), 1e-6)
        # the spot's smoothstep over its cone edge (slope 1 / (cos inner - cos
        # outer) = 10) amplifies the ulps of normalize(to_light)
        bound = 2e-4 if t == hx.LIGHT_SPOT else 1e-5
        assert np.quantile(rel_li, 0.999) < bound, (t, rel_li.max())
        assert rel_pdf.max() < 1e-5, (t, rel_pdf.max())
    world.close()
    osc.close()


def _paths(scene, W, H, bounces, camera, env_size=None, frame=1):
    osc = ob.OracleScene(scene)
    world = glslref.RefWorld(scene, osc, env_size=env_size)
    f = hx.frame_desc(camera, W, H)
    d = integrator_desc(W, H, bounces=bounces, policy="reference")
    ref, prim, t = world.sample_radiance(d, f, frame)
    ora, hits = osc.sample_radiance(d, f, frame, 32)
    world.close()
    osc.close()
    return ref, prim, t, ora, hits


@pytest.mark.parametrize("kind", ["box", "lights", "lights_dof", "icospheres"])
def test_paths_equal_reference_code(kind):
    """Whole camera samples through the reference's ray-gen / closest-hit /
    any-hit / miss / shadow shaders (payload recursion as written) against
    the oracle's loop: primary hit triangles identical, t within 2e-6 relative,
    >= 99.9 % of the per-sample radiances within 1e-4 relative."""
    if kind == "box":
        hs = hx.HostScene(hx.SCENE_BOX)
        args = (64, 64, 5, hs.camera(), None)
    elif kind.startswith("lights"):
        hs = LightsScene()
        args = (96, 64, 6, hs.camera(aperture=0.1 if kind == "lights_dof" else 0.0), (64, 32))
    else:
        hs = small_icosphere_scene()
        args = (96, 54, 8, hs.camera(), (hs.params.env_width, hs.params.env_height))
    ref, prim, t, ora, hits = _paths(hs, *args)
    assert np.array_equal(prim, hits["prim"])
    # the camera direction carries normalize's rounding (twice through the
    # thin lens), so t agrees to a few ulps
    assert (np.abs(t - hits["t"]) <= 2e-6 * np.abs(hits["t"])).all()
    close = np.all(np.abs(ref - ora) <= 1e-4 * np.maximum(1.0, np.abs(ora)), axis=1)
    assert close.mean() >= 0.999, close.mean()


def test_accumulation_equals_reference_code():
    """Six progressive frames through the reference's ray-gen main(), which
    blends each clamped sample into the ping-pong images (running mean,
    frame 1 overwriting frame 0: path_trace_rgen.glsl:217-248), against the
    oracle's accumulation."""
    hs = LightsScene()
    osc = ob.OracleScene(hs)
    world = glslref.RefWorld(hs, osc, env_size=(64, 32))
    W, H = 48, 32
    f = hx.frame_desc(hs.camera(aperture=0.1), W, H)
    d = integrator_desc(W, H, bounces=6, policy="reference")
    img = world.render(d, f, 6)
    o, _ = osc.render(d, f, 6, precision=32)
    assert (img[..., 3] == 1.0).all()
    assert rel_rmse(img[..., :3].reshape(-1, 3), o) < 1e-4
    world.close()
    osc.close()


@pytest.mark.parametrize("op", [hx.TONEMAP_ACES, hx.TONEMAP_REINHARD, hx.TONEMAP_NONE])
def test_tonemap_equals_reference_code(op):
    """tone_map.frag (exposure, ACES fit / Reinhard, gamma 1/2.2) with the
    UNORM8 store, on log-normal HDR values: identical bytes."""
    rng = np.random.default_rng(14)
    hdr = np.exp(rng.normal(-1.0, 1.5, (64, 96, 4))).astype(np.float32)
    for exposure in (0.7, 1.0, 2.5):
        a = glslref.tonemap(hdr, op, exposure)
        b = ob.tonemap(hdr, op, exposure)
        assert np.array_equal(a, b)
