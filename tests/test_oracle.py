"""CPU tests: the oracle against the golden vectors and its own invariants."""
import json
import os

import numpy as np
import pytest

import helios_gb300 as hx
from oracle import binding as ob
from tests.helpers import integrator_desc, random_rays, rel_rmse, small_icosphere_scene

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_rng_known_answers():
    kat = json.load(open(os.path.join(GOLDEN, "rng_kat.json")))
    seeds = np.array([c["seed"] for c in kat["streams"]], np.uint32)
    xo = ob.rng_streams(0, seeds, kat["draws"])
    pc = ob.rng_streams(1, seeds, kat["draws"])
    for i, c in enumerate(kat["streams"]):
        assert xo[i].tolist() == c["xoroshiro64star"]
        assert pc[i].tolist() == c["pcg"]
    for v, h in kat["hashes"]["wang"]:
        assert ob.lib().oracle_wang_hash(v) == h
    for v, h in kat["hashes"]["pcg"]:
        assert ob.lib().oracle_pcg_hash(v) == h


def test_half_conversion_round_trip():
    vals = np.array([0.0, 1.0, -2.5, 65504.0, 1e-5, 3.14159, 0.1, 6.1e-5, 5.96e-8, 70000.0], np.float32)
    for v in vals:
        h = ob.lib().oracle_float_to_half(float(v))
        assert np.float16(v).view(np.uint16) == h, v
        assert ob.lib().oracle_half_to_float(h) == np.float32(np.float16(v))


def _scene(kind):
    if kind == "box":
        return hx.HostScene(hx.SCENE_BOX)
    return small_icosphere_scene()


@pytest.mark.parametrize("kind", ["box", "ico"])
def test_bvh_traversal_matches_brute_force(kind):
    hs = _scene(kind)
    osc = ob.OracleScene(hs)
    lo, hi = (0.05, 0.95) if kind == "box" else (-25, 25)
    rays = random_rays(4000, lo, hi, seed=3)
    for any_hit in (False, True):
        a = osc.trace(rays, any_hit=any_hit)
        b = osc.trace(rays, any_hit=any_hit, brute=True)
        assert np.array_equal(a["prim"], b["prim"])
        assert np.array_equal(a["t"], b["t"])


@pytest.mark.parametrize("kind", ["box", "ico"])
def test_bvh8_traversal_never_loses_a_hit(kind):
    """The quantised 8-wide tree, traversed in the device's arithmetic (exact
    plane decode, widened far planes, octant order), finds exactly the
    brute-force closest hits."""
    hs = _scene(kind)
    osc = ob.OracleScene(hs)
    lo, hi = (0.05, 0.95) if kind == "box" else (-25, 25)
    rays = random_rays(20000, lo, hi, seed=5)
    for any_hit in (False, True):
        a, _ = osc.trace_bvh8(rays, any_hit=any_hit)
        b = osc.trace(rays, any_hit=any_hit, brute=True)
        bad = np.nonzero(a["prim"] != b["prim"])[0]
        assert bad.size == 0, (bad[:5], a[bad[:5]], b[bad[:5]])
        assert np.array_equal(a["t"], b["t"])


@pytest.mark.parametrize("kind", ["box", "ico"])
def test_bvh8_structure(kind):
    hs = _scene(kind)
    osc = ob.OracleScene(hs)
    b = osc.export_bvh()
    n = osc.num_prims
    # every triangle lands in exactly one leaf slot
    assert np.array_equal(np.sort(b["leaf_prims"]), np.arange(n, dtype=np.uint32))
    assert np.array_equal(np.sort(b["sorted"]), np.arange(n, dtype=np.uint32))
    # Morton codes sorted along the stable order
    m = b["morton"][b["sorted"]]
    assert np.all(m[1:] >= m[:-1])
    # conservative quantisation: decoded child boxes contain their triangles
    nodes = b["nodes"]
    # every decoded plane origin + q 2^e (and origin - 2^23 2^e) is exactly
    # representable in FP32, so any single-rounding decode is exact
    scale64 = np.ldexp(1.0, nodes["exponent"].astype(np.int32))
    for qname in ("qlo", "qhi"):
        dec = nodes["origin"].astype(np.float64)[:, :, None] + nodes[qname].astype(np.float64) * scale64[:, :, None]
        assert np.array_equal(dec, dec.astype(np.float32).astype(np.float64))
    shifted = nodes["origin"].astype(np.float64) - 8388608.0 * scale64
    assert np.array_equal(shifted, shifted.astype(np.float32).astype(np.float64))
    from tests.test_oracle import _world_tris
    tris = _world_tris(hs)
    for node in nodes:
        scale = np.ldexp(np.float32(1.0), node["exponent"].astype(np.int32)).astype(np.float32)
        for c in range(8):
            meta = int(node["meta"][c])
            if meta == 0x10 or meta & 0x80:  # empty or internal slot
                continue
            assert meta >> 5 == 1  # one triangle per leaf slot
            cnt, off = 1, meta & 31
            lo = (node["origin"] + node["qlo"][:, c].astype(np.float32) * scale).astype(np.float32)
            hi = (node["origin"] + node["qhi"][:, c].astype(np.float32) * scale).astype(np.float32)
            for q in range(cnt):
                p = b["leaf_prims"][node["prim_base"] + off + q]
                v = tris[p]
                assert np.all(v >= lo - 0.0) and np.all(v <= hi + 0.0)


def _world_tris(hs):
    """World-space triangles in flattened order, computed like the oracle."""
    d = hs.desc.contents
    out = []
    for ii in range(d.num_instances):
        inst = d.instances[ii]
        M = np.array(inst.model_matrix[:], np.float32).reshape(4, 4)  # column-major: M[col][row]
        mesh = d.meshes[inst.mesh_index]
        for si in range(mesh.num_submeshes):
            sm = mesh.submeshes[si]
            for t in range(sm.index_count // 3):
                tri = []
                for c in range(3):
                    v = mesh.vertices[mesh.indices[sm.base_index + 3 * t + c]]
                    p = [np.float32(v.position[0]), np.float32(v.position[1]), np.float32(v.position[2])]
                    row = []
                    for r in range(3):
                        acc = np.float32(M[0][r] * p[0])
                        acc = np.float32(acc + np.float32(M[1][r] * p[1]))
                        acc = np.float32(acc + np.float32(M[2][r] * p[2]))
                        acc = np.float32(acc + np.float32(M[3][r] * np.float32(1.0)))
                        row.append(acc)
                    tri.append(row)
                out.append(tri)
    return np.array(out, np.float32)


def test_fp32_matches_fp64_oracle():
    hs = hx.HostScene(hx.SCENE_BOX)
    osc = ob.OracleScene(hs)
    d = integrator_desc(48, 48)
    f = hx.frame_desc(hs.camera(), 48, 48)
    a, _ = osc.render(d, f, 32, precision=32)
    b, _ = osc.render(d, f, 32, precision=64)
    assert rel_rmse(a, b) < 1e-4


def test_scaled_ray_offset_removes_the_fp32_bias_at_world_scale():
    """The terrain spans 4096 units: FP32 hit positions there carry rounding
    above the reference's fixed tmin of 1e-4 (ulp(2048) = 2.4e-4), so in FP32
    some secondary and shadow rays re-hit the surface they leave — a bias
    against the FP64 evaluation of the same samples that does not shrink with
    more samples.  HX_RAY_OFFSET_SCALED moves the origins off the surface by a
    position-relative amount; what is left between FP32 and FP64 is the noise
    of paths that diverge by rounding (it falls with the sample count).
    Measured here: 3.1e-3 with the reference's origins, 0.9e-3 with scaled
    ones; FP64 images with and without the offset differ by 1.0e-4 (the
    offset moves origins by at most 2^-15 of their coordinates)."""
    hs = hx.HostScene(hx.SCENE_TERRAIN, terrain_size=256, num_spheres=40, env_width=256, env_height=128)
    osc = ob.OracleScene(hs)
    W, H = 1920, 1080
    f = hx.frame_desc(hs.camera(), W, H)
    pix = np.random.default_rng(11).choice(W * H, size=1024, replace=False).astype(np.uint32)
    err, img64 = {}, {}
    for off in (hx.RAY_OFFSET_REFERENCE, hx.RAY_OFFSET_SCALED):
        d = integrator_desc(W, H, bounces=8, policy="reference", max_samples=1 << 30)
        d.policy.env_sampling = hx.ENV_SAMPLE_IMPORTANCE
        d.policy.ray_offset = off
        img64[off], _ = osc.render(d, f, 1024, precision=64, pixels=pix)
        r32, _ = osc.render(d, f, 1024, precision=32, pixels=pix)
        err[off] = rel_rmse(r32, img64[off])
    print("FP32 vs FP64 relative RMSE (reference origins, scaled origins):", err)
    assert err[hx.RAY_OFFSET_SCALED] < 0.4 * err[hx.RAY_OFFSET_REFERENCE], err
    assert err[hx.RAY_OFFSET_SCALED] < 1.5e-3, err
    assert rel_rmse(img64[hx.RAY_OFFSET_SCALED], img64[hx.RAY_OFFSET_REFERENCE]) < 5e-4


def test_scaled_origins_leave_the_surface_at_world_scale():
    """HX_RAY_OFFSET_SCALED as a property: FP32 hit points (barycentric
    interpolation of triangles whose coordinates reach 4096) offset along the
    FP32 geometric normal lie strictly on the side the ray leaves on, measured
    against the exact (FP64) plane of the triangle, for every one of 200,000
    hits; the raw FP32 hit points (the reference's origins) fall on the wrong
    side or on the plane for a large share of them."""
    import ctypes as C
    rng = np.random.default_rng(21)
    n = 200_000
    c = rng.uniform(-4096, 4096, (n, 1, 3))
    v = (c + rng.uniform(-4, 4, (n, 3, 3))).astype(np.float32)
    b = rng.dirichlet((1, 1, 1), n).astype(np.float32)
    p32 = (v[:, 0] * b[:, :1] + v[:, 1] * b[:, 1:2] + v[:, 2] * b[:, 2:3]).astype(np.float32)
    e1, e2 = (v[:, 1] - v[:, 0]), (v[:, 2] - v[:, 0])
    ng = np.cross(e1, e2).astype(np.float32)
    ng /= np.linalg.norm(ng, axis=1, keepdims=True)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    out = np.zeros((n, 3), np.float32)
    ptr = lambda a: np.ascontiguousarray(a, np.float32).ctypes.data_as(C.c_void_p)
    p32c, ngc, dc = (np.ascontiguousarray(a, np.float32) for a in (p32, ng, d))
    ob.lib().oracle_offset_origins(ptr(p32c), ptr(ngc), ptr(dc), n, out.ctypes.data_as(C.c_void_p))
    v64 = v.astype(np.float64)
    n64 = np.cross(v64[:, 1] - v64[:, 0], v64[:, 2] - v64[:, 0])
    n64 /= np.linalg.norm(n64, axis=1, keepdims=True)
    side = np.sign(np.einsum("ij,ij->i", d.astype(np.float64), n64))
    keep = side != 0
    dist_off = np.einsum("ij,ij->i", out.astype(np.float64) - v64[:, 0], n64) * side
    dist_raw = np.einsum("ij,ij->i", p32.astype(np.float64) - v64[:, 0], n64) * side
    assert (dist_off[keep] > 0).all(), np.sort(dist_off[keep])[:5]
    wrong_raw = (dist_raw[keep] <= 0).mean()
    print("raw FP32 hit points on the wrong side or on the plane:", wrong_raw)
    assert wrong_raw > 0.2


def test_light_list_reference_order():
    hs = small_icosphere_scene()
    osc = ob.OracleScene(hs)
    L = osc.lights()
    types = L[:, 0].astype(int).tolist()
    # no emissive materials: environment first, then the 4 point lights
    assert types == [hx.LIGHT_ENVIRONMENT] + [hx.LIGHT_POINT] * 4
    box = ob.OracleScene(hx.HostScene(hx.SCENE_BOX)).lights()
    assert box.shape[0] == 1 and int(box[0, 0]) == hx.LIGHT_AREA
    assert box[0, 1] == 3 and box[0, 2] == 3 and box[0, 4] == 2  # instance 3, material 3, 2 triangles


def test_policy_differences_change_the_image():
    hs = hx.HostScene(hx.SCENE_BOX)
    osc = ob.OracleScene(hs)
    f = hx.frame_desc(hs.camera(), 32, 32)
    a, _ = osc.render(integrator_desc(32, 32, policy="spec"), f, 16)
    b, _ = osc.render(integrator_desc(32, 32, policy="reference"), f, 16)
    # the reference samples only triangle 0 of the quad light (light_data1.z is never written)
    assert a.mean() > b.mean()


def test_oracle_srgb_texture_decode():
    """An sRGB-flagged texture decodes its RGB with the sRGB transfer function
    before filtering (resource_manager.cpp:48-67 creates such textures with
    *_SRGB formats); a UNORM one reads q / 255.  A constant texture makes the
    filtered value the decoded texel itself."""
    from tests.helpers import TexturedQuadScene
    tex = np.full((8, 8, 4), 128, np.uint8)
    c = 128 / 255.0
    want = {True: np.float32(((c + 0.055) / 1.055) ** 2.4), False: np.float32(128) / np.float32(255)}
    for srgb in (True, False):
        qs = TexturedQuadScene(tex, albedo_srgb=srgb)
        osc = ob.OracleScene(qs)
        W, H = 40, 30
        f = hx.frame_desc(qs.camera(), W, H)
        alb = osc.output_view(f, W, H, hx.OUTPUT_ALBEDO)
        hit = np.any(alb[..., :3] != 0, axis=-1)
        assert hit.mean() > 0.3
        assert np.all(alb[hit][:, :3] == want[srgb]), (srgb, np.unique(alb[hit][:, :3]))


def test_oracle_albedo_view_reproduces_material_albedos():
    """The oracle's output-buffer view (debug_visualization.frag fetch_albedo)
    on the untextured box: every hit pixel holds exactly one of the scene's
    material albedos, the clear colour elsewhere; roughness likewise."""
    hs = hx.HostScene(hx.SCENE_BOX)
    osc = ob.OracleScene(hs)
    d = hs.desc.contents
    mats = [d.materials[k] for k in range(d.num_materials)]
    albedos = {tuple(np.float32(m.albedo[c]) for c in range(3)) for m in mats}
    rough = {np.float32(m.roughness_metallic[0]) for m in mats}
    W, H = 48, 40
    f = hx.frame_desc(hs.camera(), W, H)
    alb = osc.output_view(f, W, H, hx.OUTPUT_ALBEDO)
    rgh = osc.output_view(f, W, H, hx.OUTPUT_ROUGHNESS)
    hit = np.any(alb[..., :3] != 0, axis=-1)
    assert hit.mean() > 0.5 and np.all(alb[..., 3] == 1.0)
    assert {tuple(p) for p in alb[hit][:, :3].tolist()} <= {tuple(float(x) for x in a) for a in albedos}
    assert set(np.unique(rgh[hit][:, 0]).tolist()) <= {float(r) for r in rough}


def test_oracle_visualize_nans_marks_the_nan_surface():
    """VISUALIZE_NANS in the oracle: a quad whose material emits NaN turns
    exactly its covered pixels (1, 0, 0); the rest stays black (no lights)."""
    from tests.helpers import TriangleSoupScene, integrator_desc
    q = np.array([[[-1, -1, 0], [1, -1, 0], [1, 1, 0]], [[-1, -1, 0], [1, 1, 0], [-1, 1, 0]]], np.float32)
    soup = TriangleSoupScene(q)
    soup._mat[0].emissive[0] = float("nan")
    cam = hx.Camera()
    cam.position[:] = [0.0, 0.0, 4.0]
    cam.target[:] = [0.0, 0.0, 0.0]
    cam.up[:] = [0.0, 1.0, 0.0]
    cam.fov_y_degrees, cam.near_plane, cam.far_plane = 60.0, 1.0, 1000.0
    cam.focal_length, cam.aperture_radius = 8.0, 0.0
    osc = ob.OracleScene(soup)
    W, H = 32, 24
    f = hx.frame_desc(cam, W, H)
    d = integrator_desc(W, H, bounces=2, policy="reference")
    d.policy.visualize_nans = 1
    img, _ = osc.render(d, f, 1)
    red = np.all(img == np.array([1.0, 0.0, 0.0]), axis=1)
    assert 0.1 < red.mean() < 0.9
    assert np.all(img[~red] == 0.0)
    d.policy.visualize_nans = 0
    raw, _ = osc.render(d, f, 1)
    assert np.array_equal(np.isnan(raw[:, 0]), red)
