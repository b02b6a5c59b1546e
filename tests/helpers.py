"""Shared helpers for the tests (scene/integrator descriptors, metrics)."""
import ctypes as C

import numpy as np

import helios_gb300 as hx


def integrator_desc(width, height, bounces=5, max_samples=5000, policy="spec", bias=0.0, tiled=False):
    d = hx.IntegratorDesc()
    d.width, d.height = width, height
    d.max_ray_bounces, d.max_samples = bounces, max_samples
    d.shadow_ray_bias = bias
    d.tiled = 1 if tiled else 0
    d.policy = hx.policy_spec() if policy == "spec" else hx.policy_reference()
    return d


def rel_rmse(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def small_icosphere_scene(level=3, quads=2000, pool=4, mask=64, env=(128, 64), seed=7):
    return hx.HostScene(hx.SCENE_ICOSPHERES, icosphere_level=level, num_alpha_quads=quads, mask_pool=pool,
                        mask_size=mask, env_width=env[0], env_height=env[1], seed=seed)


def random_rays(n, lo, hi, seed=1, tmin=0.0001, tmax=1e4):
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, size=(n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3] = o
    r[:, 3] = tmin
    r[:, 4:7] = d.astype(np.float32)
    r[:, 7] = tmax
    return r


class TriangleSoupScene:
    """One opaque mesh of free triangles (N x 3 x 3 float32), one grey
    material, an identity instance, no lights and no environment: a scene for
    traversal tests.  .desc points at its hx_scene_desc (arrays kept alive)."""

    def __init__(self, tris):
        tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 3, 3)
        n = tris.shape[0]
        self._verts = (hx.Vertex * (3 * n))()
        for i in range(n):
            for c in range(3):
                v = self._verts[3 * i + c]
                v.position[0], v.position[1], v.position[2], v.position[3] = (float(tris[i, c, 0]), float(tris[i, c, 1]),
                                                                              float(tris[i, c, 2]), 0.0)
                v.normal[1] = 1.0
        self._idx = (C.c_uint32 * (3 * n))(*range(3 * n))
        self._sub = (hx.Submesh * 1)()
        self._sub[0].base_index, self._sub[0].index_count, self._sub[0].material, self._sub[0].flags = 0, 3 * n, 0, 0
        self._mesh = (hx.MeshDesc * 1)()
        m = self._mesh[0]
        m.vertices, m.num_vertices = self._verts, 3 * n
        m.indices, m.num_indices = self._idx, 3 * n
        m.submeshes, m.num_submeshes = self._sub, 1
        self._mat = (hx.Material * 1)()
        mat = self._mat[0]
        for k in range(4):
            mat.texture_indices0[k] = -1
            mat.texture_indices1[k] = -1
        mat.albedo[0] = mat.albedo[1] = mat.albedo[2] = 0.5
        mat.roughness_metallic[0] = 0.5
        self._inst = (hx.Instance * 1)()
        inst = self._inst[0]
        for k in range(4):
            inst.model_matrix[5 * k] = 1.0
            inst.normal_matrix[5 * k] = 1.0
        inst.mesh_index, inst.material_override = 0, -1
        self._desc = hx.SceneDesc()
        d = self._desc
        d.meshes, d.num_meshes = self._mesh, 1
        d.instances, d.num_instances = self._inst, 1
        d.materials, d.num_materials = self._mat, 1
        d.num_textures = 0
        d.num_punctual_lights = 0
        d.environment.kind = 0

    @property
    def desc(self):
        return C.pointer(self._desc)


def decode_png(data):
    """Independent PNG reader (stdlib zlib): checks the signature and every
    chunk CRC, returns (H, W, 4) uint8 for 8-bit RGBA with filter 0 rows."""
    import struct
    import zlib
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, ihdr = 8, b"", None
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        typ, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        (crc,) = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(typ + body) & 0xffffffff, typ
        if typ == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    assert typ == b"IEND" and pos == len(data)
    w, h, depth, ctype, comp, filt, inter = ihdr
    assert (depth, ctype, comp, filt, inter) == (8, 6, 0, 0, 0)
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 4 * w + 1)
    assert (raw[:, 0] == 0).all()
    return raw[:, 1:].reshape(h, w, 4)



class TexturedQuadScene:
    """A floor quad (y = 0, x and z in [-1, 1], 4 x 4 UV repeats) with one
    GGX/Lambert material: an RGBA8 albedo texture (optionally sRGB-encoded),
    an optional tangent-space normal map, tangent +x and bitangent +z; one
    point light above; no environment.  .desc points at its hx_scene_desc,
    .camera() looks down at the quad."""

    def __init__(self, albedo, albedo_srgb=True, normal_map=None, roughness=0.5, albedo_format=0, albedo_wh=None):
        # albedo: (H, W, 4) RGBA8, or block-compressed bytes with albedo_format / albedo_wh = (W, H)
        self._tex_data = [np.ascontiguousarray(albedo, np.uint8)]
        if normal_map is not None:
            self._tex_data.append(np.ascontiguousarray(normal_map, np.uint8))
        pos = [(-1, 0, -1), (1, 0, -1), (1, 0, 1), (-1, 0, 1)]
        uv = [(0, 0), (4, 0), (4, 4), (0, 4)]
        self._verts = (hx.Vertex * 4)()
        for i in range(4):
            v = self._verts[i]
            v.position[0], v.position[1], v.position[2], v.position[3] = pos[i][0], pos[i][1], pos[i][2], 0.0
            v.tex_coord[0], v.tex_coord[1] = uv[i]
            v.normal[1] = 1.0
            v.tangent[0] = 1.0
            v.bitangent[2] = 1.0
        self._idx = (C.c_uint32 * 6)(0, 2, 1, 0, 3, 2)
        self._sub = (hx.Submesh * 1)()
        self._sub[0].base_index, self._sub[0].index_count, self._sub[0].material, self._sub[0].flags = 0, 6, 0, 0
        self._mesh = (hx.MeshDesc * 1)()
        m = self._mesh[0]
        m.vertices, m.num_vertices = self._verts, 4
        m.indices, m.num_indices = self._idx, 6
        m.submeshes, m.num_submeshes = self._sub, 1
        self._mat = (hx.Material * 1)()
        mat = self._mat[0]
        for k in range(4):
            mat.texture_indices0[k] = -1
            mat.texture_indices1[k] = -1
        mat.texture_indices0[0] = 0
        if normal_map is not None:
            mat.texture_indices0[1] = 1
        mat.albedo[0] = mat.albedo[1] = mat.albedo[2] = mat.albedo[3] = 1.0
        mat.roughness_metallic[0] = roughness
        self._tex = (hx.TextureDesc * len(self._tex_data))()
        for k, t in enumerate(self._tex_data):
            self._tex[k].rgba8 = t.ctypes.data_as(C.POINTER(C.c_uint8))
            if k == 0 and albedo_format:
                self._tex[k].width, self._tex[k].height = albedo_wh
                self._tex[k].format = albedo_format
            else:
                self._tex[k].height, self._tex[k].width = t.shape[0], t.shape[1]
            self._tex[k].srgb = 1 if (k == 0 and albedo_srgb) else 0
        self._inst = (hx.Instance * 1)()
        inst = self._inst[0]
        for k in range(4):
            inst.model_matrix[5 * k] = 1.0
            inst.normal_matrix[5 * k] = 1.0
        inst.mesh_index, inst.material_override = 0, -1
        self._light = (hx.Light * 1)()
        lt = self._light[0]
        lt.data0[0], lt.data0[1], lt.data0[2], lt.data0[3] = float(hx.LIGHT_POINT), 1.0, 0.9, 0.8
        lt.data1[3] = 4.0
        lt.data2[0], lt.data2[1], lt.data2[2], lt.data2[3] = 0.3, 1.2, -0.2, 0.05
        self._desc = hx.SceneDesc()
        d = self._desc
        d.meshes, d.num_meshes = self._mesh, 1
        d.instances, d.num_instances = self._inst, 1
        d.materials, d.num_materials = self._mat, 1
        d.textures, d.num_textures = self._tex, len(self._tex_data)
        d.punctual_lights, d.num_punctual_lights = self._light, 1
        d.environment.kind = 0

    @property
    def desc(self):
        return C.pointer(self._desc)

    def camera(self):
        cam = hx.Camera()
        cam.position[:] = [0.0, 1.6, 1.9]
        cam.target[:] = [0.0, 0.0, 0.0]
        cam.up[:] = [0.0, 1.0, 0.0]
        cam.fov_y_degrees, cam.near_plane, cam.far_plane = 50.0, 1.0, 1000.0
        cam.focal_length, cam.aperture_radius = 8.0, 0.0
        return cam


def bump_normal_map(size=64, freq=3, amp=0.35):
    """Tangent-space normal map (RGB = n * 0.5 + 0.5) of a sinusoidal height field."""
    u = (np.arange(size) + 0.5) / size
    du = amp * 2 * np.pi * freq * np.cos(2 * np.pi * freq * u)
    nx, ny = np.meshgrid(-du, -du)
    n = np.stack([nx, ny, np.ones_like(nx)], -1)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    rgba = np.empty((size, size, 4), np.uint8)
    rgba[..., :3] = np.clip(np.round((n * 0.5 + 0.5) * 255), 0, 255).astype(np.uint8)
    rgba[..., 3] = 255
    return rgba


def checker_texture(size=32, a=(200, 180, 150), b=(40, 60, 90)):
    y, x = np.mgrid[0:size, 0:size]
    sel = ((x // 4 + y // 4) % 2 == 0)[..., None]
    rgba = np.where(sel, np.array(a + (255,), np.uint8), np.array(b + (255,), np.uint8)).astype(np.uint8)
    return rgba
