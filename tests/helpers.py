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
        v = np.frombuffer(self._verts, dtype=np.float32).reshape(3 * n, 20)
        v[:, 0:3] = tris.reshape(-1, 3)
        v[:, 9] = 1.0  # normal.y
        self._idx = (C.c_uint32 * (3 * n))()
        np.frombuffer(self._idx, dtype=np.uint32)[:] = np.arange(3 * n, dtype=np.uint32)
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

    def __init__(self, albedo, albedo_srgb=True, normal_map=None, roughness=0.5, albedo_format=0, albedo_wh=None,
                 non_opaque=False, roughness_channel=None):
        # albedo: (H, W, 4) RGBA8, or the bytes of another format (block-compressed, RGBA16F) with
        # albedo_format / albedo_wh = (W, H); non_opaque: alpha-tested submesh; roughness_channel: roughness
        # read from that channel of the albedo texture
        a = np.ascontiguousarray(albedo)
        self._tex_data = [a if a.dtype == np.uint8 else a.view(np.uint8)]
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
        self._sub[0].base_index, self._sub[0].index_count, self._sub[0].material = 0, 6, 0
        self._sub[0].flags = HX_NON_OPAQUE if non_opaque else 0
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
        if roughness_channel is not None:
            mat.texture_indices0[2], mat.texture_indices1[2] = 0, roughness_channel
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


def random_bc7_blocks(n, seed=0):
    """n random BC7 blocks (16 bytes each) cycling through all eight modes:
    the low bits of byte 0 select the mode, every other bit is random."""
    rng = np.random.default_rng(seed)
    blocks = rng.integers(0, 256, size=(n, 16), dtype=np.uint8)
    for i in range(n):
        m = i % 8
        blocks[i, 0] = (int(blocks[i, 0]) & ~((1 << (m + 1)) - 1) & 0xFF) | (1 << m)
    return blocks


BC6H_MODE_CODES = [0b00, 0b01, 0b00010, 0b00110, 0b01010, 0b01110, 0b10010, 0b10110, 0b11010, 0b11110, 0b00011,
                   0b00111, 0b01011, 0b01111]
BC6H_RESERVED_CODES = [0b10011, 0b10111, 0b11011, 0b11111]


def random_bc6h_blocks(n, seed=0, reserved=True):
    """n random BC6H blocks (16 bytes each) cycling through the fourteen mode
    codes (and the four reserved codes when `reserved`): the low two or five
    bits of byte 0 set the code, every other bit is random."""
    rng = np.random.default_rng(seed)
    blocks = rng.integers(0, 256, size=(n, 16), dtype=np.uint8)
    codes = BC6H_MODE_CODES + (BC6H_RESERVED_CODES if reserved else [])
    for i in range(n):
        c = codes[i % len(codes)]
        nb = 2 if c < 2 else 5
        blocks[i, 0] = (int(blocks[i, 0]) & ~((1 << nb) - 1) & 0xFF) | c
    return blocks


def bc6h_mode11_blocks(n, lo=0, hi=256, seed=0):
    """n BC6H blocks of the one-region, untransformed mode (code 00011) with
    every 10-bit endpoint channel drawn from [lo, hi) and random 4-bit indices:
    with hi <= 512 the signed format decodes them to moderate positive values
    (endpoint 248 is about 1.0)."""
    rng = np.random.default_rng(seed)
    out = np.zeros((n, 16), np.uint8)
    for i in range(n):
        bits = 0b00011
        pos = 5
        for _ in range(6):
            bits |= int(rng.integers(lo, hi)) << pos
            pos += 10
        for t in range(16):
            nb = 3 if t == 0 else 4
            bits |= int(rng.integers(0, 1 << nb)) << pos
            pos += nb
        out[i] = np.frombuffer(bits.to_bytes(16, "little"), np.uint8)
    return out


def checker_texture(size=32, a=(200, 180, 150), b=(40, 60, 90)):
    y, x = np.mgrid[0:size, 0:size]
    sel = ((x // 4 + y // 4) % 2 == 0)[..., None]
    rgba = np.where(sel, np.array(a + (255,), np.uint8), np.array(b + (255,), np.uint8)).astype(np.uint8)
    return rgba


def _mat(model):
    """(model, normal) matrices as column-major float lists; normal = inverse transpose."""
    m = np.asarray(model, np.float64)
    n = np.eye(4)
    n[:3, :3] = np.linalg.inv(m[:3, :3]).T
    return m.T.reshape(-1).tolist(), n.T.reshape(-1).tolist()


def _rot_y(deg):
    c, s = np.cos(np.radians(deg)), np.sin(np.radians(deg))
    return np.array([[c, 0, s, 0], [0, 1, 0, 0], [-s, 0, c, 0], [0, 0, 0, 1]])


def _translate_scale(t, s=1.0):
    m = np.eye(4)
    m[:3, :3] *= s
    m[:3, 3] = t
    return m


class LightsScene:
    """A small scene that exercises every light type and surface path of the
    reference's closest-hit shader: a textured (sRGB albedo, tangent-space
    normal map) floor, two instances of a GGX box mesh (rotated and scaled),
    an emissive quad (area light), an alpha-tested quad (non-opaque submesh,
    any-hit), and a point, a spot (distinct cone edges) and a directional
    light, with a small lat-long environment.  .desc points at its
    hx_scene_desc (arrays kept alive); .camera() frames it."""

    def __init__(self, spot_equal_edges=False, env=True):
        self._keep = []
        verts, idx, subs = [], [], []

        def vtx(p, n, uv, t=(1, 0, 0), b=(0, 0, 1), w=0.0):
            v = hx.Vertex()
            v.position[:] = [p[0], p[1], p[2], w]
            v.normal[:] = [n[0], n[1], n[2], 0.0]
            v.tex_coord[:] = [uv[0], uv[1], 0.0, 0.0]
            v.tangent[:] = [t[0], t[1], t[2], 0.0]
            v.bitangent[:] = [b[0], b[1], b[2], 0.0]
            return v

        def quad(c, u, v, n, uv_scale=1.0):
            c, u, v = np.asarray(c, float), np.asarray(u, float), np.asarray(v, float)
            ps = [c - u - v, c + u - v, c + u + v, c - u + v]
            uvs = [(0, 0), (uv_scale, 0), (uv_scale, uv_scale), (0, uv_scale)]
            tu, tv = u / np.linalg.norm(u), v / np.linalg.norm(v)
            return [vtx(p, n, q, tu, tv) for p, q in zip(ps, uvs)], [0, 2, 1, 0, 3, 2]

        meshes = []
        # mesh 0: floor (material 0: sRGB checker albedo + normal map)
        vs, ix = quad((0, 0, 0), (3, 0, 0), (0, 0, 3), (0, 1, 0), uv_scale=3.0)
        meshes.append((vs, ix, [(0, 6, 0, 0)]))
        # mesh 1: unit box (material 1: GGX metal)
        bv, bi = [], []
        for ax in range(3):
            for sgn in (-1, 1):
                n = np.zeros(3)
                n[ax] = sgn
                u = np.zeros(3)
                u[(ax + 1) % 3] = 0.5
                v = np.zeros(3)
                v[(ax + 2) % 3] = 0.5 * sgn
                qv, qi = quad(n * 0.5, u, v, n)
                bi += [k + len(bv) for k in qi]
                bv += qv
        meshes.append((bv, bi, [(0, 36, 1, 0)]))
        # mesh 2: emissive quad facing down (material 2), position.w = 0 (submesh index)
        vs, ix = quad((0.2, 2.4, 0.3), (0.3, 0, 0), (0, 0, -0.25), (0, -1, 0))
        meshes.append((vs, ix, [(0, 6, 2, 0)]))
        # mesh 3: alpha-tested upright quad (material 3, non-opaque)
        vs, ix = quad((0, 1.0, -1.5), (1.2, 0, 0), (0, 1.0, 0), (0, 0, 1), uv_scale=2.0)
        meshes.append((vs, ix, [(0, 6, 3, HX_NON_OPAQUE)]))

        self._mesh = (hx.MeshDesc * len(meshes))()
        for k, (vs, ix, sm) in enumerate(meshes):
            va = (hx.Vertex * len(vs))(*vs)
            ia = (C.c_uint32 * len(ix))(*ix)
            sa = (hx.Submesh * len(sm))()
            for j, (base, cnt, mat, fl) in enumerate(sm):
                sa[j].base_index, sa[j].index_count, sa[j].material, sa[j].flags = base, cnt, mat, fl
            self._keep += [va, ia, sa]
            m = self._mesh[k]
            m.vertices, m.num_vertices = va, len(vs)
            m.indices, m.num_indices = ia, len(ix)
            m.submeshes, m.num_submeshes = sa, len(sm)

        checker = checker_texture(32)
        normal = bump_normal_map(32, freq=2, amp=0.3)
        alpha = checker_texture(32, a=(230, 120, 60), b=(60, 160, 220)).copy()
        yy, xx = np.mgrid[0:32, 0:32]
        alpha[..., 3] = np.where(((xx // 8) + (yy // 8)) % 2 == 0, 255, 0)
        self._tex_data = [checker, normal, alpha]
        self._tex = (hx.TextureDesc * 3)()
        for k, t in enumerate(self._tex_data):
            self._tex[k].rgba8 = t.ctypes.data_as(C.POINTER(C.c_uint8))
            self._tex[k].height, self._tex[k].width = t.shape[0], t.shape[1]
            self._tex[k].srgb = 1 if k in (0, 2) else 0
            self._tex[k].format = 0

        mats = [dict(tex0=(0, 1, -1, -1), albedo=(1, 1, 1, 1), rm=(0.6, 0.2)),
                dict(tex0=(-1, -1, -1, -1), albedo=(0.8, 0.6, 0.3, 1), rm=(0.3, 0.8)),
                dict(tex0=(-1, -1, -1, -1), albedo=(0.9, 0.9, 0.9, 1), rm=(0.5, 0.0), emissive=(6.0, 5.0, 4.0)),
                dict(tex0=(2, -1, -1, -1), albedo=(1, 1, 1, 1), rm=(0.4, 0.0))]
        self._mat = (hx.Material * len(mats))()
        for k, md in enumerate(mats):
            m = self._mat[k]
            for j in range(4):
                m.texture_indices0[j] = md["tex0"][j]
                m.texture_indices1[j] = -1
            m.albedo[:] = list(md["albedo"])
            m.emissive[:] = list(md.get("emissive", (0, 0, 0))) + [0.0]
            m.roughness_metallic[0], m.roughness_metallic[1] = md["rm"]

        inst = [(0, np.eye(4)), (1, _translate_scale((-1.0, 0.5, 0.0)) @ _rot_y(30.0)),
                (1, _translate_scale((1.1, 0.25, 0.8), 0.5) @ _rot_y(-20.0)), (2, np.eye(4)), (3, np.eye(4))]
        self._inst = (hx.Instance * len(inst))()
        for k, (mesh, model) in enumerate(inst):
            mm, nm = _mat(model)
            self._inst[k].model_matrix[:] = mm
            self._inst[k].normal_matrix[:] = nm
            self._inst[k].mesh_index = mesh
            self._inst[k].material_override = -1

        self._light = (hx.Light * 3)()
        pt, sp, di = self._light[0], self._light[1], self._light[2]
        pt.data0[:] = [float(hx.LIGHT_POINT), 1.0, 0.9, 0.8]
        pt.data1[3] = 6.0
        pt.data2[:] = [0.5, 2.0, 1.0, 0.05]
        sdir = np.array([1.0, -2.5, -1.5])
        sdir /= np.linalg.norm(sdir)
        sp.data0[:] = [float(hx.LIGHT_SPOT), 0.6, 0.8, 1.0]
        sp.data1[:] = [float(sdir[0]), float(sdir[1]), float(sdir[2]), 15.0]
        sp.data2[:] = [-1.5, 2.5, 1.5, 0.05]
        sp.data3[0], sp.data3[1] = (0.9, 0.9) if spot_equal_edges else (0.95, 0.85)
        ddir = np.array([-0.3, -1.0, -0.2])
        ddir /= np.linalg.norm(ddir)
        di.data0[:] = [float(hx.LIGHT_DIRECTIONAL), 1.0, 0.95, 0.9]
        di.data1[:] = [float(ddir[0]), float(ddir[1]), float(ddir[2]), 2.0]
        di.data2[3] = 0.02

        self._desc = hx.SceneDesc()
        d = self._desc
        d.meshes, d.num_meshes = self._mesh, len(meshes)
        d.instances, d.num_instances = self._inst, len(inst)
        d.materials, d.num_materials = self._mat, len(mats)
        d.textures, d.num_textures = self._tex, 3
        d.punctual_lights, d.num_punctual_lights = self._light, 3
        if env:
            ew, eh = 64, 32
            v = (np.arange(eh) + 0.5) / eh
            u = (np.arange(ew) + 0.5) / ew
            e = np.zeros((eh, ew, 4), np.float32)
            e[..., 0] = 0.25 + 0.2 * np.cos(np.pi * v)[:, None]
            e[..., 1] = 0.3 + 0.1 * np.sin(2 * np.pi * u)[None, :]
            e[..., 2] = 0.5 + 0.3 * np.cos(np.pi * v)[:, None]
            e[..., 3] = 1.0
            self._env = np.ascontiguousarray(e)
            d.environment.kind = hx.ENV_EQUIRECT
            d.environment.width, d.environment.height = ew, eh
            d.environment.rgba32f = self._env.ctypes.data_as(C.POINTER(C.c_float))
        else:
            d.environment.kind = 0

    @property
    def desc(self):
        return C.pointer(self._desc)

    def camera(self, aperture=0.0, focal_length=8.0):
        cam = hx.Camera()
        cam.position[:] = [0.3, 2.2, 4.5]
        cam.target[:] = [0.0, 0.6, 0.0]
        cam.up[:] = [0.0, 1.0, 0.0]
        cam.fov_y_degrees, cam.near_plane, cam.far_plane = 45.0, 1.0, 1000.0
        cam.focal_length, cam.aperture_radius = focal_length, aperture
        return cam


HX_NON_OPAQUE = 1
