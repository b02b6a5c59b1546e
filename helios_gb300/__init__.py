"""helios_gb300 — Python view of the helios-gb300 C-ABI (include/hx.h).

The product is the CUDA library ``libhx.so`` (sm_103a); this module is a thin
ctypes mirror of its C-ABI plus the engine-shaped classes the reference
exposes to its renderer (``PathIntegrator``, ``Renderer``, ``Scene``).  There
is no CPU fallback: every call goes to the CUDA library and fails loudly when
it is missing or when no GB300 is present.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libhx.so")

# status codes (hx_status)
HX_OK, HX_ERR_INVALID_ARG, HX_ERR_OOM_BUDGET, HX_ERR_TIMEOUT, HX_ERR_DEVICE, HX_ERR_NOT_READY, \
    HX_ERR_UNSUPPORTED, HX_ERR_CANCELLED = range(8)
LIGHT_DIRECTIONAL, LIGHT_SPOT, LIGHT_POINT, LIGHT_ENVIRONMENT, LIGHT_AREA = range(5)
ENV_NONE, ENV_EQUIRECT, ENV_HOSEK_WILKIE = range(3)
RNG_XOROSHIRO64STAR, RNG_PCG = 0, 1
ACCUM_RUNNING_MEAN, ACCUM_KAHAN = 0, 1
ENV_SAMPLE_COSINE, ENV_SAMPLE_IMPORTANCE = 0, 1
PAYLOAD_FP32, PAYLOAD_FP16 = 0, 1
RAY_OFFSET_REFERENCE, RAY_OFFSET_SCALED = 0, 1
TONEMAP_ACES, TONEMAP_REINHARD, TONEMAP_NONE = 0, 1, 2
TEXTURE_RGBA8, TEXTURE_BC1_RGB, TEXTURE_BC1_RGBA, TEXTURE_BC2, TEXTURE_BC3, TEXTURE_BC4, TEXTURE_BC5, TEXTURE_BC7 = range(8)
TEXTURE_BC6H_SF16, TEXTURE_BC6H_UF16, TEXTURE_RGBA16F, TEXTURE_RGBA8_SNORM = 8, 9, 10, 11
OUTPUT_ALBEDO, OUTPUT_NORMALS, OUTPUT_ROUGHNESS, OUTPUT_METALLIC, OUTPUT_EMISSIVE, OUTPUT_FINAL = 0, 1, 2, 3, 4, 5
SCENE_BOX, SCENE_ICOSPHERES, SCENE_TERRAIN = 0, 1, 2
SUBMESH_NON_OPAQUE = 1
NO_HIT = 0xFFFFFFFF


class HxError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("hx status %d: %s" % (status, msg))
        self.status = status


# ---------------------------------------------------------------------------
# Struct mirrors (layouts of include/hx.h)
# ---------------------------------------------------------------------------
class Vertex(C.Structure):
    _fields_ = [("position", C.c_float * 4), ("tex_coord", C.c_float * 4), ("normal", C.c_float * 4),
                ("tangent", C.c_float * 4), ("bitangent", C.c_float * 4)]


class Submesh(C.Structure):
    _fields_ = [("base_index", C.c_uint32), ("index_count", C.c_uint32), ("material", C.c_uint32),
                ("flags", C.c_uint32)]


class MeshDesc(C.Structure):
    _fields_ = [("vertices", C.POINTER(Vertex)), ("num_vertices", C.c_uint32),
                ("indices", C.POINTER(C.c_uint32)), ("num_indices", C.c_uint32),
                ("submeshes", C.POINTER(Submesh)), ("num_submeshes", C.c_uint32)]


class Material(C.Structure):
    _fields_ = [("texture_indices0", C.c_int32 * 4), ("texture_indices1", C.c_int32 * 4),
                ("albedo", C.c_float * 4), ("emissive", C.c_float * 4), ("roughness_metallic", C.c_float * 4)]


class Light(C.Structure):
    _fields_ = [("data0", C.c_float * 4), ("data1", C.c_float * 4), ("data2", C.c_float * 4),
                ("data3", C.c_float * 4)]


class Instance(C.Structure):
    _fields_ = [("model_matrix", C.c_float * 16), ("normal_matrix", C.c_float * 16), ("mesh_index", C.c_uint32),
                ("material_override", C.c_int32), ("padding", C.c_float * 2)]


class TextureDesc(C.Structure):
    _fields_ = [("rgba8", C.POINTER(C.c_uint8)), ("width", C.c_uint32), ("height", C.c_uint32),
                ("srgb", C.c_uint32), ("format", C.c_uint32)]


class EnvironmentDesc(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32),
                ("rgba32f", C.POINTER(C.c_float)), ("sun_direction", C.c_float * 4), ("coeffs", C.c_float * 40)]


class SceneDesc(C.Structure):
    _fields_ = [("meshes", C.POINTER(MeshDesc)), ("num_meshes", C.c_uint32),
                ("instances", C.POINTER(Instance)), ("num_instances", C.c_uint32),
                ("materials", C.POINTER(Material)), ("num_materials", C.c_uint32),
                ("textures", C.POINTER(TextureDesc)), ("num_textures", C.c_uint32),
                ("punctual_lights", C.POINTER(Light)), ("num_punctual_lights", C.c_uint32),
                ("environment", EnvironmentDesc)]


class Policy(C.Structure):
    _fields_ = [("rng", C.c_uint32), ("rr_start_depth", C.c_uint32), ("rr_clamp", C.c_uint32),
                ("radiance_clamp", C.c_float), ("accumulation", C.c_uint32), ("area_count_from_x", C.c_uint32),
                ("area_w_one", C.c_uint32), ("env_sampling", C.c_uint32), ("payload", C.c_uint32),
                ("visualize_nans", C.c_uint32), ("ray_offset", C.c_uint32), ("reserved", C.c_uint32)]


class IntegratorDesc(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("max_ray_bounces", C.c_uint32),
                ("max_samples", C.c_uint32), ("shadow_ray_bias", C.c_float), ("tiled", C.c_uint32),
                ("max_paths_in_flight", C.c_uint32), ("reserved", C.c_uint32), ("policy", Policy)]


class FrameDesc(C.Structure):
    _fields_ = [("view_proj_inverse", C.c_float * 16), ("camera_pos", C.c_float * 4),
                ("up_direction", C.c_float * 4), ("right_direction", C.c_float * 4),
                ("focal_plane", C.c_float * 4), ("focal_length", C.c_float), ("aperture_radius", C.c_float),
                ("reserved", C.c_float * 2)]


class Camera(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("target", C.c_float * 3), ("up", C.c_float * 3),
                ("fov_y_degrees", C.c_float), ("near_plane", C.c_float), ("far_plane", C.c_float),
                ("focal_length", C.c_float), ("aperture_radius", C.c_float)]


class Hit(C.Structure):
    _fields_ = [("t", C.c_float), ("prim", C.c_uint32), ("u", C.c_float), ("v", C.c_float)]


HIT_DTYPE = np.dtype([("t", np.float32), ("prim", np.uint32), ("u", np.float32), ("v", np.float32)])


class Stats(C.Structure):
    _fields_ = [("paths", C.c_uint64), ("extension_rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("ms_total", C.c_double), ("ms_raygen", C.c_double), ("ms_trace", C.c_double),
                ("ms_shade", C.c_double), ("ms_shadow", C.c_double), ("ms_accumulate", C.c_double),
                ("trace_launches", C.c_uint32), ("kernel_launches", C.c_uint32),
                ("node_visits", C.c_uint64), ("tri_tests", C.c_uint64),
                ("warp_node_steps", C.c_uint64), ("warp_tri_steps", C.c_uint64),
                ("warp_loop_iters", C.c_uint64), ("lane_loop_busy", C.c_uint64), ("alpha_tests", C.c_uint64)]


class SceneInfo(C.Structure):
    _fields_ = [("num_triangles", C.c_uint32), ("num_bvh8_nodes", C.c_uint32), ("num_binary_nodes", C.c_uint32),
                ("num_lights", C.c_uint32), ("device_bytes", C.c_uint64), ("build_ms", C.c_double),
                ("scene_min", C.c_float * 3), ("scene_max", C.c_float * 3)]


class ProceduralParams(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("seed", C.c_uint64), ("num_alpha_quads", C.c_uint32),
                ("mask_pool", C.c_uint32), ("mask_size", C.c_uint32), ("icosphere_level", C.c_uint32),
                ("env_width", C.c_uint32), ("env_height", C.c_uint32), ("sun_elevation_deg", C.c_float),
                ("turbidity", C.c_float), ("terrain_size", C.c_uint32), ("num_spheres", C.c_uint32),
                ("ground_albedo", C.c_float)]


class ServerDesc(C.Structure):
    _fields_ = [("request_arena_bytes", C.c_uint64), ("max_paths_per_tick", C.c_uint32),
                ("max_ray_bounces", C.c_uint32), ("policy", Policy), ("result_arena_bytes", C.c_uint64),
                ("admitted_work_paths", C.c_uint64), ("max_concurrent_ticks", C.c_uint32),
                ("max_paths_per_long_tick", C.c_uint32)]


class RequestDesc(C.Structure):
    _fields_ = [("scene_id", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32), ("spp", C.c_uint32),
                ("denoise", C.c_uint32), ("tonemap_op", C.c_uint32), ("exposure", C.c_float),
                ("reserved", C.c_uint32), ("frame", FrameDesc), ("user_tag", C.c_uint64)]


class RequestResult(C.Structure):
    _fields_ = [("request_id", C.c_uint64), ("user_tag", C.c_uint64), ("paths", C.c_uint64),
                ("queue_ms", C.c_double), ("latency_ms", C.c_double), ("status", C.c_int), ("reserved", C.c_uint32)]


class ServerStats(C.Structure):
    _fields_ = [("paths", C.c_uint64), ("ticks", C.c_uint64), ("requests_done", C.c_uint64),
                ("requests_pending", C.c_uint64), ("requests_active", C.c_uint64), ("arena_bytes", C.c_uint64),
                ("arena_used", C.c_uint64), ("seconds", C.c_double), ("requests_denoised", C.c_uint64),
                ("requests_active_peak", C.c_uint64), ("arena_used_peak", C.c_uint64)]


BVH8_NODE_BYTES = 80
BVH8_DTYPE = np.dtype([("origin", np.float32, 3), ("exponent", np.int8, 3), ("internal_mask", np.uint8),
                       ("child_base", np.uint32), ("prim_base", np.uint32), ("meta", np.uint8, 8),
                       ("qlo", np.uint8, (3, 8)), ("qhi", np.uint8, (3, 8))])
assert BVH8_DTYPE.itemsize == BVH8_NODE_BYTES

# C-ABI entry points: name -> (restype, argtypes)
_P = C.c_void_p
_SIGS = {
    "hx_version": (C.c_char_p, []),
    "hx_last_error_string": (C.c_char_p, []),
    "hx_policy_reference": (None, [C.POINTER(Policy)]),
    "hx_policy_spec": (None, [C.POINTER(Policy)]),
    "hx_camera_to_frame_desc": (C.c_int, [C.POINTER(Camera), C.c_uint32, C.c_uint32, C.POINTER(FrameDesc)]),
    "hx_context_create": (C.c_int, [C.c_int, C.c_uint64, C.POINTER(_P)]),
    "hx_context_destroy": (C.c_int, [_P]),
    "hx_context_synchronize": (C.c_int, [_P]),
    "hx_context_memory": (C.c_int, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "hx_measure_read_bandwidth": (C.c_int, [_P, C.c_uint64, C.c_uint32, C.POINTER(C.c_double)]),
    "hx_scene_upload": (C.c_int, [_P, C.POINTER(SceneDesc), C.POINTER(_P)]),
    "hx_scene_destroy": (C.c_int, [_P]),
    "hx_scene_info_get": (C.c_int, [_P, C.POINTER(SceneInfo)]),
    "hx_scene_set_traversal_stack_limit": (C.c_int, [_P, C.c_uint32]),
    "hx_scene_lights": (C.c_int, [_P, C.POINTER(Light), C.c_uint32, C.POINTER(C.c_uint32)]),
    "hx_scene_export_bvh": (C.c_int, [_P, _P, _P, _P, _P, _P]),
    "hx_scene_trace": (C.c_int, [_P, _P, C.c_uint32, C.c_uint32, _P]),
    "hx_integrator_create": (C.c_int, [_P, _P, C.POINTER(IntegratorDesc), C.POINTER(_P)]),
    "hx_integrator_destroy": (C.c_int, [_P]),
    "hx_integrator_render": (C.c_int, [_P, C.POINTER(FrameDesc)]),
    "hx_integrator_render_frames": (C.c_int, [_P, C.POINTER(FrameDesc), C.c_uint32]),
    "hx_integrator_restart_bake": (C.c_int, [_P]),
    "hx_integrator_set_max_ray_bounces": (C.c_int, [_P, C.c_uint32]),
    "hx_integrator_set_max_samples": (C.c_int, [_P, C.c_uint32]),
    "hx_integrator_set_shadow_ray_bias": (C.c_int, [_P, C.c_float]),
    "hx_integrator_set_tiled": (C.c_int, [_P, C.c_uint32]),
    "hx_integrator_set_policy": (C.c_int, [_P, C.POINTER(Policy)]),
    "hx_integrator_progress": (C.c_int, [_P, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "hx_integrator_tonemap": (C.c_int, [_P, C.c_uint32, C.c_float, _P]),
    "hx_integrator_read_accumulation": (C.c_int, [_P, _P]),
    "hx_integrator_checkpoint_size": (C.c_int, [_P, C.POINTER(C.c_size_t)]),
    "hx_integrator_save_checkpoint": (C.c_int, [_P, _P, C.c_size_t]),
    "hx_integrator_load_checkpoint": (C.c_int, [_P, _P, C.c_size_t]),
    "hx_integrator_render_output": (C.c_int, [_P, C.POINTER(FrameDesc), C.c_uint32, _P]),
    "hx_integrator_gather_debug_rays": (C.c_int, [_P, C.POINTER(FrameDesc), C.c_uint32, C.c_uint32, C.c_uint32, _P,
                                                  C.c_uint32, C.POINTER(C.c_uint32)]),
    "hx_integrator_set_timing": (C.c_int, [_P, C.c_uint32]),
    "hx_integrator_stats": (C.c_int, [_P, C.POINTER(Stats)]),
    "hx_integrator_set_counting": (C.c_int, [_P, C.c_uint32]),
    "hx_event_create": (C.c_int, [_P, C.POINTER(_P)]),
    "hx_event_record": (C.c_int, [_P]),
    "hx_event_elapsed": (C.c_int, [_P, _P, C.POINTER(C.c_float)]),
    "hx_event_destroy": (C.c_int, [_P]),
    "hx_pinned_alloc": (C.c_int, [C.c_size_t, C.POINTER(_P)]),
    "hx_pinned_free": (C.c_int, [_P]),
    "hx_scene_export_env": (C.c_int, [_P, _P]),
    "hx_lbvh_sort_noalloc": (C.c_int, [_P, C.c_uint32, _P, _P, _P]),
    "hx_server_create": (C.c_int, [_P, C.POINTER(ServerDesc), C.POINTER(_P)]),
    "hx_server_add_scene": (C.c_int, [_P, _P, C.POINTER(C.c_uint32)]),
    "hx_server_start": (C.c_int, [_P]),
    "hx_server_submit": (C.c_int, [_P, C.POINTER(RequestDesc), C.POINTER(C.c_uint64)]),
    "hx_server_poll": (C.c_int, [_P, C.POINTER(RequestResult), C.c_uint32, C.POINTER(C.c_uint32), C.c_double]),
    "hx_server_fetch": (C.c_int, [_P, C.c_uint64, _P]),
    "hx_server_cancel": (C.c_int, [_P, C.c_uint64]),
    "hx_server_stats_get": (C.c_int, [_P, C.POINTER(ServerStats)]),
    "hx_server_destroy": (C.c_int, [_P]),
    "hx_integrator_primary_hits": (C.c_int, [_P, C.POINTER(FrameDesc), C.c_uint32, _P]),
    "hx_integrator_sample_radiance": (C.c_int, [_P, C.POINTER(FrameDesc), C.c_uint32, _P]),
    "hx_rng_streams": (C.c_int, [_P, C.c_uint32, _P, C.c_uint32, C.c_uint32, _P]),
    "hx_procedural_defaults": (None, [C.c_uint32, C.POINTER(ProceduralParams)]),
    "hx_procedural_scene_create": (C.c_int, [C.POINTER(ProceduralParams), C.POINTER(_P)]),
    "hx_host_scene_desc": (C.POINTER(SceneDesc), [_P]),
    "hx_host_scene_camera": (C.c_int, [_P, C.POINTER(Camera)]),
    "hx_host_scene_destroy": (C.c_int, [_P]),
    "hx_hosek_wilkie_coefficients": (C.c_int, [C.POINTER(C.c_float), C.c_float, C.c_float, C.POINTER(C.c_float)]),
    "hx_hosek_wilkie_sky": (C.c_int, [_P, C.c_float, C.c_float, C.c_float, _P]),
    "hx_device_alloc": (C.c_int, [_P, C.c_uint64, C.POINTER(_P)]),
    "hx_device_free": (C.c_int, [_P, _P]),
    "hx_device_copy": (C.c_int, [_P, _P, _P, C.c_uint64, C.c_uint32]),
    "hx_denoiser_create": (C.c_int, [_P, C.POINTER(_P)]),
    "hx_denoiser_destroy": (C.c_int, [_P]),
    "hx_denoiser_num_params": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "hx_denoiser_set_params": (C.c_int, [_P, _P, C.c_uint64]),
    "hx_denoiser_get_params": (C.c_int, [_P, _P, C.c_uint64]),
    "hx_denoiser_forward_backward": (C.c_int, [_P, _P, _P, C.c_uint32, C.c_uint32, C.c_uint32,
                                               C.POINTER(C.c_float)]),
    "hx_denoiser_get_gradients": (C.c_int, [_P, _P, C.c_uint64]),
    "hx_denoiser_adam_step": (C.c_int, [_P, C.c_float]),
    "hx_denoiser_train_step": (C.c_int, [_P, _P, _P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_float,
                                         C.POINTER(C.c_float)]),
    "hx_denoiser_infer": (C.c_int, [_P, _P, C.c_uint32, C.c_uint32, C.c_uint32, _P]),
    "hx_denoiser_check": (C.c_int, [_P]),
    "hx_denoiser_set_wait_budget": (C.c_int, [_P, C.c_uint64]),
    "hx_denoiser_init_params": (C.c_int, [_P, C.c_uint64]),
    "hx_denoiser_read_tensor": (C.c_int, [_P, C.c_uint32, C.c_uint32, C.c_uint32, _P, C.c_uint64]),
    "hx_denoiser_read_output": (C.c_int, [_P, C.c_uint32, _P, C.c_uint64]),
    "hx_integrator_features": (C.c_int, [_P, C.POINTER(FrameDesc), C.c_uint32, _P]),
    "hx_integrator_resolve": (C.c_int, [_P, _P]),
    "hx_integrator_denoise": (C.c_int, [_P, _P, C.POINTER(FrameDesc), C.c_uint32, C.c_float, _P, _P]),
    "hx_server_set_denoiser": (C.c_int, [_P, _P]),
    "hx_denoiser_set_loss": (C.c_int, [_P, C.c_uint32]),
    "hx_integrator_set_aov_accumulation": (C.c_int, [_P, C.c_uint32]),
    "hx_encode_png": (C.c_int, [_P, C.c_uint32, C.c_uint32, _P, C.c_uint64, C.POINTER(C.c_uint64)]),
    "hx_save_png": (C.c_int, [C.c_char_p, _P, C.c_uint32, C.c_uint32]),
    "hx_texture_decode": (C.c_int, [C.POINTER(TextureDesc), _P]),
    "hx_texture_decode_hdr": (C.c_int, [C.POINTER(TextureDesc), _P]),
}

_lib_handle = None


def lib():
    """Loads libhx.so (built in-tree by ``__graft_entry__.build()``)."""
    global _lib_handle
    if _lib_handle is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("helios_gb300: CUDA library %s is missing; build it with "
                               "python -c 'import __graft_entry__ as g; g.build()'" % LIB_PATH)
        h = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(h, name)
            f.restype = res
            f.argtypes = args
        _lib_handle = h
    return _lib_handle


def exported_symbols():
    return sorted(_SIGS)


def check(status):
    if status != HX_OK:
        raise HxError(status, lib().hx_last_error_string().decode())


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def policy_reference():
    p = Policy()
    lib().hx_policy_reference(C.byref(p))
    return p


def policy_spec():
    p = Policy()
    lib().hx_policy_spec(C.byref(p))
    return p


def frame_desc(camera, width, height):
    f = FrameDesc()
    check(lib().hx_camera_to_frame_desc(C.byref(camera), width, height, C.byref(f)))
    return f


def hosek_wilkie_coefficients(sun_direction, turbidity=3.0, normalized_sun_y=1.15, albedo=0.1):
    d = (C.c_float * 3)(*sun_direction)
    out = (C.c_float * 40)()
    check(lib().hx_hosek_wilkie_sky(d, turbidity, albedo, normalized_sun_y, out))
    return np.array(out[:], dtype=np.float32).reshape(10, 4)[:, :3]


def encode_png(rgba8):
    """PNG file bytes of an (H, W, 4) uint8 image (Renderer::save_image_to_disk's format)."""
    img = np.ascontiguousarray(rgba8, dtype=np.uint8)
    h, w = img.shape[0], img.shape[1]
    n = C.c_uint64()
    check(lib().hx_encode_png(_ptr(img), w, h, None, 0, C.byref(n)))
    out = np.zeros(n.value, np.uint8)
    check(lib().hx_encode_png(_ptr(img), w, h, _ptr(out), out.size, C.byref(n)))
    return out.tobytes()


def texture_decode(data, width, height, fmt):
    """RGBA8 (height, width, 4) of a texture in format fmt (TEXTURE_*): data = its bytes."""
    buf = np.ascontiguousarray(data, np.uint8)
    t = TextureDesc()
    t.rgba8 = buf.ctypes.data_as(C.POINTER(C.c_uint8))
    t.width, t.height, t.format = width, height, fmt
    out = np.zeros((height, width, 4), np.uint8)
    check(lib().hx_texture_decode(C.byref(t), _ptr(out)))
    return out


def texture_decode_hdr(data, width, height, fmt):
    """RGBA16F (height, width, 4) float16 of a half-float texture (TEXTURE_BC6H_SF16/_UF16/RGBA16F)."""
    buf = np.ascontiguousarray(np.frombuffer(np.ascontiguousarray(data).tobytes(), np.uint8))
    t = TextureDesc()
    t.rgba8 = buf.ctypes.data_as(C.POINTER(C.c_uint8))
    t.width, t.height, t.format = width, height, fmt
    out = np.zeros((height, width, 4), np.uint16)
    check(lib().hx_texture_decode_hdr(C.byref(t), _ptr(out)))
    return out.view(np.float16)


def save_png(path, rgba8):
    img = np.ascontiguousarray(rgba8, dtype=np.uint8)
    check(lib().hx_save_png(os.fsencode(path), _ptr(img), img.shape[1], img.shape[0]))


class HostScene:
    """Seeded procedural scene (host arrays in the hx.h layouts)."""

    def __init__(self, kind=SCENE_BOX, **overrides):
        p = ProceduralParams()
        lib().hx_procedural_defaults(kind, C.byref(p))
        for k, v in overrides.items():
            setattr(p, k, v)
        self.params = p
        h = C.c_void_p()
        check(lib().hx_procedural_scene_create(C.byref(p), C.byref(h)))
        self.handle = h

    @property
    def desc(self):
        return lib().hx_host_scene_desc(self.handle)

    def camera(self):
        c = Camera()
        check(lib().hx_host_scene_camera(self.handle, C.byref(c)))
        return c

    def close(self):
        if self.handle:
            lib().hx_host_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Context:
    """One GPU + stream + HBM budget (the role of vk::Backend)."""

    def __init__(self, device=0, hbm_budget_bytes=0):
        h = C.c_void_p()
        check(lib().hx_context_create(device, hbm_budget_bytes, C.byref(h)))
        self.handle = h

    def synchronize(self):
        check(lib().hx_context_synchronize(self.handle))

    def memory(self):
        u, b = C.c_uint64(), C.c_uint64()
        check(lib().hx_context_memory(self.handle, C.byref(u), C.byref(b)))
        return u.value, b.value

    def read_bandwidth(self, nbytes, passes):
        """GB/s of one launch reading an nbytes buffer `passes` times (L1 bypassed)."""
        g = C.c_double()
        check(lib().hx_measure_read_bandwidth(self.handle, nbytes, passes, C.byref(g)))
        return g.value

    def rng_streams(self, kind, seeds, draws):
        seeds = np.ascontiguousarray(seeds, dtype=np.uint32)
        n = seeds.size // 2
        out = np.zeros((n, draws), dtype=np.uint32)
        check(lib().hx_rng_streams(self.handle, kind, _ptr(seeds), n, draws, _ptr(out)))
        return out

    def close(self):
        if self.handle:
            lib().hx_context_destroy(self.handle)
            self.handle = None


class Event:
    """Device timestamp recorded on a context's stream."""

    def __init__(self, ctx):
        h = C.c_void_p()
        check(lib().hx_event_create(ctx.handle, C.byref(h)))
        self.handle = h

    def record(self):
        check(lib().hx_event_record(self.handle))

    def elapsed_ms(self, end):
        ms = C.c_float()
        check(lib().hx_event_elapsed(self.handle, end.handle, C.byref(ms)))
        return ms.value

    def close(self):
        if self.handle:
            lib().hx_event_destroy(self.handle)
            self.handle = None


class PinnedBuffer:
    """Page-locked host memory viewed as a numpy array."""

    def __init__(self, shape, dtype):
        dtype = np.dtype(dtype)
        nbytes = int(np.prod(shape)) * dtype.itemsize
        h = C.c_void_p()
        check(lib().hx_pinned_alloc(nbytes, C.byref(h)))
        self.handle = h
        buf = (C.c_uint8 * nbytes).from_address(h.value)
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape)

    def close(self):
        if self.handle:
            self.array = None
            lib().hx_pinned_free(self.handle)
            self.handle = None


class Scene:
    """Device-resident scene: flattened triangles, BVH8, lights, environment
    (replaces Scene::create_gpu_resources and the BLAS/TLAS builds)."""

    def __init__(self, ctx, desc):
        self.ctx = ctx
        self._src = desc  # keeps a HostScene alive during the copy
        if hasattr(desc, "desc"):
            desc = desc.desc
        h = C.c_void_p()
        d = desc if isinstance(desc, SceneDesc) else desc.contents
        check(lib().hx_scene_upload(ctx.handle, C.byref(d), C.byref(h)))
        self.handle = h

    def info(self):
        i = SceneInfo()
        check(lib().hx_scene_info_get(self.handle, C.byref(i)))
        return i

    def set_traversal_stack_limit(self, entries):
        """Diagnostic: stack entries a ray may use (1..32, default 32)."""
        check(lib().hx_scene_set_traversal_stack_limit(self.handle, entries))

    def lights(self):
        n = C.c_uint32()
        check(lib().hx_scene_lights(self.handle, None, 0, C.byref(n)))
        arr = (Light * max(1, n.value))()
        check(lib().hx_scene_lights(self.handle, arr, n.value, C.byref(n)))
        return [arr[i] for i in range(n.value)]

    def export_bvh(self):
        info = self.info()
        n = info.num_triangles
        morton = np.zeros(n, np.uint32)
        sorted_ = np.zeros(n, np.uint32)
        children = np.zeros(max(0, 2 * (n - 1)), np.uint32)
        nodes = np.zeros(info.num_bvh8_nodes, BVH8_DTYPE)
        leaf = np.zeros(n, np.uint32)
        check(lib().hx_scene_export_bvh(self.handle, _ptr(morton), _ptr(sorted_),
                                        _ptr(children) if children.size else None, _ptr(nodes), _ptr(leaf)))
        return dict(morton=morton, sorted=sorted_, children=children, nodes=nodes, leaf_prims=leaf)

    def export_env(self, width, height):
        out = np.zeros((height, width, 3), np.float32)
        check(lib().hx_scene_export_env(self.handle, _ptr(out)))
        return out

    def trace(self, rays, any_hit=False):
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        hits = np.zeros(rays.shape[0], HIT_DTYPE)
        check(lib().hx_scene_trace(self.handle, _ptr(rays), rays.shape[0], 1 if any_hit else 0, _ptr(hits)))
        return hits

    def close(self):
        if self.handle:
            lib().hx_scene_destroy(self.handle)
            self.handle = None


class PathIntegrator:
    """Mirror of helios::PathIntegrator (include/gfx/path_integrator.h:9-62)."""

    def __init__(self, ctx, scene, width, height, max_ray_bounces=7, max_samples=5000, shadow_ray_bias=0.0,
                 tiled=False, policy=None, max_paths_in_flight=0):
        d = IntegratorDesc()
        d.width, d.height = width, height
        d.max_ray_bounces, d.max_samples = max_ray_bounces, max_samples
        d.shadow_ray_bias = shadow_ray_bias
        d.tiled = 1 if tiled else 0
        d.max_paths_in_flight = max_paths_in_flight
        d.policy = policy if policy is not None else policy_reference()
        self.desc = d
        self.width, self.height = width, height
        h = C.c_void_p()
        check(lib().hx_integrator_create(ctx.handle, scene.handle, C.byref(d), C.byref(h)))
        self.handle = h
        self.ctx, self.scene = ctx, scene

    def render(self, frame, num_frames=1):
        check(lib().hx_integrator_render_frames(self.handle, C.byref(frame), num_frames))

    def restart_bake(self):
        check(lib().hx_integrator_restart_bake(self.handle))

    def set_max_ray_bounces(self, n):
        check(lib().hx_integrator_set_max_ray_bounces(self.handle, n))

    def set_max_samples(self, n):
        check(lib().hx_integrator_set_max_samples(self.handle, n))

    def set_shadow_ray_bias(self, b):
        check(lib().hx_integrator_set_shadow_ray_bias(self.handle, b))

    def set_tiled(self, tiled):
        check(lib().hx_integrator_set_tiled(self.handle, 1 if tiled else 0))

    def set_policy(self, policy):
        check(lib().hx_integrator_set_policy(self.handle, C.byref(policy)))

    def progress(self):
        a, t, g = C.c_uint32(), C.c_uint32(), C.c_uint32()
        check(lib().hx_integrator_progress(self.handle, C.byref(a), C.byref(t), C.byref(g)))
        return a.value, t.value, g.value

    def num_accumulated_samples(self):
        return self.progress()[0]

    def tile_idx(self):
        return self.progress()[1]

    def num_target_samples(self):
        return self.progress()[2]

    def read_accumulation(self):
        out = np.zeros((self.height, self.width, 4), np.float32)
        check(lib().hx_integrator_read_accumulation(self.handle, _ptr(out)))
        return out

    def save_checkpoint(self):
        """The progressive bake state (header + images) as bytes."""
        n = C.c_size_t()
        check(lib().hx_integrator_checkpoint_size(self.handle, C.byref(n)))
        buf = np.empty(n.value, np.uint8)
        check(lib().hx_integrator_save_checkpoint(self.handle, _ptr(buf), buf.size))
        return buf.tobytes()

    def load_checkpoint(self, data):
        """Restore a state written by save_checkpoint (same size, max_samples, tiling, accumulation mode)."""
        buf = np.frombuffer(bytes(data), np.uint8)
        check(lib().hx_integrator_load_checkpoint(self.handle, _ptr(buf), buf.size))

    def render_output(self, frame, output_buffer):
        """Renderer output buffer (OUTPUT_ALBEDO .. OUTPUT_FINAL): (H, W, 4) float32, display row order."""
        out = np.zeros((self.height, self.width, 4), np.float32)
        check(lib().hx_integrator_render_output(self.handle, C.byref(frame), output_buffer, _ptr(out)))
        return out

    def gather_debug_rays(self, frame, pixel_x, pixel_y, num_debug_rays):
        """Ray-debug segments through a display pixel: (V, 8) float32 vertices
        (position xyz1, colour rgb1), two per segment, in shading order."""
        cap = 2 * num_debug_rays * max(1, self.desc.max_ray_bounces)
        out = np.zeros((cap, 8), np.float32)
        n = C.c_uint32()
        check(lib().hx_integrator_gather_debug_rays(self.handle, C.byref(frame), pixel_x, pixel_y, num_debug_rays,
                                                    _ptr(out), cap, C.byref(n)))
        return out[:n.value]

    def tonemap(self, op=TONEMAP_ACES, exposure=1.0, to_host=True):
        out = np.zeros((self.height, self.width, 4), np.uint8) if to_host else None
        check(lib().hx_integrator_tonemap(self.handle, op, exposure, _ptr(out)))
        return out

    def set_timing(self, on=True):
        check(lib().hx_integrator_set_timing(self.handle, 1 if on else 0))

    def set_counting(self, on=True):
        check(lib().hx_integrator_set_counting(self.handle, 1 if on else 0))

    def stats(self):
        s = Stats()
        check(lib().hx_integrator_stats(self.handle, C.byref(s)))
        return s

    def primary_hits(self, frame, frame_index=0):
        out = np.zeros(self.width * self.height, HIT_DTYPE)
        check(lib().hx_integrator_primary_hits(self.handle, C.byref(frame), frame_index, _ptr(out)))
        return out

    def sample_radiance(self, frame, frame_index=0):
        out = np.zeros((self.width * self.height, 3), np.float32)
        check(lib().hx_integrator_sample_radiance(self.handle, C.byref(frame), frame_index, _ptr(out)))
        return out

    def set_aov_accumulation(self, on=True):
        check(lib().hx_integrator_set_aov_accumulation(self.handle, 1 if on else 0))

    def features(self, frame, buf, offset=0, frame_index=0):
        """Denoiser features (width*height*12 floats) into a DeviceBuffer at a byte offset."""
        check(lib().hx_integrator_features(self.handle, C.byref(frame), frame_index, buf.at(offset)))

    def resolve(self, buf, offset=0):
        """The accumulated image (RGBA floats) into a DeviceBuffer at a byte offset."""
        check(lib().hx_integrator_resolve(self.handle, buf.at(offset)))

    def denoise(self, denoiser, frame, op=0, exposure=1.0, hdr=True, ldr=False):
        """Denoise the accumulated image; returns (rgba8 or None, rgba32f or None)."""
        o8 = np.zeros((self.height, self.width, 4), np.uint8) if ldr else None
        o32 = np.zeros((self.height, self.width, 4), np.float32) if hdr else None
        check(lib().hx_integrator_denoise(self.handle, denoiser.handle, C.byref(frame), op, exposure, _ptr(o8),
                                          _ptr(o32)))
        return o8, o32

    def close(self):
        if self.handle:
            lib().hx_integrator_destroy(self.handle)
            self.handle = None


class DeviceBuffer:
    """Device memory from a context's budgeted allocator."""

    def __init__(self, ctx, nbytes):
        h = C.c_void_p()
        check(lib().hx_device_alloc(ctx.handle, int(nbytes), C.byref(h)))
        self.ctx, self.ptr, self.nbytes = ctx, h.value, int(nbytes)

    def at(self, offset=0):
        if offset < 0 or offset > self.nbytes:
            raise ValueError("offset %d outside a %d-byte buffer" % (offset, self.nbytes))
        return C.c_void_p(self.ptr + offset)

    def upload(self, array, offset=0):
        a = np.ascontiguousarray(array)
        if offset + a.nbytes > self.nbytes:
            raise ValueError("upload past the end of the buffer")
        check(lib().hx_device_copy(self.ctx.handle, self.at(offset), _ptr(a), a.nbytes, 0))

    def download(self, shape, dtype=np.float32, offset=0):
        out = np.zeros(shape, dtype)
        if offset + out.nbytes > self.nbytes:
            raise ValueError("download past the end of the buffer")
        check(lib().hx_device_copy(self.ctx.handle, _ptr(out), self.at(offset), out.nbytes, 1))
        return out

    def copy_from(self, src, nbytes, dst_offset=0, src_offset=0):
        if dst_offset + nbytes > self.nbytes or src_offset + nbytes > src.nbytes:
            raise ValueError("copy out of range")
        check(lib().hx_device_copy(self.ctx.handle, self.at(dst_offset), src.at(src_offset), nbytes, 2))

    def close(self):
        if self.ptr:
            lib().hx_device_free(self.ctx.handle, C.c_void_p(self.ptr))
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# Denoiser tensors in network order: (name, channels, level)
DENOISER_TENSORS = [("x", 32, 0), ("a0", 32, 0), ("a0b", 32, 0), ("p0", 32, 1), ("a1", 64, 1), ("p1", 64, 2),
                    ("a2", 64, 2), ("p2", 64, 3), ("a3", 96, 3), ("p3", 96, 4), ("a4", 128, 4), ("a4b", 128, 4),
                    ("u3", 128, 3), ("d3", 96, 3), ("u2", 96, 2), ("d2", 64, 2), ("u1", 64, 1), ("d1", 64, 1),
                    ("u0", 64, 0), ("d0", 32, 0), ("d0b", 32, 0), ("gy", 32, 0)]
# Denoiser convolutions in network order: (input tensors, output channels)
DENOISER_LAYERS = [(("x",), 32), (("a0",), 32), (("p0",), 64), (("p1",), 64), (("p2",), 96), (("p3",), 128),
                   (("a4",), 128), (("u3", "a3"), 96), (("u2", "a2"), 64), (("u1", "a1"), 64), (("u0", "a0b"), 32),
                   (("d0",), 32), (("d0b",), 3)]


def denoiser_conv_flops_per_pixel():
    """Forward FLOPs of the denoiser per full-resolution pixel: 2 * 9 * cin * N
    per output pixel of each convolution (N = output channels rounded up to the
    MMA width of 16), at that convolution's level (1 / 4 per level)."""
    info = {n: (c, lev) for n, c, lev in DENOISER_TENSORS}
    tot = 0.0
    for srcs, cout in DENOISER_LAYERS:
        cin = sum(info[s][0] for s in srcs)
        tot += 2.0 * 9 * cin * ((cout + 15) // 16 * 16) / 4 ** info[srcs[0]][1]
    return tot


FEATURE_CHANNELS = 12
DN_LOSS_L1_LOG, DN_LOSS_L2_LINEAR = 0, 1


def _bf16_to_f32(u16):
    return (u16.astype(np.uint32) << 16).view(np.float32)


class Denoiser:
    """The learned denoiser (tensor-core training and inference)."""

    def __init__(self, ctx):
        h = C.c_void_p()
        check(lib().hx_denoiser_create(ctx.handle, C.byref(h)))
        self.handle, self.ctx = h, ctx
        n = C.c_uint64()
        check(lib().hx_denoiser_num_params(h, C.byref(n)))
        self.num_params = n.value
        self._shape = {}

    def init_params(self, seed=0):
        """He-uniform untrained weights, zero biases (hx_denoiser_init_params)."""
        check(lib().hx_denoiser_init_params(self.handle, seed))

    def set_params(self, params):
        p = np.ascontiguousarray(params, dtype=np.float32)
        check(lib().hx_denoiser_set_params(self.handle, _ptr(p), p.size))

    def get_params(self):
        out = np.zeros(self.num_params, np.float32)
        check(lib().hx_denoiser_get_params(self.handle, _ptr(out), out.size))
        return out

    def gradients(self):
        out = np.zeros(self.num_params, np.float32)
        check(lib().hx_denoiser_get_gradients(self.handle, _ptr(out), out.size))
        return out

    def forward_backward(self, features, targets, n, h, w, feat_offset=0, tgt_offset=0):
        loss = C.c_float()
        check(lib().hx_denoiser_forward_backward(self.handle, features.at(feat_offset), targets.at(tgt_offset), n, h,
                                                 w, C.byref(loss)))
        self._shape[1] = (n, h, w)
        return loss.value

    def adam_step(self, lr):
        check(lib().hx_denoiser_adam_step(self.handle, lr))

    def set_loss(self, kind):
        check(lib().hx_denoiser_set_loss(self.handle, kind))

    def train_step(self, features, targets, n, h, w, lr, feat_offset=0, tgt_offset=0, want_loss=True):
        loss = C.c_float()
        check(lib().hx_denoiser_train_step(self.handle, features.at(feat_offset), targets.at(tgt_offset), n, h, w, lr,
                                           C.byref(loss) if want_loss else None))
        self._shape[1] = (n, h, w)
        return loss.value if want_loss else None

    def infer(self, features, n, h, w, out, feat_offset=0, out_offset=0):
        check(lib().hx_denoiser_infer(self.handle, features.at(feat_offset), n, h, w, out.at(out_offset)))
        self._shape[0] = (n, (h + 15) // 16 * 16, (w + 15) // 16 * 16)

    def check(self):
        check(lib().hx_denoiser_check(self.handle))

    def set_wait_budget(self, cycles):
        """Diagnostic: clock cycles each tensor-core pipeline wait may take (0 = default)."""
        check(lib().hx_denoiser_set_wait_budget(self.handle, cycles))

    def read_tensor(self, name, training=True, gradient=False):
        idx = [t[0] for t in DENOISER_TENSORS].index(name)
        _, c, lev = DENOISER_TENSORS[idx]
        n, h, w = self._shape[1 if training else 0]
        raw = np.zeros((n, h >> lev, w >> lev, c), np.uint16)
        check(lib().hx_denoiser_read_tensor(self.handle, 1 if training else 0, idx, 1 if gradient else 0, _ptr(raw),
                                            raw.nbytes))
        return _bf16_to_f32(raw)

    def read_output(self, training=True):
        n, h, w = self._shape[1 if training else 0]
        out = np.zeros((n, h, w, 4), np.float32)
        check(lib().hx_denoiser_read_output(self.handle, 1 if training else 0, _ptr(out), out.size))
        return out

    def close(self):
        if self.handle:
            lib().hx_denoiser_destroy(self.handle)
            self.handle = None


class Server:
    """Resident render-serving loop (hx_server_*): scenes stay on the device,
    requests are admitted by HBM budget and batched into CUDA-graph ticks."""

    def __init__(self, ctx, arena_bytes=4 << 30, max_paths_per_tick=4 << 20, max_ray_bounces=8, policy=None,
                 max_concurrent_ticks=0, max_paths_per_long_tick=0):
        d = ServerDesc()
        d.max_concurrent_ticks = max_concurrent_ticks
        d.max_paths_per_long_tick = max_paths_per_long_tick
        d.request_arena_bytes = arena_bytes
        d.max_paths_per_tick = max_paths_per_tick
        d.max_ray_bounces = max_ray_bounces
        d.policy = policy if policy is not None else policy_reference()
        h = C.c_void_p()
        check(lib().hx_server_create(ctx.handle, C.byref(d), C.byref(h)))
        self.handle = h
        self.ctx = ctx
        self.sizes = {}

    def add_scene(self, scene):
        sid = C.c_uint32()
        check(lib().hx_server_add_scene(self.handle, scene.handle, C.byref(sid)))
        return sid.value

    def start(self):
        check(lib().hx_server_start(self.handle))

    def set_denoiser(self, denoiser):
        check(lib().hx_server_set_denoiser(self.handle, denoiser.handle if denoiser else None))

    def submit(self, scene_id, frame, width, height, spp, tonemap_op=TONEMAP_ACES, exposure=1.0, user_tag=0,
               denoise=False):
        r = RequestDesc()
        r.scene_id, r.width, r.height, r.spp = scene_id, width, height, spp
        r.denoise = 1 if denoise else 0
        r.tonemap_op, r.exposure, r.user_tag = tonemap_op, exposure, user_tag
        r.frame = frame
        rid = C.c_uint64()
        check(lib().hx_server_submit(self.handle, C.byref(r), C.byref(rid)))
        self.sizes[rid.value] = (width, height)
        return rid.value

    def poll(self, wait_seconds=0.0, capacity=256):
        arr = (RequestResult * capacity)()
        n = C.c_uint32()
        check(lib().hx_server_poll(self.handle, arr, capacity, C.byref(n), wait_seconds))
        return [arr[i] for i in range(n.value)]

    def cancel(self, request_id):
        check(lib().hx_server_cancel(self.handle, request_id))

    def fetch(self, request_id):
        w, h = self.sizes.pop(request_id)
        out = np.zeros((h, w, 4), np.uint8)
        check(lib().hx_server_fetch(self.handle, request_id, _ptr(out)))
        return out

    def stats(self):
        s = ServerStats()
        check(lib().hx_server_stats_get(self.handle, C.byref(s)))
        return s

    def close(self):
        if self.handle:
            lib().hx_server_destroy(self.handle)
            self.handle = None


class Renderer:
    """Mirror of the helios::Renderer surface this path owns
    (include/gfx/renderer.h:83-97): render, tone-map operator, exposure,
    save image."""

    def __init__(self, integrator, tone_map_operator=TONEMAP_ACES, exposure=1.0):
        self.integrator = integrator
        self.tone_map_operator = tone_map_operator
        self.exposure = exposure

    def set_tone_map_operator(self, op):
        self.tone_map_operator = op

    def set_exposure(self, e):
        self.exposure = e

    def render(self, frame):
        self.integrator.render(frame)
        return self.integrator.tonemap(self.tone_map_operator, self.exposure, to_host=False)

    def save_image_to_disk(self, path):
        """Writes the tone-mapped RGBA8 image as binary PPM (no image
        library dependency)."""
        img = self.integrator.tonemap(self.tone_map_operator, self.exposure)
        h, w = img.shape[:2]
        with open(path, "wb") as f:
            f.write(b"P6\n%d %d\n255\n" % (w, h))
            f.write(np.ascontiguousarray(img[:, :, :3]).tobytes())
        return img
