"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE).

Loaded only by tests/, __graft_entry__.smoke() and the CPU-baseline leg of
bench.py, as the checker; the product library never imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liboracle.so")

_P = C.c_void_p


class Counters(C.Structure):
    _fields_ = [("paths", C.c_uint64), ("extension_rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("seconds", C.c_double), ("threads", C.c_int)]


_SIGS = {
    "oracle_scene_create": (_P, [_P]),
    "oracle_scene_destroy": (None, [_P]),
    "oracle_output_view": (None, [_P, _P, C.c_uint32, C.c_uint32, C.c_uint32, _P]),
    "oracle_debug_rays": (C.c_uint32, [_P, _P, _P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, _P, C.c_uint32]),
    "oracle_scene_num_prims": (C.c_uint32, [_P]),
    "oracle_scene_num_bvh8_nodes": (C.c_uint32, [_P]),
    "oracle_scene_num_lights": (C.c_uint32, [_P]),
    "oracle_scene_lights": (None, [_P, _P]),
    "oracle_scene_env": (None, [_P, _P]),
    "oracle_bvh_export": (None, [_P, _P, _P, _P, _P, _P]),
    "oracle_trace": (None, [_P, _P, C.c_uint32, C.c_uint32, C.c_uint32, _P]),
    "oracle_primary_rays": (None, [_P, _P, C.c_uint32, _P]),
    "oracle_trace_bvh8": (None, [_P, _P, C.c_uint32, C.c_uint32, _P, C.POINTER(C.c_uint64)]),
    "oracle_sample_radiance": (None, [_P, _P, _P, C.c_uint32, C.c_uint32, _P, C.c_uint32, _P, _P]),
    "oracle_render": (None, [_P, _P, _P, C.c_uint32, C.c_uint32, _P, C.c_uint32, _P, C.c_int, C.POINTER(Counters)]),
    "oracle_tonemap": (None, [_P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_float, _P]),
    "oracle_rng_streams": (None, [C.c_uint32, _P, C.c_uint32, C.c_uint32, _P]),
    "oracle_wang_hash": (C.c_uint32, [C.c_uint32]),
    "oracle_pcg_hash": (C.c_uint32, [C.c_uint32]),
    "oracle_float_to_half": (C.c_uint16, [C.c_float]),
    "oracle_half_to_float": (C.c_float, [C.c_uint16]),
    "oracle_max_threads": (C.c_int, []),
    "oracle_offset_origins": (None, [_P, _P, _P, C.c_uint32, _P]),
}

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            subprocess.run(["make", "-s", "-C", _HERE], check=True)
        h = C.CDLL(LIB_PATH)
        for n, (r, a) in _SIGS.items():
            f = getattr(h, n)
            f.restype = r
            f.argtypes = a
        _lib = h
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


HIT_DTYPE = np.dtype([("t", np.float32), ("prim", np.uint32), ("u", np.float32), ("v", np.float32)])
BVH8_DTYPE = np.dtype([("origin", np.float32, 3), ("exponent", np.int8, 3), ("internal_mask", np.uint8),
                       ("child_base", np.uint32), ("prim_base", np.uint32), ("meta", np.uint8, 8),
                       ("qlo", np.uint8, (3, 8)), ("qhi", np.uint8, (3, 8))])


class OracleScene:
    """The oracle's own copy of a scene (flattened, BVH, lights, environment)."""

    def __init__(self, scene):
        # scene: an object with a .desc pointer (kept alive during the copy) or the pointer itself
        self._src = scene
        ptr = scene.desc if hasattr(scene, "desc") else scene
        self.handle = lib().oracle_scene_create(C.cast(ptr, C.c_void_p))
        if not self.handle:
            raise ValueError("oracle scene: textures must be RGBA8")

    @property
    def num_prims(self):
        return lib().oracle_scene_num_prims(self.handle)

    def lights(self):
        n = lib().oracle_scene_num_lights(self.handle)
        out = np.zeros((n, 16), np.float32)
        lib().oracle_scene_lights(self.handle, _ptr(out))
        return out

    def env(self, width, height):
        out = np.zeros((height, width, 3), np.float32)
        lib().oracle_scene_env(self.handle, _ptr(out))
        return out

    def export_bvh(self):
        n = self.num_prims
        nn = lib().oracle_scene_num_bvh8_nodes(self.handle)
        morton = np.zeros(n, np.uint32)
        sorted_ = np.zeros(n, np.uint32)
        children = np.zeros(max(0, 2 * (n - 1)), np.uint32)
        nodes = np.zeros(nn, BVH8_DTYPE)
        leaf = np.zeros(n, np.uint32)
        lib().oracle_bvh_export(self.handle, _ptr(morton), _ptr(sorted_), _ptr(children) if children.size else None,
                                _ptr(nodes), _ptr(leaf))
        return dict(morton=morton, sorted=sorted_, children=children, nodes=nodes, leaf_prims=leaf)

    def trace(self, rays, any_hit=False, brute=False):
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        hits = np.zeros(rays.shape[0], HIT_DTYPE)
        lib().oracle_trace(self.handle, _ptr(rays), rays.shape[0], 1 if any_hit else 0, 1 if brute else 0, _ptr(hits))
        return hits

    def output_view(self, frame, width, height, which):
        """Output-buffer view (albedo 0 .. emissive 4), (H, W, 4) float32, display row order."""
        out = np.zeros((height, width, 4), np.float32)
        lib().oracle_output_view(self.handle, C.byref(frame), width, height, which, _ptr(out))
        return out

    def debug_rays(self, idesc, frame, px, py, num_rays, sample_index):
        """Ray-debug segments: (V, 8) float32 vertices (position xyz1, colour rgb1), paths in order."""
        cap = 2 * num_rays * max(1, idesc.max_ray_bounces)
        out = np.zeros((cap, 8), np.float32)
        n = lib().oracle_debug_rays(self.handle, C.byref(idesc), C.byref(frame), px, py, num_rays, sample_index,
                                    _ptr(out), cap)
        return out[:n]

    def trace_bvh8(self, rays, any_hit=False):
        """Closest hits through the 8-wide tree in the device arithmetic."""
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        hits = np.zeros(rays.shape[0], HIT_DTYPE)
        nv = C.c_uint64()
        lib().oracle_trace_bvh8(self.handle, _ptr(rays), rays.shape[0], 1 if any_hit else 0, _ptr(hits), C.byref(nv))
        return hits, nv.value

    def sample_radiance(self, idesc, frame, frame_index=0, precision=32, pixels=None):
        pix = None if pixels is None else np.ascontiguousarray(pixels, dtype=np.uint32)
        n = idesc.width * idesc.height if pix is None else pix.size
        out = np.zeros((n, 3), np.float32)
        prim = np.zeros(n, HIT_DTYPE)
        lib().oracle_sample_radiance(self.handle, C.byref(idesc), C.byref(frame), frame_index, precision, _ptr(pix),
                                     0 if pix is None else pix.size, _ptr(out), _ptr(prim))
        return out, prim

    def render(self, idesc, frame, num_frames, precision=32, pixels=None, threads=0):
        pix = None if pixels is None else np.ascontiguousarray(pixels, dtype=np.uint32)
        n = idesc.width * idesc.height if pix is None else pix.size
        out = np.zeros((n, 3), np.float64)
        cnt = Counters()
        lib().oracle_render(self.handle, C.byref(idesc), C.byref(frame), num_frames, precision, _ptr(pix),
                            0 if pix is None else pix.size, _ptr(out), threads, C.byref(cnt))
        return out, cnt

    def close(self):
        if self.handle:
            lib().oracle_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def primary_rays(idesc, frame, frame_index=0):
    out = np.zeros((idesc.width * idesc.height, 8), np.float32)
    lib().oracle_primary_rays(C.byref(idesc), C.byref(frame), frame_index, _ptr(out))
    return out


def tonemap(accum_rgba, op, exposure):
    h, w = accum_rgba.shape[:2]
    a = np.ascontiguousarray(accum_rgba, dtype=np.float32)
    out = np.zeros((h, w, 4), np.uint8)
    lib().oracle_tonemap(_ptr(a), w, h, op, exposure, _ptr(out))
    return out


def rng_streams(kind, seeds, draws):
    seeds = np.ascontiguousarray(seeds, dtype=np.uint32)
    n = seeds.size // 2
    out = np.zeros((n, draws), np.uint32)
    lib().oracle_rng_streams(kind, _ptr(seeds), n, draws, _ptr(out))
    return out
