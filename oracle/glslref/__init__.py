"""ctypes binding of oracle/_ref/libglslref.so (TEST INFRASTRUCTURE).

The library holds the reference's own shader functions compiled as C++
(oracle/glslref/build.py) beside the oracle's restatement; the tests use it
to check the restatement against the reference's code.  load() builds it on
first use and returns None when the reference tree is absent.
"""
import ctypes as C

import numpy as np

from . import build as _build

_P = C.c_void_p
_SIGS = {
    "glslref_world_create": (_P, [_P, _P, C.c_uint32, _P, C.c_uint32, C.c_uint32]),
    "glslref_world_destroy": (None, [_P]),
    "glslref_sample_radiance": (None, [_P, _P, _P, C.c_uint32, _P, C.c_uint32, _P, _P, _P]),
    "glslref_render": (None, [_P, _P, _P, C.c_uint32, _P]),
    "glslref_tonemap": (None, [_P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_float, _P]),
    "glslref_rng_cases": (None, [_P, C.c_uint32, C.c_uint32, _P, _P]),
    "glslref_brdf_cases": (None, [_P, _P, C.c_uint32, _P, _P]),
    "glslref_sample_light_cases": (None, [_P, _P, _P, _P, _P, C.c_uint32, _P, _P]),
    "glslref_camera_cases": (None, [_P, _P, C.c_uint32, _P, C.c_uint32, _P, _P]),
}
_lib = None


def load():
    global _lib
    if _lib is None:
        path = _build.build()
        if path is None:
            return None
        h = C.CDLL(path)
        for n, (r, a) in _SIGS.items():
            fn = getattr(h, n)
            fn.restype = r
            fn.argtypes = a
        _lib = h
    return _lib


def _ptr(a):
    return a.ctypes.data_as(_P) if a is not None else None


class RefWorld:
    """A scene as the reference's shaders see it: the scene arrays, the
    oracle's packed light list and its lat-long environment map."""

    def __init__(self, scene, oracle_scene, env_size=None):
        self.lib = load()
        self.lights = np.ascontiguousarray(oracle_scene.lights(), np.float32)
        env = None
        ew = eh = 0
        if env_size:
            ew, eh = env_size
            env = np.ascontiguousarray(oracle_scene.env(ew, eh), np.float32)
        self._env = env
        ptr = scene.desc if hasattr(scene, "desc") else scene
        self.handle = self.lib.glslref_world_create(C.cast(ptr, _P), _ptr(self.lights), self.lights.shape[0],
                                                    _ptr(env), ew, eh)
        if not self.handle:
            raise ValueError("reference world: textures must be RGBA8")

    def sample_radiance(self, idesc, frame, frame_index=0, pixels=None):
        pix = None if pixels is None else np.ascontiguousarray(pixels, np.uint32)
        n = idesc.width * idesc.height if pix is None else pix.size
        out = np.zeros((n, 3), np.float32)
        prim = np.zeros(n, np.uint32)
        t = np.zeros(n, np.float32)
        self.lib.glslref_sample_radiance(self.handle, C.byref(idesc), C.byref(frame), frame_index, _ptr(pix), n,
                                         _ptr(out), _ptr(prim), _ptr(t))
        return out, prim, t

    def render(self, idesc, frame, num_frames):
        out = np.zeros((idesc.height, idesc.width, 4), np.float32)
        self.lib.glslref_render(self.handle, C.byref(idesc), C.byref(frame), num_frames, _ptr(out))
        return out

    def sample_light_cases(self, oracle_scene, idesc, cases, rng_states):
        cases = np.ascontiguousarray(cases, np.float32)
        rng_states = np.ascontiguousarray(rng_states, np.uint32)
        n = cases.shape[0]
        a = np.zeros((n, 16), np.float32)
        b = np.zeros((n, 16), np.float32)
        self.lib.glslref_sample_light_cases(self.handle, oracle_scene.handle, C.byref(idesc), _ptr(cases),
                                            _ptr(rng_states), n, _ptr(a), _ptr(b))
        return a, b

    def close(self):
        if self.handle:
            self.lib.glslref_world_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def rng_cases(seeds, draws):
    lib = load()
    seeds = np.ascontiguousarray(seeds, np.uint32)
    n = seeds.shape[0]
    a = np.zeros((n, draws * 3), np.uint32)
    b = np.zeros((n, draws * 3), np.uint32)
    lib.glslref_rng_cases(_ptr(seeds), n, draws, _ptr(a), _ptr(b))
    return a, b


def brdf_cases(cases, rng_states):
    lib = load()
    cases = np.ascontiguousarray(cases, np.float32)
    rng_states = np.ascontiguousarray(rng_states, np.uint32)
    n = cases.shape[0]
    a = np.zeros((n, 18), np.float32)
    b = np.zeros((n, 18), np.float32)
    lib.glslref_brdf_cases(_ptr(cases), _ptr(rng_states), n, _ptr(a), _ptr(b))
    return a, b


def camera_cases(idesc, frame, frame_index, pixels):
    lib = load()
    pixels = np.ascontiguousarray(pixels, np.uint32)
    n = pixels.size
    a = np.zeros((n, 8), np.float32)
    b = np.zeros((n, 8), np.float32)
    lib.glslref_camera_cases(C.byref(idesc), C.byref(frame), frame_index, _ptr(pixels), n, _ptr(a), _ptr(b))
    return a, b


def tonemap(accum_rgba, op, exposure):
    lib = load()
    h, w = accum_rgba.shape[:2]
    a = np.ascontiguousarray(accum_rgba, np.float32)
    out = np.zeros((h, w, 4), np.uint8)
    lib.glslref_tonemap(_ptr(a), w, h, op, exposure, _ptr(out))
    return out
