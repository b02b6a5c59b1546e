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
