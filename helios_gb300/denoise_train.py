"""Training data and training loop of the learned denoiser.

Training pairs come from this tracer: seeded variants of the icosphere scene
(the seed draws instance transforms, materials, point lights and alpha-quad
masks; the sun elevation is drawn from U(10, 80) degrees; the camera orbits
the scene at a seeded angle, radius and height).  For each variant the
integrator renders a low-spp image with its AOV features (the network input)
— at one or several progressive sample counts — and a high-spp image of the
same view (the target), all kept on the device.  A training step takes
`batch` images at random from the set and gathers them into the batch
buffers with device-to-device copies.
"""
import ctypes
import time

import numpy as np

import helios_gb300 as hx

FEATURE_BYTES = 12 * 4
TARGET_BYTES = 16


def variant_scene(seed, quads=20000, level=4, env=(512, 256), mask_pool=8, mask_size=128):
    """(HostScene, Camera) of one seeded variant of the icosphere scene."""
    rng = np.random.default_rng(seed)
    sun = float(rng.uniform(10.0, 80.0))
    hs = hx.HostScene(hx.SCENE_ICOSPHERES, seed=int(seed), sun_elevation_deg=sun, num_alpha_quads=quads,
                      icosphere_level=level, mask_pool=mask_pool, mask_size=mask_size, env_width=env[0],
                      env_height=env[1])
    cam = hs.camera()
    ang = rng.uniform(0.0, 2.0 * np.pi)
    rad = rng.uniform(22.0, 34.0)
    hgt = rng.uniform(-2.0, 14.0)
    cam.position[0], cam.position[1], cam.position[2] = rad * np.sin(ang), hgt, rad * np.cos(ang)
    cam.target[0], cam.target[1], cam.target[2] = rng.uniform(-3, 3), rng.uniform(-5, 1), rng.uniform(-3, 3)
    return hs, cam


def crop_frame(frame, full_w, full_h, x0, y0, w, h):
    """Frame constants of the w x h window at (x0, y0) of a full_w x full_h
    view: the same rays as the full frame's pixels there (camera NDC of the
    window mapped onto the full frame's NDC in view_proj_inverse)."""
    f = hx.FrameDesc()
    ctypes.memmove(ctypes.addressof(f), ctypes.addressof(frame), ctypes.sizeof(f))
    m = list(frame.view_proj_inverse)
    sx, sy = w / full_w, h / full_h
    bx, by = (2.0 * x0 + w) / full_w - 1.0, (2.0 * y0 + h) / full_h - 1.0
    for r in range(4):
        f.view_proj_inverse[0 * 4 + r] = sx * m[0 * 4 + r]
        f.view_proj_inverse[1 * 4 + r] = sy * m[1 * 4 + r]
        f.view_proj_inverse[3 * 4 + r] = bx * m[0 * 4 + r] + by * m[1 * 4 + r] + m[3 * 4 + r]
    return f


class PairSet:
    """Device-resident (features, target) images, all width x height."""

    def __init__(self, ctx, count, width, height):
        self.ctx, self.count, self.width, self.height = ctx, count, width, height
        px = width * height
        self.features = hx.DeviceBuffer(ctx, count * px * FEATURE_BYTES)
        self.targets = hx.DeviceBuffer(ctx, count * px * TARGET_BYTES)
        self.render_s = 0.0

    def feat_offset(self, i):
        return i * self.width * self.height * FEATURE_BYTES

    def tgt_offset(self, i):
        return i * self.width * self.height * TARGET_BYTES

    def close(self):
        self.features.close()
        self.targets.close()


def render_pairs(ctx, seeds, width, height, spp_in, spp_target, bounces=8, policy=None, scene_kw=None,
                 full_res=None):
    """One pair per (seed, input spp): the target is the seed's image at
    spp_target; the inputs are the features of the progressive image after
    each count in spp_in (ascending; an int means one count).  The input
    samples are the first frames of the same sample sequence as the target,
    a shared fraction of spp_in / spp_target; the auxiliary features are
    averaged over the same samples as the input radiance.  With full_res = (W, H) each
    image is a seeded width x height window of the W x H view (the pixel
    scale of full-resolution renders), else the whole view at width x height."""
    pol = policy if policy is not None else hx.policy_reference()
    counts = sorted(spp_in) if isinstance(spp_in, (list, tuple, np.ndarray)) else [int(spp_in)]
    ps = PairSet(ctx, len(seeds) * len(counts), width, height)
    t0 = time.time()
    k = 0
    for seed in seeds:
        hs, cam = variant_scene(seed, **(scene_kw or {}))
        sc = hx.Scene(ctx, hs)
        if full_res:
            rng = np.random.default_rng(seed + 77)
            x0 = int(rng.integers(0, full_res[0] - width + 1))
            y0 = int(rng.integers(0, full_res[1] - height + 1))
            f = crop_frame(hx.frame_desc(cam, full_res[0], full_res[1]), full_res[0], full_res[1], x0, y0, width,
                           height)
        else:
            f = hx.frame_desc(cam, width, height)
        it = hx.PathIntegrator(ctx, sc, width, height, max_ray_bounces=bounces, max_samples=1 << 30, policy=pol)
        it.render(f, spp_target)
        it.resolve(ps.targets, ps.tgt_offset(k))
        for j in range(1, len(counts)):
            ps.targets.copy_from(ps.targets, width * height * TARGET_BYTES, ps.tgt_offset(k + j), ps.tgt_offset(k))
        it.restart_bake()
        it.set_aov_accumulation(True)  # input features: AOVs averaged over the input's samples
        done = 0
        for c in counts:
            it.render(f, c - done)
            done = c
            it.features(f, ps.features, ps.feat_offset(k))
            k += 1
        ctx.synchronize()
        it.close()
        sc.close()
    ps.render_s = time.time() - t0
    return ps


def train(dn, data, steps, batch=16, lr=1e-3, seed=0, log_every=0, lr_final=None, count=None):
    """Adam over random batches of images [0, count) of the set (default
    all); returns the loss history (every log_every steps, else the first and
    last step)."""
    rng = np.random.default_rng(seed)
    count = data.count if count is None else count
    n = min(batch, count)
    px = data.width * data.height
    bf = hx.DeviceBuffer(data.ctx, n * px * FEATURE_BYTES)
    bt = hx.DeviceBuffer(data.ctx, n * px * TARGET_BYTES)
    hist = []
    for s in range(steps):
        pick = rng.choice(count, size=n, replace=False)
        for j, k in enumerate(pick):
            bf.copy_from(data.features, px * FEATURE_BYTES, j * px * FEATURE_BYTES, data.feat_offset(int(k)))
            bt.copy_from(data.targets, px * TARGET_BYTES, j * px * TARGET_BYTES, data.tgt_offset(int(k)))
        cur = lr if lr_final is None else lr * (lr_final / lr) ** (s / max(1, steps - 1))
        want = s == 0 or s == steps - 1 or bool(log_every and s % log_every == 0)
        loss = dn.train_step(bf, bt, n, data.height, data.width, cur, want_loss=want)
        if want:
            hist.append((s, loss))
    bf.close()
    bt.close()
    return hist


def rel_rmse(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def evaluate(ctx, dn, data, first, count):
    """Relative RMSE (linear radiance, rgb) against the targets of images
    [first, first + count): plain accumulation vs the denoised image."""
    w, h = data.width, data.height
    out = hx.DeviceBuffer(ctx, count * w * h * 16)
    dn.infer(data.features, count, h, w, out, feat_offset=data.feat_offset(first))
    dn.check()
    den = out.download((count, h, w, 4))[..., 0:3]
    feats = data.features.download((count, h, w, 12), offset=data.feat_offset(first))
    tgt = data.targets.download((count, h, w, 4), offset=data.tgt_offset(first))[..., 0:3]
    out.close()
    return rel_rmse(feats[..., 0:3], tgt), rel_rmse(den, tgt), den, tgt
