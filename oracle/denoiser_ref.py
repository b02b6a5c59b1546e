"""CPU oracle of the learned denoiser (test infrastructure only).

The denoiser has no counterpart in the reference engine; its inputs reuse the
reference's AOV definitions (albedo and shading normal as in
`src/gfx/shader/debug_visualization.frag:142-161`, buffer list in
`include/gfx/renderer.h:27-35`).  This module restates the network the CUDA
kernels run — same layer list, same parameter layout, same points where a
tensor is rounded to BF16 — in float64 numpy, forward and backward, so the
tests can check the device's activations and gradients.  With `rnd=False`
nothing is rounded, and `finite_difference_check` pins the backward pass to
central differences of the forward pass.

Network (5 levels, 3x3 'same' convolutions, ReLU, 2x2 average pooling,
nearest 2x upsampling, skip connections by concatenation):

    x   (32 ch: log1p radiance, albedo, normal, depth, noise level, zero padding)
    a0  = relu(conv(x))            32   level 0
    a0b = relu(conv(a0))           32   level 0   (skip)
    a1  = relu(conv(pool(a0b)))    64   level 1   (skip)
    a2  = relu(conv(pool(a1)))     64   level 2   (skip)
    a3  = relu(conv(pool(a2)))     96   level 3   (skip)
    a4  = relu(conv(pool(a3)))    128   level 4
    a4b = relu(conv(a4))          128   level 4
    d3  = relu(conv([up(a4b), a3]))  96
    d2  = relu(conv([up(d3), a2]))   64
    d1  = relu(conv([up(d2), a1]))   64
    d0  = relu(conv([up(d1), a0b]))  32
    d0b = relu(conv(d0))             32
    y   = x[..., 0:3] + conv(d0b)     3   (residual: the input's log1p radiance
                                           + a linear correction)

Loss: mean over pixels and the 3 channels of |y - log1p(target)| ("l1log"),
or of (expm1(y) - target)^2 ("l2lin").
"""
import numpy as np

# (name, [(source, channels), ...], cout, relu)
LAYERS = [
    ("e0", [("x", 32)], 32, True),
    ("e0b", [("a0", 32)], 32, True),
    ("e1", [("p0", 32)], 64, True),
    ("e2", [("p1", 64)], 64, True),
    ("e3", [("p2", 64)], 96, True),
    ("e4", [("p3", 96)], 128, True),
    ("e4b", [("a4", 128)], 128, True),
    ("d3", [("u3", 128), ("a3", 96)], 96, True),
    ("d2", [("u2", 96), ("a2", 64)], 64, True),
    ("d1", [("u1", 64), ("a1", 64)], 64, True),
    ("d0", [("u0", 64), ("a0b", 32)], 32, True),
    ("d0b", [("d0", 32)], 32, True),
    ("out", [("d0b", 32)], 3, False),
]
OUTPUT_OF = ["a0", "a0b", "a1", "a2", "a3", "a4", "a4b", "d3", "d2", "d1", "d0", "d0b", "y"]
IN_CHANNELS = 32
FEATURES = 12  # radiance rgb, pad, albedo rgb, depth, normal xyz, pad


def layer_shapes():
    """(cin, cout) per layer; parameters are stored per layer as W[9][cout][cin]
    (tap = ky*3 + kx) followed by b[cout], all float32, layers in order."""
    return [(sum(c for _, c in srcs), cout) for _, srcs, cout, _ in LAYERS]


def num_params():
    return sum(9 * ci * co + co for ci, co in layer_shapes())


def split_params(flat):
    out, o = [], 0
    for ci, co in layer_shapes():
        w = flat[o:o + 9 * co * ci].reshape(9, co, ci)
        o += 9 * co * ci
        b = flat[o:o + co]
        o += co
        out.append((w, b))
    return out


def init_params(seed):
    """He-uniform weights from a seeded generator, zero biases (the device
    takes its initial parameters from the host, so any init works)."""
    rng = np.random.default_rng(seed)
    parts = []
    for ci, co in layer_shapes():
        bound = np.sqrt(6.0 / (9 * ci))
        parts.append(rng.uniform(-bound, bound, size=9 * co * ci))
        parts.append(np.zeros(co))
    return np.concatenate(parts).astype(np.float32)


def bf16(a):
    """Round float array to bfloat16 (round to nearest even), returned as float64."""
    f = np.asarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    r = np.where(np.isnan(f), u | 0x400000, r)
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def pack_input(features, rnd=True):
    """features [n,h,w,12] float32 -> x [n,h,w,32]: log1p(max(radiance,0)),
    albedo, normal, depth, noise level (feature 3), then zeros."""
    f = np.asarray(features, np.float64)
    n, h, w, _ = f.shape
    x = np.zeros((n, h, w, IN_CHANNELS))
    x[..., 0:3] = np.log1p(np.maximum(f[..., 0:3], 0.0))
    x[..., 3:6] = f[..., 4:7]
    x[..., 6:9] = f[..., 8:11]
    x[..., 9] = f[..., 7]
    x[..., 10] = f[..., 3]
    return bf16(x) if rnd else x


def _shift(x, dy, dx):
    """out[y, x] = in[y + dy, x + dx] with zero padding."""
    n, h, w, c = x.shape
    o = np.zeros_like(x)
    ys, yd = (slice(dy, h), slice(0, h - dy)) if dy >= 0 else (slice(0, h + dy), slice(-dy, h))
    xs, xd = (slice(dx, w), slice(0, w - dx)) if dx >= 0 else (slice(0, w + dx), slice(-dx, w))
    o[:, yd, xd] = x[:, ys, xs]
    return o


def conv(x, w, b):
    """3x3 'same' conv: out[p, co] = sum_tap sum_ci x[p + off(tap), ci] w[tap, co, ci] + b."""
    n, h, wd, ci = x.shape
    out = np.zeros((n, h, wd, w.shape[1]))
    for t in range(9):
        ky, kx = divmod(t, 3)
        out += _shift(x, ky - 1, kx - 1).reshape(-1, ci).dot(w[t].T).reshape(n, h, wd, -1)
    return out + b


def conv_dgrad(g, w):
    n, h, wd, co = g.shape
    out = np.zeros((n, h, wd, w.shape[2]))
    for t in range(9):
        ky, kx = divmod(t, 3)
        out += _shift(g, 1 - ky, 1 - kx).reshape(-1, co).dot(w[t]).reshape(n, h, wd, -1)
    return out


def conv_wgrad(x, g):
    n, h, wd, ci = x.shape
    co = g.shape[3]
    dw = np.zeros((9, co, ci))
    g2 = g.reshape(-1, co)
    for t in range(9):
        ky, kx = divmod(t, 3)
        dw[t] = g2.T.dot(_shift(x, ky - 1, kx - 1).reshape(-1, ci))
    return dw, g2.sum(axis=0)


def pool(x):
    n, h, w, c = x.shape
    return x.reshape(n, h // 2, 2, w // 2, 2, c).sum(axis=(2, 4)) * 0.25


def up(x):
    return x.repeat(2, axis=1).repeat(2, axis=2)


def up_bwd(g):
    n, h, w, c = g.shape
    return g.reshape(n, h // 2, 2, w // 2, 2, c).sum(axis=(2, 4))


def forward(params, features, rnd=True):
    """Returns a dict of every activation (BF16-rounded where the device
    stores BF16) and y, the FP32 network output (log1p radiance)."""
    R = bf16 if rnd else (lambda a: a)
    P = split_params(np.asarray(params, np.float64))
    if rnd:
        P = [(bf16(w), np.asarray(b, np.float32).astype(np.float64)) for w, b in P]
    t = {"x": pack_input(features, rnd)}
    for i, (name, srcs, cout, relu) in enumerate(LAYERS):
        if name == "e1":
            t["p0"] = R(pool(t["a0b"]))
        elif name == "e2":
            t["p1"] = R(pool(t["a1"]))
        elif name == "e3":
            t["p2"] = R(pool(t["a2"]))
        elif name == "e4":
            t["p3"] = R(pool(t["a3"]))
        elif name == "d3":
            t["u3"] = up(t["a4b"])
        elif name == "d2":
            t["u2"] = up(t["d3"])
        elif name == "d1":
            t["u1"] = up(t["d2"])
        elif name == "d0":
            t["u0"] = up(t["d1"])
        x = np.concatenate([t[s] for s, _ in srcs], axis=3)
        w, b = P[i]
        o = conv(x, w, b)
        if relu:
            t[OUTPUT_OF[i]] = R(np.maximum(o, 0.0))
        else:
            o = o + t["x"][..., 0:3]
            t[OUTPUT_OF[i]] = np.asarray(o, np.float32).astype(np.float64) if rnd else o
    t["_params"] = P
    return t


def loss_and_grad(params, features, targets, rnd=True, loss="l1log"):
    """Forward + backward.  Returns (loss, flat gradient float64, tensors).
    loss: "l1log" = mean |y - log1p(t)|, "l2lin" = mean (expm1(y) - t)^2."""
    R = bf16 if rnd else (lambda a: a)
    t = forward(params, features, rnd)
    P = t["_params"]
    tl = np.maximum(np.asarray(targets, np.float64)[..., 0:3], 0.0)
    if loss == "l2lin":
        e = np.exp(t["y"])
        diff = (e - 1.0) - tl
        count = diff.size
        lval = (diff * diff).sum() / count
        gy = R(2.0 * diff * e)
    else:
        tgt = np.log1p(tl)
        diff = t["y"] - (np.asarray(tgt, np.float32).astype(np.float64) if rnd else tgt)
        count = diff.size
        lval = np.abs(diff).sum() / count
        gy = np.sign(diff)
    scale = 1.0 / count
    grads = [None] * len(LAYERS)
    g = {"y": gy}
    # pre-activation gradients flow backwards; masks from the stored outputs
    for i in reversed(range(len(LAYERS))):
        name, srcs, cout, relu = LAYERS[i]
        out = OUTPUT_OF[i]
        go = g.pop(out)
        x = np.concatenate([t[s] for s, _ in srcs], axis=3)
        dw, db = conv_wgrad(x, go)
        grads[i] = (dw * scale, db * scale)
        if i == 0:
            break
        w = P[i][0]
        dx = conv_dgrad(go, w)
        o = 0
        for s, c in srcs:
            part = dx[..., o:o + c]
            o += c
            if s.startswith("p"):
                # through the pooling into the (masked) skip tensor
                a = {"p0": "a0b", "p1": "a1", "p2": "a2", "p3": "a3"}[s]
                gp = R(part)
                contrib = np.where(t[a] > 0, up(gp) * 0.25, 0.0)
                g[a] = R(g[a] + contrib) if a in g else R(contrib)
            elif s.startswith("u"):
                src = {"u3": "a4b", "u2": "d3", "u1": "d2", "u0": "d1"}[s]
                gm = R(np.where(t[s] > 0, part, 0.0))
                g[src] = R(up_bwd(gm))
            else:
                gm = R(np.where(t[s] > 0, part, 0.0))
                g[s] = R(g[s] + gm) if s in g else gm
    flat = np.concatenate([np.concatenate([dw.ravel(), db]) for dw, db in grads])
    return lval, flat, t


def finite_difference_check(seed=0, n=1, h=16, w=16, probes=24, eps=1e-6, loss="l1log"):
    """Analytic (float64, no rounding) vs central-difference gradients of the
    loss on random features; returns the worst relative error over probes."""
    rng = np.random.default_rng(seed)
    params = init_params(seed).astype(np.float64)
    params += rng.normal(0, 0.01, params.shape)  # non-zero biases
    feats = rng.uniform(0, 1, (n, h, w, FEATURES))
    tg = rng.uniform(0, 2, (n, h, w, 4))
    _, g, _ = loss_and_grad(params, feats, tg, rnd=False, loss=loss)
    worst = 0.0
    idx = rng.choice(params.size, probes, replace=False)
    for k in idx:
        p1, p2 = params.copy(), params.copy()
        p1[k] += eps
        p2[k] -= eps
        l1, _, _ = loss_and_grad(p1, feats, tg, rnd=False, loss=loss)
        l2, _, _ = loss_and_grad(p2, feats, tg, rnd=False, loss=loss)
        num = (l1 - l2) / (2 * eps)
        worst = max(worst, abs(num - g[k]) / max(1e-6, abs(num) + abs(g[k])))
    return worst


def adam(params, m, v, grad, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (bias-corrected), float32 state like the device."""
    m[:] = b1 * m + (1 - b1) * grad
    v[:] = b2 * v + (1 - b2) * grad * grad
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    params -= lr * mh / (np.sqrt(vh) + eps)
    return params
